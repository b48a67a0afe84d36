"""ctypes wrapper of the C oracle (oracle/mpf_oracle.c).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path in tests/ and
__graft_entry__.smoke(), and the timed CPU baseline of bench.py.  Nothing in
the product imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmpf_oracle.so")

STOP = {"redshift": 0, "r": 1, "radius": 1, "lambda": 2, "t": 3, "eta": 3, "a": 4, "plane": 5, "s": 6}
PHOTON_FIELDS = ("a t x y z dtdl dxdl dydl dzdl level ah rho phi dphidx dphidy dphidz dphidt dphidl "
                 "laplacian redshift dsdl2 error isw iswold chi lambda s index").split()
PLANE_FIELDS = ("firstid f x y z distance A11 A12 A22 t a redshift chi lambda s isw rho phi rho_max "
                "valid").split()

_lib = None
_p = C.c_void_p
_i64 = C.c_int64
_d = C.c_double


SOURCES = ("mpf_oracle.c", "mpf_oracle_cells.c")
HEADERS = ("mpf_oracle.h", "mpf_oracle_keys.h")


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/ (no FMA contraction)."""
    srcs = [os.path.join(HERE, f) for f in SOURCES]
    newest = max(os.path.getmtime(os.path.join(HERE, f)) for f in SOURCES + HEADERS)
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < newest:
        os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
        tmp = LIB_PATH + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O3", "-std=gnu11", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp] + srcs + ["-lm", "-lpthread"])
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


class _Velocity(C.Structure):
    _fields_ = [("v", _p), ("vobs", _d * 3)]


class _Tree(C.Structure):
    _fields_ = [("n", _i64), ("keys", _p), ("fields", _p), ("vel", C.POINTER(_Velocity))]


class _Cosmo(C.Structure):
    _fields_ = [("n", _i64), ("t", _p), ("a", _p), ("dadt", _p)]


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.mpfo_locate.restype = _i64
        L.mpfo_locate.argtypes = [_p, _d, _d, _d]
        L.mpfo_cic.argtypes = [_p, _d, _d, _d, _p]
        L.mpfo_tsc.argtypes = [_p, _d, _d, _d, _p]
        L.mpfo_interpolate.restype = _d
        L.mpfo_interpolate.argtypes = [_d, _p, _p, _i64]
        L.mpfo_key_compute.argtypes = [C.c_uint, _d, _d, _d, _p]
        L.mpfo_propagate.restype = C.c_int
        L.mpfo_propagate.argtypes = [_p, _p, C.c_int, _d, C.c_uint, C.c_int, _d, _p, _i64, _p, C.c_int, _p,
                                     C.c_int, _p, _p, _p, C.c_int]
        L.mpfo_trajectory.restype = _i64
        L.mpfo_trajectory.argtypes = [_p, _p, C.c_int, _d, C.c_uint, C.c_int, _d, _p, _p, _i64]
        L.mpfo_propagate_bundle.restype = _i64
        L.mpfo_propagate_bundle.argtypes = [_p, _p, C.c_int, _d, C.c_uint, _p, C.c_uint, _d, _d, C.c_int, _d, _p, _i64]
        L.mpfo_bundle.restype = C.c_int
        L.mpfo_bundle.argtypes = [_p, _p, C.c_int, _d, C.c_uint, C.c_int, _i64, _p, C.c_int, _p, C.c_int, C.c_int, _d,
                                  _p, _p, C.c_int]
        L.mpfo_catalogue_jac.restype = C.c_int
        L.mpfo_catalogue_jac.argtypes = [_p, _p, C.c_int, _d, C.c_uint, _i64, _p, _p, _p, _d, _d, _d, C.c_int,
                                         C.c_int, C.c_int, C.c_int, _d, _p, C.c_int]
        L.mpfo_born.restype = C.c_int
        L.mpfo_born.argtypes = [_p, _p, _d, C.c_uint, C.c_int, _d, _i64, _p, C.c_int, _p, _p, _p]
        L.mpfo_catalogue.restype = C.c_int
        L.mpfo_catalogue.argtypes = [_p, _p, C.c_int, _d, C.c_uint, _i64, _p, _p, _p, _d, _d, _d, C.c_int, _p,
                                     C.c_int]
        L.mpfo_velocity_deposit.restype = C.c_int
        L.mpfo_velocity_deposit.argtypes = [_p, _p, _p, C.c_int, _i64, _p, _p, C.c_int]
        for f in ("mpfo_batch_locate", "mpfo_batch_cic", "mpfo_batch_tsc", "mpfo_batch_ngp"):
            getattr(L, f).argtypes = [_p, _i64, _p, _p, C.c_int]
        L.mpfo_cells_parse.restype = _i64
        L.mpfo_cells_parse.argtypes = [C.c_char_p, _i64, _p, _i64]
        L.mpfo_cells_build.restype = _i64
        L.mpfo_cells_build.argtypes = [_p, _i64, _p, _p, _p, _i64, _p, _p]
        _lib = L
    return _lib


class _CellsParams(C.Structure):
    _fields_ = [("cone_vertex", _d * 3), ("cone_base", _d * 3), ("cone_angle", _d), ("sphere_center", _d * 3),
                ("sphere_radius", _d), ("rotm1", _p), ("h", _d), ("lboxmpch", _d), ("mpc", _d),
                ("coarseonly", C.c_int), ("ncoarse", C.c_int), ("correction", C.c_int),
                ("coarsecorrection", C.c_int), ("acorrection", C.c_int), ("order", C.c_int),
                ("completion_waves", C.c_int)]


def cells_parse(text: str) -> np.ndarray:
    """The reference's ASCII cell reads: rows of 10 floats."""
    L = lib()
    raw = text.encode()
    n = L.mpfo_cells_parse(raw, len(raw), None, 0)
    if n < 0:
        raise ValueError("malformed cell rows")
    rows = np.zeros((n, 10), dtype=np.float32)
    L.mpfo_cells_parse(raw, len(raw), _ptr(rows), n)
    return rows


def cells_build(rows, cosmo: dict, cone7, sphere4, h: float, lboxmpch: float, mpc: float, order: int = 2,
                correction: bool = True, coarsecorrection: bool = True, acorrection: bool = False, rotm1=None,
                coarseonly: bool = False, ncoarse: int = 0, completion_waves: int = 0):
    """Create_octree's per-cone build (importascii + correctOctree) on the CPU:
    (48-byte records as uint8, amin or None, completion info dict)."""
    L = lib()
    rows = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, 10)
    p = _CellsParams()
    for d in range(3):
        p.cone_vertex[d], p.cone_base[d], p.sphere_center[d] = cone7[d], cone7[3 + d], sphere4[d]
    p.cone_angle, p.sphere_radius = float(cone7[6]), float(sphere4[3])
    rot = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64).reshape(9)
    p.rotm1 = rot.ctypes.data if rot is not None else None
    p.h, p.lboxmpch, p.mpc = float(h), float(lboxmpch), float(mpc)
    p.coarseonly, p.ncoarse = int(bool(coarseonly)), int(ncoarse)
    p.correction, p.coarsecorrection, p.acorrection = int(bool(correction)), int(bool(coarsecorrection)), int(bool(acorrection))
    p.order, p.completion_waves = int(order), int(completion_waves)
    a = np.ascontiguousarray(cosmo["a"], dtype=np.float64)
    dadt = np.ascontiguousarray(cosmo["dadt"], dtype=np.float64)
    t = np.ascontiguousarray(cosmo.get("t", cosmo["a"]), dtype=np.float64)
    cs = _Cosmo(a.shape[0], t.ctypes.data, a.ctypes.data, dadt.ctypes.data)
    amin = np.full(1, np.nan)
    info = np.zeros(4, dtype=np.int64)
    cap = 2 * rows.shape[0] + 64
    out = np.zeros(cap * 48, dtype=np.uint8)
    n = L.mpfo_cells_build(_ptr(rows), rows.shape[0], C.byref(p), C.byref(cs), _ptr(out), cap, _ptr(amin), _ptr(info))
    if n > cap:
        cap = n
        out = np.zeros(cap * 48, dtype=np.uint8)
        n = L.mpfo_cells_build(_ptr(rows), rows.shape[0], C.byref(p), C.byref(cs), _ptr(out), cap, _ptr(amin),
                               _ptr(info))
    if n < 0:
        raise RuntimeError("mpfo_cells_build failed (%d)" % n)
    return (out[:48 * n].copy(), None if np.isnan(amin[0]) else float(amin[0]),
            {"incomplete": int(info[0]), "in_waves": int(info[1]), "waves": int(info[2]), "sequential": int(info[3])})


def _ptr(a):
    return a.ctypes.data_as(_p)


def fields7(records: np.ndarray) -> np.ndarray:
    """7-float rows (rho phi dphidx dphidy dphidz a dphidt) of 48-B records."""
    return np.stack([records[k] for k in ("rho", "phi", "dphidx", "dphidy", "dphidz", "a", "dphidt")],
                    axis=1).astype(np.float32)


class Oracle:
    def __init__(self, records: np.ndarray, cosmo: dict, length: float, nthreads: int = 0):
        self.keys = np.ascontiguousarray(np.stack([records["hi"], records["lo"]], axis=1).astype(np.uint64))
        self.fields = np.ascontiguousarray(fields7(records))
        self.tree = _Tree(records.shape[0], _ptr(self.keys), _ptr(self.fields))
        self.t = np.ascontiguousarray(cosmo["t"], dtype=np.float64)
        self.a = np.ascontiguousarray(cosmo["a"], dtype=np.float64)
        self.dadt = np.ascontiguousarray(cosmo["dadt"], dtype=np.float64)
        self.cosmo = _Cosmo(self.t.shape[0], _ptr(self.t), _ptr(self.a), _ptr(self.dadt))
        self.length = float(length)
        self.nthreads = nthreads or (os.cpu_count() or 1)
        self.L = lib()
        self.vel = None

    # -- velocity field (the reference's -DVELOCITYFIELD build) --
    def set_velocity(self, v3, vobs=(0.0, 0.0, 0.0)):
        """Trace as the velocity-field build: per-cell velocities v3 (n x 3)
        and the observer velocity; v3 = None goes back to the plain build."""
        if v3 is None:
            self.vel = None
            self.tree.vel = C.POINTER(_Velocity)()
            return
        self.vel = np.ascontiguousarray(v3, dtype=np.float32).reshape(-1, 3)
        self._velstruct = _Velocity(_ptr(self.vel), (_d * 3)(*[float(x) for x in vobs]))
        self.tree.vel = C.pointer(self._velstruct)

    def set_vobs(self, vobs):
        if self.vel is None:
            raise ValueError("no velocity field")
        for k in range(3):
            self._velstruct.vobs[k] = float(vobs[k])

    def deposit_velocity(self, pos, vel, scheme="cic", begin=True, finish=True):
        """Hmaps::CreateOctreeVelocityWithCIC / WithTSC on one thread, with the
        zeroed masses before and the normalisation and parent fill after; the
        oracle's rho and velocity field change in place."""
        if self.vel is None:
            self.set_velocity(np.zeros((self.keys.shape[0], 3), dtype=np.float32))
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
        flags = (1 if begin else 0) | (2 if finish else 0)
        sch = {"cic": 1, "tsc": 2}[scheme] if isinstance(scheme, str) else int(scheme)
        rc = self.L.mpfo_velocity_deposit(C.byref(self.tree), _ptr(self.fields), _ptr(self.vel), sch, p.shape[0],
                                          _ptr(p), _ptr(v), flags)
        if rc != 0:
            raise ValueError("oracle deposit failed: %d" % rc)
        return self.vel, self.fields[:, 0]

    def locate(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros(xyz.shape[0], dtype=np.int64)
        self.L.mpfo_batch_locate(C.byref(self.tree), xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def cic(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.mpfo_batch_cic(C.byref(self.tree), xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def tsc(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.mpfo_batch_tsc(C.byref(self.tree), xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def ngp(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.mpfo_batch_ngp(C.byref(self.tree), xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def propagate(self, launch, order=2, nsteps=10, stop="redshift", stop_ref=0.5, planes=None, jacobian=True,
                  ki_target=None, nthreads=None):
        launch = np.ascontiguousarray(launch, dtype=np.float64)
        n = launch.shape[0]
        pl = np.ascontiguousarray(planes if planes is not None else np.zeros(0), dtype=np.float64)
        npl = pl.shape[0]
        steps = np.zeros(n, dtype=np.int64)
        final = np.zeros((n, 28))
        pout = np.zeros((n, max(npl, 1), 20))
        ki = np.ascontiguousarray(ki_target if ki_target is not None else np.zeros(3), dtype=np.float64)
        rc = self.L.mpfo_propagate(C.byref(self.tree), C.byref(self.cosmo), order, self.length, nsteps,
                                   STOP[stop], stop_ref, _ptr(ki), n, _ptr(launch), npl,
                                   _ptr(pl) if npl else None, int(bool(jacobian)), _ptr(steps), _ptr(final),
                                   _ptr(pout), int(nthreads or self.nthreads))
        if rc != 0:
            raise ValueError("oracle propagate failed: %d" % rc)
        return steps, final, pout[:, :npl]

    def trajectory(self, launch, order=2, nsteps=10, stop="redshift", stop_ref=0.5, cap=200000):
        L = np.ascontiguousarray(launch, dtype=np.float64)
        out = np.zeros((cap, 28))
        m = self.L.mpfo_trajectory(C.byref(self.tree), C.byref(self.cosmo), order, self.length, nsteps,
                                   STOP[stop], stop_ref, _ptr(L), _ptr(out), cap)
        return out[:min(m, cap)]

    def propagate_bundle(self, photon, count, angle, rotation=0.0, interp="redshift", amin=0.0, order=2, nsteps=10,
                         cap=100000):
        """Integrator::propagate: photon = start xyz + direction as launched.
        Returns the central trajectory (m x 29, file column order); empty when rejected."""
        ph = np.ascontiguousarray(photon, dtype=np.float64)
        out = np.zeros((cap, 29))
        m = self.L.mpfo_propagate_bundle(C.byref(self.tree), C.byref(self.cosmo), order, self.length, nsteps, _ptr(ph),
                                         int(count), float(angle), float(rotation), STOP.get(interp, 0), float(amin),
                                         _ptr(out), cap)
        return out[:min(m, cap)]

    def catalogue(self, sources, order=2, nsteps=10, cat_accuracy=1e-8, h=0.68, mpc=3.08568e22,
                  vobs=(0.0, 0.0, 0.0), rotm1=None, max_iterations=10, nthreads=None, jacobiantype="infinitesimal",
                  plane="normal", stop_bundle="r", openingmin=0.0):
        """relCat rows (n x 16) for sources (n x 6: x y z vx vy vz)."""
        src = np.ascontiguousarray(np.asarray(sources)[:, :6], dtype=np.float64)
        vo = np.ascontiguousarray(vobs, dtype=np.float64)
        rot = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64).reshape(9)
        out = np.zeros((src.shape[0], 16))
        rc = self.L.mpfo_catalogue_jac(C.byref(self.tree), C.byref(self.cosmo), order, self.length, nsteps,
                                       src.shape[0], _ptr(src), _ptr(rot) if rot is not None else None, _ptr(vo),
                                       float(cat_accuracy), float(h), float(mpc), int(max_iterations),
                                       {"bundle": 1, "infinitesimal_born": 2}.get(jacobiantype, 0),
                                       1 if plane == "sachs" else 0,
                                       STOP[stop_bundle], float(openingmin), _ptr(out), int(nthreads or self.nthreads))
        if rc != 0:
            raise ValueError("oracle catalogue failed: %d" % rc)
        return out

    def born(self, launch, dist, nsteps=10, stop="redshift", stop_ref=0.5):
        """FillMap's lensing_born rays: (Born trajectory sizes n, Jacobians n x nd x 3)."""
        launch = np.ascontiguousarray(launch, dtype=np.float64)
        dist = np.ascontiguousarray(dist, dtype=np.float64)
        n = launch.shape[0]
        size = np.zeros(n, dtype=np.int64)
        A = np.zeros((n, dist.shape[0], 3))
        rc = self.L.mpfo_born(C.byref(self.tree), C.byref(self.cosmo), self.length, nsteps, STOP[stop], float(stop_ref),
                              n, _ptr(launch), dist.shape[0], _ptr(dist), _ptr(size), _ptr(A))
        if rc != 0:
            raise ValueError("oracle born failed: %d" % rc)
        return size, A

    def bundle(self, launch, planes, order=2, nsteps=10, stop="redshift", plane="sachs", stop_bundle="redshift",
               openingmin=0.0, nthreads=None):
        """FillMap with the bundle Jacobian: (surface records n x np x 20, Jacobians n x np x 4)."""
        launch = np.ascontiguousarray(launch, dtype=np.float64)
        pl = np.ascontiguousarray(planes, dtype=np.float64)
        n, npl = launch.shape[0], pl.shape[0]
        pout = np.zeros((n, npl, 20))
        jac = np.zeros((n, npl, 4))
        rc = self.L.mpfo_bundle(C.byref(self.tree), C.byref(self.cosmo), order, self.length, nsteps, STOP[stop], n,
                                _ptr(launch), npl, _ptr(pl), 1 if plane == "sachs" else 0, STOP[stop_bundle],
                                float(openingmin), _ptr(pout), _ptr(jac), int(nthreads or self.nthreads))
        if rc != 0:
            raise ValueError("oracle bundle failed: %d" % rc)
        return pout, jac
