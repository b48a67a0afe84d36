"""ctypes wrapper of the reference harness (oracle/_ref/libref_o{0,1,2}.so, and
libref_vel_o{0,1,2}.so: the reference's velocity-field build, -DVELOCITYFIELD).

Test infrastructure only: used to generate golden fixtures and to pin the
C restatement (oracle/mpf_oracle.c) to the reference in this container.  The
library exists only where the reference sources were available at build time.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIBS = {}

_d = C.c_double
_i64 = C.c_int64
_p = C.c_void_p


def _ptr(a):
    return a.ctypes.data_as(_p)


def _name(order: int, velocity: bool) -> str:
    return os.path.join(HERE, "_ref", ("libref_vel_o%d.so" if velocity else "libref_o%d.so") % order)


def available(order: int = 2, velocity: bool = False) -> bool:
    return os.path.exists(_name(order, velocity))


def lib(order: int = 2, velocity: bool = False):
    if (order, velocity) not in _LIBS:
        path = _name(order, velocity)
        L = C.CDLL(path, mode=C.RTLD_LOCAL)
        L.ref_load.restype = _i64
        L.ref_load.argtypes = [C.c_char_p]
        L.ref_size.restype = _i64
        L.ref_keys.argtypes = [_p]
        L.ref_compute.argtypes = [C.c_uint, _d, _d, _d, _p]
        L.ref_cipher.argtypes = [_d, _d, _d, _p]
        L.ref_key_level.restype = C.c_uint
        L.ref_key_level.argtypes = [C.c_uint64, C.c_uint64]
        L.ref_key_center.restype = _d
        L.ref_key_center.argtypes = [C.c_uint64, C.c_uint64, C.c_uint]
        L.ref_key_containing.restype = C.c_int
        L.ref_key_containing.argtypes = [C.c_uint64] * 4
        L.ref_locate.restype = _i64
        L.ref_locate.argtypes = [_d, _d, _d]
        for f in ("ref_batch_locate", "ref_batch_cic", "ref_batch_tsc", "ref_batch_ngp"):
            getattr(L, f).argtypes = [_i64, _p, _p, C.c_int]
        L.ref_seq_tsc.argtypes = [_i64, _p, _p]
        L.ref_cosmology.restype = _i64
        L.ref_cosmology.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, _p]
        L.ref_cosmology_get.argtypes = [_p, _p, _p, _p]
        L.ref_cosmology_set.argtypes = [_i64, _p, _p, _p, _p, _d]
        L.ref_interpolate.restype = _d
        L.ref_interpolate.argtypes = [_d, C.c_int]
        L.ref_integrate.argtypes = [_i64, _p, C.c_char_p, _d, C.c_uint, C.c_int, _p, _p, _p, _p, C.c_int]
        L.ref_trajectory.restype = _i64
        L.ref_trajectory.argtypes = [_p, C.c_char_p, _d, C.c_uint, _p, _i64]
        L.ref_homogeneous.restype = C.c_int
        L.ref_homogeneous.argtypes = [C.c_int, _p, _p]
        L.ref_fillmap.restype = C.c_int
        L.ref_fillmap.argtypes = [C.c_long, C.c_int, _p, C.c_char_p, C.c_char_p, C.c_uint, _i64, _p, _p, _p]
        L.ref_fillmap_jac.restype = C.c_int
        L.ref_fillmap_jac.argtypes = [C.c_long, C.c_int, _p, C.c_char_p, C.c_char_p, C.c_uint, _i64, _p, _p, _p,
                                      C.c_char_p, C.c_char_p, C.c_char_p, _d]
        L.ref_pix2vec_ring.argtypes = [C.c_long, _i64, _p, _p]
        L.ref_catalogue.argtypes = [_i64, _p, _p, _p, _d, C.c_uint, _d, _d, _p, C.c_int]
        L.ref_catalogue_jac.argtypes = [_i64, _p, _p, _p, _d, C.c_uint, _d, _d, _p, C.c_int, C.c_char_p, C.c_char_p,
                                        C.c_char_p, _d]
        L.ref_propagate_bundle.restype = _i64
        L.ref_propagate_bundle.argtypes = [_p, C.c_uint, _d, _d, C.c_char_p, _d, C.c_uint, _p, _i64, C.c_char_p, _i64]
        L.ref_propagate_bundle_flrw.restype = _i64
        L.ref_propagate_bundle_flrw.argtypes = [_p, C.c_uint, _d, C.c_char_p, C.c_uint, C.c_uint, _p, _i64]
        L.ref_build_cone.restype = _i64
        L.ref_build_cone.argtypes = [C.c_char_p, _p, _p, _p, C.c_uint, C.c_uint, C.c_uint, C.c_uint, C.c_uint, _d, _d, _d,
                                     _d, _p, _i64, _p]
        L.ref_velocityfield.restype = C.c_int
        L.ref_set_vobs.argtypes = [_d, _d, _d]
        if velocity:
            L.ref_velocity_deposit.restype = C.c_int
            L.ref_velocity_deposit.argtypes = [C.c_int, _i64, _p, _p, C.c_int]
            L.ref_velocity_get.argtypes = [_p, _p]
            L.ref_velocity_set.argtypes = [_p, _p]
        _LIBS[(order, velocity)] = L
    return _LIBS[(order, velocity)]


class Reference:
    """The reference's own octree / integrator / map driver, one per ORDER."""

    def __init__(self, order: int = 2, nthreads: int = 0, velocity: bool = False):
        self.L = lib(order, velocity)
        self.velocity_build = velocity
        self.order = order
        self.nthreads = nthreads or (os.cpu_count() or 1)

    def load(self, path: str) -> int:
        n = self.L.ref_load(path.encode())
        if n < 0:
            raise IOError("reference could not load %s" % path)
        return n

    # -- the velocity-field build --
    def set_vobs(self, vobs):
        self.L.ref_set_vobs(*[float(v) for v in vobs])

    def deposit_velocity(self, pos, vel, scheme="cic", begin=True, finish=True):
        """The map driver's particle stage (hmaps.cpp:395-441) on one thread."""
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
        flags = (1 if begin else 0) | (2 if finish else 0)
        rc = self.L.ref_velocity_deposit({"cic": 1, "tsc": 2}[scheme], p.shape[0], _ptr(p), _ptr(v), flags)
        if rc != 0:
            raise RuntimeError("ref_velocity_deposit failed: %d" % rc)

    def velocity(self):
        n = self.L.ref_size()
        v = np.zeros((n, 3), dtype=np.float32)
        r = np.zeros(n, dtype=np.float32)
        self.L.ref_velocity_get(_ptr(v), _ptr(r))
        return v, r

    def set_velocity(self, v3, rho=None):
        v = np.ascontiguousarray(v3, dtype=np.float32)
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float32)
        self.L.ref_velocity_set(_ptr(v), _ptr(r) if r is not None else None)

    def keys(self):
        n = self.L.ref_size()
        out = np.zeros((n, 2), dtype=np.uint64)
        self.L.ref_keys(_ptr(out))
        return out

    def compute(self, level, x, y, z):
        out = np.zeros(2, dtype=np.uint64)
        self.L.ref_compute(level, x, y, z, _ptr(out))
        return int(out[0]), int(out[1])

    def cipher(self, x, y, z):
        out = np.zeros(2, dtype=np.uint64)
        self.L.ref_cipher(x, y, z, _ptr(out))
        return int(out[0]), int(out[1])

    def locate(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros(xyz.shape[0], dtype=np.int64)
        self.L.ref_batch_locate(xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def ngp(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.ref_batch_ngp(xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def cic(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.ref_batch_cic(xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def tsc(self, xyz):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        self.L.ref_batch_tsc(xyz.shape[0], _ptr(xyz), _ptr(out), self.nthreads)
        return out

    def cosmology(self, celldir, paramfile, evolfile):
        hol = np.zeros(4)
        n = self.L.ref_cosmology(celldir.encode(), paramfile.encode(), evolfile.encode(), _ptr(hol))
        if n < 0:
            raise RuntimeError("reference cosmology failed")
        t, a, dadt, d2 = (np.zeros(n) for _ in range(4))
        self.L.ref_cosmology_get(_ptr(t), _ptr(a), _ptr(dadt), _ptr(d2))
        return dict(t=t, a=a, dadt=dadt, d2adt2=d2, h=hol[0], omega_m=hol[1], lbox=hol[2], length=hol[3])

    def set_cosmology(self, t, a, dadt, d2adt2, length):
        arrs = [np.ascontiguousarray(v, dtype=np.float64) for v in (t, a, dadt, d2adt2)]
        self.L.ref_cosmology_set(arrs[0].shape[0], *[_ptr(v) for v in arrs], float(length))
        self._keep = arrs

    def integrate(self, launch, stop="redshift", stop_ref=0.5, nsteps=10, dists=None):
        launch = np.ascontiguousarray(launch, dtype=np.float64)
        n = launch.shape[0]
        d = np.ascontiguousarray(dists if dists is not None else np.zeros(0), dtype=np.float64)
        nd = d.shape[0]
        steps = np.zeros(n, dtype=np.int64)
        final = np.zeros((n, 28))
        jac = np.zeros((n, max(nd, 1), 4))
        self.L.ref_integrate(n, _ptr(launch), stop.encode(), stop_ref, nsteps, nd, _ptr(d) if nd else None,
                             _ptr(steps), _ptr(final), _ptr(jac), self.nthreads)
        return steps, final, jac[:, :nd]

    def trajectory(self, launch, stop="redshift", stop_ref=0.5, nsteps=10, cap=200000):
        L = np.ascontiguousarray(launch, dtype=np.float64)
        out = np.zeros((cap, 28))
        m = self.L.ref_trajectory(_ptr(L), stop.encode(), stop_ref, nsteps, _ptr(out), cap)
        return out[:min(m, cap)]

    def propagate_bundle(self, launch, count, angle, rotation, interp="redshift", amin=0.0, nsteps=10, cap=100000,
                         text_cap=1 << 24):
        """Integrator::propagate: the central trajectory (m x 29, file column
        order) and its Output::save text; (empty, "") when rejected."""
        L = np.ascontiguousarray(launch, dtype=np.float64)
        out = np.zeros((cap, 29))
        buf = C.create_string_buffer(text_cap)
        m = self.L.ref_propagate_bundle(_ptr(L), int(count), float(angle), float(rotation), interp.encode(), float(amin),
                                        int(nsteps), _ptr(out), cap, buf, text_cap)
        return out[:min(m, cap)], buf.value.decode()

    def propagate_bundle_flrw(self, launch, count, angle, interp="redshift", nsteps=10, level=4, cap=200000):
        """The rays driver's FLRW reference bundle (Order = -1 on a uniform level-`level` octree)."""
        L = np.ascontiguousarray(launch, dtype=np.float64)
        out = np.zeros((cap, 29))
        m = self.L.ref_propagate_bundle_flrw(_ptr(L), int(count), float(angle), interp.encode(), int(nsteps), int(level),
                                             _ptr(out), cap)
        return out[:min(m, cap)]

    def build_cone(self, cellfile, cone7, sphere4, rotm1=None, coarseonly=0, ncoarse=0, correction=1,
                   coarsecorrection=1, acorrection=0, mpc=3.08568e22, h=0.68, omegam=0.31, lboxmpch=2048.0,
                   cap=1 << 22):
        """create_octree for one cone from one ASCII cell file: (48-byte records, amin)."""
        rec = np.zeros(cap * 48, dtype=np.uint8)
        amin = np.zeros(1)
        c7 = np.ascontiguousarray(cone7, dtype=np.float64)
        s4 = np.ascontiguousarray(sphere4, dtype=np.float64)
        rm = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64)
        m = self.L.ref_build_cone(cellfile.encode(), _ptr(c7), _ptr(s4), _ptr(rm) if rm is not None else None,
                                  coarseonly, ncoarse, correction, coarsecorrection, acorrection, mpc, h, omegam,
                                  lboxmpch, _ptr(rec), cap, _ptr(amin))
        return rec[:48 * min(m, cap)].copy(), float(amin[0])

    def homogeneous(self, zs):
        zs = np.ascontiguousarray(zs, dtype=np.float64)
        out = np.zeros((zs.shape[0], 5))
        if self.L.ref_homogeneous(zs.shape[0], _ptr(zs), _ptr(out)) != 0:
            raise RuntimeError("homogeneous quantities failed")
        return out

    def fillmap(self, nside, zs, pixels, stop_ray="redshift", comps="lensing", nsteps=10, jacobiantype="infinitesimal",
                plane="normal", stop_bundle="redshift", openingmin=0.0):
        zs = np.ascontiguousarray(zs, dtype=np.float64)
        pix = np.ascontiguousarray(pixels, dtype=np.int64)
        nmaps_guess = 32
        maps = np.zeros(nmaps_guess * zs.shape[0] * pix.shape[0], dtype=np.float32)
        nm = C.c_int(0)
        rc = self.L.ref_fillmap_jac(nside, zs.shape[0], _ptr(zs), stop_ray.encode(), comps.encode(), nsteps,
                                    pix.shape[0], _ptr(pix), _ptr(maps), C.byref(nm), jacobiantype.encode(),
                                    plane.encode(), stop_bundle.encode(), float(openingmin))
        if rc != 0:
            raise RuntimeError("ref_fillmap failed: %d" % rc)
        return maps[: nm.value * zs.shape[0] * pix.shape[0]].reshape(zs.shape[0], nm.value, pix.shape[0])

    def pix2vec(self, nside, pixels):
        pix = np.ascontiguousarray(pixels, dtype=np.int64)
        out = np.zeros((pix.shape[0], 3))
        self.L.ref_pix2vec_ring(nside, pix.shape[0], _ptr(pix), _ptr(out))
        return out

    def catalogue(self, sources, cat_accuracy=1e-8, nsteps=10, h=0.68, mpc=3.08568e22, vobs=(0.0, 0.0, 0.0), rotm1=None,
                  jacobiantype="infinitesimal", plane="normal", stop_bundle="r", openingmin=0.0):
        """relCat rows (n x 16) for sources (n x 6: x y z vx vy vz)."""
        src = np.ascontiguousarray(sources[:, :6], dtype=np.float64)
        vo = np.ascontiguousarray(vobs, dtype=np.float64)
        rot = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64).reshape(9)
        out = np.zeros((src.shape[0], 16))
        self.L.ref_catalogue_jac(src.shape[0], _ptr(src), _ptr(rot) if rot is not None else None, _ptr(vo),
                                 float(cat_accuracy), int(nsteps), float(h), float(mpc), _ptr(out), self.nthreads,
                                 jacobiantype.encode(), plane.encode(), stop_bundle.encode(), float(openingmin))
        return out
