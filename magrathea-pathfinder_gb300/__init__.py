"""GB300 photon-propagation path of Magrathea-Pathfinder (host-side mirror).

The compute runs in libmpf_gb300.so (CUDA, sm_103a) through its C ABI
(include/mpf_gb300.h); this module mirrors the reference's interface for the
path:

==========================  ==================================================
reference                   here
==========================  ==================================================
Input::load / loadOctree    ``Octree.load(path)`` / ``Octree.from_records``
SimpleHyperOctree::locate   ``Octree.locate(xyz)``
SimpleHyperOctree::cic/tsc  ``Octree.cic(xyz)`` / ``Octree.tsc(xyz)``
Input::acquire+correct      ``Cosmology(t, a, dadt, d2adt2)`` (the table)
Integrator::integrate       ``propagate(...)`` (batched over rays), with
 + Lensing::dbetadtheta_     the infinitesimal Jacobian and FillMap's
   infinitesimal            per-surface values at each surface
Catalogues::relCat /        ``catalogue(...)``: the Newton root-finder for a
  iterateNewtonMethod       batch of sources, relCat's 16-column rows
Hmaps::FillMap              ``hmaps_fill(...)``: pixels in, float map rows out
create_octree (ASCII)       ``cells_parse`` + ``cells_build``: cell rows in,
 importascii+correctOctree   sorted 48-byte cone records out
Integrator::propagate       ``rays_propagate(...)``: the rays driver's bundles
 (rays)                      and the central ray's angular diameter distance
pix2vec_ring                ``pix2vec_ring(nside, pixels)`` (device)
==========================  ==================================================
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .capi import MPF_PHOTON_FIELDS, MPF_PLANE_FIELDS, MpfError

PHOTON_FIELDS = ("a t x y z dtdl dxdl dydl dzdl level ah rho phi dphidx dphidy dphidz dphidt dphidl "
                 "laplacian redshift dsdl2 error isw iswold chi lambda s index").split()
PLANE_FIELDS = ("firstid f x y z distance A11 A12 A22 t a redshift chi lambda s isw rho phi rho_max "
                "valid").split()

CATALOGUE_FIELDS = ("phi theta phi_obs theta_obs miss iterations z_flrw z_pot z_dopp z_tdopp z_isw z_gr "
                    "a11 a12 a21 a22").split()

__all__ = ["Octree", "Cosmology", "propagate", "rays_propagate", "catalogue", "hmaps_fill", "pix2vec_ring", "autotune_info",
           "MpfError", "PHOTON_FIELDS", "PLANE_FIELDS",
           "CATALOGUE_FIELDS", "library"]


def library():
    """The loaded native library (raises ImportError if it is not built)."""
    return capi.load()


class Octree:
    """Device octree (cone records sorted by 128-bit key)."""

    def __init__(self, handle):
        self._h = handle
        self._lib = capi.load()

    @classmethod
    def from_records(cls, records: np.ndarray) -> "Octree":
        L = capi.load()
        rec = np.ascontiguousarray(records)
        if rec.dtype.itemsize != 48:
            raise ValueError("records must be 48-byte cone records")
        h = C.c_void_p()
        capi.check(L.mpf_octree_upload(capi.ptr(rec), rec.shape[0], C.byref(h)))
        return cls(h)

    @classmethod
    def load(cls, path: str) -> "Octree":
        L = capi.load()
        h = C.c_void_p()
        capi.check(L.mpf_octree_load(path.encode(), C.byref(h)))
        return cls(h)

    @property
    def info(self) -> dict:
        i = capi.OctreeInfo()
        capi.check(self._lib.mpf_octree_get_info(self._h, C.byref(i)))
        return dict(cells=i.cells, nodes=i.nodes, level_min=i.level_min, level_max=i.level_max,
                    top_level=i.top_level, grid=tuple(i.grid), device_bytes=i.device_bytes)

    def locate(self, xyz) -> np.ndarray:
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        out = np.zeros(xyz.shape[0], dtype=np.int64)
        capi.check(self._lib.mpf_locate(self._h, xyz.shape[0], capi.ptr(xyz), capi.ptr(out)))
        return out

    def _interp(self, order, xyz, exact):
        xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1, 3)
        out = np.zeros((xyz.shape[0], 7), dtype=np.float32)
        capi.check(self._lib.mpf_interpolate(self._h, order, int(bool(exact)), xyz.shape[0], capi.ptr(xyz),
                                             capi.ptr(out)))
        return out

    def cic(self, xyz, exact: bool = True) -> np.ndarray:
        """rho phi dphidx dphidy dphidz a dphidt at each position."""
        return self._interp(1, xyz, exact)

    def tsc(self, xyz, exact: bool = True) -> np.ndarray:
        return self._interp(2, xyz, exact)

    def ngp(self, xyz) -> np.ndarray:
        """The containing cell's record (the reference's ORDER = 0)."""
        return self._interp(0, xyz, True)

    # -- velocity field (the reference's -DVELOCITYFIELD build) --
    def set_velocity(self, v3, rho=None):
        """Attach per-cell velocities (n x 3, record order; None removes the
        field); rho (n) replaces the cells' rho when given."""
        n = self.info["cells"]
        if v3 is None:
            capi.check(self._lib.mpf_octree_set_velocity(self._h, None, None))
            return
        v = np.ascontiguousarray(v3, dtype=np.float32).reshape(n, 3)
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float32).reshape(n)
        capi.check(self._lib.mpf_octree_set_velocity(self._h, capi.ptr(v), capi.ptr(r)))

    def velocity(self):
        """(velocities n x 3, rho n) of the cells."""
        n = self.info["cells"]
        v = np.zeros((n, 3), dtype=np.float32)
        r = np.zeros(n, dtype=np.float32)
        capi.check(self._lib.mpf_octree_get_velocity(self._h, capi.ptr(v), capi.ptr(r)))
        return v, r

    def deposit_velocity(self, pos, vel, scheme="cic", begin=True, finish=True):
        """Hmaps::CreateOctreeVelocityWithCIC / WithTSC of particles (n x 3
        positions in octree units, n x 3 velocities), with the zeroed masses
        before (begin) and the mass normalisation and parent fill after
        (finish)."""
        p = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
        v = np.ascontiguousarray(vel, dtype=np.float32).reshape(-1, 3)
        if p.shape != v.shape:
            raise ValueError("pos and vel must have the same shape")
        flags = (capi.MPF_VELOCITY_BEGIN if begin else 0) | (capi.MPF_VELOCITY_FINISH if finish else 0)
        sch = {"cic": 1, "tsc": 2}[scheme] if isinstance(scheme, str) else int(scheme)
        capi.check(self._lib.mpf_velocity_deposit(self._h, sch, p.shape[0], capi.ptr(p), capi.ptr(v), flags))

    def deposit_velocity_device(self, pos_ptr, vel_ptr, n, scheme="cic", begin=True, finish=True, stream=None):
        """The same with the particles in device memory (pointers to n x 3
        floats each), on a CUDA stream handle (None: the legacy default)."""
        flags = (capi.MPF_VELOCITY_BEGIN if begin else 0) | (capi.MPF_VELOCITY_FINISH if finish else 0)
        sch = {"cic": 1, "tsc": 2}[scheme] if isinstance(scheme, str) else int(scheme)
        capi.check(self._lib.mpf_velocity_deposit_device(self._h, sch, int(n), capi.ptr(pos_ptr), capi.ptr(vel_ptr),
                                                         flags, capi.ptr(stream)))

    def deposit_pairs(self) -> int:
        """(cell, particle, vertex) pairs the last deposit sorted."""
        k = C.c_int64()
        capi.check(self._lib.mpf_velocity_deposit_pairs(self._h, C.byref(k)))
        return k.value

    def close(self):
        if self._h:
            self._lib.mpf_octree_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cosmology:
    """Conformal time / scale factor table on the device."""

    def __init__(self, t, a, dadt, d2adt2=None):
        L = capi.load()
        self._arr = [np.ascontiguousarray(v, dtype=np.float64) for v in
                     (t, a, dadt, d2adt2 if d2adt2 is not None else np.zeros(len(t)))]
        h = C.c_void_p()
        capi.check(L.mpf_cosmology_upload(*[capi.ptr(v) for v in self._arr], self._arr[0].shape[0], C.byref(h)))
        self._h = h
        self._lib = L

    def close(self):
        if self._h:
            self._lib.mpf_cosmology_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def propagate(octree: Octree, cosmology: Cosmology, launch, length: float, nsteps: int = 10, order: int = 2,
              stop: str = "redshift", stop_value: float = 0.0, planes=None, jacobian: bool = True,
              exact: bool = False, max_steps: int = 0, plane_normal=(0.0, 0.0, 0.0), want_final: bool = True,
              vobs=(0.0, 0.0, 0.0)):
    """Integrate rays launched from launch[:, 0:3] toward launch[:, 3:6].

    vobs: the observer velocity, read when the octree carries a velocity field.
    Returns (steps[n], final[n, 28] or None, planes[n, nplanes, 20] or None, status).
    """
    L = capi.load()
    launch = np.ascontiguousarray(launch, dtype=np.float64).reshape(-1, 6)
    n = launch.shape[0]
    p, keep = capi.make_params(length, nsteps, order, stop, stop_value, planes, jacobian, exact, max_steps,
                               plane_normal, vobs)
    steps = np.zeros(n, dtype=np.int64)
    final = np.zeros((n, MPF_PHOTON_FIELDS)) if want_final else None
    np_ = p.nplanes
    pout = np.zeros((n, np_, MPF_PLANE_FIELDS)) if np_ > 0 else None
    rc = L.mpf_propagate(octree._h, cosmology._h, C.byref(p), n, capi.ptr(launch), capi.ptr(steps),
                         capi.ptr(final), capi.ptr(pout))
    capi.check(rc)
    del keep
    return steps, final, pout, rc


def propagate_accuracy(octree: Octree, cosmology: Cosmology, launch, length: float, sample: int = 256,
                       nsteps: int = 10, order: int = 2, stop: str = "redshift", stop_value: float = 0.0, planes=None,
                       jacobian: bool = True, max_steps: int = 0, plane_normal=(0.0, 0.0, 0.0), vobs=(0.0, 0.0, 0.0)):
    """Errors of the FP32-gather kernel against the float64 kernel (the
    reference's operation order) on `sample` rays of the batch, as a dict in
    the layout of accuracy.compare()."""
    L = capi.load()
    launch = np.ascontiguousarray(launch, dtype=np.float64).reshape(-1, 6)
    p, keep = capi.make_params(length, nsteps, order, stop, stop_value, planes, jacobian, False, max_steps,
                               plane_normal, vobs)
    a = capi.Accuracy()
    capi.check(L.mpf_propagate_accuracy(octree._h, cosmology._h, C.byref(p), launch.shape[0], capi.ptr(launch),
                                        int(sample), C.byref(a)))
    del keep
    out = {"rays": a.rays, "step_count_differs": a.step_count_differs, "max_step_diff": a.max_step_diff,
           "deflection_rel": {"max": a.deflection_rel_max, "median": a.deflection_rel_median},
           "redshift_rel": {"max": a.redshift_rel_max, "median": a.redshift_rel_median},
           "surface_valid_differs": a.surface_valid_differs}
    if p.nplanes:
        for q, name in enumerate(("kappa", "gamma1", "gamma2", "inv_mu")):
            out[name] = {"abs_max": a.lensing_abs_max[q], "scale": a.lensing_scale[q],
                         "of_scale": a.lensing_abs_max[q] / max(a.lensing_scale[q], 1e-300)}
    return out


def rays_propagate(octree: Octree, cosmology: Cosmology, photons, length: float, count: int, angle: float,
                   rotation=None, interpolation: str = "redshift", amin: float = 0.0, nsteps: int = 10, order: int = 2,
                   exact: bool = False, capacity: int = 20000, max_steps: int = 0, homogeneous_level: int = -1):
    """Integrator::propagate for n central photons (the rays driver's bundles).

    photons[n, 6]: start x y z and the launch direction (not renormalised);
    rotation[n]: the circle's rotation (None: 0).  Returns (sizes[n],
    central[n, capacity, 29]): each central trajectory in the trajectory
    file's column order with its angular diameter distance; size 0 when the
    bundle is rejected.  homogeneous_level >= 0: the FLRW reference bundle
    (the homogeneous field on a uniform octree of that level; the octree
    argument is not read).
    """
    L = capi.load()
    ph = np.ascontiguousarray(photons, dtype=np.float64).reshape(-1, 6)
    n = ph.shape[0]
    rot = None if rotation is None else np.ascontiguousarray(rotation, dtype=np.float64).reshape(n)
    p, keep = capi.make_params(length, nsteps, order, "r", 0.0, None, False, exact, max_steps)
    bp = capi.BundleParams()
    bp.count, bp.angle, bp.amin, bp.capacity = int(count), float(angle), float(amin), int(capacity)
    bp.interpolation = capi.STOP.get(interpolation, 0)
    bp.homogeneous_level = int(homogeneous_level)
    sizes = np.zeros(n, dtype=np.int64)
    central = np.zeros((n, int(capacity), capi.MPF_TRAJECTORY_FIELDS))
    capi.check(L.mpf_rays_propagate(octree._h, cosmology._h, C.byref(p), C.byref(bp), n, capi.ptr(ph), capi.ptr(rot),
                                    capi.ptr(sizes), capi.ptr(central)))
    del keep
    return sizes, central


def cells_parse(text) -> np.ndarray:
    """ASCII cell rows (level x y z rho phi fx fy fz a) read as the reference
    reads them (an unsigned level, then floats): float32 array n x 10."""
    L = capi.load()
    raw = text.encode() if isinstance(text, str) else bytes(text)
    n = C.c_int64()
    L.mpf_cells_parse(raw, len(raw), None, 0, C.byref(n))
    rows = np.zeros((n.value, 10), dtype=np.float32)
    capi.check(L.mpf_cells_parse(raw, len(raw), capi.ptr(rows), n.value, C.byref(n)))
    return rows


def cells_build(rows, cosmology: Cosmology, cone_vertex, cone_base, cone_angle, sphere_center, sphere_radius,
                h: float, omegam: float, lboxmpch: float, mpc: float = 3.08568e22, rotm1=None, coarseonly: bool = False,
                ncoarse: int = 0, coarsecorrection: bool = True, order: int = 2, correction: bool = True,
                acorrection: bool = False):
    """create_octree's per-cone build (importascii + correctOctree) on the
    device: the 48-byte cone records, sorted by key, as a uint8 array.
    correction: refined cells' non-normal dphidt / rho from their parent and
    incomplete octs completed (True), or the parents of refined cells with a
    non-normal rho and the incomplete octs coarsened (False).  acorrection:
    the scale factors snapped to their table (Full Universe Run); then the
    result is (records, amin)."""
    L = capi.load()
    rows = np.ascontiguousarray(rows, dtype=np.float32).reshape(-1, 10)
    p = capi.CellsParams()
    for d in range(3):
        p.cone_vertex[d], p.cone_base[d], p.sphere_center[d] = cone_vertex[d], cone_base[d], sphere_center[d]
    p.cone_angle, p.sphere_radius = float(cone_angle), float(sphere_radius)
    rot = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64).reshape(9)
    p.rotm1 = rot.ctypes.data if rot is not None else None
    p.h, p.omegam, p.lboxmpch, p.mpc = float(h), float(omegam), float(lboxmpch), float(mpc)
    p.coarseonly, p.ncoarse, p.correction, p.coarsecorrection = int(bool(coarseonly)), int(ncoarse), int(bool(correction)), int(bool(coarsecorrection))
    amin = np.zeros(1)
    p.acorrection, p.order, p.amin = int(bool(acorrection)), int(order), amin.ctypes.data
    cap = 2 * rows.shape[0] + 64
    out = np.zeros(cap * 48, dtype=np.uint8)
    n = C.c_int64()
    rc = L.mpf_cells_build(capi.ptr(rows), rows.shape[0], C.byref(p), cosmology._h, capi.ptr(out), cap, C.byref(n))
    if rc == -1 and n.value > cap:   # MPF_BAD_INPUT: more cells than the first guess; build again at the size
        cap = n.value
        out = np.zeros(cap * 48, dtype=np.uint8)
        rc = L.mpf_cells_build(capi.ptr(rows), rows.shape[0], C.byref(p), cosmology._h, capi.ptr(out), cap, C.byref(n))
    capi.check(rc)
    rec = out[:48 * n.value].copy()
    return (rec, float(amin[0])) if acorrection else rec


def cells_completion_info() -> dict:
    """How the calling thread's last cells_build completed its incomplete
    octs: the incomplete cells, the children filled in waves of independent
    gathers, the waves run and the children filled in order after them."""
    L = capi.load()
    info = np.zeros(4, dtype=np.int64)
    capi.check(L.mpf_cells_completion_info(capi.ptr(info)))
    return {"incomplete": int(info[0]), "in_waves": int(info[1]), "waves": int(info[2]), "sequential": int(info[3])}


def catalogue(octree: Octree, cosmology: Cosmology, sources, length: float, h: float, mpc: float = 3.08568e22,
              cat_accuracy: float = 1e-8, nsteps: int = 10, order: int = 2, vobs=(0.0, 0.0, 0.0), rotm1=None,
              exact: bool = False, max_iterations: int = 10, jacobian: str = "infinitesimal", plane: str = "normal",
              stop_bundle: str = "r", openingmin: float = 0.0):
    """Catalogues::relCat for a batch of sources (rows of >= 6 doubles: x y z vx vy vz ...).

    Returns (rows[n, 16] in relCat's column order, stats dict, status).
    """
    L = capi.load()
    src = np.ascontiguousarray(sources, dtype=np.float64)
    if src.ndim != 2 or src.shape[1] < 6:
        raise ValueError("sources must be n x (>= 6)")
    n, stride = src.shape
    p, rot = catalogue_params(length, h, mpc, cat_accuracy, nsteps, order, vobs, rotm1, exact, max_iterations,
                              jacobian, plane, stop_bundle, openingmin)
    rows = np.zeros((n, capi.MPF_CATALOGUE_FIELDS))
    st = capi.CatalogueStats()
    rc = L.mpf_catalogue_newton(octree._h, cosmology._h, C.byref(p), n, capi.ptr(src), stride, capi.ptr(rows),
                                C.byref(st))
    capi.check(rc)
    del rot
    return rows, catalogue_stats(st), rc


def catalogue_params(length, h, mpc=3.08568e22, cat_accuracy=1e-8, nsteps=10, order=2, vobs=(0.0, 0.0, 0.0),
                     rotm1=None, exact=False, max_iterations=10, jacobian="infinitesimal", plane="normal",
                     stop_bundle="r", openingmin=0.0):
    """mpf_catalogue_params plus the rotation array that must outlive the call."""
    p = capi.CatalogueParams()
    p.length, p.h, p.mpc, p.cat_accuracy = float(length), float(h), float(mpc), float(cat_accuracy)
    for k in range(3):
        p.vobs[k] = float(vobs[k])
    rot = None if rotm1 is None else np.ascontiguousarray(rotm1, dtype=np.float64).reshape(9)
    p.rotm1 = rot.ctypes.data if rot is not None else None
    p.nsteps, p.order, p.exact, p.max_iterations = int(nsteps), int(order), int(bool(exact)), int(max_iterations)
    if jacobian not in ("infinitesimal", "bundle", "infinitesimal_born"):
        raise ValueError("jacobian must be infinitesimal, bundle or infinitesimal_born")
    p.jacobian_bundle = 1 if jacobian == "bundle" else 0
    p.jacobian_born = 1 if jacobian == "infinitesimal_born" else 0
    p.plane_sachs = 1 if plane == "sachs" else 0
    p.stop_bundle = capi.STOP[stop_bundle]
    p.openingmin = float(openingmin)
    return p, rot


def catalogue_stats(st) -> dict:
    return dict(rays=st.rays, photon_steps=st.photon_steps, photon_steps_jacobian=st.photon_steps_jacobian,
                iterations=st.iterations, kernel_launches=st.kernel_launches)


def hmaps_fill(octree: Octree, cosmology: Cosmology, nside: int, pixels, surfaces, homogeneous, components,
               length: float, nsteps: int = 10, order: int = 2, stop: str = "redshift", exact: bool = False,
               max_steps: int = 0, jacobian: str = "infinitesimal", plane: str = "sachs",
               stop_bundle: str = "redshift", openingmin: float = 0.0, vobs=(0.0, 0.0, 0.0)):
    """Hmaps::FillMap for the given RING pixels: float maps [nsurfaces, nmaps, npix].

    surfaces: the stop-quantity values of the map surfaces (interpRefvec);
    homogeneous: [nsurfaces, 5] = t, chi, lambda, a, z of the FLRW ray there;
    components: the reference's map component names, in order ("lensing_born":
    the infinitesimal Jacobian along each pixel's FLRW ray);
    jacobian: "infinitesimal" or "bundle" (then plane, stop_bundle and
    openingmin, in radians, as the reference's parameters); vobs: the
    observer velocity (v0x v0y v0z), read when the octree carries a velocity
    field.
    """
    L = capi.load()
    pix = np.ascontiguousarray(pixels, dtype=np.int64)
    comps = [capi.MAP_COMPONENTS[c] for c in components]
    bundle = jacobian == "bundle"
    nm = sum((5 if bundle else 4) if c == 0 else 4 if c == 1 else 2 if c == 13 else 1 for c in comps)
    p, keep = capi.make_params(length, nsteps, order, stop, 0.0, surfaces, True, exact, max_steps, vobs=vobs)
    hom = np.ascontiguousarray(homogeneous, dtype=np.float64).reshape(-1, 5)
    cc = np.ascontiguousarray(comps, dtype=np.int32)
    nz = p.nplanes
    maps = np.zeros((nz, nm, pix.shape[0]), dtype=np.float32)
    if bundle:
        rc = L.mpf_hmaps_fill_bundle(octree._h, cosmology._h, C.byref(p), int(nside), pix.shape[0], capi.ptr(pix),
                                     len(comps), capi.ptr(cc), capi.ptr(hom), 1 if plane == "sachs" else 0,
                                     capi.STOP[stop_bundle], float(openingmin), capi.ptr(maps))
    else:
        rc = L.mpf_hmaps_fill(octree._h, cosmology._h, C.byref(p), int(nside), pix.shape[0], capi.ptr(pix),
                              len(comps), capi.ptr(cc), capi.ptr(hom), capi.ptr(maps))
    capi.check(rc)
    del keep
    return maps


def autotune_info(octree: Octree, kind: str = "propagate", order: int = 2):
    """The autotuned launch shape for this octree: (threads per block, rays per
    lane per work-queue claim, candidates' photon-steps/s), or None before the
    first batch large enough to tune.  kind: "propagate" or "catalogue"."""
    L = capi.load()
    tpb, depth = C.c_int(), C.c_int()
    rates = np.zeros(4)
    capi.check(L.mpf_autotune_info(octree._h, 0 if kind == "propagate" else 1, int(order), C.byref(tpb), C.byref(depth),
                                   capi.ptr(rates)))
    if tpb.value == 0:
        return None
    return tpb.value, depth.value, rates[: 4 if kind == "propagate" else 3].tolist()


def pix2vec_ring(nside: int, pixels) -> np.ndarray:
    """RING pixel centres computed on the device: [n, 3]."""
    L = capi.load()
    pix = np.ascontiguousarray(pixels, dtype=np.int64)
    out = np.zeros((pix.shape[0], 3))
    capi.check(L.mpf_pix2vec_ring(int(nside), pix.shape[0], capi.ptr(pix), capi.ptr(out)))
    return out
