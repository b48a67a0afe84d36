"""ctypes binding of libmpf_gb300.so (declarations: include/mpf_gb300.h).

The binding loads the in-tree library and fails loudly when it is missing:
there is no CPU fallback on this path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmpf_gb300.so")

MPF_PHOTON_FIELDS = 28
MPF_PLANE_FIELDS = 20
MPF_MAX_PLANES = 16

STATUS = {0: "MPF_OK", 1: "MPF_WARN_MAX_STEPS", -1: "MPF_BAD_INPUT", -2: "MPF_OUT_OF_MEMORY", -3: "MPF_CUDA_ERROR",
          -4: "MPF_NOT_SORTED", -5: "MPF_NO_DEVICE", -6: "MPF_IO_ERROR", -7: "MPF_DEVICE_TIMEOUT"}

STOP = {"redshift": 0, "r": 1, "radius": 1, "lambda": 2, "t": 3, "eta": 3, "a": 4, "plane": 5, "s": 6}

# every symbol include/mpf_gb300.h declares
EXPORTS = ("mpf_version", "mpf_last_error", "mpf_device_count", "mpf_octree_upload", "mpf_octree_load",
           "mpf_octree_get_info", "mpf_octree_destroy", "mpf_cosmology_upload", "mpf_cosmology_destroy", "mpf_locate",
           "mpf_interpolate", "mpf_propagate", "mpf_propagate_device", "mpf_propagate_noalloc",
           "mpf_noalloc_last_error", "mpf_catalogue_newton",
           "mpf_catalogue_newton_device", "mpf_hmaps_fill", "mpf_hmaps_fill_bundle", "mpf_pix2vec_ring",
           "mpf_surrogate_create", "mpf_surrogate_destroy", "mpf_surrogate_train", "mpf_surrogate_sample",
           "mpf_surrogate_get_params", "mpf_surrogate_set_params", "mpf_surrogate_loss_grad", "mpf_surrogate_eval",
           "mpf_surrogate_propagate", "mpf_rays_propagate", "mpf_cells_build", "mpf_cells_parse", "mpf_autotune_info",
           "mpf_octree_set_velocity", "mpf_octree_get_velocity", "mpf_velocity_deposit",
           "mpf_velocity_deposit_device", "mpf_velocity_deposit_pairs", "mpf_propagate_accuracy",
           "mpf_cells_completion_info")

MPF_VELOCITY_BEGIN = 1
MPF_VELOCITY_FINISH = 2

MPF_TRAJECTORY_FIELDS = 29

MPF_SURROGATE_PARAMS = 68112
MPF_SURROGATE_NORM = 274

# map component names (the reference's map_components keys) -> mpf_map_component
MAP_COMPONENTS = {"lensing": 0, "lensing_born": 1, "dr": 2, "dl": 3, "dt": 4, "da": 5, "dz": 6, "ds": 7, "isw": 8, "dens": 9,
                  "dens_max": 10, "steps": 11, "phi": 12, "deflection": 13}

MPF_CATALOGUE_FIELDS = 16


class MpfError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s (%d): %s" % (STATUS.get(code, "?"), code, msg))
        self.code = code


class OctreeInfo(C.Structure):
    _fields_ = [("cells", C.c_int64), ("nodes", C.c_int64), ("level_min", C.c_int), ("level_max", C.c_int),
                ("top_level", C.c_int), ("grid", C.c_int * 3), ("device_bytes", C.c_int64)]


class Params(C.Structure):
    _fields_ = [("length", C.c_double), ("stop_value", C.c_double), ("plane_normal", C.c_double * 3),
                ("planes", C.c_void_p), ("nplanes", C.c_int), ("nsteps", C.c_uint), ("order", C.c_int),
                ("stop", C.c_int), ("jacobian", C.c_int), ("exact", C.c_int), ("max_steps", C.c_int64),
                ("vobs", C.c_double * 3)]


class CatalogueParams(C.Structure):
    _fields_ = [("length", C.c_double), ("h", C.c_double), ("mpc", C.c_double), ("cat_accuracy", C.c_double),
                ("vobs", C.c_double * 3), ("rotm1", C.c_void_p), ("nsteps", C.c_uint), ("order", C.c_int),
                ("exact", C.c_int), ("max_iterations", C.c_int), ("jacobian_bundle", C.c_int),
                ("plane_sachs", C.c_int), ("stop_bundle", C.c_int), ("openingmin", C.c_double),
                ("jacobian_born", C.c_int)]


class CatalogueStats(C.Structure):
    _fields_ = [("rays", C.c_int64), ("photon_steps", C.c_int64), ("photon_steps_jacobian", C.c_int64),
                ("iterations", C.c_int), ("kernel_launches", C.c_int)]


class CellsParams(C.Structure):
    _fields_ = [("cone_vertex", C.c_double * 3), ("cone_base", C.c_double * 3), ("cone_angle", C.c_double),
                ("sphere_center", C.c_double * 3), ("sphere_radius", C.c_double), ("rotm1", C.c_void_p),
                ("h", C.c_double), ("omegam", C.c_double), ("lboxmpch", C.c_double), ("mpc", C.c_double),
                ("coarseonly", C.c_int), ("ncoarse", C.c_int), ("correction", C.c_int), ("coarsecorrection", C.c_int),
                ("acorrection", C.c_int), ("order", C.c_int), ("amin", C.c_void_p)]


class BundleParams(C.Structure):
    _fields_ = [("count", C.c_int), ("angle", C.c_double), ("interpolation", C.c_int), ("amin", C.c_double),
                ("capacity", C.c_int64), ("homogeneous_level", C.c_int)]


class SurrogateDomain(C.Structure):
    _fields_ = [("tan_half", C.c_double * 2), ("r_min", C.c_double), ("r_max", C.c_double), ("a_min", C.c_double),
                ("a_max", C.c_double), ("freq_sigma", C.c_double * 4), ("seed", C.c_uint64)]


class SurrogateTrainParams(C.Structure):
    _fields_ = [("samples", C.c_int64), ("batch", C.c_int64), ("lr", C.c_double), ("stat_samples", C.c_int64)]


class SurrogateTrainStats(C.Structure):
    _fields_ = [("loss_first", C.c_double), ("loss_last", C.c_double), ("steps", C.c_int64), ("seconds", C.c_double),
                ("samples_per_second", C.c_double), ("kernel_launches_per_step", C.c_int)]


class SurrogatePropParams(C.Structure):
    _fields_ = [("tolerance", C.c_double), ("check_every", C.c_int), ("fallback", C.c_int)]


class SurrogatePropStats(C.Structure):
    _fields_ = [("photon_steps", C.c_int64), ("flagged_photons", C.c_int64), ("fallback_photons", C.c_int64),
                ("fallback_steps", C.c_int64), ("surrogate_seconds", C.c_double), ("fallback_seconds", C.c_double)]


_lib = None


class Accuracy(C.Structure):
    _fields_ = [("rays", C.c_int64), ("step_count_differs", C.c_int64), ("max_step_diff", C.c_int64),
                ("deflection_rel_max", C.c_double), ("deflection_rel_median", C.c_double),
                ("redshift_rel_max", C.c_double), ("redshift_rel_median", C.c_double),
                ("surface_valid_differs", C.c_int64), ("lensing_abs_max", C.c_double * 4),
                ("lensing_scale", C.c_double * 4)]


def load(path: str = LIB_PATH):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libmpf_gb300.so not built: run __graft_entry__.build() (or python %s)"
                          % os.path.join(HERE, "build.py"))
    L = C.CDLL(path)
    vp, i64, d = C.c_void_p, C.c_int64, C.c_double
    L.mpf_version.restype = C.c_int
    L.mpf_last_error.restype = C.c_char_p
    L.mpf_device_count.restype = C.c_int
    L.mpf_octree_upload.argtypes = [vp, i64, C.POINTER(vp)]
    L.mpf_octree_load.argtypes = [C.c_char_p, C.POINTER(vp)]
    L.mpf_octree_get_info.argtypes = [vp, C.POINTER(OctreeInfo)]
    L.mpf_octree_destroy.argtypes = [vp]
    L.mpf_octree_destroy.restype = None
    L.mpf_cosmology_upload.argtypes = [vp, vp, vp, vp, i64, C.POINTER(vp)]
    L.mpf_cosmology_destroy.argtypes = [vp]
    L.mpf_cosmology_destroy.restype = None
    L.mpf_locate.argtypes = [vp, i64, vp, vp]
    L.mpf_interpolate.argtypes = [vp, C.c_int, C.c_int, i64, vp, vp]
    L.mpf_propagate.argtypes = [vp, vp, C.POINTER(Params), i64, vp, vp, vp, vp]
    L.mpf_propagate_device.argtypes = [vp, vp, C.POINTER(Params), i64, vp, vp, vp, vp, vp, vp]
    L.mpf_propagate_noalloc.argtypes = [vp, vp, C.POINTER(Params), i64, vp, vp, vp, vp]
    L.mpf_noalloc_last_error.restype = C.c_char_p
    L.mpf_catalogue_newton.argtypes = [vp, vp, C.POINTER(CatalogueParams), i64, vp, i64, vp,
                                       C.POINTER(CatalogueStats)]
    L.mpf_catalogue_newton_device.argtypes = [vp, vp, C.POINTER(CatalogueParams), i64, vp, i64, vp,
                                              C.POINTER(CatalogueStats), vp]
    L.mpf_hmaps_fill.argtypes = [vp, vp, C.POINTER(Params), i64, i64, vp, C.c_int, vp, vp, vp]
    L.mpf_hmaps_fill_bundle.argtypes = [vp, vp, C.POINTER(Params), i64, i64, vp, C.c_int, vp, vp, C.c_int, C.c_int, d,
                                        vp]
    L.mpf_pix2vec_ring.argtypes = [i64, i64, vp, vp]
    L.mpf_octree_set_velocity.argtypes = [vp, vp, vp]
    L.mpf_octree_get_velocity.argtypes = [vp, vp, vp]
    L.mpf_velocity_deposit.argtypes = [vp, C.c_int, i64, vp, vp, C.c_int]
    L.mpf_velocity_deposit_device.argtypes = [vp, C.c_int, i64, vp, vp, C.c_int, vp]
    L.mpf_velocity_deposit_pairs.argtypes = [vp, C.POINTER(i64)]
    L.mpf_propagate_accuracy.argtypes = [vp, vp, C.POINTER(Params), i64, vp, i64, C.POINTER(Accuracy)]
    L.mpf_autotune_info.argtypes = [vp, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), vp]
    L.mpf_cells_build.argtypes = [vp, i64, C.POINTER(CellsParams), vp, vp, i64, C.POINTER(i64)]
    L.mpf_cells_parse.argtypes = [C.c_char_p, i64, vp, i64, C.POINTER(i64)]
    L.mpf_cells_completion_info.argtypes = [vp]
    L.mpf_rays_propagate.argtypes = [vp, vp, C.POINTER(Params), C.POINTER(BundleParams), i64, vp, vp, vp, vp]
    L.mpf_surrogate_create.argtypes = [C.POINTER(SurrogateDomain), C.POINTER(vp)]
    L.mpf_surrogate_destroy.argtypes = [vp]
    L.mpf_surrogate_destroy.restype = None
    L.mpf_surrogate_train.argtypes = [vp, vp, C.POINTER(SurrogateTrainParams), C.POINTER(SurrogateTrainStats)]
    L.mpf_surrogate_sample.argtypes = [vp, vp, C.c_uint64, i64, vp, vp]
    L.mpf_surrogate_get_params.argtypes = [vp, vp, vp]
    L.mpf_surrogate_set_params.argtypes = [vp, vp, vp]
    L.mpf_surrogate_loss_grad.argtypes = [vp, i64, vp, vp, C.POINTER(d), vp]
    L.mpf_surrogate_eval.argtypes = [vp, i64, vp, vp]
    L.mpf_surrogate_propagate.argtypes = [vp, vp, vp, C.POINTER(Params), C.POINTER(SurrogatePropParams), i64, vp, vp,
                                          vp, vp, vp, C.POINTER(SurrogatePropStats)]
    for name in EXPORTS:
        if name not in ("mpf_version", "mpf_last_error", "mpf_device_count", "mpf_octree_destroy",
                        "mpf_cosmology_destroy", "mpf_noalloc_last_error", "mpf_surrogate_destroy"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def check(code: int, allow_warning: bool = True) -> int:
    if code < 0 or (code > 0 and not allow_warning):
        msg = _lib.mpf_last_error().decode(errors="replace") if _lib is not None else ""
        raise MpfError(code, msg)
    return code


def ptr(a) -> C.c_void_p:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return C.c_void_p(a.ctypes.data)
    return C.c_void_p(int(a))


def make_params(length, nsteps=10, order=2, stop="redshift", stop_value=0.0, planes=None, jacobian=True, exact=False,
                max_steps=0, plane_normal=(0.0, 0.0, 0.0), vobs=(0.0, 0.0, 0.0)):
    """Params struct plus the array that must outlive the call."""
    pl = np.ascontiguousarray(planes if planes is not None else np.zeros(0), dtype=np.float64)
    if pl.shape[0] > MPF_MAX_PLANES:
        raise ValueError("at most %d surfaces" % MPF_MAX_PLANES)
    p = Params()
    p.length = float(length)
    p.stop_value = float(stop_value)
    for k in range(3):
        p.plane_normal[k] = float(plane_normal[k])
    p.planes = pl.ctypes.data if pl.shape[0] else None
    p.nplanes = int(pl.shape[0])
    p.nsteps = int(nsteps)
    p.order = int(order)
    p.stop = STOP[stop] if isinstance(stop, str) else int(stop)
    p.jacobian = int(bool(jacobian))
    p.exact = int(bool(exact))
    p.max_steps = int(max_steps)
    for k in range(3):
        p.vobs[k] = float(vobs[k])
    return p, pl
