"""The allocation-free propagation entry point, mpf_propagate_noalloc.

It is for callers that cannot call cudaMalloc / cudaFree while they trace
rays: a pooling allocator owns the GPU's memory, the process runs under a hard
device-memory cap, or the loop cannot afford the device synchronisation an
allocation may cause.  It stages everything through the library's static
device scratch array, so its results must equal those of mpf_propagate (which
allocates) for the same rays, on two calls in a row (the second call reuses
the array left by the first, so anything not cleared would show up), and a
batch too large for the array must be refused with a clear error.
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def _noalloc(L, capi, tree, cos, p, launch, nplanes):
    n = launch.shape[0]
    steps = np.zeros(n, dtype=np.int64)
    final = np.zeros((n, capi.MPF_PHOTON_FIELDS))
    planes = np.zeros((n, max(nplanes, 1), capi.MPF_PLANE_FIELDS))
    rc = L.mpf_propagate_noalloc(tree._h, cos._h, ctypes.byref(p), n, capi.ptr(launch), capi.ptr(steps),
                                 capi.ptr(final), capi.ptr(planes) if nplanes else None)
    return rc, steps, final, planes[:, :nplanes]


@pytest.mark.parametrize("exact", [False, True])
def test_noalloc_matches_allocating_call_twice(gpu_lib, pkg, exact):
    import importlib
    capi = importlib.import_module("magrathea-pathfinder_gb300.capi")
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    length = float(g["cosmo_length"])
    zs = g["zs"]
    launch = np.ascontiguousarray(g["launch"])
    ref_steps, ref_final, ref_planes, rc = pkg.propagate(tree, cos, launch, length, nsteps=8, order=2, stop="redshift",
                                                         planes=zs, jacobian=True, exact=exact)
    assert rc == 0
    p, keep = capi.make_params(length, nsteps=8, order=2, stop="redshift", planes=zs, jacobian=True, exact=exact)
    for _ in range(2):
        rc, steps, final, planes = _noalloc(gpu_lib, capi, tree, cos, p, launch, zs.shape[0])
        assert rc == 0, gpu_lib.mpf_noalloc_last_error()
        # same kernel on the same rays: identical to the allocating entry point
        np.testing.assert_array_equal(steps, ref_steps)
        np.testing.assert_array_equal(final.view(np.uint64), ref_final.view(np.uint64))
        np.testing.assert_array_equal(planes.view(np.uint64), ref_planes.view(np.uint64))
    # a different, smaller batch after the first two: no stale queue or status state
    rc, steps, final, _ = _noalloc(gpu_lib, capi, tree, cos, p, launch[:7].copy(), zs.shape[0])
    assert rc == 0
    np.testing.assert_array_equal(steps, ref_steps[:7])
    del keep


@pytest.mark.parametrize("exact", [False, True])
def test_noalloc_ngp_and_optional_outputs(gpu_lib, pkg, exact):
    """ORDER = 0 (nearest grid point) is accepted as by mpf_propagate, which
    runs it in the float64 kernel whatever `exact` says, and the step counts
    are optional (NULL) as there."""
    import importlib
    capi = importlib.import_module("magrathea-pathfinder_gb300.capi")
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    length = float(g["cosmo_length"])
    zs = g["zs"]
    launch = np.ascontiguousarray(g["launch"])
    ref_steps, ref_final, ref_planes, rc = pkg.propagate(tree, cos, launch, length, nsteps=8, order=0, stop="redshift",
                                                         planes=zs, jacobian=True, exact=exact)
    assert rc == 0
    p, keep = capi.make_params(length, nsteps=8, order=0, stop="redshift", planes=zs, jacobian=True, exact=exact)
    for _ in range(2):
        rc, steps, final, planes = _noalloc(gpu_lib, capi, tree, cos, p, launch, zs.shape[0])
        assert rc == 0, gpu_lib.mpf_noalloc_last_error()
        np.testing.assert_array_equal(steps, ref_steps)
        np.testing.assert_array_equal(final.view(np.uint64), ref_final.view(np.uint64))
        np.testing.assert_array_equal(planes.view(np.uint64), ref_planes.view(np.uint64))
    # steps = NULL: the other outputs are still written
    final = np.zeros((launch.shape[0], capi.MPF_PHOTON_FIELDS))
    rc = gpu_lib.mpf_propagate_noalloc(tree._h, cos._h, ctypes.byref(p), launch.shape[0], capi.ptr(launch), None,
                                       capi.ptr(final), None)
    assert rc == 0, gpu_lib.mpf_noalloc_last_error()
    np.testing.assert_array_equal(final.view(np.uint64), ref_final.view(np.uint64))
    del keep


def test_noalloc_rejects_batches_beyond_the_scratch(gpu_lib, pkg):
    import importlib
    capi = importlib.import_module("magrathea-pathfinder_gb300.capi")
    g = load_golden("uniform")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    p, keep = capi.make_params(float(g["cosmo_length"]), nsteps=10, order=2, stop="redshift", stop_value=0.2)
    n = 100000      # 100k rays x (48 + 8 + 224) bytes > 16 MiB
    launch = np.zeros((n, 6))
    launch[:, 3] = 1.0
    rc, _, _, _ = _noalloc(gpu_lib, capi, tree, cos, p, launch, 0)
    assert rc == -1
    assert b"static scratch" in gpu_lib.mpf_noalloc_last_error()
    del keep
