"""The launch-shape autotuner (mpf_autotune_info).

The first batch of at least 2^17 rays for an octree is traced in four slices,
each with one candidate shape (threads per block x rays per lane per
work-queue claim), and the fastest shape is kept for later batches.  A ray's
results do not depend on the shape, so the tuning batch, a later batch with
the tuned shape and small batches (one-warp blocks) give bit-identical rays.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_autotuned_shape_changes_no_ray(gpu_lib, pkg, synth):
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    length = float(g["cosmo_length"])
    launch = synth.photon_grid(363, 2.4, 2.4)          # 131 769 rays >= 2^17
    assert launch.shape[0] >= 1 << 17
    assert pkg.autotune_info(tree, "propagate", 2) is None
    kw = dict(nsteps=8, order=2, stop="redshift", stop_value=0.1, planes=np.array([0.05, 0.1]), jacobian=True,
              exact=False)
    s1, f1, p1, rc = pkg.propagate(tree, cos, launch, length, **kw)     # tunes, in four slices
    assert rc == 0
    info = pkg.autotune_info(tree, "propagate", 2)
    assert info is not None
    tpb, depth, rates = info
    assert (tpb, depth) in ((128, 1), (64, 1), (32, 1), (128, 2))
    assert all(r > 0 for r in rates) and max(rates) == pytest.approx(rates[[(128, 1), (64, 1), (32, 1), (128, 2)].index((tpb, depth))])
    s2, f2, p2, _ = pkg.propagate(tree, cos, launch, length, **kw)      # the tuned shape
    np.testing.assert_array_equal(s1, s2)
    np.testing.assert_array_equal(f1.view(np.uint64), f2.view(np.uint64))
    np.testing.assert_array_equal(p1.view(np.uint64), p2.view(np.uint64))
    sel = np.arange(0, launch.shape[0], 97)
    s3, f3, p3, _ = pkg.propagate(tree, cos, launch[sel], length, **kw)  # a small batch: one-warp blocks
    np.testing.assert_array_equal(s3, s1[sel])
    np.testing.assert_array_equal(f3.view(np.uint64), f1[sel].view(np.uint64))
    np.testing.assert_array_equal(p3.view(np.uint64), p1[sel].view(np.uint64))
    tree.close()
    cos.close()
