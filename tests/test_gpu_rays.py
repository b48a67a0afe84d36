"""GPU ray bundles (mpf_rays_propagate, Integrator::propagate) against the
reference's outputs (tests/golden/rays.npz) and the C oracle.

Tolerances: exact mode is bit-identical (sizes and every column of the central
trajectory, the angular diameter distance included).  Fast mode (FP32
gathers): same accept / reject decisions and sizes within 1 point; positions
within 1e-9 and redshift within 1e-7 relative, the distance within 1e-5
relative (it is a difference of nearby rays' positions)."""
import numpy as np
import pytest

from conftest import load_golden
from test_rays_oracle import central_photons

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def rays_dev(gpu_lib, pkg):
    g = load_golden("rays")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    yield g, tree, cos
    tree.close()
    cos.close()


def _run(pkg, g, tree, cos, i, order, exact, cap=400):
    ph = central_photons(g)[i:i + 1]
    return pkg.rays_propagate(tree, cos, ph, float(g["cosmo_length"]), int(g["count"][i]), float(g["angle"][i]),
                              rotation=g["rotation"][i:i + 1], interpolation=str(g["interp"][i]), amin=float(g["amin"][i]),
                              nsteps=int(g["nsteps"]), order=order, exact=exact, capacity=cap)


@pytest.mark.parametrize("order", [1, 2])
def test_bundles_exact_bit_exact(rays_dev, pkg, order):
    g, tree, cos = rays_dev
    sizes, ref = g["ref_sizes_o%d" % order], g["ref_traj_o%d" % order]
    for i in range(sizes.shape[0]):
        s, t = _run(pkg, g, tree, cos, i, order, True)
        assert s[0] == sizes[i], i
        np.testing.assert_array_equal(t[0, :sizes[i]].view(np.uint64), ref[i, :sizes[i]].view(np.uint64))


@pytest.mark.parametrize("order", [1, 2])
def test_bundles_fast_within_tolerance(rays_dev, pkg, order):
    g, tree, cos = rays_dev
    sizes, ref = g["ref_sizes_o%d" % order], g["ref_traj_o%d" % order]
    for i in range(sizes.shape[0]):
        s, t = _run(pkg, g, tree, cos, i, order, False)
        assert (s[0] == 0) == (sizes[i] == 0), i
        if sizes[i] == 0:
            continue
        assert abs(int(s[0]) - int(sizes[i])) <= 1
        m = min(int(s[0]), int(sizes[i])) - 1
        got, want = t[0, :m], ref[i, :m]
        assert np.all(np.abs(got[:, 3:6] - want[:, 3:6]) <= 1e-9)
        assert np.all(np.abs(got[:, 19] - want[:, 19]) <= 1e-7 * np.abs(want[:, 19]) + 1e-12)
        assert np.all(np.abs(got[:, 22] - want[:, 22]) <= 1e-5 * np.abs(want[:, 22]) + 1e-30)


def test_batch_of_bundles_matches_oracle(rays_dev, pkg, oracle_mod, synth):
    """Many bundles in one call (the trajectory buffers hold all of them at
    once) against the C oracle, exact mode."""
    g, tree, cos = rays_dev
    n = 24
    grid = synth.photon_grid(5, 1.0, 1.0)[:n]
    ph = np.concatenate([grid[:, :3], grid[:, 3:]], axis=1)
    rot = np.linspace(0.0, 3.0, n)
    kw = dict(nsteps=int(g["nsteps"]), order=2)
    sizes, traj = pkg.rays_propagate(tree, cos, ph, float(g["cosmo_length"]), 6, np.radians(0.25), rotation=rot,
                                     interpolation="r", exact=True, capacity=400, **kw)
    O = oracle_mod.Oracle(g["records"], {"t": g["cosmo_t"], "a": g["cosmo_a"], "dadt": g["cosmo_dadt"]},
                          float(g["cosmo_length"]), nthreads=1)
    for i in range(n):
        ref = O.propagate_bundle(ph[i], 6, np.radians(0.25), rot[i], "r", 0.0, **kw)
        assert sizes[i] == ref.shape[0], i
        np.testing.assert_array_equal(traj[i, :sizes[i]].view(np.uint64), ref.view(np.uint64))
    assert (sizes > 0).sum() >= n // 2


def test_capacity_too_small_is_an_error(rays_dev, pkg):
    g, tree, cos = rays_dev
    with pytest.raises(pkg.MpfError):
        _run(pkg, g, tree, cos, 0, 2, True, cap=10)


def test_flrw_reference_bundle_bit_exact(rays_dev, pkg):
    """The rays driver's FLRW reference bundle (Order = -1 on a uniform octree)
    against the reference's own, every 8th point and the last."""
    g, tree, cos = rays_dev
    level, nst, every = int(g["flrw_level"]), int(g["flrw_nsteps"]), int(g["flrw_every"])
    ph = np.array([[0.0, 0.0, 0.0, 1.0, 0.0, 0.0]])     # Integrator::launch(0, 0, 0, 2, 0, 0)
    for j in range(g["flrw_count"].shape[0]):
        size = int(g["flrw_size_%d" % j])
        sizes, traj = pkg.rays_propagate(tree, cos, ph, float(g["cosmo_length"]), int(g["flrw_count"][j]),
                                         float(g["flrw_angle"][j]), interpolation=str(g["flrw_interp"][j]), nsteps=nst,
                                         order=1, exact=True, capacity=size + 8, homogeneous_level=level)
        assert sizes[0] == size
        np.testing.assert_array_equal(traj[0, :size:every].view(np.uint64), g["flrw_traj_%d" % j].view(np.uint64))
        np.testing.assert_array_equal(traj[0, size - 1].view(np.uint64), g["flrw_last_%d" % j].view(np.uint64))
