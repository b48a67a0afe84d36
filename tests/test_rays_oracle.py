"""Ray bundles (Integrator::propagate, src/integrator.h:861-1015) on the CPU:
the C oracle's restatement and the trajectory writer against the reference's
own outputs recorded in tests/golden/rays.npz (bit-exact)."""
import importlib

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def rays_golden():
    return load_golden("rays")


def central_photons(g):
    """The photons the reference launched: Integrator::launch(start, end) ->
    start and (end - start) / |end - start| (integrator.h:265-289)."""
    L = g["launch"]
    d = L[:, 3:] - L[:, :3]
    norm = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    return np.concatenate([L[:, :3], d / norm[:, None]], axis=1)


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_bundles_bit_exact(rays_golden, oracle_mod, order):
    g = rays_golden
    O = oracle_mod.Oracle(g["records"], {"t": g["cosmo_t"], "a": g["cosmo_a"], "dadt": g["cosmo_dadt"]},
                          float(g["cosmo_length"]), nthreads=1)
    ph = central_photons(g)
    sizes, ref = g["ref_sizes_o%d" % order], g["ref_traj_o%d" % order]
    assert (sizes == 0).sum() >= 2 and (sizes > 0).sum() >= 6     # rejected and accepted bundles
    for i in range(ph.shape[0]):
        t = O.propagate_bundle(ph[i], int(g["count"][i]), float(g["angle"][i]), float(g["rotation"][i]),
                               str(g["interp"][i]), float(g["amin"][i]), order=order, nsteps=int(g["nsteps"]))
        assert t.shape[0] == sizes[i], i
        np.testing.assert_array_equal(t.view(np.uint64), ref[i, :sizes[i]].view(np.uint64))


def test_distance_column_is_filled(rays_golden):
    g = rays_golden
    for i, n in enumerate(g["ref_sizes_o2"]):
        if n == 0:
            continue
        d = g["ref_traj_o2"][i, :n, 22]
        if g["count"][i] == 0:
            assert np.all(d == 0)
        else:
            assert d[0] == 0 and np.all(d[1:] > 0)


@pytest.mark.parametrize("order", [1, 2])
def test_trajectory_writer_matches_output_save(rays_golden, order):
    W = importlib.import_module("magrathea-pathfinder_gb300.writers")
    g = rays_golden
    n = int(g["ref_sizes_o%d" % order][0])
    assert W.trajectory_text(g["ref_traj_o%d" % order][0, :n]) == str(g["ref_text_o%d" % order])
