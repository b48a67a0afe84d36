"""The rays driver's distance statistics (src/rays.cpp:280-455) on CPU: the
interpolation against the C oracle's Utility::interpolate (bit-exact), the
statistics of the golden bundles on one process, and the same statistics
with the rays split over two gloo ranks (the rays path's one collective)."""
import importlib
import os
import socket

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def rays_mod():
    return importlib.import_module("magrathea-pathfinder_gb300.rays")


def _inputs():
    g = load_golden("rays")
    sizes, T = g["ref_sizes_o2"], g["ref_traj_o2"]
    central = [T[i, :n] for i, n in enumerate(sizes)]
    return central, g["flrw_traj_0"], float(1.0 / g["cosmo_length"])


def test_interpolate_matches_oracle(rays_mod, oracle_mod):
    import ctypes as C
    L = oracle_mod.lib()
    rng = np.random.default_rng(3)
    x = np.sort(rng.uniform(0, 1, 50))
    x[10] = x[11]                      # a repeated abscissa
    y = rng.normal(0, 1, 50)
    x0 = np.concatenate([rng.uniform(-0.2, 1.2, 200), x[:5], [x[10]]])
    got = rays_mod.interpolate(x0, x, y)
    ref = np.array([L.mpfo_interpolate(float(v), x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), 50)
                    for v in x0])
    np.testing.assert_array_equal(got.view(np.uint64), ref.view(np.uint64))


@pytest.mark.parametrize("interp", ["redshift", "r", "a", "t", "lambda"])
@pytest.mark.parametrize("stat", ["distance", "distance2", "homogeneous", "inhomogeneous"])
def test_statistics_one_rank(rays_mod, interp, stat):
    central, ref, inv = _inputs()
    r = rays_mod.statistics(central, ref, interp, stat, nstat=40, invlength=inv)
    accepted = sum(1 for c in central if c.shape[0])
    assert r["count"] == r["gcount"] == accepted
    n = r["z"].shape[0]
    assert 40 <= n <= 80 and np.all(np.diff(r["z"]) > 0)
    ys = np.array([rays_mod.interpolate(r["x"], rays_mod._x(c, rays_mod._INTERP_CASE.get(interp, 0)),
                                        rays_mod._y(c, rays_mod._STAT_CASE[stat], inv)) for c in central if c.shape[0]])
    np.testing.assert_allclose(r["mean"], ys.mean(axis=0), rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(r["std"], ys.std(axis=0, ddof=1), rtol=1e-9, atol=1e-300)
    np.testing.assert_array_equal(r["gmean"], r["mean"])
    text = rays_mod.statistics_text(r["z"], r["y"], r["gmean"], r["gstd"], r["gcount"])
    lines = text.splitlines()
    assert lines[0] == "# %d" % accepted and len(lines) == n + 1 and len(lines[1].split()) == 4


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, outdir):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "tests")):
        if p not in sys.path:
            sys.path.insert(0, p)
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    R = importlib.import_module("magrathea-pathfinder_gb300.rays")
    from test_rays_stats import _inputs
    central, ref, inv = _inputs()
    mine = central[rank::world]
    r = R.statistics(mine, ref, "redshift", "distance", nstat=40, invlength=inv, dist=dist)
    np.savez(os.path.join(outdir, "r%d.npz" % rank), **{k: np.asarray(v) for k, v in r.items()})
    dist.barrier()
    dist.destroy_process_group()


def test_statistics_reduce_over_two_ranks(tmp_path, rays_mod):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    central, ref, inv = _inputs()
    one = rays_mod.statistics(central, ref, "redshift", "distance", nstat=40, invlength=inv)
    parts = [dict(np.load(tmp_path / ("r%d.npz" % r))) for r in range(world)]
    for p in parts:
        assert int(p["gcount"]) == one["count"]
        np.testing.assert_allclose(p["gmean"], one["mean"], rtol=1e-13)
        np.testing.assert_allclose(p["gstd"], one["std"], rtol=1e-10)
    assert sum(int(p["count"]) for p in parts) == one["count"]
