"""CPU tests of the benchmark's workload definitions (bench.py): the ray grid
traces each of the 1000 x 1000 directions of the 10 x 10 degree cone once,
the catalogue sources are uniform in comoving volume inside the stated cone
to z = 2, the benchmark octree is the stated construction, and the FP64-pipe
roofline is the stated arithmetic."""
import importlib
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)
bench = importlib.import_module("bench")


def test_ray_grid_covers_the_cone_once():
    g = bench.ray_grid()
    assert g.shape == (1000 * 1000, 6)
    assert not g[:, :3].any()                                     # launched from the observer
    np.testing.assert_allclose(np.linalg.norm(g[:, 3:], axis=1), 1.0, rtol=0, atol=1e-15)
    ph = np.degrees(np.arctan2(g[:, 4], g[:, 3]))
    th = np.degrees(np.arccos(g[:, 5]))
    assert np.abs(ph).max() < 5.0 and np.abs(th - 90.0).max() < 5.0
    # every grid direction exactly once
    iy = np.rint((ph / 5.0 + 1.0) / 2.0 * 1000 - 0.5).astype(int)
    iz = np.rint(((th - 90.0) / 5.0 + 1.0) / 2.0 * 1000 - 0.5).astype(int)
    assert np.unique(iy * 1000 + iz).shape[0] == 1000 * 1000
    # the shuffled 8 x 4 tiles: neighbouring rays of a warp stay neighbours on the sky
    w = slice(0, 32)
    assert np.ptp(iy[w]) == 7 and np.ptp(iz[w]) == 3


def test_catalogue_sources_fill_the_cone_to_z2():
    synth = importlib.import_module(bench.PKG + ".synth")
    n = 200000
    src = bench.catalogue_sources(synth, n, 17)
    assert src.shape == (n, 8)
    chi2 = float(synth.Cosmology().chi_of_z(2.0)[0]) / 2048.0
    d = np.linalg.norm(src[:, :3], axis=1)
    assert d.max() <= chi2 * (1 + 1e-12) and d.min() >= chi2 * 0.02 ** (1 / 3) * (1 - 1e-12)
    # uniform in volume: the fraction within half the distance is about 1/8 of the shell's volume share
    inner = np.mean(d < chi2 / 2)
    expect = (0.125 - 0.02) / (1 - 0.02)
    assert abs(inner - expect) < 0.005
    ph = np.degrees(np.arctan2(src[:, 1], src[:, 0]))
    assert np.abs(ph).max() <= 4.5 + 1e-9
    np.testing.assert_array_equal(src[:, 6], np.arange(n))
    assert (src[:, 7] == 1.0).all()


def test_benchmark_octree_spec():
    synth = importlib.import_module(bench.PKG + ".synth")
    spec = bench.workload_spec(synth, "amr")
    # 256^3 base at octree level 10 refined to 14 in 2000 NFW haloes, to z = 2 over 10 x 10 degrees
    assert (spec.base_level, spec.box_cells, spec.max_level, spec.halos) == (10, 256, 14, 2000)
    assert spec.half_y == 5.0 and spec.half_z == 5.0
    chi2 = float(synth.Cosmology().chi_of_z(2.0)[0])
    assert abs(spec.chi_max / chi2 - 1.02) < 1e-12


def test_fp64_roofline_arithmetic():
    r = bench.fp64_roofline(8.0e8, {"sm_mhz": 2000.0})
    peak = 152 * 2 * 2000.0e6 / 1e12      # 152 SMs: the GB300's count, and the default without a GPU
    assert abs(r["peak"] - peak) < 1e-12
    assert abs(r["achieved"] - 8.0e8 * bench.FP64_OPS_PER_PHOTON_STEP / 1e12) < 1e-12
    assert abs(r["frac"] - r["achieved"] / r["peak"]) < 1e-15
