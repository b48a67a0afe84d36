"""GPU parity on whole rays, against the C oracle (the reference's float64
algorithm, pinned bit-exact to the reference's own build):

* an AMR cone octree (64^3 base at octree level 8, refined to level 11 in 50
  NFW haloes), rays to z = 2 (about 1000 steps each) with the infinitesimal
  Jacobian, CIC and TSC: the same construction as the benchmark octree at a
  size the oracle traces in a second;
* the uniform 64^3 field at file level 6 (octree level 8) over a 5 x 5 degree
  cone along the narrow-cone axis phi = theta = 20 degrees, written as the
  reference's 10-column ASCII cells and built into the cone octree on the
  GPU (mpf_cells_build), 4096 rays on a 64 x 64 grid, CIC, 10 steps per cell,
  to z = 0.5 with the Jacobian at z = 0.25 and 0.5.

Tolerances:
  exact mode (reference float64 order): step counts, every field of the final
    photon records and every surface field but the Jacobian bit-identical;
    the Jacobian (running sums, CUDA trig) within 1e-12 absolute.
  fast mode (FP32 gathers, FP64 state): the same step counts and surfaces on
    every ray; deflection and redshift within 1e-6 relative on every ray;
    kappa, gamma1, gamma2 within 1e-6 of the map's scale and 1/mu within 1e-6.
"""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ACC = importlib.import_module("magrathea-pathfinder_gb300.accuracy")


def _amr_spec(S):
    cosmo = S.Cosmology()
    chi2 = float(cosmo.chi_of_z(2.0)[0])
    return S.OctreeSpec(base_level=8, box_cells=64, lbox=2048.0, half_y=5.0, half_z=5.0, chi_max=chi2 * 1.02,
                        halos=50, max_level=11, refine_cells=2.5, seed=42)


def _exact_equal(s, f, pl, s_r, f_r, pl_r):
    np.testing.assert_array_equal(s, s_r)
    np.testing.assert_array_equal(f.view(np.uint64), f_r.view(np.uint64))
    jac = np.zeros(pl.shape[-1], dtype=bool)
    jac[6:9] = True
    np.testing.assert_array_equal(pl[..., ~jac].view(np.uint64), pl_r[..., ~jac].view(np.uint64))
    assert np.abs(pl[..., jac] - pl_r[..., jac]).max() <= 1e-12


@pytest.fixture(scope="module")
def amr(gpu_lib, pkg, synth, oracle_mod):
    spec = _amr_spec(synth)
    rec = synth.make_octree(spec)
    cos = synth.Cosmology().conformal_table(n=4000, amin=0.05)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    tree = pkg.Octree.from_records(rec)
    cosmo = pkg.Cosmology(*cos)
    O = oracle_mod.Oracle(rec, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length)
    launch = synth.photon_grid(16, 4.5, 4.5)          # 256 rays over the 9 x 9 degree grid
    yield tree, cosmo, O, launch, length
    tree.close()
    cosmo.close()


@pytest.mark.parametrize("order", [1, 2])
def test_amr_to_z2_every_ray(amr, pkg, order):
    tree, cosmo, O, launch, length = amr
    planes = np.array([1.0, 2.0])
    s_r, f_r, p_r = O.propagate(launch, order=order, nsteps=8, stop="redshift", stop_ref=2.0, planes=planes,
                                jacobian=True)
    assert s_r.min() > 500          # whole rays through the refinement shells
    s, f, p, rc = pkg.propagate(tree, cosmo, launch, length, nsteps=8, order=order, stop="redshift", planes=planes,
                                jacobian=True, exact=False)
    assert rc == 0
    rep = ACC.compare(launch, s, f, p, s_r, f_r, p_r)
    assert ACC.within(rep, 1e-6, 1e-6), rep
    s, f, p, rc = pkg.propagate(tree, cosmo, launch, length, nsteps=8, order=order, stop="redshift", planes=planes,
                                jacobian=True, exact=True)
    assert rc == 0
    _exact_equal(s, f, p, s_r, f_r, p_r)


@pytest.fixture(scope="module")
def uniform_cone(gpu_lib, pkg, synth, oracle_mod):
    """The uniform 64^3 cone along phi = theta = 20 deg, through the ASCII cells
    and the device build; the oracle traces the same built records."""
    spec = synth.uniform_grid_cone(0.5, (20.0, 20.0))
    rec = synth.make_octree(spec)
    rows = synth.cells_ramses(rec, spec).astype(np.float32)
    cos = synth.Cosmology().conformal_table(n=4000, amin=0.05)
    cosmo = pkg.Cosmology(*cos)
    axis = spec.frame()[:, 0]
    built = pkg.cells_build(rows, cosmo, (0.0, 0.0, 0.0), axis * (spec.chi_max / spec.lbox),
                            np.radians(2.5 * np.sqrt(2.0)), (0.0, 0.0, 0.0), 4.0 / 64.0, spec.cosmo.h,
                            spec.cosmo.omega_m, spec.lbox, synth.MPC, order=1)
    built = np.frombuffer(built.tobytes(), dtype=synth.RECORD)
    length = spec.lbox * synth.MPC / spec.cosmo.h
    tree = pkg.Octree.from_records(built)
    O = oracle_mod.Oracle(built, {"t": cos[0], "a": cos[1], "dadt": cos[2]}, length)
    launch = synth.photon_grid(64, 2.5, 2.5, spec.frame())
    yield tree, cosmo, O, launch, length, rec, built
    tree.close()
    cosmo.close()


def test_uniform_cone_build_keeps_the_cells(uniform_cone):
    """Every cell of the 64^3 field inside the cone survives the ASCII round
    trip and the cone filter with its key, its level and its potential to
    float rounding."""
    *_, rec, built = uniform_cone
    keys = lambda r: r["hi"].astype(object) * (1 << 64) + r["lo"].astype(object)
    have = dict(zip(keys(built), built["phi"]))
    got = np.array([have.get(k, np.nan) for k in keys(rec)], dtype=np.float64)
    assert np.isfinite(got).mean() > 0.9
    ok = np.isfinite(got)
    assert np.all(np.abs(got[ok] - rec["phi"][ok]) <= 1e-6 * np.abs(rec["phi"]).max())


@pytest.mark.parametrize("exact", [True, False])
def test_uniform_cone_4096_rays(uniform_cone, pkg, exact):
    tree, cosmo, O, launch, length, _, _ = uniform_cone
    assert launch.shape[0] == 4096
    planes = np.array([0.25, 0.5])
    s_r, f_r, p_r = O.propagate(launch, order=1, nsteps=10, stop="redshift", stop_ref=0.5, planes=planes,
                                jacobian=True)
    assert s_r.min() > 300 and (p_r[..., 19] != 0).all()
    s, f, p, rc = pkg.propagate(tree, cosmo, launch, length, nsteps=10, order=1, stop="redshift", planes=planes,
                                jacobian=True, exact=exact)
    assert rc == 0
    if exact:
        _exact_equal(s, f, p, s_r, f_r, p_r)
    else:
        rep = ACC.compare(launch, s, f, p, s_r, f_r, p_r)
        assert ACC.within(rep, 1e-6, 1e-6), rep


@pytest.mark.parametrize("order", [1, 2])
def test_accuracy_statistic_of_the_call(amr, pkg, order):
    """mpf_propagate_accuracy (the per-call statement of the FP32-gather
    kernel's error against the float64 kernel) gives what the same two runs
    compared in numpy give, and states errors inside the 1e-6 bound."""
    tree, cosmo, O, launch, length = amr
    planes = np.array([1.0, 2.0])
    kw = dict(nsteps=8, order=order, stop="redshift", planes=planes, jacobian=True)
    got = pkg.propagate_accuracy(tree, cosmo, launch, length, sample=64, **kw)
    idx = (np.arange(64) * launch.shape[0]) // 64
    sub = launch[idx]
    s0, f0, p0, _ = pkg.propagate(tree, cosmo, sub, length, exact=True, **kw)
    s1, f1, p1, _ = pkg.propagate(tree, cosmo, sub, length, exact=False, **kw)
    ref = ACC.compare(sub, s1, f1, p1, s0, f0, p0)
    assert got["rays"] == 64
    for k in ("step_count_differs", "max_step_diff", "surface_valid_differs"):
        assert got[k] == ref[k], k
    # the deflection is the angle of a cross product of nearly parallel vectors:
    # the two codes' roundings (the host compiler may contract to FMA) agree to
    # ~1e-12 of the angle, i.e. to 1e-11 absolute in its relative error
    for k, tol in (("deflection_rel", 1e-11), ("redshift_rel", 1e-15)):
        for s in ("max", "median"):
            assert got[k][s] == pytest.approx(ref[k][s], rel=1e-6, abs=tol), (k, s)
    for k in ACC.LENSING:
        # the lensing quantities are formed on the host, where FMA contraction moves them by ~1e-16
        assert got[k]["abs_max"] == pytest.approx(ref[k]["abs_max"], rel=1e-9, abs=1e-15)
        assert got[k]["scale"] == pytest.approx(ref[k]["scale"], rel=1e-14)   # 1/mu: FMA contraction of a11 a22 - a12^2
    assert ACC.within(got, 1e-6, 1e-6), got
