"""GPU parity of the velocity-field path (the reference's -DVELOCITYFIELD
build) against the reference's own outputs in tests/golden/velocity.npz:

* mpf_velocity_deposit (CIC and TSC, two particle files between BEGIN and
  FINISH): every cell's velocity and mass bit-identical to the reference's
  deposit on one thread;
* rays traced with the Doppler, ISW and observer terms: exact mode gives the
  reference's step counts and final photon records bit for bit, on the
  reference's field and on the device's own deposit; the FP32-gather kernel
  (its velocity instantiation) the same step counts and the redshift,
  deflection and convergence within 1e-6;
* FillMap with the observer velocity: the map rows within the map tests'
  tolerances (the device's pixel centres are a few ulps from the harness's);
* the catalogue root-finder and the surrogate refuse such an octree, and
  removing the field gives back the plain build's results.
"""
import importlib

import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

ACC = importlib.import_module("magrathea-pathfinder_gb300.accuracy")


@pytest.fixture(scope="module")
def vel():
    return load_golden("velocity")


@pytest.fixture(scope="module")
def amr():
    return load_golden("amr")


@pytest.fixture(scope="module")
def cosmo(gpu_lib, pkg, amr):
    c = pkg.Cosmology(amr["cosmo_t"], amr["cosmo_a"], amr["cosmo_dadt"], amr["cosmo_d2adt2"])
    yield c
    c.close()


def _deposit(pkg, amr, vel, scheme):
    tree = pkg.Octree.from_records(amr["records"])
    pos, pv, k = vel["part_pos"], vel["part_vel"], int(vel["part_split"])
    tree.deposit_velocity(pos[:k], pv[:k], scheme, begin=True, finish=False)
    tree.deposit_velocity(pos[k:], pv[k:], scheme, begin=False, finish=True)
    return tree


@pytest.mark.parametrize("scheme", ["cic", "tsc"])
def test_deposit_bit_exact(gpu_lib, pkg, amr, vel, scheme):
    tree = _deposit(pkg, amr, vel, scheme)
    v, rho = tree.velocity()
    np.testing.assert_array_equal(v.view(np.uint32), vel["ref_vel_" + scheme].view(np.uint32))
    np.testing.assert_array_equal(rho.view(np.uint32), vel["ref_rho_" + scheme].view(np.uint32))
    tree.close()


def test_deposit_large_batch_is_deterministic(gpu_lib, pkg, synth, amr):
    """200k particles (several internal passes of the pair sort are not
    needed for this size, but the per-cell runs are long): two deposits give
    the same bits, and the masses sum to the weights the particles spread."""
    pos, pv = synth.velocity_particles(amr["records"], 200000, seed=9)
    t1 = pkg.Octree.from_records(amr["records"])
    t2 = pkg.Octree.from_records(amr["records"])
    t1.deposit_velocity(pos, pv, "tsc")
    t2.deposit_velocity(pos[:70000], pv[:70000], "tsc", True, False)
    t2.deposit_velocity(pos[70000:], pv[70000:], "tsc", False, True)
    v1, r1 = t1.velocity()
    v2, r2 = t2.velocity()
    np.testing.assert_array_equal(v1.view(np.uint32), v2.view(np.uint32))
    np.testing.assert_array_equal(r1.view(np.uint32), r2.view(np.uint32))
    assert np.isfinite(v1).all() and (r1 > 0).mean() > 0.9
    t1.close()
    t2.close()


@pytest.mark.parametrize("scheme,order", [("cic", 1), ("tsc", 2)])
@pytest.mark.parametrize("source", ["reference_field", "device_deposit"])
def test_exact_rays_bit_exact(gpu_lib, pkg, amr, vel, cosmo, scheme, order, source):
    if source == "device_deposit":
        tree = _deposit(pkg, amr, vel, scheme)
    else:
        tree = pkg.Octree.from_records(amr["records"])
        tree.set_velocity(vel["ref_vel_" + scheme], vel["ref_rho_" + scheme])
    s, f, _, rc = pkg.propagate(tree, cosmo, vel["launch"], float(amr["cosmo_length"]), nsteps=int(vel["nsteps"]),
                                order=order, stop="redshift", stop_value=float(vel["zs"][-1]), jacobian=False,
                                exact=True, vobs=vel["vobs"])
    assert rc == 0
    np.testing.assert_array_equal(s, vel["ref_steps_o%d" % order])
    np.testing.assert_array_equal(f.view(np.uint64), vel["ref_final_o%d" % order].view(np.uint64))
    tree.close()


@pytest.mark.parametrize("scheme,order", [("cic", 1), ("tsc", 2)])
def test_fast_rays_within_tolerance(gpu_lib, pkg, oracle_mod, amr, vel, cosmo, scheme, order):
    """The FP32-gather kernel's velocity instantiation against the oracle
    (pinned to the reference's velocity build) on rays with surfaces and the
    Jacobian."""
    tree = pkg.Octree.from_records(amr["records"])
    tree.set_velocity(vel["ref_vel_" + scheme], vel["ref_rho_" + scheme])
    cos = {"t": amr["cosmo_t"], "a": amr["cosmo_a"], "dadt": amr["cosmo_dadt"]}
    O = oracle_mod.Oracle(amr["records"], cos, float(amr["cosmo_length"]))
    O.fields[:, 0] = vel["ref_rho_" + scheme]
    O.set_velocity(vel["ref_vel_" + scheme], vel["vobs"])
    launch = vel["launch"]
    zs = vel["zs"]
    s_r, f_r, p_r = O.propagate(launch, order=order, nsteps=int(vel["nsteps"]), stop="redshift", stop_ref=float(zs[-1]),
                                planes=zs, jacobian=True)
    s, f, p, rc = pkg.propagate(tree, cosmo, launch, float(amr["cosmo_length"]), nsteps=int(vel["nsteps"]), order=order,
                                stop="redshift", planes=zs, jacobian=True, exact=False, vobs=vel["vobs"])
    assert rc == 0
    rep = ACC.compare(launch, s, f, p, s_r, f_r, p_r)
    assert ACC.within(rep, 1e-6, 1e-6), rep
    # the Doppler term is in the surfaces' redshifts: the plain kernel misses them by far more
    tree.set_velocity(None)
    s0, f0, p0, _ = pkg.propagate(tree, cosmo, launch, float(amr["cosmo_length"]), nsteps=int(vel["nsteps"]),
                                  order=order, stop="redshift", planes=zs, jacobian=True, exact=False)
    assert np.abs(f0[:, 19] - f_r[:, 19]).max() > 1e-5 or not np.array_equal(s0, s_r)
    tree.close()


@pytest.mark.parametrize("exact", [True, False])
def test_hmaps_fill_with_velocity_matches_reference(gpu_lib, pkg, amr, vel, cosmo, exact):
    tree = pkg.Octree.from_records(amr["records"])
    tree.set_velocity(vel["ref_vel_tsc"], vel["ref_rho_tsc"])
    comps = str(vel["components"]).split(",")
    got = pkg.hmaps_fill(tree, cosmo, int(vel["nside"]), vel["pixels"], vel["zs"], amr["homogeneous"], comps,
                         float(amr["cosmo_length"]), nsteps=int(vel["nsteps"]), order=2, exact=exact, vobs=vel["vobs"])
    ref = vel["ref_maps_o2"]
    assert got.shape == ref.shape
    srow = 4 + comps.index("steps") - 1
    np.testing.assert_array_equal(got[:, srow] != 0, ref[:, srow] != 0)
    for row in range(4):
        scale = max(np.abs(ref[:, row]).max(), 1e-6)
        assert np.abs(got[:, row] - ref[:, row]).max() <= 1e-6 * scale + 2e-7 * (row == 3), row
    for row in range(4, ref.shape[1]):
        scale = np.abs(ref[:, row]).max() + 1e-30
        assert np.abs(got[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row
    tree.close()


def test_catalogue_and_surrogate_refuse_a_velocity_field(gpu_lib, pkg, amr, vel, cosmo):
    capi = importlib.import_module("magrathea-pathfinder_gb300.capi")
    tree = pkg.Octree.from_records(amr["records"])
    tree.set_velocity(vel["ref_vel_cic"])
    with pytest.raises(capi.MpfError) as e:
        pkg.catalogue(tree, cosmo, np.zeros((2, 6)) + 0.1, float(amr["cosmo_length"]), h=0.68)
    assert "velocity" in str(e.value)
    sur = importlib.import_module("magrathea-pathfinder_gb300.surrogate")
    s = sur.Surrogate((0.05, 0.05), 0.5, 0.8)
    with pytest.raises(capi.MpfError) as e:
        s.propagate(tree, cosmo, np.array([[0, 0, 0, 1.0, 0, 0]]), float(amr["cosmo_length"]))
    assert "velocity" in str(e.value)
    s.close()
    tree.close()


def test_removing_the_field_restores_the_plain_build(gpu_lib, pkg, amr, cosmo):
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    tree.set_velocity(np.zeros((g["records"].shape[0], 3), np.float32))
    tree.set_velocity(None)
    s, f, _, rc = pkg.propagate(tree, cosmo, g["launch"], float(g["cosmo_length"]), nsteps=int(g["nsteps"]), order=2,
                                stop="redshift", stop_value=float(g["zs"][-1]), jacobian=False, exact=True)
    np.testing.assert_array_equal(s, g["ref_steps_o2"])
    np.testing.assert_array_equal(f.view(np.uint64), g["ref_final_o2"].view(np.uint64))
    tree.close()
