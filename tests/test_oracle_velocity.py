"""CPU tests: the C oracle's velocity-field path against the reference's own
velocity-field build (-DVELOCITYFIELD, tests/golden/velocity.npz):

* the particle deposit (Hmaps::CreateOctreeVelocityWithCIC / WithTSC over
  two particle files, then the mass normalisation and the parent fill of
  hmaps.cpp:424-441): every cell's velocity and mass bit-identical;
* whole rays traced with the Doppler, ISW and observer terms in the redshift
  (integrator.h:707-708, 765-767): step counts and every field of the final
  photon records bit-identical.

Plus properties of the restatement: one deposit call equals the same
particles split over files; with zero velocities and no observer velocity
the velocity-field redshift differs from the plain build's by the ISW term
alone."""
import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def vel():
    return load_golden("velocity")


@pytest.fixture(scope="module")
def amr():
    return load_golden("amr")


def _oracle(oracle_mod, amr):
    cos = {"t": amr["cosmo_t"], "a": amr["cosmo_a"], "dadt": amr["cosmo_dadt"]}
    return oracle_mod.Oracle(amr["records"], cos, float(amr["cosmo_length"]))


def test_fixture_octree_is_the_amr_fixture(vel, amr):
    import sys
    from conftest import GOLDEN
    sys.path.insert(0, GOLDEN)
    import make_golden
    assert make_golden.records_sha(amr["records"]) == str(vel["records_sha"])


@pytest.mark.parametrize("scheme", ["cic", "tsc"])
def test_deposit_bit_exact(vel, amr, oracle_mod, scheme):
    O = _oracle(oracle_mod, amr)
    pos, pv, k = vel["part_pos"], vel["part_vel"], int(vel["part_split"])
    O.deposit_velocity(pos[:k], pv[:k], scheme, begin=True, finish=False)
    v, rho = O.deposit_velocity(pos[k:], pv[k:], scheme, begin=False, finish=True)
    np.testing.assert_array_equal(v.view(np.uint32), vel["ref_vel_" + scheme].view(np.uint32))
    np.testing.assert_array_equal(rho.view(np.uint32), vel["ref_rho_" + scheme].view(np.uint32))
    # the parent fill ran: massless cells carry a velocity
    massless = vel["ref_rho_" + scheme] == 0
    if scheme == "cic":
        assert massless.sum() > 10 and np.abs(v[massless]).max() > 0


def test_deposit_split_over_files_equals_one_call(vel, amr, oracle_mod):
    O1, O2 = _oracle(oracle_mod, amr), _oracle(oracle_mod, amr)
    pos, pv = vel["part_pos"], vel["part_vel"]
    v1, r1 = O1.deposit_velocity(pos, pv, "tsc")
    O2.deposit_velocity(pos[:500], pv[:500], "tsc", True, False)
    O2.deposit_velocity(pos[500:1100], pv[500:1100], "tsc", False, False)
    v2, r2 = O2.deposit_velocity(pos[1100:], pv[1100:], "tsc", False, True)
    np.testing.assert_array_equal(v1, v2)
    np.testing.assert_array_equal(r1, r2)


@pytest.mark.parametrize("scheme,order", [("cic", 1), ("tsc", 2)])
def test_rays_with_doppler_bit_exact(vel, amr, oracle_mod, scheme, order):
    O = _oracle(oracle_mod, amr)
    O.fields[:, 0] = vel["ref_rho_" + scheme]
    O.set_velocity(vel["ref_vel_" + scheme], vel["vobs"])
    steps, final, _ = O.propagate(vel["launch"], order=order, nsteps=int(vel["nsteps"]), stop="redshift",
                                  stop_ref=float(vel["zs"][-1]), jacobian=False)
    np.testing.assert_array_equal(steps, vel["ref_steps_o%d" % order])
    np.testing.assert_array_equal(final.view(np.uint64), vel["ref_final_o%d" % order].view(np.uint64))


def test_zero_velocity_field_adds_the_isw_term(vel, amr, oracle_mod):
    """a0/a (1 + phi0/c^2 - phi/c^2 + isw) - 1 against a0/a (1 + phi0/c^2 - phi/c^2) - 1
    on the same trajectory (fixed step count: the stop is the radius)."""
    plain = _oracle(oracle_mod, amr)
    velo = _oracle(oracle_mod, amr)
    velo.set_velocity(np.zeros((amr["records"].shape[0], 3), np.float32), (0.0, 0.0, 0.0))
    launch = vel["launch"][:16]
    s0, f0, _ = plain.propagate(launch, order=2, nsteps=8, stop="r", stop_ref=0.3, jacobian=False)
    s1, f1, _ = velo.propagate(launch, order=2, nsteps=8, stop="r", stop_ref=0.3, jacobian=False)
    np.testing.assert_array_equal(s0, s1)
    np.testing.assert_array_equal(f0[:, :19], f1[:, :19])       # the trajectory itself is unchanged
    a0 = 1.0
    isw_term = a0 / f1[:, 0] * f1[:, 22]
    assert np.abs(f1[:, 22]).max() > 0
    np.testing.assert_allclose(f1[:, 19] - f0[:, 19], isw_term, rtol=1e-6, atol=1e-15)
