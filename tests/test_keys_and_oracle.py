"""CPU tests: the key arithmetic and the C oracle against the reference's own
outputs recorded in tests/golden (bit-exact)."""
import numpy as np
import pytest


def test_keys_match_reference(golden, synth):
    for lvl, pos, ref in zip(golden["key_level"], golden["key_pos"], golden["key_ref"]):
        hi, lo = synth.compute_key(int(lvl), pos[None])
        assert (int(hi[0]), int(lo[0])) == (int(ref[0]), int(ref[1])), (lvl, pos)
    hi, lo = golden["records"]["hi"], golden["records"]["lo"]
    lev = synth.key_level(hi, lo)
    assert lev.min() >= 0 and lev.max() <= 32
    # records strictly increasing by key (the reference's sorted container)
    assert np.all((hi[1:] > hi[:-1]) | ((hi[1:] == hi[:-1]) & (lo[1:] > lo[:-1])))


def _oracle(golden, oracle_mod):
    cos = {k: golden["cosmo_" + k] for k in ("t", "a", "dadt")}
    return oracle_mod.Oracle(golden["records"], cos, float(golden["cosmo_length"]))


def test_oracle_gathers_bit_exact(golden, oracle_mod):
    O = _oracle(golden, oracle_mod)
    pts = golden["pts"]
    np.testing.assert_array_equal(O.locate(pts), golden["ref_locate"])
    np.testing.assert_array_equal(O.cic(pts).view(np.uint32), golden["ref_cic"].view(np.uint32))
    np.testing.assert_array_equal(O.tsc(pts).view(np.uint32), golden["ref_tsc"].view(np.uint32))


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_integrate_bit_exact(golden, oracle_mod, order):
    O = _oracle(golden, oracle_mod)
    steps, final, _ = O.propagate(golden["launch"], order=order, nsteps=int(golden["nsteps"]), stop="redshift",
                                  stop_ref=float(golden["zs"][-1]))
    np.testing.assert_array_equal(steps, golden["ref_steps_o%d" % order])
    np.testing.assert_array_equal(final.view(np.uint64), golden["ref_final_o%d" % order].view(np.uint64))


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_maps_bit_exact(golden, oracle_mod, maps_mod, order):
    O = _oracle(golden, oracle_mod)
    dirs = golden["pixel_dirs"]
    launch = np.zeros((dirs.shape[0], 6))
    launch[:, 3:] = dirs
    _, _, planes = O.propagate(launch, order=order, nsteps=int(golden["nsteps"]), stop="redshift",
                               planes=golden["zs"], jacobian=True)
    comps = str(golden["components"]).split(",")
    maps = maps_mod.assemble(planes, dirs, golden["homogeneous"], comps)
    ref = golden["ref_maps_o%d" % order]
    assert maps.shape == ref.shape
    np.testing.assert_array_equal(maps.view(np.uint32), ref.view(np.uint32))


BUNDLES = (("sachs", "redshift"), ("normal", "r"), ("sachs", "plane"), ("normal", "plane"))
OPENING = 0.2 / 60.0 * 3.141592653589793 / 180.0


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("plane,stop_bundle", BUNDLES)
def test_oracle_bundle_maps_bit_exact(golden, oracle_mod, maps_mod, order, plane, stop_bundle):
    """FillMap with jacobiantype = bundle (Lensing::dbetadtheta): the oracle's
    surfaces and four-ray Jacobians, assembled into maps, equal the reference's."""
    O = _oracle(golden, oracle_mod)
    dirs = golden["pixel_dirs"]
    launch = np.zeros((dirs.shape[0], 6))
    launch[:, 3:] = dirs
    planes, jac = O.bundle(launch, golden["zs"], order=order, nsteps=int(golden["nsteps"]), stop="redshift",
                           plane=plane, stop_bundle=stop_bundle, openingmin=OPENING)
    comps = str(golden["components"]).split(",")
    maps = maps_mod.assemble(planes, dirs, golden["homogeneous"], comps, bundle_jac=jac)
    ref = golden["ref_maps_bundle_o%d_%s_%s" % (order, plane, stop_bundle)]
    assert maps.shape == ref.shape
    np.testing.assert_array_equal(maps.view(np.uint32), ref.view(np.uint32))


@pytest.mark.parametrize("order", [1, 2])
def test_oracle_catalogue_bit_exact(golden, oracle_mod, order):
    """Catalogue rows (Newton root-finder) of the C oracle == the reference's
    iterateNewtonMethod at three accuracies, and through a frame rotation."""
    O = _oracle(golden, oracle_mod)
    kw = dict(order=order, nsteps=int(golden["nsteps"]), h=float(golden["cosmo_h"]), mpc=float(golden["cosmo_mpc"]),
              vobs=golden["cat_vobs"])
    for ia, acc in enumerate(golden["cat_accuracy"]):
        rows = O.catalogue(golden["cat_src"], cat_accuracy=float(acc), **kw)
        np.testing.assert_array_equal(rows.view(np.uint64), golden["ref_cat_o%d_a%d" % (order, ia)].view(np.uint64))
    rows = O.catalogue(golden["cat_src_rotated"], cat_accuracy=float(golden["cat_accuracy"][0]),
                       rotm1=golden["cat_rotm1"], **kw)
    np.testing.assert_array_equal(rows.view(np.uint64), golden["ref_cat_rot_o%d" % order].view(np.uint64))


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("plane,stop_bundle", BUNDLES)
def test_oracle_catalogue_bundle_bit_exact(golden, oracle_mod, order, plane, stop_bundle):
    """jacobiantype = bundle: the Newton rounds from iteration 5 and the final
    Jacobian use Lensing::dbetadtheta; the oracle's rows equal the reference's."""
    O = _oracle(golden, oracle_mod)
    kw = dict(order=order, nsteps=int(golden["nsteps"]), h=float(golden["cosmo_h"]), mpc=float(golden["cosmo_mpc"]),
              vobs=golden["cat_vobs"], jacobiantype="bundle", plane=plane, stop_bundle=stop_bundle, openingmin=OPENING)
    for ia in (0, 2):
        rows = O.catalogue(golden["cat_src"], cat_accuracy=float(golden["cat_accuracy"][ia]), **kw)
        ref = golden["ref_cat_bundle_o%d_a%d_%s_%s" % (order, ia, plane, stop_bundle)]
        np.testing.assert_array_equal(rows.view(np.uint64), ref.view(np.uint64))


def test_catalogue_fixture_covers_every_outcome(golden):
    """The fixture holds converged (2-4 rays, so the infinitesimal-Jacobian
    steps run), rejected (42 after 11 rays) and failed (phi = theta = 42) sources."""
    r8 = golden["ref_cat_o2_a0"]
    r13 = golden["ref_cat_o2_a1"]
    r0 = golden["ref_cat_o2_a2"]
    failed = r8[:, 2] == 42
    assert 1 <= failed.sum() < r8.shape[0] // 2
    assert np.all(r8[~failed, 5] >= 2) and np.all(r8[~failed, 5] <= 3)
    assert np.any(r13[~failed, 5] == 4)
    assert np.all(r0[~failed, 5] == 42)
    # converged rows carry a Jacobian near the identity and six redshifts
    assert np.all(np.abs(r8[~failed, 12] - 1) < 1e-2) and np.all(r8[~failed, 6] > 0)


def test_amr_fixture_exercises_levels(synth):
    from conftest import load_golden
    g = load_golden("amr")
    lev = synth.key_level(g["records"]["hi"], g["records"]["lo"])
    assert lev.max() - lev.min() >= 3
    # some reference rays end in refined cells and some are longer than uniform ones
    assert len(np.unique(g["ref_final_o2"][:, 9])) >= 2


def test_oracle_ngp_bit_exact(golden, oracle_mod, maps_mod):
    """ORDER = 0 (nearest grid point): the oracle's point gathers, rays, maps
    and catalogue rows equal those of the reference built at ORDER=0."""
    O = _oracle(golden, oracle_mod)
    np.testing.assert_array_equal(O.ngp(golden["pts"]).view(np.uint32), golden["ref_ngp"].view(np.uint32))
    n = int(golden["nsteps"])
    steps, final, _ = O.propagate(golden["launch"], order=0, nsteps=n, stop="redshift", stop_ref=float(golden["zs"][-1]))
    np.testing.assert_array_equal(steps, golden["ref_steps_o0"])
    np.testing.assert_array_equal(final.view(np.uint64), golden["ref_final_o0"].view(np.uint64))
    dirs = golden["pixel_dirs"]
    launch = np.zeros((dirs.shape[0], 6))
    launch[:, 3:] = dirs
    _, _, planes = O.propagate(launch, order=0, nsteps=n, stop="redshift", planes=golden["zs"], jacobian=True)
    maps = maps_mod.assemble(planes, dirs, golden["homogeneous"], str(golden["components"]).split(","))
    np.testing.assert_array_equal(maps.view(np.uint32), golden["ref_maps_o0"].view(np.uint32))
    rows = O.catalogue(golden["cat_src"], cat_accuracy=float(golden["cat_accuracy"][0]), order=0, nsteps=n,
                       h=float(golden["cosmo_h"]), mpc=float(golden["cosmo_mpc"]), vobs=golden["cat_vobs"])
    np.testing.assert_array_equal(rows.view(np.uint64), golden["ref_cat_o0_a0"].view(np.uint64))


def test_oracle_born_bit_exact(golden, oracle_mod, maps_mod):
    """lensing_born (hmaps.h:706-712, 771-785) and jacobiantype =
    infinitesimal_born (catalogues.h:670-673): the oracle's Order = -1 rays and
    the Jacobian along them give the reference's Born map rows and catalogue
    rows bit for bit."""
    O = _oracle(golden, oracle_mod)
    n = int(golden["nsteps"])
    dirs = golden["pixel_dirs"]
    launch = np.zeros((dirs.shape[0], 6))
    launch[:, 3:] = dirs
    size, A = O.born(launch, golden["homogeneous"][:, 1], nsteps=n, stop="redshift", stop_ref=float(golden["zs"][-1]))
    a11, a12, a22 = A[..., 0], A[..., 1], A[..., 2]
    born = np.stack([1 - (a11 + a22) * 0.5, -0.5 * (a11 - a22), -a12, a11 * a22 - a12 * a12], axis=0)  # 4 x npix x nz
    ref = golden["ref_maps_bornonly_o2"]                                                                # nz x 4 x npix
    got = np.where((size > 1)[None, :, None], born, 0.0).transpose(2, 0, 1).astype(np.float32)
    np.testing.assert_array_equal(got.view(np.uint32), ref.view(np.uint32))
    for ia in (0, 1):
        rows = O.catalogue(golden["cat_src"], cat_accuracy=float(golden["cat_accuracy"][ia]), order=1, nsteps=n,
                           h=float(golden["cosmo_h"]), mpc=float(golden["cosmo_mpc"]), vobs=golden["cat_vobs"],
                           jacobiantype="infinitesimal_born")
        np.testing.assert_array_equal(rows.view(np.uint64), golden["ref_cat_born_o1_a%d" % ia].view(np.uint64))
