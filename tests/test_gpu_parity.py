"""GPU parity: the CUDA path (through the C ABI) against the reference's
outputs recorded in tests/golden and against the C oracle.

Tolerances:
  exact mode (reference float64 order): cell indices, CIC/TSC fields, step
    counts and every field of the final photon record are bit-identical;
    surface values other than the Jacobian are bit-identical; the Jacobian
    (re-associated into running sums, CUDA trig) within 1e-9 relative of
    |A - 1| + 1e-13 absolute.
  fast mode (FP32 gather arithmetic): fields within 2e-6 relative of the
    field's scale; redshift and deflection within 1e-6 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev(gpu_lib, pkg, golden):
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    yield tree, cos
    tree.close()
    cos.close()


def test_octree_info(dev, golden, synth):
    tree, _ = dev
    info = tree.info
    lev = synth.key_level(golden["records"]["hi"], golden["records"]["lo"])
    assert info["cells"] == golden["records"].shape[0]
    assert info["level_min"] == lev.min() and info["level_max"] == lev.max()
    assert info["nodes"] >= info["cells"]


def test_locate_bit_exact(dev, golden):
    tree, _ = dev
    np.testing.assert_array_equal(tree.locate(golden["pts"]), golden["ref_locate"])


def test_cic_tsc_exact_bit_exact(dev, golden):
    tree, _ = dev
    np.testing.assert_array_equal(tree.cic(golden["pts"], exact=True).view(np.uint32), golden["ref_cic"].view(np.uint32))
    np.testing.assert_array_equal(tree.tsc(golden["pts"], exact=True).view(np.uint32), golden["ref_tsc"].view(np.uint32))


def test_cic_tsc_fast_within_tolerance(dev, golden):
    tree, _ = dev
    for got, ref in ((tree.cic(golden["pts"], exact=False), golden["ref_cic"]),
                     (tree.tsc(golden["pts"], exact=False), golden["ref_tsc"])):
        np.testing.assert_array_equal(got == 0, ref == 0)   # same empty / non-empty pattern
        scale = np.abs(ref).max(axis=0) + 1e-30
        assert np.all(np.abs(got - ref) <= 2e-6 * scale[None, :] + 1e-30)


@pytest.mark.parametrize("order", [1, 2])
def test_propagate_exact_bit_exact(dev, golden, pkg, order):
    tree, cos = dev
    steps, final, _, rc = pkg.propagate(tree, cos, golden["launch"], float(golden["cosmo_length"]),
                                        nsteps=int(golden["nsteps"]), order=order, stop="redshift",
                                        stop_value=float(golden["zs"][-1]), exact=True, jacobian=False)
    assert rc == 0
    np.testing.assert_array_equal(steps, golden["ref_steps_o%d" % order])
    np.testing.assert_array_equal(final.view(np.uint64), golden["ref_final_o%d" % order].view(np.uint64))


def _deflection(launch, final):
    """Angle between the launch direction and the final position, accurate
    for small angles (atan2 of the cross and dot products)."""
    d = launch[:, 3:]
    x = final[:, 2:5]
    return np.arctan2(np.linalg.norm(np.cross(d, x), axis=1), np.sum(d * x, axis=1))


@pytest.mark.parametrize("order", [1, 2])
def test_propagate_fast_within_tolerance(dev, golden, pkg, order):
    tree, cos = dev
    steps, final, _, rc = pkg.propagate(tree, cos, golden["launch"], float(golden["cosmo_length"]),
                                        nsteps=int(golden["nsteps"]), order=order, stop="redshift",
                                        stop_value=float(golden["zs"][-1]), exact=False, jacobian=False)
    ref_steps, ref = golden["ref_steps_o%d" % order], golden["ref_final_o%d" % order]
    assert np.all(np.abs(steps - ref_steps) <= 1)
    same = steps == ref_steps
    assert same.mean() > 0.95
    z, zr = final[same, 19], ref[same, 19]
    assert np.all(np.abs(z - zr) <= 1e-6 * np.abs(zr))
    dg, dr = _deflection(golden["launch"][same], final[same]), _deflection(golden["launch"][same], ref[same])
    assert np.all(np.abs(dg - dr) <= 1e-6 * np.abs(dr) + 1e-13)


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
def test_maps_against_reference_fillmap(dev, golden, pkg, maps_mod, order, exact):
    tree, cos = dev
    dirs = golden["pixel_dirs"]
    launch = np.zeros((dirs.shape[0], 6))
    launch[:, 3:] = dirs
    _, _, planes, rc = pkg.propagate(tree, cos, launch, float(golden["cosmo_length"]), nsteps=int(golden["nsteps"]),
                                     order=order, stop="redshift", planes=golden["zs"], jacobian=True, exact=exact)
    comps = str(golden["components"]).split(",")
    got = maps_mod.assemble(planes, dirs, golden["homogeneous"], comps)
    ref = golden["ref_maps_o%d" % order]
    assert got.shape == ref.shape
    # the steps row (firstid) is >= 1 exactly where the surface was valid, 0 elsewhere
    assert comps[0] == "lensing"
    srow = 4 + comps.index("steps") - 1          # lensing fills rows 0-3, one row per component after it
    valid_ref = ref[:, srow] != 0
    valid_got = got[:, srow] != 0
    np.testing.assert_array_equal(valid_got, valid_ref)
    # lensing rows: kappa gamma1 gamma2 (small) and 1/mu (~1)
    for row, tol in ((0, 1e-9), (1, 1e-9), (2, 1e-9), (3, 1e-9)):
        scale = np.abs(ref[:, row]).max() + 1e-12
        tol_abs = (1e-6 if not exact else 1e-9) * max(scale, 1e-6)
        assert np.abs(got[:, row] - ref[:, row]).max() <= tol_abs + 2e-7 * (row == 3), (row, exact)
    # remaining rows: exact mode bit-identical except the angle rows; fast mode 1e-6 relative
    for row in range(4, ref.shape[1]):
        if exact and row < ref.shape[1] - 2:
            np.testing.assert_array_equal(got[:, row].view(np.uint32), ref[:, row].view(np.uint32), err_msg=str(row))
        else:
            # dz is ~1e-16 by construction (the surface is a redshift): absolute floor
            scale = np.abs(ref[:, row]).max() + 1e-30
            assert np.abs(got[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row


def test_against_oracle_larger_batch(gpu_lib, pkg, oracle_mod, synth):
    """GPU exact mode == C oracle on a finer ray grid over the AMR fixture."""
    from conftest import load_golden
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    O = oracle_mod.Oracle(g["records"], {k: g["cosmo_" + k] for k in ("t", "a", "dadt")}, float(g["cosmo_length"]))
    launch = synth.photon_grid(48, 2.4, 2.4)
    for order in (1, 2):
        s_ref, f_ref, _ = O.propagate(launch, order=order, nsteps=8, stop="redshift", stop_ref=0.2)
        s, f, _, _ = pkg.propagate(tree, cos, launch, float(g["cosmo_length"]), nsteps=8, order=order,
                                   stop="redshift", stop_value=0.2, exact=True, jacobian=False)
        np.testing.assert_array_equal(s, s_ref)
        np.testing.assert_array_equal(f.view(np.uint64), f_ref.view(np.uint64))


def test_edge_cases(gpu_lib, pkg, oracle_mod, golden):
    """Rays that leave the data at once, rays starting outside the octree,
    zero rays, and the max_steps warning."""
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    O = oracle_mod.Oracle(golden["records"], {k: golden["cosmo_" + k] for k in ("t", "a", "dadt")},
                          float(golden["cosmo_length"]))
    L = float(golden["cosmo_length"])
    launch = np.array([[0, 0, 0, -1, 0, 0],         # away from the cone: data runs out
                       [0, 0, 0, 0, 0, 1],          # perpendicular
                       [0.0, 0.0, 0.0, 1, 0.01, 0.0]])
    s_ref, f_ref, _ = O.propagate(launch, order=2, nsteps=10, stop="redshift", stop_ref=0.2)
    s, f, _, _ = pkg.propagate(tree, cos, launch, L, nsteps=10, order=2, stop="redshift", stop_value=0.2, exact=True,
                               jacobian=False)
    np.testing.assert_array_equal(s, s_ref)
    np.testing.assert_array_equal(f.view(np.uint64), f_ref.view(np.uint64))
    s0, f0, _, rc = pkg.propagate(tree, cos, np.zeros((0, 6)), L)
    assert rc == 0 and s0.shape == (0,)
    with pytest.raises(Exception):
        pkg.propagate(tree, cos, launch, L, order=3)
    s, f, _, rc = pkg.propagate(tree, cos, launch[2:], L, nsteps=10, order=2, stop="redshift", stop_value=0.2,
                                max_steps=5)
    assert rc == 1 and s[0] <= 6


def test_unsorted_records_are_refused(gpu_lib, pkg, golden):
    """The upload checks the key order the reference's binary searches rely
    on: two swapped records give MPF_NOT_SORTED, not a wrong octree."""
    import ctypes
    rec = np.array(golden["records"]).copy()
    rec[[10, 11]] = rec[[11, 10]]
    L = pkg.library()
    h = ctypes.c_void_p()
    assert L.mpf_octree_upload(ctypes.c_void_p(rec.ctypes.data), rec.shape[0], ctypes.byref(h)) == -4
    assert not h.value


# ORDER = 0 (nearest grid point, simplehyperoctree.h:1396-1401): the reference
# built with it gives the fixture's ref_*_o0 entries; NGP has no interpolation
# arithmetic, so both modes run the float64 kernel and match bit for bit.
def test_ngp_bit_exact(dev, golden):
    tree, _ = dev
    np.testing.assert_array_equal(tree.ngp(golden["pts"]).view(np.uint32), golden["ref_ngp"].view(np.uint32))


@pytest.mark.parametrize("exact", [True, False])
def test_propagate_ngp_bit_exact(dev, golden, pkg, exact):
    tree, cos = dev
    steps, final, _, rc = pkg.propagate(tree, cos, golden["launch"], float(golden["cosmo_length"]),
                                        nsteps=int(golden["nsteps"]), order=0, stop="redshift",
                                        stop_value=float(golden["zs"][-1]), exact=exact, jacobian=False)
    assert rc == 0
    np.testing.assert_array_equal(steps, golden["ref_steps_o0"])
    np.testing.assert_array_equal(final.view(np.uint64), golden["ref_final_o0"].view(np.uint64))
