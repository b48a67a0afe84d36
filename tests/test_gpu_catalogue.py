"""Catalogue root-finder on the GPU (mpf_catalogue_newton) against the
reference's own Catalogues::iterateNewtonMethod rows in tests/golden.

Column layout (relCat, catalogues.h:840-855): 0-1 comoving phi theta, 2-3
observed phi theta, 4 miss, 5 rays used (42: rejected), 6-11 redshifts,
12-15 the Jacobian.

Exact mode follows the reference's float64 operation order, but the device's
trigonometric functions (launch direction, Newton update, Jacobian angles) are
not glibc's, and the lensing Jacobian is accumulated as two separable sums, so
rows agree to rounding, not bit for bit: angles to 1e-12 rad, redshifts to
1e-12, Jacobian entries to 1e-10.  Fast mode (FP32 gathers) agrees to 1e-9
rad, 1e-8 in redshift and 1e-7 in the Jacobian.  Integer outcomes (which
sources fail, their firstid, how many rays a source needs) are compared
exactly, except at cat_accuracy = 1e-13 where the miss sits at the float64
rounding floor and a source may need one ray more or less.
"""
import numpy as np
import pytest

from conftest import load_golden

pytestmark = pytest.mark.gpu

TOL = {True: dict(angle=1e-12, miss=1e-13, z=1e-12, jac=1e-10),
       False: dict(angle=1e-9, miss=1e-9, z=1e-8, jac=1e-7)}


@pytest.fixture(scope="module", params=["uniform", "amr"])
def cat_setup(request, gpu_lib, pkg):
    g = load_golden(request.param)
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    return g, tree, cos


def _run(pkg, g, tree, cos, order, exact, acc, src=None, rotm1=None, jacobian="infinitesimal"):
    return pkg.catalogue(tree, cos, g["cat_src"] if src is None else src, float(g["cosmo_length"]),
                         float(g["cosmo_h"]), float(g["cosmo_mpc"]), cat_accuracy=acc, nsteps=int(g["nsteps"]),
                         order=order, vobs=g["cat_vobs"], rotm1=rotm1, exact=exact, jacobian=jacobian)


def _compare(got, ref, exact, allow_count_mismatch=0):
    tol = TOL[exact]
    failed = ref[:, 2] == 42
    np.testing.assert_array_equal(got[:, 2] == 42, failed)
    # unreachable sources: firstid and zero miss as the reference writes them
    np.testing.assert_array_equal(got[failed, 5], ref[failed, 5])
    assert np.all(got[failed, 4] == 0)
    # comoving first guess: atan2 / acos of the source position
    assert np.abs(got[:, :2] - ref[:, :2]).max() <= 1e-15
    same = ~failed & (got[:, 5] == ref[:, 5])
    assert (~failed).sum() - same.sum() <= allow_count_mismatch, (got[~failed, 5], ref[~failed, 5])
    assert np.abs(got[same, 2:4] - ref[same, 2:4]).max(initial=0) <= tol["angle"]
    assert np.abs(got[same, 4] - ref[same, 4]).max(initial=0) <= tol["miss"]
    conv = same & (ref[:, 5] != 42)
    assert np.abs(got[conv, 6:12] - ref[conv, 6:12]).max(initial=0) <= tol["z"]
    # the interpolated redshift is written at every round that reached the source
    assert np.abs(got[same, 7] - ref[same, 7]).max(initial=0) <= tol["z"]
    assert np.abs(got[same, 12:16] - ref[same, 12:16]).max(initial=0) <= tol["jac"]
    return same.sum()


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
def test_catalogue_matches_reference(cat_setup, pkg, order, exact):
    g, tree, cos = cat_setup
    for ia, acc in enumerate(g["cat_accuracy"]):
        ref = g["ref_cat_o%d_a%d" % (order, ia)]
        if not exact and acc < 1e-9:
            continue   # FP32 gathers: the miss floor is above 1e-13
        rows, stats, rc = _run(pkg, g, tree, cos, order, exact, float(acc))
        assert rc == 0
        allow = 3 if acc == 1e-13 else 0
        n_same = _compare(rows, ref, exact, allow)
        assert n_same >= 30
        assert stats["rays"] >= (ref[:, 2] != 42).sum() and stats["photon_steps"] > 0
        assert 1 <= stats["iterations"] <= 11


@pytest.mark.parametrize("exact", [True, False])
def test_catalogue_rotated_frame(cat_setup, pkg, exact):
    g, tree, cos = cat_setup
    rows, _, rc = _run(pkg, g, tree, cos, 2, exact, float(g["cat_accuracy"][0]), src=g["cat_src_rotated"],
                       rotm1=g["cat_rotm1"])
    assert rc == 0
    ref = g["ref_cat_rot_o2"]
    tol = TOL[exact]
    failed = ref[:, 2] == 42
    np.testing.assert_array_equal(rows[:, 2] == 42, failed)
    np.testing.assert_array_equal(rows[~failed, 5], ref[~failed, 5])
    assert np.abs(rows[~failed, 2:4] - ref[~failed, 2:4]).max() <= tol["angle"]
    assert np.abs(rows[~failed, 6:12] - ref[~failed, 6:12]).max() <= tol["z"]


def test_catalogue_eight_column_sources_and_edges(gpu_lib, pkg):
    """The reference's 8-column source rows (id and npart after the velocity)
    give the same result; a source at the observer is unreachable; an empty
    batch is fine; a stride below 6 is refused."""
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    src6 = g["cat_src"][:8].copy()
    src8 = np.concatenate([src6, np.arange(8.0)[:, None] * 1000, np.full((8, 1), 64.0)], axis=1)
    src8[3, :3] = 0.0
    src6[3, :3] = 0.0
    r6, _, _ = _run(pkg, g, tree, cos, 2, True, 1e-8, src=src6)
    r8, _, _ = _run(pkg, g, tree, cos, 2, True, 1e-8, src=src8)
    np.testing.assert_array_equal(r6.view(np.uint64), r8.view(np.uint64))
    assert r6[3, 2] == 42 and r6[3, 3] == 42
    rows, stats, rc = _run(pkg, g, tree, cos, 2, True, 1e-8, src=np.zeros((0, 6)))
    assert rc == 0 and rows.shape == (0, 16) and stats["rays"] == 0
    with pytest.raises(ValueError):
        _run(pkg, g, tree, cos, 2, True, 1e-8, src=np.zeros((4, 5)))


def test_catalogue_larger_batch_against_oracle(gpu_lib, pkg, oracle_mod):
    """512 seeded sources on the AMR fixture: exact mode against the C oracle
    (itself bit-exact with the reference)."""
    g = load_golden("amr")
    tree = pkg.Octree.from_records(g["records"])
    cos = pkg.Cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"])
    rng = np.random.default_rng(99)
    n = 512
    d = rng.uniform(0.03, 0.45, n)
    ph = np.radians(rng.uniform(-2.2, 2.2, n))
    th = np.pi / 2 + np.radians(rng.uniform(-2.2, 2.2, n))
    src = np.stack([d * np.cos(ph) * np.sin(th), d * np.sin(ph) * np.sin(th), d * np.cos(th)], axis=1)
    src = np.concatenate([src, rng.normal(0, 1e-3, (n, 3))], axis=1)
    O = oracle_mod.Oracle(g["records"], {k: g["cosmo_" + k] for k in ("t", "a", "dadt")}, float(g["cosmo_length"]))
    for order in (1, 2):
        ref = O.catalogue(src, order=order, nsteps=int(g["nsteps"]), cat_accuracy=1e-8, h=float(g["cosmo_h"]),
                          mpc=float(g["cosmo_mpc"]), vobs=g["cat_vobs"])
        rows, _, rc = _run(pkg, g, tree, cos, order, True, 1e-8, src=src)
        assert rc == 0
        _compare(rows, ref, True, 0)


OPENING = 0.2 / 60.0 * 3.141592653589793 / 180.0


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("plane,stop_bundle", [("sachs", "redshift"), ("normal", "r"), ("sachs", "plane"), ("normal", "plane")])
def test_catalogue_bundle_matches_reference(cat_setup, pkg, order, exact, plane, stop_bundle):
    """jacobiantype = bundle: four-ray Jacobians from the sixth ray on and at
    convergence.  The finite difference over a 0.2 arcmin screen divides ray
    position errors by ~6e-5 of the distance, so the Jacobian columns agree to
    1e-6 (exact) / 1e-2 (fast); angles and redshifts as in the infinitesimal
    case (the Newton iteration converges to the same root)."""
    g, tree, cos = cat_setup
    for ia in (0, 2):
        acc = float(g["cat_accuracy"][ia])
        rows, stats, rc = pkg.catalogue(tree, cos, g["cat_src"], float(g["cosmo_length"]), float(g["cosmo_h"]),
                                        float(g["cosmo_mpc"]), cat_accuracy=acc, nsteps=int(g["nsteps"]), order=order,
                                        vobs=g["cat_vobs"], exact=exact, jacobian="bundle", plane=plane,
                                        stop_bundle=stop_bundle, openingmin=OPENING)
        assert rc == 0
        ref = g["ref_cat_bundle_o%d_a%d_%s_%s" % (order, ia, plane, stop_bundle)]
        tol = TOL[exact]
        failed = ref[:, 2] == 42
        np.testing.assert_array_equal(rows[:, 2] == 42, failed)
        np.testing.assert_array_equal(rows[failed, 5], ref[failed, 5])
        same = ~failed & (rows[:, 5] == ref[:, 5])
        assert (~failed).sum() - same.sum() <= 0
        # rejected sources went through 6 bundle Newton steps: the angle error is the Jacobian's times the miss
        atol = tol["angle"] if ia == 0 else (1e-10 if exact else 1e-8)
        assert np.abs(rows[same, 2:4] - ref[same, 2:4]).max(initial=0) <= atol
        conv = same & (ref[:, 5] != 42)
        assert np.abs(rows[conv, 6:12] - ref[conv, 6:12]).max(initial=0) <= tol["z"]
        jtol = 1e-6 if exact else 1e-2
        assert np.abs(rows[same, 12:16] - ref[same, 12:16]).max(initial=0) <= jtol
        assert stats["rays"] > (~failed).sum()


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
def test_catalogue_born_matches_reference(cat_setup, pkg, order, exact):
    """jacobiantype = infinitesimal_born: the Newton rounds as "infinitesimal",
    the converged rows' Jacobian along the Born ray of the observed direction
    (catalogues.h:670-673), traced by the Born instantiation of each mode's kernel."""
    g, tree, cos = cat_setup
    for ia in (0, 1):
        acc = float(g["cat_accuracy"][ia])
        if not exact and acc < 1e-9:
            continue
        ref = g["ref_cat_born_o%d_a%d" % (order, ia)]
        rows, stats, rc = _run(pkg, g, tree, cos, order, exact, acc, jacobian="infinitesimal_born")
        assert rc == 0
        assert _compare(rows, ref, exact, 3 if acc == 1e-13 else 0) >= 30
        # the Born Jacobian is not the traced ray's
        plain = g["ref_cat_o%d_a%d" % (order, ia)]
        conv = (ref[:, 5] != 42) & (ref[:, 2] != 42)
        assert np.abs(ref[conv, 12:16] - plain[conv, 12:16]).max() > 1e-9


@pytest.mark.parametrize("exact", [True, False])
def test_catalogue_ngp_matches_reference(cat_setup, pkg, exact):
    """ORDER = 0: the catalogue of the reference built with NGP gathers (the
    rays run through the float64 kernel in both modes)."""
    g, tree, cos = cat_setup
    rows, stats, rc = _run(pkg, g, tree, cos, 0, exact, float(g["cat_accuracy"][0]))
    assert rc == 0
    assert _compare(rows, g["ref_cat_o0_a0"], True) >= 30


def test_catalogue_work_queue_plan_reuse(cat_setup, pkg):
    """Fast mode runs as one persistent launch fed by a device work queue,
    from a CUDA graph kept per stream and reused by later calls with at most
    as many sources; a larger batch builds it again.  A source's rays do not
    depend on the other sources of the call, so its row is bit-identical
    whatever the batch: the first call, a smaller one reusing the plan, and a
    batch beyond the plan's capacity holding the same sources many times."""
    g, tree, cos = cat_setup
    src = g["cat_src"]
    ref, st, _ = _run(pkg, g, tree, cos, 2, False, 1e-8)
    assert st["kernel_launches"] == 28         # one graph: set-up, 8 sort passes of 3 kernels, fill, persistent kernel
    assert st["rays"] >= src.shape[0]
    small, _, _ = _run(pkg, g, tree, cos, 2, False, 1e-8, src=src[:13])
    np.testing.assert_array_equal(small.view(np.uint64), ref[:13].view(np.uint64))
    reps = (1 << 16) // src.shape[0] + 2
    big, st_big, _ = _run(pkg, g, tree, cos, 2, False, 1e-8, src=np.tile(src, (reps, 1)))
    np.testing.assert_array_equal(big.view(np.uint64), np.tile(ref, (reps, 1)).view(np.uint64))
    assert st_big["rays"] == reps * st["rays"]
