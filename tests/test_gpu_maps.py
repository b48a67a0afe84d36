"""Map filling on the GPU (mpf_hmaps_fill: pixels in, float map rows out)
against the reference's own Hmaps::FillMap maps in tests/golden.

The device computes the RING pixel centres itself; they agree with the
harness's pix2vec_ring (the same published formulas with glibc's cos / sin)
to 4e-16, so exact-mode rays start a few ulps apart from the reference's and
the maps are compared with the fast-mode tolerances: the validity pattern
exactly, lensing rows within 1e-6 of their scale, the other rows within
2e-6 of their scale plus 1e-12."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pix2vec_matches_harness(gpu_lib, pkg, golden):
    v = pkg.pix2vec_ring(int(golden["nside"]), golden["pixels"])
    assert np.abs(v - golden["pixel_dirs"]).max() <= 4e-16
    # pixels over the whole sphere: unit vectors, and the ring latitudes of the scheme
    nside = 8
    allv = pkg.pix2vec_ring(nside, np.arange(12 * nside * nside))
    assert np.allclose(np.linalg.norm(allv, axis=1), 1.0, atol=1e-15)
    assert np.unique(np.round(allv[:, 2], 12)).shape[0] == 4 * nside - 1
    assert abs(allv[:, 2].mean()) < 1e-12     # equal-area pixels: zero mean z


def test_pix2vec_known_centres(gpu_lib, pkg):
    """RING pixel centres that the HEALPix scheme fixes (Gorski et al. 2005,
    ApJ 622, 759, the base tessellation of its Fig. 3): at nside 1 the north
    cap ring at z = 2/3 with phi = pi/4 + k pi/2, the equator at z = 0 with
    phi = k pi/2, the south ring at z = -2/3; at nside 2 the first ring at
    z = 1 - 1/(3 nside^2) = 11/12 and the ring latitudes 2/3, 1/3, 0 after it,
    the equatorial rings alternately shifted by half a pixel."""
    v = pkg.pix2vec_ring(1, np.arange(12))
    z = np.repeat([2.0 / 3.0, 0.0, -2.0 / 3.0], 4)
    phi = np.concatenate([np.pi / 4 + np.arange(4) * np.pi / 2, np.arange(4) * np.pi / 2,
                          np.pi / 4 + np.arange(4) * np.pi / 2])
    np.testing.assert_allclose(v[:, 2], z, atol=1e-15)
    np.testing.assert_allclose(np.mod(np.arctan2(v[:, 1], v[:, 0]), 2 * np.pi), phi, atol=1e-14)
    v2 = pkg.pix2vec_ring(2, np.arange(48))
    # rings: 4 (cap), 8 (cap edge), 8, 8 (equator), 8, 8, 4 pixels
    ring_z = [11.0 / 12.0, 2.0 / 3.0, 1.0 / 3.0, 0.0, -1.0 / 3.0, -2.0 / 3.0, -11.0 / 12.0]
    counts = [4, 8, 8, 8, 8, 8, 4]
    np.testing.assert_allclose(v2[:, 2], np.repeat(ring_z, counts), atol=1e-15)
    ph2 = np.mod(np.arctan2(v2[:, 1], v2[:, 0]), 2 * np.pi)
    np.testing.assert_allclose(ph2[:4], np.pi / 4 + np.arange(4) * np.pi / 2, atol=1e-14)
    np.testing.assert_allclose(ph2[4:12], np.pi / 8 + np.arange(8) * np.pi / 4, atol=1e-14)
    # equatorial rings (z = 1/3, 0, -1/3): shifted by pi/8, not shifted, shifted
    np.testing.assert_allclose(ph2[12:20], np.arange(8) * np.pi / 4, atol=1e-14)
    np.testing.assert_allclose(ph2[20:28], np.pi / 8 + np.arange(8) * np.pi / 4, atol=1e-14)
    np.testing.assert_allclose(ph2[28:36], np.arange(8) * np.pi / 4, atol=1e-14)


@pytest.mark.parametrize("order", [0, 1, 2])
@pytest.mark.parametrize("exact", [True, False])
def test_hmaps_fill_matches_reference_fillmap(gpu_lib, pkg, golden, order, exact):
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    comps = str(golden["components"]).split(",")
    got = pkg.hmaps_fill(tree, cos, int(golden["nside"]), golden["pixels"], golden["zs"], golden["homogeneous"], comps,
                         float(golden["cosmo_length"]), nsteps=int(golden["nsteps"]), order=order, exact=exact)
    ref = golden["ref_maps_o%d" % order]
    assert got.shape == ref.shape
    srow = 4 + comps.index("steps") - 1
    np.testing.assert_array_equal(got[:, srow] != 0, ref[:, srow] != 0)
    for row in range(4):
        scale = max(np.abs(ref[:, row]).max(), 1e-6)
        assert np.abs(got[:, row] - ref[:, row]).max() <= 1e-6 * scale + 2e-7 * (row == 3), row
    for row in range(4, ref.shape[1]):
        scale = np.abs(ref[:, row]).max() + 1e-30
        assert np.abs(got[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row


BUNDLES = (("sachs", "redshift"), ("normal", "r"), ("sachs", "plane"), ("normal", "plane"))
OPENING = 0.2 / 60.0 * 3.141592653589793 / 180.0


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("plane,stop_bundle", BUNDLES)
def test_hmaps_fill_bundle_matches_reference(gpu_lib, pkg, golden, order, exact, plane, stop_bundle):
    """jacobiantype = bundle: the four-ray Jacobian is a finite difference over
    a 0.2 arcmin screen, so position errors are divided by ~6e-5 of the
    distance: exact mode (ulp-level launch differences) agrees to 1e-6 of the
    lensing rows' scale, fast mode (FP32 gathers and FP32 RK4 stage
    corrections: the four rays' end points agree with the float64 ones to
    ~1e-12 relative, ~2e-8 of a Jacobian entry after the division) to 1e-3
    of the scale plus 3e-8.  The rotation w (row 3, the Jacobian's
    antisymmetric part) is second order and several times smaller than kappa
    and gamma; it comes out of the same four rays, so its error is measured
    against the scale of the four Jacobian rows."""
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    comps = str(golden["components"]).split(",")
    got = pkg.hmaps_fill(tree, cos, int(golden["nside"]), golden["pixels"], golden["zs"], golden["homogeneous"], comps,
                         float(golden["cosmo_length"]), nsteps=int(golden["nsteps"]), order=order, exact=exact,
                         jacobian="bundle", plane=plane, stop_bundle=stop_bundle, openingmin=OPENING)
    ref = golden["ref_maps_bundle_o%d_%s_%s" % (order, plane, stop_bundle)]
    assert got.shape == ref.shape
    srow = 5 + comps.index("steps") - 1
    np.testing.assert_array_equal(got[:, srow] != 0, ref[:, srow] != 0)
    tol = 1e-6 if exact else 1e-3
    jac_scale = np.abs(ref[:, :4]).max()
    for row in range(5):
        scale = max(np.abs(ref[:, row]).max(), 1e-9) if row != 3 else jac_scale
        floor = 0.0 if exact else 3e-8
        assert np.abs(got[:, row] - ref[:, row]).max() <= tol * scale + floor + 2e-7 * (row == 4), (row, exact)
    for row in range(5, ref.shape[1]):
        scale = np.abs(ref[:, row]).max() + 1e-30
        assert np.abs(got[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row


# lensing_born (hmaps.h:706-712, 771-785): the Jacobian along each pixel's
# FLRW ray, with the traced ray's rows, alone, and beside the bundle Jacobian
BORN_MAPS = (("born", "lensing,lensing_born,dz,steps", "infinitesimal"), ("bornonly", "lensing_born", "infinitesimal"),
             ("born_bundle", "lensing_born,lensing,dr", "bundle"))


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("exact", [True, False])
@pytest.mark.parametrize("key,comps,jt", BORN_MAPS)
def test_hmaps_fill_born_matches_reference(gpu_lib, pkg, golden, order, exact, key, comps, jt):
    """The Born rows (each mode's Born kernel: float64 gathers, or FP32 ones for
    the Jacobian) agree to 1e-6 of their scale; the other rows
    keep the tolerances of the tests above (bundle rows 1e-3 in fast mode)."""
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    names = comps.split(",")
    got = pkg.hmaps_fill(tree, cos, int(golden["nside"]), golden["pixels"], golden["zs"], golden["homogeneous"], names,
                         float(golden["cosmo_length"]), nsteps=int(golden["nsteps"]), order=order, exact=exact,
                         jacobian=jt, plane="sachs", stop_bundle="redshift", openingmin=OPENING)
    ref = golden["ref_maps_%s_o%d" % (key, order)]
    assert got.shape == ref.shape
    # the zeroed (pixel, surface) pairs agree
    np.testing.assert_array_equal(np.all(got == 0, axis=1), np.all(ref == 0, axis=1))
    row = 0
    for c in names:
        nrow = {"lensing": 5 if jt == "bundle" else 4, "lensing_born": 4, "deflection": 2}.get(c, 1)
        for r in range(row, row + nrow):
            scale = max(np.abs(ref[:, r]).max(), 1e-6)
            if c == "lensing_born" or (c == "lensing" and jt != "bundle"):
                tol = 1e-6 * scale + 2e-7 * (r - row == 3)
            elif c == "lensing":
                if r - row == 3:   # w: against the scale of the four Jacobian rows, as above
                    scale = np.abs(ref[:, row:row + 4]).max()
                tol = 1e-6 * scale if exact else 1e-3 * scale + 3e-8   # the bundle test's tolerances
            else:
                tol = 2e-6 * (np.abs(ref[:, r]).max() + 1e-30) + 1e-12
            assert np.abs(got[:, r] - ref[:, r]).max() <= tol, (c, r, np.abs(got[:, r] - ref[:, r]).max(), tol)
        row += nrow
    tree.close()
    cos.close()


def test_hmaps_fill_large_call_equals_small_calls(gpu_lib, pkg, golden):
    """A call of many pixels (nside 4096: the ~78 000 pixels within 2 degrees
    of the cone's axis, one persistent launch with the autotuned shape) writes
    the same map bits as the same pixels in calls of 4096 pixels (one-warp
    blocks): a pixel's rows do not depend on the batch it is traced in."""
    ns = 4096
    ncap = 2 * ns * (ns - 1)
    # candidate pixels of the equatorial rings near z = 0 and phi = 0, then the exact cut
    rings = np.arange(2 * ns - 300, 2 * ns + 301)
    cols = np.concatenate([np.arange(0, 140), np.arange(4 * ns - 140, 4 * ns)])
    cand = (ncap + (rings[:, None] - ns) * 4 * ns + cols[None, :]).reshape(-1).astype(np.int64)
    v = pkg.pix2vec_ring(ns, cand)
    phi = np.arctan2(v[:, 1], v[:, 0])
    th = np.arccos(v[:, 2])
    sel = (np.abs(phi) < np.radians(2.0)) & (np.abs(th - np.pi / 2) < np.radians(2.0))
    pix = np.sort(cand[sel])
    assert pix.shape[0] >= 65536, pix.shape
    tree = pkg.Octree.from_records(golden["records"])
    cos = pkg.Cosmology(golden["cosmo_t"], golden["cosmo_a"], golden["cosmo_dadt"], golden["cosmo_d2adt2"])
    comps = str(golden["components"]).split(",")
    kw = dict(nsteps=int(golden["nsteps"]), order=2, exact=False)
    whole = pkg.hmaps_fill(tree, cos, ns, pix, golden["zs"], golden["homogeneous"], comps,
                           float(golden["cosmo_length"]), **kw)
    parts = [pkg.hmaps_fill(tree, cos, ns, pix[i:i + 4096], golden["zs"], golden["homogeneous"], comps,
                            float(golden["cosmo_length"]), **kw) for i in range(0, pix.shape[0], 4096)]
    np.testing.assert_array_equal(whole.view(np.uint32), np.concatenate(parts, axis=2).view(np.uint32))
    tree.close()
    cos.close()
