"""Generate the golden fixtures of the photon-propagation path by running the
reference's own code (oracle/ref_harness.cpp built by oracle/build_ref.sh from
the reference sources) on seeded synthetic inputs.

Run in a container that has the reference sources:
    ./oracle/build_ref.sh && python tests/golden/make_golden.py

Each fixture holds the octree records it was computed on (so the GPU machine,
which has no reference, reads exactly the same bytes), the cosmology table
the reference derived from its evolution file (Input::acquire + correct), and
the reference's outputs: locate / cic / tsc at random points, per-ray step
counts and final photon records (Integrator::integrate), FillMap maps, and
catalogue rows (Catalogues::iterateNewtonMethod through relCat's per-source
setup) for seeded sources at three accuracies, with and without a rotation,
and FillMap maps with the bundle Jacobian (Lensing::dbetadtheta) for two
screen / stop_bundle choices; the reference's velocity-field build
(-DVELOCITYFIELD): particle deposits and rays traced with the Doppler term;
and its cone octree build from ASCII cells (create_octree): every correction
option, a file with many incomplete octs, a rotated narrow cone.
"""
from __future__ import annotations

import importlib
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
S = importlib.import_module("magrathea-pathfinder_gb300.synth")
from refharness import Reference  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
COMPONENTS = "lensing,dr,dz,isw,dens,dens_max,steps,phi,deflection"

CASES = {
    # uniform level-7 grid (file level 5), 2.5 degree cone to 900 Mpc/h
    "uniform": dict(spec=dict(base_level=7, box_cells=32, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=900.0),
                    zs=[0.1, 0.15, 0.2], nsteps=10, nside=256, rays=16),
    # AMR: the same base refined three levels around four NFW haloes
    "amr": dict(spec=dict(base_level=7, box_cells=32, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=900.0, halos=6,
                          max_level=10, mass_min=3e14, mass_max=2e15, refine_cells=1.5, seed=7),
                zs=[0.1, 0.15, 0.2], nsteps=8, nside=256, rays=16),
}


def cone_pixels(R, nside, half_deg):
    ncap = 2 * nside * (nside - 1)
    allp = np.arange(ncap, 12 * nside * nside - ncap)
    v = R.pix2vec(nside, allp)
    phi = np.arctan2(v[:, 1], v[:, 0])
    th = np.arccos(v[:, 2])
    sel = (np.abs(phi) < np.radians(half_deg)) & (np.abs(th - np.pi / 2) < np.radians(half_deg))
    return allp[sel]


# bundle Jacobian (jacobiantype = bundle): screen plane and stop_bundle pairs, opening 0.2 arcmin
BUNDLES = (("sachs", "redshift"), ("normal", "r"), ("sachs", "plane"), ("normal", "plane"))
OPENING = 0.2 / 60.0 * 3.141592653589793 / 180.0
# lensing_born maps: (fixture key, components, jacobiantype)
BORN_MAPS = (("born", "lensing,lensing_born,dz,steps", "infinitesimal"), ("bornonly", "lensing_born", "infinitesimal"),
             ("born_bundle", "lensing_born,lensing,dr", "bundle"))
CAT_ACCURACIES = (1e-8, 1e-13, 0.0)   # job default; deep enough for the Jacobian steps; never met (rejects)
CAT_VOBS = (1e-4, -2e-4, 5e-5)


def catalogue_sources(rng, n, chi_max_box):
    """Sources in the octree frame: most inside the data, the last 4 beyond it (failures)."""
    d = rng.uniform(0.05, 0.95 * chi_max_box, n)
    d[-4:] = rng.uniform(1.15 * chi_max_box, 1.4 * chi_max_box, 4)
    ph = np.radians(rng.uniform(-2.0, 2.0, n))
    th = np.pi / 2 + np.radians(rng.uniform(-2.0, 2.0, n))
    src = np.zeros((n, 6))
    src[:, 0] = d * np.cos(ph) * np.sin(th)
    src[:, 1] = d * np.sin(ph) * np.sin(th)
    src[:, 2] = d * np.cos(th)
    src[:, 3:] = rng.normal(0.0, 1e-3, (n, 3))
    return src


def rotation(ax, ay, az):
    cx, sx, cy, sy, cz, sz = np.cos(ax), np.sin(ax), np.cos(ay), np.sin(ay), np.cos(az), np.sin(az)
    Rx = np.array([[1, 0, 0], [0, cx, -sx], [0, sx, cx]])
    Ry = np.array([[cy, 0, sy], [0, 1, 0], [-sy, 0, cy]])
    Rz = np.array([[cz, -sz, 0], [sz, cz, 0], [0, 0, 1]])
    return Rz @ Ry @ Rx


def make(name, cfg):
    spec = S.OctreeSpec(**cfg["spec"])
    rec = S.make_octree(spec)
    tmp = tempfile.mkdtemp(prefix="mpf_golden_")
    binpath = os.path.join(tmp, "cone.bin")
    S.write_bin(binpath, rec)
    celldir, pf, ef = S.write_param_files(tmp, spec.cosmo, spec.lbox)
    out = dict(records=rec, nsteps=cfg["nsteps"], zs=np.array(cfg["zs"]), nside=cfg["nside"],
               components=np.array(COMPONENTS))
    rng = np.random.default_rng(11)
    levels = S.key_level(rec["hi"], rec["lo"])
    centers = np.zeros((rec.shape[0], 3))
    for L in np.unique(levels):
        m = levels == L
        centers[m] = S.cell_center(int(L), S.key_coords(rec["hi"][m], rec["lo"][m], int(L)))
    idx = rng.integers(0, rec.shape[0], 3000)
    span = 4.0 / 2.0 ** levels[idx]
    pts = centers[idx] + rng.uniform(-0.75, 0.75, (3000, 3)) * span[:, None]
    pts[:4] = 0.0
    pts[4:20] = np.round(pts[4:20] * 256) / 256        # exact cell boundaries
    out["pts"] = pts
    # keys at random positions / levels
    kp = rng.uniform(-2, 2, (400, 3))
    kl = rng.integers(0, 33, 400)
    R = Reference(1)
    out["key_pos"], out["key_level"] = kp, kl
    out["key_ref"] = np.array([R.compute(int(l), *p) for l, p in zip(kl, kp)], dtype=np.uint64)
    for order in (1, 2):
        R = Reference(order)
        cos = R.cosmology(celldir, pf, ef)
        R.load(binpath)
        if order == 1:
            for k in ("t", "a", "dadt", "d2adt2", "length"):
                out["cosmo_" + k] = cos[k]
            out["ref_locate"] = R.locate(pts)
            out["ref_cic"] = R.cic(pts)
            out["ref_tsc"] = R.tsc(pts)
            out["homogeneous"] = R.homogeneous(out["zs"])
        launch = S.photon_grid(cfg["rays"], 2.0, 2.0)
        out["launch"] = launch
        steps, final, _ = R.integrate(launch, "redshift", cfg["zs"][-1], cfg["nsteps"])
        out["ref_steps_o%d" % order] = steps
        out["ref_final_o%d" % order] = final
        pix = cone_pixels(R, cfg["nside"], 1.8)
        out["pixels"] = pix
        out["pixel_dirs"] = R.pix2vec(cfg["nside"], pix)
        out["ref_maps_o%d" % order] = R.fillmap(cfg["nside"], out["zs"], pix, "redshift", COMPONENTS, cfg["nsteps"])
        for plane, sb in BUNDLES:
            out["ref_maps_bundle_o%d_%s_%s" % (order, plane, sb)] = R.fillmap(
                cfg["nside"], out["zs"], pix, "redshift", COMPONENTS, cfg["nsteps"], "bundle", plane, sb, OPENING)
        # lensing_born (hmaps.h:706-712, 771-785): the Jacobian along the FLRW ray of each pixel, with the
        # traced ray's components, alone (no traced ray), and beside a bundle Jacobian
        for key, comps, jt in BORN_MAPS:
            out["ref_maps_%s_o%d" % (key, order)] = R.fillmap(cfg["nside"], out["zs"], pix, "redshift", comps,
                                                              cfg["nsteps"], jt, "sachs", "redshift", OPENING)
        if order == 1:
            crng = np.random.default_rng(23)
            src = catalogue_sources(crng, 40, spec.chi_max / spec.lbox)
            rot = rotation(0.3, -0.2, 0.7)
            out["cat_src"] = src
            # the same sources given in a rotated frame, with the rotation to the octree frame
            out["cat_src_rotated"] = np.concatenate([src[:, :3] @ rot, src[:, 3:] @ rot], axis=1)
            out["cat_rotm1"] = rot
            out["cat_vobs"] = np.array(CAT_VOBS)
            out["cat_accuracy"] = np.array(CAT_ACCURACIES)
            out["cosmo_h"] = cos["h"]
            out["cosmo_mpc"] = 3.08568e22
        for ia, acc in enumerate(CAT_ACCURACIES):
            out["ref_cat_o%d_a%d" % (order, ia)] = R.catalogue(out["cat_src"], acc, cfg["nsteps"], out["cosmo_h"],
                                                               out["cosmo_mpc"], CAT_VOBS)
        out["ref_cat_rot_o%d" % order] = R.catalogue(out["cat_src_rotated"], CAT_ACCURACIES[0], cfg["nsteps"],
                                                     out["cosmo_h"], out["cosmo_mpc"], CAT_VOBS, out["cat_rotm1"])
        # jacobiantype = infinitesimal_born: the final Jacobian along the FLRW ray (catalogues.h:670-673)
        for ia in (0, 1):
            out["ref_cat_born_o%d_a%d" % (order, ia)] = R.catalogue(
                out["cat_src"], CAT_ACCURACIES[ia], cfg["nsteps"], out["cosmo_h"], out["cosmo_mpc"], CAT_VOBS, None,
                "infinitesimal_born")
        # jacobiantype = bundle: converged at 1e-8, and every source through the bundle Newton rounds at 0
        for ia in (0, 2):
            for plane, sb in BUNDLES:
                out["ref_cat_bundle_o%d_a%d_%s_%s" % (order, ia, plane, sb)] = R.catalogue(
                    out["cat_src"], CAT_ACCURACIES[ia], cfg["nsteps"], out["cosmo_h"], out["cosmo_mpc"], CAT_VOBS,
                    None, "bundle", plane, sb, OPENING)
    # ORDER = 0 (nearest grid point, simplehyperoctree.h:1396-1401): point
    # gathers, rays, maps and catalogue rows of the reference built with it
    R = Reference(0)
    R.cosmology(celldir, pf, ef)
    R.load(binpath)
    out["ref_ngp"] = R.ngp(pts)
    out["ref_steps_o0"], out["ref_final_o0"], _ = R.integrate(launch, "redshift", cfg["zs"][-1], cfg["nsteps"])
    out["ref_maps_o0"] = R.fillmap(cfg["nside"], out["zs"], pix, "redshift", COMPONENTS, cfg["nsteps"])
    out["ref_cat_o0_a0"] = R.catalogue(out["cat_src"], CAT_ACCURACIES[0], cfg["nsteps"], out["cosmo_h"],
                                       out["cosmo_mpc"], CAT_VOBS)
    path = os.path.join(HERE, "%s.npz" % name)
    np.savez_compressed(path, **out)
    print("%s: %d cells (levels %d-%d), %d rays, %d pixels -> %s (%d KB)" % (
        name, rec.shape[0], levels.min(), levels.max(), launch.shape[0], pix.shape[0], path, os.path.getsize(path) // 1024))


# rays bundles (Integrator::propagate): a cone deep enough for the bundle checks
# (the rays must travel more than a quarter of the extent), a few haloes
RAYS_SPEC = dict(base_level=6, box_cells=16, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=2600.0, halos=3,
                 max_level=8, mass_min=3e14, mass_max=2e15, refine_cells=1.5, seed=5)
RAYS_NSTEPS = 4
# (direction offsets in degrees (y, z), count, opening in degrees, rotation, interpolation, amin)
RAYS_CASES = (
    ((0.3, -0.2), 4, 0.5, 0.3, "redshift", 0.0),
    ((-0.6, 0.4), 8, 0.2, 1.1, "r", 0.0),
    ((0.1, 0.9), 3, 0.3, 0.0, "a", 0.0),
    ((-0.2, -0.7), 4, 0.3, 2.0, "lambda", 0.0),
    ((0.8, 0.1), 4, 0.3, 0.5, "t", 0.0),
    ((0.0, 0.0), 4, 0.3, 0.5, "redshift", 0.2),     # rejected: the last a of the data is above amin
    ((0.4, 0.4), 0, 0.3, 0.0, "redshift", 0.0),     # no bundle: the central ray alone, distance 0
    ((2.0, 0.0), 4, 1.5, 0.0, "redshift", 0.0),     # a wide opening near the cone's edge
    ((30.0, 0.0), 4, 0.5, 0.0, "redshift", 0.0),    # leaves the cone at once: rejected (a quarter of the extent)
)


# the rays driver's FLRW reference bundle (rays.cpp:244-249): Order = -1 on a
# uniform octree of level ncoarse / 2, nsteps = EXTENT nsteps 2^(ncoarse - ncoarse/2) 2,
# launched from the centre toward +x; (count, opening in degrees, interpolation)
FLRW_NCOARSE = 6
FLRW_CASES = ((4, 0.3, "redshift"), (6, 0.2, "r"))
FLRW_EVERY = 8     # points kept in the fixture: every 8th, and the last


def make_rays():
    spec = S.OctreeSpec(**RAYS_SPEC)
    rec = S.make_octree(spec)
    tmp = tempfile.mkdtemp(prefix="mpf_golden_")
    binpath = os.path.join(tmp, "cone.bin")
    S.write_bin(binpath, rec)
    celldir, pf, ef = S.write_param_files(tmp, spec.cosmo, spec.lbox)
    launch = np.zeros((len(RAYS_CASES), 6))
    for i, ((dy, dz), *_rest) in enumerate(RAYS_CASES):
        ph, th = np.radians(dy), np.pi / 2 + np.radians(dz)
        launch[i, 3:] = (np.sin(th) * np.cos(ph), np.sin(th) * np.sin(ph), np.cos(th))
    out = dict(records=rec, nsteps=RAYS_NSTEPS, launch=launch,
               count=np.array([c[1] for c in RAYS_CASES]), angle=np.radians([c[2] for c in RAYS_CASES]),
               rotation=np.array([c[3] for c in RAYS_CASES]), interp=np.array([c[4] for c in RAYS_CASES]),
               amin=np.array([c[5] for c in RAYS_CASES]))
    for order in (1, 2):
        R = Reference(order)
        cos = R.cosmology(celldir, pf, ef)
        R.load(binpath)
        if order == 1:
            for k in ("t", "a", "dadt", "d2adt2", "length"):
                out["cosmo_" + k] = cos[k]
            level = FLRW_NCOARSE // 2
            nst = 4 * RAYS_NSTEPS * (1 << (FLRW_NCOARSE - level)) * 2
            out["flrw_level"], out["flrw_nsteps"] = level, nst
            out["flrw_count"] = np.array([c[0] for c in FLRW_CASES])
            out["flrw_angle"] = np.radians([c[1] for c in FLRW_CASES])
            out["flrw_interp"] = np.array([c[2] for c in FLRW_CASES])
            out["flrw_every"] = FLRW_EVERY
            for j, (count, ang, interp) in enumerate(FLRW_CASES):
                t = R.propagate_bundle_flrw(np.array([0.0, 0.0, 0.0, 2.0, 0.0, 0.0]), count, np.radians(ang), interp, nst,
                                            level)
                out["flrw_size_%d" % j] = t.shape[0]
                out["flrw_traj_%d" % j] = t[::FLRW_EVERY]
                out["flrw_last_%d" % j] = t[-1]
        sizes, trajs = [], []
        for i, (_, count, ang, rot, interp, amin) in enumerate(RAYS_CASES):
            traj, text = R.propagate_bundle(launch[i], count, np.radians(ang), rot, interp, amin, RAYS_NSTEPS)
            sizes.append(traj.shape[0])
            trajs.append(traj)
            if i == 0:
                out["ref_text_o%d" % order] = np.array(text)
        cap = max(sizes)
        T = np.zeros((len(trajs), cap, 29))
        for i, t in enumerate(trajs):
            T[i, :t.shape[0]] = t
        out["ref_sizes_o%d" % order] = np.array(sizes, dtype=np.int64)
        out["ref_traj_o%d" % order] = T
    path = os.path.join(HERE, "rays.npz")
    np.savez_compressed(path, **out)
    print("rays: %d cells, sizes o1 %s o2 %s -> %s (%d KB)" % (rec.shape[0], out["ref_sizes_o1"].tolist(),
                                                            out["ref_sizes_o2"].tolist(), path, os.path.getsize(path) // 1024))


# create_octree from ASCII cells (Input::importascii + Miscellaneous::correctOctree):
# the synthetic cone written as RAMSES-unit rows, with duplicated cells of a
# neighbouring light-cone shell (different a and phi), non-normal densities
# at the coarse and refined levels, and refined cells missing some children
CELLS_SPEC = dict(base_level=6, box_cells=16, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=1000.0, halos=3,
                  max_level=8, mass_min=3e14, mass_max=2e15, refine_cells=1.5, seed=9)


# correction / coarsecorrection pairs of Input::correct (input.h:1398-1482)
CELLS_CORRECTIONS = {"full": dict(correction=1, coarsecorrection=1), "nocorr": dict(correction=0, coarsecorrection=0),
                     "nocorr_coarse": dict(correction=0, coarsecorrection=1),
                     "corr_nocoarse": dict(correction=1, coarsecorrection=0),
                     "acorr": dict(correction=1, coarsecorrection=1, acorrection=1),
                     "nocorr_acorr": dict(correction=0, coarsecorrection=0, acorrection=1),
                     # the reference built with ORDER=1: CIC gathers for the completed children
                     "full_o1": dict(correction=1, coarsecorrection=1, order=1),
                     "full_o0": dict(correction=1, coarsecorrection=1, order=0)}


def make_cells():
    spec = S.OctreeSpec(**CELLS_SPEC)
    rec = S.make_octree(spec)
    rows = S.cells_ramses(rec, spec)
    rng = np.random.default_rng(31)
    lev = rows[:, 0].astype(int)
    coarse = np.flatnonzero(lev == lev.min())
    fine = np.flatnonzero(lev > lev.min())
    rows[rng.choice(coarse, 6, replace=False), 4] = 0.0        # non-normal coarse densities
    rows[rng.choice(fine, 6, replace=False), 4] = 0.0          # non-normal refined densities
    dup = rng.choice(rows.shape[0], rows.shape[0] // 20, replace=False)
    extra = rows[dup].copy()
    extra[:, 9] *= 1.0 - 3e-4                                  # the neighbouring shell: earlier a ...
    extra[:, 5] *= 1.02                                        # ... and a different potential
    # a refined parent whose children are partly missing
    deep = np.flatnonzero(lev == lev.max())
    drop = deep[:3] if deep.shape[0] >= 8 else np.zeros(0, dtype=int)
    keep = np.ones(rows.shape[0], dtype=bool)
    keep[drop] = False
    allrows = np.concatenate([rows[keep], extra])
    allrows = allrows[rng.permutation(allrows.shape[0])]
    tmp = tempfile.mkdtemp(prefix="mpf_golden_")
    cellfile = os.path.join(tmp, "cells_00000.dat")
    S.write_cells(cellfile, allrows)
    celldir, pf, ef = S.write_param_files(tmp, spec.cosmo, spec.lbox)
    cone7 = np.array([0.0, 0.0, 0.0, spec.chi_max / spec.lbox, 0.0, 0.0, np.radians(2.0)])
    sphere4 = np.array([0.0, 0.0, 0.0, 1.0 / 32.0])
    text = open(cellfile).read()
    out = dict(cells_text=np.array(text), cone7=cone7, sphere4=sphere4, lboxmpch=spec.lbox, h=spec.cosmo.h,
               omegam=spec.cosmo.omega_m, mpc=S.MPC)
    R = Reference(2)
    cos = R.cosmology(celldir, pf, ef)
    for k in ("t", "a", "dadt", "d2adt2", "length"):
        out["cosmo_" + k] = cos[k]
    refs = {2: R}
    for name, kw in CELLS_CORRECTIONS.items():
        kw = dict(kw)
        order = kw.pop("order", 2)
        if order not in refs:
            refs[order] = Reference(order)
            refs[order].cosmology(celldir, pf, ef)
        recs, amin = refs[order].build_cone(cellfile, cone7, sphere4, mpc=S.MPC, h=spec.cosmo.h,
                                            omegam=spec.cosmo.omega_m, lboxmpch=spec.lbox, **kw)
        out["ref_records_" + name] = recs
        out["ref_amin_" + name] = amin
        print("cells %s: %d rows in, %d cells out" % (name, allrows.shape[0], recs.shape[0] // 48))
    path = os.path.join(HERE, "cells.npz")
    np.savez_compressed(path, **out)
    print("cells -> %s (%d KB)" % (path, os.path.getsize(path) // 1024))


# many incomplete octs: a quarter of the refined cells dropped at random and a
# cone narrower than the field, so that the completion's appended children
# read one another (Input::correct's sequential appends, input.h:1451-1482)
CELLS_SPARSE_SPEC = dict(base_level=6, box_cells=16, lbox=2048.0, half_y=2.5, half_z=2.5, chi_max=1000.0, halos=12,
                         max_level=9, mass_min=3e14, mass_max=2e15, refine_cells=2.5, seed=13)


def make_cells_sparse():
    spec = S.OctreeSpec(**CELLS_SPARSE_SPEC)
    rec = S.make_octree(spec)
    rows = S.cells_ramses(rec, spec)
    rng = np.random.default_rng(37)
    lev = rows[:, 0].astype(int)
    fine = np.flatnonzero(lev > lev.min())
    keep = np.ones(rows.shape[0], dtype=bool)
    keep[rng.choice(fine, fine.shape[0] // 4, replace=False)] = False
    rows = rows[keep]
    rows = rows[rng.permutation(rows.shape[0])]
    tmp = tempfile.mkdtemp(prefix="mpf_golden_")
    cellfile = os.path.join(tmp, "cells_00000.dat")
    S.write_cells(cellfile, rows)
    celldir, pf, ef = S.write_param_files(tmp, spec.cosmo, spec.lbox)
    cone7 = np.array([0.0, 0.0, 0.0, spec.chi_max / spec.lbox, 0.0, 0.0, np.radians(1.5)])
    sphere4 = np.array([0.0, 0.0, 0.0, 1.0 / 32.0])
    out = dict(cells_text=np.array(open(cellfile).read()), cone7=cone7, sphere4=sphere4, lboxmpch=spec.lbox,
               h=spec.cosmo.h, omegam=spec.cosmo.omega_m, mpc=S.MPC)
    for order in (1, 2):
        R = Reference(order)
        cos = R.cosmology(celldir, pf, ef)
        if order == 2:
            for k in ("t", "a", "dadt", "d2adt2", "length"):
                out["cosmo_" + k] = cos[k]
        recs, _ = R.build_cone(cellfile, cone7, sphere4, mpc=S.MPC, h=spec.cosmo.h, omegam=spec.cosmo.omega_m,
                               lboxmpch=spec.lbox, correction=1, coarsecorrection=1)
        out["ref_records_o%d" % order] = recs
        print("cells_sparse o%d: %d rows in, %d cells out" % (order, rows.shape[0], recs.shape[0] // 48))
        if order == 2:
            # a narrow cone's rotation of the cells (importascii's rotm1, input.h:1034-1039)
            rot = rotation(0.004, -0.006, 0.009)
            recs, _ = R.build_cone(cellfile, cone7, sphere4, rotm1=rot, mpc=S.MPC, h=spec.cosmo.h,
                                   omegam=spec.cosmo.omega_m, lboxmpch=spec.lbox, correction=1, coarsecorrection=1)
            out["rotm1"] = rot
            out["ref_records_rot"] = recs
            print("cells_sparse rotated: %d cells out" % (recs.shape[0] // 48))
    path = os.path.join(HERE, "cells_sparse.npz")
    np.savez_compressed(path, **out)
    print("cells_sparse -> %s (%d KB)" % (path, os.path.getsize(path) // 1024))


def records_sha(rec) -> str:
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(rec).tobytes()).hexdigest()


def whole_rays_specs():
    """Two whole-ray workloads: the AMR construction of the benchmark octree at
    a small size (64^3 base at octree level 8, refined to 11 in 50 NFW haloes)
    to z = 2, and the uniform 64^3 cone along phi = theta = 20 deg to z = 0.5."""
    chi2 = float(S.Cosmology().chi_of_z(2.0)[0])
    amr = S.OctreeSpec(base_level=8, box_cells=64, lbox=2048.0, half_y=5.0, half_z=5.0, chi_max=chi2 * 1.02, halos=50,
                       max_level=11, refine_cells=2.5, seed=42)
    return {"amr_z2": (amr, S.photon_grid(8, 4.5, 4.5), 2.0, 8, (1, 2)),
            "cone20_z05": (S.uniform_grid_cone(0.5, (20.0, 20.0)), None, 0.5, 10, (1,))}


def make_whole_rays():
    """The reference's Integrator::integrate on whole rays of the two
    workloads (step counts and final photon records), with the records' hash
    so that a test regenerates exactly the same octree."""
    out = {}
    table = S.Cosmology().conformal_table(n=4000, amin=0.05)
    for name, (spec, launch, zstop, nsteps, orders) in whole_rays_specs().items():
        rec = S.make_octree(spec)
        if launch is None:
            launch = S.photon_grid(8, 2.5, 2.5, spec.frame())
        tmp = tempfile.mkdtemp(prefix="mpf_golden_")
        binpath = os.path.join(tmp, "cone.bin")
        S.write_bin(binpath, rec)
        length = spec.lbox * S.MPC / spec.cosmo.h
        out[name + "_sha"] = np.array(records_sha(rec))
        out[name + "_launch"] = launch
        for order in orders:
            R = Reference(order)
            R.set_cosmology(*table, length)
            R.load(binpath)
            steps, final, _ = R.integrate(launch, "redshift", zstop, nsteps)
            out["%s_steps_o%d" % (name, order)] = steps
            out["%s_final_o%d" % (name, order)] = final
            print("%s order %d: %d rays, %.0f steps on average" % (name, order, launch.shape[0], steps.mean()))
    path = os.path.join(HERE, "whole_rays.npz")
    np.savez_compressed(path, **out)
    print("whole rays -> %s (%d KB)" % (path, os.path.getsize(path) // 1024))


VEL_VOBS = (3e-4, -2e-4, 1e-4)         # observer velocity, in the units of the particle velocities (c)
VEL_COMPONENTS = "lensing,dz,isw,dens,steps"


def make_velocity():
    """The reference's velocity-field build (-DVELOCITYFIELD) on the AMR
    fixture's octree: seeded particles deposited with CIC and with TSC in two
    particle files (BEGIN + first file, second file + FINISH: the map driver's
    loop over shell files, hmaps.cpp:395-441), the cells' velocities and
    masses, then whole rays (Integrator::integrate) and FillMap maps traced
    with the observer velocity: ORDER = 1 on the CIC field, 2 on the TSC one."""
    g = np.load(os.path.join(HERE, "amr.npz"))
    rec = g["records"]
    tmp = tempfile.mkdtemp(prefix="mpf_golden_")
    binpath = os.path.join(tmp, "cone.bin")
    S.write_bin(binpath, rec)
    pos, vel = S.velocity_particles(rec, 1500, seed=5)
    split = 900
    zs, nsteps, nside, pix = g["zs"], int(g["nsteps"]), int(g["nside"]), g["pixels"]
    launch = S.photon_grid(8, 2.0, 2.0)
    out = dict(records_sha=np.array(records_sha(rec)), part_pos=pos, part_vel=vel, part_split=split,
               vobs=np.array(VEL_VOBS), zs=zs, nsteps=nsteps, nside=nside, pixels=pix, launch=launch,
               components=np.array(VEL_COMPONENTS))
    for scheme, order in (("cic", 1), ("tsc", 2)):
        R = Reference(order, velocity=True)
        R.set_cosmology(g["cosmo_t"], g["cosmo_a"], g["cosmo_dadt"], g["cosmo_d2adt2"], float(g["cosmo_length"]))
        R.load(binpath)
        R.deposit_velocity(pos[:split], vel[:split], scheme, True, False)
        R.deposit_velocity(pos[split:], vel[split:], scheme, False, True)
        v, rho = R.velocity()
        out["ref_vel_" + scheme], out["ref_rho_" + scheme] = v, rho
        R.set_vobs(VEL_VOBS)
        steps, final, _ = R.integrate(launch, "redshift", float(zs[-1]), nsteps)
        out["ref_steps_o%d" % order], out["ref_final_o%d" % order] = steps, final
        out["ref_maps_o%d" % order] = R.fillmap(nside, zs, pix, "redshift", VEL_COMPONENTS, nsteps)
        print("velocity %s: %d of %d cells without mass, %.0f steps per ray" % (scheme, int((rho == 0).sum()),
                                                                                 rho.shape[0], steps.mean()))
    path = os.path.join(HERE, "velocity.npz")
    np.savez_compressed(path, **out)
    print("velocity -> %s (%d KB)" % (path, os.path.getsize(path) // 1024))


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES) + ["rays", "cells", "cells_sparse", "whole_rays", "velocity"]
    for name in names:
        if name == "velocity":
            make_velocity()
        elif name == "whole_rays":
            make_whole_rays()
        elif name == "rays":
            make_rays()
        elif name in ("cells", "cells_sparse"):
            if names == [name]:
                make_cells() if name == "cells" else make_cells_sparse()
            else:
                # in a process of its own: the reference's SimpleHyperOctree::update reads one element past
                # its container for the last cell (simplehyperoctree.h:1299), so that record, and through its
                # scale factor acorrection's table, depends on the heap the process has used before
                import subprocess
                subprocess.run([sys.executable, os.path.abspath(__file__), name], check=True)
        else:
            make(name, CASES[name])
