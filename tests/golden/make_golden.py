"""Generate the golden fixtures of the photon-propagation path by running the
reference's own code (oracle/ref_harness.cpp built by oracle/build_ref.sh from
the reference sources) on seeded synthetic inputs.

Run in a container that has the reference sources:
    ./oracle/build_ref.sh && python tests/golden/make_golden.py

Each fixture holds the octree records it was computed on (so the GPU machine,
which has no reference, reads exactly the same bytes), the cosmology table
the reference derived from its evolution file (Input::acquire + correct), and
the reference's outputs: locate / cic / tsc at random points, per-ray step
counts and final photon records (Integrator::integrate), and FillMap maps.
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
    path = os.path.join(HERE, "%s.npz" % name)
    np.savez_compressed(path, **out)
    print("%s: %d cells (levels %d-%d), %d rays, %d pixels -> %s (%d KB)" % (
        name, rec.shape[0], levels.min(), levels.max(), launch.shape[0], pix.shape[0], path, os.path.getsize(path) // 1024))


if __name__ == "__main__":
    for name, cfg in CASES.items():
        make(name, cfg)
