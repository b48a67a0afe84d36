"""Per-output errors of a propagation against a float64 run of the same rays.

The outputs compared are the ones a map or catalogue is made of: the step
count (trajectory size), the angular deflection (angle between the launch
direction and the ray's last position), the redshift of the last point and,
at a surface, the lensing quantities FillMap writes from the Jacobian
(src/hmaps.h:759-762): kappa = 1 - (a11 + a22) / 2, gamma1 = -(a11 - a22) / 2,
gamma2 = -a12, 1/mu = a11 a22 - a12^2.

The float64 run is the reference's algorithm in its own operation order: the
exact mode of this library, or a CPU run of the reference's code.
"""
from __future__ import annotations

import numpy as np

LENSING = ("kappa", "gamma1", "gamma2", "inv_mu")


def deflection(launch: np.ndarray, final: np.ndarray) -> np.ndarray:
    """Angle (rad) between each launch direction and the ray's last position,
    accurate for small angles (atan2 of the cross and dot products)."""
    d = launch[:, 3:6] - launch[:, 0:3]
    x = final[:, 2:5] - launch[:, 0:3]
    return np.arctan2(np.linalg.norm(np.cross(d, x), axis=1), np.sum(d * x, axis=1))


def lensing(plane_rec: np.ndarray) -> np.ndarray:
    """kappa, gamma1, gamma2, 1/mu (n x nplanes x 4) from surface records."""
    a11, a12, a22 = plane_rec[..., 6], plane_rec[..., 7], plane_rec[..., 8]
    return np.stack([1.0 - (a11 + a22) * 0.5, -0.5 * (a11 - a22), -a12, a11 * a22 - a12 * a12], axis=-1)


def compare(launch, steps, final, planes, ref_steps, ref_final, ref_planes) -> dict:
    """Errors of (steps, final, planes) against the float64 run (ref_*).

    Deflection and redshift errors are relative, per ray; lensing errors are
    absolute and also given relative to the largest |value| over the rays
    (the scale of the map).  Surfaces a ray did not reach in both runs are
    left out of the lensing errors and counted in `surface_valid_differs`."""
    launch = np.asarray(launch)
    out = {"rays": int(launch.shape[0])}
    ds = np.abs(np.asarray(steps, dtype=np.int64) - np.asarray(ref_steps, dtype=np.int64))
    out["step_count_differs"] = int((ds != 0).sum())
    out["max_step_diff"] = int(ds.max()) if ds.size else 0
    dg, dr = deflection(launch, final), deflection(launch, ref_final)
    rel = np.abs(dg - dr) / np.maximum(np.abs(dr), 1e-300)
    z, zr = final[:, 19], ref_final[:, 19]
    zrel = np.abs(z - zr) / np.maximum(np.abs(zr), 1e-300)
    out["deflection_rel"] = {"max": float(rel.max()), "median": float(np.median(rel))} if rel.size else None
    out["deflection_median_rad"] = float(np.median(dr)) if dr.size else None
    out["redshift_rel"] = {"max": float(zrel.max()), "median": float(np.median(zrel))} if zrel.size else None
    if planes is not None and ref_planes is not None and planes.size:
        valid = (planes[..., 19] != 0) & (ref_planes[..., 19] != 0)
        out["surface_valid_differs"] = int(((planes[..., 19] != 0) != (ref_planes[..., 19] != 0)).sum())
        if valid.any():
            L, Lr = lensing(planes)[valid], lensing(ref_planes)[valid]
            err = np.abs(L - Lr).max(axis=0)
            scale = np.abs(Lr).max(axis=0)
            for q, name in enumerate(LENSING):
                out[name] = {"abs_max": float(err[q]), "scale": float(scale[q]),
                             "of_scale": float(err[q] / max(scale[q], 1e-300))}
    return out


def within(report: dict, rel_tol: float = 1e-6, lensing_tol: float = 1e-6) -> bool:
    """Whether a compare() report is inside the tolerances: deflection and
    redshift within rel_tol relative on every ray, lensing quantities within
    lensing_tol of the map's scale (1/mu: of 1), the same step counts and
    surfaces."""
    if report["step_count_differs"] or report.get("surface_valid_differs", 0):
        return False
    if report["deflection_rel"] and report["deflection_rel"]["max"] > rel_tol:
        return False
    if report["redshift_rel"] and report["redshift_rel"]["max"] > rel_tol:
        return False
    for name in LENSING:
        if name in report:
            scale = 1.0 if name == "inv_mu" else max(report[name]["scale"], 1e-6)
            if report[name]["abs_max"] > lensing_tol * scale:
                return False
    return True
