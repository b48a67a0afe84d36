"""Per-pixel map values from surface records, as Hmaps::FillMap writes them
(src/hmaps.h:701-832, infinitesimal Jacobian branch).

Component names and their rows, in the order given (src/hmaps.cpp:196-269):
  lensing     kappa, gamma1, gamma2, 1/mu   (4 rows)
  dr dl dt da dz ds                          relative to the FLRW value
  isw dens dens_max steps phi                interpolated / raw values
  deflection  phi - beta1, theta - beta2     (2 rows)
A pixel whose surface was not crossed properly gets 0 in every row.
"""
from __future__ import annotations

import numpy as np

ROWS = {"lensing": 4, "lensing_born": 4, "deflection": 2}
# plane record columns
F = {k: i for i, k in enumerate("firstid f x y z distance A11 A12 A22 t a redshift chi lambda s isw rho phi rho_max "
                                 "valid".split())}


def nmaps(components, bundle: bool = False) -> int:
    return sum((5 if bundle else 4) if c == "lensing" else ROWS.get(c, 1) for c in components)


def assemble(planes: np.ndarray, directions: np.ndarray, homogeneous: np.ndarray, components,
             bundle_jac: np.ndarray = None) -> np.ndarray:
    """planes: [npix, nz, 20]; directions: [npix, 3] launch directions;
    homogeneous: [nz, 5] = t, chi, lambda, a, z of the FLRW ray at each surface;
    bundle_jac: [npix, nz, 4] (a11 a12 a21 a22) of the bundle Jacobian, or None
    for the infinitesimal one.  Returns float32 maps [nz, nmaps, npix]."""
    if "lensing_born" in components:
        raise ValueError("lensing_born needs the Born rays' surface records: hmaps_fill computes it")
    npix, nz = planes.shape[0], planes.shape[1]
    out = np.zeros((nz, nmaps(components, bundle_jac is not None), npix), dtype=np.float32)
    ph = np.arctan2(directions[:, 1], directions[:, 0])
    th = np.arccos(directions[:, 2])
    for iz in range(nz):
        p = planes[:, iz]
        valid = p[:, F["valid"]] > 0
        rows = []
        for c in components:
            if c == "lensing" and bundle_jac is not None:
                # hmaps.h:725-747: image rotation w, then kappa, gamma1, gamma2, w, 1/mu;
                # a Jacobian flagged 42 zeroes the whole surface
                b11, b12, b21, b22 = (bundle_jac[:, iz, q] for q in range(4))
                valid = valid & (b11 != 42)
                w = -np.arctan2(b12 - b21, b11 + b22)
                rows += [1 - (b11 + b22) * 0.5 / np.cos(w), -0.5 * (np.cos(w) * (b11 - b22) + np.sin(w) * (b12 + b21)),
                         -0.5 * (np.cos(w) * (b12 + b21) + np.sin(w) * (b22 - b11)), w, b11 * b22 - b12 * b21]
            elif c == "lensing":
                a11, a12, a22 = p[:, F["A11"]], p[:, F["A12"]], p[:, F["A22"]]
                rows += [1 - (a11 + a22) * 0.5, -0.5 * (a11 - a22), -a12, a11 * a22 - a12 * a12]
            elif c == "dr":
                rows.append(p[:, F["chi"]] / homogeneous[iz, 1] - 1)
            elif c == "dl":
                rows.append(p[:, F["lambda"]] / homogeneous[iz, 2] - 1)
            elif c == "dt":
                rows.append(p[:, F["t"]] / homogeneous[iz, 0] - 1)
            elif c == "da":
                rows.append(p[:, F["a"]] / homogeneous[iz, 3] - 1)
            elif c == "dz":
                rows.append(p[:, F["redshift"]] / homogeneous[iz, 4] - 1)
            elif c == "ds":
                rows.append(p[:, F["s"]] / homogeneous[iz, 1] - 1)
            elif c == "isw":
                rows.append(p[:, F["isw"]])
            elif c == "dens":
                rows.append(p[:, F["rho"]])
            elif c == "dens_max":
                rows.append(p[:, F["rho_max"]])
            elif c == "steps":
                rows.append(p[:, F["firstid"]])
            elif c == "phi":
                rows.append(p[:, F["phi"]])
            elif c == "deflection":
                x, y, z, d = p[:, F["x"]], p[:, F["y"]], p[:, F["z"]], p[:, F["distance"]]
                with np.errstate(invalid="ignore", divide="ignore"):
                    rows += [ph - np.arctan2(y, x), th - np.arccos(z / d)]
            else:
                raise ValueError("unknown map component %r" % c)
        for k, v in enumerate(rows):
            out[iz, k] = np.where(valid, v, 0).astype(np.float32)
    return out
