"""On-disk outputs of the hmaps and catalogues drivers, host side.

* Catalogue ASCII files, as Catalogues::relCat writes them
  (src/catalogues.h:864-902): ``<name>.txt`` for converged sources (id, the
  16 catalogue columns, npart; 17 significant digits), ``<name>_err.txt`` for
  sources the rays cannot reach (id and columns 0-4 then column 4 again, at
  the stream's default 6 significant digits) and ``<name>_reject.txt`` for
  sources that did not converge (same columns as the main file).
* Ray trajectories as the rays driver writes them (Output::save,
  src/output.h:200-211): 29 columns per point, 17 significant digits.
* HEALPix maps as FITS binary tables (the reference calls chealpix's
  write_healpix_map, src/hmaps.cpp:496-510): one float column, RING (or
  NESTED) ordering, the HEALPix keywords, non-normal values replaced by
  Healpix_undef, and the reference's file name pattern.  cfitsio and HEALPix
  are not available here, so the layout follows the FITS standard and the
  HEALPix conventions rather than a byte comparison with chealpix.
"""
from __future__ import annotations

import os

import numpy as np

HEALPIX_UNDEF = -1.6375e30
FITS_BLOCK = 2880


# --------------------------------------------------------------------------
# catalogues
# --------------------------------------------------------------------------
def _g(x, digits):
    return "%.*g" % (digits, x)


def catalogue_files(name: str):
    """Output::name(filename, ".txt"), (filename, "_err", ".txt"), (filename, "_reject", ".txt")."""
    return name + ".txt", name + "_err.txt", name + "_reject.txt"


def write_catalogue(name: str, rows: np.ndarray, sources: np.ndarray) -> tuple:
    """Write relCat's three files.  rows: n x 16 catalogue rows; sources: the
    n x 8 source rows (column 6 = id, column 7 = npart).  Returns the paths."""
    rows = np.asarray(rows, dtype=np.float64)
    sources = np.asarray(sources, dtype=np.float64)
    if rows.ndim != 2 or rows.shape[1] != 16 or sources.shape[0] != rows.shape[0] or sources.shape[1] < 8:
        raise ValueError("rows must be n x 16 and sources n x 8")
    good, err, rej = catalogue_files(name)
    with open(good, "w") as fg, open(err, "w") as fe, open(rej, "w") as fr:
        for c, s in zip(rows, sources):
            if c[2] != 42 and c[3] != 42 and c[5] != 42:
                fg.write(" ".join([_g(s[6], 17)] + [_g(v, 17) for v in c] + [_g(s[7], 17)]) + "\n")
            elif c[2] == 42 and c[3] == 42:
                fe.write(" ".join([_g(s[6], 6)] + [_g(v, 6) for v in c[:5]] + [_g(c[4], 6)]) + "\n")
            else:
                fr.write(" ".join([_g(s[6], 17)] + [_g(v, 17) for v in c] + [_g(s[7], 17)]) + "\n")
    return good, err, rej


# --------------------------------------------------------------------------
# trajectories
# --------------------------------------------------------------------------
TRAJECTORY_COLUMNS = ("index a t x y z dtdl dxdl dydl dzdl level ah rho phi dphidx dphidy dphidz dphidl laplacian "
                      "redshift dsdl2 error distance isw iswold chi lambda dphidt s").split()


def trajectory_text(points: np.ndarray) -> str:
    """A trajectory as Output::save writes it (src/output.h:200-211): one
    photon per line, its 29 values separated by spaces at 17 significant
    digits (the step index as an integer)."""
    pts = np.asarray(points, dtype=np.float64)
    if pts.ndim != 2 or pts.shape[1] != len(TRAJECTORY_COLUMNS):
        raise ValueError("a trajectory is m x 29")
    lines = []
    for row in pts:
        lines.append(" ".join(["%d" % int(row[0])] + [_g(v, 17) for v in row[1:]]))
    return "".join(l + "\n" for l in lines)


def write_trajectory(path: str, points: np.ndarray) -> str:
    with open(path, "w") as f:
        f.write(trajectory_text(points))
    return path


# --------------------------------------------------------------------------
# HEALPix FITS maps
# --------------------------------------------------------------------------
def clean_map(values: np.ndarray) -> np.ndarray:
    """Non-normal values (0, subnormal, inf, nan) -> Healpix_undef, as hmaps.cpp:498-502."""
    m = np.asarray(values, dtype=np.float32)
    a = np.abs(m)
    normal = np.isfinite(m) & (a >= np.finfo(np.float32).tiny)
    return np.where(normal, m, np.float32(HEALPIX_UNDEF)).astype(np.float32)


def map_filename(outputdir: str, prefix: str, nside: int, index: int, z: float, stop_ray: str) -> str:
    """hmaps.cpp:508: outputdir + prefix + "_nside" + nside + "_" + i + "_z_" + std::to_string(z) + "_" + stop_ray + ".fits"."""
    return "%s%s_nside%d_%d_z_%s_%s.fits" % (outputdir, prefix, int(nside), int(index), "%f" % z, stop_ray)


def _card(key: str, value=None, comment: str = "") -> bytes:
    if value is None:
        s = key.ljust(80)
    else:
        if isinstance(value, bool):
            v = ("T" if value else "F").rjust(20)
        elif isinstance(value, (int, np.integer)):
            v = str(int(value)).rjust(20)
        elif isinstance(value, float):
            v = ("%.17G" % value).rjust(20)
        else:
            v = ("'%s'" % str(value).ljust(8))
        s = ("%-8s= %s" % (key, v))
        if comment:
            s += " / " + comment
        s = s[:80].ljust(80)
    return s.encode("ascii")


def _pad(b: bytes, fill: bytes) -> bytes:
    r = len(b) % FITS_BLOCK
    return b if r == 0 else b + fill * (FITS_BLOCK - r)


def write_healpix_fits(path: str, values: np.ndarray, nside: int, nest: bool = False, coordsys: str = "C",
                       clean: bool = True) -> str:
    """One HEALPix map as a FITS binary table with a single float column."""
    m = clean_map(values) if clean else np.asarray(values, dtype=np.float32)
    npix = 12 * int(nside) * int(nside)
    if m.shape != (npix,):
        raise ValueError("a full-sky map of nside %d has %d pixels, got %s" % (nside, npix, m.shape))
    primary = b"".join([_card("SIMPLE", True), _card("BITPIX", 8), _card("NAXIS", 0), _card("EXTEND", True),
                        _card("END")])
    ext = b"".join([
        _card("XTENSION", "BINTABLE"), _card("BITPIX", 8), _card("NAXIS", 2), _card("NAXIS1", 4),
        _card("NAXIS2", npix), _card("PCOUNT", 0), _card("GCOUNT", 1), _card("TFIELDS", 1),
        _card("TTYPE1", "SIGNAL"), _card("TFORM1", "1E"),
        _card("PIXTYPE", "HEALPIX", "HEALPIX pixelisation"),
        _card("ORDERING", "NESTED" if nest else "RING", "Pixel ordering scheme"),
        _card("NSIDE", int(nside), "Resolution parameter for HEALPIX"),
        _card("FIRSTPIX", 0, "First pixel # (0 based)"), _card("LASTPIX", npix - 1, "Last pixel # (0 based)"),
        _card("INDXSCHM", "IMPLICIT", "Indexing: IMPLICIT or EXPLICIT"),
        _card("OBJECT", "FULLSKY", "Sky coverage"), _card("COORDSYS", coordsys, "Pixelisation coordinate system"),
        _card("END")])
    data = m.astype(">f4").tobytes()
    tmp = path + ".tmp"
    with open(tmp, "wb") as f:
        f.write(_pad(primary, b" "))
        f.write(_pad(ext, b" "))
        f.write(_pad(data, b"\0"))
    os.replace(tmp, path)
    return path


def read_healpix_fits(path: str):
    """(map, header dict) of a file written by write_healpix_fits."""
    raw = open(path, "rb").read()
    hdr, pos, seen_end = {}, FITS_BLOCK, 0
    # skip the primary header, then parse the extension header
    while True:
        block = raw[pos:pos + FITS_BLOCK]
        pos += FITS_BLOCK
        for i in range(0, FITS_BLOCK, 80):
            card = block[i:i + 80].decode("ascii")
            key = card[:8].strip()
            if key == "END":
                seen_end = 1
                break
            if card[8:10] == "= ":
                val = card[10:].split("/")[0].strip()
                hdr[key] = val.strip("'").strip() if val.startswith("'") else val
        if seen_end:
            break
    n = int(hdr["NAXIS2"])
    m = np.frombuffer(raw[pos:pos + 4 * n], dtype=">f4").astype(np.float32)
    return m, hdr
