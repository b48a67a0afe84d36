"""CPU tests of the host-side writers: the catalogue ASCII files (relCat's
three files) and HEALPix FITS maps."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import load_golden


@pytest.fixture(scope="module")
def writers():
    import importlib
    return importlib.import_module("magrathea-pathfinder_gb300.writers")


def _catalogue_rows():
    g = load_golden("amr")
    good = g["ref_cat_o2_a0"]          # converged and unreachable sources
    rej = g["ref_cat_o2_a2"][:5]       # rejected (42 in column 5)
    rows = np.concatenate([good, rej])
    src = np.zeros((rows.shape[0], 8))
    src[:, 6] = np.arange(rows.shape[0]) + 1000
    src[:, 7] = 7
    return rows, src


def test_catalogue_files_split_and_round_trip(tmp_path, writers):
    rows, src = _catalogue_rows()
    good, err, rej = writers.write_catalogue(str(tmp_path / "cat_00000"), rows, src)
    assert os.path.basename(err) == "cat_00000_err.txt" and os.path.basename(rej) == "cat_00000_reject.txt"
    gl = [l.split() for l in open(good)]
    el = [l.split() for l in open(err)]
    rl = [l.split() for l in open(rej)]
    failed = rows[:, 2] == 42
    rejected = ~failed & (rows[:, 5] == 42)
    assert len(gl) == (~failed & ~rejected).sum() and len(el) == failed.sum() and len(rl) == rejected.sum() == 5
    assert all(len(l) == 18 for l in gl + rl) and all(len(l) == 7 for l in el)
    # 17 significant digits: every value reads back exactly
    ok = np.flatnonzero(~failed & ~rejected)
    back = np.array([[float(v) for v in l] for l in gl])
    np.testing.assert_array_equal(back[:, 1:17], rows[ok])
    np.testing.assert_array_equal(back[:, 0], src[ok, 6])


def test_catalogue_number_format_matches_iostreams(tmp_path, writers):
    """%.17g / %.6g are what std::ostream prints with setprecision(17) and
    with its default precision (checked against a compiled stream)."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    vals = [0.0, 1.0, 42.0, -1.5e-10, 3.0000000000000004, 1234567.0, 2.0 / 3.0, 1e22, 5e-324, 0.1]
    src = tmp_path / "fmt.cpp"
    src.write_text('#include <iostream>\n#include <iomanip>\nint main(){double v[]={%s};\n'
                   'for(double x: v) std::cout<<std::setprecision(17)<<x<<"\\n";\n'
                   'std::cout<<std::setprecision(6);\nfor(double x: v) std::cout<<x<<"\\n";}\n'
                   % ",".join(repr(v) for v in vals))
    exe = tmp_path / "fmt"
    subprocess.check_call([cxx, "-O0", str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split()
    assert out == [writers._g(v, 17) for v in vals] + [writers._g(v, 6) for v in vals]


def test_healpix_fits_round_trip(tmp_path, writers):
    nside = 4
    m = np.linspace(-1, 1, 12 * nside * nside).astype(np.float32)
    m[3] = 0.0
    m[5] = np.nan
    m[7] = np.inf
    m[9] = 1e-40          # subnormal in float32
    name = writers.map_filename(str(tmp_path) + "/", "run", nside, 2, 0.5, "redshift")
    assert os.path.basename(name) == "run_nside4_2_z_0.500000_redshift.fits"
    writers.write_healpix_fits(name, m, nside)
    assert os.path.getsize(name) % 2880 == 0
    got, hdr = writers.read_healpix_fits(name)
    assert hdr["PIXTYPE"] == "HEALPIX" and hdr["ORDERING"] == "RING" and int(hdr["NSIDE"]) == nside
    assert int(hdr["LASTPIX"]) == 12 * nside * nside - 1 and hdr["TFORM1"] == "1E"
    undef = np.float32(writers.HEALPIX_UNDEF)
    assert got[3] == undef and got[5] == undef and got[7] == undef and got[9] == undef
    keep = np.ones_like(m, dtype=bool)
    keep[[3, 5, 7, 9]] = False
    keep &= m != 0
    np.testing.assert_array_equal(got[keep], m[keep])
    with pytest.raises(ValueError):
        writers.write_healpix_fits(str(tmp_path / "bad.fits"), m[:-1], nside)
