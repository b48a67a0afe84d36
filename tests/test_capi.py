"""CPU tests of the C ABI library: it builds, loads, exports every declared
symbol, and reports errors as status codes (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, PKG


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "mpf_gb300.h")).read()
    decl = r"^\s*(?:int|void|const\s+char\s*\*|int64_t|uint32_t)\s*\**\s*(mpf_[a-z_0-9]+)\s*\("
    return sorted(set(re.findall(decl, src, flags=re.M)))


def test_library_exports_every_declared_symbol(pkg):
    import importlib
    importlib.import_module(PKG + ".build").build()
    L = pkg.library()
    names = declared_symbols()
    assert len(names) >= 10
    for name in names:
        assert hasattr(L, name), name
    from importlib import import_module
    capi = import_module(PKG + ".capi")
    assert set(capi.EXPORTS) == set(names)


def test_bad_input_is_a_status_not_a_crash(pkg):
    L = pkg.library()
    h = ctypes.c_void_p()
    assert L.mpf_octree_upload(None, 0, ctypes.byref(h)) == -1
    assert b"null" in L.mpf_last_error() or b"empty" in L.mpf_last_error()
    rc = L.mpf_octree_load(b"/nonexistent/cone.bin", ctypes.byref(h))
    assert rc == -6
    from importlib import import_module
    capi = import_module(PKG + ".capi")
    cp = capi.CatalogueParams()
    rows = np.zeros((1, 16))
    src = np.zeros((1, 6))
    assert L.mpf_catalogue_newton(None, None, ctypes.byref(cp), 1, capi.ptr(src), 6, capi.ptr(rows), None) == -1
    assert b"mpf_catalogue_newton" in L.mpf_last_error()
    p, keep = capi.make_params(1.0, planes=[0.1])
    comps = np.zeros(1, dtype=np.int32)
    maps = np.zeros(4, dtype=np.float32)
    pix = np.zeros(1, dtype=np.int64)
    assert L.mpf_hmaps_fill(None, None, ctypes.byref(p), 4, 1, capi.ptr(pix), 1, capi.ptr(comps), capi.ptr(rows),
                            capi.ptr(maps)) == -1
    assert L.mpf_pix2vec_ring(0, 1, capi.ptr(pix), capi.ptr(rows)) == -1
    assert L.mpf_cells_completion_info(None) == -1
    info = np.full(4, 7, dtype=np.int64)
    assert L.mpf_cells_completion_info(capi.ptr(info)) == 0 and not info.any()   # no build on this thread yet
    pix[0] = 12 * 4 * 4      # out of range for nside 4
    assert L.mpf_pix2vec_ring(4, 1, capi.ptr(pix), capi.ptr(rows)) == -1
    del keep
    if L.mpf_device_count() == 0:
        rec = np.zeros(2, dtype=np.dtype([("b", "u1", 48)]))
        assert L.mpf_octree_upload(ctypes.c_void_p(rec.ctypes.data), 2, ctypes.byref(h)) == -5


def test_corrupt_cone_file_is_an_io_error(pkg, tmp_path):
    """A cone .bin whose size is not a whole number of 48-byte records (a
    truncated write), or an empty one, is refused before any device work."""
    L = pkg.library()
    h = ctypes.c_void_p()
    bad = tmp_path / "truncated.bin"
    bad.write_bytes(b"\0" * (48 * 3 + 17))
    assert L.mpf_octree_load(str(bad).encode(), ctypes.byref(h)) == -6
    assert b"multiple of 48" in L.mpf_last_error()
    empty = tmp_path / "empty.bin"
    empty.write_bytes(b"")
    assert L.mpf_octree_load(str(empty).encode(), ctypes.byref(h)) == -6
    assert not h.value


def test_host_side_argument_checks(pkg):
    """Choices the host layer refuses before any library call."""
    from importlib import import_module
    maps = import_module(pkg.__name__ + ".maps")
    with pytest.raises(ValueError):
        pkg.catalogue_params(1.0, 0.68, jacobian="exact")    # the reference's plane = "exact" is not implemented either
    p, _ = pkg.catalogue_params(1.0, 0.68, jacobian="infinitesimal_born")
    assert p.jacobian_born == 1 and p.jacobian_bundle == 0
    planes = np.zeros((2, 1, 20))
    with pytest.raises(ValueError):
        maps.assemble(planes, np.zeros((2, 3)), np.ones((1, 5)), ["lensing_born"])
    assert maps.nmaps(["lensing", "lensing_born", "deflection", "dz"]) == 11


def test_cpp_call_sites_compile_against_the_header(pkg):
    """The INTEGRATION.md call sites (tests/cpp/integration_calls.cpp) compile
    as C++17 against include/mpf_gb300.h and link to the library; they run on
    a GPU in tests/test_gpu_cpp_boundary.py."""
    import os
    import shutil
    import subprocess
    import tempfile
    from conftest import ROOT
    pkg.library()
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        import pytest
        pytest.skip("no C++ compiler")
    libdir = os.path.join(ROOT, "magrathea-pathfinder_gb300")
    with tempfile.TemporaryDirectory() as d:
        subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "integration_calls.cpp"), "-o", os.path.join(d, "ic"),
                        "-L", libdir, "-lmpf_gb300"], check=True)


def test_cpp_call_sites_compile_and_link(pkg, tmp_path):
    """The reference-side C++ call sites (tests/cpp/integration_calls.cpp:
    octree and cosmology upload, FillMap's map rows, relCat's catalogue rows,
    the velocity-field deposit and maps) compile as C++17 against
    include/mpf_gb300.h with every warning an error, and link against the
    library; the GPU tests run the program."""
    import importlib
    import shutil
    import subprocess
    importlib.import_module(PKG + ".build").build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    libdir = os.path.join(ROOT, PKG)
    exe = str(tmp_path / "integration_calls")
    r = subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "integration_calls.cpp"), "-o", exe, "-L", libdir,
                        "-lmpf_gb300", "-Wl,-rpath," + libdir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)


def test_header_compiles_as_c(tmp_path):
    """The header is plain C: a C11 translation unit that includes it and
    takes the address of every declared entry point compiles warning-free."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    names = declared_symbols()
    src = tmp_path / "uses.c"
    src.write_text('#include "mpf_gb300.h"\nvoid* table[] = {\n%s\n};\nint main(void) { return table[0] == 0; }\n'
                   % ",\n".join("    (void*)&%s" % n for n in names))
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Wextra", "-Werror", "-pedantic", "-Wno-error=pedantic", "-c",
                        "-I", os.path.join(ROOT, "include"), str(src), "-o", str(tmp_path / "uses.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
