"""The C++ side of the boundary: tests/cpp/integration_calls.cpp holds the
reference-side call sites of INTEGRATION.md (octree and cosmology upload,
FillMap's map rows, relCat's catalogue rows) written with the reference's
container types, compiled as C++17 against include/mpf_gb300.h and linked to
libmpf_gb300.so.  It runs on the AMR golden fixture; its rows must equal the
reference's FillMap maps and relCat rows within the exact-mode tolerances of
tests/test_gpu_maps.py and tests/test_gpu_catalogue.py."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def program(gpu_lib, tmp_path_factory):
    out = tmp_path_factory.mktemp("cpp")
    exe = str(out / "integration_calls")
    libdir = os.path.join(ROOT, "magrathea-pathfinder_gb300")
    cxx = shutil.which("g++") or shutil.which("c++")
    assert cxx, "no C++ compiler"
    subprocess.run([cxx, "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "integration_calls.cpp"), "-o", exe, "-L", libdir,
                    "-lmpf_gb300", "-Wl,-rpath," + libdir], check=True)
    return exe


@pytest.mark.parametrize("order", [1, 2])
def test_cpp_call_sites_match_reference(program, tmp_path, order):
    g = load_golden("amr")
    d = str(tmp_path)
    np.ascontiguousarray(g["records"]).tofile(os.path.join(d, "records.in"))
    np.concatenate([g["cosmo_" + k] for k in ("t", "a", "dadt", "d2adt2")]).tofile(os.path.join(d, "cosmology.in"))
    acc = float(g["cat_accuracy"][0])
    np.array([float(g["cosmo_length"]), float(g["cosmo_h"]), float(g["cosmo_mpc"]), float(g["nsteps"]),
              float(g["nside"]), float(order), acc, *g["cat_vobs"]]).tofile(os.path.join(d, "scalars.in"))
    np.ascontiguousarray(g["zs"], dtype=np.float64).tofile(os.path.join(d, "surfaces.in"))
    np.ascontiguousarray(g["homogeneous"], dtype=np.float64).tofile(os.path.join(d, "homogeneous.in"))
    np.ascontiguousarray(g["pixels"], dtype=np.int64).tofile(os.path.join(d, "pixels.in"))
    src = g["cat_src"]
    src8 = np.concatenate([src, np.arange(src.shape[0], dtype=float)[:, None], np.ones((src.shape[0], 1))], axis=1)
    np.ascontiguousarray(src8).tofile(os.path.join(d, "sources.in"))
    r = subprocess.run([program, d], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ref = g["ref_maps_o%d" % order]
    maps = np.fromfile(os.path.join(d, "maps.out"), dtype=np.float32).reshape(ref.shape)
    assert str(g["components"]) == "lensing,dr,dz,isw,dens,dens_max,steps,phi,deflection"
    for row in range(4):
        scale = max(np.abs(ref[:, row]).max(), 1e-6)
        assert np.abs(maps[:, row] - ref[:, row]).max() <= 1e-6 * scale + 2e-7 * (row == 3), row
    for row in range(4, ref.shape[1]):
        scale = np.abs(ref[:, row]).max() + 1e-30
        assert np.abs(maps[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row
    rows = np.fromfile(os.path.join(d, "catalogue.out")).reshape(-1, 16)
    cref = g["ref_cat_o%d_a0" % order]
    failed = cref[:, 2] == 42
    np.testing.assert_array_equal(rows[:, 2] == 42, failed)
    np.testing.assert_array_equal(rows[~failed, 5], cref[~failed, 5])
    assert np.abs(rows[~failed, 2:4] - cref[~failed, 2:4]).max() <= 1e-12
    assert np.abs(rows[~failed, 6:12] - cref[~failed, 6:12]).max() <= 1e-12
    assert np.abs(rows[~failed, 12:16] - cref[~failed, 12:16]).max() <= 1e-10


def test_cpp_velocity_map_driver(program, tmp_path):
    """The velocity-field map driver's call sites (velocity-field
    maps) in C++: the deposit over two particle files gives the reference's
    velocities and masses bit for bit, the maps traced with the observer
    velocity the reference's rows within the map tolerances, and the accuracy
    statistic of the FP32-gather call stays inside 1e-6."""
    g = load_golden("amr")
    v = load_golden("velocity")
    d = str(tmp_path)
    np.ascontiguousarray(g["records"]).tofile(os.path.join(d, "records.in"))
    np.concatenate([g["cosmo_" + k] for k in ("t", "a", "dadt", "d2adt2")]).tofile(os.path.join(d, "cosmology.in"))
    np.array([float(g["cosmo_length"]), float(v["nsteps"]), float(v["nside"]), *v["vobs"],
              float(v["part_split"])]).tofile(os.path.join(d, "scalars.in"))
    np.ascontiguousarray(v["zs"], dtype=np.float64).tofile(os.path.join(d, "surfaces.in"))
    np.ascontiguousarray(g["homogeneous"], dtype=np.float64).tofile(os.path.join(d, "homogeneous.in"))
    np.ascontiguousarray(v["pixels"], dtype=np.int64).tofile(os.path.join(d, "pixels.in"))
    np.ascontiguousarray(v["part_pos"], dtype=np.float32).tofile(os.path.join(d, "pos.in"))
    np.ascontiguousarray(v["part_vel"], dtype=np.float32).tofile(os.path.join(d, "vel.in"))
    r = subprocess.run([program, d, "velocity"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    vel = np.fromfile(os.path.join(d, "velocity.out"), dtype=np.float32).reshape(-1, 3)
    rho = np.fromfile(os.path.join(d, "rho.out"), dtype=np.float32)
    np.testing.assert_array_equal(vel.view(np.uint32), v["ref_vel_tsc"].view(np.uint32))
    np.testing.assert_array_equal(rho.view(np.uint32), v["ref_rho_tsc"].view(np.uint32))
    ref = v["ref_maps_o2"]
    maps = np.fromfile(os.path.join(d, "maps.out"), dtype=np.float32).reshape(ref.shape)
    for row in range(4):
        scale = max(np.abs(ref[:, row]).max(), 1e-6)
        assert np.abs(maps[:, row] - ref[:, row]).max() <= 1e-6 * scale + 2e-7 * (row == 3), row
    for row in range(4, ref.shape[1]):
        scale = np.abs(ref[:, row]).max() + 1e-30
        assert np.abs(maps[:, row] - ref[:, row]).max() <= 2e-6 * scale + 1e-12, row
    rays, differs, defl, red, kabs, kscale = np.fromfile(os.path.join(d, "accuracy.out"))
    assert rays == 64 and differs == 0 and defl <= 1e-6 and red <= 1e-6 and kabs <= 1e-6 * max(kscale, 1e-6)
