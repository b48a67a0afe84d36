"""Build recipe of the native library (libmpf_gb300.so) for sm_103a.

Compiles each CUDA translation unit with nvcc in parallel and links a shared
library next to this file.  The reference-order translation unit, the
catalogue root-finder, the map rows and the ray bundles are built with
-fmad=false so their float64 arithmetic keeps the reference's rounding (the
bundles' and the cell build's host code also without FMA contraction); the
others keep FMA contraction.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmpf_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

UNITS = [
    ("mpf_prop_exact.cu", ["-fmad=false"]),
    ("mpf_prop_fast.cu", []),
    ("mpf_octree.cu", []),
    ("mpf_capi.cu", []),
    ("mpf_noalloc.cu", []),
    ("mpf_catalogue.cu", ["-fmad=false"]),
    ("mpf_cat_persist.cu", []),
    ("mpf_maps.cu", ["-fmad=false"]),
    ("mpf_surrogate.cu", []),
    ("mpf_rays.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("mpf_build.cu", ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]),
    ("mpf_velocity.cu", ["-fmad=false"]),
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _sources_mtime() -> float:
    m = 0.0
    for d in (CSRC, os.path.join(HERE, "..", "include")):
        for f in os.listdir(d):
            m = max(m, os.path.getmtime(os.path.join(d, f)))
    return m


STAMP = os.path.join(OUT, "flags.txt")


def _extra_flags():
    """Extra nvcc flags from MPF_NVCC_EXTRA (tuning sweeps, e.g. -DMPF_FAST_MINB=2)."""
    return os.environ.get("MPF_NVCC_EXTRA", "").split()


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> str:
    extra = _extra_flags()
    stamp = " ".join(extra)
    same_flags = os.path.exists(STAMP) and open(STAMP).read() == stamp
    if not force and same_flags and os.path.exists(LIB) and os.path.getmtime(LIB) >= _sources_mtime():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    cc = nvcc()
    common = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", CSRC,
                     "-I", os.path.join(HERE, "..", "include")] + extra
    if ptxas_info:
        common += ["-Xptxas", "-v"]

    def one(unit):
        src, extra = unit
        obj = os.path.join(OUT, src.replace(".cu", ".o"))
        cmd = [cc, "-c", os.path.join(CSRC, src), "-o", obj] + common + extra
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        results = list(ex.map(one, UNITS))
    if verbose or ptxas_info:
        for obj, err in results:
            if err:
                sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [cc, "-shared", "-o", tmp] + [r[0] for r in results] + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_info="-v" in sys.argv)
    print(LIB)
