#!/usr/bin/env bash
# Builds the reference CPU oracle into oracle/_ref/ from the reference sources
# where they lie: MPF_REFERENCE_SRC, else the reference checked out beside
# this repository (../reference/src relative to the repository root).
#
# Steps:
#  1. Write a patched copy of magrathea/simplehyperoctree.h into
#     oracle/_ref/patched/: its never-instantiated field accessors
#     (declarations at lines 184-197, definitions at 1046-1259) do not compile
#     with GCC 13 ("data is not a template"); they are commented out / #if 0'd.
#     Nothing else is changed.
#  2. Compile with the reference Makefile's flags (-O3 -std=c++17 -DEXTENT=4
#     -DSIZEOFOCTREE=48 -DIOGROUPSIZE=1 -DMEMORY_SAVING, no -march), with
#     single-rank MPI and inert HDF5 stand-ins from oracle/stubs/.
#     Outputs: libref_o0.so / libref_o1.so / libref_o2.so (ref_harness.cpp at ORDER=0 / 1 / 2),
#     libref_vel_o0.so / _o1 / _o2 (the same with -DVELOCITYFIELD, the reference's
#     velocity-field build: gravity2.h cells, the Doppler redshift, the particle deposit)
#     and the reference's own create_octree executable.
#  -ffp-contract=off keeps the x86 and Arm builds free of FMA contraction, as
#  the reference's x86-64 build is.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
SRC="${MPF_REFERENCE_SRC:-$HERE/../../reference/src}"
OUT="$HERE/_ref"
if [ ! -f "$SRC/magrathea/simplehyperoctree.h" ]; then
    echo "reference sources not found at $SRC" >&2
    exit 2
fi
mkdir -p "$OUT/patched/magrathea"
sed -e '184,197s|^|//|' -e '1046i #if 0' -e '1259a #endif' \
    "$SRC/magrathea/simplehyperoctree.h" > "$OUT/patched/magrathea/simplehyperoctree.h"
CXX="${CXX:-g++}"
FLAGS=(-O3 -std=c++17 -ffp-contract=off -DEXTENT=4 -DSIZEOFOCTREE=48 -DIOGROUPSIZE=1 -DMEMORY_SAVING
       -w -I"$HERE/stubs" -I"$OUT/patched" -I"$SRC" -I"$SRC/magrathea")
pids=()
for o in 0 1 2; do
    "$CXX" "${FLAGS[@]}" -DORDER=$o -fPIC -shared "$HERE/ref_harness.cpp" -o "$OUT/libref_o$o.so" -lpthread &
    pids+=($!)
    "$CXX" "${FLAGS[@]}" -DORDER=$o -DVELOCITYFIELD -fPIC -shared "$HERE/ref_harness.cpp" \
        -o "$OUT/libref_vel_o$o.so" -lpthread &
    pids+=($!)
done
"$CXX" "${FLAGS[@]}" -DORDER=1 -include "$OUT/patched/magrathea/simplehyperoctree.h" \
    "$SRC/create_octree.cpp" -o "$OUT/create_octree" -lpthread &
pids+=($!)
rc=0
for p in "${pids[@]}"; do wait "$p" || rc=1; done
# keep only the built binaries in oracle/_ref/
rm -rf "$OUT/patched"
exit $rc
