#!/usr/bin/env bash
# Build the SFCMM/LBM reference's own CPU solver as a test oracle.
#
# TEST INFRASTRUCTURE ONLY.  Everything this script writes goes to oracle/_ref/
# (git-ignored).  It never writes to the reference tree.
#
# Recipe (the reference's CMake build is not used):
#   1. copy the reference's src/ to oracle/_ref/src and make one
#      behaviour-neutral edit for GCC 13: src/lbm/bnd/bnd_wall.h:84 takes
#      `&m_dirichletValue[index][0]` of a zero-length std::array for no-slip
#      walls, which libstdc++ 13 turns into a trap; `.data()` yields the same
#      (never dereferenced) pointer without indexing;
#   2. derive oracle/_ref/config.h from src/config.h.in with ENABLE_BACKTRACE
#      off (the vendored boost stacktrace is incomplete) and the CMake
#      placeholders filled in;
#   3. compile the reference's grid generator TU and oracle/ref_harness.cpp
#      (which includes src/lbm/solver.cpp) against a serial MPI stub
#      (oracle/mpi_stub/mpi.h), and link oracle/_ref/ref_harness; link the
#      same generator TU with oracle/ref_gridgen_harness.cpp into
#      oracle/_ref/ref_gridgen_harness (the generator's cell tree).
#
# Usage: oracle/build_ref.sh [reference_root]
#        oracle/build_ref.sh --root     print the reference root it would use
# The root is the argument, else $LBM_REFERENCE_ROOT, else the checkout this
# recipe was written against (/root/reference).  Exit status 3: no reference
# sources there (nothing is built).
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
if [ "${1:-}" = "--root" ]; then
  echo "${LBM_REFERENCE_ROOT:-/root/reference}"
  exit 0
fi
REF="${1:-${LBM_REFERENCE_ROOT:-/root/reference}}"
OUT="$HERE/_ref"
if [ ! -d "$REF/src/lbm" ]; then
  echo "reference sources not found at $REF" >&2
  exit 3
fi
mkdir -p "$OUT"
rm -rf "$OUT/src"
cp -r "$REF/src" "$OUT/src"
chmod -R u+w "$OUT/src"
python3 - "$OUT/src/lbm/bnd/bnd_wall.h" <<'PY'
import sys
p = sys.argv[1]
s = open(p).read()
old = "&m_dirichletValue[index][0]"
if old not in s:
    sys.exit("expected expression not found in bnd_wall.h")
open(p, "w").write(s.replace(old, "m_dirichletValue[index].data()", 1))
PY
sed -e 's|^#define ENABLE_BACKTRACE|// #define ENABLE_BACKTRACE|' \
    -e 's|@PROJECT_VERSION@|0.0.2|' -e 's|@CMAKE_CXX_COMPILER_VERSION@|13|' \
    -e 's|@CMAKE_CXX_COMPILER_ID@|GNU|' -e 's|@CMAKE_BUILD_TYPE@|Release|' \
    "$REF/src/config.h.in" > "$OUT/config.h"

CXX="${CXX:-g++}"
FLAGS=(-std=c++17 -O3 -fopenmp -w -I"$HERE/mpi_stub" -I"$OUT" -I"$OUT/src" -I"$REF/include" -isystem "$REF/external")
"$CXX" "${FLAGS[@]}" -c "$OUT/src/gridgenerator/gridGenerator.cpp" -o "$OUT/gridGenerator.o" &
P1=$!
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_harness.cpp" -o "$OUT/ref_harness.o" &
P2=$!
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_lpt_harness.cpp" -o "$OUT/ref_lpt_harness.o" &
P3=$!
"$CXX" "${FLAGS[@]}" -c "$HERE/ref_gridgen_harness.cpp" -o "$OUT/ref_gridgen_harness.o" &
P4=$!
wait $P1
wait $P2
wait $P3
wait $P4
"$CXX" -fopenmp "$OUT/gridGenerator.o" "$OUT/ref_harness.o" -o "$OUT/ref_harness" -ldl -lpthread
"$CXX" -fopenmp "$OUT/ref_lpt_harness.o" -o "$OUT/ref_lpt_harness" -ldl -lpthread
"$CXX" -fopenmp "$OUT/gridGenerator.o" "$OUT/ref_gridgen_harness.o" -o "$OUT/ref_gridgen_harness" -ldl -lpthread
echo "built $OUT/ref_harness $OUT/ref_lpt_harness $OUT/ref_gridgen_harness"
