#!/usr/bin/env bash
# Builds oracle/_ref/libseismic_ref.so from the reference's own C++ sources, in
# place (they are read, never copied), plus oracle/ref_harness.cpp, a
# single-rank MPI stub header (oracle/mpi_stub/mpi.h) and stubs for the two
# off-path RTM streaming classes whose shipped sources do not compile
# (oracle/ref_stubs.cpp). Flags are the reference's own (CMakeLists.txt:24-35)
# plus -fno-finite-math-only: under plain -ffast-math GCC folds std::isfinite
# to true, which deletes the reference's NaN/Inf guards
# (wave_equation.cpp:345-397, rtm_engine.cpp:45-48, fault_tolerance.cpp:72-157);
# the fixtures pin the guards as written in the source.
# x86-64 only (the reference includes <x86intrin.h>/<immintrin.h>); the GPU
# box has no reference sources, so this runs only where they are present.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${SEISMIC_REFERENCE_DIR:-/root/reference}"
SRC="$REF/src/cpp"
OUT="$HERE/_ref"
if [ ! -d "$SRC" ]; then
  echo "reference sources not found at $SRC; skipping oracle/_ref" >&2
  exit 0
fi
case "$(uname -m)" in
  x86_64) ARCHFLAGS="-march=native -mavx2 -mfma" ;;
  *) echo "reference sources need x86 intrinsics; skipping oracle/_ref on $(uname -m)" >&2; exit 0 ;;
esac
mkdir -p "$OUT"
g++ -std=c++17 -O3 -ffast-math -fno-finite-math-only $ARCHFLAGS -fPIC -shared -w \
  -include functional -I"$HERE/mpi_stub" -I"$SRC" \
  "$SRC/core/grid.cpp" "$SRC/core/mpi_context.cpp" "$SRC/core/config.cpp" \
  "$SRC/core/fault_tolerance.cpp" "$SRC/solver/wave_equation.cpp" "$SRC/solver/boundary.cpp" \
  "$SRC/rtm/rtm_engine.cpp" "$SRC/rtm/mmap_writer.cpp" "$SRC/sparse/csr_matrix.cpp" \
  "$HERE/ref_stubs.cpp" "$HERE/ref_harness.cpp" \
  -o "$OUT/libseismic_ref.so.tmp" -Wl,--no-undefined -lpthread
mv "$OUT/libseismic_ref.so.tmp" "$OUT/libseismic_ref.so"
echo "built $OUT/libseismic_ref.so"
