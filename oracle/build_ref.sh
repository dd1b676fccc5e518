#!/usr/bin/env bash
# Build the reference CPU oracle (oracle/_ref/libppkmhd_ref{64,32}.so) from the
# read-only ppkMHD sources, against the Kokkos-API shim in oracle/kokkos_shim.
# Test infrastructure only: used to pin the C restatement and to regenerate
# tests/golden/.  Does not run the reference's own CMake build.
#
# usage: oracle/build_ref.sh [REFERENCE_ROOT]
#   REFERENCE_ROOT defaults to $PPKMHD_REFERENCE_ROOT, else /root/reference.
#   Where that tree is absent (the GPU host) the script does nothing.
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-${PPKMHD_REFERENCE_ROOT:-/root/reference}}"
if [ ! -d "$REF/src/muscl" ]; then
  echo "reference tree not found at $REF: oracle/_ref not built"
  exit 0
fi
OUT="$HERE/_ref"
mkdir -p "$OUT"
SRCS=(
  "$HERE/ref_harness.cpp"
  "$HERE/ref_harness_hydro.cpp"
  "$REF/src/shared/HydroParams.cpp"
  "$REF/src/utils/config/ConfigMap.cpp"
  "$REF/src/utils/config/inih/INIReader.cpp"
  "$REF/src/utils/config/inih/ini.cpp"
  "$REF/src/utils/io/IO_VTK.cpp"
)
INC=(-I "$HERE/kokkos_shim" -I "$REF/src" -I "$REF/src/utils")
# -ffp-contract=off: no FMA contraction, as a plain x86-64 g++ build of the
# reference (no -mfma) computes.
FLAGS=(-std=c++17 -O2 -fPIC -shared -fopenmp -ffp-contract=off -w)
g++ "${FLAGS[@]}" -DUSE_DOUBLE "${INC[@]}" "${SRCS[@]}" -o "$OUT/libppkmhd_ref64.so" &
P64=$!
g++ "${FLAGS[@]}" "${INC[@]}" "${SRCS[@]}" -o "$OUT/libppkmhd_ref32.so" &
P32=$!
wait $P64
wait $P32
echo "built $OUT/libppkmhd_ref64.so $OUT/libppkmhd_ref32.so"
