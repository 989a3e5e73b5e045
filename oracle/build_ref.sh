#!/usr/bin/env bash
# Builds the reference's own CPU stage implementation into oracle/_ref/libref.so.
#
# TEST INFRASTRUCTURE ONLY: the result pins the C restatement (oracle/oracle.c)
# and generates tests/golden/. It compiles the reference sources where they lie
# (read-only, never copied) plus oracle/ref_harness.cpp and the glm stand-in in
# oracle/glm_shim/. Outputs go to oracle/_ref/ only.
#
# Flags: -O2 as the reference's release build; -ffp-contract=off so no FMA
# contraction changes the FP32 Morton quantisation or decode; -mlzcnt on x86 so
# __builtin_clz(0) is 32 as on aarch64 and on the GPU (only the degenerate
# two-key radix tree evaluates it).
#
# Usage: oracle/build_ref.sh [REFERENCE_ROOT]   (default: /root/reference)
set -euo pipefail
HERE="$(cd "$(dirname "${BASH_SOURCE[0]}")" && pwd)"
REF="${1:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -d "$REF/kernels" ]; then
  echo "reference sources not found at $REF; skipping oracle/_ref" >&2
  exit 0
fi
mkdir -p "$OUT"
ARCHFLAGS=""
case "$(uname -m)" in
  x86_64) ARCHFLAGS="-mlzcnt" ;;
esac
SRCS=(
  "$REF/kernels/00_init.cpp" "$REF/kernels/01_morton.cpp" "$REF/kernels/02_sort.cpp"
  "$REF/kernels/03_unique.cpp" "$REF/kernels/04_radix_tree.cpp" "$REF/kernels/05_edge_count.cpp"
  "$REF/kernels/06_partial_sum.cpp" "$REF/kernels/07_octree.cpp" "$HERE/ref_harness.cpp"
)
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off $ARCHFLAGS -fPIC -shared \
  -I "$HERE/glm_shim" -I "$REF/include" "${SRCS[@]}" -o "$OUT/libref.so"
echo "built $OUT/libref.so"
