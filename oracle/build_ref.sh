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
# The reference's checkTree (apps/cpu_demo/main.cpp:13-35), compiled from the
# unmodified demo with its main renamed and CLI11 / spdlog served by the
# stand-ins in oracle/ref_check/, driven by oracle/ref_check_main.cpp.
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off $ARCHFLAGS \
  -Dmain=ref_demo_main -I "$HERE/ref_check" -I "$HERE/glm_shim" -I "$REF/include" \
  -c "$REF/apps/cpu_demo/main.cpp" -o "$OUT/cpu_demo_main.o"
g++ -std=c++17 -O2 -fopenmp -ffp-contract=off $ARCHFLAGS \
  -I "$HERE/glm_shim" -I "$REF/include" "$HERE/ref_check_main.cpp" "$OUT/cpu_demo_main.o" \
  "${SRCS[@]:0:8}" -o "$OUT/ref_check"
echo "built $OUT/ref_check"
# The reference's device generator gpu::k_InitRandomVec4
# (kernels/cuda/00_init.cu), compiled unmodified for sm_103a into a cubin that
# tests/golden/make_device_init.py loads and launches on a GB300 the way
# apps/gpu_demo/main.cu:168-175 does (the cubin is built here, where the
# reference sources are, and run where the GPU is).
NVCC="${NVCC:-$(command -v nvcc || echo /usr/local/cuda/bin/nvcc)}"
if [ -x "$NVCC" ]; then
  "$NVCC" -cubin -gencode arch=compute_103a,code=sm_103a -O3 --expt-relaxed-constexpr \
    -I "$HERE/glm_shim" -I "$REF/include" "$REF/kernels/cuda/00_init.cu" \
    -o "$OUT/init_ref.sm_103a.cubin"
  echo "built $OUT/init_ref.sm_103a.cubin"
fi
