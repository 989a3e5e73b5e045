// Stages 7-8: octree nodes and leaf links.
//
// Replaces k_MakeOctNodes / k_LinkLeafNodes (reference
// include/kernels/07_octree.hpp:5-25, include/shared/oct.h:9-134; GPU form
// kernels/cuda/07_octree.cu:8-67) and the caller's root set-up
// (apps/cpu_demo/main.cpp:125-132).
//
// The reference's node slots come from an inclusive prefix sum, so the slot
// ranges of consecutive radix nodes overlap and several radix nodes write the
// same OctNode fields; its parallel loops then race. The contract is the
// result of a sequential run in ascending radix-node order (LinkLeaf's left
// write before its right one, all LinkLeaf writes after all MakeOctNodes
// writes). The GPU reproduces it without ordering threads:
//
//   emit      one thread per radix node computes every write it would make
//             and records, per (slot, child), the largest sequence tag
//             (atomicMax), per slot the largest writer of corner/cell_size,
//             and ORs child_node_mask bits;
//   finalize  one thread per slot turns the winning tags back into values
//             (a tag names its radix node and step) and writes the 60-byte
//             node once, coalesced.
//
// Sequence tags (32-bit, larger = later):
//   MakeOctNodes step j of node i : ((i << 4) | j) + 1        (i < 2^27)
//   LinkLeafNodes side s of node i: 0x80000000 | (i << 1) | s
#include <algorithm>

#include "octree.cuh"

namespace octgb {

size_t oct_tags_bytes(int cap) {
  const size_t c = cap > 0 ? (size_t)cap : 1;
  return align_up(c * 8 * 4, 256) + align_up(c * 4, 256) * 2;
}

OctTags oct_tags_carve(void* base, int cap) {
  const size_t c = cap > 0 ? (size_t)cap : 1;
  char* p = static_cast<char*>(base);
  OctTags t;
  t.child = reinterpret_cast<uint32_t*>(p);
  p += align_up(c * 8 * 4, 256);
  t.owner = reinterpret_cast<uint32_t*>(p);
  p += align_up(c * 4, 256);
  t.mask = reinterpret_cast<uint32_t*>(p);
  t.cap = cap;
  return t;
}

__global__ void __launch_bounds__(256) oct_zero_kernel(OctArgs a, OctTags t,
                                                       uint32_t* __restrict__ status) {
  chain_enter();
  const Sizes z = read_sizes(a);
  if (!z.fits) {
    if (blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, kStatusCapacity);
    return;
  }
  if (z.n_oct > 0)
    clear_tag_range(t, 0, (size_t)z.n_oct - 1, blockIdx.x * blockDim.x + threadIdx.x,
                    gridDim.x * blockDim.x);
}

__global__ void __launch_bounds__(256, 8) oct_emit_kernel(int mode, OctArgs a, OctTags t,
                                                       uint32_t* __restrict__ status,
                                                       bool report_capacity) {
  chain_enter();
  const Sizes z = read_sizes(a);
  if (!z.fits) {
    if (report_capacity && blockIdx.x == 0 && threadIdx.x == 0) raise_status(status, kStatusCapacity);
    return;
  }
  const int stride = gridDim.x * blockDim.x;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < z.n_brt; i += stride)
    emit_node(mode, i, a, t, z, status);
}

__global__ void __launch_bounds__(kFinThreads, 8) oct_finalize_kernel(int mode, OctArgs a, OctTags t) {
  chain_enter();
  __shared__ __align__(16) int s_nodes[kFinThreads * kNodeWords];
  const Sizes z = read_sizes(a);
  if (!z.fits || z.n_brt < 1) return;
  const int root_level = a.prefix_n[0] / 3;
  const bool fresh = mode & kOctFresh;
  int* out_words = reinterpret_cast<int*>(a.nodes);
  for (int blk = blockIdx.x * kFinThreads; blk < z.n_oct; blk += gridDim.x * kFinThreads) {
    const int p = blk + threadIdx.x;
    const int count = min(kFinThreads, z.n_oct - blk);
    if (p < z.n_oct) finalize_slot(fresh, p, a, t, root_level, s_nodes + threadIdx.x * kNodeWords);
    bulk_fence_writes();
    __syncthreads();
    int* dst = out_words + (size_t)blk * kNodeWords;
    // 256 nodes are 960 16-byte words; blk is a multiple of 256, so dst is
    // 16-byte aligned whenever the node array is.
    const int words = count * kNodeWords;
    if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0 && (words & 3) == 0) {
      // one bulk copy of the staged block (the TMA engine writes it)
      if (threadIdx.x == 0) {
        bulk_store_s2g(dst, s_nodes, (uint32_t)words * 4u);
        bulk_wait_read();  // the stage is free for the next block
      }
    } else {
      int k0 = 0;
      if ((reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        const int quads = words >> 2;
        const uint4* src4 = reinterpret_cast<const uint4*>(s_nodes);
        uint4* dst4 = reinterpret_cast<uint4*>(dst);
        for (int k = threadIdx.x; k < quads; k += kFinThreads) dst4[k] = src4[k];
        k0 = quads << 2;
      }
      for (int k = k0 + threadIdx.x; k < words; k += kFinThreads) dst[k] = s_nodes[k];
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

cudaError_t launch_octree(int mode, const OctArgs& a, const OctTags& t, uint32_t* status,
                          cudaStream_t s, Recorder* rec, bool tags_clear) {
  cudaError_t e;
  if (!tags_clear) {
    const int zgrid = device_sm_count() * 8;
    e = launch_chained(oct_zero_kernel, dim3(zgrid), dim3(256), 0, s, a, t, status);
    if (e != cudaSuccess) return e;
    mark(rec, s);
  }
  int nb = a.d_unique ? a.n_brt_host : a.n_brt_host;
  int egrid = (nb + 255) / 256;
  if (egrid < 1) egrid = 1;
  e = launch_chained(oct_emit_kernel, dim3(egrid), dim3(256), 0, s, mode, a, t, status, tags_clear);
  if (e != cudaSuccess) return e;
  mark(rec, s);
  // One wave at 8 CTAs per SM, each walking the 256-slot blocks: the node
  // count is known only on the device, and a grid sized by the capacity would
  // leave its CTAs past the last node to start, wait and exit in the tail.
  int fgrid = (a.cap + kFinThreads - 1) / kFinThreads;
  fgrid = std::min(fgrid, device_sm_count() * 8);
  if (fgrid < 1) fgrid = 1;
  e = launch_chained(oct_finalize_kernel, dim3(fgrid), dim3(kFinThreads), 0, s, mode, a, t);
  if (e == cudaSuccess) mark(rec, s);
  return e;
}

__global__ void publish_counts_kernel(const int* d_unique, const int* d_max_slot,
                                      const uint32_t* status, int* out) {
  chain_enter();
  const int u = *d_unique;
  const int b = max(u - 1, 0);
  out[0] = u;
  out[1] = b;
  out[2] = b >= 1 ? *d_max_slot + 1 : 0;
  out[3] = status ? (int)*status : 0;
}

cudaError_t launch_publish_counts(const int* d_unique, const int* d_max_slot,
                                  const uint32_t* status, int* out, cudaStream_t s) {
  return launch_chained(publish_counts_kernel, dim3(1), dim3(1), 0, s, d_unique, d_max_slot, status,
                        out);
}

}  // namespace octgb
