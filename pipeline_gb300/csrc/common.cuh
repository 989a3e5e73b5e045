// Shared device helpers for the sm_103a octree-build kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace octgb {

// Device status word bits (mirrored by OCT_STATUS_* in include/octree_gb300.h).
constexpr uint32_t kStatusSpinTimeout = 1u;  // a look-back wait ran out its bound
constexpr uint32_t kStatusWalkLimit = 2u;    // a parent walk exceeded its bound
constexpr uint32_t kStatusRange = 4u;        // a coordinate outside [min, min + range]
constexpr uint32_t kStatusCapacity = 8u;     // octree node capacity too small

// Look-back waits are bounded in time: a wait that has not seen the flag it
// polls after kWaitLimitNs of %globaltimer gives up, sets the status bit and
// lets its kernel return (no wait lasts longer than this, and a build in
// which one gave up reports OCT_STATUS_SPIN_TIMEOUT instead of hanging).
// kWaitPollCap also ends a wait after that many polls (at least 64 ns each)
// should the timer not advance.
constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s
constexpr uint32_t kWaitPollCap = 1u << 26;

constexpr int kWarp = 32;

// Programmatic dependent launch. A kernel launched by launch_chained (host
// side, kernels.cuh) into a CUDA graph may have its CTAs scheduled while the
// kernel before it is still finishing; chain_wait() blocks until that kernel has
// completed and its writes are visible (for a kernel launched without the
// attribute it returns at once). Every kernel that launch_chained launches
// calls chain_wait() before its first global-memory access, then
// chain_release(), which lets the next kernel's CTAs be scheduled once all of
// this kernel's CTAs have started: so at most one waiting grid sits beside a
// running one, and no running grid ever lacks the slots its later CTAs need.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_release() {
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}
__device__ __forceinline__ void chain_enter() {
  chain_wait();
  chain_release();
}

__device__ __forceinline__ uint32_t lane_id() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%laneid;" : "=r"(r));
  return r;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(r));
  return r;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Relaxed (no ordering) loads for look-back words whose flag and value share
// one word: independent loads of a window can all be in flight at once.
__device__ __forceinline__ uint32_t ld_relaxed_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// Streaming (evict-first) 128-bit load for data read exactly once.
__device__ __forceinline__ float4 ld_stream_f4(const float4* p) {
  float4 v;
  asm volatile("ld.global.cs.v4.f32 {%0,%1,%2,%3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p));
  return v;
}

// Bulk (TMA engine) copy of `bytes` from shared to global memory, issued by
// one thread: both addresses 16-byte aligned, bytes a multiple of 16. The
// fence makes the block's ordinary shared-memory stores (ordered by a
// preceding barrier) visible to the copy; wait_read returns once the source
// may be overwritten, wait_all once the writes are done.
// Every thread that wrote shared memory a bulk copy will read runs this
// before the barrier that precedes the copy: its generic-proxy writes are
// then ordered before the async proxy's reads.
__device__ __forceinline__ void bulk_fence_writes() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bulk_store_s2g(void* gdst, const void* ssrc, uint32_t bytes) {
  const uint32_t s = (uint32_t)__cvta_generic_to_shared(ssrc);
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(gdst), "r"(s),
               "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.commit_group;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_read() {
  asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
}
__device__ __forceinline__ void bulk_wait_all() {
  asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Bound of one wait. expired() is called after every poll that did not find
// its flag: it backs off (64 ns sleeps after the first few polls), reads the
// timer on the first poll and every 32nd after it, and returns true once
// limit_ns have passed since the first poll (or after kWaitPollCap polls).
struct WaitBound {
  unsigned long long limit_ns;
  unsigned long long t0 = 0;
  uint32_t polls = 0;
  __device__ __forceinline__ explicit WaitBound(unsigned long long limit) : limit_ns(limit) {}
  __device__ __forceinline__ bool expired() {
    ++polls;
    if (polls > 8) __nanosleep(64);
    if ((polls & 31u) == 1u) {
      const unsigned long long now = global_ns();
      if (polls == 1u) t0 = now;
      else if (now - t0 > limit_ns) return true;
    }
    return polls > kWaitPollCap;
  }
};

__device__ __forceinline__ void raise_status(uint32_t* status, uint32_t bit) {
  if (status) atomicOr(status, bit);
}

// Karras-tree helpers with the reference's integer semantics
// (kernels/04_radix_tree.cpp:16-37): delta is clz(a ^ b) - 1 stored in a
// uint8_t (so keys differing in bit 31 give 255); clz(0) is 32.
__device__ __forceinline__ int delta_u8(uint32_t a, uint32_t b) {
  return (int)(uint8_t)(__clz(a ^ b) - 1);
}

__device__ __forceinline__ int log2_ceil_u32(uint32_t x) {
  const int fl = 31 - __clz(x);
  return fl + ((1u << fl) < x);
}

// Morton helpers (include/shared/morton.h:15-80), restated.
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  uint32_t x = v & 0x3ffu;
  x = (x | (x << 16)) & 0x030000ffu;
  x = (x | (x << 8)) & 0x0300f00fu;
  x = (x | (x << 4)) & 0x030c30c3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__device__ __forceinline__ uint32_t compact3(uint32_t m) {
  uint32_t x = m & 0x09249249u;
  x = (x ^ (x >> 2)) & 0x030c30c3u;
  x = (x ^ (x >> 4)) & 0x0300f00fu;
  x = (x ^ (x >> 8)) & 0x030000ffu;
  x = (x ^ (x >> 16)) & 0x000003ffu;
  return x;
}

// FP32 quantisation in the reference's operation order, each step rounded to
// nearest with no contraction: (v - min) / range * 1024, truncated.
// One axis of include/shared/morton.h:15-22: (uint32)((v - min) / range * 1024)
// with an IEEE single division, sets ok = false outside [min, min + range]
// (or NaN), where the reference's float-to-uint cast is undefined.
//
// Only floor(RN(a / range) * 1024) is needed (a = v - min, the * 1024 is
// exact), so t = RN(a * scale), scale = RN(1024 / range), stands in for it
// whenever no integer lies within t * 2^-20 of t: t and RN(a / range) * 1024
// are each within a relative 2^-23 of a * 1024 / range, so they are within
// t * 2^-22.3 of each other and have the same floor. Otherwise (near a cell
// boundary, t < 0, huge, NaN) the division itself decides.
__device__ __forceinline__ uint32_t quantise(float v, float min_coord, float range, float scale,
                                             bool& ok) {
  const float a = __fsub_rn(v, min_coord);
  const float t = __fmul_rn(a, scale);
  const float k = floorf(t);
  const float f = __fsub_rn(t, k);
  const float m = __fmul_rn(t, 0x1p-20f);
  if (t >= 0.0f && t < 0x1p22f && f > m && __fsub_rn(1.0f, f) > m) {
    ok = ok && k < 1024.0f;
    return (uint32_t)k;
  }
  const float q = __fmul_rn(__fdiv_rn(a, range), 1024.0f);
  ok = ok && q >= 0.0f && q <= 1024.0f;
  return __float2uint_rz(q);
}

// 30-bit Morton code of a point (morton.h:15-39); ok as for quantise.
__device__ __forceinline__ uint32_t morton_code(float x, float y, float z, float min_coord,
                                                float range, bool& ok) {
  const float scale = __fdiv_rn(1024.0f, range);
  ok = true;
  const uint32_t qx = quantise(x, min_coord, range, scale, ok);
  const uint32_t qy = quantise(y, min_coord, range, scale, ok);
  const uint32_t qz = quantise(z, min_coord, range, scale, ok);
  return spread3(qx) | (spread3(qy) << 1) | (spread3(qz) << 2);
}

// The same code with the bit spreads read from a table in shared memory
// (lut[v] = spread3(v), v < 1024: fill_spread_lut) and the 1024 / range
// quotient computed by the caller (scale = __fdiv_rn(1024.0f, range)).
__device__ __forceinline__ void fill_spread_lut(uint32_t* lut) {
  for (uint32_t v = threadIdx.x; v < 1024u; v += blockDim.x) lut[v] = spread3(v);
}
__device__ __forceinline__ uint32_t morton_code_lut(float x, float y, float z, float min_coord,
                                                    float range, float scale,
                                                    const uint32_t* lut, bool& ok) {
  ok = true;
  const uint32_t qx = quantise(x, min_coord, range, scale, ok);
  const uint32_t qy = quantise(y, min_coord, range, scale, ok);
  const uint32_t qz = quantise(z, min_coord, range, scale, ok);
  return lut[qx & 0x3ffu] | (lut[qy & 0x3ffu] << 1) | (lut[qz & 0x3ffu] << 2);
}

// morton32_to_xyz: per axis (raw / 1024) * range + min, w = 1.
__device__ __forceinline__ float4 decode_corner(uint32_t code, float min_coord, float range) {
  float4 c;
  // v / 1024 for an integer v < 1024 is exact, so it is the product v * 2^-10.
  c.x = __fadd_rn(__fmul_rn(__fmul_rn((float)compact3(code), 0x1p-10f), range), min_coord);
  c.y = __fadd_rn(__fmul_rn(__fmul_rn((float)compact3(code >> 1), 0x1p-10f), range), min_coord);
  c.z = __fadd_rn(__fmul_rn(__fmul_rn((float)compact3(code >> 2), 0x1p-10f), range), min_coord);
  c.w = 1.0f;
  return c;
}

// Block-wide exclusive sum of one value per thread (THREADS a multiple of 32).
template <int THREADS, typename T>
__device__ __forceinline__ T block_exclusive_sum(T v, T* warp_tot /* THREADS/32 */, T* total) {
  constexpr int W = THREADS / kWarp;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  T inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    T x = lane < W ? warp_tot[lane] : T(0);
    T xi = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      T t = __shfl_up_sync(0xffffffffu, xi, o);
      if (lane >= o) xi += t;
    }
    if (lane < W) warp_tot[lane] = xi - x;
    if (lane == W - 1) *total = xi;
  }
  __syncthreads();
  const T r = warp_tot[w] + inc - v;
  __syncthreads();
  return r;
}

}  // namespace octgb
