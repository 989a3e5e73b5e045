// Learned CDF model: blob layout, device-side tables and bucket inference.
#pragma once

#include "kernels.cuh"

namespace octgb {

constexpr int kLcdfMaxSegments = 4096;             // K <= 4096 segments
constexpr int kLcdfMaxKnots = kLcdfMaxSegments + 1; // K + 1 knot positions
constexpr int kLcdfLutBits = 12;
constexpr int kLcdfLutSize = 1 << kLcdfLutBits;
constexpr uint32_t kLcdfKeyEnd = 1u << 30;
constexpr int kLcdfFix = 16;
constexpr int kLcdfMaxBuckets = 65536;
// Bucket lookup used by the bucketed sort: the exact bucket boundaries plus a
// 2^14-entry table of the bucket at the start of each 2^16-key cell.
constexpr int kLcdfBlutBits = 14;
constexpr int kLcdfBlutSize = 1 << kLcdfBlutBits;
constexpr uint32_t kLcdfMagic = 0x4643444cu;  // "LDCF"
constexpr uint32_t kLcdfVersion = 2;

// Blob header (first 256 bytes of a model buffer; persisted with the model).
struct LcdfHeader {
  uint32_t magic;
  uint32_t version;
  int32_t n_knots;    // K: segments (knot positions K + 1)
  int32_t max_knots;  // capacity the blob was laid out for
  int32_t n_sample;   // keys the fit used
  int32_t steps;      // Adam steps taken
  float loss;         // training loss of the current heights
  float z;            // sum of softplus(theta)
  int32_t n_buckets;  // NB the fixed-point tables were built for (0 = none)
};

struct LcdfLayout {
  int max_knots;
  size_t x, theta, adam_m, adam_v, y, g, yq, slope, lut, bounds, blut, bytes;
};

LcdfLayout lcdf_layout(int max_knots);

// Tables staged in shared memory for inference.
struct LcdfTables {
  const uint32_t* x;
  const uint32_t* yq;
  const unsigned long long* slope;
  const uint16_t* lut;
  int K;
  int nb;
};

size_t lcdf_tables_smem(int max_knots);

// Cooperative copy of the inference tables into shared memory (all threads of
// the block must call it; ends with a barrier).
__device__ __forceinline__ LcdfTables lcdf_load_tables(const char* blob, const LcdfLayout& L,
                                                       unsigned char* sm) {
  const LcdfHeader* h = reinterpret_cast<const LcdfHeader*>(blob);
  const int K = h->n_knots;
  unsigned long long* sslope = reinterpret_cast<unsigned long long*>(sm);
  uint32_t* sx = reinterpret_cast<uint32_t*>(sslope + L.max_knots);
  uint32_t* syq = sx + (L.max_knots + 1);
  uint16_t* slut = reinterpret_cast<uint16_t*>(syq + (L.max_knots + 1));
  const uint32_t* x = reinterpret_cast<const uint32_t*>(blob + L.x);
  const uint32_t* yq = reinterpret_cast<const uint32_t*>(blob + L.yq);
  const unsigned long long* slope = reinterpret_cast<const unsigned long long*>(blob + L.slope);
  const uint16_t* lut = reinterpret_cast<const uint16_t*>(blob + L.lut);
  for (int k = threadIdx.x; k <= K; k += blockDim.x) {
    sx[k] = x[k];
    syq[k] = yq[k];
    if (k < K) sslope[k] = slope[k];
  }
  for (int p = threadIdx.x; p <= kLcdfLutSize; p += blockDim.x) slut[p] = lut[p];
  __syncthreads();
  LcdfTables t;
  t.x = sx;
  t.yq = syq;
  t.slope = sslope;
  t.lut = slut;
  t.K = K;
  t.nb = h->n_buckets;
  return t;
}

// The same tables read in place from the model buffer (global memory).
__device__ __forceinline__ LcdfTables lcdf_tables_global(const char* blob, const LcdfLayout& L) {
  const LcdfHeader* h = reinterpret_cast<const LcdfHeader*>(blob);
  LcdfTables t;
  t.x = reinterpret_cast<const uint32_t*>(blob + L.x);
  t.yq = reinterpret_cast<const uint32_t*>(blob + L.yq);
  t.slope = reinterpret_cast<const unsigned long long*>(blob + L.slope);
  t.lut = reinterpret_cast<const uint16_t*>(blob + L.lut);
  t.K = h->n_knots;
  t.nb = h->n_buckets;
  return t;
}

// bucket(v) for a 30-bit key; never decreases with v.
__device__ __forceinline__ uint32_t lcdf_bucket(const LcdfTables& t, uint32_t v) {
  v = min(v, kLcdfKeyEnd - 1u);
  if (v < t.x[0]) return 0u;
  const uint32_t p = v >> (30 - kLcdfLutBits);
  int lo = max((int)t.lut[p] - 1, 0);
  int hi = max((int)t.lut[p + 1] - 1, 0);
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (t.x[mid] <= v) lo = mid;
    else hi = mid - 1;
  }
  const unsigned long long dv = (unsigned long long)(v - t.x[lo]);
  const uint32_t fx = t.yq[lo] + (uint32_t)((dv * t.slope[lo]) >> 32);
  return min(fx >> kLcdfFix, (uint32_t)(t.nb - 1));
}

cudaError_t launch_lcdf_fit(const uint32_t* sorted_sample, int S, int k_req, int steps, float lr,
                            char* blob, const LcdfLayout& L, int nb, cudaStream_t s);
cudaError_t launch_lcdf_train(const uint32_t* sorted_sample, int S, int steps, float lr, char* blob,
                              const LcdfLayout& L, cudaStream_t s);
cudaError_t launch_lcdf_loss_grad(const uint32_t* sorted_sample, int S, char* blob,
                                  const LcdfLayout& L, float* grad_out, cudaStream_t s);
cudaError_t launch_lcdf_tables(char* blob, const LcdfLayout& L, int nb, cudaStream_t s);
cudaError_t launch_lcdf_buckets(const char* blob, const LcdfLayout& L, const uint32_t* keys, int n,
                                uint32_t* out, cudaStream_t s);

}  // namespace octgb
