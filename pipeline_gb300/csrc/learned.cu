// Learned CDF of the Morton-key distribution (fit, inference).
//
// Model: a monotone piecewise-linear CDF. Knots x_0 < ... < x_K (x_K = 2^30)
// are distinct keys at evenly spaced ranks of a sorted training sample of keys
// the pipeline produced; heights y_k = (sum_{m<k} softplus(theta_m)) / Z with
// Z = sum_m softplus(theta_m), so 0 = y_0 <= y_1 <= ... <= y_K = 1. A key v in
// segment k maps to F(v) = y_k + (y_{k+1} - y_k) (v - x_k) / (x_{k+1} - x_k).
//
// Fit (all on the GPU): knots from the sorted sample, then Adam steps on
// L = mean_i (F(v_i) - (i + 1/2) / S)^2 with our own forward/backward kernels
// (analytic gradient through the normalised cumulative softplus).
//
// Buckets: exact integer arithmetic on fixed-point tables, so bucket(v) never
// decreases with v and the CPU reference reproduces it bit for bit:
//   Yq_k = round(y_k NB 2^16) (non-decreasing, Yq_0 = 0, Yq_K = NB 2^16),
//   slope_k = floor((Yq_{k+1} - Yq_k) 2^32 / (x_{k+1} - x_k)),
//   bucket(v) = min(NB - 1, (Yq_k + ((v - x_k) slope_k >> 32)) >> 16).
// A 4096-entry table on the top 12 key bits narrows the knot search.
#include "learned.cuh"

namespace octgb {

// ---------------------------------------------------------------- layout --
LcdfLayout lcdf_layout(int max_knots) {
  LcdfLayout L{};
  const size_t K = (size_t)max_knots;  // segments
  size_t o = 256;                      // header
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + bytes, 256);
    return at;
  };
  L.max_knots = max_knots;
  L.x = take(4 * (K + 1));
  L.theta = take(4 * K);
  L.adam_m = take(4 * K);
  L.adam_v = take(4 * K);
  L.y = take(4 * (K + 1));
  L.g = take(4 * (K + 1));
  L.yq = take(4 * (K + 1));
  L.slope = take(8 * K);
  L.lut = take(2 * (kLcdfLutSize + 1));
  L.bounds = take(4 * ((size_t)kLcdfMaxBuckets + 1));
  L.blut = take(2 * ((size_t)kLcdfBlutSize + 1));
  L.bytes = o;
  return L;
}

__device__ __forceinline__ float softplusf(float t) { return t > 20.f ? t : log1pf(expf(t)); }
__device__ __forceinline__ float sigmoidf_(float t) { return 1.f / (1.f + expf(-t)); }

// Largest k in [lo, hi] with x[k] <= v (x[lo] <= v assumed unless k = lo).
__device__ __forceinline__ int knot_search(const uint32_t* x, int lo, int hi, uint32_t v) {
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (x[mid] <= v) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// ------------------------------------------------------------- knots init --
// One block: knots from the sorted sample; theta = log(e - 1) (softplus 1).
__global__ void __launch_bounds__(1024)
    lcdf_knots_kernel(const uint32_t* __restrict__ sample, int S, int k_req, char* blob,
                      LcdfLayout L) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t total;
  LcdfHeader* h = reinterpret_cast<LcdfHeader*>(blob);
  uint32_t* x = reinterpret_cast<uint32_t*>(blob + L.x);
  constexpr int PER = (kLcdfMaxKnots + 1023) / 1024;
  uint32_t cand[PER];
  uint32_t keep = 0;
  int cnt = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int k = threadIdx.x * PER + j;
    cand[j] = 0;
    if (k < k_req) {
      const long long idx = (long long)k * S / k_req;
      cand[j] = sample[idx];
      const uint32_t prev = k == 0 ? 0u : sample[(long long)(k - 1) * S / k_req];
      if (k == 0 || cand[j] != prev) {
        keep |= 1u << j;
        ++cnt;
      }
    }
  }
  uint32_t pos = block_exclusive_sum<1024>((uint32_t)cnt, warp_tot, &total);
#pragma unroll
  for (int j = 0; j < PER; ++j)
    if (keep >> j & 1u) x[pos++] = cand[j];
  const int K = (int)total;
  if (threadIdx.x == 0) {
    x[K] = kLcdfKeyEnd;
    h->magic = kLcdfMagic;
    h->version = kLcdfVersion;
    h->n_knots = K;
    h->max_knots = L.max_knots;
    h->n_sample = S;
    h->steps = 0;
    h->loss = 0.f;
    h->n_buckets = 0;
  }
  float* theta = reinterpret_cast<float*>(blob + L.theta);
  float* m = reinterpret_cast<float*>(blob + L.adam_m);
  float* v = reinterpret_cast<float*>(blob + L.adam_v);
  for (int k = threadIdx.x; k < K; k += 1024) {
    theta[k] = 0.5413248546129181f;  // log(e - 1)
    m[k] = 0.f;
    v[k] = 0.f;
  }
}

// -------------------------------------------------------------- heights --
// One block: y from theta; zero the gradient accumulators and the loss.
__global__ void __launch_bounds__(1024) lcdf_prep_kernel(char* blob, LcdfLayout L) {
  __shared__ float warp_tot[32];
  __shared__ float total;
  LcdfHeader* h = reinterpret_cast<LcdfHeader*>(blob);
  const int K = h->n_knots;
  const float* theta = reinterpret_cast<const float*>(blob + L.theta);
  float* y = reinterpret_cast<float*>(blob + L.y);
  float* g = reinterpret_cast<float*>(blob + L.g);
  constexpr int PER = (kLcdfMaxKnots + 1023) / 1024;
  float s[PER];
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int k = threadIdx.x * PER + j;
    s[j] = k < K ? softplusf(theta[k]) : 0.f;
    sum += s[j];
  }
  float run = block_exclusive_sum<1024>(sum, warp_tot, &total);
  const float Z = total;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int k = threadIdx.x * PER + j;
    if (k < K) y[k] = run / Z;
    run += s[j];
  }
  for (int k = threadIdx.x; k <= K; k += 1024) g[k] = 0.f;
  if (threadIdx.x == 0) {
    y[K] = 1.f;
    h->z = Z;
    h->loss = 0.f;
  }
}

// ------------------------------------------------------ forward/backward --
// One thread per sample key (sorted): loss and dL/dy accumulated per knot.
__global__ void __launch_bounds__(256)
    lcdf_fwd_bwd_kernel(const uint32_t* __restrict__ sample, int S, char* blob, LcdfLayout L) {
  extern __shared__ __align__(16) unsigned char sm[];
  LcdfHeader* h = reinterpret_cast<LcdfHeader*>(blob);
  const int K = h->n_knots;
  uint32_t* sx = reinterpret_cast<uint32_t*>(sm);
  float* sy = reinterpret_cast<float*>(sx + (K + 1));
  float* sg = sy + (K + 1);
  __shared__ float s_loss[8];
  const uint32_t* x = reinterpret_cast<const uint32_t*>(blob + L.x);
  const float* y = reinterpret_cast<const float*>(blob + L.y);
  for (int k = threadIdx.x; k <= K; k += blockDim.x) {
    sx[k] = x[k];
    sy[k] = y[k];
    sg[k] = 0.f;
  }
  __syncthreads();
  float lsum = 0.f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S; i += gridDim.x * blockDim.x) {
    const uint32_t v = sample[i];
    int k = 0;
    float f = 0.f;
    if (v >= sx[0]) {
      k = knot_search(sx, 0, K - 1, v);
      f = (float)(v - sx[k]) / (float)(sx[k + 1] - sx[k]);
    }
    const float F = sy[k] + (sy[k + 1] - sy[k]) * f;
    const float t = ((float)i + 0.5f) / (float)S;
    const float r = F - t;
    lsum += r * r;
    const float dF = 2.f * r / (float)S;
    atomicAdd(&sg[k], dF * (1.f - f));
    atomicAdd(&sg[k + 1], dF * f);
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if ((threadIdx.x & 31) == 0) s_loss[threadIdx.x >> 5] = lsum;
  __syncthreads();
  float* g = reinterpret_cast<float*>(blob + L.g);
  for (int k = threadIdx.x; k <= K; k += blockDim.x)
    if (sg[k] != 0.f) atomicAdd(&g[k], sg[k]);
  if (threadIdx.x == 0) {
    float tot = 0.f;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot += s_loss[w];
    atomicAdd(&h->loss, tot / (float)S);
  }
}

// --------------------------------------------------------- grad + Adam --
// One block: dL/dtheta_m = sigmoid(theta_m) (sum_{k>m} g_k - sum_k g_k y_k) / Z.
// With grad_out != nullptr the gradient is written out; with lr > 0 one Adam
// step (beta1 0.9, beta2 0.999, eps 1e-8) updates theta.
__global__ void __launch_bounds__(1024)
    lcdf_grad_kernel(char* blob, LcdfLayout L, float* grad_out, float lr) {
  __shared__ float warp_tot[32];
  __shared__ float total;
  __shared__ float red[32];
  LcdfHeader* h = reinterpret_cast<LcdfHeader*>(blob);
  const int K = h->n_knots;
  const float Z = h->z;
  float* theta = reinterpret_cast<float*>(blob + L.theta);
  float* m = reinterpret_cast<float*>(blob + L.adam_m);
  float* v = reinterpret_cast<float*>(blob + L.adam_v);
  const float* y = reinterpret_cast<const float*>(blob + L.y);
  const float* g = reinterpret_cast<const float*>(blob + L.g);
  // gy = sum_k g_k y_k
  float part = 0.f;
  for (int k = threadIdx.x; k <= K; k += 1024) part += g[k] * y[k];
  for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = part;
  __syncthreads();
  if (threadIdx.x < 32) {
    float t = red[threadIdx.x];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) red[0] = t;
  }
  __syncthreads();
  const float gy = red[0];
  // suffix sums over g_1..g_K in reversed blocked order: suf(m+1) = sum_{k>m} g_k
  constexpr int PER = (kLcdfMaxKnots + 1023) / 1024;
  float gv[PER];
  float sum = 0.f;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int r = threadIdx.x * PER + j;  // r-th from the end: k = K - r
    const int k = K - r;
    gv[j] = (r < K) ? g[k] : 0.f;        // k in [1, K]
    sum += gv[j];
  }
  float run = block_exclusive_sum<1024>(sum, warp_tot, &total);
  const int step = h->steps + 1;
  const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int r = threadIdx.x * PER + j;
    run += gv[j];  // now sum of g over k in [K - r, K]
    if (r < K) {
      const int mi = K - r - 1;  // theta index: suffix from k = mi + 1
      const float grad = sigmoidf_(theta[mi]) * (run - gy) / Z;
      if (grad_out) grad_out[mi] = grad;
      if (lr > 0.f) {
        const float mm = b1 * m[mi] + (1.f - b1) * grad;
        const float vv = b2 * v[mi] + (1.f - b2) * grad * grad;
        m[mi] = mm;
        v[mi] = vv;
        theta[mi] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
      }
    }
  }
  if (threadIdx.x == 0 && lr > 0.f) h->steps = step;
}

// ------------------------------------------------------ fixed-point tables --
// One block: Yq, slopes and the top-bits lookup table for NB buckets.
__global__ void __launch_bounds__(1024) lcdf_tables_kernel(char* blob, LcdfLayout L, int nb) {
  __shared__ uint32_t warp_tot[32];
  LcdfHeader* h = reinterpret_cast<LcdfHeader*>(blob);
  const int K = h->n_knots;
  const uint32_t* x = reinterpret_cast<const uint32_t*>(blob + L.x);
  const float* y = reinterpret_cast<const float*>(blob + L.y);
  uint32_t* yq = reinterpret_cast<uint32_t*>(blob + L.yq);
  unsigned long long* slope = reinterpret_cast<unsigned long long*>(blob + L.slope);
  uint16_t* lut = reinterpret_cast<uint16_t*>(blob + L.lut);
  const uint32_t top = (uint32_t)nb << kLcdfFix;
  // Yq_k = round(y_k * NB * 2^16), then a running max keeps it non-decreasing.
  constexpr int PER = (kLcdfMaxKnots + 1023) / 1024;
  uint32_t q[PER];
  uint32_t mx = 0;
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int k = threadIdx.x * PER + j;
    q[j] = 0;
    if (k <= K) {
      double t = (double)y[k] * (double)top;
      uint32_t u = (uint32_t)min((double)top, max(0.0, rint(t)));
      if (k == 0) u = 0;
      if (k == K) u = top;
      q[j] = u;
    }
    mx = max(mx, q[j]);
    q[j] = mx;  // running max within the thread's block
  }
  // exclusive max-scan across threads
  uint32_t inc = mx;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc = max(inc, t);
  }
  if (lane == 31) warp_tot[w] = inc;
  __syncthreads();
  if (w == 0) {
    uint32_t t = warp_tot[lane];
    uint32_t ti = t;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t u = __shfl_up_sync(0xffffffffu, ti, o);
      if (lane >= o) ti = max(ti, u);
    }
    warp_tot[lane] = ti;  // inclusive max of warps 0..lane
  }
  __syncthreads();
  uint32_t before = __shfl_up_sync(0xffffffffu, inc, 1);
  if (lane == 0) before = 0;
  if (w > 0) before = max(before, warp_tot[w - 1]);
#pragma unroll
  for (int j = 0; j < PER; ++j) {
    const int k = threadIdx.x * PER + j;
    if (k <= K) yq[k] = max(before, q[j]);
  }
  __syncthreads();
  for (int k = threadIdx.x; k < K; k += 1024) {
    const unsigned long long dy = (unsigned long long)(yq[k + 1] - yq[k]);
    slope[k] = (dy << 32) / (unsigned long long)(x[k + 1] - x[k]);
  }
  // lut[p] = number of knots x_k (k < K) with x_k <= p << 18, for p in [0, 4096].
  for (int p = threadIdx.x; p <= kLcdfLutSize; p += 1024) {
    const uint32_t v = (uint32_t)p << (30 - kLcdfLutBits);
    int lo = 0, hi = K;  // count of x[0..K) <= v
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (x[mid] <= v) lo = mid + 1;
      else hi = mid;
    }
    lut[p] = (uint16_t)lo;
  }
  if (threadIdx.x == 0) h->n_buckets = nb;
}

// Bucket boundaries of the fixed-point model, for the bucketed sort:
// bounds[b] = smallest key v with bucket(v) >= b (bounds[0] = 0; 2^30 when no
// key reaches b; bounds[nb] = 2^30), and blut[p] = bucket(p << 16) for the
// 2^14 cells of 2^16 keys (blut[2^14] = bucket(2^30 - 1)). Because bucket()
// never decreases, bucket(v) = the largest b with bounds[b] <= v, and that b
// lies in [blut[v >> 16], blut[(v >> 16) + 1]].
__global__ void __launch_bounds__(256) lcdf_bounds_kernel(char* blob, LcdfLayout L, int nb) {
  const LcdfTables t = lcdf_tables_global(blob, L);
  uint32_t* bounds = reinterpret_cast<uint32_t*>(blob + L.bounds);
  uint16_t* blut = reinterpret_cast<uint16_t*>(blob + L.blut);
  const int items = nb + 1 + kLcdfBlutSize + 1;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < items; it += gridDim.x * blockDim.x) {
    if (it <= nb) {
      const uint32_t b = (uint32_t)it;
      uint32_t v;
      if (b == 0) {
        v = 0;
      } else if (b == (uint32_t)nb || lcdf_bucket(t, kLcdfKeyEnd - 1u) < b) {
        v = kLcdfKeyEnd;
      } else {
        uint32_t lo = 0, hi = kLcdfKeyEnd - 1u;  // bucket(hi) >= b
        while (lo < hi) {
          const uint32_t mid = lo + ((hi - lo) >> 1);
          if (lcdf_bucket(t, mid) >= b) hi = mid;
          else lo = mid + 1;
        }
        v = lo;
      }
      bounds[b] = v;
    } else {
      const int p = it - (nb + 1);
      const uint32_t v = min((uint32_t)p << (30 - kLcdfBlutBits), kLcdfKeyEnd - 1u);
      blut[p] = (uint16_t)lcdf_bucket(t, v);
    }
  }
}

static void launch_lcdf_bounds(char* blob, const LcdfLayout& L, int nb, cudaStream_t s) {
  const int items = nb + 1 + kLcdfBlutSize + 1;
  lcdf_bounds_kernel<<<(items + 255) / 256, 256, 0, s>>>(blob, L, nb);
}

// ------------------------------------------------------------- inference --
__global__ void __launch_bounds__(256)
    lcdf_bucket_kernel(const char* __restrict__ blob, LcdfLayout L, const uint32_t* __restrict__ keys,
                       int n, uint32_t* __restrict__ out) {
  extern __shared__ __align__(16) unsigned char sm[];
  LcdfTables t = lcdf_load_tables(blob, L, sm);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = lcdf_bucket(t, keys[i]);
}

size_t lcdf_tables_smem(int max_knots) {
  return align_up(8 * (size_t)max_knots + 4 * (size_t)(max_knots + 1) * 2 +
                      2 * (kLcdfLutSize + 1),
                  16);
}

cudaError_t launch_lcdf_fit(const uint32_t* sorted_sample, int S, int k_req, int steps, float lr,
                            char* blob, const LcdfLayout& L, int nb, cudaStream_t s) {
  lcdf_knots_kernel<<<1, 1024, 0, s>>>(sorted_sample, S, k_req, blob, L);
  const size_t fb_smem = 12 * (size_t)(L.max_knots + 1);
  int grid = (S + 255) / 256;
  if (grid > device_sm_count() * 4) grid = device_sm_count() * 4;
  if (grid < 1) grid = 1;
  set_smem_limit(lcdf_fwd_bwd_kernel, 12 * (kLcdfMaxSegments + 1));
  for (int it = 0; it < steps; ++it) {
    lcdf_prep_kernel<<<1, 1024, 0, s>>>(blob, L);
    lcdf_fwd_bwd_kernel<<<grid, 256, fb_smem, s>>>(sorted_sample, S, blob, L);
    lcdf_grad_kernel<<<1, 1024, 0, s>>>(blob, L, nullptr, lr);
  }
  // final heights, loss of the trained model, tables
  lcdf_prep_kernel<<<1, 1024, 0, s>>>(blob, L);
  lcdf_fwd_bwd_kernel<<<grid, 256, fb_smem, s>>>(sorted_sample, S, blob, L);
  lcdf_tables_kernel<<<1, 1024, 0, s>>>(blob, L, nb);
  launch_lcdf_bounds(blob, L, nb, s);
  return cudaGetLastError();
}

cudaError_t launch_lcdf_train(const uint32_t* sorted_sample, int S, int steps, float lr, char* blob,
                              const LcdfLayout& L, cudaStream_t s) {
  const size_t fb_smem = 12 * (size_t)(L.max_knots + 1);
  set_smem_limit(lcdf_fwd_bwd_kernel, 12 * (kLcdfMaxSegments + 1));
  int grid = (S + 255) / 256;
  if (grid > device_sm_count() * 4) grid = device_sm_count() * 4;
  if (grid < 1) grid = 1;
  for (int it = 0; it < steps; ++it) {
    lcdf_prep_kernel<<<1, 1024, 0, s>>>(blob, L);
    lcdf_fwd_bwd_kernel<<<grid, 256, fb_smem, s>>>(sorted_sample, S, blob, L);
    lcdf_grad_kernel<<<1, 1024, 0, s>>>(blob, L, nullptr, lr);
  }
  return cudaGetLastError();
}

cudaError_t launch_lcdf_loss_grad(const uint32_t* sorted_sample, int S, char* blob,
                                  const LcdfLayout& L, float* grad_out, cudaStream_t s) {
  const size_t fb_smem = 12 * (size_t)(L.max_knots + 1);
  set_smem_limit(lcdf_fwd_bwd_kernel, 12 * (kLcdfMaxSegments + 1));
  int grid = (S + 255) / 256;
  if (grid > device_sm_count() * 4) grid = device_sm_count() * 4;
  if (grid < 1) grid = 1;
  lcdf_prep_kernel<<<1, 1024, 0, s>>>(blob, L);
  lcdf_fwd_bwd_kernel<<<grid, 256, fb_smem, s>>>(sorted_sample, S, blob, L);
  lcdf_grad_kernel<<<1, 1024, 0, s>>>(blob, L, grad_out, 0.f);
  return cudaGetLastError();
}

cudaError_t launch_lcdf_tables(char* blob, const LcdfLayout& L, int nb, cudaStream_t s) {
  lcdf_prep_kernel<<<1, 1024, 0, s>>>(blob, L);
  lcdf_tables_kernel<<<1, 1024, 0, s>>>(blob, L, nb);
  launch_lcdf_bounds(blob, L, nb, s);
  return cudaGetLastError();
}

cudaError_t launch_lcdf_buckets(const char* blob, const LcdfLayout& L, const uint32_t* keys, int n,
                                uint32_t* out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const size_t smem = lcdf_tables_smem(L.max_knots);
  set_smem_limit(lcdf_bucket_kernel, (int)lcdf_tables_smem(kLcdfMaxSegments));
  int grid = (n + 255) / 256;
  if (grid > device_sm_count() * 8) grid = device_sm_count() * 8;
  lcdf_bucket_kernel<<<grid, 256, smem, s>>>(blob, L, keys, n, out);
  return cudaGetLastError();
}

}  // namespace octgb

// ------------------------------------------------------------------ C ABI --
extern "C" {

OCT_API int oct_lcdf_layout(int max_segments, size_t offsets[12]) {
  using namespace octgb;
  if (max_segments < 1 || max_segments > kLcdfMaxSegments || !offsets) return OCT_ERR_INVALID_ARG;
  const LcdfLayout L = lcdf_layout(max_segments);
  const size_t v[12] = {L.x,   L.theta, L.adam_m, L.adam_v, L.y,    L.g,
                        L.yq,  L.slope, L.lut,    L.bounds, L.blut, L.bytes};
  for (int i = 0; i < 12; ++i) offsets[i] = v[i];
  return OCT_OK;
}

OCT_API size_t oct_lcdf_fit_workspace_bytes(int n_sample) {
  using namespace octgb;
  if (n_sample < 1) return 0;
  return align_up(sort_plan(n_sample, 30).bytes, 256) + 2 * align_up(4 * (size_t)n_sample, 256);
}

OCT_API int oct_lcdf_fit(const uint32_t* sample_keys, int n_sample, int n_segments, int steps,
                         float lr, int n_buckets, void* model, int max_segments, void* workspace,
                         size_t workspace_bytes, oct_stream_t stream) {
  using namespace octgb;
  if (!sample_keys || !model || !workspace || n_sample < 1 || n_sample > OCT_MAX_N ||
      n_segments < 1 || n_segments > max_segments || max_segments > kLcdfMaxSegments ||
      steps < 0 || n_buckets < 1 || n_buckets > kLcdfMaxBuckets || (reinterpret_cast<uintptr_t>(workspace) & 255))
    return OCT_ERR_INVALID_ARG;
  if (workspace_bytes < oct_lcdf_fit_workspace_bytes(n_sample)) return OCT_ERR_WORKSPACE;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  const SortPlan p = sort_plan(n_sample, 30);
  char* w = static_cast<char*>(workspace);
  uint32_t* keys = reinterpret_cast<uint32_t*>(w + align_up(p.bytes, 256));
  uint32_t* alt = keys + align_up(4 * (size_t)n_sample, 256) / 4;
  cudaError_t e = cudaMemcpyAsync(keys, sample_keys, 4 * (size_t)n_sample, cudaMemcpyDeviceToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(w, 0, p.zero_bytes, s);
  if (e == cudaSuccess) e = launch_histogram(keys, &p, w, s);
  uint32_t* sorted = keys;
  if (e == cudaSuccess) e = launch_sort_passes(keys, alt, &p, w, nullptr, s, &sorted);
  const LcdfLayout L = lcdf_layout(max_segments);
  if (e == cudaSuccess)
    e = launch_lcdf_fit(sorted, n_sample, n_segments, steps, lr, static_cast<char*>(model), L,
                        n_buckets, s);
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

OCT_API int oct_lcdf_loss_grad(const uint32_t* sorted_sample, int n_sample, void* model,
                               int max_segments, float* d_grad, oct_stream_t stream) {
  using namespace octgb;
  if (!sorted_sample || !model || n_sample < 1 || max_segments < 1 ||
      max_segments > kLcdfMaxSegments)
    return OCT_ERR_INVALID_ARG;
  const LcdfLayout L = lcdf_layout(max_segments);
  cudaError_t e = launch_lcdf_loss_grad(sorted_sample, n_sample, static_cast<char*>(model), L,
                                        d_grad, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

OCT_API int oct_lcdf_tables(void* model, int max_segments, int n_buckets, oct_stream_t stream) {
  using namespace octgb;
  if (!model || max_segments < 1 || max_segments > kLcdfMaxSegments || n_buckets < 1 ||
      n_buckets > kLcdfMaxBuckets)
    return OCT_ERR_INVALID_ARG;
  const LcdfLayout L = lcdf_layout(max_segments);
  cudaError_t e = launch_lcdf_tables(static_cast<char*>(model), L, n_buckets,
                                     reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

OCT_API int oct_lcdf_buckets(const void* model, int max_segments, const uint32_t* keys, int n,
                             uint32_t* d_buckets, oct_stream_t stream) {
  using namespace octgb;
  if (!model || n < 0 || max_segments < 1 || max_segments > kLcdfMaxSegments) return OCT_ERR_INVALID_ARG;
  if (n == 0) return OCT_OK;
  if (!keys || !d_buckets) return OCT_ERR_INVALID_ARG;
  const LcdfLayout L = lcdf_layout(max_segments);
  cudaError_t e = launch_lcdf_buckets(static_cast<const char*>(model), L, keys, n, d_buckets,
                                      reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

}  // extern "C"

extern "C" {

// `steps` further Adam steps on the model's current parameters (sorted sample).
OCT_API int oct_lcdf_train_steps(const uint32_t* sorted_sample, int n_sample, void* model,
                                 int max_segments, int steps, float lr, oct_stream_t stream) {
  using namespace octgb;
  if (!sorted_sample || !model || n_sample < 1 || steps < 0 || max_segments < 1 ||
      max_segments > kLcdfMaxSegments || !(lr > 0.f))
    return OCT_ERR_INVALID_ARG;
  const LcdfLayout L = lcdf_layout(max_segments);
  cudaError_t e = launch_lcdf_train(sorted_sample, n_sample, steps, lr, static_cast<char*>(model),
                                    L, reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) {
    set_last_error(cudaGetErrorString(e));
    return OCT_ERR_CUDA;
  }
  return OCT_OK;
}

}  // extern "C"
