// Allocation-free sort entry point: oct_sort_keys_noalloc.
//
// Some callers cannot call cudaMalloc: a host whose device memory is owned by
// another allocator (a framework's caching allocator, or a fixed pool reserved
// at start-up that leaves nothing to allocate from), or a frame loop that must
// not stall, where cudaMalloc would synchronise the device. Such a caller
// cannot size and allocate the workspace oct_sort_keys asks for. This variant
// takes the same inputs and outputs (keys and the n-entry keys_alt buffer, as
// the reference's k_SimpleRadixSort(keys, keys_alt, n) does) and keeps its
// scratch (digit histograms, tile counters, look-back flags) in a file-scope
// __device__ array of fixed size instead.
//
//  - Limit: n <= OCT_NOALLOC_SORT_MAX_KEYS (4,194,304 keys); larger n returns
//    OCT_ERR_TOO_LARGE without launching anything.
//  - Memory: the array (OCT_NOALLOC_SORT_SCRATCH_BYTES, 6.5 MiB) is part of
//    the library's device image, so every GPU that loads the library holds it
//    until the process exits.
//  - Set-up: the first call on a device resolves the array's device address
//    with cudaGetSymbolAddress while that device is current; make that first
//    call before any stream capture on the device. The address is kept for
//    the life of the process: cudaDeviceReset on a device after its first
//    call is not supported (the array would be reloaded at another address).
//    Each device of a process has its own array and address.
//  - Sharing: every call uses the same array and clears the part it needs at
//    the start of the call. Calls that overlap on the GPU (on different
//    streams, or from different host threads without ordering) race on it.
//  - No call here allocates or frees device memory.
#include <stdio.h>

#include <mutex>

#include "kernels.cuh"

namespace {

constexpr int kMaxKeys = OCT_NOALLOC_SORT_MAX_KEYS;
constexpr size_t kScratchBytes = OCT_NOALLOC_SORT_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

// The scratch itself. In host code `g_sort_scratch` names a host-side shadow,
// not device memory: only the address from cudaGetSymbolAddress may be passed
// to a kernel.
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

std::mutex g_mu;
void* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_sort_scratch for the current device (set up once).
cudaError_t scratch_for_current_device(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return cudaSuccess;
}

int fail(int code, const char* msg) {
  octgb::set_last_error(msg);
  return code;
}

}  // namespace

extern "C" {

OCT_API int oct_sort_keys_noalloc(uint32_t* keys, uint32_t* keys_alt, int n, int key_bits,
                                  uint32_t* d_status, oct_stream_t stream) {
  using namespace octgb;
  if (n < 0 || key_bits < 1 || key_bits > 32) return OCT_ERR_INVALID_ARG;
  if (n > kMaxKeys)
    return fail(OCT_ERR_TOO_LARGE,
                "oct_sort_keys_noalloc: n exceeds the static scratch limit of 4194304 keys");
  if (n <= 1) return OCT_OK;
  if (!keys || !keys_alt) return OCT_ERR_INVALID_ARG;
  const SortPlan p = sort_plan(n, key_bits);
  if (p.bytes > kScratchBytes)
    return fail(OCT_ERR_TOO_LARGE, "oct_sort_keys_noalloc: scratch plan exceeds the static array");
  void* scratch = nullptr;
  cudaError_t e = scratch_for_current_device(&scratch);
  if (e != cudaSuccess) {
    char msg[192];
    snprintf(msg, sizeof(msg), "oct_sort_keys_noalloc: cudaGetSymbolAddress: %s",
             cudaGetErrorString(e));
    return fail(OCT_ERR_CUDA, msg);
  }
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  // The array keeps the previous call's counters and flags: clear them.
  e = cudaMemsetAsync(scratch, 0, p.zero_bytes, s);
  if (e == cudaSuccess) e = launch_histogram(keys, &p, scratch, s);
  uint32_t* result = keys;
  if (e == cudaSuccess) e = launch_sort_passes(keys, keys_alt, &p, scratch, d_status, s, &result);
  if (e == cudaSuccess && result != keys)
    e = cudaMemcpyAsync(keys, result, sizeof(uint32_t) * (size_t)n, cudaMemcpyDeviceToDevice, s);
  if (e != cudaSuccess) {
    char msg[192];
    snprintf(msg, sizeof(msg), "oct_sort_keys_noalloc: %s", cudaGetErrorString(e));
    return fail(OCT_ERR_CUDA, msg);
  }
  return OCT_OK;
}

}  // extern "C"
