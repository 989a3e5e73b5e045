// Comparison bar for the sort stage: CUB's DeviceRadixSort::SortKeys on the
// same keys (the library sort the reference benchmarks against,
// benchmarks/cuda/bm_02_sort.cuh:117-140). Built by cub_bar/build.py into its
// own library, used only by bench.py; no product path links it.
#include <cub/device/device_radix_sort.cuh>
#include <cuda_runtime.h>
#include <stdint.h>

extern "C" {

__attribute__((visibility("default"))) int bar_cub_sort_keys(const uint32_t* keys_in,
                                                             uint32_t* keys_out, int n,
                                                             int end_bit, void* temp,
                                                             size_t* temp_bytes, void* stream) {
  const cudaError_t e = cub::DeviceRadixSort::SortKeys(
      temp, *temp_bytes, keys_in, keys_out, n, 0, end_bit, reinterpret_cast<cudaStream_t>(stream));
  return e == cudaSuccess ? 0 : (int)e;
}

}  // extern "C"
