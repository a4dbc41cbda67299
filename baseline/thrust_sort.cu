// Comparison-only build of the reference's GPU local sort, for bench.py's
// "reference GPU sort" line. It is never linked into the engine library and
// nothing on the engine's path calls it.
//
// The reference sorts each chunk with thrust::sort over a
// thrust::device_vector under thrust::less<T> (src/cuda_utils.cu:403-445,
// the call at :424), which Thrust dispatches to CUB's device radix sort. Two
// entry points time that on device-resident data:
//   ref_thrust_sort_u32 - thrust::sort in place, as the reference calls it
//                         (Thrust allocates its temporary storage per call);
//   ref_cub_sort_u32    - cub::DeviceRadixSort::SortKeys with caller-owned
//                         temporary storage: the same kernels without the
//                         per-call allocation.
#include <cstddef>
#include <cstdint>

#include <cub/device/device_radix_sort.cuh>
#include <thrust/execution_policy.h>
#include <thrust/functional.h>
#include <thrust/sort.h>

extern "C" {

int ref_thrust_sort_u32(uint32_t* keys, uint64_t n, cudaStream_t stream) {
  try {
    thrust::sort(thrust::cuda::par.on(stream), keys, keys + n, thrust::less<uint32_t>());
  } catch (...) {
    return -1;
  }
  return int(cudaGetLastError());
}

size_t ref_cub_temp_bytes_u32(uint64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortKeys(nullptr, bytes, static_cast<const uint32_t*>(nullptr),
                                 static_cast<uint32_t*>(nullptr), int64_t(n));
  return bytes;
}

int ref_cub_sort_u32(const uint32_t* in, uint32_t* out, uint64_t n, void* temp,
                     size_t temp_bytes, cudaStream_t stream) {
  size_t bytes = temp_bytes;
  return int(cub::DeviceRadixSort::SortKeys(temp, bytes, in, out, int64_t(n), 0, 32, stream));
}

}  // extern "C"
