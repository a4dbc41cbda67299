// Sample-sort bucketing: the SampleSort shape of the reference
// (include/helpers/samplesort_helper.h:390-565) on one GPU. The p ranks'
// regular samples, bitonic sort of the samples and Allgather of the
// splitters (SelectSplitters, :390-417) become one CTA that sorts an
// oversampled sample in shared memory and keeps p-1 splitters; the
// upper_bound bucketing and Alltoallv exchange (TransferData, :504-565)
// become a bucket histogram and one onesweep scatter pass whose digit is
// the key's bucket. Each bucket is then sorted by the batched sort, as the
// reference re-sorts each rank's received data (:486).
#include <cstddef>
#include <cstdint>

#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int SAMPLE_THREADS = 1024;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // SplitMix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct SampleParams {
  const void* keys;
  uint64_t n;
  uint32_t key_kind, desc;
  uint32_t parts;      // p
  uint32_t samples;    // p * oversample
  uint32_t padded;     // next power of two >= samples
  uint64_t seed;
  void* splitters;     // p - 1 order-bit splitters out
};

// One CTA: draw `samples` keys at seeded positions, bitonic-sort their order
// bits in shared memory, keep every (samples/p)-th as a splitter.
template <typename K>
__global__ void __launch_bounds__(SAMPLE_THREADS) sample_kernel(SampleParams p) {
  extern __shared__ __align__(16) uint8_t s_dyn[];
  K* s = reinterpret_cast<K*>(s_dyn);
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* keys = static_cast<const K*>(p.keys);
  for (uint32_t i = threadIdx.x; i < p.padded; i += blockDim.x) {
    if (i < p.samples) {
      const uint64_t pos = mix64(p.seed ^ (uint64_t(i) * 0xD6E8FEB86659FD93ull)) % p.n;
      s[i] = kx.fwd(keys[pos]);
    } else {
      s[i] = ~K(0);
    }
  }
  __syncthreads();
  for (uint32_t size = 2; size <= p.padded; size <<= 1) {
    for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
      for (uint32_t i = threadIdx.x; i < p.padded / 2; i += blockDim.x) {
        const uint32_t lo = 2 * stride * (i / stride) + (i % stride);
        const uint32_t hi = lo + stride;
        const bool up = (lo & size) == 0;
        const K a = s[lo], b = s[hi];
        if ((a > b) == up) {
          s[lo] = b;
          s[hi] = a;
        }
      }
      __syncthreads();
    }
  }
  K* out = static_cast<K*>(p.splitters);
  for (uint32_t j = threadIdx.x; j + 1 < p.parts; j += blockDim.x)
    out[j] = s[(uint64_t(j + 1) * p.samples) / p.parts];
}

struct BucketHistParams {
  const void* keys;
  uint64_t n;
  uint32_t key_kind, desc;
  const void* splitters;
  uint32_t nsplit;
  uint32_t* hist;  // RADIX counters (digit row 0 of the work area)
};

constexpr int HIST_THREADS = 512;
constexpr int HIST_UNROLL = 8;  // keys per thread per step: loads in flight

template <typename K>
__global__ void __launch_bounds__(HIST_THREADS) bucket_hist_kernel(BucketHistParams p) {
  __shared__ K s_tree[RADIX];
  __shared__ uint32_t s_h[RADIX];
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const uint32_t levels = tree_levels(p.nsplit);
  for (uint32_t i = threadIdx.x; i < RADIX; i += blockDim.x) s_h[i] = 0;
  build_split_tree(static_cast<const K*>(p.splitters), p.nsplit, s_tree, levels);
  __syncthreads();
  const K* keys = static_cast<const K*>(p.keys);
  constexpr uint64_t CHUNK = uint64_t(HIST_THREADS) * HIST_UNROLL;
  for (uint64_t base = uint64_t(blockIdx.x) * CHUNK; base < p.n; base += uint64_t(gridDim.x) * CHUNK) {
    K y[HIST_UNROLL];
#pragma unroll
    for (int u = 0; u < HIST_UNROLL; ++u) {
      const uint64_t i = base + uint64_t(u) * HIST_THREADS + threadIdx.x;
      y[u] = i < p.n ? kx.fwd(keys[i]) : K(0);
    }
#pragma unroll
    for (int u = 0; u < HIST_UNROLL; ++u) {
      const uint64_t i = base + uint64_t(u) * HIST_THREADS + threadIdx.x;
      if (i < p.n) atomicAdd(&s_h[tree_bucket(s_tree, levels, p.nsplit, y[u])], 1u);
    }
  }
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < RADIX; i += blockDim.x)
    if (s_h[i]) atomicAdd(&p.hist[i], s_h[i]);
}

template <typename K>
cudaError_t bucketing_t(const RadixJob& job, const SampleJob& sj, const DeviceProps& props,
                        cudaStream_t st) {
  cudaError_t e = cudaMemsetAsync(job.work, 0, offsetof(SortWork, plan), st);
  if (e != cudaSuccess) return e;
  uint32_t padded = 1;
  while (padded < sj.samples) padded <<= 1;
  SampleParams sp{job.keys_in, job.n, job.key_kind, uint32_t(job.desc), sj.parts, sj.samples,
                  padded, sj.seed, sj.splitters};
  const size_t dyn = size_t(padded) * sizeof(K);
  e = cudaFuncSetAttribute(sample_kernel<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(dyn));
  if (e != cudaSuccess) return e;
  sample_kernel<K><<<1, SAMPLE_THREADS, dyn, st>>>(sp);
  BucketHistParams hp{job.keys_in, job.n, job.key_kind, uint32_t(job.desc), sj.splitters,
                      sj.parts - 1, &job.work->hist[0][0]};
  uint64_t blocks = (job.n + HIST_THREADS * HIST_UNROLL - 1) / (HIST_THREADS * HIST_UNROLL);
  const uint64_t cap = uint64_t(props.num_sms) * 4;
  if (blocks > cap) blocks = cap;
  bucket_hist_kernel<K><<<unsigned(blocks), HIST_THREADS, 0, st>>>(hp);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  return launch_bucket_pass(job, sj.splitters, sj.parts - 1, props, st);
}

}  // namespace

cudaError_t launch_sample_bucketing(const RadixJob& job, const SampleJob& sj,
                                    const DeviceProps& props, cudaStream_t st) {
  if (sj.parts < 2 || sj.parts > RADIX || sj.samples < sj.parts || sj.samples > 8192)
    return cudaErrorInvalidValue;
  if (job.key_bytes == 4) return bucketing_t<uint32_t>(job, sj, props, st);
  return bucketing_t<uint64_t>(job, sj, props, st);
}

}  // namespace gs
