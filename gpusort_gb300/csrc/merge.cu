// Merge-path merge of sorted runs: the HykSort shape of the reference on
// one GPU. HykSort sorts each rank's data locally, then per round exchanges
// buckets and merges the received runs pairwise (HykSortHelper::Merge,
// include/helpers/hyksort_helper.h:307-332, with OmpUtils::Merge,
// include/omp/omp_utils.h:54-145, splitting each merge across threads by
// sampled cross ranks). Here the p locally sorted partitions are merged by
// a tree of batched 2-way merges; each CTA finds its part of the merge path
// by binary search (so the work splits exactly, with no sampling), stages
// its two sub-runs in shared memory, and each thread merges its own
// sub-path. Ties take the left run first (std::merge order).
#include <cstdint>

#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int MERGE_THREADS = 256;
constexpr int MERGE_ITEMS = 8;
constexpr uint32_t MERGE_TILE = MERGE_THREADS * MERGE_ITEMS;  // outputs per CTA

struct MergeParams {
  const void* in;
  void* out;
  uint64_t n;
  uint64_t run;            // input run length (the last run may be shorter)
  uint64_t tiles_per_pair;
  uint32_t key_kind, desc;
};

// Number of elements taken from A among the first d outputs of merging A
// and B (A first on ties). `less(x, y)`: x orders before y.
template <typename K, typename GetA, typename GetB, typename Less>
__device__ __forceinline__ uint64_t merge_path(uint64_t d, uint64_t la, uint64_t lb, GetA a, GetB b,
                                               Less less) {
  uint64_t lo = d > lb ? d - lb : 0;
  uint64_t hi = d < la ? d : la;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (less(b(d - mid - 1), a(mid))) hi = mid; else lo = mid + 1;
  }
  return lo;
}

template <typename K>
__global__ void __launch_bounds__(MERGE_THREADS) merge_pass_kernel(MergeParams p) {
  __shared__ K s_in[MERGE_TILE];
  __shared__ K s_out[MERGE_TILE];
  __shared__ uint64_t s_split[2];
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* in = static_cast<const K*>(p.in);
  K* out = static_cast<K*>(p.out);
  const uint64_t pair = blockIdx.x / p.tiles_per_pair;
  const uint64_t t = blockIdx.x % p.tiles_per_pair;
  const uint64_t base = pair * 2 * p.run;
  if (base >= p.n) return;
  const uint64_t a0 = base, la = min(p.run, p.n - a0);
  const uint64_t b0 = a0 + la, lb = min(p.run, p.n - b0);
  const uint64_t total = la + lb;
  const uint64_t d0 = t * MERGE_TILE;
  if (d0 >= total) return;
  const uint64_t d1 = min(d0 + MERGE_TILE, total);
  auto ga = [&](uint64_t i) { return kx.fwd(in[a0 + i]); };
  auto gb = [&](uint64_t i) { return kx.fwd(in[b0 + i]); };
  auto less = [](K x, K y) { return x < y; };
  if (threadIdx.x < 2) {
    const uint64_t d = threadIdx.x == 0 ? d0 : d1;
    s_split[threadIdx.x] = merge_path<K>(d, la, lb, ga, gb, less);
  }
  __syncthreads();
  const uint64_t ia0 = s_split[0], ia1 = s_split[1];
  const uint64_t ib0 = d0 - ia0, ib1 = d1 - ia1;
  const uint32_t na = uint32_t(ia1 - ia0), nb = uint32_t(ib1 - ib0);
  // Stage A's part then B's part (order bits).
  for (uint32_t i = threadIdx.x; i < na + nb; i += MERGE_THREADS)
    s_in[i] = i < na ? kx.fwd(in[a0 + ia0 + i]) : kx.fwd(in[b0 + ib0 + (i - na)]);
  __syncthreads();
  // Each thread merges MERGE_ITEMS outputs from its own split point.
  const uint32_t cnt = na + nb;
  const uint32_t my0 = threadIdx.x * MERGE_ITEMS;
  if (my0 < cnt) {
    auto sa = [&](uint64_t i) { return s_in[i]; };
    auto sb = [&](uint64_t i) { return s_in[na + i]; };
    uint32_t i = uint32_t(merge_path<K>(my0, na, nb, sa, sb, less));
    uint32_t j = my0 - i;
    const uint32_t my1 = min(my0 + MERGE_ITEMS, cnt);
    for (uint32_t k = my0; k < my1; ++k) {
      const bool take_a = j >= nb || (i < na && !(s_in[na + j] < s_in[i]));
      s_out[k] = take_a ? s_in[i++] : s_in[na + j++];
    }
  }
  __syncthreads();
  for (uint32_t k = threadIdx.x; k < cnt; k += MERGE_THREADS) out[base + d0 + k] = kx.inv(s_out[k]);
}

}  // namespace

cudaError_t launch_merge_pass(const void* in, void* out, uint64_t n, uint64_t run, int key_bytes,
                              uint32_t key_kind, bool desc, cudaStream_t st) {
  if (run == 0 || run >= n) return cudaErrorInvalidValue;
  const uint64_t pairs = (n + 2 * run - 1) / (2 * run);
  const uint64_t tpp = (2 * run + MERGE_TILE - 1) / MERGE_TILE;
  const uint64_t blocks = pairs * tpp;
  if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  MergeParams p{in, out, n, run, tpp, key_kind, uint32_t(desc)};
  if (key_bytes == 4) merge_pass_kernel<uint32_t><<<unsigned(blocks), MERGE_THREADS, 0, st>>>(p);
  else merge_pass_kernel<uint64_t><<<unsigned(blocks), MERGE_THREADS, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace gs
