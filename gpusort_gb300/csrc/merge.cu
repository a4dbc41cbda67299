// Merge-path merge of sorted runs: the HykSort shape of the reference on
// one GPU. HykSort sorts each rank's data locally, then per round exchanges
// buckets and merges the received runs pairwise (HykSortHelper::Merge,
// include/helpers/hyksort_helper.h:307-332, with OmpUtils::Merge,
// include/omp/omp_utils.h:54-145, splitting each merge across threads by
// sampled cross ranks). Here the p locally sorted partitions are merged by
// a tree of batched 2-way merges. Each level first finds the merge-path
// split of every output tile by binary search (so the work splits exactly,
// with no sampling), all tiles' searches in parallel; then each CTA stages
// its tile's two sub-runs in shared memory and each thread merges its own
// sub-path. Ties take the left run first (std::merge order).
#include <cstdint>

#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int MERGE_THREADS = 256;
// Outputs per thread: a tile is 16 KB of keys in shared memory either way.
template <typename K> struct MergeItems {
  static constexpr int value = sizeof(K) == 4 ? 16 : 8;
  static constexpr uint32_t tile = uint32_t(MERGE_THREADS) * value;
};

struct MergeParams {
  const void* in;
  void* out;
  uint64_t n;
  uint64_t run;            // input run length (the last run may be shorter)
  uint64_t tiles_per_pair;
  uint32_t key_kind, desc;
  uint64_t* splits;        // per pair: tiles_per_pair + 1 merge-path splits
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

// The two runs merged by `pair`: A = [a0, a0 + la), B = [a0 + la, + lb).
__device__ __forceinline__ void pair_runs(const MergeParams& p, uint64_t pair, uint64_t* a0,
                                          uint64_t* la, uint64_t* lb) {
  *a0 = pair * 2 * p.run;
  *la = min(p.run, p.n - *a0);
  *lb = min(p.run, p.n - (*a0 + *la));
}

// Merge-path split of every tile boundary (tile t of a pair starts at
// output t * TILE), one thread each: the binary searches over global memory
// run side by side instead of one at the head of each merge CTA.
template <typename K>
__global__ void __launch_bounds__(256) merge_split_kernel(MergeParams p, uint64_t count) {
  const uint64_t g = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (g >= count) return;
  const uint64_t pair = g / (p.tiles_per_pair + 1);
  const uint64_t t = g % (p.tiles_per_pair + 1);
  uint64_t a0, la, lb;
  pair_runs(p, pair, &a0, &la, &lb);
  const uint64_t d = min(t * MergeItems<K>::tile, la + lb);
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* in = static_cast<const K*>(p.in);
  auto ga = [&](uint64_t i) { return kx.fwd(in[a0 + i]); };
  auto gb = [&](uint64_t i) { return kx.fwd(in[a0 + la + i]); };
  p.splits[g] = merge_path<K>(d, la, lb, ga, gb, [](K x, K y) { return x < y; });
}

// Shared-memory slot of tile element i: one pad element after every 128
// bytes. Threads read and write ITEMS-strided runs (thread t near element
// t * ITEMS); unpadded, a warp's accesses fall in a few banks (16-way
// conflicts for 32-bit keys), padded they spread over all of them.
template <typename K> struct Pad {
  static constexpr uint32_t SHIFT = sizeof(K) == 4 ? 5 : 4;
  __device__ __forceinline__ static uint32_t at(uint32_t i) { return i + (i >> SHIFT); }
};

// One tile of a pair's merge: its parts of A and B are staged in shared
// memory (coalesced), each thread finds its own split there and merges
// ITEMS outputs in registers, and the tile is written back coalesced.
template <typename K>
__global__ void __launch_bounds__(MERGE_THREADS) merge_pass_kernel(MergeParams p) {
  constexpr int ITEMS = MergeItems<K>::value;
  constexpr uint32_t TILE = MergeItems<K>::tile;
  __shared__ K s[TILE + (TILE >> Pad<K>::SHIFT)];
  auto pad = [](uint32_t i) { return Pad<K>::at(i); };
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* in = static_cast<const K*>(p.in);
  K* out = static_cast<K*>(p.out);
  const uint64_t pair = blockIdx.x / p.tiles_per_pair;
  const uint64_t t = blockIdx.x % p.tiles_per_pair;
  uint64_t a0, la, lb;
  pair_runs(p, pair, &a0, &la, &lb);
  const uint64_t total = la + lb;
  const uint64_t d0 = t * TILE;
  if (d0 >= total) return;
  const uint64_t d1 = min(d0 + TILE, total);
  const uint64_t* sp = p.splits + pair * (p.tiles_per_pair + 1) + t;
  const uint64_t ia0 = sp[0], ia1 = sp[1];
  const uint64_t ib0 = d0 - ia0;
  const uint32_t na = uint32_t(ia1 - ia0), cnt = uint32_t(d1 - d0), nb = cnt - na;
  const K* pa = in + a0 + ia0;
  const K* pb = in + a0 + la + ib0;
  const int tid = threadIdx.x;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t i = uint32_t(tid + k * MERGE_THREADS);
    if (i < cnt) s[pad(i)] = kx.fwd(i < na ? pa[i] : pb[i - na]);
  }
  __syncthreads();
  const uint32_t my0 = uint32_t(tid) * ITEMS;
  K r[ITEMS];
  if (my0 < cnt) {
    auto sa = [&](uint64_t i) { return s[pad(uint32_t(i))]; };
    auto sb = [&](uint64_t i) { return s[pad(na + uint32_t(i))]; };
    uint32_t i = uint32_t(merge_path<K>(my0, na, nb, sa, sb, [](K x, K y) { return x < y; }));
    uint32_t j = my0 - i;
    K x = i < na ? s[pad(i)] : K(0);
    K y = j < nb ? s[pad(na + j)] : K(0);
#pragma unroll
    for (int k = 0; k < ITEMS; ++k) {
      const bool take_a = j >= nb || (i < na && !(y < x));
      r[k] = take_a ? x : y;
      if (take_a) {
        ++i;
        if (i < na) x = s[pad(i)];
      } else {
        ++j;
        if (j < nb) y = s[pad(na + j)];
      }
    }
  }
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ITEMS; ++k)
    if (my0 + k < cnt) s[pad(my0 + k)] = r[k];
  __syncthreads();
  K* po = out + a0 + d0;
#pragma unroll
  for (int k = 0; k < ITEMS; ++k) {
    const uint32_t i = uint32_t(tid + k * MERGE_THREADS);
    if (i < cnt) po[i] = kx.inv(s[pad(i)]);
  }
}

template <typename K>
cudaError_t merge_pass_t(const void* in, void* out, uint64_t n, uint64_t run, uint32_t key_kind,
                         bool desc, uint64_t* splits, cudaStream_t st) {
  constexpr uint32_t TILE = MergeItems<K>::tile;
  const uint64_t pairs = (n + 2 * run - 1) / (2 * run);
  const uint64_t tpp = (2 * run + TILE - 1) / TILE;
  const uint64_t blocks = pairs * tpp;
  if (blocks > 0x7FFFFFFFull) return cudaErrorInvalidValue;
  MergeParams p{in, out, n, run, tpp, key_kind, uint32_t(desc), splits};
  const uint64_t count = pairs * (tpp + 1);
  merge_split_kernel<K><<<unsigned((count + 255) / 256), 256, 0, st>>>(p, count);
  merge_pass_kernel<K><<<unsigned(blocks), MERGE_THREADS, 0, st>>>(p);
  return cudaGetLastError();
}

}  // namespace

size_t merge_split_words(uint64_t n, uint64_t run, int key_bytes) {
  if (run == 0) return 0;
  const uint64_t tile = key_bytes == 4 ? MergeItems<uint32_t>::tile : MergeItems<uint64_t>::tile;
  const uint64_t pairs = (n + 2 * run - 1) / (2 * run);
  return size_t(pairs * ((2 * run + tile - 1) / tile + 1));
}

cudaError_t launch_merge_pass(const void* in, void* out, uint64_t n, uint64_t run, int key_bytes,
                              uint32_t key_kind, bool desc, uint64_t* splits, cudaStream_t st) {
  if (run == 0 || run >= n || splits == nullptr) return cudaErrorInvalidValue;
  if (key_bytes == 4) return merge_pass_t<uint32_t>(in, out, n, run, key_kind, desc, splits, st);
  return merge_pass_t<uint64_t>(in, out, n, run, key_kind, desc, splits, st);
}

}  // namespace gs
