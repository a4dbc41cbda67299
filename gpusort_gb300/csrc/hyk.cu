// The HykSort shape on one GPU: the reference's p MPI ranks are p runs of
// one array in HBM. After the local sorts, each round of the reference's
// SortAmongProcesses (include/helpers/hyksort_helper.h:453-536) runs as
// three device steps over all groups of ranks at once:
//
//  1. SelectSplitters (:335-450): one CTA per group of n_p ranks chooses
//     k-1 splitters by the reference's iteration - random samples drawn
//     inside each splitter's current interval of every rank (beta =
//     3 * (1/tol)^(1/3) of them, tol = 0.01 / (k-1); with more ranks than
//     beta, each rank contributes one sample with probability beta *
//     local / total), the samples sorted, their global ranks summed over
//     the group's ranks by lower_bound, the sample nearest below each
//     expected rank (i+1) * N / k kept and the intervals narrowed, until
//     the largest rank error is at most N * tol.
//  2. TransferData (:546-633): every rank's sorted run is cut at the
//     splitters by lower_bound (:563-568). Rank (block b, position q) of a
//     group receives piece b of the k ranks i * n_p/k + q. In HBM the
//     exchange moves nothing: the pieces are ranges of the source buffer.
//  3. Merge (:307-332): the k pieces of every receiving rank are merged in
//     one pass (the reference merges them pairwise in a binary tree). The
//     output of a rank is split into tiles at regular samples of its pieces
//     (every S-th element of each piece, S = C / k) under the total order
//     (value, piece, index): a tile then holds at most S elements of each
//     piece, so at most C, whatever the duplicates. Each sample's cut in
//     every piece comes from binary searches; each CTA merges one tile in
//     shared memory, every element finding its output position from its
//     index and its count of earlier elements in the other pieces.
//
// The rounds repeat on groups of n_p / k ranks until every group is one
// rank; the ranks' runs then lie in rank order in the output, which is the
// globally sorted array - the reference's concatenated result.
#include <cstddef>
#include <cstdint>
#include <cmath>

#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int SELECT_THREADS = 1024;
constexpr int MERGE_THREADS = 512;
constexpr uint32_t MAX_SAMPLES = 4096;  // samples of one selection round
constexpr uint32_t MAX_ITERS = 64;

__device__ __forceinline__ uint64_t hmix(uint64_t x) {  // SplitMix64 finaliser
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// First index of a[0, n) whose order bits are >= y (lower_bound under the
// sort's comparator), or > y when `upper` (upper_bound).
template <typename K>
__device__ __forceinline__ uint64_t bound(const K* a, uint64_t n, K y, const OrderXform<K>& kx,
                                          bool upper) {
  uint64_t lo = 0, hi = n;
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    const K v = kx.fwd(a[mid]);
    if (v < y || (upper && v == y)) lo = mid + 1; else hi = mid;
  }
  return lo;
}

struct SelectParams {
  const void* data;        // current buffer: rank r's sorted run is [roff[r], roff[r+1])
  const uint64_t* roff;
  uint32_t n_p;            // ranks per group
  uint32_t kway;           // k of this round (kway - 1 splitters)
  uint32_t key_kind, desc;
  uint64_t seed;
  void* splitters;         // out: per group, kway - 1 order-bit splitters
  uint32_t* iters;         // out: iterations per group
};

template <typename K>
size_t select_smem(uint32_t n_p, uint32_t kway) {
  const size_t kw = kway - 1;
  return size_t(n_p) * 8 + 2 * kw * n_p * 8 + size_t(MAX_SAMPLES) * (sizeof(K) + 8);
}

// Step 1: one CTA per group of ranks.
template <typename K>
__global__ void __launch_bounds__(SELECT_THREADS) hyk_select_kernel(SelectParams p) {
  extern __shared__ __align__(16) uint8_t s_dyn[];
  const uint32_t np = p.n_p;
  const uint32_t kw = p.kway - 1;  // splitters
  const uint32_t r0 = blockIdx.x * np;
  int64_t* s_len = reinterpret_cast<int64_t*>(s_dyn);
  int64_t* s_start = s_len + np;        // [kw][np]
  int64_t* s_end = s_start + kw * np;   // [kw][np]
  unsigned long long* s_grank = reinterpret_cast<unsigned long long*>(s_end + kw * np);
  K* s_samp = reinterpret_cast<K*>(s_grank + MAX_SAMPLES);
  __shared__ int64_t s_exp[MAX_KWAY], s_totsz[MAX_KWAY];
  __shared__ K s_split[MAX_KWAY];
  __shared__ int s_lb[MAX_KWAY], s_ub[MAX_KWAY], s_upd[MAX_KWAY];
  __shared__ unsigned long long s_tot;
  __shared__ unsigned int s_cnt;
  __shared__ long long s_maxerr, s_newmax;
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* data = static_cast<const K*>(p.data);
  const int tid = threadIdx.x;

  if (tid == 0) s_tot = 0;
  __syncthreads();
  for (uint32_t r = tid; r < np; r += blockDim.x) {
    s_len[r] = int64_t(p.roff[r0 + r + 1] - p.roff[r0 + r]);
    atomicAdd(&s_tot, (unsigned long long)s_len[r]);
  }
  __syncthreads();
  const int64_t tot = int64_t(s_tot);
  // tol and beta as the reference computes them (int truncation included).
  const double tol = 1e-2 / double(kw);
  const int beta = int(pow(1.0 / tol, 1.0 / 3.0) * 3.0);
  const int64_t cond = int64_t(double(tot) * tol);
  for (uint32_t t = tid; t < kw * np; t += blockDim.x) {
    s_start[t] = 0;
    s_end[t] = s_len[t % np];
  }
  if (tid < int(kw)) {
    s_exp[tid] = (int64_t(tid + 1) * tot) / int64_t(p.kway);
    s_split[tid] = K(0);
  }
  if (tid == 0) s_maxerr = tot;
  __syncthreads();
  uint32_t it = 0;
  while (tot > 0 && s_maxerr > cond && it < MAX_ITERS) {
    // Interval sizes per splitter, summed over the group's ranks.
    if (tid < int(kw)) {
      int64_t sz = 0;
      for (uint32_t r = 0; r < np; ++r) sz += s_end[tid * np + r] - s_start[tid * np + r];
      s_totsz[tid] = sz;
    }
    if (tid == 0) {
      s_cnt = 0;
      s_newmax = 0;
    }
    __syncthreads();
    // Samples: per splitter and rank, inside the rank's current interval.
    for (uint32_t t = tid; t < kw * np; t += blockDim.x) {
      const uint32_t i = t / np, r = t % np;
      const int64_t loc = s_end[t] - s_start[t];
      const int64_t tsz = s_totsz[i];
      const uint64_t h = p.seed ^ (uint64_t(blockIdx.x) << 40) ^ (uint64_t(it) << 24) ^
                         (uint64_t(t) * 0x9E3779B97F4A7C15ull);
      int take = tsz == 0 ? 1 : int(int64_t(beta) * loc / tsz);
      if (int(np) > beta) {
        const double u = double(hmix(h ^ 0xA5A5A5A5ull) >> 11) * (1.0 / 9007199254740992.0);
        take = (u * double(tsz) < double(beta) * double(loc)) ? 1 : 0;
      }
      if (loc <= 0) take = 0;  // nothing to draw from (the reference would read past the run)
      if (take <= 0) continue;
      const unsigned base = atomicAdd(&s_cnt, unsigned(take));
      const K* run = data + p.roff[r0 + r];
      for (int j = 0; j < take && base + j < MAX_SAMPLES; ++j) {
        const int64_t idx = s_start[t] + int64_t(hmix(h + uint64_t(j) + 1) % uint64_t(loc));
        s_samp[base + j] = kx.fwd(run[idx]);
      }
    }
    __syncthreads();
    const uint32_t cnt = s_cnt < MAX_SAMPLES ? s_cnt : MAX_SAMPLES;
    if (cnt == 0) {  // no sample drawn this time: draw again
      ++it;
      __syncthreads();
      continue;
    }
    // Sort the samples (bitonic over the next power of two, padded with the
    // largest key) and clear their global ranks.
    uint32_t padded = 1;
    while (padded < cnt) padded <<= 1;
    for (uint32_t i = cnt + tid; i < padded; i += blockDim.x) s_samp[i] = ~K(0);
    for (uint32_t i = tid; i < padded; i += blockDim.x) s_grank[i] = 0;
    __syncthreads();
    for (uint32_t size = 2; size <= padded; size <<= 1) {
      for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
        for (uint32_t i = tid; i < padded / 2; i += blockDim.x) {
          const uint32_t lo = 2 * stride * (i / stride) + (i % stride);
          const uint32_t hi = lo + stride;
          const bool up = (lo & size) == 0;
          const K a = s_samp[lo], b = s_samp[hi];
          if ((a > b) == up) {
            s_samp[lo] = b;
            s_samp[hi] = a;
          }
        }
        __syncthreads();
      }
    }
    // Global rank of every sample: lower_bound in each rank's whole run.
    for (uint32_t t = tid; t < cnt * np; t += blockDim.x) {
      const uint32_t s = t / np, r = t % np;
      const uint64_t lb = bound(data + p.roff[r0 + r], uint64_t(s_len[r]), s_samp[s], kx, false);
      atomicAdd(&s_grank[s], (unsigned long long)lb);
    }
    __syncthreads();
    // Per splitter: the sample just below its expected rank.
    if (tid < int(kw)) {
      uint32_t lo = 0, hi = cnt;  // upper_bound of exp in the ranks
      while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (int64_t(s_grank[mid]) <= s_exp[tid]) lo = mid + 1; else hi = mid;
      }
      const int ub = int(lo);
      const int lb = ub > 0 ? ub - 1 : 0;
      const int64_t gr = int64_t(s_grank[lb]);
      const int64_t err = gr > s_exp[tid] ? gr - s_exp[tid] : s_exp[tid] - gr;
      s_upd[tid] = err < s_maxerr ? 1 : 0;
      s_lb[tid] = lb;
      s_ub[tid] = ub;
      if (s_upd[tid]) {
        s_split[tid] = s_samp[lb];
        atomicMax(&s_newmax, (long long)err);
      }
    }
    __syncthreads();
    // Narrow the updated splitters' intervals in every rank.
    for (uint32_t t = tid; t < kw * np; t += blockDim.x) {
      const uint32_t i = t / np, r = t % np;
      if (!s_upd[i]) continue;
      const K* run = data + p.roff[r0 + r];
      const uint64_t len = uint64_t(s_len[r]);
      s_start[t] = int64_t(s_grank[s_lb[i]]) > s_exp[i]
                       ? 0
                       : int64_t(bound(run, len, s_samp[s_lb[i]], kx, false));
      s_end[t] = uint32_t(s_ub[i]) == cnt ? int64_t(len)
                                          : int64_t(bound(run, len, s_samp[s_ub[i]], kx, false));
    }
    __syncthreads();
    if (tid == 0) s_maxerr = s_newmax;
    ++it;
    __syncthreads();
  }
  if (tid < int(kw)) static_cast<K*>(p.splitters)[blockIdx.x * kw + tid] = s_split[tid];
  if (tid == 0 && p.iters) p.iters[blockIdx.x] = it;
}

struct CutParams {
  const void* data;
  const uint64_t* roff;
  uint32_t p, n_p, kway;
  uint32_t key_kind, desc;
  const void* splitters;
  uint64_t* cuts;  // p x (kway + 1)
};

// Step 2: rank r's run cut at its group's splitters (lower_bound).
template <typename K>
__global__ void __launch_bounds__(256) hyk_cut_kernel(CutParams p) {
  const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const uint32_t kw = p.kway;
  if (t >= uint64_t(p.p) * (kw + 1)) return;
  const uint32_t r = uint32_t(t / (kw + 1)), i = uint32_t(t % (kw + 1));
  const uint64_t len = p.roff[r + 1] - p.roff[r];
  uint64_t c;
  if (i == 0) {
    c = 0;
  } else if (i == kw) {
    c = len;
  } else {
    const OrderXform<K> kx(p.key_kind, p.desc != 0);
    const K y = static_cast<const K*>(p.splitters)[(r / p.n_p) * (kw - 1) + (i - 1)];
    c = bound(static_cast<const K*>(p.data) + p.roff[r], len, y, kx, false);
  }
  p.cuts[t] = c;
}

// Merge tiling. Samples are taken every S = GAP / k elements of each piece,
// so consecutive samples of a rank (in the order (value, piece, index)) are
// at most GAP output positions apart. Tile u of a rank starts at the largest
// sample position not above u * SPAN (SPAN = 3 * GAP), so a tile holds at
// most SPAN + GAP = CAP elements, SPAN on average.
template <typename K> struct MergeGeom {
  static constexpr uint32_t GAP = sizeof(K) == 4 ? 2048u : 1024u;
  static constexpr uint32_t SPAN = 3 * GAP;
  static constexpr uint32_t CAP = SPAN + GAP;  // 32 KB of keys per staging buffer
};

struct MergeParams {
  const void* src;
  void* dst;
  const HykPiece* pieces;
  uint32_t npieces;
  uint32_t kway;
  uint64_t nsamples;
  uint32_t stride;         // S: a sample every S elements of a piece
  uint32_t key_kind, desc;
  uint64_t* samp_rank;     // [nsamples]: the sample's position in its rank's output
  uint64_t* samp_cut;      // [nsamples][kway]: elements of each piece before the sample
  const uint64_t* rtile;   // [p + 1]: first tile of each receiving rank
  uint32_t p;              // receiving ranks
  uint64_t ntiles;
  uint64_t* tile_out;      // [ntiles]: output position of the tile's first element
  uint64_t* tile_src;      // [ntiles][kway]: source position of the tile's run of each piece
  uint32_t* tile_len;      // [ntiles][kway]: length of that run
  uint32_t* err;           // device error word
};

// Piece holding global sample s: the last piece whose first sample is <= s
// (pieces without samples share their successor's first sample).
__device__ __forceinline__ uint32_t piece_of(const HykPiece* pc, uint32_t np, uint64_t s) {
  uint32_t lo = 0, hi = np;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (pc[mid].sample0 <= s) lo = mid + 1; else hi = mid;
  }
  return lo - 1;
}

// Step 3a: position of every sample in its rank's output, and its cut in
// every piece, under the order (value, piece, index).
template <typename K>
__global__ void __launch_bounds__(256) hyk_sample_kernel(MergeParams p) {
  const uint64_t s = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (s >= p.nsamples) return;
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* src = static_cast<const K*>(p.src);
  const HykPiece P = p.pieces[piece_of(p.pieces, p.npieces, s)];
  const uint64_t e = (s - P.sample0) * p.stride;
  const K x = kx.fwd(src[P.src + e]);
  uint64_t rank = 0;
  for (uint32_t i = 0; i < p.kway; ++i) {
    const HykPiece Q = p.pieces[P.first + i];
    const uint64_t c = i == P.j ? e : bound(src + Q.src, Q.len, x, kx, i < P.j);
    p.samp_cut[s * p.kway + i] = c;
    rank += c;
  }
  p.samp_rank[s] = rank;
}

// The sample of rank r's pieces whose position is the largest not above d
// (position 0 is always a sample: the rank's first element).
__device__ __forceinline__ uint64_t sample_at(const MergeParams& p, uint32_t first, uint64_t d) {
  uint64_t best = ~uint64_t(0), best_rank = 0;
  for (uint32_t i = 0; i < p.kway; ++i) {
    const HykPiece Q = p.pieces[first + i];
    const uint64_t ns = (Q.len + p.stride - 1) / p.stride;
    uint64_t lo = 0, hi = ns;  // first sample of piece i above d
    while (lo < hi) {
      const uint64_t mid = (lo + hi) >> 1;
      if (p.samp_rank[Q.sample0 + mid] <= d) lo = mid + 1; else hi = mid;
    }
    if (lo > 0) {
      const uint64_t c = Q.sample0 + lo - 1;
      const uint64_t rk = p.samp_rank[c];
      if (best == ~uint64_t(0) || rk > best_rank) {
        best = c;
        best_rank = rk;
      }
    }
  }
  return best;
}

// Step 3b: one thread per tile writes the tile's descriptor: its output
// position and the run of each piece it merges.
template <typename K>
__global__ void __launch_bounds__(256) hyk_tile_kernel(MergeParams p) {
  const uint64_t t = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= p.ntiles) return;
  uint32_t lo = 0, hi = p.p;  // receiving rank: last r with rtile[r] <= t
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (p.rtile[mid] <= t) lo = mid; else hi = mid;
  }
  const uint32_t r = lo;
  const uint32_t first = r * p.kway;
  const uint64_t u = t - p.rtile[r];
  uint64_t len = 0;
  for (uint32_t i = 0; i < p.kway; ++i) len += p.pieces[first + i].len;
  constexpr uint64_t SPAN = MergeGeom<K>::SPAN;
  const uint64_t sb = u == 0 ? ~uint64_t(0) : sample_at(p, first, u * SPAN);
  const uint64_t se = (u + 1) * SPAN >= len ? ~uint64_t(0) : sample_at(p, first, (u + 1) * SPAN);
  const HykPiece P0 = p.pieces[first];
  p.tile_out[t] = P0.out + (sb == ~uint64_t(0) ? 0 : p.samp_rank[sb]);
  for (uint32_t i = 0; i < p.kway; ++i) {
    const HykPiece Q = p.pieces[first + i];
    const uint64_t c0 = sb == ~uint64_t(0) ? 0 : p.samp_cut[sb * p.kway + i];
    const uint64_t c1 = se == ~uint64_t(0) ? Q.len : p.samp_cut[se * p.kway + i];
    p.tile_src[t * p.kway + i] = Q.src + c0;
    p.tile_len[t * p.kway + i] = uint32_t(c1 - c0);
  }
}

// Step 3c: one CTA per tile. The tile's run of each piece is staged in
// shared memory (order bits), then merged by log2(k) levels of 2-way merges
// in shared memory: level by level, runs 2q and 2q+1 become one, the lower
// run first on ties, which keeps the order (value, piece) the tiles were cut
// by. Each thread writes a range of consecutive outputs of a level (the
// tile's length over the threads): one merge-path search for its start,
// then a sequential merge. Measured at 2^26 u32 keys, k = 4: 292 us per
// merge launch; fixed runs of 16 outputs per thread with an unrolled merge
// and a padded layout, 418 us; padding alone, 383 us.
template <typename K, int KW>
__global__ void __launch_bounds__(MERGE_THREADS) hyk_merge_kernel(MergeParams p) {
  constexpr uint32_t CAP = MergeGeom<K>::CAP;
  extern __shared__ __align__(16) uint8_t s_dyn[];
  K* s_a = reinterpret_cast<K*>(s_dyn);
  K* s_b = s_a + CAP;
  __shared__ uint32_t s_off[KW + 1];
  __shared__ uint64_t s_src[KW];
  const uint64_t t = blockIdx.x;
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* src = static_cast<const K*>(p.src);
  const int tid = threadIdx.x;
  if (tid < KW) {
    s_src[tid] = p.tile_src[t * KW + tid];
    s_off[tid + 1] = p.tile_len[t * KW + tid];
  }
  __syncthreads();
  if (tid == 0) {
    s_off[0] = 0;
    for (int i = 1; i <= KW; ++i) s_off[i] += s_off[i - 1];
  }
  __syncthreads();
  const uint32_t total = s_off[KW];
  if (total > CAP) {  // cannot happen: tiles are cut at most CAP apart
    if (tid == 0) atomicOr(p.err, ERR_SCATTER_RANGE);
    return;
  }
  // All of a thread's loads are issued before the first staging store, so
  // they are in flight together.
  constexpr int LPT = int(CAP / MERGE_THREADS);
  {
    K v[LPT];
#pragma unroll
    for (int u = 0; u < LPT; ++u) {
      const uint32_t e = uint32_t(tid + u * MERGE_THREADS);
      if (e < total) {
        int j = 0;
#pragma unroll
        for (int i = 1; i < KW; ++i) j += e >= s_off[i] ? 1 : 0;
        v[u] = src[s_src[j] + (e - s_off[j])];
      }
    }
#pragma unroll
    for (int u = 0; u < LPT; ++u) {
      const uint32_t e = uint32_t(tid + u * MERGE_THREADS);
      if (e < total) s_a[e] = kx.fwd(v[u]);
    }
  }
  __syncthreads();
  const uint32_t per = (total + MERGE_THREADS - 1) / MERGE_THREADS;
  const uint32_t e0 = min(total, tid * per), e1 = min(total, e0 + per);
  K* in = s_a;
  K* out = s_b;
#pragma unroll
  for (int runs = KW; runs > 1; runs >>= 1) {
    uint32_t e = e0;
    int q = 0;
    while (e < e1) {
      while (s_off[2 * q + 2] <= e) ++q;  // the pair holding output e
      const uint32_t a0 = s_off[2 * q], na = s_off[2 * q + 1] - a0;
      const uint32_t nb = s_off[2 * q + 2] - s_off[2 * q + 1];
      const K* A = in + a0;
      const K* B = A + na;
      const uint32_t d = e - a0;
      uint32_t lo = d > nb ? d - nb : 0, hi = d < na ? d : na;
      while (lo < hi) {  // outputs of the first d that come from A
        const uint32_t mid = (lo + hi) >> 1;
        if (B[d - mid - 1] < A[mid]) hi = mid; else lo = mid + 1;
      }
      uint32_t i = lo, j = d - lo;
      K x = i < na ? A[i] : K(0);
      K y = j < nb ? B[j] : K(0);
      const uint32_t end = min(e1, s_off[2 * q + 2]);
      for (; e < end; ++e) {
        const bool take_a = j >= nb || (i < na && !(y < x));
        out[e] = take_a ? x : y;
        if (take_a) {
          if (++i < na) x = A[i];
        } else {
          if (++j < nb) y = B[j];
        }
      }
    }
    __syncthreads();
    if (tid == 0) {
      for (int r = 1; r <= runs / 2; ++r) s_off[r] = s_off[2 * r];
    }
    __syncthreads();
    K* tmp = in;
    in = out;
    out = tmp;
  }
  K* dst = static_cast<K*>(p.dst) + p.tile_out[t];
#pragma unroll
  for (int u = 0; u < LPT; ++u) {
    const uint32_t e = uint32_t(tid + u * MERGE_THREADS);
    if (e < total) dst[e] = kx.inv(in[e]);
  }
}

template <typename K, int KW>
cudaError_t merge_t(MergeParams mp, cudaStream_t st) {
  constexpr size_t SMEM = 2 * size_t(MergeGeom<K>::CAP) * sizeof(K);
  auto mk = hyk_merge_kernel<K, KW>;
  cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(mk), SMEM);
  if (e != cudaSuccess) return e;
  const unsigned sb = unsigned((mp.nsamples + 255) / 256);
  hyk_sample_kernel<K><<<sb, 256, 0, st>>>(mp);
  hyk_tile_kernel<K><<<unsigned((mp.ntiles + 255) / 256), 256, 0, st>>>(mp);
  mk<<<unsigned(mp.ntiles), MERGE_THREADS, SMEM, st>>>(mp);
  return cudaGetLastError();
}

template <typename K>
cudaError_t merge_k(MergeParams mp, cudaStream_t st) {
  switch (mp.kway) {
    case 2: return merge_t<K, 2>(mp, st);
    case 4: return merge_t<K, 4>(mp, st);
    case 8: return merge_t<K, 8>(mp, st);
    case 16: return merge_t<K, 16>(mp, st);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

uint32_t hyk_sample_stride(int key_bytes, uint32_t kway) {
  return (key_bytes == 4 ? MergeGeom<uint32_t>::GAP : MergeGeom<uint64_t>::GAP) / kway;
}

uint32_t hyk_tile_span(int key_bytes) {
  return key_bytes == 4 ? MergeGeom<uint32_t>::SPAN : MergeGeom<uint64_t>::SPAN;
}

size_t hyk_select_smem(int key_bytes, uint32_t n_p, uint32_t kway) {
  return key_bytes == 4 ? select_smem<uint32_t>(n_p, kway) : select_smem<uint64_t>(n_p, kway);
}

cudaError_t launch_hyk_select(const HykRound& r, cudaStream_t st) {
  SelectParams sp{r.data, r.roff, r.n_p, r.kway, r.key_kind, uint32_t(r.desc), r.seed,
                  r.splitters, r.iters};
  CutParams cp{r.data, r.roff, r.p, r.n_p, r.kway, r.key_kind, uint32_t(r.desc), r.splitters,
               r.cuts};
  const unsigned groups = r.p / r.n_p;
  const size_t smem = hyk_select_smem(r.key_bytes, r.n_p, r.kway);
  const uint64_t ncut = uint64_t(r.p) * (r.kway + 1);
  // allow_dynamic_smem opts a kernel in once, so once at the largest size
  // any round can ask for.
  const size_t smem_max = hyk_select_smem(r.key_bytes, HYK_MAX_RANKS, MAX_KWAY);
  if (smem > smem_max) return cudaErrorInvalidValue;
  auto go = [&](auto sel, auto cut) -> cudaError_t {
    cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(sel), smem_max);
    if (e != cudaSuccess) return e;
    sel<<<groups, SELECT_THREADS, smem, st>>>(sp);
    cut<<<unsigned((ncut + 255) / 256), 256, 0, st>>>(cp);
    return cudaGetLastError();
  };
  if (r.key_bytes == 4) return go(hyk_select_kernel<uint32_t>, hyk_cut_kernel<uint32_t>);
  return go(hyk_select_kernel<uint64_t>, hyk_cut_kernel<uint64_t>);
}

cudaError_t launch_hyk_merge(const HykRound& r, const HykPiece* pieces, uint32_t npieces,
                             uint64_t nsamples, const uint64_t* rtile, uint64_t ntiles,
                             const void* src, void* dst, cudaStream_t st) {
  if (ntiles == 0) return cudaSuccess;
  if (ntiles > 0x7FFFFFFFull || nsamples > 0x7FFFFFFFull * 256ull) return cudaErrorInvalidValue;
  MergeParams mp{src, dst, pieces, npieces, r.kway, nsamples,
                 hyk_sample_stride(r.key_bytes, r.kway), r.key_kind, uint32_t(r.desc),
                 r.samp_rank, r.samp_cut, rtile, r.p, ntiles, r.tile_out, r.tile_src,
                 r.tile_len, r.err};
  if (r.key_bytes == 4) return merge_k<uint32_t>(mp, st);
  return merge_k<uint64_t>(mp, st);
}

}  // namespace gs
