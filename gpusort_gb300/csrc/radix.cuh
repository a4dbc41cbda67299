// Onesweep LSD radix sort for one array (keys, optionally with a payload).
//
// This is the engine's local sort. It replaces the reference's Thrust call
// (src/cuda_utils.cu:403-445 SortByThrust, :447-506 for pairs) and its
// OpenMP merge sort (include/omp/omp_utils.h:147-207). The pipeline per
// sort is:
//   1. upsweep_kernel  - one read of the input, histograms of every 8-bit
//                        digit of the order-mapped keys (and values when
//                        ties are ordered by value);
//   2. plan_kernel     - exclusive scans of those histograms (global bin
//                        bases), skip decisions for digits whose histogram
//                        has a single non-empty bin, ping-pong buffer plan;
//   3. pass_kernel x D - one pass per digit: warp match_any ranking, tile
//                        aggregate published at once, decoupled look-back
//                        across tiles with bounded waits, tile reordered in
//                        shared memory, coalesced scatter by digit.
// Everything is enqueued on one stream without host round trips, so the
// pipeline is graph-capturable.
#pragma once

#include "common.cuh"
#include "radix_types.cuh"

namespace gs {

// ---------------------------------------------------------------------------
// Upsweep: all digit histograms in one read.
// ---------------------------------------------------------------------------

// Count digit `d` in histogram `h`. When the whole warp holds the same digit
// (sorted runs, all-equal or low-cardinality inputs) one lane adds 32, so a
// skewed input does not serialise on one shared-memory word.
__device__ __forceinline__ void add_digit(uint32_t* h, uint32_t d, bool valid) {
  const uint32_t d0 = __shfl_sync(0xffffffffu, d, 0);
  if (__all_sync(0xffffffffu, valid && d == d0)) {
    if ((threadIdx.x & 31) == 0) atomicAdd(&h[d0], 32u);
  } else if (valid) {
    atomicAdd(&h[d], 1u);
  }
}

template <typename K, typename V, int THREADS, int UNROLL>
__global__ void __launch_bounds__(THREADS)
upsweep_kernel(UpsweepParams p) {
  constexpr int KD = Bits<K>::DIGITS;
  constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  __shared__ uint32_t s_hist[MAX_DIGITS * RADIX];
  const uint32_t vd = p.val_digits;
  const uint32_t total_digits = vd + KD;
  for (uint32_t i = threadIdx.x; i < total_digits * RADIX; i += THREADS) s_hist[i] = 0;
  __syncthreads();

  const K* keys = static_cast<const K*>(p.keys);
  const bool desc = p.desc != 0;
  const uint64_t n = p.n;
  const uint64_t chunk = uint64_t(THREADS) * UNROLL;
  for (uint64_t base = uint64_t(blockIdx.x) * chunk; base < n;
       base += uint64_t(gridDim.x) * chunk) {
    K k[UNROLL];
    bool valid[UNROLL];
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const uint64_t idx = base + uint64_t(u) * THREADS + threadIdx.x;
      valid[u] = idx < n;
      k[u] = valid[u] ? ld_stream(keys + idx) : K(0);
    }
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      const K b = order_bits<K>(k[u], p.key_kind, desc);
#pragma unroll
      for (int d = 0; d < KD; ++d) {
        add_digit(s_hist + (vd + d) * RADIX, uint32_t(b >> (RADIX_BITS * d)) & (RADIX - 1),
                  valid[u]);
      }
    }
    if constexpr (HAS_V) {
      if (vd > 0) {
        const V* vals = static_cast<const V*>(p.vals);
        V v[UNROLL];
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
          const uint64_t idx = base + uint64_t(u) * THREADS + threadIdx.x;
          v[u] = valid[u] ? ld_stream(vals + idx) : V(0);
        }
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
          const V b = order_bits<V>(v[u], p.val_kind, desc);
#pragma unroll
          for (int d = 0; d < Bits<V>::DIGITS; ++d) {
            add_digit(s_hist + d * RADIX, uint32_t(b >> (RADIX_BITS * d)) & (RADIX - 1),
                      valid[u]);
          }
        }
      }
    }
  }
  __syncthreads();
  uint32_t* g = &p.work->hist[0][0];
  for (uint32_t i = threadIdx.x; i < total_digits * RADIX; i += THREADS) {
    const uint32_t c = s_hist[i];
    if (c) atomicAdd(&g[i], c);
  }
}

// ---------------------------------------------------------------------------
// Plan: bin bases, skipped digits, pass numbering. One block of 256 threads.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) plan_kernel(PlanParams p) {
  __shared__ uint32_t s_tmp[8];
  __shared__ uint32_t s_trivial[MAX_DIGITS];
  SortPlan& plan = p.work->plan;
  const uint32_t tid = threadIdx.x;
  if (tid < MAX_DIGITS) s_trivial[tid] = 0;
  __syncthreads();
  for (uint32_t q = 0; q < p.digits; ++q) {
    const uint32_t c = p.work->hist[q][tid];
    if (uint64_t(c) == p.n) s_trivial[q] = 1;  // one bin holds every key
    const uint32_t ex = block_excl_scan_256(c, s_tmp);
    plan.binbase[q][tid] = ex;
  }
  if (tid < MAX_DIGITS) plan.tile_counter[tid] = 0;
  __syncthreads();
  if (tid == 0) {
    bool exec[MAX_DIGITS];
    uint32_t m = 0;
    for (uint32_t q = 0; q < MAX_DIGITS; ++q) {
      exec[q] = (q < p.digits) && !s_trivial[q];
      m += exec[q];
    }
    // Every key equal: nothing to reorder, but a copy (or the reversal of a
    // stable descending pair sort) still has to reach the output.
    if (m == 0 && (!p.in_place || p.reverse_first)) {
      exec[p.digits - 1] = true;
      m = 1;
    }
    // In place, the first pass may not write its own input: make the pass
    // count even so the first pass writes the scratch buffer.
    if (p.in_place && (m & 1u)) {
      for (uint32_t q = 0; q < p.digits; ++q) {
        if (!exec[q]) { exec[q] = true; ++m; break; }
      }
    }
    uint32_t j = 0;
    for (uint32_t q = 0; q < MAX_DIGITS; ++q) plan.exec_index[q] = exec[q] ? j++ : PASS_SKIPPED;
    plan.m_exec = m;
  }
}

// ---------------------------------------------------------------------------
// One onesweep pass.
// ---------------------------------------------------------------------------
template <typename K, typename V, int THREADS, int ITEMS>
struct PassConfig {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * ITEMS;
  static constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  static constexpr size_t VAL_BYTES = HAS_V ? sizeof(typename std::conditional<HAS_V, V, uint32_t>::type) : 0;
  static constexpr size_t SMEM_KEYS = size_t(TILE) * sizeof(K);
  static constexpr size_t SMEM_VALS = size_t(TILE) * VAL_BYTES;
  static constexpr size_t DYN_SMEM = SMEM_KEYS + SMEM_VALS;
};

template <typename K, typename V, int THREADS, int ITEMS, int MIN_BLOCKS>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
pass_kernel(PassParams p) {
  using Cfg = PassConfig<K, V, THREADS, ITEMS>;
  constexpr int WARPS = Cfg::WARPS;
  constexpr int TILE = Cfg::TILE;
  constexpr bool HAS_V = Cfg::HAS_V;
  using VS = typename std::conditional<HAS_V, V, uint32_t>::type;  // storage type

  extern __shared__ __align__(16) uint8_t s_dyn[];
  __shared__ uint32_t s_warp_hist[WARPS][RADIX + 1];
  __shared__ uint32_t s_tile_excl[RADIX];
  __shared__ uint32_t s_dst_base[RADIX];
  __shared__ uint32_t s_tmp[8];
  __shared__ uint32_t s_tile;

  SortPlan& plan = p.work->plan;
  const uint32_t j = plan.exec_index[p.pass];
  if (j == PASS_SKIPPED) return;
  const uint32_t m = plan.m_exec;

  // Ping-pong: pass j writes `out` when (m - j) is odd, so the last pass
  // always lands in `out`; pass 0 reads the caller's input.
  const bool dst_is_out = ((m - j) & 1u) != 0;
  const K* src_k;
  const VS* src_v = nullptr;
  if (j == 0) {
    src_k = static_cast<const K*>(p.keys_in);
    if constexpr (HAS_V) src_v = static_cast<const VS*>(p.vals_in);
  } else {
    src_k = static_cast<const K*>(dst_is_out ? p.keys_alt : p.keys_out);
    if constexpr (HAS_V) src_v = static_cast<const VS*>(dst_is_out ? p.vals_alt : p.vals_out);
  }
  K* dst_k = static_cast<K*>(dst_is_out ? p.keys_out : p.keys_alt);
  VS* dst_v = nullptr;
  if constexpr (HAS_V) dst_v = static_cast<VS*>(dst_is_out ? p.vals_out : p.vals_alt);
  const bool reverse = (j == 0) && p.reverse_first;

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint64_t n = p.n;
  const bool desc = p.desc != 0;
  const bool from_val = p.pass < p.val_digits;
  const uint32_t shift = RADIX_BITS * (from_val ? p.pass : (p.pass - p.val_digits));

  if (tid == 0) s_tile = atomicAdd(&plan.tile_counter[p.pass], 1u);
  for (int i = tid; i < WARPS * (RADIX + 1); i += THREADS) (&s_warp_hist[0][0])[i] = 0;
  __syncthreads();
  const uint32_t tile = s_tile;
  const uint64_t tile_base = uint64_t(tile) * TILE;
  const uint64_t warp_base = tile_base + uint64_t(warp) * 32 * ITEMS;

  auto digit_of_key = [&](K k) -> uint32_t {
    return uint32_t(order_bits<K>(k, p.key_kind, desc) >> shift) & (RADIX - 1);
  };
  auto digit_of_val = [&](VS v) -> uint32_t {
    return uint32_t(order_bits<VS>(v, p.val_kind, desc) >> shift) & (RADIX - 1);
  };

  // Load: item i of lane l is element warp_base + 32*i + l, so (i, lane)
  // order is input order and the ranking below is stable.
  K keys[ITEMS];
  VS vals[HAS_V ? ITEMS : 1];
  uint32_t rank[ITEMS];
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const uint64_t idx = warp_base + uint64_t(i) * 32 + lane;
    const bool valid = idx < n;
    const uint64_t sidx = reverse ? (n - 1 - idx) : idx;
    keys[i] = valid ? ld_stream(src_k + sidx) : K(0);
    if constexpr (HAS_V) vals[i] = valid ? ld_stream(src_v + sidx) : VS(0);
  }

  // Warp ranking with match_any: peers holding the same digit get
  // consecutive ranks in lane order; the group's lowest lane bumps the
  // warp's counter for that digit.
  const uint32_t lt = lanemask_lt();
  uint32_t* wh = s_warp_hist[warp];
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const uint64_t idx = warp_base + uint64_t(i) * 32 + lane;
    uint32_t d;
    if constexpr (HAS_V) {
      d = from_val ? digit_of_val(vals[i]) : digit_of_key(keys[i]);
    } else {
      d = digit_of_key(keys[i]);
    }
    d = (idx < n) ? d : uint32_t(RADIX);  // padding lanes use the spare bin
    const uint32_t peers = __match_any_sync(0xffffffffu, d);
    const uint32_t base = wh[d];
    rank[i] = base + __popc(peers & lt);
    __syncwarp();
    if ((peers & lt) == 0) wh[d] = base + __popc(peers);
    __syncwarp();
  }
  __syncthreads();

  // Per digit: exclusive offsets of each warp, tile count, aggregate out.
  uint32_t count = 0;
  uint64_t* status = p.status + uint64_t(tile) * RADIX;
  if (tid < RADIX) {
    uint32_t run = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
      const uint32_t c = s_warp_hist[w][tid];
      s_warp_hist[w][tid] = run;
      run += c;
    }
    count = run;
    st_relaxed(status + tid, make_status(tile == 0 ? FLAG_INC : FLAG_AGG, p.gen, count));
  }
  const uint32_t tile_excl = block_excl_scan_256(count, s_tmp);

  // Decoupled look-back over preceding tiles, bounded.
  if (tid < RADIX) {
    uint32_t prefix = 0;
    if (tile > 0) {
      int64_t t = int64_t(tile) - 1;
      uint32_t spins = 0;
      uint32_t backoff = 8;
      const bool stall = p.inject_stall && tile == 1;
      while (true) {
        const uint64_t w = stall ? 0ull : ld_relaxed(p.status + uint64_t(t) * RADIX + tid);
        const uint64_t flag = w & FLAG_MASK;
        if (flag == 0 || uint32_t(w >> 32 & GEN_MASK) != (p.gen & GEN_MASK)) {
          if (++spins > p.spin_limit) {
            atomicOr(p.err, ERR_LOOKBACK_TIMEOUT);
            break;
          }
          __nanosleep(backoff);
          if (backoff < 1024) backoff <<= 1;
          continue;
        }
        prefix += uint32_t(w);
        if (flag == FLAG_INC || t == 0) break;
        --t;
        backoff = 8;
      }
      st_relaxed(status + tid, make_status(FLAG_INC, p.gen, prefix + count));
    }
    s_tile_excl[tid] = tile_excl;
    s_dst_base[tid] = plan.binbase[p.pass][tid] + prefix - tile_excl;
  }
  __syncthreads();

  // Reorder the tile in shared memory by digit.
  K* s_keys = reinterpret_cast<K*>(s_dyn);
  VS* s_vals = reinterpret_cast<VS*>(s_dyn + Cfg::SMEM_KEYS);
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const uint64_t idx = warp_base + uint64_t(i) * 32 + lane;
    if (idx < n) {
      uint32_t d;
      if constexpr (HAS_V) {
        d = from_val ? digit_of_val(vals[i]) : digit_of_key(keys[i]);
      } else {
        d = digit_of_key(keys[i]);
      }
      const uint32_t pos = s_tile_excl[d] + s_warp_hist[warp][d] + rank[i];
      s_keys[pos] = keys[i];
      if constexpr (HAS_V) s_vals[pos] = vals[i];
    }
  }
  __syncthreads();

  // Scatter: consecutive tile positions of one digit go to consecutive
  // output addresses.
  const uint64_t remaining = n - tile_base;
  const uint32_t tile_n = remaining < uint64_t(TILE) ? uint32_t(remaining) : uint32_t(TILE);
#pragma unroll
  for (int i = 0; i < ITEMS; ++i) {
    const uint32_t r = uint32_t(i) * THREADS + tid;
    if (r < tile_n) {
      const K k = s_keys[r];
      uint32_t d;
      VS v;
      if constexpr (HAS_V) {
        v = s_vals[r];
        d = from_val ? digit_of_val(v) : digit_of_key(k);
      } else {
        d = digit_of_key(k);
      }
      const uint32_t dst = s_dst_base[d] + r;
      if (uint64_t(dst) < n) {
        dst_k[dst] = k;
        if constexpr (HAS_V) dst_v[dst] = v;
      } else {
        atomicOr(p.err, ERR_SCATTER_RANGE);
      }
    }
  }
}

}  // namespace gs
