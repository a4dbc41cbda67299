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
//   3. pass_kernel x D - one pass per digit: stable warp ranking through
//                        shared peer masks (the first pass may use one shared
//                        atomic per element instead), tile aggregate
//                        published at once, windowed decoupled look-back with
//                        bounded waits, tile reordered in shared memory,
//                        coalesced scatter by digit.
// Everything is enqueued on one stream without host round trips, so the
// pipeline is graph-capturable.
#pragma once

#include "common.cuh"
#include "radix_types.cuh"

namespace gs {

// Branch-free order transform of one element type: forward maps raw bits
// to bits whose unsigned order is the requested order (std::less, or
// std::greater when `desc`; include/common.h:156-164 maps the comparator to
// that flag); inverse undoes it. Signed keys flip the sign bit; IEEE keys
// flip every bit of negative values and only the sign bit of the others,
// so -inf < ... < -0 < +0 < ... < +inf.
template <typename U>
struct OrderXform {
  U fmask, smask, dmask;
  __device__ __forceinline__ OrderXform(uint32_t kind, bool desc)
      : fmask(kind == KIND_FLOAT ? ~U(0) : U(0)),
        smask(kind == KIND_UNSIGNED ? U(0) : Bits<U>::SIGN),
        dmask(desc ? ~U(0) : U(0)) {}
  // Order bits of -0.0 and +0.0 (both 0 for integer kinds).
  __device__ __forceinline__ U neg_zero() const { return fmask ? fwd(Bits<U>::SIGN) : U(0); }
  __device__ __forceinline__ U pos_zero() const { return fmask ? fwd(U(0)) : U(0); }
  __device__ __forceinline__ U fwd(U x) const {
    using S = typename std::make_signed<U>::type;
    const U neg = U(S(x) >> (8 * sizeof(U) - 1));
    return x ^ ((neg & fmask) | smask) ^ dmask;
  }
  __device__ __forceinline__ U inv(U y) const {
    using S = typename std::make_signed<U>::type;
    const U t = y ^ dmask;
    const U was_neg = U(S(~t) >> (8 * sizeof(U) - 1));
    return t ^ ((was_neg & fmask) | smask);
  }
};

// ---------------------------------------------------------------------------
// Upsweep: all digit histograms in one read.
// ---------------------------------------------------------------------------

// The histograms live in shared memory as hist[digit][bin][column], with
// 2^CL columns and lane l counting into column l mod 2^CL: lanes of a warp
// that draw the same bank for different bins then mostly land in different
// banks, so the random-bin atomics of a warp take about 2 shared-memory
// wavefronts instead of 3.5 (16 columns). CL is a compile-time constant so
// each counter's address is one shift-add. Atomics to one address from a
// whole warp are combined in hardware, so skewed inputs need no special
// case.
template <typename K, typename V, int THREADS, int UNROLL, int CL>
__global__ void __launch_bounds__(THREADS)
upsweep_kernel(UpsweepParams p) {
  constexpr int KD = Bits<K>::DIGITS;
  constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  constexpr uint32_t NC = 1u << CL;  // columns per bin
  extern __shared__ __align__(16) uint32_t s_hist[];  // [digits][RADIX][NC]
  const uint32_t vd = p.val_digits;
  const uint32_t total_digits = vd + KD;
  const uint32_t words = total_digits * RADIX * NC;
  for (uint32_t i = threadIdx.x; i < words; i += THREADS) s_hist[i] = 0;
  __syncthreads();
  // This thread's column; digit q's histogram starts at q * RADIX * NC.
  uint32_t* const hk = s_hist + vd * RADIX * NC + (threadIdx.x & (NC - 1));
  uint32_t* const hv = s_hist + (threadIdx.x & (NC - 1));

  const K* keys = static_cast<const K*>(p.keys);
  const V* vals = nullptr;
  if constexpr (HAS_V) vals = static_cast<const V*>(p.vals);
  const bool desc = p.desc != 0;
  const uint64_t n = p.n;
  const uint64_t chunk = uint64_t(THREADS) * UNROLL;
  K* const copy_k = static_cast<K*>(p.copy_keys);
  // Keys only: interior chunks are read as 16-byte vectors when the
  // buffers are 16-byte aligned (2^30 u32 keys: 1.00 -> 0.86 ms), the next
  // chunk's loads in flight while this one is counted (0.86 -> 0.82 ms).
  constexpr int KPV = int(16 / sizeof(K));  // keys per vector
  constexpr bool VEC = !HAS_V && UNROLL % KPV == 0;
  const bool vec = VEC && (reinterpret_cast<uintptr_t>(keys) & 15u) == 0 &&
                   (reinterpret_cast<uintptr_t>(copy_k) & 15u) == 0;
  V* copy_v = nullptr;
  if constexpr (HAS_V) copy_v = static_cast<V*>(p.copy_vals);
  // Pair sorts: -0.0 counts as +0.0 (see pass_kernel).
  K zneg = 0, zpos = 0;
  if (HAS_V && p.key_kind == KIND_FLOAT) {
    zneg = order_bits<K>(Bits<K>::SIGN, p.key_kind, desc);
    zpos = order_bits<K>(K(0), p.key_kind, desc);
  }
  auto count = [&](const K (&k)[UNROLL], const bool (&valid)[UNROLL]) {
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      K b = order_bits<K>(k[u], p.key_kind, desc);
      if constexpr (HAS_V) b = b == zneg ? zpos : b;
#pragma unroll
      for (int d = 0; d < KD; ++d) {
        const uint32_t bin = uint32_t(b >> (RADIX_BITS * d)) & (RADIX - 1);
        if (valid[u]) atomicAdd(hk + d * RADIX * NC + (bin << CL), 1u);
      }
    }
  };
  auto count_vals = [&](uint64_t base, const bool (&valid)[UNROLL]) {
    if constexpr (HAS_V) {
      V v[UNROLL];
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint64_t idx = base + uint64_t(u) * THREADS + threadIdx.x;
        v[u] = valid[u] ? ld_stream(vals + idx) : V(0);
        if (copy_v && valid[u]) copy_v[idx] = v[u];
      }
      if (vd == 0) return;  // values only copied
      if (p.check_val_order) {
        // Each value against its successor in input order (lane 31's
        // successor is the next warp's first element).
        bool broken = false;
#pragma unroll
        for (int u = 0; u < UNROLL; ++u) {
          const uint64_t idx = base + uint64_t(u) * THREADS + threadIdx.x;
          V nx = __shfl_down_sync(0xFFFFFFFFu, v[u], 1);
          if ((threadIdx.x & 31) == 31 && idx + 1 < n) nx = ld_stream(vals + idx + 1);
          if (valid[u] && idx + 1 < n &&
              order_bits<V>(nx, p.val_kind, false) < order_bits<V>(v[u], p.val_kind, false))
            broken = true;
        }
        if (__any_sync(0xFFFFFFFFu, broken) && (threadIdx.x & 31) == 0)
          atomicOr(&p.work->val_order_break, 1u);
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const V b = order_bits<V>(v[u], p.val_kind, desc);
#pragma unroll
        for (int d = 0; d < Bits<V>::DIGITS; ++d) {
          const uint32_t bin = uint32_t(b >> (RADIX_BITS * d)) & (RADIX - 1);
          if (valid[u]) atomicAdd(hv + d * RADIX * NC + (bin << CL), 1u);
        }
      }
    }
  };
  uint64_t base = uint64_t(blockIdx.x) * chunk;
  const uint64_t stride = uint64_t(gridDim.x) * chunk;
  if (VEC && vec) {
    // Interior chunks, keys only, software-pipelined: the next chunk's
    // vectors load while this one's keys are counted. Thread t's items are
    // the keys of 16-byte vectors t, t + THREADS, ... (the order of a
    // histogram's counts does not matter).
    constexpr int NV = UNROLL / KPV;
    uint4 q[NV], qn[NV];
    auto load = [&](uint64_t b, uint4 (&dst)[NV]) {
      const uint32_t* kb = reinterpret_cast<const uint32_t*>(keys + b);
#pragma unroll
      for (int u = 0; u < NV; ++u) dst[u] = ld_stream_v4(kb + 4 * (u * THREADS + threadIdx.x));
    };
    if (base + chunk <= n) load(base, q);
    while (base + chunk <= n) {
      const uint64_t nb = base + stride;
      const bool more = nb + chunk <= n;
      if (more) load(nb, qn);
      K k[UNROLL];
      bool valid[UNROLL];
#pragma unroll
      for (int u = 0; u < NV; ++u) {
        if constexpr (KPV == 4) {
          k[4 * u] = K(q[u].x);
          k[4 * u + 1] = K(q[u].y);
          k[4 * u + 2] = K(q[u].z);
          k[4 * u + 3] = K(q[u].w);
        } else {
          k[2 * u] = K(q[u].x) | (K(q[u].y) << 32);
          k[2 * u + 1] = K(q[u].z) | (K(q[u].w) << 32);
        }
      }
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) valid[u] = true;
      if (copy_k) {
        uint32_t* cb = reinterpret_cast<uint32_t*>(copy_k + base);
#pragma unroll
        for (int u = 0; u < NV; ++u)
          *reinterpret_cast<uint4*>(cb + 4 * (u * THREADS + threadIdx.x)) = q[u];
      }
      count(k, valid);
#pragma unroll
      for (int u = 0; u < NV; ++u) q[u] = qn[u];
      base = nb;
      if (!more) break;
    }
  }
  for (; base < n; base += stride) {
    K k[UNROLL];
    bool valid[UNROLL];
    if (base + chunk <= n) {  // interior chunk: no bounds checks
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        valid[u] = true;
        k[u] = ld_stream(keys + base + uint64_t(u) * THREADS + threadIdx.x);
      }
    } else {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        const uint64_t idx = base + uint64_t(u) * THREADS + threadIdx.x;
        valid[u] = idx < n;
        k[u] = valid[u] ? ld_stream(keys + idx) : K(0);
      }
    }
    if (copy_k) {
#pragma unroll
      for (int u = 0; u < UNROLL; ++u)
        if (valid[u]) copy_k[base + uint64_t(u) * THREADS + threadIdx.x] = k[u];
    }
    count(k, valid);
    if constexpr (HAS_V) {
      if (vd > 0 || copy_v) count_vals(base, valid);
    }
  }
  __syncthreads();
  uint32_t* g = &p.work->hist[0][0];
  for (uint32_t i = threadIdx.x; i < total_digits * RADIX; i += THREADS) {
    uint32_t c = 0;
#pragma unroll
    for (uint32_t j = 0; j < NC; ++j) c += s_hist[i * NC + ((j + i) & (NC - 1))];
    if (c) atomicAdd(&g[i], c);
  }
}

// ---------------------------------------------------------------------------
// One onesweep pass.
// ---------------------------------------------------------------------------
// Ranking of the stable passes (a pass-kernel template parameter):
//   RANK_TABLE - each lane sets its bit in the digit's peer mask in a
//                per-warp shared table, reads the mask back with the digit's
//                running count (one 64-bit word), and the group's lowest
//                lane advances the count: three shared accesses per element;
//   RANK_HALF  - the same with each 16-lane half of a warp ranking on its
//                own, so that a digit's peer mask (16 bits) and running
//                count (16 bits) share one 32-bit word: the accesses spread
//                over all 32 banks, where the 64-bit entries of RANK_TABLE
//                use 16 bank pairs. A half-warp's items are a contiguous run
//                of the input, so ranking half 0 before half 1 keeps input
//                order. Measured on GB300 (2^30 u32 keys): stable passes
//                3.97 ms vs 4.30 ms; shared-memory bank conflicts are what
//                bound the pass. Eight warp ballots per row instead of the
//                peer table halve the shared-memory wavefronts but triple
//                the ALU instructions and made the pass ALU-bound (4.51 ms).
//   RANK_UNSTABLE - the keys-only lowest-digit pass, which always ranks
//                unstably (one shared atomic per element): without the
//                stable rankings' code and tables the kernel keeps its
//                registers and leaves more of the SM's L1 as cache.
enum RankMode : int { RANK_TABLE = 0, RANK_UNSTABLE = 1, RANK_HALF = 2 };

template <typename K, typename V, int THREADS, int ITEMS, int RANK = RANK_TABLE>
struct PassConfig {
  static constexpr int WARPS = THREADS / 32;
  static constexpr int TILE = THREADS * ITEMS;
  static_assert(TILE <= 65536, "ranks are packed as 16-bit fields");
  static constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  static constexpr size_t VAL_BYTES = HAS_V ? sizeof(typename std::conditional<HAS_V, V, uint32_t>::type) : 0;
  static constexpr size_t SMEM_KEYS = size_t(TILE) * sizeof(K);
  static constexpr size_t SMEM_VALS = size_t(TILE) * VAL_BYTES;
  // Dynamic shared memory: the ranking table (per warp and digit: a 64-bit
  // mask and count for RANK_TABLE, two 32-bit ones for RANK_HALF) and the
  // reorder staging of the tile are never live at the same time, so they
  // share one region; the per-ranker digit offsets, live from the count
  // phase to the end of the reorder, follow it.
  // Items of one ranker (a warp, or a half-warp for RANK_HALF) are STRIDE
  // apart in the tile.
  static constexpr int STRIDE = RANK == RANK_HALF ? 16 : 32;
  static constexpr size_t TAB_BYTES =
      RANK == RANK_UNSTABLE ? size_t(RADIX) * sizeof(uint32_t)
      : RANK == RANK_TABLE  ? size_t(WARPS) * (RADIX + 1) * sizeof(uint64_t)
                            : ((size_t(WARPS) * (RADIX + 1) * 2 * sizeof(uint32_t) + 15) & ~size_t(15));
  static_assert(TAB_BYTES % 16 == 0, "the table is cleared in 16-byte units");
  static constexpr size_t STAGE_BYTES = SMEM_KEYS + SMEM_VALS;
  static constexpr size_t UNION_BYTES = ((STAGE_BYTES > TAB_BYTES ? STAGE_BYTES : TAB_BYTES) + 15) & ~size_t(15);
  // Per warp and digit: a 16-bit tile offset, or (RANK_HALF) two, one per
  // half, in one 32-bit word.
  using OffT = typename std::conditional<RANK == RANK_HALF, uint32_t, uint16_t>::type;
  static constexpr size_t OFF_BYTES = size_t(RANK == RANK_UNSTABLE ? 1 : WARPS) * RADIX * sizeof(OffT);
  static constexpr size_t DYN_SMEM = UNION_BYTES + OFF_BYTES;
  // BUCKET mode also stages each element's bucket (one byte) for the scatter.
  static constexpr size_t DYN_SMEM_BUCKET = DYN_SMEM + size_t(TILE);
};

// Splitter search tree: the nsplit sorted splitters as a complete binary
// search tree of `levels` = ceil(log2(nsplit + 1)) levels in breadth-first
// order (node v at tree[v], children 2v and 2v + 1, v = 1 .. 2^levels - 1),
// slots past the last splitter holding the largest key. A search is one
// shared load, one compare and one shift-add per level, the same for every
// lane. nsplit < 256, so tree has room for 256 entries.
__host__ __device__ __forceinline__ uint32_t tree_levels(uint32_t nsplit) {
  uint32_t l = 0;
  while ((1u << l) - 1u < nsplit) ++l;
  return l;
}

// Fill tree[1 .. 2^levels) from sorted[0 .. nsplit), by all threads of the
// block (the caller synchronises afterwards). Node v on level L (v = 2^L +
// j) holds in-order element (2j + 1) * 2^(levels - L - 1) - 1.
template <typename K>
__device__ __forceinline__ void build_split_tree(const K* sorted, uint32_t nsplit, K* tree,
                                                 uint32_t levels) {
  const uint32_t nodes = (1u << levels) - 1u;
  for (uint32_t v = threadIdx.x + 1; v <= nodes; v += blockDim.x) {
    const uint32_t L = 31u - __clz(v);
    const uint32_t j = v - (1u << L);
    const uint32_t r = ((2u * j + 1u) << (levels - L - 1u)) - 1u;
    tree[v] = r < nsplit ? sorted[r] : ~K(0);
  }
}

// Number of splitters <= y (upper_bound), i.e. y's bucket among nsplit + 1.
template <typename K>
__device__ __forceinline__ uint32_t tree_bucket(const K* tree, uint32_t levels, uint32_t nsplit,
                                                K y) {
  uint32_t v = 1;
  for (uint32_t l = 0; l < levels; ++l) v = 2u * v + (tree[v] <= y ? 1u : 0u);
  const uint32_t b = v - (1u << levels);
  return b < nsplit ? b : nsplit;  // padding slots equal to y == ~0 count past the end
}

// Keys live in the transformed domain between passes: the first pass that
// runs transforms them on load, the last one restores raw bits on store.
// Values stay raw and are transformed only to extract a value digit.
template <typename K, typename V, int THREADS, int ITEMS, int MIN_BLOCKS, int RANK = RANK_TABLE,
          bool BUCKET = false, bool SEG = false>
__global__ void __launch_bounds__(THREADS, MIN_BLOCKS)
pass_kernel(PassParams p) {
  using Cfg = PassConfig<K, V, THREADS, ITEMS, RANK>;
  constexpr int WARPS = Cfg::WARPS;
  constexpr int TILE = Cfg::TILE;
  constexpr int STRIDE = Cfg::STRIDE;
  using OffT = typename Cfg::OffT;
  constexpr bool HAS_V = Cfg::HAS_V;
  constexpr int LB_WIN = 4;         // look-back words read per round
  constexpr int LB_SLEEP_NS = 128;  // pause after a round without progress
  using VS = typename std::conditional<HAS_V, V, uint32_t>::type;  // storage type

  extern __shared__ __align__(16) uint8_t s_dyn[];
  // Ranking table, in the region the reorder stages the tile in later.
  // RANK_TABLE: per warp and digit, the peer mask of the current item row
  // and the running count (mask in the low half for even digits, in the
  // high half for odd ones). The unstable ranking uses the first RADIX
  // 32-bit words as tile counters.
  uint64_t (*const s_tab)[RADIX + 1] = reinterpret_cast<uint64_t (*)[RADIX + 1]>(s_dyn);
  // RANK_HALF: per warp, digit and half: peer mask (low 16 bits) and
  // running count (high 16 bits).
  uint32_t (*const s_htab)[RADIX + 1][2] = reinterpret_cast<uint32_t (*)[RADIX + 1][2]>(s_dyn);
  // Per warp and digit: the ranker's start of the digit in the tile (stable
  // ranking; RANK_HALF: half 0 in the low 16 bits, half 1 in the high 16);
  // row 0 holds the tile offsets of the unstable ranking. 16-bit fields
  // (offsets are below the tile size, at most 65536): less shared memory
  // per CTA measured faster (2^30 u32 keys: 17.30 vs 17.61 ms).
  OffT (*const s_offd)[RADIX] = reinterpret_cast<OffT (*)[RADIX]>(s_dyn + Cfg::UNION_BYTES);
  __shared__ uint32_t s_dst_base[RADIX];
  __shared__ uint32_t s_excl[RADIX];  // the tile's exclusive digit offsets
  __shared__ uint32_t s_tmp[8];
  __shared__ uint32_t s_tile;
  __shared__ uint32_t s_bad;  // a digit's destination range leaves the output
  __shared__ K s_split[BUCKET ? RADIX : 1];  // bucket mode: splitter search tree

  SortPlan& plan = p.work->plan;
  const uint32_t j = plan.exec_index[p.pass];
  if (j == PASS_SKIPPED) return;
  if (RANK == RANK_UNSTABLE && !(j == 0 && p.first_unstable && !plan.first_stable)) {
    if (threadIdx.x == 0) atomicOr(p.err, ERR_PASS_KIND);
    return;
  }
  const uint32_t m = plan.m_exec;
  const uint32_t gen = (plan.gen_base + p.pass + 1) & GEN_MASK;  // this pass's look-back tag
  const bool first = (j == 0);
  const bool last = (j + 1 == m);

  // Ping-pong: pass j writes `out` when (m - j) is odd, so the last pass
  // always lands in `out`; pass 0 reads the caller's input.
  const bool dst_is_out = ((m - j) & 1u) != 0;
  const K* src_k;
  const VS* src_v = nullptr;
  if (first) {
    src_k = static_cast<const K*>(p.keys_in);
    if constexpr (HAS_V) src_v = static_cast<const VS*>(p.vals_in);
  } else {
    src_k = static_cast<const K*>(dst_is_out ? p.keys_alt : p.keys_out);
    if constexpr (HAS_V) src_v = static_cast<const VS*>(dst_is_out ? p.vals_alt : p.vals_out);
  }
  K* dst_k = static_cast<K*>(dst_is_out ? p.keys_out : p.keys_alt);
  VS* dst_v = nullptr;
  if constexpr (HAS_V) dst_v = static_cast<VS*>(dst_is_out ? p.vals_out : p.vals_alt);
  const bool reverse = first && (p.reverse_first || plan.first_reverse);
  // The first pass that runs may order equal digits arbitrarily when the
  // requested order leaves no ties to preserve (keys only, or pairs ordered
  // by value too): equal digits there are either equal in every later digit
  // (identical elements) or separated by a later, stable pass.
  const bool unstable = RANK == RANK_UNSTABLE || (first && p.first_unstable && !plan.first_stable);

  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  const uint64_t n = p.n;
  const bool from_val = p.pass < p.val_digits;
  const uint32_t shift = RADIX_BITS * (from_val ? p.pass : (p.pass - p.val_digits));
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const OrderXform<VS> vx(p.val_kind, p.desc != 0);

  // L2 prefetch of the elements prefetch_tiles tiles further on, which a
  // CTA claims about when this one finishes (segmented sorts: the same
  // distance in elements, a hint that may cross into later segments).
  auto prefetch_from = [&](uint64_t b) {
    if (b < n) {
      const uint64_t c = n - b < uint64_t(TILE) ? n - b : uint64_t(TILE);
      auto pf = [](const void* a, uint64_t bytes) {
        bytes &= ~uint64_t(15);
        if ((reinterpret_cast<uintptr_t>(a) & 15u) == 0 && bytes != 0) prefetch_l2_bulk(a, uint32_t(bytes));
      };
      pf(src_k + b, c * sizeof(K));
      if constexpr (HAS_V) pf(src_v + b, c * sizeof(VS));
    }
  };
  // Tiles are claimed in launch order, so a tile only ever waits on tiles
  // held by CTAs that are already running.
  if (tid == 0) {
    const uint32_t t = atomicAdd(&plan.tile_counter[p.pass], 1u);
    s_tile = t;
    s_bad = 0;
    if (!SEG && p.prefetch_tiles != 0 && !reverse)
      prefetch_from((uint64_t(t) + p.prefetch_tiles) * TILE);
  }
  if ((smem_addr(s_dyn) & 15u) == 0) {
    uint4* z = reinterpret_cast<uint4*>(s_dyn);
    // The unstable ranking uses only the first RADIX words: the
    // RANK_UNSTABLE kernel clears only those, and so do the keys-only table
    // kernels when they rank a sort's first pass unstably (the same branch
    // costs the other kernels registers).
    if (RANK == RANK_UNSTABLE || (!HAS_V && RANK == RANK_TABLE && unstable)) {
      if (tid < RADIX / 4) z[tid] = make_uint4(0, 0, 0, 0);
    } else {
      constexpr int Z = int(Cfg::TAB_BYTES / 16);
      for (int i = tid; i < Z; i += THREADS) z[i] = make_uint4(0, 0, 0, 0);
    }
  } else {  // not expected (the region is declared 16-byte aligned)
    uint32_t* z = reinterpret_cast<uint32_t*>(s_dyn);
    for (int i = tid; i < int(Cfg::TAB_BYTES / 4); i += THREADS) z[i] = 0u;
    if (tid == 0) atomicOr(p.err, ERR_SMEM_ALIGN);
  }
  __syncthreads();
  const uint32_t tile = s_tile;
  // Batched sorts: the tile's segment, its element range and its first
  // tile, where the segment's look-back chain starts.
  uint32_t seg = 0, first_unit = 0;
  uint64_t e0 = 0, e1 = n;
  uint64_t tile_base;
  uint32_t tile_n;
  if constexpr (SEG) {
    const SegTile d = p.seg_tiles[tile];
    seg = d.seg;
    tile_base = d.base;
    tile_n = d.n;
    first_unit = p.seg_tile_start[seg];
    e0 = p.seg_range[2 * seg];
    e1 = p.seg_range[2 * seg + 1];
    if (tid == 0 && p.prefetch_tiles != 0 && !reverse)
      prefetch_from(tile_base + uint64_t(p.prefetch_tiles) * TILE);
  } else {
    tile_base = uint64_t(tile) * TILE;
    tile_n = tile_base >= n ? 0u : uint32_t(n - tile_base < uint64_t(TILE) ? n - tile_base : uint64_t(TILE));
  }
  // Tile index of item 0; item i is STRIDE further. RANK_HALF: lanes 0-15
  // and 16-31 of a warp hold two consecutive runs of 16 * ITEMS elements.
  const uint32_t ranker = RANK == RANK_HALF ? uint32_t(2 * warp + (lane >> 4)) : uint32_t(warp);
  const uint32_t wloc = ranker * STRIDE * ITEMS + uint32_t(lane & (STRIDE - 1));
  const uint32_t nsplit = p.nsplit;
  const uint32_t split_levels = BUCKET ? tree_levels(nsplit) : 0u;
  if constexpr (BUCKET) {
    build_split_tree(static_cast<const K*>(p.splitters), nsplit, s_split, tree_levels(nsplit));
    __syncthreads();
  }
  // Pair sorts order keys as std::less does, under which -0.0 and +0.0 are
  // equal: the digits of -0.0 are taken from +0.0, so the two tie by value
  // (or input order). Keys themselves keep their bits. Keys-only sorts put
  // -0.0 first, one of the orders std::less allows.
  K zneg = 0, zpos = 0;
  if constexpr (HAS_V) {
    zneg = kx.neg_zero();
    zpos = kx.pos_zero();
  }
  // Digit of order bits: a radix digit, or the bucket (upper_bound).
  auto key_digit = [&](K y) -> uint32_t {
    if constexpr (HAS_V) y = y == zneg ? zpos : y;
    if constexpr (!BUCKET) return uint32_t(y >> shift) & (RADIX - 1);
    return tree_bucket(s_split, split_levels, nsplit, y);
  };

  // The tile's work; FULL tiles (all but a pass's last, and a segment's
  // last) need no per-element bounds checks.
  auto body = [&](auto full_c) {
    constexpr bool FULL = decltype(full_c)::value;
    auto in_tile = [&](uint32_t idx) -> bool { return FULL || idx < tile_n; };

    // Load: item i of lane l is tile element wloc + STRIDE*i, so (ranker,
    // i, lane) order is input order and the stable ranking below keeps it.
    K keys[ITEMS];
    VS vals[HAS_V ? ITEMS : 1];
    if (!reverse) {
      const K* sk = src_k + tile_base + wloc;
      const VS* sv = nullptr;
      if constexpr (HAS_V) sv = src_v + tile_base + wloc;
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const bool valid = in_tile(wloc + STRIDE * i);
        keys[i] = valid ? ld_stream(sk + STRIDE * i) : K(0);
        if constexpr (HAS_V) vals[i] = valid ? ld_stream(sv + STRIDE * i) : VS(0);
      }
    } else {
      const K* sk = src_k + (n - 1 - tile_base - wloc);
      const VS* sv = nullptr;
      if constexpr (HAS_V) sv = src_v + (n - 1 - tile_base - wloc);
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const bool valid = in_tile(wloc + STRIDE * i);
        keys[i] = valid ? ld_stream(sk - STRIDE * i) : K(0);
        if constexpr (HAS_V) vals[i] = valid ? ld_stream(sv - STRIDE * i) : VS(0);
      }
    }
    if (first) {
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) keys[i] = kx.fwd(keys[i]);
    }
    // BUCKET mode: each item's bucket is searched once and kept, one byte each.
    uint32_t bdig[BUCKET ? (ITEMS + 3) / 4 : 1];
    if constexpr (BUCKET) {
#pragma unroll
      for (int i = 0; i < (ITEMS + 3) / 4; ++i) bdig[i] = 0;
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
        if (in_tile(wloc + STRIDE * i)) bdig[i >> 2] |= key_digit(keys[i]) << (8 * (i & 3));
    }
    auto digit_at = [&](int i) -> uint32_t {
      if constexpr (BUCKET) return (bdig[i >> 2] >> (8 * (i & 3))) & 0xFFu;
      if constexpr (HAS_V) {
        if (from_val) return uint32_t(vx.fwd(vals[i]) >> shift) & (RADIX - 1);
      }
      return key_digit(keys[i]);
    };

    // Ranks are below the tile size (< 2^16): two per register.
    uint32_t rank2[(ITEMS + 1) / 2];
#pragma unroll
    for (int i = 0; i < (ITEMS + 1) / 2; ++i) rank2[i] = 0;
    auto set_rank = [&](int i, uint32_t r) { rank2[i >> 1] |= r << (16 * (i & 1)); };
    auto get_rank = [&](int i) -> uint32_t { return (rank2[i >> 1] >> (16 * (i & 1))) & 0xFFFFu; };

    uint32_t* s_cnt = reinterpret_cast<uint32_t*>(s_dyn);
    if constexpr (RANK == RANK_UNSTABLE) {
      // The tile's digit counts; each element takes its place in the
      // reorder below, by one more atomic on the digit's running offset.
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        if (in_tile(wloc + STRIDE * i)) atomicAdd(&s_cnt[digit_at(i)], 1u);
      }
    } else if (unstable) {
      // One shared atomic per element: its rank among the tile's elements of
      // the same digit, in no particular order.
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        if (in_tile(wloc + STRIDE * i)) set_rank(i, atomicAdd(&s_cnt[digit_at(i)], 1u));
      }
    } else if constexpr (RANK == RANK_HALF) {
      // Stable half-warp ranking: as below, with a 32-bit word per digit and
      // half (16-bit peer mask, 16-bit count); a half-warp's count of one
      // digit is at most 16 * ITEMS.
      static_assert(16 * ITEMS < 65536, "half-warp counts are 16-bit");
      const uint32_t h = uint32_t(lane) >> 4;
      const uint32_t sl = uint32_t(lane) & 15u;
      const uint32_t lt = (1u << sl) - 1u;
      const uint32_t bit = 1u << sl;
      uint32_t (*tab)[2] = s_htab[warp];
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const uint32_t d = in_tile(wloc + STRIDE * i) ? digit_at(i) : uint32_t(RADIX);
        uint32_t* e = &tab[d][h];
        atomicOr(e, bit);
        __syncwarp();
        const uint32_t w = *e;
        __syncwarp();
        const uint32_t peers = w & 0xFFFFu;
        const uint32_t base = w >> 16;
        const uint32_t below = peers & lt;
        set_rank(i, base + __popc(below));
        if (below == 0) *e = (base + __popc(peers)) << 16;
        __syncwarp();
      }
    } else if constexpr (RANK == RANK_TABLE) {
      // Stable warp ranking: each lane sets its bit in the digit's peer mask,
      // reads back the mask and the digit's running count; the group's lowest
      // lane advances the count and clears the mask.
      // Odd digits keep the mask in the high half and the count in the low
      // half.
      const uint32_t lt = lanemask_lt();
      const uint32_t bit = 1u << lane;
      uint64_t* tab = s_tab[warp];
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const uint32_t d = in_tile(wloc + STRIDE * i) ? digit_at(i) : uint32_t(RADIX);
        const uint32_t odd = d & 1u;
        atomicOr(reinterpret_cast<uint32_t*>(&tab[d]) + odd, bit);
        __syncwarp();
        const uint64_t e = tab[d];
        __syncwarp();
        const uint32_t lo = uint32_t(e), hi = uint32_t(e >> 32);
        const uint32_t peers = odd ? hi : lo;
        const uint32_t base = odd ? lo : hi;
        const uint32_t below = peers & lt;
        set_rank(i, base + __popc(below));
        if (below == 0) {
          const uint64_t c = base + __popc(peers);
          tab[d] = odd ? c : (c << 32);
        }
        __syncwarp();
      }
    }
    __syncthreads();

    // Counts of digit d of warp w's rankers (one 64-bit word either way).
    auto ranker_counts = [&](int w, uint32_t d, uint32_t& c0, uint32_t& c1) {
      if constexpr (RANK == RANK_HALF) {
        const uint2 e = *reinterpret_cast<const uint2*>(&s_htab[w][d][0]);
        c0 = e.x >> 16;
        c1 = e.y >> 16;
      } else {
        const uint64_t e = s_tab[w][d];
        c0 = (d & 1u) ? uint32_t(e) : uint32_t(e >> 32);
        c1 = 0;
      }
    };
    // Per digit: the tile's count.
    uint32_t count = 0;
    if (tid < RADIX) {
      if (unstable) {
        count = s_cnt[tid];
      } else {
#pragma unroll
        for (int w = 0; w < WARPS; ++w) {
          uint32_t c0, c1;
          ranker_counts(w, tid, c0, c1);
          count += c0 + c1;
        }
      }
    }
    uint64_t* status = p.status + uint64_t(tile) * RADIX;
    if (tid < RADIX) {
      st_relaxed(status + tid,
                 make_status(tile == first_unit ? FLAG_INC : FLAG_AGG, gen, count));
    }
    const uint32_t tile_excl = block_excl_scan_256(count, s_tmp, s_excl);

    // Per warp and digit: where the ranker's elements of the digit start in
    // the reordered tile.
    // (The unstable-only kernel places elements by running offsets instead.)
    if constexpr (RANK != RANK_UNSTABLE) {
      if (tid < RADIX) {
        const uint32_t d = uint32_t(tid);
        uint32_t run = tile_excl;
        if (unstable) {
          s_offd[0][d] = OffT(RANK == RANK_HALF ? (run | (run << 16)) : run);
        } else {
#pragma unroll
          for (int w = 0; w < WARPS; ++w) {
            uint32_t c0, c1;
            ranker_counts(w, d, c0, c1);
            s_offd[w][d] = OffT(RANK == RANK_HALF ? (run | ((run + c0) << 16)) : run);
            run += c0 + c1;
          }
        }
      }
    }

    // Decoupled look-back over preceding tiles, LB_WIN words per round,
    // bounded by spin_limit rounds without progress. While the nearest word
    // is pending, one word is polled per round after a short sleep, so
    // waiting warps leave issue slots and L1 bandwidth to the tiles they
    // wait for.
    auto lookback = [&]() {
    uint32_t prefix = 0;
    if (tid < RADIX) {
      if (tile > first_unit) {
        int64_t t = int64_t(tile) - 1;
        uint32_t idle_rounds = 0;
        const bool stall = p.inject_stall && tile == 1;
        int win = LB_WIN;
        while (true) {
          uint64_t w[LB_WIN];
#pragma unroll
          for (int k = 0; k < LB_WIN; ++k) {
            const int64_t tt = t - k;
            w[k] = (k < win && tt >= 0 && !stall) ? ld_relaxed(p.status + uint64_t(tt) * RADIX + tid)
                                                  : 0ull;
          }
          int consumed = 0;
          bool done = false;
#pragma unroll
          for (int k = 0; k < LB_WIN; ++k) {
            const uint64_t wk = w[k];
            const bool ready = (wk & FLAG_MASK) != 0 && uint32_t((wk >> 32) & GEN_MASK) == gen;
            if (!done && consumed == k && ready) {
              prefix += uint32_t(wk);
              consumed = k + 1;
              done = (wk & FLAG_MASK) == FLAG_INC;
            }
          }
          if (done) break;
          t -= consumed;
          if (consumed == 0) {
            if (++idle_rounds > p.spin_limit) {
              atomicOr(p.err, ERR_LOOKBACK_TIMEOUT);
              break;
            }
            __nanosleep(LB_SLEEP_NS);
            win = 1;
          } else {
            win = LB_WIN;
          }
        }
        st_relaxed(status + tid, make_status(FLAG_INC, gen, prefix + count));
      }
      const uint32_t bb = p.seg_binbase != nullptr
                              ? p.seg_binbase[(size_t(seg) * p.seg_digits + p.pass) * RADIX + tid]
                              : plan.binbase[p.pass][tid];
      s_dst_base[tid] = uint32_t(e0) + bb + prefix - tile_excl;
      // This tile writes the digit's elements to [e0 + bb + prefix, + count):
      // the range is checked once per digit, not per element.
      if (count != 0 && uint64_t(e0) + bb + prefix + count > e1) {
        s_bad = 1;
        atomicOr(p.err, ERR_SCATTER_RANGE);
      }
    }
    };

    // Reorder the tile in shared memory by digit (keys in transformed form).
    K* s_keys = reinterpret_cast<K*>(s_dyn);
    VS* s_vals = reinterpret_cast<VS*>(s_dyn + Cfg::SMEM_KEYS);
    uint8_t* s_bdig = s_dyn + Cfg::DYN_SMEM;  // BUCKET mode only
    auto reorder = [&]() {
      const OffT* s_off = s_offd[unstable ? 0 : warp];
      const uint32_t hsh = RANK == RANK_HALF ? 16u * (uint32_t(lane) >> 4) : 0u;
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        if (in_tile(wloc + STRIDE * i)) {
          const uint32_t d = digit_at(i);
          uint32_t pos;
          if constexpr (RANK == RANK_UNSTABLE) pos = atomicAdd(&s_excl[d], 1u);
          else pos = ((uint32_t(s_off[d]) >> hsh) & 0xFFFFu) + get_rank(i);
          s_keys[pos] = keys[i];
          if constexpr (HAS_V) s_vals[pos] = vals[i];
          if constexpr (BUCKET) s_bdig[pos] = uint8_t(d);
        }
      }
    };
    // The reorder needs only the tile's own offsets, so it runs before the
    // look-back, which then finds more of the preceding tiles done (2^30 u32
    // keys: stable passes 3.58 -> 3.54 ms against the look-back first).
    __syncthreads();
    reorder();
    lookback();
    __syncthreads();

    // Scatter: consecutive tile positions of one digit go to consecutive
    // output addresses. A tile that failed the range check writes nothing.
    auto scatter = [&](auto last_c) {
      constexpr bool LAST = decltype(last_c)::value;
      if (s_bad) return;
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const uint32_t r = uint32_t(i) * THREADS + tid;
        if (in_tile(r)) {
          const K k = s_keys[r];
          uint32_t d;
          VS v;
          if constexpr (HAS_V) {
            v = s_vals[r];
            d = from_val ? (uint32_t(vx.fwd(v) >> shift) & (RADIX - 1)) : key_digit(k);
          } else if constexpr (BUCKET) {
            d = s_bdig[r];
          } else {
            d = key_digit(k);
          }
          const uint32_t dst = s_dst_base[d] + r;
          dst_k[dst] = LAST ? kx.inv(k) : k;
          if constexpr (HAS_V) dst_v[dst] = v;
        }
      }
    };
    if (last) scatter(std::true_type{});
    else scatter(std::false_type{});
  };
  if (tile_n == uint32_t(TILE)) body(std::true_type{});
  else body(std::false_type{});
}

}  // namespace gs
