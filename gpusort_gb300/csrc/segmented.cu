// Batched sorting of many independent segments (gs_segmented_sort_keys and
// the plan/run pair used for CUDA-graph capture).
//
// Each segment is sorted on its own, as one rank's local sort of the
// reference would be (include/omp/omp_utils.h:147-207). Two kernels share
// the work:
// * group_sort_kernel: segments of at most GROUP_KEYS keys are packed, in
//   order, into groups of consecutive segments; one CTA loads a group into
//   shared memory and radix-sorts it by (local segment id, key) - an LSD
//   sort over the key's digits and then the segment id - and writes it back
//   in place of the group;
// * tiny_sort_kernel: a group made only of segments of at most 32 keys is
//   not radix-sorted; each of its segments is sorted by one warp with a
//   bitonic network in registers (one key per lane, 15 compare-exchange
//   stages by shuffles), so a 16-key segment no longer pays for LSD passes
//   over a shared 4096-key tile;
// * the onesweep pass kernel (radix.cuh) in its segmented form for larger
//   segments: tiles never straddle segments, each segment has its own bin
//   bases, and each segment's first tile starts its own look-back chain.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gpusort_gb300.h"
#include "engine.h"
#include "radix.cuh"

namespace gs {

constexpr int GROUP_THREADS = 256;
constexpr int GROUP_ITEMS = 16;
constexpr uint32_t GROUP_KEYS = GROUP_THREADS * GROUP_ITEMS;  // 4096
constexpr uint32_t GROUP_MAX_SEGS = 256;                     // segment id is one digit

struct SegGroup {
  uint64_t start;      // first element of the group
  uint32_t count;      // elements in the group (<= GROUP_KEYS)
  uint32_t first_seg;  // index of its first segment in seg_starts_rel
  uint32_t nsegs;      // segments in the group (<= GROUP_MAX_SEGS)
  uint32_t pad;
};

constexpr uint32_t TINY_KEYS = 32;  // one key per lane of a warp

struct TinySeg {
  uint64_t start;
  uint32_t len;  // 1 .. TINY_KEYS
  uint32_t pad;
};

// One warp per segment of at most 32 keys: lane l holds key l (or the
// largest order bits as padding) and a bitonic network sorts the warp's
// keys by shuffles; `in` may equal `out` (every lane reads before any
// writes).
template <typename K>
__global__ void __launch_bounds__(256) tiny_sort_kernel(const void* in_, void* out_,
                                                        const TinySeg* segs, uint32_t nseg,
                                                        uint32_t key_kind, uint32_t desc) {
  const uint32_t w = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (w >= nseg) return;  // whole warps leave together
  const uint32_t lane = threadIdx.x & 31;
  const TinySeg sg = segs[w];
  const OrderXform<K> kx(key_kind, desc != 0);
  const K* in = static_cast<const K*>(in_) + sg.start;
  K x = lane < sg.len ? kx.fwd(in[lane]) : ~K(0);
#pragma unroll
  for (uint32_t k = 2; k <= 32; k <<= 1) {
#pragma unroll
    for (uint32_t j = k >> 1; j > 0; j >>= 1) {
      const K y = __shfl_xor_sync(0xFFFFFFFFu, x, j);
      const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
      x = keep_min ? (y < x ? y : x) : (y < x ? x : y);
    }
  }
  if (lane < sg.len) static_cast<K*>(out_)[sg.start + lane] = kx.inv(x);
}

struct GroupSortParams {
  const void* in;
  void* out;
  const SegGroup* groups;          // null: one group of single_count elements
  const uint32_t* seg_starts_rel;  // per group: nsegs + 1 offsets relative to start
  uint32_t key_kind;
  uint32_t desc;
  uint32_t single_count;
  const SmallSortReq* reqs;        // set: CTA b sorts the independent array reqs[b]
};

// One CTA sorts one group in shared memory: LSD passes over the key's
// digits, then one pass over the local segment id when the group holds
// several segments. The first key pass ranks unstably (a digit count per
// key, then an atomic on the digit's running offset places it): equal
// digits there are either equal keys of one segment, which cannot be told
// apart, or are ordered by a later pass. The later passes rank stably with
// per-half-warp peer masks (16-bit mask and 16-bit count in one word), as
// the pass kernel's half-warp ranking does; a half-warp's items are a
// contiguous run of the group.
//
// Shared memory: two buffer sets {keys, 8-bit segment ids} (the source and
// the destination of a pass), then per-warp digit offsets (both halves'
// in one word). The ranking table of a stable pass lives in the
// destination set, which the pass writes only after the table's counts
// became offsets. 32-bit keys: 48 KB, four CTAs per SM.
template <typename K>
__host__ __device__ constexpr size_t group_set_bytes() {
  return (size_t(GROUP_KEYS) * (sizeof(K) + 1) + 15) & ~size_t(15);
}
constexpr size_t GROUP_OFF_BYTES = size_t(GROUP_THREADS / 32) * RADIX * sizeof(uint32_t);

template <typename K>
__global__ void __launch_bounds__(GROUP_THREADS)
group_sort_kernel(GroupSortParams p) {
  constexpr int THREADS = GROUP_THREADS;
  constexpr int ITEMS = GROUP_ITEMS;
  constexpr int WARPS = THREADS / 32;
  constexpr int TILE = GROUP_KEYS;
  constexpr size_t SET = group_set_bytes<K>();
  static_assert(size_t(WARPS) * (RADIX + 1) * 2 * sizeof(uint32_t) <= SET, "table fits a buffer set");
  static_assert(16 * ITEMS < 65536, "half-warp counts are 16-bit");
  static_assert(GROUP_MAX_SEGS <= 256, "segment ids are one byte");
  extern __shared__ __align__(16) uint8_t s_dyn[];
  auto set_keys = [&](int b) { return reinterpret_cast<K*>(s_dyn + b * SET); };
  auto set_sid = [&](int b) { return s_dyn + b * SET + size_t(TILE) * sizeof(K); };
  uint32_t (*const s_off)[RADIX] = reinterpret_cast<uint32_t (*)[RADIX]>(s_dyn + 2 * SET);
  uint32_t* const s_cnt = reinterpret_cast<uint32_t*>(s_dyn + 2 * SET);  // unstable pass
  __shared__ uint32_t s_sstart[GROUP_MAX_SEGS + 1];
  __shared__ uint32_t s_tmp[8];

  const SmallSortReq* rq = p.reqs ? p.reqs + blockIdx.x : nullptr;
  const SegGroup g = rq ? SegGroup{0, rq->n, 0, 1, 0}
                   : p.groups ? p.groups[blockIdx.x] : SegGroup{0, p.single_count, 0, 1, 0};
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const OrderXform<K> kx(rq ? rq->kind : p.key_kind, (rq ? rq->desc : p.desc) != 0);
  const K* in = static_cast<const K*>(rq ? rq->in : p.in) + g.start;
  K* out = static_cast<K*>(rq ? rq->out : p.out) + g.start;
  const uint32_t cnt = g.count;
  for (uint32_t i = tid; i <= g.nsegs; i += THREADS)
    s_sstart[i] = p.groups ? p.seg_starts_rel[g.first_seg + i] : (i == 0 ? 0u : cnt);
  __syncthreads();
  // Load (transformed) keys and local segment ids into set 0.
  {
    K* k0 = set_keys(0);
    uint8_t* d0 = set_sid(0);
    for (uint32_t i = tid; i < cnt; i += THREADS) {
      k0[i] = kx.fwd(in[i]);
      uint32_t lo = 0, hi = g.nsegs;  // last s with s_sstart[s] <= i
      while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_sstart[mid] <= i) lo = mid; else hi = mid;
      }
      d0[i] = uint8_t(lo);
    }
  }
  // Item i of lane l is element wloc + 16 i: lanes 0-15 and 16-31 of a
  // warp hold two consecutive runs of 16 * ITEMS elements.
  const uint32_t h = uint32_t(lane) >> 4;
  const uint32_t wloc = (2 * uint32_t(warp) + h) * 16 * ITEMS + (uint32_t(lane) & 15u);
  const uint32_t lt = (1u << (uint32_t(lane) & 15u)) - 1u;
  const uint32_t bit = 1u << (uint32_t(lane) & 15u);
  const int key_digits = int(sizeof(K));
  const int passes = key_digits + (g.nsegs > 1 ? 1 : 0);
  int cur = 0;
  for (int q = 0; q < passes; ++q) {
    const bool sid_pass = q == key_digits;
    const bool unstable = q == 0;
    const uint32_t shift = RADIX_BITS * uint32_t(q);
    const K* src_k = set_keys(cur);
    const uint8_t* src_s = set_sid(cur);
    K* dst_k = set_keys(cur ^ 1);
    uint8_t* dst_s = set_sid(cur ^ 1);
    uint32_t (*const tab)[RADIX + 1][2] = reinterpret_cast<uint32_t (*)[RADIX + 1][2]>(s_dyn + (cur ^ 1) * SET);
    if (unstable) {
      if (tid < RADIX) s_cnt[tid] = 0u;
    } else {
      uint64_t* z = reinterpret_cast<uint64_t*>(&tab[0][0][0]);
      for (int i = tid; i < WARPS * (RADIX + 1); i += THREADS) z[i] = 0ull;
    }
    __syncthreads();
    K keys[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const uint32_t l = wloc + 16 * i;
      keys[i] = l < cnt ? src_k[l] : K(0);
    }
    auto digit_at = [&](int i) -> uint32_t {
      return sid_pass ? uint32_t(src_s[wloc + 16 * i]) : (uint32_t(keys[i] >> shift) & (RADIX - 1));
    };
    if (unstable) {
#pragma unroll
      for (int i = 0; i < ITEMS; ++i)
        if (wloc + 16 * i < cnt) atomicAdd(&s_cnt[digit_at(i)], 1u);
      __syncthreads();
      const uint32_t c = tid < RADIX ? s_cnt[tid] : 0u;
      const uint32_t excl = block_excl_scan_256(c, s_tmp);
      if (tid < RADIX) s_cnt[tid] = excl;  // the digit's running offset
      __syncthreads();
#pragma unroll
      for (int i = 0; i < ITEMS; ++i) {
        const uint32_t l = wloc + 16 * i;
        if (l < cnt) {
          const uint32_t pos = atomicAdd(&s_cnt[digit_at(i)], 1u);
          dst_k[pos] = keys[i];
          dst_s[pos] = src_s[l];
        }
      }
      __syncthreads();
      cur ^= 1;
      continue;
    }
    uint32_t rank2[ITEMS / 2];
#pragma unroll
    for (int i = 0; i < ITEMS / 2; ++i) rank2[i] = 0;
    uint32_t (*const wt)[2] = tab[warp];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const uint32_t d = (wloc + 16 * i < cnt) ? digit_at(i) : uint32_t(RADIX);
      uint32_t* e = &wt[d][h];
      atomicOr(e, bit);
      __syncwarp();
      const uint32_t w = *e;
      __syncwarp();
      const uint32_t peers = w & 0xFFFFu, below = peers & lt, base = w >> 16;
      rank2[i >> 1] |= (base + __popc(below)) << (16 * (i & 1));
      if (below == 0) *e = (base + __popc(peers)) << 16;
      __syncwarp();
    }
    __syncthreads();
    uint32_t count = 0;
    if (tid < RADIX) {
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint2 c = *reinterpret_cast<const uint2*>(&tab[w][tid][0]);
        count += (c.x >> 16) + (c.y >> 16);
      }
    }
    const uint32_t excl = block_excl_scan_256(count, s_tmp);
    if (tid < RADIX) {
      uint32_t run = excl;
#pragma unroll
      for (int w = 0; w < WARPS; ++w) {
        const uint2 c = *reinterpret_cast<const uint2*>(&tab[w][tid][0]);
        const uint32_t c0 = c.x >> 16, c1 = c.y >> 16;
        s_off[w][tid] = run | ((run + c0) << 16);
        run += c0 + c1;
      }
    }
    __syncthreads();  // the table's counts are read: the destination set is free
    const uint32_t* off = s_off[warp];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
      const uint32_t l = wloc + 16 * i;
      if (l < cnt) {
        const uint32_t pos = ((off[digit_at(i)] >> (16 * h)) & 0xFFFFu) + ((rank2[i >> 1] >> (16 * (i & 1))) & 0xFFFFu);
        dst_k[pos] = keys[i];
        dst_s[pos] = src_s[l];
      }
    }
    __syncthreads();
    cur ^= 1;
  }
  const K* res = set_keys(cur);
  for (uint32_t i = tid; i < cnt; i += THREADS) out[i] = kx.inv(res[i]);
}

template <typename K>
constexpr size_t group_sort_dyn_smem() {
  return 2 * group_set_bytes<K>() + GROUP_OFF_BYTES;
}

// Histograms of every digit, per large segment.
struct SegHistParams {
  const void* keys;
  const uint32_t* seg_tile_start;
  const uint64_t* seg_range;
  uint32_t nseg;
  uint32_t tile;        // elements per tile (the pass kernel's)
  uint32_t total_tiles;
  uint32_t key_kind;
  uint32_t desc;
  uint32_t* hist;       // [nseg][digits][RADIX]
};

// One 1024-thread CTA per SM takes a contiguous run of tiles and, for each
// segment the run meets, counts that segment's keys in the run (16-byte
// loads between the range's 16-byte boundaries) into shared memory, then
// adds the counts to the segment's histogram. Every bin has one column per
// lane for 32-bit keys (16 for 64-bit keys), as in the upsweep, so a
// warp's atomics to random bins do not share banks. (100,000 segments,
// ~2^30 u32 keys: 2.3 ms with one counter per bin, tiles strided over the
// grid and a flush per tile; 1.76 ms with 8 columns in 256-thread CTAs.)
constexpr int SEG_HIST_THREADS = 1024;
constexpr int SEG_HIST_UNROLL = 4;  // 16-byte vectors in flight per thread
template <typename K> __host__ __device__ constexpr int seg_hist_cols() { return sizeof(K) == 4 ? 32 : 16; }
template <typename K> constexpr size_t seg_hist_smem() {
  return size_t(Bits<K>::DIGITS) * RADIX * seg_hist_cols<K>() * sizeof(uint32_t);
}

template <typename K>
__global__ void __launch_bounds__(SEG_HIST_THREADS) seg_hist_kernel(SegHistParams p) {
  constexpr int KD = Bits<K>::DIGITS;
  constexpr uint32_t NC = seg_hist_cols<K>();
  constexpr uint32_t WORDS = KD * RADIX * NC;
  constexpr uint32_t KPV = 16 / sizeof(K);  // keys per 16-byte vector
  extern __shared__ __align__(16) uint32_t s_h[];  // [digit][bin][column]
  const OrderXform<K> kx(p.key_kind, p.desc != 0);
  const K* keys = static_cast<const K*>(p.keys);
  const uint32_t tid = threadIdx.x;
  uint32_t* const hk = s_h + (tid & (NC - 1));
  const bool vec = (reinterpret_cast<uintptr_t>(keys) & 15u) == 0;
  auto count = [&](K v) {
#pragma unroll
    for (int d = 0; d < KD; ++d) atomicAdd(hk + (d * RADIX + (uint32_t(v >> (8 * d)) & 255u)) * NC, 1u);
  };
  const uint32_t per = (p.total_tiles + gridDim.x - 1) / gridDim.x;
  const uint32_t t0 = blockIdx.x * per;
  const uint32_t t1 = min(t0 + per, p.total_tiles);
  if (t0 >= t1) return;
  for (uint32_t i = tid; i < WORDS; i += SEG_HIST_THREADS) s_h[i] = 0;
  // The segment of tile t0: the last s with seg_tile_start[s] <= t0.
  uint32_t seg = 0;
  {
    uint32_t lo = 0, hi = p.nseg;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (p.seg_tile_start[mid] <= t0) lo = mid; else hi = mid;
    }
    seg = lo;
  }
  __syncthreads();
  while (true) {
    // This run's tiles of segment seg, and their elements [b, e).
    const uint32_t f = p.seg_tile_start[seg];
    const uint32_t ta = max(t0, f), tb = min(t1, p.seg_tile_start[seg + 1]);
    const uint64_t s0 = p.seg_range[2 * seg], s1 = p.seg_range[2 * seg + 1];
    const uint64_t b = s0 + uint64_t(ta - f) * p.tile;
    const uint64_t e = min(s0 + uint64_t(tb - f) * p.tile, s1);
    const uint64_t lead = (KPV - (b & (KPV - 1))) & (KPV - 1);
    const uint64_t head = vec && lead < e - b ? lead : e - b;
    const uint64_t nvec = (e - b - head) / KPV;
    const uint64_t tail = b + head + nvec * KPV;
    for (uint64_t i = b + tid; i < b + head; i += SEG_HIST_THREADS) count(kx.fwd(keys[i]));
    for (uint64_t i = tail + tid; i < e; i += SEG_HIST_THREADS) count(kx.fwd(keys[i]));
    const uint4* kv = reinterpret_cast<const uint4*>(keys + b + head);
    for (uint64_t v0 = tid; v0 < nvec; v0 += uint64_t(SEG_HIST_THREADS) * SEG_HIST_UNROLL) {
      uint4 q[SEG_HIST_UNROLL];
#pragma unroll
      for (int u = 0; u < SEG_HIST_UNROLL; ++u) {
        const uint64_t vi = v0 + uint64_t(u) * SEG_HIST_THREADS;
        q[u] = vi < nvec ? kv[vi] : make_uint4(0, 0, 0, 0);
      }
#pragma unroll
      for (int u = 0; u < SEG_HIST_UNROLL; ++u) {
        if (v0 + uint64_t(u) * SEG_HIST_THREADS < nvec) {
          if constexpr (KPV == 4) {
            count(kx.fwd(K(q[u].x)));
            count(kx.fwd(K(q[u].y)));
            count(kx.fwd(K(q[u].z)));
            count(kx.fwd(K(q[u].w)));
          } else {
            count(kx.fwd(K(q[u].x) | (K(q[u].y) << 32)));
            count(kx.fwd(K(q[u].z) | (K(q[u].w) << 32)));
          }
        }
      }
    }
    // Add the counts to the segment's histogram and clear them.
    __syncthreads();
    uint32_t* g = p.hist + size_t(seg) * KD * RADIX;
    for (uint32_t i = tid; i < uint32_t(KD * RADIX); i += SEG_HIST_THREADS) {
      uint32_t c = 0;
#pragma unroll
      for (uint32_t j = 0; j < NC; ++j) {
        const uint32_t w = i * NC + ((j + i) & (NC - 1));
        c += s_h[w];
        s_h[w] = 0;
      }
      if (c) atomicAdd(&g[i], c);
    }
    __syncthreads();
    if (tb >= t1 || seg + 1 >= p.nseg) break;
    ++seg;
  }
}

// In place: histogram -> exclusive bin bases, one block per segment.
__global__ void __launch_bounds__(256) seg_scan_kernel(uint32_t* hist, uint32_t digits) {
  __shared__ uint32_t s_tmp[8];
  uint32_t* h = hist + size_t(blockIdx.x) * digits * RADIX;
  for (uint32_t q = 0; q < digits; ++q) {
    const uint32_t c = h[q * RADIX + threadIdx.x];
    const uint32_t ex = block_excl_scan_256(c, s_tmp);
    h[q * RADIX + threadIdx.x] = ex;
  }
}

// Plan of a segmented pass sequence: every digit runs, counters cleared.
__global__ void seg_plan_kernel(SortWork* w, uint32_t digits, uint32_t* gen_counter) {
  const uint32_t t = threadIdx.x;
  if (t < MAX_DIGITS) {
    w->plan.tile_counter[t] = 0;
    w->plan.exec_index[t] = t < digits ? t : PASS_SKIPPED;
  }
  if (t == 0) {
    w->plan.first_stable = 0;
    w->plan.first_reverse = 0;
    w->plan.m_exec = digits;
    w->plan.gen_base = atomicAdd(gen_counter, uint32_t(MAX_DIGITS + 1));
  }
}

}  // namespace gs

// ---------------------------------------------------------------------------
// Host side
// ---------------------------------------------------------------------------
struct gs_seg_plan {
  int key_bytes = 4;
  uint32_t kind = 0;
  bool desc = false;
  uint64_t n = 0;
  uint32_t ngroups = 0;
  uint32_t ntiny = 0;
  uint32_t nlarge = 0;
  uint32_t large_tiles = 0;
  uint32_t tile = 0;
  int shape = 0;
  gs::SegGroup* d_groups = nullptr;
  gs::TinySeg* d_tiny = nullptr;
  uint32_t* d_starts_rel = nullptr;
  uint32_t* d_tile_start = nullptr;
  gs::SegTile* d_tiles = nullptr;
  uint64_t* d_range = nullptr;
  uint32_t* d_hist = nullptr;
  gs::SortWork* d_work = nullptr;
};

namespace gs {

// How a segmented sort treats each segment (host only): small segments
// packed in order into groups of consecutive segments (at most GROUP_KEYS
// keys and GROUP_MAX_SEGS segments; a group made only of segments of at
// most TINY_KEYS keys becomes one warp network per segment), and the large
// segments cut into pass tiles of `tile` elements.
struct SegLayout {
  std::vector<SegGroup> groups;
  std::vector<TinySeg> tiny;
  std::vector<uint32_t> rel;         // per group: segment starts relative to the group
  std::vector<uint32_t> tile_start;  // per large segment: first tile, then the tile count
  std::vector<SegTile> tile_desc;    // per tile
  std::vector<uint64_t> range;       // per large segment: [begin, end)
  uint64_t tiles = 0;
};

// kinds (optional, nseg entries): the gs_seg_kind of each segment.
std::string seg_layout(const uint64_t* off, uint32_t nseg, uint64_t n, uint32_t tile,
                       SegLayout& L, uint8_t* kinds) {
  if (off[0] != 0 || off[nseg] != n) return "offsets must start at 0 and end at n";
  SegGroup cur{};
  uint32_t cur_max = 0;    // longest segment of the open group
  uint32_t cur_first = 0;  // index of the open group's first segment
  bool open = false;
  auto close = [&](uint32_t s_end) {  // s_end: the segment after the group's last
    const bool is_tiny = open && cur.count > 0 && cur_max <= TINY_KEYS;
    if (is_tiny) {
      // Only tiny segments: one warp each instead of a group sort.
      L.rel.push_back(cur.count);
      for (uint32_t i = 0; i < cur.nsegs; ++i) {
        const uint32_t a = L.rel[cur.first_seg + i], z = L.rel[cur.first_seg + i + 1];
        L.tiny.push_back(TinySeg{cur.start + a, z - a, 0});
      }
      L.rel.resize(cur.first_seg);
    } else if (open && cur.count > 0) {
      L.rel.push_back(cur.count);  // end of the last segment
      L.groups.push_back(cur);
    } else if (open) {
      L.rel.resize(cur.first_seg);  // empty group: drop its starts
    }
    if (kinds && open) {
      for (uint32_t t = cur_first; t < s_end; ++t)
        if (off[t + 1] > off[t]) kinds[t] = is_tiny ? GS_SEG_WARP : GS_SEG_GROUP;
    }
    open = false;
  };
  for (uint32_t s = 0; s < nseg; ++s) {
    const uint64_t b = off[s], e = off[s + 1];
    if (e < b) return "offsets must be non-decreasing";
    const uint64_t len = e - b;
    if (kinds) kinds[s] = GS_SEG_EMPTY;
    if (len == 0) continue;  // nothing to move
    if (len > GROUP_KEYS) {
      close(s);
      L.tile_start.push_back(uint32_t(L.tiles));
      const uint32_t large_index = uint32_t(L.range.size() / 2);
      L.range.push_back(b);
      L.range.push_back(e);
      for (uint64_t x = b; x < e; x += tile)
        L.tile_desc.push_back(SegTile{x, uint32_t(std::min<uint64_t>(tile, e - x)), large_index});
      L.tiles += (len + tile - 1) / tile;
      if (kinds) kinds[s] = GS_SEG_PASSES;
      continue;
    }
    if (!open || cur.count + len > GROUP_KEYS || cur.nsegs + 1 > GROUP_MAX_SEGS ||
        cur.start + cur.count != b) {
      close(s);
      cur = SegGroup{b, 0, uint32_t(L.rel.size()), 0, 0};
      cur_max = 0;
      cur_first = s;
      open = true;
    }
    L.rel.push_back(cur.count);
    cur.count += uint32_t(len);
    cur.nsegs += 1;
    cur_max = std::max(cur_max, uint32_t(len));
  }
  close(nseg);
  if (L.tiles > 0xFFFFFFF0ull) return "too many tiles";
  L.tile_start.push_back(uint32_t(L.tiles));
  return "";
}

std::string seg_layout_summary(const uint64_t* off, uint32_t nseg, uint64_t n, uint32_t tile,
                               uint8_t* kinds, uint64_t counts[4]) {
  SegLayout L;
  const std::string err = seg_layout(off, nseg, n, tile, L, kinds);
  if (err.empty()) {
    counts[0] = L.groups.size();
    counts[1] = L.tiny.size();
    counts[2] = L.range.size() / 2;
    counts[3] = L.tiles;
  }
  return err;
}

// Build a plan from host offsets (nseg + 1 entries). Returns an error text
// or empty on success.
std::string seg_plan_build(gs_seg_plan* pl, const uint64_t* off, uint32_t nseg, uint64_t n,
                           int key_bytes, uint32_t kind, bool desc, int shape) {
  pl->key_bytes = key_bytes;
  pl->kind = kind;
  pl->desc = desc;
  pl->n = n;
  pl->shape = shape;
  pl->tile = radix_shape_tile(key_bytes, 0, shape);
  SegLayout L;
  const std::string err = seg_layout(off, nseg, n, pl->tile, L, nullptr);
  if (!err.empty()) return err;
  pl->ngroups = uint32_t(L.groups.size());
  pl->ntiny = uint32_t(L.tiny.size());
  pl->nlarge = uint32_t(L.range.size() / 2);
  pl->large_tiles = uint32_t(L.tiles);
  auto up = [](void** dst, const void* src, size_t bytes) -> bool {
    if (bytes == 0) return true;
    if (cudaMalloc(dst, bytes) != cudaSuccess) return false;
    return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  };
  bool ok = up(reinterpret_cast<void**>(&pl->d_groups), L.groups.data(), L.groups.size() * sizeof(SegGroup)) &&
            up(reinterpret_cast<void**>(&pl->d_tiny), L.tiny.data(), L.tiny.size() * sizeof(TinySeg)) &&
            up(reinterpret_cast<void**>(&pl->d_starts_rel), L.rel.data(), L.rel.size() * 4) &&
            up(reinterpret_cast<void**>(&pl->d_tile_start), L.tile_start.data(), L.tile_start.size() * 4) &&
            up(reinterpret_cast<void**>(&pl->d_tiles), L.tile_desc.data(), L.tile_desc.size() * sizeof(SegTile)) &&
            up(reinterpret_cast<void**>(&pl->d_range), L.range.data(), L.range.size() * 8);
  if (ok && pl->nlarge) {
    ok = cudaMalloc(&pl->d_hist, size_t(pl->nlarge) * key_bytes * RADIX * 4) == cudaSuccess &&
         cudaMalloc(&pl->d_work, sizeof(SortWork)) == cudaSuccess;
  }
  if (!ok) {
    cudaGetLastError();
    return "device allocation for the segmented plan failed";
  }
  return "";
}

void seg_plan_free(gs_seg_plan* pl) {
  void* ps[] = {pl->d_groups, pl->d_tiny, pl->d_starts_rel, pl->d_tile_start, pl->d_tiles,
                pl->d_range, pl->d_hist, pl->d_work};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete pl;
}

gs_seg_plan* seg_plan_new() { return new gs_seg_plan(); }
uint32_t seg_plan_large_tiles(const gs_seg_plan* pl) { return pl->large_tiles; }
uint64_t seg_plan_n(const gs_seg_plan* pl) { return pl->n; }
int seg_plan_key_bytes(const gs_seg_plan* pl) { return pl->key_bytes; }

template <typename K>
cudaError_t seg_run_t(const gs_seg_plan* pl, const void* in, void* out, void* alt,
                      uint64_t* status, uint32_t* gen_counter, uint32_t* err, uint32_t spin_limit,
                      const DeviceProps& props, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (pl->ntiny) {
    tiny_sort_kernel<K><<<(pl->ntiny + 7) / 8, 256, 0, st>>>(in, out, pl->d_tiny, pl->ntiny,
                                                            pl->kind, uint32_t(pl->desc));
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (pl->ngroups) {
    GroupSortParams gp{in, out, pl->d_groups, pl->d_starts_rel, pl->kind, pl->desc};
    constexpr size_t dyn = group_sort_dyn_smem<K>();
    e = allow_dynamic_smem(reinterpret_cast<const void*>(group_sort_kernel<K>), dyn);
    if (e != cudaSuccess) return e;
    group_sort_kernel<K><<<pl->ngroups, GROUP_THREADS, dyn, st>>>(gp);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (pl->nlarge == 0) return cudaSuccess;
  const uint32_t digits = Bits<K>::DIGITS;
  e = cudaMemsetAsync(pl->d_hist, 0, size_t(pl->nlarge) * digits * RADIX * 4, st);
  if (e != cudaSuccess) return e;
  SegHistParams hp{in, pl->d_tile_start, pl->d_range, pl->nlarge, pl->tile, pl->large_tiles,
                   pl->kind, pl->desc, pl->d_hist};
  // One CTA per SM (128 KB of counters).
  unsigned hb = std::min<unsigned>(pl->large_tiles, unsigned(props.num_sms));
  e = allow_dynamic_smem(reinterpret_cast<const void*>(seg_hist_kernel<K>), seg_hist_smem<K>());
  if (e != cudaSuccess) return e;
  seg_hist_kernel<K><<<hb, SEG_HIST_THREADS, seg_hist_smem<K>(), st>>>(hp);
  seg_scan_kernel<<<pl->nlarge, 256, 0, st>>>(pl->d_hist, digits);
  seg_plan_kernel<<<1, 32, 0, st>>>(pl->d_work, digits, gen_counter);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  RadixJob job;
  job.keys_in = in;
  job.keys_out = out;
  job.keys_alt = alt;
  job.n = pl->n;
  job.key_bytes = int(sizeof(K));
  job.key_kind = pl->kind;
  job.desc = pl->desc;
  job.first_unstable = true;
  job.status = status;
  job.work = pl->d_work;
  job.err = err;
  job.spin_limit = spin_limit;
  job.shape = pl->shape;
  job.gen_counter = gen_counter;
  SegJob sj{pl->d_tile_start, pl->d_range, pl->d_hist, pl->nlarge, digits, pl->large_tiles,
            pl->d_tiles};
  uint32_t unused = 0;
  return launch_radix_passes(job, sj, props, &unused, st);
}

cudaError_t seg_plan_run(const gs_seg_plan* pl, const void* in, void* out, void* alt,
                         uint64_t* status, uint32_t* gen_counter, uint32_t* err,
                         uint32_t spin_limit, const DeviceProps& props, cudaStream_t st) {
  if (pl->key_bytes == 4)
    return seg_run_t<uint32_t>(pl, in, out, alt, status, gen_counter, err, spin_limit, props, st);
  return seg_run_t<uint64_t>(pl, in, out, alt, status, gen_counter, err, spin_limit, props, st);
}

uint32_t small_sort_max() { return GROUP_KEYS; }

// One CTA sorts n <= GROUP_KEYS keys in shared memory (the batched sort's
// group kernel with a single group): one launch instead of the radix
// pipeline's five. Reads all of `in` before writing `out`, so they may alias.
cudaError_t launch_small_sort(const void* in, void* out, uint32_t n, int key_bytes,
                              uint32_t kind, bool desc, cudaStream_t st) {
  if (n == 0 || n > GROUP_KEYS) return cudaErrorInvalidValue;
  GroupSortParams gp{in, out, nullptr, nullptr, kind, uint32_t(desc), n, nullptr};
  auto go = [&](auto kern, size_t dyn) -> cudaError_t {
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(kern), dyn);
    if (e != cudaSuccess) return e;
    kern<<<1, GROUP_THREADS, dyn, st>>>(gp);
    return cudaGetLastError();
  };
  if (key_bytes == 4) return go(group_sort_kernel<uint32_t>, group_sort_dyn_smem<uint32_t>());
  return go(group_sort_kernel<uint64_t>, group_sort_dyn_smem<uint64_t>());
}

// One launch sorting `count` independent small arrays, one CTA each (their
// descriptors in memory the device can read: device or mapped host memory).
cudaError_t launch_small_sort_batch(const SmallSortReq* reqs, uint32_t count, int key_bytes,
                                    cudaStream_t st) {
  if (count == 0) return cudaSuccess;
  GroupSortParams gp{nullptr, nullptr, nullptr, nullptr, 0, 0, 0, reqs};
  auto go = [&](auto kern, size_t dyn) -> cudaError_t {
    const cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(kern), dyn);
    if (e != cudaSuccess) return e;
    kern<<<count, GROUP_THREADS, dyn, st>>>(gp);
    return cudaGetLastError();
  };
  if (key_bytes == 4) return go(group_sort_kernel<uint32_t>, group_sort_dyn_smem<uint32_t>());
  return go(group_sort_kernel<uint64_t>, group_sort_dyn_smem<uint64_t>());
}

}  // namespace gs
