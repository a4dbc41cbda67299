// Launchers of the onesweep radix pipeline (kernels in radix.cuh).
#include <cstddef>
#include <mutex>
#include <set>
#include <utility>

#include "engine.h"
#include "radix.cuh"

namespace gs {

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
  // Look-back tags come from the device, so a replayed CUDA graph never
  // meets its own earlier words with a matching tag.
  if (tid == 0) plan.gen_base = atomicAdd(p.gen_counter, uint32_t(MAX_DIGITS + 1));
  __syncthreads();
  if (tid == 0) {
    const uint32_t lo = p.digit_lo, hi = p.digit_hi;
    // Ties ordered by value, with the values already non-decreasing in
    // input order: that order is the input order, so the value digits are
    // dropped and the first pass keeps ties stable (reversed when
    // descending, as std::greater puts larger values first).
    const bool drop = p.drop_val_digits > 0 && p.work->val_order_break == 0;
    plan.first_stable = drop ? 1u : 0u;
    plan.first_reverse = (drop && p.drop_reverse) ? 1u : 0u;
    bool exec[MAX_DIGITS];
    uint32_t m = 0;
    for (uint32_t q = 0; q < MAX_DIGITS; ++q) {
      exec[q] = (q >= lo && q < hi) && !s_trivial[q] && !(drop && q < p.drop_val_digits);
      m += exec[q];
    }
    // Every key equal: nothing to reorder, but a copy (or the reversal of a
    // stable descending pair sort) still has to reach the output.
    if (m == 0 && (!p.in_place || p.reverse_first || plan.first_reverse)) {
      exec[hi - 1] = true;
      m = 1;
    }
    // The first pass may not write its own input. In place, the pass count
    // is made even so that the first pass writes the scratch buffer; with
    // the scratch aliasing the input, odd so that it writes the output. A
    // digit that needs no reordering is run as a copy to fix the parity
    // (key digits come in even numbers, so one exists when it is needed).
    const uint32_t want = p.alt_is_in ? 1u : 0u;
    if ((p.in_place || p.alt_is_in) && (m & 1u) != want) {
      for (uint32_t q = lo; q < hi; ++q) {
        if (!exec[q] && s_trivial[q]) { exec[q] = true; ++m; break; }
      }
    }
    uint32_t j = 0;
    for (uint32_t q = 0; q < MAX_DIGITS; ++q) plan.exec_index[q] = exec[q] ? j++ : PASS_SKIPPED;
    plan.m_exec = m;
  }
}


namespace {

constexpr int UPSWEEP_THREADS = 512;
constexpr int UPSWEEP_UNROLL = 8;
constexpr uint32_t UPSWEEP_SMEM = 64u << 10;  // column-spread histograms per CTA
constexpr int UPSWEEP_PER_SM = 3;

// Tile shapes of the pass kernel (threads per block, items per thread,
// blocks per SM, ranking of the stable passes), selectable per call; shape
// 0 is the default. Larger elements take fewer items per thread: each
// shape has the most items that fit its register share without spilling
// (or with a few bytes of spill where that measured faster).
//  - Shape 0: 384 threads, 3 CTAs per SM. More CTAs per SM hide more of
//    each tile's barrier and look-back latency than 512-thread tiles at 2
//    CTAs per SM: 2^30 u32 keys 14.7 vs 15.4 ms, 2^29 u64 23.4 vs 23.9 ms,
//    2^29 u64 + u32 pairs 53.4 vs 55.2 ms, u32 + u32 26.9 vs 27.7 ms.
//    (320 x 24 x 3: 15.7 ms; 256 x 24 x 4: 16.4 ms; 384 x 22 x 3: 15.1 ms;
//    384 x 32 x 2: 15.1 ms.) 64-bit keys with 64-bit payloads spill at 384
//    threads and keep 512.
//  - Shape 1: 256 threads, 4 CTAs per SM, for small sorts.
//  - Shape 2: 512 threads, 2 CTAs per SM (the previous default).
// Keys and pairs rank by half-warps: 2^30 u32 keys, stable passes 3.97 vs
// 4.30 ms with the 64-bit table; 2^29 pairs (same 384-thread tile, table vs
// half-warp): u64 Zipf(1.1) + u32 index, stable, 33.6 -> 30.9 ms (skewed
// digits), u64 + u32 uniform 50.0 -> 49.8 ms, u32 + u32 24.7 -> 24.3 ms.
// u64 + u64 pairs keep the table in their 512-thread tile (2^28 pairs:
// 38.7 ms vs 38.9 ms by half-warps).
template <int T, int I, int B, int R = RANK_TABLE> struct Shape {
  static constexpr int THREADS = T, ITEMS = I, MINB = B, RANK = R;
};
template <typename K, typename V, int S> struct PassShape;
template <> struct PassShape<uint32_t, NoValue, 0> : Shape<384, 24, 3, RANK_HALF> {};
template <> struct PassShape<uint32_t, NoValue, 1> : Shape<256, 20, 4> {};
template <> struct PassShape<uint32_t, NoValue, 2> : Shape<512, 24, 2, RANK_HALF> {};
template <> struct PassShape<uint64_t, NoValue, 0> : Shape<384, 14, 3, RANK_HALF> {};
template <> struct PassShape<uint64_t, NoValue, 1> : Shape<256, 12, 4> {};
template <> struct PassShape<uint64_t, NoValue, 2> : Shape<512, 14, 2, RANK_HALF> {};
template <> struct PassShape<uint32_t, uint32_t, 0> : Shape<384, 14, 3, RANK_HALF> {};
template <> struct PassShape<uint32_t, uint32_t, 1> : Shape<256, 12, 4> {};
template <> struct PassShape<uint32_t, uint32_t, 2> : Shape<512, 14, 2> {};
template <> struct PassShape<uint64_t, uint64_t, 0> : Shape<512, 9, 2> {};
template <> struct PassShape<uint64_t, uint64_t, 2> : Shape<512, 9, 2, RANK_HALF> {};
template <typename K, typename V, int S>
struct PassShape : Shape<(S == 0 ? 384 : S == 1 ? 256 : 512), (S == 1 ? 6 : 10),
                         (S == 0 ? 3 : S == 1 ? 4 : 2), (S == 0 ? RANK_HALF : RANK_TABLE)> {};
constexpr int NUM_SHAPES = 3;
constexpr uint32_t MIN_TILE = 1024;  // no shape has a smaller tile (smallest: 256 x 6)

// Enqueue the digit passes (plan already in job.work). With `sj` the passes
// sort the large segments of a batch.
template <typename K, typename V, int S>
cudaError_t launch_passes(const RadixJob& job, const SegJob* sj, uint32_t digits, uint32_t vd,
                          const DeviceProps& props, uint32_t* gen, cudaStream_t stream) {
  using Sh = PassShape<K, V, S>;
  using Cfg = PassConfig<K, V, Sh::THREADS, Sh::ITEMS, Sh::RANK>;
  // The lowest digit's pass, when it runs, is the first one and ranks
  // unstably in keys-only sorts. Those launch it with the unstable-only
  // kernel of the same tile (2^30 u32 keys: 2.94 -> 2.65 ms against the
  // table kernel's unstable branch; 2^29 u64 keys: 2.43 -> 2.19 ms).
  constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  using CfgU = PassConfig<K, V, Sh::THREADS, Sh::ITEMS, RANK_UNSTABLE>;
  static_assert(CfgU::TILE == Cfg::TILE, "one tile layout for every pass of a sort");
  cudaError_t e = cudaSuccess;
  // Segmented sorts (keys only) run the SEG form of the same kernels.
  const bool seg = sj != nullptr;
  auto kern = seg ? pass_kernel<K, V, Sh::THREADS, Sh::ITEMS, Sh::MINB, Sh::RANK, false, !HAS_V>
                  : pass_kernel<K, V, Sh::THREADS, Sh::ITEMS, Sh::MINB, Sh::RANK>;
  auto kernu = seg ? pass_kernel<K, V, Sh::THREADS, Sh::ITEMS, Sh::MINB, HAS_V ? Sh::RANK : RANK_UNSTABLE,
                                 false, !HAS_V>
                   : pass_kernel<K, V, Sh::THREADS, Sh::ITEMS, Sh::MINB, HAS_V ? Sh::RANK : RANK_UNSTABLE>;
  e = allow_dynamic_smem(reinterpret_cast<const void*>(kern), Cfg::DYN_SMEM);
  if (e == cudaSuccess && !HAS_V)
    e = allow_dynamic_smem(reinterpret_cast<const void*>(kernu), CfgU::DYN_SMEM);
  if (e != cudaSuccess) return e;
  const uint64_t tiles = sj != nullptr ? sj->total_tiles : (job.n + Cfg::TILE - 1) / Cfg::TILE;
  PassParams pa{};
  pa.keys_in = job.keys_in;
  pa.keys_out = job.keys_out;
  pa.keys_alt = job.keys_alt;
  pa.vals_in = job.vals_in;
  pa.vals_out = job.vals_out;
  pa.vals_alt = job.vals_alt;
  pa.n = job.n;
  pa.val_digits = vd;
  pa.key_kind = job.key_kind;
  pa.val_kind = job.val_kind;
  pa.desc = job.desc;
  pa.reverse_first = job.reverse_first;
  pa.first_unstable = job.first_unstable && !job.reverse_first;
  pa.status = job.status;
  pa.spin_limit = job.spin_limit;
  pa.inject_stall = job.inject_stall;
  pa.work = job.work;
  pa.err = job.err;
  if (sj != nullptr) {
    if (HAS_V || sj->tiles == nullptr) return cudaErrorInvalidValue;
    pa.seg_tile_start = sj->tile_start;
    pa.seg_tiles = sj->tiles;
    pa.seg_range = sj->range;
    pa.seg_binbase = sj->binbase;
    pa.nseg = sj->nseg;
    pa.seg_digits = sj->digits;
  }
  if (tiles == 0) return cudaSuccess;
  (void)gen;
  // Each CTA prefetches the tile one wave of resident CTAs ahead into L2,
  // the tile a CTA claims about when this one finishes (2^30 u32 keys:
  // passes 3.54 -> 3.48 ms; 2^29 u64 keys: 2.77 -> 2.58 ms; two waves
  // ahead gained less).
  pa.prefetch_tiles = uint32_t(props.num_sms * Sh::MINB);
  const uint32_t qlo = job.digit_hi ? job.digit_lo : 0u;
  const uint32_t qhi = job.digit_hi ? job.digit_hi : digits;
  for (uint32_t q = qlo; q < qhi; ++q) {
    pa.pass = q;
    if (q == qlo && !HAS_V && pa.first_unstable)
      kernu<<<unsigned(tiles), Sh::THREADS, CfgU::DYN_SMEM, stream>>>(pa);
    else
      kern<<<unsigned(tiles), Sh::THREADS, Cfg::DYN_SMEM, stream>>>(pa);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if (job.marks) cudaEventRecord(job.marks[3 + q], stream);
  }
  return cudaGetLastError();
}

// Zero the histograms and count every digit of the job's elements in one
// read (copying them on the way when keys_copy is set).
template <typename K, typename V>
cudaError_t launch_upsweep(const RadixJob& job, uint32_t vd, const DeviceProps& props,
                           cudaStream_t stream) {
  constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  cudaError_t e = cudaMemsetAsync(job.work, 0, offsetof(SortWork, plan), stream);
  if (e != cudaSuccess) return e;
  UpsweepParams up{};
  up.keys = job.keys_in;
  up.vals = job.vals_in;
  up.copy_keys = job.keys_copy;
  up.copy_vals = HAS_V ? job.vals_copy : nullptr;
  up.n = job.n;
  up.key_kind = job.key_kind;
  up.val_kind = job.val_kind;
  up.desc = job.desc;
  up.val_digits = vd;
  up.check_val_order = vd > 0 ? 1u : 0u;
  up.work = job.work;
  const uint32_t total_digits = vd + uint32_t(sizeof(K));
  // Key digits only: for four digits (32-bit keys) one column per lane, so
  // a warp's atomics never share a bank (128 KB); for eight, 16 columns
  // (128 KB). One 1024-thread CTA per SM; 32-bit keys keep 16 loads in
  // flight per thread. Measured at 2^30 u32 keys: 0.96 ms, from 1.17 with
  // 16 columns, three 512-thread CTAs per SM and 8 loads (1.05 with 8 loads,
  // 0.98 with 32, which spill); 2^29 u64 keys: 1.01 from 1.45 ms. With
  // value digits to count (and their order to check) the narrower form
  // stays faster: 2^29 u32 + u32 by value 2.05 vs 2.63 ms. So does it below
  // 2^20 keys, where zeroing and flushing 128 KB per CTA is the bulk.
  if (job.upsweep_per_sm == 0 && vd == 0 && (total_digits == 4 || total_digits == 8) &&
      job.n >= (uint64_t(1) << 20)) {
    auto kw = total_digits == 4
                  ? upsweep_kernel<K, V, 1024, sizeof(K) == 4 ? 16 : 8, 5>
                  : upsweep_kernel<K, V, 1024, 8, 4>;
    const uint32_t unroll = (total_digits == 4 && sizeof(K) == 4) ? 16u : 8u;
    constexpr size_t SMW = size_t(128) << 10;
    e = allow_dynamic_smem(reinterpret_cast<const void*>(kw), SMW);
    if (e != cudaSuccess) return e;
    const uint64_t chunkw = uint64_t(1024) * unroll;
    uint64_t bw = (job.n + chunkw - 1) / chunkw;
    if (bw > uint64_t(props.num_sms)) bw = uint64_t(props.num_sms);
    if (bw == 0) bw = 1;
    kw<<<unsigned(bw), 1024, SMW, stream>>>(up);
    return cudaGetLastError();
  }
  // Histogram columns: as many (4 to 16) as fit UPSWEEP_SMEM bytes.
  uint32_t cl = 2;
  while (cl < 4 && ((total_digits * RADIX) << (cl + 1)) * 4u <= UPSWEEP_SMEM) ++cl;
  const size_t usmem = size_t((total_digits * RADIX) << cl) * 4u;
  auto ukern = cl == 4 ? upsweep_kernel<K, V, UPSWEEP_THREADS, UPSWEEP_UNROLL, 4>
             : cl == 3 ? upsweep_kernel<K, V, UPSWEEP_THREADS, UPSWEEP_UNROLL, 3>
                       : upsweep_kernel<K, V, UPSWEEP_THREADS, UPSWEEP_UNROLL, 2>;
  e = allow_dynamic_smem(reinterpret_cast<const void*>(ukern), UPSWEEP_SMEM);
  if (e != cudaSuccess) return e;
  const uint64_t chunk = uint64_t(UPSWEEP_THREADS) * UPSWEEP_UNROLL;
  uint64_t ublocks = (job.n + chunk - 1) / chunk;
  const uint64_t umax =
      uint64_t(props.num_sms) * (job.upsweep_per_sm ? job.upsweep_per_sm : UPSWEEP_PER_SM);
  if (ublocks > umax) ublocks = umax;
  if (ublocks == 0) ublocks = 1;
  ukern<<<unsigned(ublocks), UPSWEEP_THREADS, usmem, stream>>>(up);
  return cudaGetLastError();
}

template <typename K, typename V, int S>
cudaError_t run(const RadixJob& job, const DeviceProps& props, uint32_t* gen,
                cudaStream_t stream) {
  constexpr bool HAS_V = !std::is_same<V, NoValue>::value;
  const uint32_t kd = Bits<K>::DIGITS;
  uint32_t vd = 0;
  if constexpr (HAS_V) vd = job.ties_by_value ? Bits<V>::DIGITS : 0;
  const uint32_t digits = kd + vd;

  static_assert(MAX_DIGITS == HIST_DIGITS && RADIX == 256, "histogram copy layout");
  if (job.digit_hi && (job.digit_hi > digits || job.digit_lo >= job.digit_hi ||
                       (job.alt_is_in && ((job.digit_hi - job.digit_lo) & 1u) == 0)))
    return cudaErrorInvalidValue;
  if (job.alt_is_in && !job.digit_hi && (digits & 1u) == 0) return cudaErrorInvalidValue;
  if (job.marks) cudaEventRecord(job.marks[0], stream);
  cudaError_t e = cudaSuccess;
  if (!job.skip_upsweep) {
    e = launch_upsweep<K, V>(job, vd, props, stream);
    if (e != cudaSuccess) return e;
    if (job.marks) cudaEventRecord(job.marks[1], stream);
    if (job.hist_copy) {
      e = cudaMemcpyAsync(job.hist_copy, &job.work->hist[0][0], sizeof(uint32_t) * HIST_WORDS,
                          cudaMemcpyDeviceToHost, stream);
      if (e != cudaSuccess) return e;
      if (job.hist_ready) cudaEventRecord(job.hist_ready, stream);
    }
    if (job.upsweep_only) return cudaSuccess;
  }

  // With copies, the passes read the copies.
  RadixJob pj = job;
  if (job.keys_copy) {
    pj.keys_in = job.keys_copy;
    if (HAS_V) pj.vals_in = job.vals_copy;
  }
  PlanParams pp{};
  pp.work = job.work;
  pp.n = job.n;
  pp.digits = digits;
  pp.in_place = (pj.keys_in == pj.keys_out) ||
                (HAS_V && pj.vals_in == pj.vals_out);
  pp.reverse_first = job.reverse_first;
  pp.digit_lo = job.digit_hi ? job.digit_lo : 0u;
  pp.digit_hi = job.digit_hi ? job.digit_hi : digits;
  pp.alt_is_in = job.alt_is_in;
  pp.drop_val_digits = vd;
  pp.drop_reverse = job.desc ? 1u : 0u;
  pp.gen_counter = job.gen_counter ? job.gen_counter : &job.work->gen_counter;
  plan_kernel<<<1, 256, 0, stream>>>(pp);
  if (job.marks) cudaEventRecord(job.marks[2], stream);
  return launch_passes<K, V, S>(pj, nullptr, digits, vd, props, gen, stream);
}

}  // namespace

template <typename K, typename V>
uint32_t shape_tile(int shape) {
  switch (shape) {
    case 1: return PassShape<K, V, 1>::THREADS * PassShape<K, V, 1>::ITEMS;
    case 2: return PassShape<K, V, 2>::THREADS * PassShape<K, V, 2>::ITEMS;
    default: return PassShape<K, V, 0>::THREADS * PassShape<K, V, 0>::ITEMS;
  }
}

uint32_t radix_shape_tile(int key_bytes, int val_bytes, int shape) {
  if (val_bytes != 0) return 0;  // segmented sorts are keys only
  return key_bytes == 4 ? shape_tile<uint32_t, NoValue>(shape) : shape_tile<uint64_t, NoValue>(shape);
}

int radix_segmented_shape(int key_bytes, uint64_t n, uint32_t nseg) {
  // Segments averaging at least 4096 keys (most keys in segments the passes
  // sort): the default 384 x 24 shape. 100,000 segments of 16 .. 2^22 keys,
  // ~2^30 in all: 19.7 ms vs 22.5 ms with the 256 x 20 shape and 21.3 ms
  // with 512 x 24. Many short segments: the 256-thread shape, whose smaller
  // tiles leave less of each segment's last tile empty.
  (void)key_bytes;
  return nseg != 0 && n / nseg >= 4096 ? 0 : 1;
}

cudaError_t launch_radix_passes(const RadixJob& job, const SegJob& sj, const DeviceProps& props,
                                uint32_t* gen, cudaStream_t stream) {
  const uint32_t digits = sj.digits;
  if (job.key_bytes == 4) {
    switch (job.shape) {
      case 0: return launch_passes<uint32_t, NoValue, 0>(job, &sj, digits, 0, props, gen, stream);
      case 1: return launch_passes<uint32_t, NoValue, 1>(job, &sj, digits, 0, props, gen, stream);
      case 2: return launch_passes<uint32_t, NoValue, 2>(job, &sj, digits, 0, props, gen, stream);
      default: return cudaErrorInvalidValue;
    }
  }
  switch (job.shape) {
    case 0: return launch_passes<uint64_t, NoValue, 0>(job, &sj, digits, 0, props, gen, stream);
    case 1: return launch_passes<uint64_t, NoValue, 1>(job, &sj, digits, 0, props, gen, stream);
    case 2: return launch_passes<uint64_t, NoValue, 2>(job, &sj, digits, 0, props, gen, stream);
    default: return cudaErrorInvalidValue;
  }
}

template <typename K>
cudaError_t bucket_pass_t(const RadixJob& job, const void* splitters, uint32_t nsplit,
                          const DeviceProps& props, cudaStream_t st) {
  // 16 (32-bit keys) or 12 (64-bit keys) items per thread leave registers
  // for the packed bucket ids.
  // The bucket scatter ranks unstably: the unstable-only kernel.
  using Sh = Shape<512, sizeof(K) == 4 ? 16 : 12, 2, RANK_UNSTABLE>;
  using Cfg = PassConfig<K, NoValue, Sh::THREADS, Sh::ITEMS, Sh::RANK>;
  PlanParams pp{};
  pp.work = job.work;
  pp.gen_counter = job.gen_counter ? job.gen_counter : &job.work->gen_counter;
  pp.n = job.n;
  pp.digits = 1;
  pp.in_place = 0;
  pp.digit_lo = 0;
  pp.digit_hi = 1;
  plan_kernel<<<1, 256, 0, st>>>(pp);
  auto kern = pass_kernel<K, NoValue, Sh::THREADS, Sh::ITEMS, Sh::MINB, Sh::RANK, true>;
  cudaError_t e = allow_dynamic_smem(reinterpret_cast<const void*>(kern), Cfg::DYN_SMEM_BUCKET);
  if (e != cudaSuccess) return e;
  PassParams pa{};
  pa.keys_in = job.keys_in;
  pa.keys_out = job.keys_out;
  pa.keys_alt = job.keys_alt;
  pa.n = job.n;
  pa.key_kind = job.key_kind;
  pa.desc = job.desc;
  pa.first_unstable = 1;
  pa.status = job.status;
  pa.spin_limit = job.spin_limit;
  pa.inject_stall = job.inject_stall;
  pa.work = job.work;
  pa.err = job.err;
  pa.pass = 0;
  pa.splitters = splitters;
  pa.nsplit = nsplit;
  pa.prefetch_tiles = uint32_t(props.num_sms * Sh::MINB);
  const uint64_t tiles = (job.n + Cfg::TILE - 1) / Cfg::TILE;
  kern<<<unsigned(tiles), Sh::THREADS, Cfg::DYN_SMEM_BUCKET, st>>>(pa);
  return cudaGetLastError();
}

cudaError_t launch_bucket_pass(const RadixJob& job, const void* splitters, uint32_t nsplit,
                               const DeviceProps& props, cudaStream_t st) {
  if (job.key_bytes == 4) return bucket_pass_t<uint32_t>(job, splitters, nsplit, props, st);
  return bucket_pass_t<uint64_t>(job, splitters, nsplit, props, st);
}

uint32_t radix_tile(int key_bytes, int val_bytes) {
  (void)key_bytes;
  (void)val_bytes;
  return MIN_TILE;
}

int radix_num_shapes() { return NUM_SHAPES; }

cudaError_t allow_dynamic_smem(const void* kern, size_t bytes) {
  static std::mutex mu;
  static std::set<std::pair<const void*, int>> done;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(mu);
  if (done.count({kern, dev})) return cudaSuccess;
  e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e == cudaSuccess) done.insert({kern, dev});
  return e;
}

namespace {
template <typename K, typename V>
void shape_info_t(int shape, uint32_t* threads, uint32_t* items) {
  switch (shape) {
    case 1: *threads = PassShape<K, V, 1>::THREADS; *items = PassShape<K, V, 1>::ITEMS; return;
    case 2: *threads = PassShape<K, V, 2>::THREADS; *items = PassShape<K, V, 2>::ITEMS; return;
    default: *threads = PassShape<K, V, 0>::THREADS; *items = PassShape<K, V, 0>::ITEMS; return;
  }
}
template <typename K>
void shape_info_k(int val_bytes, int shape, uint32_t* threads, uint32_t* items) {
  if (val_bytes == 4) shape_info_t<K, uint32_t>(shape, threads, items);
  else if (val_bytes == 8) shape_info_t<K, uint64_t>(shape, threads, items);
  else shape_info_t<K, NoValue>(shape, threads, items);
}
}  // namespace

bool radix_shape_info(int key_bytes, int val_bytes, int shape, uint32_t* threads, uint32_t* items) {
  if ((key_bytes != 4 && key_bytes != 8) || (val_bytes != 0 && val_bytes != 4 && val_bytes != 8) ||
      shape < 0 || shape >= NUM_SHAPES)
    return false;
  if (key_bytes == 4) shape_info_k<uint32_t>(val_bytes, shape, threads, items);
  else shape_info_k<uint64_t>(val_bytes, shape, threads, items);
  return true;
}

// Measured defaults on GB300 (uniform keys, 2^22..2^30): shape 0 is
// fastest for every key and value width (see the shape table). Up to 2^18
// keys (no payload) a sort is a few tiles per pass and each pass takes
// about one tile's latency, so the smaller 256-thread tiles win: 2^16 u32 keys 52.9 vs 65.0 us, u64 86.2 vs 102.7 us;
// equal or worse from 2^20.
int radix_default_shape(int key_bytes, int val_bytes, uint64_t n) {
  (void)key_bytes;
  return (val_bytes == 0 && n <= (uint64_t(1) << 18)) ? 1 : 0;
}

size_t radix_status_words(uint64_t n, int key_bytes, int val_bytes) {
  const uint64_t t = radix_tile(key_bytes, val_bytes);
  return size_t((n + t - 1) / t) * RADIX;
}

size_t radix_status_words_u32_shape0(uint64_t n) {
  constexpr uint64_t t = uint64_t(PassShape<uint32_t, NoValue, 0>::THREADS) *
                         PassShape<uint32_t, NoValue, 0>::ITEMS;
  static_assert(t == RADIX_TILE_U32_SHAPE0, "engine.h states the shape-0 tile");
  return size_t((n + t - 1) / t) * RADIX;
}

size_t sort_work_bytes() { return sizeof(SortWork); }

template <typename K, typename V>
cudaError_t run_shape(const RadixJob& job, const DeviceProps& props, uint32_t* gen,
                      cudaStream_t stream) {
  switch (job.shape) {
    case 1: return run<K, V, 1>(job, props, gen, stream);
    case 2: return run<K, V, 2>(job, props, gen, stream);
    default: return run<K, V, 0>(job, props, gen, stream);
  }
}

cudaError_t launch_radix_sort(const RadixJob& job, const DeviceProps& props,
                              uint32_t* gen, cudaStream_t stream) {
  const int kb = job.key_bytes, vb = job.val_bytes;
  if (kb == 4 && vb == 0) return run_shape<uint32_t, NoValue>(job, props, gen, stream);
  if (kb == 8 && vb == 0) return run_shape<uint64_t, NoValue>(job, props, gen, stream);
  if (kb == 4 && vb == 4) return run_shape<uint32_t, uint32_t>(job, props, gen, stream);
  if (kb == 4 && vb == 8) return run_shape<uint32_t, uint64_t>(job, props, gen, stream);
  if (kb == 8 && vb == 4) return run_shape<uint64_t, uint32_t>(job, props, gen, stream);
  if (kb == 8 && vb == 8) return run_shape<uint64_t, uint64_t>(job, props, gen, stream);
  return cudaErrorInvalidValue;
}

}  // namespace gs
