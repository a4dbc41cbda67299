// C ABI of the engine (include/gpusort_gb300.h): contexts, scratch held
// within an HBM budget, dispatch to the kernel launchers, gathers, timing
// and debug settings. The tuning table is in tuning.cu, sorts of host
// buffers in hostsort.cu.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gpusort_gb300.h"
#include "context.h"
#include "common.cuh"

namespace {

thread_local std::string g_last_global_error;

}  // namespace

namespace gs {

void set_last_global_error(const std::string& msg) { g_last_global_error = msg; }

cudaStream_t context_stream(gs_ctx* ctx) { return ctx->stream; }

gs_status fail(gs_ctx* ctx, gs_status st, const std::string& msg) {
  if (ctx) ctx->last_error = msg; else g_last_global_error = msg;
  return st;
}

gs_status cuda_fail(gs_ctx* ctx, cudaError_t e, const char* where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  if (e == cudaErrorMemoryAllocation) return fail(ctx, GS_ERR_OOM, m);
  return fail(ctx, GS_ERR_CUDA, m);
}

// Grow-only scratch, bounded by the context's HBM budget.
gs_status ensure(gs_ctx* ctx, DevBuf& b, size_t bytes, bool zero) {
  if (b.bytes >= bytes) return GS_OK;
  size_t want = bytes;
  const uint64_t next_held = ctx->held - b.bytes + want;
  if (ctx->budget && next_held > ctx->budget) {
    return fail(ctx, GS_ERR_OOM, "HBM budget exceeded: need " + std::to_string(next_held) +
                                     " bytes, budget " + std::to_string(ctx->budget));
  }
  if (b.ptr) {
    cudaStreamSynchronize(ctx->stream);
    cudaFree(b.ptr);
    ctx->held -= b.bytes;
    b.ptr = nullptr;
    b.bytes = 0;
  }
  cudaError_t e = cudaMalloc(&b.ptr, want);
  if (e != cudaSuccess) {
    cudaGetLastError();
    b.ptr = nullptr;
    return fail(ctx, GS_ERR_OOM, "cudaMalloc of " + std::to_string(want) + " bytes failed");
  }
  if (zero) {
    e = cudaMemsetAsync(b.ptr, 0, want, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemsetAsync");
  }
  b.bytes = want;
  ctx->held += want;
  return GS_OK;
}

bool dtype_info(gs_dtype t, int* bytes, uint32_t* kind) {
  switch (t) {
    case GS_U32: *bytes = 4; *kind = gs::KIND_UNSIGNED; return true;
    case GS_I32: *bytes = 4; *kind = gs::KIND_SIGNED; return true;
    case GS_F32: *bytes = 4; *kind = gs::KIND_FLOAT; return true;
    case GS_U64: *bytes = 8; *kind = gs::KIND_UNSIGNED; return true;
    case GS_I64: *bytes = 8; *kind = gs::KIND_SIGNED; return true;
    case GS_F64: *bytes = 8; *kind = gs::KIND_FLOAT; return true;
  }
  return false;
}

// Phase timing of one call: the start is marked before any work is
// enqueued, and each phase_mark ends the phase named.
void phase_reset(gs_ctx* ctx) {
  ctx->n_phases = 0;
  if (ctx->timing) cudaEventRecord(ctx->ev[0], ctx->stream);
}

void phase_mark(gs_ctx* ctx, const char* name) {
  if (!ctx->timing || ctx->n_phases >= 7) return;
  ctx->phase_names[ctx->n_phases] = name;
  ctx->n_phases++;
  cudaEventRecord(ctx->ev[ctx->n_phases], ctx->stream);
}

// Bring the look-back status words to the size a job needs and keep the
// generation tags unambiguous.
// (Look-back tags are drawn on the device from work->gen_counter; a tag
// repeats only after 2^30 passes.)
gs_status prepare_status(gs_ctx* ctx, size_t words) {
  return ensure(ctx, ctx->status, words * sizeof(uint64_t), true);
}

gs_status check_err_word(gs_ctx* ctx) {
  uint32_t h = 0;
  cudaError_t e = cudaMemcpyAsync(&h, ctx->err, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                  ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "synchronize");
  if (h) {
    cudaMemsetAsync(ctx->err, 0, sizeof(uint32_t), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    std::string m = "device error (code " + std::to_string(h) + "):";
    if (h & gs::ERR_LOOKBACK_TIMEOUT) m += " look-back wait ran out;";
    if (h & gs::ERR_SCATTER_RANGE) m += " scatter range left the output;";
    if (h & gs::ERR_PASS_KIND) m += " unstable-only pass kernel launched for a stable pass;";
    if (h & gs::ERR_SMEM_ALIGN) m += " shared memory misaligned;";
    return fail(ctx, GS_ERR_TIMEOUT, m);
  }
  if (ctx->timing && ctx->n_phases > 0) {
    for (int i = 0; i < ctx->n_phases; ++i) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, ctx->ev[i], ctx->ev[i + 1]);
      ctx->phase_ms[i] = ms;
    }
  }
  return GS_OK;
}

// The parts of a radix job that follow from the element types, the flags
// and the context (buffers left to the caller).
gs::RadixJob radix_job(gs_ctx* ctx, int kb, uint32_t kkind, int vb, uint32_t vkind, uint64_t n,
                       uint32_t flags) {
  const bool desc = flags & GS_FLAG_DESCENDING;
  const bool stable = flags & GS_FLAG_PAIRS_STABLE;
  gs::RadixJob job;
  job.n = n;
  job.key_bytes = kb;
  job.val_bytes = vb;
  job.key_kind = kkind;
  job.val_kind = vkind;
  job.desc = desc;
  job.ties_by_value = vb > 0 && !stable;
  job.reverse_first = vb > 0 && stable && desc;
  job.first_unstable = !(vb > 0 && stable);
  job.work = ctx->work;
  job.err = ctx->err;
  job.spin_limit = ctx->spin_limit;
  job.inject_stall = ctx->inject_stall;
  job.shape = pass_shape_for(ctx, kb, kkind, vb, n);
  return job;
}

}  // namespace gs

using namespace gs;

namespace {

constexpr uint64_t MAX_N = 0xFFFFFFFFull;  // 32-bit bin counters

// Device copies the upsweep makes of a host call's pinned input, which it
// reads directly across the CPU-GPU link (see sort_common).
struct HostFuse {
  void* keys_copy = nullptr;
  void* vals_copy = nullptr;
};

// Device-memory radix sort of keys or pairs.
gs_status device_sort(gs_ctx* ctx, int kb, uint32_t kkind, int vb, uint32_t vkind,
                      const void* kin, const void* vin, void* kout, void* vout,
                      uint64_t n, uint32_t flags, const HostFuse* fuse = nullptr) {
  const bool desc = flags & GS_FLAG_DESCENDING;
  // Few keys and no payload: one CTA sorts them in shared memory (one launch
  // instead of the radix pipeline's five). An explicit pass shape, timing
  // marks or an injected stall ask for the radix pipeline itself.
  if (vb == 0 && n <= gs::small_sort_max() && ctx->shape < 0 && !ctx->timing &&
      !ctx->inject_stall) {
    // (With pinned host input, kin is its device mapping: the CTA reads it
    // across the link directly.)
    cudaError_t e = gs::launch_small_sort(kin, kout, uint32_t(n), kb, kkind, desc, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "small sort launch");
    return GS_OK;
  }
  gs::RadixJob job = radix_job(ctx, kb, kkind, vb, vkind, n, flags);
  job.keys_in = kin;
  job.keys_out = kout;
  job.vals_in = vin;
  job.vals_out = vout;
  if (fuse) {
    job.keys_copy = fuse->keys_copy;
    job.vals_copy = fuse->vals_copy;
  }
  ctx->inject_stall = 0;

  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st != GS_OK) return st;
  job.keys_alt = ctx->alt_k.ptr;
  if (vb) {
    st = ensure(ctx, ctx->alt_v, size_t(n) * vb);
    if (st != GS_OK) return st;
    job.vals_alt = ctx->alt_v.ptr;
  }
  st = prepare_status(ctx, gs::radix_status_words(n, kb, vb));
  if (st != GS_OK) return st;
  job.status = static_cast<uint64_t*>(ctx->status.ptr);
  if (ctx->timing) {
    job.marks = ctx->kev;
    ctx->n_kev = 3 + int(kb + (job.ties_by_value ? vb : 0));
  }
  cudaError_t e = gs::launch_radix_sort(job, ctx->props, &ctx->gen, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "radix sort launch");
  return GS_OK;
}

// Sort each of the given segments of `in` into `out` (keys only; `scratch`
// holds n keys and differs from both; in == out sorts in place); waits.
gs_status sort_segments(gs_ctx* ctx, int kb, uint32_t kk, bool desc, const void* in, void* out,
                        void* scratch, uint64_t n, const std::vector<uint64_t>& off) {
  gs_seg_plan* pl = gs::seg_plan_new();
  const std::string err = gs::seg_plan_build(pl, off.data(), uint32_t(off.size() - 1), n, kb, kk,
                                             desc,
                                             gs::radix_segmented_shape(kb, n, uint32_t(off.size() - 1)));
  if (!err.empty()) {
    gs::seg_plan_free(pl);
    return fail(ctx, GS_ERR_OOM, err);
  }
  gs_status st =
      prepare_status(ctx, size_t(gs::seg_plan_large_tiles(pl)) * gs::RADIX + gs::RADIX);
  if (st == GS_OK) {
    cudaError_t e = gs::seg_plan_run(pl, in, out, scratch, static_cast<uint64_t*>(ctx->status.ptr),
                                     &ctx->work->gen_counter, ctx->err, ctx->spin_limit,
                                     ctx->props, ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "segment sort launch");
  }
  cudaStreamSynchronize(ctx->stream);
  gs::seg_plan_free(pl);
  return st;
}

// SampleSort shape (keys only): splitters from an oversampled sample,
// bucket scatter into p partitions, each partition sorted on its own.
gs_status sample_sort_device(gs_ctx* ctx, int kb, uint32_t kk, const void* in, void* out,
                             uint64_t n, uint32_t flags, const gs_opts* o) {
  uint32_t p = partitions_for(ctx, kb, kk, n, o);
  uint32_t os = (o && o->oversample) ? o->oversample : 32;
  if (p > gs::RADIX) p = gs::RADIX;
  if (p < 2) p = 2;
  uint32_t samples = p * os;
  if (samples > 8192) samples = 8192;
  if (samples < p) samples = p;
  const bool desc = flags & GS_FLAG_DESCENDING;
  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st == GS_OK) st = ensure(ctx, ctx->splitters, gs::RADIX * 8);
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, 0));
  if (st != GS_OK) return st;
  const void* src = in;
  if (in == out) {  // the bucket pass must not write its own input
    cudaError_t e = cudaMemcpyAsync(ctx->alt_k.ptr, in, size_t(n) * kb, cudaMemcpyDeviceToDevice,
                                    ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy");
    src = ctx->alt_k.ptr;
  }
  gs::RadixJob job;
  job.keys_in = src;
  job.keys_out = out;
  job.keys_alt = ctx->alt_k.ptr;
  job.n = n;
  job.key_bytes = kb;
  job.key_kind = kk;
  job.desc = desc;
  job.first_unstable = true;
  job.status = static_cast<uint64_t*>(ctx->status.ptr);
  job.work = ctx->work;
  job.err = ctx->err;
  job.spin_limit = ctx->spin_limit;
  gs::SampleJob sj{p, samples, o ? o->seed : 0, ctx->splitters.ptr};
  cudaError_t e = gs::launch_sample_bucketing(job, sj, ctx->props, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "sample bucketing launch");
  std::vector<uint32_t> counts(p);
  e = cudaMemcpyAsync(counts.data(), &ctx->work->hist[0][0], p * 4, cudaMemcpyDeviceToHost,
                      ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "bucket sizes");
  std::vector<uint64_t> off(p + 1, 0);
  for (uint32_t i = 0; i < p; ++i) off[i + 1] = off[i] + counts[i];
  if (off[p] != n) return fail(ctx, GS_ERR_CUDA, "bucket sizes do not add up to n");
  phase_mark(ctx, "Exchange data");
  return sort_segments(ctx, kb, kk, desc, out, out, ctx->alt_k.ptr, n, off);
}

// HykSort shape (keys only), the reference's algorithm on p partitions of
// one array (include/helpers/hyksort_helper.h:94-145 and 453-536): the
// partitions (the ranks' data, n/p keys each) are sorted on their own, then
// log_k(p) rounds each select k-1 splitters per group of ranks, cut every
// rank's run at them and merge every receiving rank's k pieces in one pass
// (hyk.cu). p and k must be powers of two, else the reference runs
// SampleSort (include/hyksort_common_vector.inl:31-43); k larger than the
// group is reduced to the group size (hyksort_helper.h:462).
gs_status hyk_sort_device(gs_ctx* ctx, int kb, uint32_t kk, const void* in, void* out,
                          uint64_t n, uint32_t flags, const gs_opts* o) {
  const uint32_t p = (o && o->partitions) ? o->partitions : 4;
  const uint32_t k = (o && o->k_way) ? o->k_way : 4;
  const bool pow2 = p && !(p & (p - 1)) && k && !(k & (k - 1));
  if (!pow2) return sample_sort_device(ctx, kb, kk, in, out, n, flags, o);
  if (p > gs::HYK_MAX_RANKS || k < 2 || k > gs::MAX_KWAY)
    return fail(ctx, GS_ERR_INVALID, "HykSort shape: at most " + std::to_string(gs::HYK_MAX_RANKS) +
                                         " partitions and 2 <= k_way <= " +
                                         std::to_string(gs::MAX_KWAY));
  const bool desc = flags & GS_FLAG_DESCENDING;
  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st != GS_OK) return st;
  uint32_t rounds = 0;
  for (uint32_t np = p; np > 1; np /= std::min(k, np)) ++rounds;
  // The rounds alternate between the output and the scratch buffer; the
  // local sorts write the one that makes the last round land in `out` (in
  // place they write `out`, and an odd round count ends with a copy).
  const bool in_place = in == out;
  void* alt = ctx->alt_k.ptr;
  void* cur = (in_place || rounds % 2 == 0) ? out : alt;
  std::vector<uint64_t> roff(p + 1);
  const uint64_t run = (n + p - 1) / p;
  for (uint32_t i = 0; i <= p; ++i) roff[i] = std::min<uint64_t>(uint64_t(i) * run, n);
  st = sort_segments(ctx, kb, kk, desc, in, cur, cur == out ? alt : out, n, roff);
  if (st != GS_OK) return st;
  phase_mark(ctx, "Local sort");
  if (rounds == 0) return GS_OK;

  // Device scratch: rank offsets, splitters, selection rounds, cuts, pieces
  // (fixed sizes), then the merge samples (grown per round).
  const uint32_t kmax = std::min(k, p);
  const size_t b_roff = size_t(p + 1) * 8, b_split = size_t(p) * gs::MAX_KWAY * 8,
               b_iters = size_t(p) * 4, b_cuts = size_t(p) * (kmax + 1) * 8,
               b_pieces = size_t(p) * kmax * sizeof(gs::HykPiece);
  auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
  st = ensure(ctx, ctx->hyk_small, al(b_roff) + al(b_split) + al(b_iters) + al(b_cuts) +
                                       al(b_pieces) + al(b_roff));
  if (st != GS_OK) return st;
  uint8_t* sm = static_cast<uint8_t*>(ctx->hyk_small.ptr);
  uint64_t* d_roff = reinterpret_cast<uint64_t*>(sm);
  void* d_split = sm + al(b_roff);
  uint32_t* d_iters = reinterpret_cast<uint32_t*>(sm + al(b_roff) + al(b_split));
  uint64_t* d_cuts = reinterpret_cast<uint64_t*>(sm + al(b_roff) + al(b_split) + al(b_iters));
  gs::HykPiece* d_pieces = reinterpret_cast<gs::HykPiece*>(sm + al(b_roff) + al(b_split) +
                                                            al(b_iters) + al(b_cuts));
  uint64_t* d_rtile = reinterpret_cast<uint64_t*>(sm + al(b_roff) + al(b_split) + al(b_iters) +
                                                  al(b_cuts) + al(b_pieces));
  const uint64_t span = gs::hyk_tile_span(kb);
  const uint64_t seed = o ? o->seed : 0;
  uint32_t np = p;
  for (uint32_t round = 0; np > 1; ++round) {
    gs::HykRound r;
    r.kway = std::min(k, np);
    r.data = cur;
    r.roff = d_roff;
    r.p = p;
    r.n_p = np;
    r.key_bytes = kb;
    r.key_kind = kk;
    r.desc = desc;
    r.seed = seed * 0x9E3779B97F4A7C15ull + round;
    r.splitters = d_split;
    r.iters = d_iters;
    r.cuts = d_cuts;
    if (gs::hyk_select_smem(kb, np, r.kway) > ctx->props.smem_optin)
      return fail(ctx, GS_ERR_INVALID, "HykSort shape: splitter selection does not fit shared memory");
    cudaError_t e = cudaMemcpyAsync(d_roff, roff.data(), b_roff, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = gs::launch_hyk_select(r, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "splitter selection launch");
    std::vector<uint64_t> cuts(size_t(p) * (r.kway + 1));
    e = cudaMemcpyAsync(cuts.data(), d_cuts, cuts.size() * 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "splitter selection");
    phase_mark(ctx, "Select splitters");
    // Rank g*np + b*blk + q receives piece b of ranks g*np + i*blk + q
    // (hyksort_helper.h:555-600: partner = blk_size * i + new_pid).
    const uint32_t blk = np / r.kway;
    const uint32_t stride = gs::hyk_sample_stride(kb, r.kway);
    std::vector<gs::HykPiece> pieces(size_t(p) * r.kway);
    std::vector<uint64_t> noff(p + 1, 0);
    uint64_t nsamples = 0;
    for (uint32_t rr = 0; rr < p; ++rr) {
      const uint32_t g = rr / np, b = (rr % np) / blk, q = rr % blk;
      uint64_t len = 0;
      for (uint32_t i = 0; i < r.kway; ++i) {
        const uint32_t from = g * np + i * blk + q;
        const uint64_t* c = &cuts[size_t(from) * (r.kway + 1)];
        gs::HykPiece& pc = pieces[size_t(rr) * r.kway + i];
        pc.src = roff[from] + c[b];
        pc.len = c[b + 1] - c[b];
        pc.sample0 = nsamples;
        pc.out = noff[rr];
        pc.first = rr * r.kway;
        pc.j = i;
        nsamples += (pc.len + stride - 1) / stride;
        len += pc.len;
      }
      noff[rr + 1] = noff[rr] + len;
    }
    if (noff[p] != n) return fail(ctx, GS_ERR_CUDA, "HykSort shape: pieces do not add up to n");
    // Merge tiles: ceil(length / span) per receiving rank.
    std::vector<uint64_t> rtile(p + 1, 0);
    for (uint32_t rr = 0; rr < p; ++rr)
      rtile[rr + 1] = rtile[rr] + (noff[rr + 1] - noff[rr] + span - 1) / span;
    const uint64_t ntiles = rtile[p];
    const size_t ns = size_t(nsamples), nt = size_t(ntiles), kw = r.kway;
    st = ensure(ctx, ctx->hyk_samples, al(ns * 8) + al(ns * kw * 8) + al(nt * 8) +
                                           al(nt * kw * 8) + al(nt * kw * 4) + 256);
    if (st != GS_OK) return st;
    uint8_t* sp = static_cast<uint8_t*>(ctx->hyk_samples.ptr);
    r.samp_rank = reinterpret_cast<uint64_t*>(sp);
    r.samp_cut = reinterpret_cast<uint64_t*>(sp + al(ns * 8));
    r.tile_out = reinterpret_cast<uint64_t*>(sp + al(ns * 8) + al(ns * kw * 8));
    r.tile_src = reinterpret_cast<uint64_t*>(sp + al(ns * 8) + al(ns * kw * 8) + al(nt * 8));
    r.tile_len = reinterpret_cast<uint32_t*>(sp + al(ns * 8) + al(ns * kw * 8) + al(nt * 8) +
                                             al(nt * kw * 8));
    r.err = ctx->err;
    e = cudaMemcpyAsync(d_pieces, pieces.data(), pieces.size() * sizeof(gs::HykPiece),
                        cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d_rtile, rtile.data(), b_roff, cudaMemcpyHostToDevice, ctx->stream);
    void* next = cur == out ? alt : out;
    if (e == cudaSuccess)
      e = gs::launch_hyk_merge(r, d_pieces, uint32_t(pieces.size()), nsamples, d_rtile, ntiles,
                               cur, next, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);  // pieces and cuts are reused
    if (e != cudaSuccess) return cuda_fail(ctx, e, "k-way merge");
    phase_mark(ctx, "Merge data");
    roff.swap(noff);
    cur = next;
    np = blk;
  }
  if (cur != out) {
    cudaError_t e = cudaMemcpyAsync(out, cur, size_t(n) * kb, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy");
  }
  return GS_OK;
}

// Strategy selection: SampleSort / HykSort shapes for keys, radix otherwise
// (every strategy gives the same bytes).
gs_status dispatch_sort(gs_ctx* ctx, int kb, uint32_t kk, int vb, uint32_t vk, const void* kin,
                        const void* vin, void* kout, void* vout, uint64_t n, uint32_t flags,
                        const gs_opts* opts) {
  const uint32_t algo = opts ? opts->algo : GS_ALGO_AUTO;
  if (vb == 0 && n >= 4096 && algo == GS_ALGO_SAMPLE)
    return sample_sort_device(ctx, kb, kk, kin, kout, n, flags, opts);
  if (vb == 0 && n >= 4096 && algo == GS_ALGO_HYK)
    return hyk_sort_device(ctx, kb, kk, kin, kout, n, flags, opts);
  return device_sort(ctx, kb, kk, vb, vk, kin, vin, kout, vout, n, flags);
}

gs_status sort_common(gs_ctx* ctx, gs_dtype kt, int has_v, gs_dtype vt, const void* kin,
                      const void* vin, void* kout, void* vout, uint64_t n, uint32_t flags,
                      const gs_opts* opts) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  int kb = 0, vb = 0;
  uint32_t kk = 0, vk = 0;
  if (!dtype_info(kt, &kb, &kk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (has_v && !dtype_info(vt, &vb, &vk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown value dtype");
  if (n == 0) return fail(ctx, GS_ERR_EMPTY, "No data to sort.");
  if (n > MAX_N) return fail(ctx, GS_ERR_TOO_LARGE, "n exceeds 2^32-1 elements");
  if (!kin || !kout || (has_v && (!vin || !vout)))
    return fail(ctx, GS_ERR_INVALID, "null data pointer");
  cudaError_t e = cudaSetDevice(ctx->props.device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  phase_reset(ctx);

  if (flags & GS_FLAG_HOST) {
    gs_status st = ensure(ctx, ctx->stage_k, size_t(n) * kb);
    if (st != GS_OK) return st;
    if (has_v) {
      st = ensure(ctx, ctx->stage_v, size_t(n) * vb);
      if (st != GS_OK) return st;
    }
    // Pinned host input on the radix path: the upsweep reads it across the
    // CPU-GPU link once and keeps a device copy for the passes, so the
    // transfer in overlaps the histogram kernel. (Writing the last pass's
    // scatter straight into pinned host output measured slower on GB300
    // than sorting in HBM and copying out: 70.6 vs 61.0 ms for 2^30 keys.)
    const uint32_t algo = opts ? opts->algo : GS_ALGO_AUTO;
    const bool radix_path = has_v || n < 4096 || (algo != GS_ALGO_SAMPLE && algo != GS_ALGO_HYK);
    const void* mk = mapped_host(kin);
    const void* mv = has_v ? mapped_host(vin) : nullptr;
    const uint32_t groups = host_groups_for(ctx, n);
    if (radix_path && mk && (!has_v || mv) && groups > 1 && mapped_host(kout) &&
        (!has_v || mapped_host(vout))) {
      if (!has_v && ctx->host_chunked_min && n >= ctx->host_chunked_min)
        return host_groups_chunked(ctx, kb, kk, mk, kout, n, flags, groups);
      return host_groups_sort(ctx, kb, kk, vb, vk, mk, mv, kout, vout, n, flags, groups);
    }
    if (radix_path && mk && (!has_v || mv)) {
      HostFuse fu;
      fu.keys_copy = ctx->stage_k.ptr;
      fu.vals_copy = has_v ? ctx->stage_v.ptr : nullptr;
      st = device_sort(ctx, kb, kk, vb, vk, mk, mv, ctx->stage_k.ptr,
                       has_v ? ctx->stage_v.ptr : nullptr, n, flags, &fu);
      if (st != GS_OK) return st;
      phase_mark(ctx, "Local sort");
      e = link_copy(ctx, kout, ctx->stage_k.ptr, uint64_t(n) * kb, false);
      if (e == cudaSuccess && has_v) e = link_copy(ctx, vout, ctx->stage_v.ptr, uint64_t(n) * vb, false);
      if (e != cudaSuccess) return cuda_fail(ctx, e, "device to host copy");
      phase_mark(ctx, "Transfer out");
      return check_err_word(ctx);
    }
    e = link_copy(ctx, ctx->stage_k.ptr, kin, uint64_t(n) * kb, true);
    if (e == cudaSuccess && has_v) e = link_copy(ctx, ctx->stage_v.ptr, vin, uint64_t(n) * vb, true);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "host to device copy");
    phase_mark(ctx, "Transfer in");
    st = dispatch_sort(ctx, kb, kk, vb, vk, ctx->stage_k.ptr, has_v ? ctx->stage_v.ptr : nullptr,
                       ctx->stage_k.ptr, has_v ? ctx->stage_v.ptr : nullptr, n, flags, opts);
    if (st != GS_OK) return st;
    phase_mark(ctx, "Local sort");
    e = link_copy(ctx, kout, ctx->stage_k.ptr, uint64_t(n) * kb, false);
    if (e == cudaSuccess && has_v) e = link_copy(ctx, vout, ctx->stage_v.ptr, uint64_t(n) * vb, false);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "device to host copy");
    phase_mark(ctx, "Transfer out");
    return check_err_word(ctx);
  }

  gs_status st = dispatch_sort(ctx, kb, kk, vb, vk, kin, has_v ? vin : nullptr, kout,
                               has_v ? vout : nullptr, n, flags, opts);
  if (st != GS_OK) return st;
  phase_mark(ctx, "Local sort");
  if (flags & GS_FLAG_SYNC) return check_err_word(ctx);
  return GS_OK;
}

__global__ void gather_kernel(const uint8_t* __restrict__ in, uint8_t* __restrict__ out,
                              uint64_t n, uint32_t eb, const uint64_t* __restrict__ perm) {
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride) {
    const uint64_t s = perm[i];
    if (s >= n) continue;
    if (eb == 4) {
      reinterpret_cast<uint32_t*>(out)[i] = reinterpret_cast<const uint32_t*>(in)[s];
    } else if (eb == 8) {
      reinterpret_cast<uint64_t*>(out)[i] = reinterpret_cast<const uint64_t*>(in)[s];
    } else {
      for (uint32_t b = 0; b < eb; ++b) out[i * eb + b] = in[s * eb + b];
    }
  }
}

}  // namespace

extern "C" {

uint32_t gs_version(void) { return 0x000100u; }

int gs_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

const char* gs_last_global_error(void) { return g_last_global_error.c_str(); }

const char* gs_last_error(gs_ctx* ctx) {
  if (!ctx) return g_last_global_error.c_str();
  return ctx->last_error.c_str();
}

gs_ctx* gs_ctx_create(int device, uint64_t hbm_budget_bytes) {
  int ndev = gs_device_count();
  if (ndev == 0) {
    g_last_global_error = "No CUDA-capable devices were detected";
    return nullptr;
  }
  if (device < 0 || device >= ndev) {
    g_last_global_error = "invalid device ordinal";
    return nullptr;
  }
  if (cudaSetDevice(device) != cudaSuccess) {
    g_last_global_error = "cudaSetDevice failed";
    return nullptr;
  }
  gs_ctx* ctx = new gs_ctx();
  ctx->props.device = device;
  cudaDeviceGetAttribute(&ctx->props.num_sms, cudaDevAttrMultiProcessorCount, device);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  ctx->props.smem_optin = size_t(optin);
  ctx->budget = hbm_budget_bytes;
  if (cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    g_last_global_error = "cudaStreamCreate failed";
    delete ctx;
    return nullptr;
  }
  ctx->stream = ctx->own_stream;
  if (cudaMalloc(&ctx->work, gs::sort_work_bytes()) != cudaSuccess ||
      cudaMalloc(&ctx->err, 256) != cudaSuccess) {
    g_last_global_error = "cudaMalloc of the context's work area failed";
    cudaGetLastError();
    gs_ctx_destroy(ctx);
    return nullptr;
  }
  ctx->held += gs::sort_work_bytes() + 256;
  cudaMemsetAsync(ctx->err, 0, 256, ctx->stream);
  cudaMemsetAsync(ctx->work, 0, gs::sort_work_bytes(), ctx->stream);
  for (auto& ev : ctx->ev) cudaEventCreate(&ev);
  for (auto& ev : ctx->kev) cudaEventCreate(&ev);
  cudaStreamSynchronize(ctx->stream);
  return ctx;
}

void gs_ctx_destroy(gs_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->props.device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  DevBuf* bufs[] = {&ctx->status, &ctx->alt_k, &ctx->alt_v, &ctx->stage_k, &ctx->stage_v,
                    &ctx->stage_off, &ctx->splitters, &ctx->hyk_small, &ctx->hyk_samples,
                    &ctx->third_k};
  for (DevBuf* b : bufs) if (b->ptr) cudaFree(b->ptr);
  if (ctx->work) cudaFree(ctx->work);
  if (ctx->err) cudaFree(ctx->err);
  for (auto& ev : ctx->ev) if (ev) cudaEventDestroy(ev);
  for (auto& ev : ctx->kev) if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : {ctx->ev_hist, ctx->ev_group, ctx->ev_copied}) if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : ctx->ev_chunk_in) if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : ctx->ev_chunk_split) if (ev) cudaEventDestroy(ev);
  for (cudaStream_t cs : {ctx->copy_stream, ctx->split_stream}) {
    if (!cs) continue;
    cudaStreamSynchronize(cs);
    cudaStreamDestroy(cs);
  }
  if (ctx->work2) cudaFree(ctx->work2);
  if (ctx->h_hist) cudaFreeHost(ctx->h_hist);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  delete ctx;
}

gs_status gs_ctx_set_stream(gs_ctx* ctx, void* stream) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->stream = static_cast<cudaStream_t>(stream);  // NULL: the legacy default stream
  return GS_OK;
}

gs_status gs_ctx_synchronize(gs_ctx* ctx) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaSetDevice(ctx->props.device);
  return check_err_word(ctx);
}

gs_status gs_sort_keys(gs_ctx* ctx, gs_dtype dtype, const void* in, void* out, uint64_t n,
                       uint32_t flags, const gs_opts* opts) {
  return sort_common(ctx, dtype, 0, GS_U32, in, nullptr, out, nullptr, n, flags, opts);
}

gs_status gs_sort_pairs(gs_ctx* ctx, gs_dtype key_dtype, gs_dtype val_dtype, const void* keys_in,
                        const void* vals_in, void* keys_out, void* vals_out, uint64_t n,
                        uint32_t flags, const gs_opts* opts) {
  return sort_common(ctx, key_dtype, 1, val_dtype, keys_in, vals_in, keys_out, vals_out, n, flags,
                     opts);
}

gs_status gs_segmented_plan_create(gs_ctx* ctx, gs_dtype dtype, uint64_t n,
                                   const uint64_t* host_offsets, uint32_t nseg, uint32_t flags,
                                   gs_seg_plan** plan) {
  if (!ctx || !plan) return fail(ctx, GS_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(ctx->mu);
  *plan = nullptr;
  int kb = 0;
  uint32_t kk = 0;
  if (!dtype_info(dtype, &kb, &kk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (n > MAX_N) return fail(ctx, GS_ERR_TOO_LARGE, "n exceeds 2^32-1 elements");
  if (!host_offsets) return fail(ctx, GS_ERR_INVALID, "null offsets");
  cudaSetDevice(ctx->props.device);
  gs_seg_plan* pl = gs::seg_plan_new();
  const int shape = ctx->shape >= 0 ? ctx->shape : gs::radix_segmented_shape(kb, n, nseg);
  const std::string err = gs::seg_plan_build(pl, host_offsets, nseg, n, kb, kk,
                                             (flags & GS_FLAG_DESCENDING) != 0, shape);
  if (!err.empty()) {
    gs::seg_plan_free(pl);
    return fail(ctx, err.find("allocation") != std::string::npos ? GS_ERR_OOM : GS_ERR_INVALID,
                err);
  }
  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st == GS_OK)
    st = prepare_status(ctx, size_t(gs::seg_plan_large_tiles(pl)) * gs::RADIX + gs::RADIX);
  if (st != GS_OK) {
    gs::seg_plan_free(pl);
    return st;
  }
  cudaStreamSynchronize(ctx->stream);
  *plan = pl;
  return GS_OK;
}

gs_status gs_segmented_layout(gs_dtype dtype, uint64_t n, const uint64_t* host_offsets,
                              uint32_t nseg, uint8_t* kinds, uint64_t counts[4]) {
  int kb = 0;
  uint32_t kk = 0;
  if (!dtype_info(dtype, &kb, &kk)) return fail(nullptr, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (n > MAX_N) return fail(nullptr, GS_ERR_TOO_LARGE, "n exceeds 2^32-1 elements");
  if (!host_offsets || !counts) return fail(nullptr, GS_ERR_INVALID, "null argument");
  const int shape = gs::radix_segmented_shape(kb, n, nseg);
  const std::string err =
      gs::seg_layout_summary(host_offsets, nseg, n, gs::radix_shape_tile(kb, 0, shape), kinds, counts);
  if (!err.empty()) return fail(nullptr, GS_ERR_INVALID, err);
  return GS_OK;
}

gs_status gs_segmented_plan_run(gs_ctx* ctx, const gs_seg_plan* plan, const void* in, void* out) {
  if (!ctx || !plan) return fail(ctx, GS_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (gs::seg_plan_n(plan) == 0) return GS_OK;
  if (!in || !out) return fail(ctx, GS_ERR_INVALID, "null data pointer");
  if (ctx->alt_k.bytes < gs::seg_plan_n(plan) * gs::seg_plan_key_bytes(plan))
    return fail(ctx, GS_ERR_INVALID, "context scratch was not sized for this plan");
  cudaError_t e = gs::seg_plan_run(plan, in, out, ctx->alt_k.ptr,
                                   static_cast<uint64_t*>(ctx->status.ptr),
                                   &ctx->work->gen_counter, ctx->err, ctx->spin_limit,
                                   ctx->props, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "segmented sort launch");
  return GS_OK;
}

void gs_segmented_plan_destroy(gs_seg_plan* plan) {
  if (plan) gs::seg_plan_free(plan);
}

gs_status gs_segmented_sort_keys(gs_ctx* ctx, gs_dtype dtype, const void* in, void* out,
                                 uint64_t n, const uint64_t* offsets, uint32_t nseg,
                                 uint32_t flags) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  int kb = 0;
  uint32_t kk = 0;
  if (!dtype_info(dtype, &kb, &kk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (!offsets) return fail(ctx, GS_ERR_INVALID, "null offsets");
  if (n == 0) return GS_OK;
  if (!in || !out) return fail(ctx, GS_ERR_INVALID, "null data pointer");
  std::vector<uint64_t> host_off;
  const uint64_t* hoff = offsets;
  if (!(flags & GS_FLAG_OFFSETS_HOST)) {
    host_off.resize(size_t(nseg) + 1);
    cudaSetDevice(ctx->props.device);
    cudaError_t e = cudaMemcpy(host_off.data(), offsets, host_off.size() * 8, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "offsets copy");
    hoff = host_off.data();
  }
  gs_seg_plan* plan = nullptr;
  gs_status st = gs_segmented_plan_create(ctx, dtype, n, hoff, nseg, flags, &plan);
  if (st != GS_OK) return st;
  const void* din = in;
  void* dout = out;
  if (flags & GS_FLAG_HOST) {
    std::lock_guard<std::mutex> lock(ctx->mu);
    st = ensure(ctx, ctx->stage_k, size_t(n) * kb);
    if (st == GS_OK) {
      cudaError_t e = cudaMemcpyAsync(ctx->stage_k.ptr, in, size_t(n) * kb,
                                      cudaMemcpyHostToDevice, ctx->stream);
      if (e != cudaSuccess) st = cuda_fail(ctx, e, "host to device copy");
    }
    din = dout = ctx->stage_k.ptr;
  }
  if (st == GS_OK) st = gs_segmented_plan_run(ctx, plan, din, dout);
  if (st == GS_OK && (flags & GS_FLAG_HOST)) {
    cudaError_t e = cudaMemcpyAsync(out, ctx->stage_k.ptr, size_t(n) * kb,
                                    cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) st = cuda_fail(ctx, e, "device to host copy");
  }
  if (st == GS_OK) {
    std::lock_guard<std::mutex> lock(ctx->mu);
    st = check_err_word(ctx);
  } else {
    cudaStreamSynchronize(ctx->stream);
  }
  gs_segmented_plan_destroy(plan);
  return st;
}

gs_status gs_gather(gs_ctx* ctx, const void* in, void* out, uint64_t n, uint32_t elem_bytes,
                    const uint64_t* perm, uint32_t flags) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (n == 0) return GS_OK;
  if (!in || !out || !perm || elem_bytes == 0 || elem_bytes > 64)
    return fail(ctx, GS_ERR_INVALID, "bad gather arguments");
  cudaSetDevice(ctx->props.device);
  const void* din = in;
  void* dout = out;
  const uint64_t* dperm = perm;
  const size_t bytes = size_t(n) * elem_bytes;
  if (flags & GS_FLAG_HOST) {  // stage: values in stage_k, perm in stage_off, result in alt_k
    gs_status st = ensure(ctx, ctx->stage_k, bytes);
    if (st == GS_OK) st = ensure(ctx, ctx->stage_off, size_t(n) * 8);
    if (st == GS_OK) st = ensure(ctx, ctx->alt_k, bytes);
    if (st != GS_OK) return st;
    cudaError_t e = cudaMemcpyAsync(ctx->stage_k.ptr, in, bytes, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(ctx->stage_off.ptr, perm, size_t(n) * 8, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "host to device copy");
    din = ctx->stage_k.ptr;
    dout = ctx->alt_k.ptr;
    dperm = static_cast<const uint64_t*>(ctx->stage_off.ptr);
  }
  unsigned blocks = unsigned((n + 255) / 256);
  const unsigned cap = unsigned(ctx->props.num_sms) * 8;
  if (blocks > cap) blocks = cap;
  gather_kernel<<<blocks, 256, 0, ctx->stream>>>(static_cast<const uint8_t*>(din),
                                                 static_cast<uint8_t*>(dout), n, elem_bytes, dperm);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(ctx, e, "gather launch");
  if (flags & GS_FLAG_HOST) {
    e = cudaMemcpyAsync(out, dout, bytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "device to host copy");
    return check_err_word(ctx);
  }
  if (flags & GS_FLAG_SYNC) return check_err_word(ctx);
  return GS_OK;
}

int gs_kernel_times(gs_ctx* ctx, double* ms, int cap) {
  if (!ctx || !ctx->timing || ctx->n_kev < 3) return 0;
  std::lock_guard<std::mutex> lock(ctx->mu);
  cudaEventSynchronize(ctx->kev[ctx->n_kev - 1]);
  int k = 0;
  for (int i = 1; i < ctx->n_kev && k < cap; ++i, ++k) {
    float t = 0.f;
    cudaEventElapsedTime(&t, ctx->kev[i - 1], ctx->kev[i]);
    ms[k] = t;
  }
  return ctx->n_kev - 1;
}

int gs_phase_times(gs_ctx* ctx, const char** names, double* ms, int cap) {
  if (!ctx) return 0;
  int n = ctx->n_phases;
  for (int i = 0; i < n && i < cap; ++i) {
    if (names) names[i] = ctx->phase_names[i];
    if (ms) ms[i] = ctx->phase_ms[i];
  }
  return n;
}

gs_status gs_ctx_set_timing(gs_ctx* ctx, int enable) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  ctx->timing = enable != 0;
  return GS_OK;
}

int gs_pass_shape_count(void) { return gs::radix_num_shapes(); }

gs_status gs_pass_shape_info(int key_bytes, int val_bytes, int shape, uint32_t* threads,
                             uint32_t* items_per_thread) {
  uint32_t t = 0, it = 0;
  if (!gs::radix_shape_info(key_bytes, val_bytes, shape, &t, &it))
    return fail(nullptr, GS_ERR_INVALID, "no such pass shape");
  if (threads) *threads = t;
  if (items_per_thread) *items_per_thread = it;
  return GS_OK;
}

gs_status gs_debug_set(gs_ctx* ctx, int key, uint64_t value) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> lock(ctx->mu);
  switch (key) {
    case GS_DEBUG_SPIN_LIMIT: ctx->spin_limit = value ? uint32_t(value) : 1u; return GS_OK;
    case GS_DEBUG_INJECT_STALL: ctx->inject_stall = value ? 1u : 0u; return GS_OK;
    case GS_DEBUG_BUDGET: ctx->budget = value; return GS_OK;
    case GS_DEBUG_PASS_SHAPE:  // UINT64_MAX restores the per-type defaults
      if (value == ~0ull) { ctx->shape = -1; return GS_OK; }
      if (value >= uint64_t(gs::radix_num_shapes())) return fail(ctx, GS_ERR_INVALID, "bad shape");
      ctx->shape = int(value);
      return GS_OK;
    case GS_DEBUG_HOST_CHUNKED: ctx->host_chunked_min = value; return GS_OK;
    case GS_DEBUG_HOST_GROUPS:  // UINT64_MAX restores the choice by size
      if (value == ~0ull) { ctx->host_groups = -1; return GS_OK; }
      if (value > 256) return fail(ctx, GS_ERR_INVALID, "at most 256 groups");
      ctx->host_groups = int(value);
      return GS_OK;
  }
  return fail(ctx, GS_ERR_INVALID, "unknown debug key");
}

}  // extern "C"
