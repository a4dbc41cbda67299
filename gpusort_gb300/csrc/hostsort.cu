// Sorts of host buffers (gs_sort_keys / gs_sort_pairs with GS_FLAG_HOST):
// transfers across the CPU-GPU link, and the bucket-group sorts that
// overlap the sort with the transfer out.
#include <algorithm>
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "context.h"

namespace gs {

// Copy kernel for transfers between device memory and pinned host memory
// that the device addresses directly (cudaHostAlloc, cudaHostRegister): the
// SMs load and store across the CPU-GPU link. Four independent 16-byte
// loads per thread keep enough requests in flight for the link's latency.
__global__ void __launch_bounds__(512) link_copy_kernel(const uint8_t* __restrict__ src,
                                                        uint8_t* __restrict__ dst,
                                                        uint64_t bytes) {
  const uint64_t n16 = bytes / 16;
  const uint4* s = reinterpret_cast<const uint4*>(src);
  uint4* d = reinterpret_cast<uint4*>(dst);
  const uint64_t stride = uint64_t(gridDim.x) * blockDim.x;
  uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (; i + 3 * stride < n16; i += 4 * stride) {
    const uint4 a = s[i], b = s[i + stride], c = s[i + 2 * stride], e = s[i + 3 * stride];
    d[i] = a;
    d[i + stride] = b;
    d[i + 2 * stride] = c;
    d[i + 3 * stride] = e;
  }
  for (; i < n16; i += stride) d[i] = s[i];
  if (blockIdx.x == 0 && threadIdx.x < (bytes & 15u)) dst[n16 * 16 + threadIdx.x] = src[n16 * 16 + threadIdx.x];
}

// The device address of pinned, device-mapped host memory, or null.
const void* mapped_host(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Host <-> device transfer on the context's stream. Pinned host memory the
// device can address, with both ends 16-byte aligned, moves through the SMs:
// on GB300 that sustained about 200 GB/s each way, while the copy engine
// gave between 56 and 200 GB/s for the same buffers. Everything else goes
// through cudaMemcpyAsync.
cudaError_t link_copy(gs_ctx* ctx, void* dst, const void* src, uint64_t bytes, bool to_device) {
  if (bytes == 0) return cudaSuccess;
  const void* host = to_device ? src : dst;
  const void* mapped = mapped_host(host);
  const bool aligned = ((reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) & 15u) == 0;
  if (!mapped || !aligned)
    return cudaMemcpyAsync(dst, src, bytes,
                           to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, ctx->stream);
  const uint8_t* s = static_cast<const uint8_t*>(to_device ? mapped : src);
  uint8_t* d = static_cast<uint8_t*>(to_device ? dst : const_cast<void*>(mapped));
  const unsigned blocks = unsigned(std::max(1, ctx->props.num_sms) * 2);
  link_copy_kernel<<<blocks, 512, 0, ctx->stream>>>(s, d, bytes);
  return cudaGetLastError();
}

// Bucket groups of a host sort of n elements (below 2: not grouped).
// Measured on GB300, 2^30 u32 keys with pinned buffers: 58.7 ms ungrouped,
// 50.1 / 48.0 / 47.0 / 48.0 ms with 4 / 8 / 16 / 32 groups; 2^26 keys: 3.76
// ms ungrouped, 3.26 with 4 or 8 groups; at 2^24 and below the grouped
// path is slower (per-group launches and host round trip).
uint32_t host_groups_for(const gs_ctx* ctx, uint64_t n) {
  if (ctx->host_groups >= 0) return n >= 4096 ? uint32_t(ctx->host_groups) : 0u;
  if (n >= (uint64_t(1) << 29)) return 24;
  if (n >= (uint64_t(1) << 28)) return 16;
  if (n >= (uint64_t(1) << 26)) return 8;
  if (n >= (uint64_t(1) << 25)) return 4;
  return 0;
}

namespace {

// A run of whole buckets: elements [begin, end), and whether more than one
// bucket holds elements.
struct BucketRun {
  uint64_t begin, end;
  bool mixed;
};

// Runs of whole buckets of `counts` (one digit's histogram, in output
// order) holding about n / groups elements each.
std::vector<BucketRun> bucket_groups(const uint32_t* counts, uint64_t n, uint32_t groups) {
  std::vector<BucketRun> out;
  uint64_t begin = 0, acc = 0;
  uint32_t filled = 0;
  for (uint32_t b = 0; b < gs::RADIX; ++b) {
    acc += counts[b];
    filled += counts[b] != 0;
    const bool close = b + 1 == uint32_t(gs::RADIX) ||
                       acc * groups >= (uint64_t(out.size()) + 1) * n;
    if (close && acc > begin) {
      out.push_back({begin, acc, filled > 1});
      begin = acc;
      filled = 0;
    }
  }
  return out;
}

// Host sorts in bucket groups: the stream, events and host memory they use,
// made on first use.
gs_status host_groups_setup(gs_ctx* ctx) {
  if (ctx->copy_stream) return GS_OK;
  cudaError_t e = cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&ctx->split_stream, cudaStreamNonBlocking);
  for (cudaEvent_t* ev : {&ctx->ev_hist, &ctx->ev_group, &ctx->ev_copied})
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(ev, cudaEventDisableTiming);
  for (uint32_t c = 0; c < HOST_CHUNKS && e == cudaSuccess; ++c) {
    e = cudaEventCreateWithFlags(&ctx->ev_chunk_in[c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_chunk_split[c], cudaEventDisableTiming);
  }
  if (e == cudaSuccess)
    e = cudaHostAlloc(reinterpret_cast<void**>(&ctx->h_hist),
                      sizeof(uint32_t) * gs::HIST_WORDS * HOST_CHUNKS, cudaHostAllocDefault);
  if (e == cudaSuccess) e = cudaMalloc(&ctx->work2, gs::sort_work_bytes());
  if (e == cudaSuccess) e = cudaMemset(ctx->work2, 0, gs::sort_work_bytes());
  if (e != cudaSuccess) return cuda_fail(ctx, e, "host-sort stream setup");
  ctx->held += gs::sort_work_bytes();
  return GS_OK;
}

// The most significant digit of a histogram set (digits x 256 counts of n
// elements) whose elements do not all share a bin; every digit above it is
// constant. Every element equal: the top digit.
uint32_t split_digit(const uint32_t* hist, uint32_t digits, uint64_t n) {
  for (uint32_t q = digits; q-- > 0;) {
    const uint32_t* h = hist + size_t(q) * gs::RADIX;
    if (!std::any_of(h, h + gs::RADIX, [&](uint32_t c) { return uint64_t(c) == n; })) return q;
  }
  return digits - 1;
}

// Sort each run of buckets and copy it to the host on the copy stream while
// the next run sorts. Each run's elements lie at [begin, end) of `in_k`
// (and `in_v`), split by digit t; `gather` (optional) puts them there first.
// `other_k` is free over the same range. A run of one bucket is sorted on
// the digits below t; a run of several on the digits up to t, since LSD
// passes on the lower digits alone would undo the split's order (the last
// pass, on t, restores it with the lower digits as the tie order). With an
// odd digit count a run writes its range of `other`, its own range serving
// as the alternate buffer; with an even count it sorts in place with
// `other` as the alternate (the plan keeps the pass count's parity, running
// a digit that needs no reordering as a copy if it must).
gs_status host_runs(gs_ctx* ctx, const gs::RadixJob& base, uint32_t t,
                    const std::vector<BucketRun>& runs, uint8_t* in_k, uint8_t* in_v,
                    uint8_t* other_k, uint8_t* other_v, void* kout, void* vout,
                    const std::function<cudaError_t(const BucketRun&)>& gather) {
  const int kb = base.key_bytes, vb = base.val_bytes;
  auto fail_after_copies = [&](cudaError_t err, const char* where) {
    cudaStreamSynchronize(ctx->copy_stream);
    return cuda_fail(ctx, err, where);
  };
  for (const BucketRun& r : runs) {
    const uint64_t b = r.begin, m = r.end - r.begin;
    const uint32_t hi = r.mixed ? t + 1 : t;
    const uint8_t* res_k = other_k + b * kb;  // where the sorted run ends up
    const uint8_t* res_v = vb ? other_v + b * vb : nullptr;
    cudaError_t e = gather ? gather(r) : cudaSuccess;
    if (e != cudaSuccess) {
    } else if (hi == 0) {
      // One bucket of the lowest digit, every higher digit constant: the
      // split already left the run in order.
      res_k = in_k + b * kb;
      res_v = vb ? in_v + b * vb : nullptr;
    } else if (vb == 0 && m <= gs::small_sort_max()) {
      e = gs::launch_small_sort(in_k + b * kb, other_k + b * kb, uint32_t(m), kb, base.key_kind,
                                base.desc, ctx->stream);
    } else {
      gs::RadixJob g = base;
      g.n = m;
      g.keys_in = in_k + b * kb;
      if (hi & 1u) {
        g.keys_out = other_k + b * kb;
        g.keys_alt = in_k + b * kb;
        g.alt_is_in = true;
      } else {
        g.keys_out = in_k + b * kb;
        g.keys_alt = other_k + b * kb;
        res_k = in_k + b * kb;
      }
      if (vb) {
        g.vals_in = in_v + b * vb;
        g.vals_out = (hi & 1u) ? other_v + b * vb : in_v + b * vb;
        g.vals_alt = (hi & 1u) ? in_v + b * vb : other_v + b * vb;
        res_v = static_cast<const uint8_t*>(g.vals_out);
      }
      g.digit_lo = 0;
      g.digit_hi = hi;
      g.reverse_first = false;  // the split took care of the reversal
      g.inject_stall = 0;
      g.shape = pass_shape_for(ctx, kb, base.key_kind, vb, m);
      e = gs::launch_radix_sort(g, ctx->props, &ctx->gen, ctx->stream);
    }
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_group, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_group, 0);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(static_cast<uint8_t*>(kout) + b * kb, res_k, m * kb,
                          cudaMemcpyDeviceToHost, ctx->copy_stream);
    if (e == cudaSuccess && vb)
      e = cudaMemcpyAsync(static_cast<uint8_t*>(vout) + b * vb, res_v, m * vb,
                          cudaMemcpyDeviceToHost, ctx->copy_stream);
    if (e != cudaSuccess) return fail_after_copies(e, "bucket run launch");
  }
  cudaError_t e = cudaEventRecord(ctx->ev_copied, ctx->copy_stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->ev_copied, 0);
  if (e != cudaSuccess) return fail_after_copies(e, "copy join");
  phase_mark(ctx, "Sort and transfer out");
  return check_err_word(ctx);
}

// The radix job of a host-groups sort (buffers left to the caller).
gs::RadixJob host_base_job(gs_ctx* ctx, int kb, uint32_t kk, int vb, uint32_t vk, uint64_t n,
                           uint32_t flags) {
  gs::RadixJob j = radix_job(ctx, kb, kk, vb, vk, n, flags);
  j.status = static_cast<uint64_t*>(ctx->status.ptr);
  ctx->inject_stall = 0;
  return j;
}

// One split pass on digit t over all n elements: stage -> scratch.
cudaError_t launch_split(gs_ctx* ctx, const gs::RadixJob& base, uint32_t t, uint8_t* sk,
                         uint8_t* sv, uint8_t* ak, uint8_t* av) {
  gs::RadixJob sp = base;
  sp.keys_in = sk;
  sp.vals_in = sv;
  sp.keys_out = ak;
  sp.vals_out = av;
  sp.keys_alt = ak;
  sp.vals_alt = av;
  sp.skip_upsweep = true;
  sp.digit_lo = t;
  sp.digit_hi = t + 1;
  return gs::launch_radix_sort(sp, ctx->props, &ctx->gen, ctx->stream);
}

}  // namespace

// Sort of pinned host buffers in bucket groups, so that the sort overlaps
// the transfer out. The upsweep reads the input across the CPU-GPU link
// into the stage buffer and counts every digit; one pass on the most
// significant digit t that varies splits the elements into its 256 buckets
// (stage -> scratch); then runs of buckets are sorted and copied out one
// after another (host_runs). The order is the one device_sort gives: the
// split pass is stable exactly when the first pass of device_sort would be
// (and reads back to front when that one does), and each run is a whole
// sort on every digit that varies within it.
gs_status host_groups_sort(gs_ctx* ctx, int kb, uint32_t kk, int vb, uint32_t vk, const void* mk,
                           const void* mv, void* kout, void* vout, uint64_t n, uint32_t flags,
                           uint32_t groups) {
  gs_status st = host_groups_setup(ctx);
  if (st == GS_OK) st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st == GS_OK && vb) st = ensure(ctx, ctx->alt_v, size_t(n) * vb);
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, vb));
  if (st != GS_OK) return st;
  uint8_t* sk = static_cast<uint8_t*>(ctx->stage_k.ptr);
  uint8_t* sv = static_cast<uint8_t*>(vb ? ctx->stage_v.ptr : nullptr);
  uint8_t* ak = static_cast<uint8_t*>(ctx->alt_k.ptr);
  uint8_t* av = static_cast<uint8_t*>(vb ? ctx->alt_v.ptr : nullptr);
  const gs::RadixJob base = host_base_job(ctx, kb, kk, vb, vk, n, flags);
  const uint32_t digits = uint32_t(kb + (base.ties_by_value ? vb : 0));

  // Upsweep across the link; histograms back to the host.
  gs::RadixJob up = base;
  up.keys_in = mk;
  up.vals_in = mv;
  up.keys_copy = sk;
  up.vals_copy = sv;
  up.upsweep_only = true;
  up.hist_copy = ctx->h_hist;
  up.hist_ready = ctx->ev_hist;
  up.inject_stall = 0;
  cudaError_t e = gs::launch_radix_sort(up, ctx->props, &ctx->gen, ctx->stream);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "upsweep launch");
  phase_mark(ctx, "Transfer in");
  e = cudaEventSynchronize(ctx->ev_hist);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "histograms");

  const uint32_t t = split_digit(ctx->h_hist, digits, n);
  e = launch_split(ctx, base, t, sk, sv, ak, av);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "split pass launch");
  phase_mark(ctx, "Split");
  return host_runs(ctx, base, t, bucket_groups(ctx->h_hist + size_t(t) * gs::RADIX, n, groups),
                   ak, av, sk, sv, kout, vout, nullptr);
}

// Keys-only host sorts of at least 2^28 keys (by default): as
// host_groups_sort, but the split no longer waits for the whole input. The
// input crosses the link in HOST_CHUNKS chunks; each chunk's upsweep (one
// CTA per SM, bound by the link) counts it and stages it, and its split on
// the top digit into its own 256 buckets runs on a second stream while the
// next chunk crosses the link, so only the last chunk's split is left once
// the input is in. A run of buckets then gathers its pieces from every
// chunk (device copies) into its stage range before it sorts, with a third
// buffer as the alternate. Ties cannot be told apart (keys only), so the
// chunk order of the pieces does not matter. When the top digit turns out
// to be the same for every key, the chunk splits are of no use and the
// single split of host_groups_sort runs on the staged input instead.
gs_status host_groups_chunked(gs_ctx* ctx, int kb, uint32_t kk, const void* mk, void* kout,
                              uint64_t n, uint32_t flags, uint32_t groups) {
  gs_status st = host_groups_setup(ctx);
  if (st == GS_OK) st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st == GS_OK) st = ensure(ctx, ctx->third_k, size_t(n) * kb);
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, 0));
  if (st != GS_OK) return st;
  uint8_t* sk = static_cast<uint8_t*>(ctx->stage_k.ptr);
  uint8_t* ak = static_cast<uint8_t*>(ctx->alt_k.ptr);
  uint8_t* tk = static_cast<uint8_t*>(ctx->third_k.ptr);
  const uint8_t* in = static_cast<const uint8_t*>(mk);
  const gs::RadixJob base = host_base_job(ctx, kb, kk, 0, 0, n, flags);
  const uint32_t digits = uint32_t(kb);
  const uint32_t top = digits - 1;
  // Chunk length: a multiple of 4096 keys, so every chunk starts 16-byte
  // aligned.
  const uint64_t len = ((n + HOST_CHUNKS - 1) / HOST_CHUNKS + 4095) & ~uint64_t(4095);
  const uint32_t chunks = uint32_t((n + len - 1) / len);
  cudaStream_t s1 = ctx->stream, s2 = ctx->split_stream;
  auto fail_after_splits = [&](cudaError_t err, const char* where) {
    cudaStreamSynchronize(s2);
    return cuda_fail(ctx, err, where);
  };
  cudaError_t e = cudaSuccess;
  for (uint32_t c = 0; c < chunks; ++c) {
    const uint64_t c0 = uint64_t(c) * len, nc = std::min(len, n - c0);
    gs::SortWork* w = (c & 1u) ? ctx->work2 : ctx->work;
    // The chunk two back used this work area; its split must be done.
    if (c >= 2) e = cudaStreamWaitEvent(s1, ctx->ev_chunk_split[c - 2], 0);
    gs::RadixJob up = base;
    up.n = nc;
    up.keys_in = in + c0 * kb;
    up.keys_copy = sk + c0 * kb;
    up.work = w;
    up.gen_counter = &ctx->work->gen_counter;  // one tag counter per status buffer
    up.upsweep_only = true;
    up.upsweep_per_sm = 1;
    up.hist_copy = ctx->h_hist + size_t(c) * gs::HIST_WORDS;
    up.inject_stall = 0;
    if (e == cudaSuccess) e = gs::launch_radix_sort(up, ctx->props, &ctx->gen, s1);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_chunk_in[c], s1);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s2, ctx->ev_chunk_in[c], 0);
    gs::RadixJob sp = base;
    sp.n = nc;
    sp.keys_in = sk + c0 * kb;
    sp.keys_out = ak + c0 * kb;
    sp.keys_alt = ak + c0 * kb;
    sp.work = w;
    sp.gen_counter = &ctx->work->gen_counter;
    sp.skip_upsweep = true;
    sp.digit_lo = top;
    sp.digit_hi = top + 1;
    sp.inject_stall = c == 0 ? base.inject_stall : 0u;
    if (e == cudaSuccess) e = gs::launch_radix_sort(sp, ctx->props, &ctx->gen, s2);
    if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_chunk_split[c], s2);
    if (e != cudaSuccess) return fail_after_splits(e, "chunk launch");
  }
  e = cudaEventRecord(ctx->ev_hist, s1);
  if (e == cudaSuccess) e = cudaEventSynchronize(ctx->ev_hist);
  if (e != cudaSuccess) return fail_after_splits(e, "histograms");
  phase_mark(ctx, "Transfer in");

  // Whole-input histograms, and each chunk's bucket starts on the top digit.
  std::vector<uint32_t> hist(gs::HIST_WORDS, 0);
  for (uint32_t c = 0; c < chunks; ++c)
    for (uint32_t i = 0; i < digits * gs::RADIX; ++i) hist[i] += ctx->h_hist[size_t(c) * gs::HIST_WORDS + i];
  // All of a chunk's splits are done once the last one is.
  e = cudaStreamWaitEvent(s1, ctx->ev_chunk_split[chunks - 1], 0);
  if (e != cudaSuccess) return fail_after_splits(e, "split join");
  const uint32_t t = split_digit(hist.data(), digits, n);
  if (t != top) {
    // The top digit is constant: split the staged input on digit t.
    gs::RadixJob sb = base;
    e = cudaMemcpyAsync(ctx->work->hist, hist.data(), sizeof(uint32_t) * digits * gs::RADIX,
                        cudaMemcpyHostToDevice, s1);
    if (e == cudaSuccess) e = launch_split(ctx, sb, t, sk, nullptr, ak, nullptr);
    if (e != cudaSuccess) return fail_after_splits(e, "split pass launch");
    phase_mark(ctx, "Split");
    return host_runs(ctx, base, t, bucket_groups(hist.data() + size_t(t) * gs::RADIX, n, groups),
                     ak, nullptr, sk, nullptr, kout, nullptr, nullptr);
  }
  phase_mark(ctx, "Split");
  std::vector<uint64_t> start(size_t(chunks) * (gs::RADIX + 1));  // chunk c, bucket b
  for (uint32_t c = 0; c < chunks; ++c) {
    const uint32_t* h = ctx->h_hist + size_t(c) * gs::HIST_WORDS + size_t(top) * gs::RADIX;
    uint64_t acc = 0;
    for (uint32_t bkt = 0; bkt <= uint32_t(gs::RADIX); ++bkt) {
      start[size_t(c) * (gs::RADIX + 1) + bkt] = acc;
      if (bkt < uint32_t(gs::RADIX)) acc += h[bkt];
    }
  }
  const auto runs = bucket_groups(hist.data() + size_t(top) * gs::RADIX, n, groups);
  // Each run's first and last bucket, for the gather.
  std::vector<std::pair<uint32_t, uint32_t>> span;
  {
    uint64_t acc = 0;
    uint32_t bkt = 0;
    for (const BucketRun& r : runs) {
      while (acc < r.begin) acc += hist[size_t(top) * gs::RADIX + bkt++];
      const uint32_t b0 = bkt;
      while (acc < r.end) acc += hist[size_t(top) * gs::RADIX + bkt++];
      span.emplace_back(b0, bkt);
    }
  }
  size_t run_index = 0;
  auto gather = [&](const BucketRun& r) -> cudaError_t {
    const auto [b0, b1] = span[run_index++];
    uint64_t dst = r.begin;
    for (uint32_t c = 0; c < chunks; ++c) {
      const uint64_t* cs = &start[size_t(c) * (gs::RADIX + 1)];
      const uint64_t m = cs[b1] - cs[b0];
      if (m == 0) continue;
      const cudaError_t ce = cudaMemcpyAsync(sk + dst * kb, ak + (uint64_t(c) * len + cs[b0]) * kb,
                                             m * kb, cudaMemcpyDeviceToDevice, s1);
      if (ce != cudaSuccess) return ce;
      dst += m;
    }
    return cudaSuccess;
  };
  return host_runs(ctx, base, top, runs, sk, nullptr, tk, nullptr, kout, nullptr, gather);
}

}  // namespace gs
