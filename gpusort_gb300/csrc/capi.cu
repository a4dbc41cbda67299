// C ABI of the engine (include/gpusort_gb300.h): contexts, scratch held
// within an HBM budget, host staging, dispatch to the kernel launchers.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <functional>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/gpusort_gb300.h"
#include "engine.h"
#include "common.cuh"
#include "radix_types.cuh"

namespace {

thread_local std::string g_last_global_error;

struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

}  // namespace

namespace gs {
void set_last_global_error(const std::string& msg) { g_last_global_error = msg; }
}  // namespace gs

struct gs_ctx {
  gs::DeviceProps props;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::mutex mu;
  std::string last_error;
  uint64_t budget = 0;  // 0: no cap
  uint64_t held = 0;
  uint32_t gen = 0;
  uint32_t spin_limit = 1u << 20;
  uint32_t inject_stall = 0;
  int shape = -1;         // pass-kernel tile shape (debug override); -1: table / default
  std::vector<gs_tuning_entry> tuning;  // autotuner table, first match wins
  bool timing = false;
  gs::SortWork* work = nullptr;
  uint32_t* err = nullptr;
  DevBuf status;     // look-back words
  DevBuf alt_k, alt_v;
  DevBuf stage_k, stage_v, stage_off;
  DevBuf splitters;  // sample sort
  DevBuf merge_splits;  // HykSort shape: merge-path splits of one level
  // phase timing
  cudaEvent_t ev[8] = {};
  int n_phases = 0;
  const char* phase_names[8] = {};
  double phase_ms[8] = {};
  // kernel timing of the last radix pipeline (3 + MAX_DIGITS marks)
  cudaEvent_t kev[3 + 16] = {};
  int n_kev = 0;
  uint32_t kev_exec_mask = 0;
  // Host-buffer sorts in bucket groups (made on first use): the stream the
  // sorted groups leave on, its events, and the histograms read back.
  int host_groups = -1;  // -1: by size (host_groups_for); 0 or 1: one sort, then one copy out
  uint64_t host_chunked_min = uint64_t(1) << 28;  // keys-only host sorts this large (0: none)
                                                  // split chunk by chunk
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t ev_hist = nullptr, ev_group = nullptr, ev_copied = nullptr;
  uint32_t* h_hist = nullptr;  // pinned, gs::HIST_WORDS words per input chunk
  // Chunked host sorts: the split stream, per-chunk events, a second work
  // area (chunks alternate) and a third key buffer.
  cudaStream_t split_stream = nullptr;
  cudaEvent_t ev_chunk_in[8] = {}, ev_chunk_split[8] = {};
  gs::SortWork* work2 = nullptr;
  DevBuf third_k;
};

namespace gs {
cudaStream_t context_stream(gs_ctx* ctx) { return ctx->stream; }
}  // namespace gs

namespace {

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
gs_status ensure(gs_ctx* ctx, DevBuf& b, size_t bytes, bool zero = false) {
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

constexpr uint64_t MAX_N = 0xFFFFFFFFull;  // 32-bit bin counters

uint32_t floor_log2(uint64_t n) { return n ? 63u - uint32_t(__builtin_clzll(n)) : 0u; }

// First tuning entry for (key width and kind, payload width, size).
const gs_tuning_entry* find_tuning(const gs_ctx* ctx, int kb, uint32_t kk, int vb, uint64_t n) {
  const uint32_t lg = floor_log2(n);
  for (const gs_tuning_entry& e : ctx->tuning) {
    int ekb = 0;
    uint32_t ekk = 0;
    if (!dtype_info(gs_dtype(e.key_dtype), &ekb, &ekk) || ekb != kb || ekk != kk) continue;
    if (e.val_bytes != vb || lg < e.log2n_min || lg > e.log2n_max) continue;
    return &e;
  }
  return nullptr;
}

int pass_shape_for(const gs_ctx* ctx, int kb, uint32_t kk, int vb, uint64_t n) {
  if (ctx->shape >= 0) return ctx->shape;
  const gs_tuning_entry* e = find_tuning(ctx, kb, kk, vb, n);
  if (e && e->pass_shape >= 0) return e->pass_shape;
  return gs::radix_default_shape(kb, vb, n);
}

uint32_t partitions_for(const gs_ctx* ctx, int kb, uint32_t kk, uint64_t n, const gs_opts* o) {
  if (o && o->partitions) return o->partitions;
  const gs_tuning_entry* e = find_tuning(ctx, kb, kk, 0, n);
  if (e && e->partitions) return e->partitions;
  return 64;
}

bool entry_valid(const gs_tuning_entry& e) {
  int kb = 0;
  uint32_t kk = 0;
  return dtype_info(gs_dtype(e.key_dtype), &kb, &kk) &&
         (e.val_bytes == 0 || e.val_bytes == 4 || e.val_bytes == 8) &&
         e.log2n_min <= e.log2n_max && e.log2n_max <= 63 && e.pass_shape >= -1 &&
         e.pass_shape < gs::radix_num_shapes() && e.partitions <= gs::RADIX &&
         (e.partitions == 0 || e.partitions >= 2);
}

// Minimal JSON reader for the tuning file: any object holding "key_dtype"
// (at any depth) is an entry; other keys and values are skipped.
struct Json {
  const char* p;
  const char* e;
  std::vector<gs_tuning_entry>* out;
  bool ok = true;

  void ws() {
    while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  bool lit(const char* w) {
    const size_t k = std::strlen(w);
    if (size_t(e - p) < k || std::strncmp(p, w, k) != 0) return false;
    p += k;
    return true;
  }
  bool str(std::string* s) {
    if (p >= e || *p != '"') return false;
    ++p;
    while (p < e && *p != '"') {
      if (*p == '\\') {
        if (++p >= e) return false;
      }
      if (s) s->push_back(*p);
      ++p;
    }
    if (p >= e) return false;
    ++p;
    return true;
  }
  bool num(double* v) {
    char* end = nullptr;
    const double x = std::strtod(p, &end);
    if (end == p || end > e) return false;
    p = end;
    if (v) *v = x;
    return true;
  }
  // value; scalars are reported through *is_num / *d / *s
  bool value(bool* is_num, double* d, std::string* s, int depth) {
    if (depth > 32) return false;
    ws();
    if (p >= e) return false;
    if (*p == '{') return object(depth + 1);
    if (*p == '[') {
      ++p;
      ws();
      if (p < e && *p == ']') { ++p; return true; }
      while (true) {
        if (!value(nullptr, nullptr, nullptr, depth + 1)) return false;
        ws();
        if (p < e && *p == ',') { ++p; continue; }
        if (p < e && *p == ']') { ++p; return true; }
        return false;
      }
    }
    if (*p == '"') {
      if (is_num) *is_num = false;
      return str(s);
    }
    if (lit("true") || lit("false") || lit("null")) {
      if (is_num) *is_num = false;
      return true;
    }
    if (is_num) *is_num = true;
    return num(d);
  }
  bool object(int depth) {
    ++p;  // '{'
    gs_tuning_entry en{-1, 0, 0, 63, -1, 0};
    bool is_entry = false, bad = false;
    ws();
    if (p < e && *p == '}') { ++p; return true; }
    while (true) {
      ws();
      std::string key;
      if (!str(&key)) return false;
      ws();
      if (p >= e || *p != ':') return false;
      ++p;
      bool isn = false;
      double d = 0;
      std::string sv;
      if (!value(&isn, &d, &sv, depth)) return false;
      auto as_int = [&](int64_t lo, int64_t hi, int64_t* o) {
        if (!isn || d != double(int64_t(d)) || d < double(lo) || d > double(hi)) { bad = true; return; }
        *o = int64_t(d);
      };
      int64_t v = 0;
      if (key == "key_dtype") {
        is_entry = true;
        static const char* names[] = {"u32", "i32", "f32", "u64", "i64", "f64"};
        if (isn) { as_int(0, 5, &v); en.key_dtype = int32_t(v); }
        else {
          en.key_dtype = -1;
          for (int i = 0; i < 6; ++i) if (sv == names[i]) en.key_dtype = i;
          if (en.key_dtype < 0) bad = true;
        }
      } else if (key == "val_bytes") { as_int(0, 8, &v); en.val_bytes = int32_t(v); }
      else if (key == "log2n_min") { as_int(0, 63, &v); en.log2n_min = uint32_t(v); }
      else if (key == "log2n_max") { as_int(0, 63, &v); en.log2n_max = uint32_t(v); }
      else if (key == "pass_shape") { as_int(-1, 1 << 20, &v); en.pass_shape = int32_t(v); }
      else if (key == "partitions") { as_int(0, 1 << 20, &v); en.partitions = uint32_t(v); }
      ws();
      if (p < e && *p == ',') { ++p; continue; }
      if (p < e && *p == '}') { ++p; break; }
      return false;
    }
    if (is_entry) {
      if (bad || !entry_valid(en)) ok = false;
      else out->push_back(en);
    }
    return true;
  }
};

int parse_tuning(const char* json, std::vector<gs_tuning_entry>* out) {
  if (!json) return -1;
  Json j{json, json + std::strlen(json), out};
  if (!j.value(nullptr, nullptr, nullptr, 0)) return -1;
  j.ws();
  if (j.p != j.e || !j.ok) return -1;
  return int(out->size());
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
gs_status prepare_status(gs_ctx* ctx, size_t words, uint32_t passes) {
  (void)passes;
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
    std::string m = "device wait ran out or scatter out of range (code " + std::to_string(h) + ")";
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

// Device copies the upsweep makes of a host call's pinned input, which it
// reads directly across the CPU-GPU link (see sort_common).
struct HostFuse {
  void* keys_copy = nullptr;
  void* vals_copy = nullptr;
};

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

// Device-memory radix sort of keys or pairs.
gs_status device_sort(gs_ctx* ctx, int kb, uint32_t kkind, int vb, uint32_t vkind,
                      const void* kin, const void* vin, void* kout, void* vout,
                      uint64_t n, uint32_t flags, const HostFuse* fuse = nullptr) {
  const bool desc = flags & GS_FLAG_DESCENDING;
  const bool stable = flags & GS_FLAG_PAIRS_STABLE;
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
  const uint32_t passes = uint32_t(kb + (job.ties_by_value ? vb : 0));
  st = prepare_status(ctx, gs::radix_status_words(n, kb, vb), passes);
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

// Sort each of the given segments of `buf` in place (keys only); waits.
gs_status sort_segments_in_place(gs_ctx* ctx, int kb, uint32_t kk, bool desc, void* buf,
                                 uint64_t n, const std::vector<uint64_t>& off) {
  gs_seg_plan* pl = gs::seg_plan_new();
  const std::string err = gs::seg_plan_build(pl, off.data(), uint32_t(off.size() - 1), n, kb, kk,
                                             desc,
                                             gs::radix_segmented_shape(kb, n, uint32_t(off.size() - 1)));
  if (!err.empty()) {
    gs::seg_plan_free(pl);
    return fail(ctx, GS_ERR_OOM, err);
  }
  gs_status st = prepare_status(ctx, size_t(gs::seg_plan_large_tiles(pl)) * gs::RADIX + gs::RADIX,
                                uint32_t(kb));
  if (st == GS_OK) {
    cudaError_t e = gs::seg_plan_run(pl, buf, buf, ctx->alt_k.ptr,
                                     static_cast<uint64_t*>(ctx->status.ptr),
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
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, 0), 1);
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
  return sort_segments_in_place(ctx, kb, kk, desc, out, n, off);
}

// HykSort shape (keys only): each of p partitions sorted on its own, then
// merged by a tree of merge-path merges. p must be a power of two (the
// reference falls back to SampleSort otherwise,
// include/hyksort_common_vector.inl:31-43).
gs_status hyk_sort_device(gs_ctx* ctx, int kb, uint32_t kk, const void* in, void* out,
                          uint64_t n, uint32_t flags, const gs_opts* o) {
  uint32_t p = (o && o->partitions) ? o->partitions : 4;
  const uint32_t k = (o && o->k_way) ? o->k_way : 4;
  const bool pow2 = p && !(p & (p - 1)) && k && !(k & (k - 1));
  if (!pow2) return sample_sort_device(ctx, kb, kk, in, out, n, flags, o);
  const bool desc = flags & GS_FLAG_DESCENDING;
  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st != GS_OK) return st;
  const uint64_t run = (n + p - 1) / p;
  std::vector<uint64_t> off(p + 1);
  for (uint32_t i = 0; i <= p; ++i) off[i] = std::min<uint64_t>(uint64_t(i) * run, n);
  if (in != out) {
    cudaError_t e = cudaMemcpyAsync(out, in, size_t(n) * kb, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy");
  }
  st = sort_segments_in_place(ctx, kb, kk, desc, out, n, off);
  if (st != GS_OK) return st;
  phase_mark(ctx, "Local sort");
  size_t split_words = 0;  // tiles are counted per pair of full runs: any level may need the most
  for (uint64_t r = run; r < n; r *= 2)
    split_words = std::max(split_words, gs::merge_split_words(n, r, kb));
  st = ensure(ctx, ctx->merge_splits, std::max<size_t>(split_words, 1) * sizeof(uint64_t));
  if (st != GS_OK) return st;
  void* cur = out;
  void* other = ctx->alt_k.ptr;
  for (uint64_t r = run; r < n; r *= 2) {
    cudaError_t e = gs::launch_merge_pass(cur, other, n, r, kb, kk, desc,
                                          static_cast<uint64_t*>(ctx->merge_splits.ptr),
                                          ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "merge launch");
    std::swap(cur, other);
  }
  if (cur != out) {
    cudaError_t e = cudaMemcpyAsync(out, cur, size_t(n) * kb, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "copy");
  }
  phase_mark(ctx, "Merge data");
  return GS_OK;
}

// Chunks of a chunked host sort (host_groups_chunked). Measured on GB300
// with pinned buffers, 2^30 u32 keys: 47.0 ms with one split after the whole
// input; 4 chunks, 16 groups: 44.8 ms; 8 chunks, 16 / 24 groups: 44.6 /
// 44.2 ms (the last chunk's split, left exposed, halves). 2^28: 11.7 vs
// 11.9 ms; 2^27: no gain.
constexpr uint32_t HOST_CHUNKS = 8;

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
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, vb), 0);
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
  if (st == GS_OK) st = prepare_status(ctx, gs::radix_status_words(n, kb, 0), 0);
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
                    &ctx->stage_off, &ctx->splitters, &ctx->merge_splits, &ctx->third_k};
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
  const std::string err = gs::seg_plan_build(pl, host_offsets, nseg, n, kb, kk,
                                             (flags & GS_FLAG_DESCENDING) != 0,
                                             gs::radix_segmented_shape(kb, n, nseg));
  if (!err.empty()) {
    gs::seg_plan_free(pl);
    return fail(ctx, err.find("allocation") != std::string::npos ? GS_ERR_OOM : GS_ERR_INVALID,
                err);
  }
  gs_status st = ensure(ctx, ctx->alt_k, size_t(n) * kb);
  if (st == GS_OK)
    st = prepare_status(ctx, size_t(gs::seg_plan_large_tiles(pl)) * gs::RADIX + gs::RADIX,
                        uint32_t(kb));
  if (st != GS_OK) {
    gs::seg_plan_free(pl);
    return st;
  }
  cudaStreamSynchronize(ctx->stream);
  *plan = pl;
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

gs_status gs_ctx_set_tuning(gs_ctx* ctx, const gs_tuning_entry* entries, uint32_t count) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  if (count && !entries) return fail(ctx, GS_ERR_INVALID, "null tuning entries");
  for (uint32_t i = 0; i < count; ++i)
    if (!entry_valid(entries[i])) return fail(ctx, GS_ERR_INVALID, "invalid tuning entry");
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tuning.assign(entries, entries + count);
  return GS_OK;
}

int gs_tuning_parse(const char* json, gs_tuning_entry* out, uint32_t capacity) {
  std::vector<gs_tuning_entry> v;
  const int k = parse_tuning(json, &v);
  if (k < 0) return -1;
  if (out && uint32_t(k) <= capacity) std::copy(v.begin(), v.end(), out);
  return k;
}

gs_status gs_ctx_load_tuning(gs_ctx* ctx, const char* path) {
  if (!ctx || !path) return fail(ctx, GS_ERR_INVALID, "null context or path");
  FILE* f = std::fopen(path, "rb");
  if (!f) return fail(ctx, GS_ERR_INVALID, std::string("cannot open tuning file ") + path);
  std::string text;
  char buf[4096];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, k);
  std::fclose(f);
  std::vector<gs_tuning_entry> v;
  if (parse_tuning(text.c_str(), &v) < 0)
    return fail(ctx, GS_ERR_INVALID, std::string("malformed tuning file ") + path);
  std::lock_guard<std::mutex> lock(ctx->mu);
  ctx->tuning = std::move(v);
  return GS_OK;
}

gs_status gs_ctx_choice(gs_ctx* ctx, gs_dtype key_dtype, int val_bytes, uint64_t n,
                        int* pass_shape, uint32_t* partitions) {
  if (!ctx) return fail(nullptr, GS_ERR_INVALID, "null context");
  int kb = 0;
  uint32_t kk = 0;
  if (!dtype_info(key_dtype, &kb, &kk)) return fail(ctx, GS_ERR_BAD_DTYPE, "unknown key dtype");
  if (val_bytes != 0 && val_bytes != 4 && val_bytes != 8)
    return fail(ctx, GS_ERR_INVALID, "payload width must be 0, 4 or 8");
  std::lock_guard<std::mutex> lock(ctx->mu);
  if (pass_shape) *pass_shape = pass_shape_for(ctx, kb, kk, val_bytes, n);
  if (partitions) *partitions = partitions_for(ctx, kb, kk, n, nullptr);
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
