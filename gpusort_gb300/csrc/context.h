// Internal to the library: the engine context (the C ABI's opaque gs_ctx)
// and the helpers the C ABI's translation units share: capi.cu (contexts,
// sorts, gathers), tuning.cu (the tuning table and its file format) and
// hostsort.cu (sorts of host buffers). Not installed.
#pragma once

#include <cstddef>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/gpusort_gb300.h"
#include "engine.h"
#include "radix_types.cuh"

namespace gs {

// A grow-only device buffer owned by a context.
struct DevBuf {
  void* ptr = nullptr;
  size_t bytes = 0;
};

// Input chunks of a chunked host sort (hostsort.cu). Measured on GB300 with
// pinned buffers, 2^30 u32 keys: 47.0 ms with one split after the whole
// input; 4 chunks, 16 groups: 44.8 ms; 8 chunks, 16 / 24 groups: 44.6 /
// 44.2 ms (the last chunk's split, left exposed, halves). 2^28: 11.7 vs
// 11.9 ms; 2^27: no gain.
constexpr uint32_t HOST_CHUNKS = 8;

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
  gs::DevBuf status;     // look-back words
  gs::DevBuf alt_k, alt_v;
  gs::DevBuf stage_k, stage_v, stage_off;
  gs::DevBuf splitters;  // sample sort
  gs::DevBuf hyk_small;     // HykSort shape: offsets, splitters, cuts, pieces
  gs::DevBuf hyk_samples;   // HykSort shape: the merge samples of one round
  // phase timing
  cudaEvent_t ev[8] = {};
  int n_phases = 0;
  const char* phase_names[8] = {};
  double phase_ms[8] = {};
  // kernel timing of the last radix pipeline (3 + MAX_DIGITS marks)
  cudaEvent_t kev[3 + 16] = {};
  int n_kev = 0;
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
  cudaEvent_t ev_chunk_in[gs::HOST_CHUNKS] = {}, ev_chunk_split[gs::HOST_CHUNKS] = {};
  gs::SortWork* work2 = nullptr;
  gs::DevBuf third_k;
};

namespace gs {

// Record msg as the context's last error (the thread's when ctx is null)
// and return st.
gs_status fail(gs_ctx* ctx, gs_status st, const std::string& msg);
gs_status cuda_fail(gs_ctx* ctx, cudaError_t e, const char* where);
// Grow-only scratch, bounded by the context's HBM budget.
gs_status ensure(gs_ctx* ctx, DevBuf& b, size_t bytes, bool zero = false);
bool dtype_info(gs_dtype t, int* bytes, uint32_t* kind);
void phase_reset(gs_ctx* ctx);
void phase_mark(gs_ctx* ctx, const char* name);
gs_status prepare_status(gs_ctx* ctx, size_t words);
// Wait for the context's stream and report a device-side error word.
gs_status check_err_word(gs_ctx* ctx);
RadixJob radix_job(gs_ctx* ctx, int kb, uint32_t kkind, int vb, uint32_t vkind, uint64_t n,
                   uint32_t flags);

// tuning.cu: the tuning table's choices (explicit settings first).
int pass_shape_for(const gs_ctx* ctx, int kb, uint32_t kk, int vb, uint64_t n);
uint32_t partitions_for(const gs_ctx* ctx, int kb, uint32_t kk, uint64_t n, const gs_opts* o);

// hostsort.cu: host-buffer transfers and sorts.
const void* mapped_host(const void* p);
cudaError_t link_copy(gs_ctx* ctx, void* dst, const void* src, uint64_t bytes, bool to_device);
uint32_t host_groups_for(const gs_ctx* ctx, uint64_t n);
gs_status host_groups_sort(gs_ctx* ctx, int kb, uint32_t kk, int vb, uint32_t vk, const void* mk,
                           const void* mv, void* kout, void* vout, uint64_t n, uint32_t flags,
                           uint32_t groups);
gs_status host_groups_chunked(gs_ctx* ctx, int kb, uint32_t kk, const void* mk, void* kout,
                              uint64_t n, uint32_t flags, uint32_t groups);

}  // namespace gs
