// Host-side internal interfaces between the C ABI (capi.cu) and the kernel
// launchers (radix.cu, ...). Not installed; include/gpusort_gb300.h is the
// public surface.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <cuda_runtime.h>

namespace gs {

struct SortWork;

struct DeviceProps {
  int device = 0;
  int num_sms = 0;
  size_t smem_optin = 0;
};

// One radix sort of keys (and an optional payload) on device memory.
struct RadixJob {
  const void* keys_in = nullptr;
  void* keys_out = nullptr;
  void* keys_alt = nullptr;         // n * key_bytes scratch
  const void* vals_in = nullptr;
  void* vals_out = nullptr;
  void* vals_alt = nullptr;         // n * val_bytes scratch
  uint64_t n = 0;
  int key_bytes = 4;                // 4 or 8
  int val_bytes = 0;                // 0 (keys only), 4 or 8
  uint32_t key_kind = 0, val_kind = 0;
  bool desc = false;
  bool ties_by_value = false;       // value digits take part in the order
  bool reverse_first = false;       // stable descending pairs
  bool first_unstable = false;      // no ties to keep: first pass may be unstable
  uint64_t* status = nullptr;       // radix_status_words(n, ...) words
  SortWork* work = nullptr;
  uint32_t* err = nullptr;
  uint32_t spin_limit = 1u << 20;
  uint32_t inject_stall = 0;
  // Optional timing marks: when set, an event is recorded before the
  // pipeline (marks[0]), after the upsweep (1), after the plan (2) and after
  // each pass q (3 + q). Needs 3 + digits events.
  cudaEvent_t* marks = nullptr;
  int shape = 0;                    // pass-kernel tile shape (0 .. radix_num_shapes()-1)
  uint32_t* gen_counter = nullptr;  // look-back tag counter of `status` (default: in work)
  // Optional: the upsweep copies keys_in / vals_in (e.g. pinned host memory
  // the device reads directly) to these device buffers and the passes read
  // the copies, so the input crosses the CPU-GPU link once.
  void* keys_copy = nullptr;
  void* vals_copy = nullptr;
  // Digit range [digit_lo, digit_hi) of the digit sequence (value digits
  // first when ties go by value) that the passes sort; digit_hi 0 means
  // every digit. The elements must already be in order by the digits above
  // the range (a run of buckets of a split by a higher digit).
  uint32_t digit_lo = 0, digit_hi = 0;
  // keys_alt (and vals_alt) is keys_in (vals_in): the first pass that runs
  // must write keys_out, so the plan makes the pass count odd. The range
  // must hold an odd number of digits.
  bool alt_is_in = false;
  // Pipeline stages, for callers that decide between them on the host: only
  // the zeroing and the upsweep (copying the histograms to `hist_copy`,
  // HIST_WORDS words of host memory, and recording `hist_ready` after), or
  // only the plan and the passes (histograms already in `work`).
  bool upsweep_only = false;
  bool skip_upsweep = false;
  uint32_t* hist_copy = nullptr;
  cudaEvent_t hist_ready = nullptr;
  // Upsweep CTAs per SM (0: the default, 3). One leaves room beside it for
  // a pass running on another stream, as when the upsweep reads across the
  // CPU-GPU link and is bound by it.
  uint32_t upsweep_per_sm = 0;
};

// Words of the digit histograms a RadixJob can copy out: 16 digits x 256
// bins; row q is digit q of the sequence.
constexpr uint32_t HIST_DIGITS = 16;
constexpr uint32_t HIST_WORDS = HIST_DIGITS * 256;

// Smallest tile (elements) of the pass kernel over all shapes: sizes the
// look-back words.
uint32_t radix_tile(int key_bytes, int val_bytes);
int radix_num_shapes();
// Threads per CTA and items per thread of a pass shape (false: no such shape).
bool radix_shape_info(int key_bytes, int val_bytes, int shape, uint32_t* threads, uint32_t* items);
int radix_default_shape(int key_bytes, int val_bytes, uint64_t n);
// Tile (keys) of shape 0 for 32-bit keys without payload, and the look-back
// words of a job run with that shape.
constexpr uint32_t RADIX_TILE_U32_SHAPE0 = 384 * 24;
size_t radix_status_words_u32_shape0(uint64_t n);
// Look-back words a job of n elements needs.
size_t radix_status_words(uint64_t n, int key_bytes, int val_bytes);
size_t sort_work_bytes();

// Large segments of a batched sort, for the segmented form of the passes.
struct SegTile;  // radix_types.cuh

struct SegJob {
  const uint32_t* tile_start;  // nseg + 1 first-tile indexes
  const uint64_t* range;       // nseg (begin, end) element pairs
  const uint32_t* binbase;     // [nseg][digits][256]
  uint32_t nseg;
  uint32_t digits;
  uint32_t total_tiles;
  const SegTile* tiles;        // total_tiles descriptors
};
uint32_t radix_shape_tile(int key_bytes, int val_bytes, int shape);
int radix_segmented_shape(int key_bytes, uint64_t n, uint32_t nseg);
// Enqueue only the digit passes over the large segments (plan and bin
// bases already prepared in job.work / sj.binbase).
cudaError_t launch_radix_passes(const RadixJob& job, const SegJob& sj, const DeviceProps& props,
                                uint32_t* gen, cudaStream_t stream);

}  // namespace gs
struct gs_seg_plan;
struct gs_ctx;
namespace gs {
// Host only: gs_segmented_layout's per-segment kinds and counts for pass
// tiles of `tile` elements.
std::string seg_layout_summary(const uint64_t* off, uint32_t nseg, uint64_t n, uint32_t tile,
                               uint8_t* kinds, uint64_t counts[4]);
std::string seg_plan_build(gs_seg_plan* pl, const uint64_t* off, uint32_t nseg, uint64_t n,
                           int key_bytes, uint32_t kind, bool desc, int shape);
void seg_plan_free(gs_seg_plan* pl);
gs_seg_plan* seg_plan_new();
uint32_t seg_plan_large_tiles(const gs_seg_plan* pl);
uint64_t seg_plan_n(const gs_seg_plan* pl);
int seg_plan_key_bytes(const gs_seg_plan* pl);
cudaError_t seg_plan_run(const gs_seg_plan* pl, const void* in, void* out, void* alt,
                         uint64_t* status, uint32_t* gen_counter, uint32_t* err,
                         uint32_t spin_limit, const DeviceProps& props, cudaStream_t st);

// Sort n <= small_sort_max() keys (no payload) in one CTA's shared memory;
// `in` may equal `out`.
uint32_t small_sort_max();
cudaError_t launch_small_sort(const void* in, void* out, uint32_t n, int key_bytes,
                              uint32_t kind, bool desc, cudaStream_t st);
// One small keys-only array of a batch (n <= small_sort_max()).
struct SmallSortReq {
  const void* in;
  void* out;
  uint32_t n;
  uint32_t kind;
  uint32_t desc;
  uint32_t pad;
};
// Sort `count` such arrays of one key width in one launch; `reqs` must be
// readable by the device (device memory or mapped pinned host memory).
cudaError_t launch_small_sort_batch(const SmallSortReq* reqs, uint32_t count, int key_bytes,
                                    cudaStream_t st);

// Sample-sort bucketing (keys only): sample + splitters + bucket histogram
// + one bucket scatter pass from job.keys_in to job.keys_out (which must
// differ). job.work->hist[0][0..parts) holds the bucket sizes afterwards.
struct SampleJob {
  uint32_t parts;     // p buckets (2..256)
  uint32_t samples;   // p * oversample (<= 8192)
  uint64_t seed;
  void* splitters;    // device buffer of >= 255 keys
};
cudaError_t launch_sample_bucketing(const RadixJob& job, const SampleJob& sj,
                                    const DeviceProps& props, cudaStream_t st);
cudaError_t launch_bucket_pass(const RadixJob& job, const void* splitters, uint32_t nsplit,
                               const DeviceProps& props, cudaStream_t st);

// HykSort shape (hyk.cu): one round of the reference's SortAmongProcesses
// over p ranks, whose sorted runs lie at roff[r] .. roff[r+1] of `data`, in
// groups of n_p consecutive ranks, k-way (kway <= n_p, powers of two).
constexpr uint32_t MAX_KWAY = 16;
constexpr uint32_t HYK_MAX_RANKS = 512;
struct HykRound {
  const void* data = nullptr;
  const uint64_t* roff = nullptr;  // device, p + 1
  uint32_t p = 0, n_p = 0, kway = 0;
  int key_bytes = 4;
  uint32_t key_kind = 0;
  bool desc = false;
  uint64_t seed = 0;
  void* splitters = nullptr;       // device, (p / n_p) x (kway - 1) keys
  uint32_t* iters = nullptr;       // device, p / n_p (selection rounds, diagnostic)
  uint64_t* cuts = nullptr;        // device, p x (kway + 1) cut offsets
  uint64_t* samp_rank = nullptr;   // device, per merge sample
  uint64_t* samp_cut = nullptr;    // device, per merge sample x kway
  uint64_t* tile_out = nullptr;    // device, per merge tile
  uint64_t* tile_src = nullptr;    // device, per merge tile x kway
  uint32_t* tile_len = nullptr;    // device, per merge tile x kway
  uint32_t* err = nullptr;         // device error word
};
// One of the kway pieces a receiving rank merges: src .. src + len of the
// source buffer; the rank's output starts at `out`; its pieces are
// first .. first + kway - 1 of the table; the piece's merge samples (one
// every hyk_sample_stride elements) are numbered from sample0.
struct HykPiece {
  uint64_t src, len, sample0, out;
  uint32_t first, j;
};
uint32_t hyk_sample_stride(int key_bytes, uint32_t kway);
// Target tile length of the merge: a receiving rank of L elements has
// ceil(L / hyk_tile_span) tiles.
uint32_t hyk_tile_span(int key_bytes);
size_t hyk_select_smem(int key_bytes, uint32_t n_p, uint32_t kway);
// Splitter selection (one CTA per group) and the ranks' cut points.
cudaError_t launch_hyk_select(const HykRound& r, cudaStream_t st);
// The k-way merge of every receiving rank's pieces from src into dst;
// rtile (device, p + 1) holds each receiving rank's first tile.
cudaError_t launch_hyk_merge(const HykRound& r, const HykPiece* pieces, uint32_t npieces,
                             uint64_t nsamples, const uint64_t* rtile, uint64_t ntiles,
                             const void* src, void* dst, cudaStream_t st);


// Allow `kern` up to `bytes` of dynamic shared memory on the current device
// (once per kernel and device; safe to call from any thread).
cudaError_t allow_dynamic_smem(const void* kern, size_t bytes);

// Set the message gs_last_global_error() returns on this thread.
void set_last_global_error(const std::string& msg);

// The CUDA stream a context enqueues on.
cudaStream_t context_stream(gs_ctx* ctx);

// Enqueue the whole radix pipeline on `stream`. `gen` is the context's
// launch-generation counter (advanced once per pass launch); the caller
// clears the status words when it wraps.
cudaError_t launch_radix_sort(const RadixJob& job, const DeviceProps& props,
                              uint32_t* gen, cudaStream_t stream);

}  // namespace gs
