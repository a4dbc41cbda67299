/*
 * gpusort_gb300.h - C ABI of the GB300 sorting engine.
 *
 * Plain C: pointers, sizes and status codes only. Every entry point below
 * replaces one reference interface on the sort path of monotone-RK/gpusort;
 * the citation beside it names that interface (path:line in the reference
 * project). The header-only C++ layer in include/gpusort/ keeps the
 * reference's templated names (HykSort, SampleSort, HyperQuickSort) and
 * calls these functions.
 *
 * Memory: by default every pointer is a device pointer on the context's
 * device and the call is asynchronous on the context's stream. With
 * GS_FLAG_HOST every pointer is host memory and the call is synchronous
 * (copy in, sort, copy out), which is how the reference's own API behaves
 * (src/cuda_utils.cu:403-445 stages host data through the device). Pinned
 * buffers (cudaHostAlloc, cudaHostRegister) are fastest: the device reads
 * the input across the CPU-GPU link itself, and large radix sorts run in
 * bucket groups that are copied out while the next group sorts (see
 * GS_DEBUG_HOST_GROUPS). The output may be the input buffer.
 */
#ifndef GPUSORT_GB300_H_
#define GPUSORT_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. The reference raises C++ exceptions instead
 * (include/exceptions/thrust_exception.h:9-22,
 *  include/exceptions/mpi_exception.h:9-22); the C++ layer maps these
 * back to the same exception types and messages. */
typedef enum gs_status {
  GS_OK = 0,
  GS_ERR_EMPTY = 1,        /* n == 0: "No data to sort."
                              (include/helpers/hyksort_helper.h:105) */
  GS_ERR_OOM = 2,          /* device allocation or HBM budget exhausted
                              (src/cuda_utils.cu:415-416,425-426) */
  GS_ERR_BAD_DTYPE = 3,    /* key/value type outside the instantiated set
                              (src/cuda_utils.cu:257-318) */
  GS_ERR_TIMEOUT = 4,      /* a bounded inter-block wait ran out; the
                              result is invalid, the context stays usable */
  GS_ERR_CUDA = 5,         /* CUDA runtime error (src/cuda_utils.cu:373-393) */
  GS_ERR_INVALID = 6,      /* bad argument (null pointer, bad option) */
  GS_ERR_NO_DEVICE = 7,    /* no CUDA device (src/cuda_utils.cu:81-92) */
  GS_ERR_TOO_LARGE = 8,    /* n beyond the engine's per-call limit */
  GS_ERR_BUSY = 9,         /* serving queue full / request not finished */
  GS_ERR_CANCELLED = 10    /* serving request cancelled before it ran */
} gs_status;

/* Key and value element types: the reference's instantiation set
 * (src/cuda_utils.cu:257-262): int, unsigned int, float, double, int64_t,
 * uint64_t. */
typedef enum gs_dtype {
  GS_U32 = 0,
  GS_I32 = 1,
  GS_F32 = 2,
  GS_U64 = 3,
  GS_I64 = 4,
  GS_F64 = 5
} gs_dtype;

/* Flags (bitwise OR). */
#define GS_FLAG_DESCENDING   0x1u  /* std::greater<T> instead of std::less<T>
                                      (include/common.h:156-164,205-213) */
#define GS_FLAG_PAIRS_STABLE 0x2u  /* pairs: ties on the key keep input order
                                      (ascending) or reverse input order
                                      (descending); equals the reference's
                                      (key, value) order when values grow
                                      along the input, e.g. global indexes
                                      (include/hyksort_common_vector.inl:
                                      552-565). Without it, ties are ordered by
                                      value like std::pair's operator<
                                      (include/helpers/hyksort_helper.h:
                                      266-280). */
#define GS_FLAG_HOST         0x4u  /* pointers are host memory; synchronous */
#define GS_FLAG_SYNC         0x8u  /* wait for completion and report
                                      GS_ERR_TIMEOUT from this call */
#define GS_FLAG_OFFSETS_HOST 0x10u /* segment offsets are in host memory */

/* Sorting strategy. Every strategy produces the same bytes. */
typedef enum gs_algo {
  GS_ALGO_AUTO = 0,       /* engine's fastest path for the size and type */
  GS_ALGO_RADIX = 1,      /* one onesweep LSD radix sort over the array */
  GS_ALGO_SAMPLE = 2,     /* SampleSort shape: splitters from an oversampled
                             sample, bucket scatter into p partitions (the
                             in-HBM Alltoallv), radix sort per partition
                             (include/helpers/samplesort_helper.h:390-565) */
  GS_ALGO_HYK = 3         /* HykSort shape: radix sort of p input partitions,
                             k-way splitters, merge-path merge of the
                             received runs
                             (include/helpers/hyksort_helper.h:307-633) */
} gs_algo;

typedef struct gs_opts {
  uint32_t algo;          /* gs_algo */
  uint32_t partitions;    /* p: virtual MPI ranks (0 = engine default) */
  uint32_t k_way;         /* HykSort k (0 = 4) */
  uint32_t oversample;    /* samples per partition (0 = 32) */
  uint64_t seed;          /* splitter sampling seed */
} gs_opts;

typedef struct gs_ctx gs_ctx;

/* Library version, e.g. 0x000100 for 0.1.0. */
uint32_t gs_version(void);

/* Number of visible CUDA devices (src/cuda_utils.cu:81-92
 * CudaUtils::GetDeviceCount). Returns 0 when there is none. */
int gs_device_count(void);

/* Create a context bound to `device`. `hbm_budget_bytes` caps the scratch
 * the context may hold (0 = no cap). Replaces the per-call device selection
 * and chunking of src/cuda_utils.cu:395-401,508-520: data stays resident
 * and no chunk split is needed while it fits. Returns NULL on failure
 * (gs_last_global_error() says why). */
gs_ctx* gs_ctx_create(int device, uint64_t hbm_budget_bytes);
void gs_ctx_destroy(gs_ctx* ctx);

/* Use an existing CUDA stream (cudaStream_t passed as void*) for all later
 * work of the context; NULL selects the CUDA legacy default stream. A new
 * context uses a non-blocking stream of its own. */
gs_status gs_ctx_set_stream(gs_ctx* ctx, void* stream);

/* Wait for all work of the context. Returns GS_ERR_TIMEOUT if a bounded
 * wait inside a kernel ran out since the last check (and clears it). */
gs_status gs_ctx_synchronize(gs_ctx* ctx);

/* Text of the last error on this context. */
const char* gs_last_error(gs_ctx* ctx);
const char* gs_last_global_error(void);

/* Sort keys.
 * Replaces CudaUtils::Sort (src/cuda_utils.cu:97-167) as called from
 * HykSortHelper::Sort (include/helpers/hyksort_helper.h:94-145) and the
 * whole SortAmongProcesses exchange (include/helpers/hyksort_helper.h:
 * 453-536; include/helpers/samplesort_helper.h:420-501): the output is the
 * concatenation of all ranks' slices, i.e. the globally sorted array.
 * `in` and `out` may alias (in-place). */
gs_status gs_sort_keys(gs_ctx* ctx, gs_dtype dtype, const void* in, void* out,
                       uint64_t n, uint32_t flags, const gs_opts* opts);

/* Sort key/value pairs.
 * Replaces CudaUtils::SortByKey (src/cuda_utils.cu:169-243) and
 * HykSortHelper::SortByKey (include/helpers/hyksort_helper.h:224-297).
 * Ties on the key are ordered by value (std::pair order) unless
 * GS_FLAG_PAIRS_STABLE is set. Outputs may alias inputs. */
gs_status gs_sort_pairs(gs_ctx* ctx, gs_dtype key_dtype, gs_dtype val_dtype,
                        const void* keys_in, const void* vals_in,
                        void* keys_out, void* vals_out, uint64_t n,
                        uint32_t flags, const gs_opts* opts);

/* Sort many independent segments in one call. Segment s is
 * [offsets[s], offsets[s+1]) of `in`; `offsets` has nseg+1 entries
 * (device memory, or host memory with GS_FLAG_OFFSETS_HOST),
 * non-decreasing, offsets[0] == 0 and offsets[nseg] == n. Each segment is
 * sorted on its own, as one rank's local sort would be
 * (include/omp/omp_utils.h:147-207 applied per segment). Empty segments are
 * allowed. Keys only (32- or 64-bit types); `in` may equal `out`. With
 * GS_FLAG_HOST, `in`/`out` are host memory. The call waits for completion. */
gs_status gs_segmented_sort_keys(gs_ctx* ctx, gs_dtype dtype, const void* in,
                                 void* out, uint64_t n, const uint64_t* offsets,
                                 uint32_t nseg, uint32_t flags);

/* The same work split in two: planning (host offsets; allocates the plan's
 * device tables) and running (enqueues kernels only on the context's
 * stream, no allocation and no host synchronisation, so a run can be
 * captured into a CUDA graph and replayed). The context's scratch is sized
 * for the plan when it is created. A plan may be run many times, on any
 * device buffers of n keys; destroy it after its last run has completed. */
typedef struct gs_seg_plan gs_seg_plan;
gs_status gs_segmented_plan_create(gs_ctx* ctx, gs_dtype dtype, uint64_t n,
                                   const uint64_t* host_offsets, uint32_t nseg,
                                   uint32_t flags, gs_seg_plan** plan);
gs_status gs_segmented_plan_run(gs_ctx* ctx, const gs_seg_plan* plan,
                                const void* in, void* out);
void gs_segmented_plan_destroy(gs_seg_plan* plan);

/* How a segmented sort of these host offsets treats each segment, computed
 * on the host alone (no context, no device): `kinds` (nseg entries, may be
 * null) receives a gs_seg_kind per segment; counts[0..3] receive the
 * number of groups sorted whole in shared memory, of segments sorted by
 * one warp each, of segments sorted by the radix passes, and of pass tiles
 * over those. The rules: segments of at most 4096 keys are packed in order
 * into groups of consecutive segments (at most 4096 keys and 256 segments
 * per group); a group made only of segments of at most 32 keys becomes one
 * warp per segment; longer segments take the passes, in tiles of the pass
 * shape a plan chooses by default. Same offsets contract as
 * gs_segmented_plan_create. */
typedef enum gs_seg_kind {
  GS_SEG_EMPTY = 0,
  GS_SEG_WARP = 1,
  GS_SEG_GROUP = 2,
  GS_SEG_PASSES = 3
} gs_seg_kind;
gs_status gs_segmented_layout(gs_dtype dtype, uint64_t n, const uint64_t* host_offsets,
                              uint32_t nseg, uint8_t* kinds, uint64_t counts[4]);

/* Apply a permutation to a value array: out[i] = in[perm[i]], element size
 * `elem_bytes` (1..64 bytes). Replaces ParUtils::ArrangeValues
 * (include/par/par_utils.h:23-86), which moves each value vector to where
 * its key went after a sort of (key, global index). Device pointers, or
 * host pointers (values, result and perm) with GS_FLAG_HOST; `in` and
 * `out` must not alias. */
gs_status gs_gather(gs_ctx* ctx, const void* in, void* out, uint64_t n,
                    uint32_t elem_bytes, const uint64_t* perm, uint32_t flags);

/* Per-phase device times (milliseconds) of the last completed sort on this
 * context, named like the reference's benchmark timers
 * (include/helpers/hyksort_helper.h:643-650): "Local sort",
 * "Select splitters", "Exchange data", "Merge data", "Total". Writes up to
 * `cap` (name, ms) entries; returns how many exist. Names are static
 * strings. Only filled when timing was enabled with gs_ctx_set_timing. */
int gs_phase_times(gs_ctx* ctx, const char** names, double* ms, int cap);
gs_status gs_ctx_set_timing(gs_ctx* ctx, int enable);

/* Device time (ms) of each kernel of the last radix pipeline when timing is
 * on: [0] upsweep histogram (with its memset), [1] plan, [2 + q] pass of
 * digit q (about 0 when the digit was skipped). Returns the entry count.
 * The reference's GPU sub-phase timers ("Local sort sort/transfer/merge",
 * src/cuda_utils.cu:29-34) are the counterpart. */
int gs_kernel_times(gs_ctx* ctx, double* ms, int cap);

/* Test hooks for failure detection without a GPU fault.
 * GS_DEBUG_SPIN_LIMIT: iteration cap of every inter-block wait.
 * GS_DEBUG_INJECT_STALL: when non-zero, one tile of the next sort waits for
 * a predecessor flag that is never set, so the wait runs out after the spin
 * limit and the call reports GS_ERR_TIMEOUT.
 * GS_DEBUG_BUDGET: replace the HBM budget (bytes).
 * GS_DEBUG_PASS_SHAPE: tile shape of the radix pass kernel (threads x items
 * per thread x blocks per SM); the autotuner sets it.
 * GS_DEBUG_HOST_GROUPS: bucket groups of a GS_FLAG_HOST radix sort with
 * pinned buffers on both ends: sorted groups leave for the host while the
 * next group sorts. 0 or 1: sort everything, then copy out; UINT64_MAX
 * (default): by size (24 from 2^29 elements, 16 from 2^28, 8 from 2^26, 4
 * from 2^25, none below).
 * GS_DEBUG_HOST_CHUNKED: from this many keys (default 2^28; 0: never), a
 * keys-only grouped host sort reads its input in 8 chunks and splits each
 * while the next crosses the link. */
#define GS_DEBUG_SPIN_LIMIT   1
#define GS_DEBUG_INJECT_STALL 2
#define GS_DEBUG_BUDGET       3
#define GS_DEBUG_PASS_SHAPE   4  /* pass-kernel tile shape 0..2 (tuning);
                                    UINT64_MAX: per-type default */
#define GS_DEBUG_HOST_GROUPS  5  /* 0..256; UINT64_MAX: by size */
#define GS_DEBUG_HOST_CHUNKED 6  /* smallest keys-only grouped host sort
                                    whose input is split chunk by chunk as
                                    it arrives (default 2^28; 0: never) */
gs_status gs_debug_set(gs_ctx* ctx, int key, uint64_t value);

/* ---- Tuning table (autotuner output) ----
 * No counterpart in the reference, whose algorithm parameters are
 * hard-coded (include/helpers/hyksort_helper.h:343-344,
 * include/helpers/samplesort_helper.h:429, src/cuda_utils.cu:515). The
 * engine's radix digit is fixed at 8 bits; what a table chooses per key
 * type, payload width and size is the pass kernel's tile shape (threads x
 * items per thread) and the SampleSort bucket count. gpusort_gb300.autotune
 * measures them on the device and writes the JSON file that
 * gs_ctx_load_tuning reads. An explicit GS_DEBUG_PASS_SHAPE or
 * gs_opts.partitions still wins over the table. */
typedef struct gs_tuning_entry {
  int32_t key_dtype;      /* gs_dtype */
  int32_t val_bytes;      /* payload bytes: 0 (keys only), 4 or 8 */
  uint32_t log2n_min;     /* applies when floor(log2(n)) is in [min, max] */
  uint32_t log2n_max;
  int32_t pass_shape;     /* radix pass tile shape, -1: engine default */
  uint32_t partitions;    /* SampleSort buckets when gs_opts leaves 0; 0: default */
} gs_tuning_entry;
/* Number of pass tile shapes and the threads / items per thread of one. */
int gs_pass_shape_count(void);
gs_status gs_pass_shape_info(int key_bytes, int val_bytes, int shape, uint32_t* threads,
                             uint32_t* items_per_thread);
/* Replace the context's table (count 0 clears it); the first matching
 * entry wins. */
gs_status gs_ctx_set_tuning(gs_ctx* ctx, const gs_tuning_entry* entries, uint32_t count);
/* Parse a tuning JSON document: {"entries": [{"key_dtype": "u32" | 0..5,
 * "val_bytes": .., "log2n_min": .., "log2n_max": .., "pass_shape": ..,
 * "partitions": ..}, ...]} (other keys are ignored). Returns the number of
 * entries (all written when <= capacity), or -1 on a syntax error. */
int gs_tuning_parse(const char* json, gs_tuning_entry* out, uint32_t capacity);
/* Read and apply a tuning JSON file. */
gs_status gs_ctx_load_tuning(gs_ctx* ctx, const char* path);
/* The pass shape and SampleSort bucket count the context uses for a call. */
gs_status gs_ctx_choice(gs_ctx* ctx, gs_dtype key_dtype, int val_bytes, uint64_t n,
                        int* pass_shape, uint32_t* partitions);

/* Sort 32-bit keys (GS_U32, GS_I32, GS_F32) in device memory WITHOUT
 * ALLOCATING. No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc - code running under a framework whose caching
 * allocator owns the device memory, latency-critical paths where
 * cudaMalloc/cudaFree would synchronise the device, plugins whose host
 * forbids allocation after start-up.
 * - Scratch is one fixed device array inside the library (about 4.2 MiB per
 *   GPU that loads it, held until the process exits). n may be at most
 *   GS_NOALLOC_MAX_KEYS; larger n returns GS_ERR_TOO_LARGE. Up to 4096
 *   keys are sorted in one CTA's shared memory and use no scratch.
 * - The caller passes device input and output (they may alias) and a CUDA
 *   stream (NULL: the legacy default stream). Flags: GS_FLAG_DESCENDING,
 *   and GS_FLAG_SYNC to wait and report GS_ERR_TIMEOUT.
 * - The first call on a device sets up that device's scratch address and
 *   clears it, waiting for the device (cudaDeviceSynchronize) so that the
 *   clear is done before any sort on any stream; make that first call
 *   before any stream capture.
 * - Every call on a device shares the one scratch array: calls that overlap
 *   on the GPU (other streams, other threads) race and corrupt each other.
 * - Errors are described by gs_last_global_error(). */
#define GS_NOALLOC_MAX_KEYS (1ull << 20)
gs_status gs_sort_keys_noalloc(gs_dtype dtype, const void* in, void* out,
                               uint64_t n, uint32_t flags, void* stream);

/* ---- Per-rank binary files ----
 * The reference's test driver keeps one file per MPI rank, <dir>/<rank><ext>
 * (".dat" by default), holding a native int64 element count followed by the
 * raw elements (src/test/utils.h:610-661: GetFilePath, ReadData, SaveData,
 * SaveMyData; src/test/ifstream.h:38-73, src/test/ofstream.h:34-64). Here
 * the p rank files of a job are the p partitions of one array.
 * - By default `dst` / `src` are device memory of the context's device and
 *   the data streams through pinned staging buffers on the context's stream
 *   (the call returns when the data has landed); with GS_FLAG_HOST they are
 *   host memory and `ctx` may be NULL.
 * - gs_partitions_write splits n elements over nparts files with the
 *   reference's block size (include/common.h:146-155) and gives the last file
 *   the remainder. (The reference's SaveData writes the block size for every
 *   rank and so drops the tail when the last block is the larger one, e.g.
 *   9 elements over 4 ranks; files it does write read back identically.)
 * - Errors are described by gs_last_global_error(). */
int64_t gs_file_count(const char* path);  /* element count, -1 if unreadable */
gs_status gs_file_read(gs_ctx* ctx, const char* path, void* dst, uint64_t capacity,
                       uint32_t elem_bytes, uint32_t flags, uint64_t* n_read);
gs_status gs_file_write(gs_ctx* ctx, const char* path, const void* src, uint64_t n,
                        uint32_t elem_bytes, uint32_t flags);
gs_status gs_partitions_read(gs_ctx* ctx, const char* dir, const char* ext, int nparts,
                             void* dst, uint64_t capacity, uint32_t elem_bytes,
                             uint32_t flags, uint64_t* n_total);
gs_status gs_partitions_write(gs_ctx* ctx, const char* dir, const char* ext, int nparts,
                              const void* src, uint64_t n, uint32_t elem_bytes,
                              uint32_t flags);
/* Elements in each of the first nparts-1 files of gs_partitions_write. */
uint64_t gs_partition_block(uint64_t n, int nparts);

/* ---- Serving loop (continuous batching) ----
 * No counterpart in the reference (its callers sort one array per call,
 * src/test/utils.h:776-791); the request interface follows the sort calls
 * above. A server owns one device:
 * - an HBM arena of `hbm_budget` bytes, allocated once, from which each
 *   admitted request takes its scratch (and, with GS_FLAG_HOST, its staged
 *   data); admission waits while the arena is full, so the budget bounds
 *   the device memory of everything in flight;
 * - `slots` CUDA streams, each with its own look-back words and work area;
 * - one device-owner thread that admits queued requests in arrival order as
 *   slots and arena space free up (a request that does not fit yet holds
 *   the head of the queue), so work of requests that arrive while others
 *   run overlaps on the device.
 * - small requests (device memory, keys only, at most 4096 keys) that are
 *   queued together run in one launch, one CTA each.
 * Requests are sorts of keys or (key, value) pairs with the flags of
 * gs_sort_pairs (GS_FLAG_DESCENDING, GS_FLAG_PAIRS_STABLE). By default the
 * pointers are device memory on the server's device, which stays the
 * caller's until the request completes (keys_out may equal keys_in); with
 * GS_FLAG_HOST they are host memory (pinned memory lets the copies overlap)
 * and the server copies in and out. Results are the bytes gs_sort_pairs /
 * gs_sort_keys return for the same input. */
typedef struct gs_server gs_server;
typedef struct gs_server_opts {
  uint64_t hbm_budget;        /* arena bytes (0: 1 GiB) */
  uint64_t max_request_keys;  /* largest n accepted (0: 2^26) */
  uint32_t slots;             /* requests on the device at once (0: 8; <= 32) */
  uint32_t max_queue;         /* queued requests before submit returns
                                 GS_ERR_BUSY (0: 65536) */
} gs_server_opts;

typedef struct gs_server_stats {
  uint64_t completed;         /* requests finished since the last reset */
  uint64_t keys_done;         /* their keys */
  uint64_t queued;            /* waiting for admission now */
  uint64_t running;           /* admitted, not finished */
  uint64_t arena_used;        /* arena bytes held now */
  uint64_t arena_peak;        /* most arena bytes held since the last reset */
  double p50_ms, p99_ms, mean_ms, max_ms;  /* submit -> completion */
} gs_server_stats;

/* Returns NULL on failure (gs_last_global_error() says why). */
gs_server* gs_server_create(int device, const gs_server_opts* opts);
/* Cancels queued requests, waits for admitted ones, frees everything. */
void gs_server_destroy(gs_server* server);
/* Queue one request; *request_id identifies it for poll/cancel. Errors:
 * GS_ERR_EMPTY (n == 0), GS_ERR_TOO_LARGE (n > max_request_keys),
 * GS_ERR_OOM (needs more than the whole arena), GS_ERR_BUSY (queue full). */
gs_status gs_server_submit(gs_server* server, gs_dtype key_dtype, int has_values,
                           gs_dtype val_dtype, const void* keys_in, const void* vals_in,
                           void* keys_out, void* vals_out, uint64_t n, uint32_t flags,
                           uint64_t* request_id);
/* GS_ERR_BUSY while the request is queued or running (wait = 0), else its
 * final status (GS_OK, GS_ERR_TIMEOUT, GS_ERR_CUDA, GS_ERR_CANCELLED); the
 * final status is returned once, after which the id is unknown
 * (GS_ERR_INVALID). latency_ms (may be NULL) gets submit -> completion. */
gs_status gs_server_poll(gs_server* server, uint64_t request_id, int wait, double* latency_ms);
/* Cancel a request that is still queued (GS_OK); GS_ERR_BUSY if it was
 * already admitted (it then runs to completion). */
gs_status gs_server_cancel(gs_server* server, uint64_t request_id);
/* Snapshot of the counters; reset != 0 clears completed/keys/latencies/peak. */
gs_status gs_server_get_stats(gs_server* server, gs_server_stats* out, int reset);

#ifdef __cplusplus
}  /* extern "C" */
#endif

#endif  /* GPUSORT_GB300_H_ */
