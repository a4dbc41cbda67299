// gs_sort_keys_noalloc: sort 32-bit keys without allocating any memory.
//
// Some callers cannot call cudaMalloc:
// - code that runs under a framework whose caching allocator already owns
//   the device memory, where an allocation from outside it can fail or
//   break the framework's accounting;
// - latency-critical paths, where cudaMalloc/cudaFree would synchronise the
//   device;
// - plugins whose host application forbids device allocation after start-up.
// For them this entry point runs the same radix pipeline as gs_sort_keys. It
// uses a fixed scratch area declared below as a file-scope device array, so
// every GPU that loads the library holds that array until the process
// exits. The caller still provides the input and output buffers.
#include <atomic>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/gpusort_gb300.h"
#include "common.cuh"
#include "engine.h"
#include "radix_types.cuh"

namespace {

constexpr uint64_t kMaxKeys = GS_NOALLOC_MAX_KEYS;           // 2^20 keys
constexpr uint32_t kTile = gs::RADIX_TILE_U32_SHAPE0;         // keys per pass tile
constexpr size_t kAltBytes = size_t(kMaxKeys) * 4;            // ping-pong keys
// One look-back word per tile and digit.
constexpr size_t kStatusBytes = size_t((kMaxKeys + kTile - 1) / kTile) * gs::RADIX * 8;
constexpr size_t kWorkBytes = (sizeof(gs::SortWork) + 255) / 256 * 256;
constexpr size_t kErrBytes = 256;
constexpr size_t kScratchBytes = kAltBytes + kStatusBytes + kWorkBytes + kErrBytes;

// The shared scratch of every call on this device (about 4.2 MB). Host code
// must not use this name as an address: it is the host-side shadow of the
// symbol. The device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
struct DeviceSlot {
  std::once_flag once;
  cudaError_t setup_err = cudaSuccess;
  unsigned char* scratch = nullptr;  // device address of g_noalloc_scratch
  gs::DeviceProps props;
  std::atomic<uint32_t> gen{0};
};
DeviceSlot g_slots[kMaxDevices];

gs_status fail(gs_status st, const std::string& msg) {
  gs::set_last_global_error(msg);  // read with gs_last_global_error()
  return st;
}

// Once per device, with that device current: find the array's device
// address and clear the look-back words and the work area (the look-back
// tags are drawn from a counter there, which must start at 0). cudaMemset
// is asynchronous and runs on the legacy default stream, which a
// non-blocking caller stream does not wait for, so the set-up waits for the
// device: the clear is done before the first sort is enqueued on any stream.
// This is why the first call on a device must not come during a stream
// capture.
void setup(int dev, DeviceSlot& s) {
  void* p = nullptr;
  s.setup_err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (s.setup_err != cudaSuccess) return;
  s.scratch = static_cast<unsigned char*>(p);
  s.setup_err = cudaMemset(s.scratch + kAltBytes, 0, kStatusBytes + kWorkBytes);
  if (s.setup_err == cudaSuccess) s.setup_err = cudaDeviceSynchronize();
  if (s.setup_err != cudaSuccess) return;
  s.props.device = dev;
  cudaDeviceGetAttribute(&s.props.num_sms, cudaDevAttrMultiProcessorCount, dev);
  int optin = 0;
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  s.props.smem_optin = size_t(optin);
}

}  // namespace

extern "C" {

gs_status gs_sort_keys_noalloc(gs_dtype dtype, const void* in, void* out, uint64_t n,
                               uint32_t flags, void* stream) {
  uint32_t kind = 0;
  switch (dtype) {
    case GS_U32: kind = gs::KIND_UNSIGNED; break;
    case GS_I32: kind = gs::KIND_SIGNED; break;
    case GS_F32: kind = gs::KIND_FLOAT; break;
    default: return fail(GS_ERR_BAD_DTYPE, "gs_sort_keys_noalloc sorts 32-bit keys only");
  }
  if (n == 0) return fail(GS_ERR_EMPTY, "No data to sort.");
  if (n > kMaxKeys)
    return fail(GS_ERR_TOO_LARGE, "gs_sort_keys_noalloc: n = " + std::to_string(n) +
                                      " exceeds its fixed scratch limit of " +
                                      std::to_string(kMaxKeys) + " keys");
  if (!in || !out) return fail(GS_ERR_INVALID, "null data pointer");
  if (gs::radix_status_words_u32_shape0(n) * sizeof(uint64_t) > kStatusBytes)
    return fail(GS_ERR_INVALID, "gs_sort_keys_noalloc: look-back area too small");
  if (flags & GS_FLAG_HOST)
    return fail(GS_ERR_INVALID, "gs_sort_keys_noalloc takes device pointers only");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(GS_ERR_NO_DEVICE, "no current CUDA device");
  DeviceSlot& s = g_slots[dev];
  std::call_once(s.once, setup, dev, std::ref(s));
  if (s.setup_err != cudaSuccess)
    return fail(GS_ERR_CUDA, std::string("no-alloc scratch set-up: ") +
                                 cudaGetErrorString(s.setup_err));
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (n <= gs::small_sort_max()) {
    // One CTA sorts in its shared memory: no scratch at all.
    cudaError_t e = gs::launch_small_sort(in, out, uint32_t(n), 4, kind,
                                          (flags & GS_FLAG_DESCENDING) != 0, st);
    if (e == cudaSuccess && (flags & GS_FLAG_SYNC)) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(GS_ERR_CUDA, std::string("small sort: ") +
                                                       cudaGetErrorString(e));
    return GS_OK;
  }
  unsigned char* base = s.scratch;
  gs::RadixJob job;
  job.keys_in = in;
  job.keys_out = out;
  job.keys_alt = base;
  job.status = reinterpret_cast<uint64_t*>(base + kAltBytes);
  job.work = reinterpret_cast<gs::SortWork*>(base + kAltBytes + kStatusBytes);
  job.err = reinterpret_cast<uint32_t*>(base + kAltBytes + kStatusBytes + kWorkBytes);
  job.n = n;
  job.key_bytes = 4;
  job.key_kind = kind;
  job.desc = (flags & GS_FLAG_DESCENDING) != 0;
  // Look-back tags are drawn on the device from the work area's counter.
  uint32_t gen = 0;
  cudaError_t e = cudaMemsetAsync(job.err, 0, sizeof(uint32_t), st);
  if (e == cudaSuccess) e = gs::launch_radix_sort(job, s.props, &gen, st);
  if (e != cudaSuccess) return fail(GS_ERR_CUDA, std::string("launch: ") + cudaGetErrorString(e));
  if (flags & GS_FLAG_SYNC) {
    uint32_t h = 0;
    e = cudaStreamSynchronize(st);
    if (e == cudaSuccess) e = cudaMemcpy(&h, job.err, sizeof(h), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return fail(GS_ERR_CUDA, cudaGetErrorString(e));
    if (h) return fail(GS_ERR_TIMEOUT, "device wait ran out or scatter out of range");
  }
  return GS_OK;
}

}  // extern "C"
