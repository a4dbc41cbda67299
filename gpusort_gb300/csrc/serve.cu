// Serving loop: sort requests of mixed sizes and key types admitted by HBM
// budget, with continuous batching on CUDA streams (gs_server_* in
// gpusort_gb300.h). The reference has no server; this subsystem sits in
// front of the same radix pipeline the plain calls use, so a request's
// bytes are the ones gs_sort_pairs / gs_sort_keys give for its input.
//
// * Memory: one arena of the admission budget is allocated when the server
//   starts; each request takes its scratch (and, for host requests, its
//   staged data) from it, first fit over a coalescing free list. The loop
//   itself never allocates or frees device memory (cudaFree would
//   synchronise the device and stall the other streams).
// * Slots: each slot owns a non-blocking stream, a work area, look-back
//   words sized for the largest admissible request, an error word and a
//   pinned copy of it. A request runs on one slot: [copy in], radix sort,
//   [copy out], error word to the host, then a host callback that marks the
//   slot finished and wakes the loop (no polling of events).
// * Loop: one device-owner thread reaps finished slots, then admits queued
//   requests in arrival order while a slot is idle and the arena has room.
//   A request that does not fit yet holds the head of the queue, so large
//   requests are not starved by smaller ones behind them. Kernel launches
//   happen outside the lock, so submitters never wait on the GPU.
// * Batching: small requests (device memory, keys only, at most 4096 keys)
//   need no scratch. The ones queued together behind each other, of one key
//   width, take one slot and run as one launch: one CTA per request sorts it
//   in shared memory, reading its descriptor from the slot's mapped pinned
//   array.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/gpusort_gb300.h"
#include "common.cuh"
#include "engine.h"
#include "radix_types.cuh"

namespace {

using Clock = std::chrono::steady_clock;

constexpr uint32_t MAX_SLOTS = 32;
constexpr uint64_t ALIGN = 256;

uint64_t align_up(uint64_t b) { return (b + ALIGN - 1) & ~(ALIGN - 1); }

// First-fit allocator over one device range; neighbours coalesce on release.
struct Arena {
  uint8_t* base = nullptr;
  uint64_t size = 0;
  uint64_t used = 0, peak = 0;
  std::map<uint64_t, uint64_t> free_list;  // offset -> length

  bool alloc(uint64_t bytes, uint64_t* off) {
    for (auto it = free_list.begin(); it != free_list.end(); ++it) {
      if (it->second < bytes) continue;
      *off = it->first;
      const uint64_t rest = it->second - bytes, roff = it->first + bytes;
      free_list.erase(it);
      if (rest) free_list[roff] = rest;
      used += bytes;
      peak = std::max(peak, used);
      return true;
    }
    return false;
  }
  void release(uint64_t off, uint64_t bytes) {
    used -= bytes;
    auto it = free_list.emplace(off, bytes).first;
    auto next = std::next(it);
    if (next != free_list.end() && it->first + it->second == next->first) {
      it->second += next->second;
      free_list.erase(next);
    }
    if (it != free_list.begin()) {
      auto prev = std::prev(it);
      if (prev->first + prev->second == it->first) {
        prev->second += it->second;
        free_list.erase(it);
      }
    }
  }
};

enum class State { QUEUED, RUNNING, DONE };

struct Request {
  uint64_t id = 0;
  bool has_v = false, host = false;
  const void* kin = nullptr;
  const void* vin = nullptr;
  void* kout = nullptr;
  void* vout = nullptr;
  uint64_t n = 0;
  uint32_t flags = 0;
  int kb = 4, vb = 0;
  uint32_t kk = 0, vk = 0;
  uint64_t off = 0, bytes = 0;  // arena range
  bool small = false;           // device keys-only of <= small_sort_max keys: batched
  Clock::time_point t_submit, t_done;
  State state = State::QUEUED;
  gs_status status = GS_OK;
};

struct Slot {
  gs_server* server = nullptr;
  cudaStream_t stream = nullptr;
  gs::SortWork* work = nullptr;
  uint64_t* status = nullptr;
  uint32_t* err = nullptr;
  uint32_t* h_err = nullptr;  // pinned
  gs::SmallSortReq* h_reqs = nullptr;        // pinned, device-mapped batch descriptors
  gs::SmallSortReq* d_reqs = nullptr;        // the device's view of h_reqs
  std::vector<Request*> batch;               // running requests; empty: idle
  bool finished = false;
  bool launch_failed = false;
};

// Small requests (device memory, keys only, at most small_sort_max keys) of
// one key width that are queued together run in one launch, one CTA each.
constexpr uint32_t MAX_BATCH = 256;

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

}  // namespace

struct gs_server {
  int device = 0;
  gs::DeviceProps props;
  uint64_t max_n = 0;
  uint32_t max_queue = 0;
  size_t status_words = 0;
  Arena arena;
  std::vector<Slot> slots;
  std::mutex mu;
  std::condition_variable cv;       // wakes the loop
  std::condition_variable done_cv;  // wakes pollers
  uint64_t events = 0;              // bumped on every change the loop reacts to
  std::deque<Request*> queue;
  std::unordered_map<uint64_t, Request*> reqs;
  std::vector<double> latencies_ms;
  uint64_t completed = 0, keys_done = 0;
  uint64_t next_id = 1;
  bool running = true;
  std::thread loop;
};

namespace {

void notify_locked(gs_server* s) {
  ++s->events;
  s->cv.notify_all();
}

// Runs on a CUDA driver thread after the slot's work: no CUDA calls here.
void CUDART_CB slot_done(void* p) {
  Slot* sl = static_cast<Slot*>(p);
  gs_server* s = sl->server;
  std::lock_guard<std::mutex> lock(s->mu);
  sl->finished = true;
  const auto now = Clock::now();
  for (Request* r : sl->batch) r->t_done = now;
  notify_locked(s);
}

// Enqueue a batch of small requests: one launch sorts each in its own CTA.
void start_small(gs_server* s, Slot& sl) {
  const uint32_t count = uint32_t(sl.batch.size());
  for (uint32_t i = 0; i < count; ++i) {
    const Request* r = sl.batch[i];
    sl.h_reqs[i] = gs::SmallSortReq{r->kin, r->kout, uint32_t(r->n), r->kk,
                                    (r->flags & GS_FLAG_DESCENDING) ? 1u : 0u, 0u};
  }
  cudaError_t e = cudaMemsetAsync(sl.err, 0, sizeof(uint32_t), sl.stream);
  if (e == cudaSuccess) e = gs::launch_small_sort_batch(sl.d_reqs, count, sl.batch[0]->kb, sl.stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_err, sl.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.stream);
  if (e == cudaSuccess) e = cudaLaunchHostFunc(sl.stream, slot_done, &sl);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaStreamSynchronize(sl.stream);
    std::lock_guard<std::mutex> lock(s->mu);
    sl.launch_failed = true;
    sl.finished = true;
    for (Request* r : sl.batch) r->t_done = Clock::now();
    notify_locked(s);
  }
}

// Enqueue a request's work on its slot (owner thread, lock not held).
void start(gs_server* s, Slot& sl) {
  if (sl.batch[0]->small) {
    start_small(s, sl);
    return;
  }
  Request* r = sl.batch[0];
  uint8_t* base = s->arena.base + r->off;
  const uint64_t n = r->n, kbytes = n * r->kb, vbytes = n * r->vb;
  const void* kin = r->kin;
  const void* vin = r->vin;
  void* kout = r->kout;
  void* vout = r->vout;
  uint8_t* p = base;
  cudaError_t e = cudaSuccess;
  if (r->host) {  // staged: sort in place in the arena
    void* dk = p;
    p += align_up(kbytes);
    void* dv = r->has_v ? p : nullptr;
    p += align_up(vbytes);
    e = cudaMemcpyAsync(dk, r->kin, kbytes, cudaMemcpyHostToDevice, sl.stream);
    if (e == cudaSuccess && r->has_v)
      e = cudaMemcpyAsync(dv, r->vin, vbytes, cudaMemcpyHostToDevice, sl.stream);
    kin = kout = dk;
    vin = vout = dv;
  }
  void* ak = p;
  p += align_up(kbytes);
  void* av = r->has_v ? p : nullptr;
  if (e == cudaSuccess) e = cudaMemsetAsync(sl.err, 0, sizeof(uint32_t), sl.stream);
  gs::RadixJob job;
  job.keys_in = kin;
  job.keys_out = kout;
  job.keys_alt = ak;
  job.vals_in = vin;
  job.vals_out = vout;
  job.vals_alt = av;
  job.n = n;
  job.key_bytes = r->kb;
  job.val_bytes = r->vb;
  job.key_kind = r->kk;
  job.val_kind = r->vk;
  job.desc = r->flags & GS_FLAG_DESCENDING;
  const bool stable = r->flags & GS_FLAG_PAIRS_STABLE;
  job.ties_by_value = r->has_v && !stable;
  job.reverse_first = r->has_v && stable && job.desc;
  job.first_unstable = !(r->has_v && stable);
  job.status = sl.status;
  job.work = sl.work;
  job.err = sl.err;
  job.shape = gs::radix_default_shape(r->kb, r->vb, n);
  uint32_t gen_unused = 0;
  if (e == cudaSuccess) {
    if (!r->has_v && n <= gs::small_sort_max())  // one CTA in shared memory
      e = gs::launch_small_sort(kin, kout, uint32_t(n), r->kb, r->kk, job.desc, sl.stream);
    else
      e = gs::launch_radix_sort(job, s->props, &gen_unused, sl.stream);
  }
  if (r->host) {
    if (e == cudaSuccess) e = cudaMemcpyAsync(r->kout, kout, kbytes, cudaMemcpyDeviceToHost, sl.stream);
    if (e == cudaSuccess && r->has_v)
      e = cudaMemcpyAsync(r->vout, vout, vbytes, cudaMemcpyDeviceToHost, sl.stream);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_err, sl.err, sizeof(uint32_t), cudaMemcpyDeviceToHost, sl.stream);
  if (e == cudaSuccess) e = cudaLaunchHostFunc(sl.stream, slot_done, &sl);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaStreamSynchronize(sl.stream);
    std::lock_guard<std::mutex> lock(s->mu);
    sl.launch_failed = true;
    sl.finished = true;
    r->t_done = Clock::now();
    notify_locked(s);
  }
}

// Retire a finished slot (lock held).
void finish_locked(gs_server* s, Slot& sl) {
  for (Request* r : sl.batch) {
    if (sl.launch_failed) r->status = GS_ERR_CUDA;
    else r->status = *sl.h_err ? GS_ERR_TIMEOUT : GS_OK;
    if (r->bytes) s->arena.release(r->off, r->bytes);
    r->state = State::DONE;
    s->latencies_ms.push_back(
        std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count());
    ++s->completed;
    s->keys_done += r->n;
  }
  sl.batch.clear();
  sl.finished = false;
  sl.launch_failed = false;
  s->done_cv.notify_all();
}

void run_loop(gs_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lock(s->mu);
  std::vector<Slot*> to_start;
  while (true) {
    const uint64_t seen = s->events;
    bool busy = false;
    for (Slot& sl : s->slots) {
      if (!sl.batch.empty() && sl.finished) finish_locked(s, sl);
      busy |= !sl.batch.empty();
    }
    to_start.clear();
    for (Slot& sl : s->slots) {
      if (s->queue.empty()) break;
      if (!sl.batch.empty()) continue;
      Request* r = s->queue.front();
      if (r->small) {  // this and the small requests right behind it, one launch
        const int kb = r->kb;
        while (!s->queue.empty() && s->queue.front()->small && s->queue.front()->kb == kb &&
               sl.batch.size() < MAX_BATCH) {
          Request* q = s->queue.front();
          q->state = State::RUNNING;
          s->queue.pop_front();
          sl.batch.push_back(q);
        }
      } else {
        uint64_t off = 0;
        if (!s->arena.alloc(r->bytes, &off)) break;  // holds the head
        r->off = off;
        r->state = State::RUNNING;
        s->queue.pop_front();
        sl.batch.push_back(r);
      }
      to_start.push_back(&sl);
    }
    if (!to_start.empty()) {
      lock.unlock();
      for (Slot* sl : to_start) start(s, *sl);
      lock.lock();
      continue;
    }
    if (!s->running && s->queue.empty() && !busy) return;
    s->cv.wait(lock, [&] { return s->events != seen; });
  }
}

void free_server(gs_server* s) {
  cudaSetDevice(s->device);
  for (Slot& sl : s->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.work) cudaFree(sl.work);
    if (sl.status) cudaFree(sl.status);
    if (sl.err) cudaFree(sl.err);
    if (sl.h_err) cudaFreeHost(sl.h_err);
    if (sl.h_reqs) cudaFreeHost(sl.h_reqs);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  if (s->arena.base) cudaFree(s->arena.base);
  for (auto& kv : s->reqs) delete kv.second;
  delete s;
}

}  // namespace

extern "C" {

gs_server* gs_server_create(int device, const gs_server_opts* opts) {
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    gs::set_last_global_error("no such CUDA device for the server");
    return nullptr;
  }
  gs_server_opts o{};
  if (opts) o = *opts;
  if (o.hbm_budget == 0) o.hbm_budget = 1ull << 30;
  if (o.max_request_keys == 0) o.max_request_keys = 1ull << 26;
  if (o.max_request_keys > 0xFFFFFFFFull) o.max_request_keys = 0xFFFFFFFFull;
  if (o.slots == 0) o.slots = 8;
  if (o.slots > MAX_SLOTS) o.slots = MAX_SLOTS;
  if (o.max_queue == 0) o.max_queue = 65536;
  cudaSetDevice(device);
  gs_server* s = new gs_server();
  s->device = device;
  s->props.device = device;
  int v = 0;
  cudaDeviceGetAttribute(&s->props.num_sms, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
  s->props.smem_optin = size_t(v);
  s->max_n = o.max_request_keys;
  s->max_queue = o.max_queue;
  for (int kb : {4, 8})
    for (int vb : {0, 4, 8})
      s->status_words = std::max(s->status_words, gs::radix_status_words(s->max_n, kb, vb));
  const size_t status_bytes = s->status_words * sizeof(uint64_t);
  s->arena.size = o.hbm_budget & ~(ALIGN - 1);
  bool ok = cudaMalloc(&s->arena.base, s->arena.size) == cudaSuccess;
  if (ok) s->arena.free_list[0] = s->arena.size;
  s->slots.resize(o.slots);
  for (Slot& sl : s->slots) {
    sl.server = s;
    ok = ok && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) == cudaSuccess &&
         cudaMalloc(&sl.work, gs::sort_work_bytes()) == cudaSuccess &&
         cudaMalloc(&sl.status, status_bytes) == cudaSuccess &&
         cudaMalloc(&sl.err, ALIGN) == cudaSuccess &&
         cudaMallocHost(&sl.h_err, sizeof(uint32_t)) == cudaSuccess &&
         cudaHostAlloc(&sl.h_reqs, MAX_BATCH * sizeof(gs::SmallSortReq), cudaHostAllocMapped) ==
             cudaSuccess &&
         cudaHostGetDevicePointer(reinterpret_cast<void**>(&sl.d_reqs), sl.h_reqs, 0) ==
             cudaSuccess &&
         cudaMemset(sl.work, 0, gs::sort_work_bytes()) == cudaSuccess &&
         cudaMemset(sl.status, 0, status_bytes) == cudaSuccess;
  }
  if (ok) ok = cudaDeviceSynchronize() == cudaSuccess;
  if (!ok) {
    cudaGetLastError();
    gs::set_last_global_error("server allocation failed (HBM budget or slots too large)");
    free_server(s);
    return nullptr;
  }
  s->loop = std::thread(run_loop, s);
  return s;
}

void gs_server_destroy(gs_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->running = false;
    for (Request* r : s->queue) {
      r->state = State::DONE;
      r->status = GS_ERR_CANCELLED;
      r->t_done = Clock::now();
    }
    s->queue.clear();
    notify_locked(s);
    s->done_cv.notify_all();
  }
  if (s->loop.joinable()) s->loop.join();
  free_server(s);
}

gs_status gs_server_submit(gs_server* s, gs_dtype key_dtype, int has_values, gs_dtype val_dtype,
                           const void* keys_in, const void* vals_in, void* keys_out,
                           void* vals_out, uint64_t n, uint32_t flags, uint64_t* request_id) {
  auto fail = [](gs_status st, const char* m) {
    gs::set_last_global_error(m);
    return st;
  };
  if (!s || !request_id) return fail(GS_ERR_INVALID, "null server or request id");
  Request r;
  if (!dtype_info(key_dtype, &r.kb, &r.kk)) return fail(GS_ERR_BAD_DTYPE, "unknown key dtype");
  r.has_v = has_values != 0;
  if (r.has_v && !dtype_info(val_dtype, &r.vb, &r.vk))
    return fail(GS_ERR_BAD_DTYPE, "unknown value dtype");
  if (!r.has_v) r.vb = 0;
  if (n == 0) return fail(GS_ERR_EMPTY, "No data to sort.");
  if (n > s->max_n) return fail(GS_ERR_TOO_LARGE, "request larger than max_request_keys");
  if (!keys_in || !keys_out || (r.has_v && (!vals_in || !vals_out)))
    return fail(GS_ERR_INVALID, "null data pointer");
  if (flags & ~(GS_FLAG_DESCENDING | GS_FLAG_PAIRS_STABLE | GS_FLAG_HOST))
    return fail(GS_ERR_INVALID, "unsupported flag for a served request");
  r.host = flags & GS_FLAG_HOST;
  if (!r.host) {  // device requests must live on the server's device
    const void* ptrs[4] = {keys_in, keys_out, r.has_v ? vals_in : nullptr,
                           r.has_v ? vals_out : nullptr};
    for (const void* ptr : ptrs) {
      if (!ptr) continue;
      cudaPointerAttributes a{};
      if (cudaPointerGetAttributes(&a, ptr) != cudaSuccess ||
          (a.type != cudaMemoryTypeDevice && a.type != cudaMemoryTypeManaged) ||
          a.device != s->device) {
        cudaGetLastError();
        return fail(GS_ERR_INVALID, "pointer is not device memory of the server's device");
      }
    }
  }
  const uint64_t kbytes = align_up(n * r.kb), vbytes = align_up(n * r.vb);
  r.small = !r.host && !r.has_v && n <= gs::small_sort_max();
  r.bytes = r.small ? 0 : (r.host ? 2 : 1) * (kbytes + vbytes);
  if (r.bytes > s->arena.size) return fail(GS_ERR_OOM, "request larger than the HBM budget");
  r.kin = keys_in;
  r.vin = r.has_v ? vals_in : nullptr;
  r.kout = keys_out;
  r.vout = r.has_v ? vals_out : nullptr;
  r.n = n;
  r.flags = flags;
  r.t_submit = Clock::now();
  std::lock_guard<std::mutex> lock(s->mu);
  if (!s->running) return fail(GS_ERR_INVALID, "server is shutting down");
  if (s->queue.size() >= s->max_queue) return fail(GS_ERR_BUSY, "server queue is full");
  Request* q = new Request(r);
  q->id = s->next_id++;
  s->reqs[q->id] = q;
  s->queue.push_back(q);
  *request_id = q->id;
  notify_locked(s);
  return GS_OK;
}

gs_status gs_server_poll(gs_server* s, uint64_t request_id, int wait, double* latency_ms) {
  if (!s) return GS_ERR_INVALID;
  std::unique_lock<std::mutex> lock(s->mu);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return GS_ERR_INVALID;
  Request* r = it->second;
  if (wait) s->done_cv.wait(lock, [&] { return r->state == State::DONE; });
  if (r->state != State::DONE) return GS_ERR_BUSY;
  const gs_status st = r->status;
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  s->reqs.erase(it);
  delete r;
  return st;
}

gs_status gs_server_cancel(gs_server* s, uint64_t request_id) {
  if (!s) return GS_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  auto it = s->reqs.find(request_id);
  if (it == s->reqs.end()) return GS_ERR_INVALID;
  Request* r = it->second;
  if (r->state != State::QUEUED) return GS_ERR_BUSY;
  s->queue.erase(std::find(s->queue.begin(), s->queue.end(), r));
  r->state = State::DONE;
  r->status = GS_ERR_CANCELLED;
  r->t_done = Clock::now();
  notify_locked(s);
  s->done_cv.notify_all();
  return GS_OK;
}

gs_status gs_server_get_stats(gs_server* s, gs_server_stats* out, int reset) {
  if (!s || !out) return GS_ERR_INVALID;
  std::lock_guard<std::mutex> lock(s->mu);
  std::vector<double> v = s->latencies_ms;
  std::sort(v.begin(), v.end());
  auto pct = [&](double q) {  // nearest rank
    if (v.empty()) return 0.0;
    size_t k = size_t(q * double(v.size()) + 0.999999);
    k = std::min(std::max<size_t>(k, 1), v.size());
    return v[k - 1];
  };
  gs_server_stats st{};
  st.completed = s->completed;
  st.keys_done = s->keys_done;
  st.queued = s->queue.size();
  for (const Slot& sl : s->slots) st.running += sl.batch.size();
  st.arena_used = s->arena.used;
  st.arena_peak = s->arena.peak;
  st.p50_ms = pct(0.50);
  st.p99_ms = pct(0.99);
  double sum = 0;
  for (double x : v) sum += x;
  st.mean_ms = v.empty() ? 0.0 : sum / double(v.size());
  st.max_ms = v.empty() ? 0.0 : v.back();
  *out = st;
  if (reset) {
    s->latencies_ms.clear();
    s->completed = 0;
    s->keys_done = 0;
    s->arena.peak = s->arena.used;
  }
  return GS_OK;
}

}  // extern "C"
