// Launchers of the onesweep radix pipeline (kernels in radix.cuh).
#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int UPSWEEP_THREADS = 512;
constexpr int UPSWEEP_UNROLL = 8;
constexpr int PASS_THREADS = 512;

// Items per thread of the pass kernel, by bytes per element (key + value).
template <typename K, typename V> struct PassItems;
template <> struct PassItems<uint32_t, NoValue> { static constexpr int v = 16; };
template <> struct PassItems<uint64_t, NoValue> { static constexpr int v = 12; };
template <> struct PassItems<uint32_t, uint32_t> { static constexpr int v = 12; };
template <> struct PassItems<uint32_t, uint64_t> { static constexpr int v = 8; };
template <> struct PassItems<uint64_t, uint32_t> { static constexpr int v = 8; };
template <> struct PassItems<uint64_t, uint64_t> { static constexpr int v = 8; };

template <typename K, typename V>
cudaError_t run(const RadixJob& job, const DeviceProps& props, uint32_t* gen,
                cudaStream_t stream) {
  constexpr int ITEMS = PassItems<K, V>::v;
  constexpr int MINB = 2;
  using Cfg = PassConfig<K, V, PASS_THREADS, ITEMS>;
  constexpr bool HAS_V = Cfg::HAS_V;
  const uint32_t kd = Bits<K>::DIGITS;
  uint32_t vd = 0;
  if constexpr (HAS_V) vd = job.ties_by_value ? Bits<V>::DIGITS : 0;
  const uint32_t digits = kd + vd;

  if (job.marks) cudaEventRecord(job.marks[0], stream);
  cudaError_t e = cudaMemsetAsync(job.work, 0, sizeof(uint32_t) * MAX_DIGITS * RADIX, stream);
  if (e != cudaSuccess) return e;

  UpsweepParams up{};
  up.keys = job.keys_in;
  up.vals = job.vals_in;
  up.n = job.n;
  up.key_kind = job.key_kind;
  up.val_kind = job.val_kind;
  up.desc = job.desc;
  up.val_digits = vd;
  up.work = job.work;
  const uint64_t chunk = uint64_t(UPSWEEP_THREADS) * UPSWEEP_UNROLL;
  uint64_t ublocks = (job.n + chunk - 1) / chunk;
  const uint64_t umax = uint64_t(props.num_sms) * 4;
  if (ublocks > umax) ublocks = umax;
  if (ublocks == 0) ublocks = 1;
  upsweep_kernel<K, V, UPSWEEP_THREADS, UPSWEEP_UNROLL>
      <<<unsigned(ublocks), UPSWEEP_THREADS, 0, stream>>>(up);
  if (job.marks) cudaEventRecord(job.marks[1], stream);

  PlanParams pp{};
  pp.work = job.work;
  pp.n = job.n;
  pp.digits = digits;
  pp.in_place = (job.keys_in == job.keys_out) ||
                (HAS_V && job.vals_in == job.vals_out);
  pp.reverse_first = job.reverse_first;
  plan_kernel<<<1, 256, 0, stream>>>(pp);
  if (job.marks) cudaEventRecord(job.marks[2], stream);

  auto kern = pass_kernel<K, V, PASS_THREADS, ITEMS, MINB>;
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(Cfg::DYN_SMEM));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const uint64_t tiles = (job.n + Cfg::TILE - 1) / Cfg::TILE;
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
  pa.status = job.status;
  pa.spin_limit = job.spin_limit;
  pa.inject_stall = job.inject_stall;
  pa.work = job.work;
  pa.err = job.err;
  for (uint32_t q = 0; q < digits; ++q) {
    pa.pass = q;
    pa.gen = ++(*gen);
    kern<<<unsigned(tiles), PASS_THREADS, Cfg::DYN_SMEM, stream>>>(pa);
    if (job.marks) cudaEventRecord(job.marks[3 + q], stream);
  }
  return cudaGetLastError();
}

}  // namespace

uint32_t radix_tile(int key_bytes, int val_bytes) {
  if (key_bytes == 4 && val_bytes == 0) return PASS_THREADS * PassItems<uint32_t, NoValue>::v;
  if (key_bytes == 8 && val_bytes == 0) return PASS_THREADS * PassItems<uint64_t, NoValue>::v;
  if (key_bytes == 4 && val_bytes == 4) return PASS_THREADS * PassItems<uint32_t, uint32_t>::v;
  return PASS_THREADS * 8;
}

size_t radix_status_words(uint64_t n, int key_bytes, int val_bytes) {
  const uint64_t t = radix_tile(key_bytes, val_bytes);
  return size_t((n + t - 1) / t) * RADIX;
}

size_t sort_work_bytes() { return sizeof(SortWork); }

cudaError_t launch_radix_sort(const RadixJob& job, const DeviceProps& props,
                              uint32_t* gen, cudaStream_t stream) {
  const int kb = job.key_bytes, vb = job.val_bytes;
  if (kb == 4 && vb == 0) return run<uint32_t, NoValue>(job, props, gen, stream);
  if (kb == 8 && vb == 0) return run<uint64_t, NoValue>(job, props, gen, stream);
  if (kb == 4 && vb == 4) return run<uint32_t, uint32_t>(job, props, gen, stream);
  if (kb == 4 && vb == 8) return run<uint32_t, uint64_t>(job, props, gen, stream);
  if (kb == 8 && vb == 4) return run<uint64_t, uint32_t>(job, props, gen, stream);
  if (kb == 8 && vb == 8) return run<uint64_t, uint64_t>(job, props, gen, stream);
  return cudaErrorInvalidValue;
}

}  // namespace gs
