// Launchers of the onesweep radix pipeline (kernels in radix.cuh).
#include "engine.h"
#include "radix.cuh"

namespace gs {

namespace {

constexpr int UPSWEEP_THREADS = 512;
constexpr int UPSWEEP_UNROLL = 8;

// Tile shapes of the pass kernel (threads per block, items per thread,
// blocks per SM), selectable per call; shape 0 is the default. Larger
// elements take fewer items per thread.
template <int T, int I, int B, int C = 8> struct Shape {
  static constexpr int THREADS = T, ITEMS = I, MINB = B, CLUSTER = C;
};
template <typename K, typename V, int S> struct PassShape;
// Shape 2 of keys-only sorts uses thread-block clusters (one look-back per
// 8 tiles); it measured slower than per-tile look-back on GB300 and is kept
// selectable for tuning. Key/value sorts never use clusters: a clustered
// 256-thread pair variant raised an illegal-instruction fault on GB300
// whose cause is not yet understood.
template <> struct PassShape<uint32_t, NoValue, 0> : Shape<512, 16, 2, 1> {};
template <> struct PassShape<uint32_t, NoValue, 1> : Shape<256, 24, 4, 1> {};
template <> struct PassShape<uint32_t, NoValue, 2> : Shape<512, 16, 2, 8> {};
template <> struct PassShape<uint64_t, NoValue, 0> : Shape<512, 12, 2, 1> {};
template <> struct PassShape<uint64_t, NoValue, 1> : Shape<256, 16, 4, 1> {};
template <> struct PassShape<uint64_t, NoValue, 2> : Shape<512, 12, 2, 8> {};
template <> struct PassShape<uint32_t, uint32_t, 0> : Shape<512, 12, 2, 1> {};
template <> struct PassShape<uint32_t, uint32_t, 1> : Shape<256, 12, 4, 1> {};
template <> struct PassShape<uint32_t, uint32_t, 2> : Shape<256, 16, 4, 1> {};
template <typename K, typename V, int S>
struct PassShape : Shape<(S == 0 ? 512 : 256), 8, (S == 0 ? 2 : 4), 1> {};
constexpr int NUM_SHAPES = 3;
constexpr uint32_t MIN_TILE = 256 * 8;  // smallest tile of any shape

template <typename K, typename V, int S>
cudaError_t run(const RadixJob& job, const DeviceProps& props, uint32_t* gen,
                cudaStream_t stream) {
  constexpr int PASS_THREADS = PassShape<K, V, S>::THREADS;
  constexpr int ITEMS = PassShape<K, V, S>::ITEMS;
  constexpr int MINB = PassShape<K, V, S>::MINB;
  constexpr int CLUSTER = PassShape<K, V, S>::CLUSTER;
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

  auto kern = pass_kernel<K, V, PASS_THREADS, ITEMS, MINB, CLUSTER>;
  static bool attr_set = false;
  if (!attr_set) {
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             int(Cfg::DYN_SMEM));
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const uint64_t tiles = (job.n + Cfg::TILE - 1) / Cfg::TILE;
  const uint64_t units = (tiles + CLUSTER - 1) / CLUSTER;  // look-back units (cluster-tiles)
  cudaLaunchConfig_t lc = {};
  cudaLaunchAttribute attr[1];
  lc.gridDim = dim3(unsigned(units * CLUSTER));
  lc.blockDim = dim3(PASS_THREADS);
  lc.dynamicSmemBytes = Cfg::DYN_SMEM;
  lc.stream = stream;
  if (CLUSTER > 1) {
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = CLUSTER;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
  }
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
  for (uint32_t q = 0; q < digits; ++q) {
    pa.pass = q;
    pa.gen = ++(*gen);
    e = cudaLaunchKernelEx(&lc, kern, pa);
    if (e != cudaSuccess) return e;
    if (job.marks) cudaEventRecord(job.marks[3 + q], stream);
  }
  return cudaGetLastError();
}

}  // namespace

uint32_t radix_tile(int key_bytes, int val_bytes) {
  (void)key_bytes;
  (void)val_bytes;
  return MIN_TILE;
}

int radix_num_shapes() { return NUM_SHAPES; }

// Measured defaults on GB300 (2^30 uniform keys): 32-bit keys run fastest
// with 256-thread CTAs of 24 items, four per SM.
int radix_default_shape(int key_bytes, int val_bytes) {
  return (val_bytes == 0) ? 1 : 0;
}

size_t radix_status_words(uint64_t n, int key_bytes, int val_bytes) {
  const uint64_t t = radix_tile(key_bytes, val_bytes);
  return size_t((n + t - 1) / t) * RADIX;
}

size_t radix_status_words_u32_shape0(uint64_t n) {
  constexpr uint64_t t = uint64_t(PassShape<uint32_t, NoValue, 0>::THREADS) *
                         PassShape<uint32_t, NoValue, 0>::ITEMS;
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
