// Shared device helpers of the GB300 sort engine: order-preserving key
// transforms, status words of the decoupled look-back, small block scans.
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

namespace gs {

constexpr int RADIX_BITS = 8;
constexpr int RADIX = 1 << RADIX_BITS;
constexpr int MAX_DIGITS = 16;          // 64-bit key + 64-bit value, 8-bit digits
constexpr uint32_t PASS_SKIPPED = 0xFFFFFFFFu;

// Key classes: how raw bits map to an unsigned order.
enum KeyKind : uint32_t { KIND_UNSIGNED = 0, KIND_SIGNED = 1, KIND_FLOAT = 2 };

// Device error word bits.
enum ErrBits : uint32_t {
  ERR_LOOKBACK_TIMEOUT = 1u,
  ERR_SCATTER_RANGE = 2u,
  ERR_PASS_KIND = 4u,  // an unstable-only pass kernel launched for a stable pass
  ERR_SMEM_ALIGN = 8u
};

struct NoValue {};

template <typename U> struct Bits;
template <> struct Bits<uint32_t> {
  static constexpr uint32_t SIGN = 0x80000000u;
  static constexpr int DIGITS = 4;
};
template <> struct Bits<uint64_t> {
  static constexpr uint64_t SIGN = 0x8000000000000000ull;
  static constexpr int DIGITS = 8;
};

// Map raw key bits to an unsigned integer whose natural order is the
// requested order: std::less for unsigned/signed/IEEE keys, std::greater
// when `desc` (include/common.h:156-164 maps the comparator to this flag).
// IEEE: negative values have every bit flipped, non-negative ones only the
// sign bit, so -inf < ... < -0 < +0 < ... < +inf.
template <typename U>
__device__ __forceinline__ U order_bits(U x, uint32_t kind, bool desc) {
  const U sign = Bits<U>::SIGN;
  U mask;
  if (kind == KIND_FLOAT) {
    mask = (x & sign) ? ~U(0) : sign;
  } else if (kind == KIND_SIGNED) {
    mask = sign;
  } else {
    mask = U(0);
  }
  U y = x ^ mask;
  return desc ? U(~y) : y;
}

// Status words of the decoupled look-back, one per (tile, digit):
//   [63:62] flag (0 not ready, 1 tile aggregate, 2 inclusive prefix)
//   [61:32] launch generation (a word from an older launch reads as not ready)
//   [31:0]  count
constexpr uint64_t FLAG_AGG = 1ull << 62;
constexpr uint64_t FLAG_INC = 2ull << 62;
constexpr uint64_t FLAG_MASK = 3ull << 62;
constexpr uint32_t GEN_MASK = 0x3FFFFFFFu;

__device__ __forceinline__ uint64_t make_status(uint64_t flag, uint32_t gen,
                                                uint32_t count) {
  return flag | (uint64_t(gen & GEN_MASK) << 32) | uint64_t(count);
}

__device__ __forceinline__ uint64_t ld_relaxed(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_relaxed(uint64_t* p, uint64_t v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}

// Streaming loads (evict-first): each pass reads its source exactly once.
__device__ __forceinline__ uint32_t ld_stream(const uint32_t* p) {
  uint32_t v;
  asm("ld.global.cs.u32 %0, [%1];" : "=r"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ uint64_t ld_stream(const uint64_t* p) {
  uint64_t v;
  asm("ld.global.cs.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}
// Four consecutive 32-bit words; p is 16-byte aligned.
__device__ __forceinline__ uint4 ld_stream_v4(const uint32_t* p) {
  uint4 v;
  asm("ld.global.cs.v4.u32 {%0, %1, %2, %3}, [%4];"
      : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  return v;
}

// Bulk prefetch of [p, p + bytes) into L2 (one instruction, one thread):
// p 16-byte aligned, bytes a non-zero multiple of 16, the range inside the
// allocation.
__device__ __forceinline__ void prefetch_l2_bulk(const void* p, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" :: "l"(p), "r"(bytes) : "memory");
}

// Shared-memory address of a generic pointer (alignment checks).
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint32_t lanemask_lt() {
  uint32_t m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Exclusive scan of one value per thread over the first 256 threads of the
// block (all threads of the block must call it; threads >= 256 pass 0).
// `s_tmp` holds at least 8 words. Returns the exclusive prefix; with `s_out`
// the first 256 threads also store it there, visible to the whole block on
// return.
__device__ __forceinline__ uint32_t block_excl_scan_256(uint32_t v, uint32_t* s_tmp,
                                                        uint32_t* s_out = nullptr) {
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  const int warp = tid >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (tid < 256 && lane == 31) s_tmp[warp] = x;
  __syncthreads();
  uint32_t wsum = 0;
  if (tid < 256) {
    for (int w = 0; w < warp; ++w) wsum += s_tmp[w];
  }
  const uint32_t ex = wsum + x - v;
  if (s_out != nullptr && tid < 256) s_out[tid] = ex;
  __syncthreads();
  return ex;
}

}  // namespace gs
