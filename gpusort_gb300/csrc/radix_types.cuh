// Parameter blocks and device work areas of the radix pipeline (shared by
// the kernels in radix.cuh and the host code that sizes their scratch).
#pragma once

#include "common.cuh"

namespace gs {

struct SortPlan {
  uint32_t m_exec;                        // passes that run
  uint32_t exec_index[MAX_DIGITS];        // 0..m_exec-1, or PASS_SKIPPED
  uint32_t tile_counter[MAX_DIGITS];      // tile claim counters per pass
  uint32_t binbase[MAX_DIGITS][RADIX];    // global start of each bin
};

// Scratch words of one sort: histograms (zeroed before the upsweep) + plan.
struct SortWork {
  uint32_t hist[MAX_DIGITS][RADIX];
  SortPlan plan;
};

struct UpsweepParams {
  const void* keys;
  const void* vals;       // read only when val_digits > 0
  uint64_t n;
  uint32_t key_kind, val_kind;
  uint32_t desc;
  uint32_t val_digits;    // 0, or the value's digit count (ties by value)
  SortWork* work;
};

struct PlanParams {
  SortWork* work;
  uint64_t n;
  uint32_t digits;        // val_digits + key_digits
  uint32_t in_place;      // an output aliases its input
  uint32_t reverse_first; // first pass reads the input back to front
};

struct PassParams {
  const void* keys_in;
  void* keys_out;
  void* keys_alt;
  const void* vals_in;
  void* vals_out;
  void* vals_alt;
  uint64_t n;
  uint32_t pass;          // digit index q: q < val_digits -> value digit q
  uint32_t val_digits;
  uint32_t key_kind, val_kind;
  uint32_t desc;
  uint32_t reverse_first;
  uint32_t first_unstable;  // the first pass that runs may rank unstably
  uint64_t* status;       // num_tiles * RADIX look-back words
  uint32_t gen;
  uint32_t spin_limit;
  uint32_t inject_stall;  // test hook: tile 1 waits on a flag nobody sets
  SortWork* work;
  uint32_t* err;
};

}  // namespace gs
