// Parameter blocks and device work areas of the radix pipeline (shared by
// the kernels in radix.cuh and the host code that sizes their scratch).
#pragma once

#include "common.cuh"

namespace gs {

struct SortPlan {
  uint32_t gen_base;                      // look-back tag of this sort (pass q: +q+1)
  uint32_t m_exec;                        // passes that run
  uint32_t exec_index[MAX_DIGITS];        // 0..m_exec-1, or PASS_SKIPPED
  uint32_t tile_counter[MAX_DIGITS];      // tile claim counters per pass
  uint32_t binbase[MAX_DIGITS][RADIX];    // global start of each bin
  // Set when the value digits were dropped because the values already run
  // in order (ties by value = input order): the first pass that runs must
  // then rank stably, and read back to front for a descending sort.
  uint32_t first_stable;
  uint32_t first_reverse;
};

// Scratch words of one sort: histograms and the value-order flag (zeroed
// before the upsweep), plan.
struct SortWork {
  uint32_t hist[MAX_DIGITS][RADIX];
  uint32_t val_order_break;  // a value orders before its predecessor in the input
  SortPlan plan;
  uint32_t gen_counter;  // per status buffer: the next free look-back tag
};

struct UpsweepParams {
  const void* keys;
  const void* vals;       // read only when val_digits > 0
  uint64_t n;
  uint32_t key_kind, val_kind;
  uint32_t desc;
  uint32_t val_digits;    // 0, or the value's digit count (ties by value)
  SortWork* work;
  void* copy_keys;        // when set: every key read is also stored here
  void* copy_vals;        // (and every value, when val_digits > 0)
  uint32_t check_val_order;  // set work->val_order_break if the values are
                             // not non-decreasing (std::less) in input order
};

struct PlanParams {
  SortWork* work;
  uint32_t* gen_counter;  // shared by every sort that uses the same status words
  uint64_t n;
  uint32_t digits;        // val_digits + key_digits
  uint32_t in_place;      // an output aliases its input
  uint32_t reverse_first; // first pass reads the input back to front
  uint32_t digit_lo, digit_hi;  // digits that may run: [digit_lo, digit_hi)
  uint32_t alt_is_in;     // scratch aliases the input: the pass count must be odd
  // Value digits 0 .. drop_val_digits-1 may be dropped when the upsweep
  // found the values in order; the sort then keeps ties in input order
  // (reversed when drop_reverse: descending).
  uint32_t drop_val_digits;
  uint32_t drop_reverse;
};

// One tile of a segmented pass: its first element, element count and
// segment (built with the plan, so a tile finds its place with one load).
struct SegTile {
  uint64_t base;
  uint32_t n;
  uint32_t seg;
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
  uint32_t spin_limit;
  uint32_t inject_stall;  // test hook: tile 1 waits on a flag nobody sets
  SortWork* work;
  uint32_t* err;
  // Batched (segmented) sorts: when seg_tile_start is set, tiles of
  // segment s are [seg_tile_start[s], seg_tile_start[s+1]), its elements
  // [seg_range[2s], seg_range[2s+1]), and its bin bases are
  // seg_binbase[(s * seg_digits + pass) * RADIX + digit]. Each segment's
  // first tile starts its own look-back chain.
  const uint32_t* seg_tile_start;
  const uint64_t* seg_range;
  const SegTile* seg_tiles;  // per tile
  const uint32_t* seg_binbase;
  uint32_t nseg;
  uint32_t seg_digits;
  // Bucket mode (sample sort): the "digit" of a key is the number of
  // splitters not greater than its order bits (upper_bound), i.e. its bucket
  // among nsplit + 1 <= RADIX buckets; splitters are sorted order bits.
  const void* splitters;
  uint32_t nsplit;
  // Unsegmented forward passes: tile t's CTA prefetches tile t +
  // prefetch_tiles of its source into L2 (0: none).
  uint32_t prefetch_tiles;
};

}  // namespace gs
