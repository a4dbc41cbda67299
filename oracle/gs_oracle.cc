// gs_oracle.cc - CPU ORACLE for the GB300 sort engine. TEST INFRASTRUCTURE.
//
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
// reference arm may load this library, and only as the checker or the
// timed CPU baseline - never as the product path.
//
// It restates, in plain C++, what the reference's sort path computes:
//
//  * oracle_sort_keys: the concatenated output of HykSort / SampleSort /
//    HyperQuickSort on keys is the globally sorted multiset under
//    std::less<T> or std::greater<T> (include/helpers/hyksort_helper.h:
//    94-145 local sort + SortAmongProcesses 453-536; include/omp/
//    omp_utils.h:147-207 MergeSort; include/common.h:156-164 ConvertComp).
//    A sorted multiset is unique, so std::sort, or the parallel merge sort
//    of the reference's OpenMP local sort (p parts, std::sort each, tree of
//    2-way merges), reproduces it bit for bit (given no NaN; -0.0 and +0.0
//    compare equal, so keys-only inputs avoid -0.0, and pair inputs holding
//    both zeros have distinct values). Large inputs use that parallel form
//    on every host core, so full-size outputs are checked in seconds.
//
//  * oracle_sort_pairs: the CPU key/value path sorts std::pair<K,V> with
//    ConvertComp<pair>(comp), i.e. lexicographic (key, value) order, both
//    ascending for std::less and both descending for std::greater
//    (include/helpers/hyksort_helper.h:266-280). With `stable` the order is
//    std::stable_sort by key (ascending) or its exact reverse (descending):
//    that is the (key, global index) order of the multi-value path
//    (include/hyksort_common_vector.inl:137-162,552-565).
//
//  * oracle_hyksort_cpu: the reference's CPU HykSort algorithm restated on
//    p thread-ranks sharing memory: per-rank OpenMP-style merge sort
//    (omp_utils.h:147-207, parallel 2-way Merge 54-145), iterative k-way
//    splitter selection (hyksort_helper.h:335-450), bucket boundaries by
//    lower_bound and the k-way exchange (546-633), binary merge tree of the
//    received runs (307-332), group split into p/k (515), repeated while
//    more than one rank is left. Used as the timed CPU baseline ("port")
//    and, concatenated, it must equal oracle_sort_keys.
#include <algorithm>
#include <atomic>
#include <barrier>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <numeric>
#include <random>
#include <thread>
#include <utility>
#include <vector>

namespace {

enum Dtype { U32 = 0, I32 = 1, F32 = 2, U64 = 3, I64 = 4, F64 = 5 };

template <typename T, typename Cmp>
void par_sort(T* v, int64_t n, int threads, Cmp cmp, bool stable);

// Keys: the sorted multiset under std::less / std::greater, by the parallel
// merge sort below (`threads` workers; one worker is plain std::sort).
template <typename T>
void sort_keys_t(const void* in, void* out, uint64_t n, bool desc, int threads) {
  const T* a = static_cast<const T*>(in);
  T* b = static_cast<T*>(out);
  if (a != b) std::memcpy(b, a, n * sizeof(T));
  if (desc) par_sort(b, int64_t(n), threads, std::greater<T>(), false);
  else par_sort(b, int64_t(n), threads, std::less<T>(), false);
}

template <typename K, typename V>
void sort_pairs_t(const void* kin, const void* vin, void* kout, void* vout, uint64_t n,
                  bool desc, bool stable, int threads) {
  const K* k = static_cast<const K*>(kin);
  const V* v = static_cast<const V*>(vin);
  std::vector<std::pair<K, V>> items(n);
  for (uint64_t i = 0; i < n; ++i) items[i] = std::make_pair(k[i], v[i]);
  std::pair<K, V>* it = items.data();
  if (stable) {
    par_sort(it, int64_t(n), threads,
             [](const std::pair<K, V>& a, const std::pair<K, V>& b) { return a.first < b.first; },
             true);
    if (desc) std::reverse(items.begin(), items.end());
  } else if (desc) {
    par_sort(it, int64_t(n), threads, std::greater<std::pair<K, V>>(), false);
  } else {
    par_sort(it, int64_t(n), threads, std::less<std::pair<K, V>>(), false);
  }
  K* ko = static_cast<K*>(kout);
  V* vo = static_cast<V*>(vout);
  for (uint64_t i = 0; i < n; ++i) {
    ko[i] = items[i].first;
    vo[i] = items[i].second;
  }
}

template <typename K>
bool dispatch_v(int vt, const void* kin, const void* vin, void* kout, void* vout, uint64_t n,
                bool desc, bool stable, int th) {
  switch (vt) {
    case U32: sort_pairs_t<K, uint32_t>(kin, vin, kout, vout, n, desc, stable, th); return true;
    case I32: sort_pairs_t<K, int32_t>(kin, vin, kout, vout, n, desc, stable, th); return true;
    case F32: sort_pairs_t<K, float>(kin, vin, kout, vout, n, desc, stable, th); return true;
    case U64: sort_pairs_t<K, uint64_t>(kin, vin, kout, vout, n, desc, stable, th); return true;
    case I64: sort_pairs_t<K, int64_t>(kin, vin, kout, vout, n, desc, stable, th); return true;
    case F64: sort_pairs_t<K, double>(kin, vin, kout, vout, n, desc, stable, th); return true;
  }
  return false;
}

// ---------------------------------------------------------------------------
// HykSort on thread-ranks (CPU baseline port).
// ---------------------------------------------------------------------------

// Parallel 2-way merge: split both inputs at sampled ranks so `threads`
// workers merge equal shares (include/omp/omp_utils.h:54-145 samples 10 per
// worker per input and binary-searches the cross ranks; here the exact
// merge-path split is used, which gives the same merged output).
template <typename T, typename Cmp>
void par_merge(const T* a, int64_t na, const T* b, int64_t nb, T* out, int threads, Cmp cmp) {
  if (threads <= 1 || na + nb < 65536) {
    std::merge(a, a + na, b, b + nb, out, cmp);
    return;
  }
  std::vector<int64_t> sa(threads + 1), sb(threads + 1);
  sa[0] = sb[0] = 0;
  sa[threads] = na;
  sb[threads] = nb;
  for (int t = 1; t < threads; ++t) {
    int64_t diag = (na + nb) * t / threads;
    int64_t lo = std::max<int64_t>(0, diag - nb), hi = std::min<int64_t>(diag, na);
    while (lo < hi) {  // first i with !(b[diag-i-1] < a[i]) ... merge path
      int64_t i = (lo + hi) / 2;
      if (cmp(b[diag - i - 1], a[i])) hi = i; else lo = i + 1;
    }
    sa[t] = lo;
    sb[t] = diag - lo;
  }
  std::vector<std::thread> ws;
  for (int t = 0; t < threads; ++t) {
    ws.emplace_back([&, t] {
      std::merge(a + sa[t], a + sa[t + 1], b + sb[t], b + sb[t + 1], out + sa[t] + sb[t], cmp);
    });
  }
  for (auto& w : ws) w.join();
}

// Parallel merge sort (include/omp/omp_utils.h:147-207 MergeSort): split in
// `threads` parts, sort each (std::sort, or std::stable_sort when `stable`),
// then merge pairs of runs level by level with the parallel 2-way merge.
// std::merge and the merge-path split take ties from the left run first, so
// the stable variant stays stable.
template <typename T, typename Cmp>
void par_sort(T* v, int64_t n, int threads, Cmp cmp, bool stable) {
  if (threads <= 1 || n < 65536 || n < 2 * threads) {
    if (stable) std::stable_sort(v, v + n, cmp);
    else std::sort(v, v + n, cmp);
    return;
  }
  std::vector<int64_t> split(threads + 1);
  for (int i = 0; i <= threads; ++i) split[i] = n * i / threads;
  {
    std::vector<std::thread> ws;
    for (int i = 0; i < threads; ++i)
      ws.emplace_back([&, i] {
        if (stable) std::stable_sort(v + split[i], v + split[i + 1], cmp);
        else std::sort(v + split[i], v + split[i + 1], cmp);
      });
    for (auto& w : ws) w.join();
  }
  std::vector<T> buf(n);
  T* a = v;
  T* b = buf.data();
  for (int j = 1; j < threads; j *= 2) {
    for (int i = 0; i < threads; i += 2 * j) {
      if (i + j < threads) {
        const int e = std::min(i + 2 * j, threads);
        par_merge(a + split[i], split[i + j] - split[i], a + split[i + j],
                  split[e] - split[i + j], b + split[i], threads, cmp);
      } else {
        std::copy(a + split[i], a + split[threads], b + split[i]);
      }
    }
    std::swap(a, b);
  }
  if (a != v) std::copy(a, a + n, v);
}

// Local merge sort of one rank of the HykSort port.
template <typename T, typename Cmp>
void local_merge_sort(std::vector<T>& v, int threads, Cmp cmp) {
  par_sort(v.data(), int64_t(v.size()), threads, cmp, false);
}

template <typename T, typename Cmp>
struct HykShared {
  int p = 0;
  int k = 0;
  int threads = 1;
  Cmp cmp;
  std::vector<std::vector<T>>* data = nullptr;
  // One barrier per rank group: groups of a round are the blocks the
  // previous round split the ranks into (indexed by group size, first rank).
  std::vector<std::pair<std::pair<int, int>, std::barrier<>*>> bars;
  std::barrier<>* bar(int np, int g0) {
    for (auto& b : bars)
      if (b.first.first == np && b.first.second == g0) return b.second;
    return nullptr;
  }
  // per-rank scratch published between barriers
  std::vector<std::vector<T>> samples;
  std::vector<std::vector<int64_t>> loc_ranks;
  std::vector<std::vector<T>> splitters;
  std::vector<std::vector<int64_t>> send_disp;   // per rank, k+1 cut points
};

// One rank's part of SortAmongProcesses. Ranks of a group [g0, g0+np) with
// np > 1 choose k-1 splitters together, then rank r receives bucket
// (r - g0) / (np/k) from the np/k... partners of its new block.
template <typename T, typename Cmp>
void hyk_rank(HykShared<T, Cmp>& S, int rank, uint64_t seed) {
  auto& my = (*S.data)[rank];
  local_merge_sort(my, S.threads, S.cmp);
  std::mt19937_64 rng(seed + uint64_t(rank));
  int g0 = 0, np = S.p;
  while (np > 1) {
    std::barrier<>* B = S.bar(np, g0);
    const int kw = std::min(S.k, np);
    const int blk = np / kw;
    const int me = rank - g0;
    // --- iterative splitter selection (hyksort_helper.h:335-450)
    const int64_t nloc = int64_t(my.size());
    int64_t tot = 0;
    B->arrive_and_wait();
    for (int r = g0; r < g0 + np; ++r) tot += int64_t((*S.data)[r].size());
    const int ks = kw - 1;
    const double tol = 1e-2 / ks;
    const int beta = int(std::pow(1.0 / tol, 1.0 / 3.0) * 3.0);
    std::vector<int64_t> start(ks, 0), end(ks, nloc), exp_rank(ks);
    for (int i = 0; i < ks; ++i) exp_rank[i] = (int64_t(i + 1) * tot) / kw;
    std::vector<T> split(ks);
    int64_t max_err = tot;
    const int64_t cond = int64_t(double(tot) * tol);
    while (max_err > cond) {
      // interval sizes summed over the group
      std::vector<int64_t> loc_size(ks), tot_size(ks, 0);
      for (int i = 0; i < ks; ++i) loc_size[i] = end[i] - start[i];
      S.loc_ranks[rank] = loc_size;
      B->arrive_and_wait();
      for (int r = g0; r < g0 + np; ++r)
        for (int i = 0; i < ks; ++i) tot_size[i] += S.loc_ranks[r][i];
      B->arrive_and_wait();
      std::vector<T> ls;
      for (int i = 0; i < ks; ++i) {
        int cnt = tot_size[i] == 0 ? 1 : int(int64_t(beta) * (end[i] - start[i]) / tot_size[i]);
        if (np > beta) {
          double r = std::uniform_real_distribution<double>(0, double(tot_size[i]))(rng);
          cnt = (r < double(beta) * double(loc_size[i])) ? 1 : 0;
        }
        for (int j = 0; j < cnt && loc_size[i] > 0; ++j) {
          int64_t r = std::uniform_int_distribution<int64_t>(0, loc_size[i] - 1)(rng);
          ls.push_back(my[start[i] + r]);
        }
      }
      S.samples[rank] = ls;
      B->arrive_and_wait();
      std::vector<T> gs;
      for (int r = g0; r < g0 + np; ++r)
        gs.insert(gs.end(), S.samples[r].begin(), S.samples[r].end());
      std::sort(gs.begin(), gs.end(), S.cmp);
      const int gc = int(gs.size());
      std::vector<int64_t> lr(gc, 0);
      for (int i = 0; i < gc; ++i)
        lr[i] = std::lower_bound(my.begin(), my.end(), gs[i], S.cmp) - my.begin();
      B->arrive_and_wait();
      S.loc_ranks[rank] = lr;
      B->arrive_and_wait();
      std::vector<int64_t> gr(gc, 0);
      for (int r = g0; r < g0 + np; ++r)
        for (int i = 0; i < gc; ++i) gr[i] += S.loc_ranks[r][i];
      B->arrive_and_wait();
      int64_t new_err = 0;
      for (int i = 0; i < ks; ++i) {
        if (gc == 0) break;
        int ub = int(std::upper_bound(gr.begin(), gr.end(), exp_rank[i]) - gr.begin());
        int lb = std::max(ub - 1, 0);
        int64_t err = std::llabs(gr[lb] - exp_rank[i]);
        if (err < max_err) {
          start[i] = (gr[lb] > exp_rank[i]) ? 0 : lr[lb];
          end[i] = (ub == gc) ? nloc : lr[ub];
          split[i] = gs[lb];
          new_err = std::max(new_err, err);
        }
      }
      max_err = new_err;
      if (gc == 0) max_err = 0;
    }
    // --- bucket cut points by lower_bound (hyksort_helper.h:563-568)
    std::vector<int64_t> disp(kw + 1);
    disp[0] = 0;
    disp[kw] = nloc;
    for (int i = 0; i < ks; ++i)
      disp[i + 1] = std::lower_bound(my.begin(), my.end(), split[i], S.cmp) - my.begin();
    for (int i = 1; i <= kw; ++i) disp[i] = std::max(disp[i], disp[i - 1]);
    S.send_disp[rank] = disp;
    B->arrive_and_wait();
    // --- exchange: block b = me / blk receives bucket b from the partners
    //     with the same position in each block (hyksort_helper.h:577-609)
    const int b = me / blk;
    const int pid = me % blk;
    std::vector<std::vector<T>> runs;
    for (int i = 0; i < kw; ++i) {
      const int partner = g0 + blk * i + pid;
      const auto& pd = S.send_disp[partner];
      const auto& src = (*S.data)[partner];
      runs.emplace_back(src.begin() + pd[b], src.begin() + pd[b + 1]);
    }
    B->arrive_and_wait();
    // --- binary merge tree of the k runs (hyksort_helper.h:307-332)
    while (runs.size() > 1) {
      std::vector<std::vector<T>> next;
      for (size_t i = 0; i + 1 < runs.size(); i += 2) {
        std::vector<T> m(runs[i].size() + runs[i + 1].size());
        par_merge(runs[i].data(), int64_t(runs[i].size()), runs[i + 1].data(),
                  int64_t(runs[i + 1].size()), m.data(), S.threads, S.cmp);
        next.push_back(std::move(m));
      }
      if (runs.size() & 1) next.push_back(std::move(runs.back()));
      runs.swap(next);
    }
    my = std::move(runs[0]);
    B->arrive_and_wait();
    // --- communicator split (hyksort_helper.h:515): new group = block b
    g0 = g0 + b * blk;
    np = blk;
  }
}

template <typename T, typename Cmp>
void hyksort_t(void* data, uint64_t n, int p, int k, int threads, uint64_t seed, Cmp cmp) {
  T* a = static_cast<T*>(data);
  std::vector<std::vector<T>> ranks(p);
  for (int r = 0; r < p; ++r) {
    const uint64_t b = n * uint64_t(r) / uint64_t(p), e = n * uint64_t(r + 1) / uint64_t(p);
    ranks[r].assign(a + b, a + e);
  }
  HykShared<T, Cmp> S;
  std::vector<std::unique_ptr<std::barrier<>>> owned;
  for (int np = p; np > 1;) {
    for (int g0 = 0; g0 < p; g0 += np) {
      owned.emplace_back(new std::barrier<>(np));
      S.bars.push_back({{np, g0}, owned.back().get()});
    }
    np = np / std::min(k, np);
  }
  S.p = p;
  S.k = k;
  S.threads = threads;
  S.cmp = cmp;
  S.data = &ranks;
  S.samples.resize(p);
  S.loc_ranks.resize(p);
  S.splitters.resize(p);
  S.send_disp.resize(p);
  std::vector<std::thread> ws;
  for (int r = 0; r < p; ++r) ws.emplace_back([&, r] { hyk_rank<T, Cmp>(S, r, seed); });
  for (auto& w : ws) w.join();
  uint64_t off = 0;
  for (int r = 0; r < p; ++r) {
    std::copy(ranks[r].begin(), ranks[r].end(), a + off);
    off += ranks[r].size();
  }
}

template <typename T>
void hyksort_dir(void* data, uint64_t n, int p, int k, int threads, uint64_t seed, bool desc) {
  if (desc) hyksort_t<T>(data, n, p, k, threads, seed, std::greater<T>());
  else hyksort_t<T>(data, n, p, k, threads, seed, std::less<T>());
}

bool is_pow2(unsigned v) { return v && !(v & (v - 1)); }

}  // namespace

extern "C" {

// `threads` workers (<= 1: one).
int oracle_sort_keys(int dtype, const void* in, void* out, uint64_t n, int desc, int threads) {
  switch (dtype) {
    case U32: sort_keys_t<uint32_t>(in, out, n, desc, threads); return 0;
    case I32: sort_keys_t<int32_t>(in, out, n, desc, threads); return 0;
    case F32: sort_keys_t<float>(in, out, n, desc, threads); return 0;
    case U64: sort_keys_t<uint64_t>(in, out, n, desc, threads); return 0;
    case I64: sort_keys_t<int64_t>(in, out, n, desc, threads); return 0;
    case F64: sort_keys_t<double>(in, out, n, desc, threads); return 0;
  }
  return -1;
}

int oracle_sort_pairs(int kt, int vt, const void* kin, const void* vin, void* kout, void* vout,
                      uint64_t n, int desc, int stable, int threads) {
  bool ok = false;
  switch (kt) {
    case U32: ok = dispatch_v<uint32_t>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
    case I32: ok = dispatch_v<int32_t>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
    case F32: ok = dispatch_v<float>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
    case U64: ok = dispatch_v<uint64_t>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
    case I64: ok = dispatch_v<int64_t>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
    case F64: ok = dispatch_v<double>(vt, kin, vin, kout, vout, n, desc, stable, threads); break;
  }
  return ok ? 0 : -1;
}

// Batched sort: each segment [off[s], off[s+1]) sorted on its own, as each
// rank's local sort is (include/omp/omp_utils.h:147-207); `threads` workers
// take segments in turn.
int oracle_segmented_sort_keys(int dtype, const void* in, void* out, uint64_t n,
                               const uint64_t* off, uint32_t nseg, int desc, int threads) {
  if (dtype < U32 || dtype > F64) return -1;
  const size_t eb = (dtype <= F32) ? 4 : 8;
  if (in != out) std::memcpy(out, in, n * eb);
  uint8_t* base = static_cast<uint8_t*>(out);
  std::atomic<uint32_t> next{0};
  auto work = [&] {
    for (uint32_t s = next++; s < nseg; s = next++) {
      const uint64_t b = off[s], e = off[s + 1];
      if (e > b) oracle_sort_keys(dtype, base + b * eb, base + b * eb, e - b, desc, 1);
    }
  };
  const int t = threads < 1 ? 1 : threads;
  std::vector<std::thread> ws;
  for (int i = 1; i < t; ++i) ws.emplace_back(work);
  work();
  for (auto& w : ws) w.join();
  return 0;
}

// In-place HykSort of `n` keys over `p` thread-ranks (each rank gets the
// contiguous slice [n*r/p, n*(r+1)/p)), k-way, `threads` workers per rank.
// p or k not a power of two: the reference switches to SampleSort
// (include/hyksort_common_vector.inl:31-43), whose concatenated output is the
// same sorted array; here that case returns -2 and the caller uses
// oracle_sort_keys.
int oracle_hyksort_cpu(int dtype, void* data, uint64_t n, int p, int k, int threads,
                       uint64_t seed, int desc) {
  if (p < 1 || k < 2 || !is_pow2(unsigned(p)) || !is_pow2(unsigned(k))) return -2;
  if (n == 0) return -3;
  switch (dtype) {
    case U32: hyksort_dir<uint32_t>(data, n, p, k, threads, seed, desc); return 0;
    case I32: hyksort_dir<int32_t>(data, n, p, k, threads, seed, desc); return 0;
    case F32: hyksort_dir<float>(data, n, p, k, threads, seed, desc); return 0;
    case U64: hyksort_dir<uint64_t>(data, n, p, k, threads, seed, desc); return 0;
    case I64: hyksort_dir<int64_t>(data, n, p, k, threads, seed, desc); return 0;
    case F64: hyksort_dir<double>(data, n, p, k, threads, seed, desc); return 0;
  }
  return -1;
}

}  // extern "C"
