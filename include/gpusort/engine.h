// gpusort/engine.h - the C++ layer of gpusort_gb300 (header only).
//
// It keeps monotone-RK/gpusort's C++ entry points - HykSort, SampleSort,
// HyperQuickSort with the same overload shapes (keys; keys + comparator;
// keys + values; keys + several value vectors; user-defined records with a
// key function) - and runs them on one GPU through the C ABI of
// gpusort_gb300.h. The p MPI ranks of the reference become p partitions of
// one array in HBM: `PartitionComm` takes the place of MpiComm, and the
// vector passed in is the whole array, sorted globally in place.
#ifndef GPUSORT_GB300_ENGINE_HPP_
#define GPUSORT_GB300_ENGINE_HPP_

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <functional>
#include <iostream>
#include <map>
#include <string>
#include <type_traits>
#include <vector>

#include "../gpusort_gb300.h"

namespace gpusort {

// Same names and meaning as the reference's exception types
// (include/exceptions/mpi_exception.h:9-22,
//  include/exceptions/thrust_exception.h:9-22).
class MpiException : public std::exception {
 public:
  explicit MpiException(const std::string& msg) : msg_(msg) {}
  const char* what() const noexcept override { return msg_.c_str(); }
 private:
  std::string msg_;
};

class ThrustException : public std::exception {
 public:
  explicit ThrustException(const std::string& msg) : msg_(msg) {}
  const char* what() const noexcept override { return msg_.c_str(); }
 private:
  std::string msg_;
};

// p virtual ranks on one GPU: the stand-in for MPI_Comm. `size` is p (the
// reference's MpiCommSize), `device` the CUDA device.
struct PartitionComm {
  int size;
  int device;
  explicit PartitionComm(int p = 1, int dev = 0) : size(p), device(dev) {}
};
typedef PartitionComm MpiComm;

namespace detail {

template <typename T> struct Dtype;
template <> struct Dtype<unsigned int> { static constexpr gs_dtype v = GS_U32; };
template <> struct Dtype<int> { static constexpr gs_dtype v = GS_I32; };
template <> struct Dtype<float> { static constexpr gs_dtype v = GS_F32; };
template <> struct Dtype<unsigned long> { static constexpr gs_dtype v = sizeof(unsigned long) == 8 ? GS_U64 : GS_U32; };
template <> struct Dtype<unsigned long long> { static constexpr gs_dtype v = GS_U64; };
template <> struct Dtype<long> { static constexpr gs_dtype v = sizeof(long) == 8 ? GS_I64 : GS_I32; };
template <> struct Dtype<long long> { static constexpr gs_dtype v = GS_I64; };
template <> struct Dtype<double> { static constexpr gs_dtype v = GS_F64; };

template <typename T, typename = void> struct HasDtype : std::false_type {};
template <typename T> struct HasDtype<T, decltype(void(Dtype<T>::v))> : std::true_type {};

// std::less / std::greater only (the comparators the reference's GPU path
// instantiates, src/cuda_utils.cu:249-255).
template <typename C> struct Direction;
template <typename T> struct Direction<std::less<T>> { static constexpr bool desc = false; };
template <typename T> struct Direction<std::greater<T>> { static constexpr bool desc = true; };

template <typename C, typename = void> struct IsComparator : std::false_type {};
template <typename C>
struct IsComparator<C, decltype(void(Direction<C>::desc))> : std::true_type {};
template <typename C>
using EnableIfComparator = typename std::enable_if<IsComparator<C>::value>::type;

enum Family { kHyk, kSample, kHyperQuick };

// The engine has no CPU path: a request for the reference's CPU local sort
// (is_using_gpu == false) is refused rather than served elsewhere.
inline void RequireGpu(bool is_using_gpu) {
  if (!is_using_gpu)
    throw ThrustException("gpusort_gb300 sorts on the GPU only (is_using_gpu is false)");
}

inline bool IsPowerOfTwo(unsigned v) { return v && !(v & (v - 1)); }

// One engine context per thread and device (the reference selects device
// (rank + 1) % ndev per call, src/cuda_utils.cu:395-401; here the comm
// names it).
inline gs_ctx* Context(int device) {
  thread_local std::map<int, gs_ctx*> ctxs;
  auto it = ctxs.find(device);
  if (it != ctxs.end()) return it->second;
  gs_ctx* c = gs_ctx_create(device, 0);
  if (!c) throw ThrustException(gs_last_global_error());
  // An autotuner table (python -m gpusort_gb300.autotune) named by
  // GPUSORT_GB300_TUNING applies to every context of the process.
  if (const char* path = std::getenv("GPUSORT_GB300_TUNING")) {
    if (gs_ctx_load_tuning(c, path) != GS_OK) {
      const std::string msg = gs_last_error(c);
      gs_ctx_destroy(c);
      throw ThrustException(msg.c_str());
    }
  }
  ctxs[device] = c;
  return c;
}

// Strategy of the entry points: the engine's fastest path by default (every
// strategy gives the same bytes); GPUSORT_GB300_ALGO=radix|sample|hyk picks
// one explicitly.
inline uint32_t Strategy(Family f) {
  const char* s = std::getenv("GPUSORT_GB300_ALGO");
  if (!s) return GS_ALGO_AUTO;
  if (!std::strcmp(s, "radix")) return GS_ALGO_RADIX;
  if (!std::strcmp(s, "sample")) return GS_ALGO_SAMPLE;
  if (!std::strcmp(s, "hyk")) return f == kHyk ? GS_ALGO_HYK : GS_ALGO_SAMPLE;
  return GS_ALGO_AUTO;
}

[[noreturn]] inline void Raise(Family f, gs_status st, const char* msg) {
  // Empty input: HykSort raises ThrustException, SampleSort and
  // HyperQuickSort MpiException, all with "No data to sort."
  // (include/helpers/hyksort_helper.h:105, samplesort_helper.h:69,
  //  hyperquicksort_helper.h:74). Device errors are ThrustExceptions
  // (src/cuda_utils.cu:373-393).
  if (st == GS_ERR_EMPTY && f != kHyk) throw MpiException(msg);
  throw ThrustException(msg);
}

inline void Check(gs_ctx* c, Family f, gs_status st) {
  if (st != GS_OK) Raise(f, st, gs_last_error(c));
}

// HYKSORT_CHECK / HYPERQUICKSORT_CHECK (include/hyksort_common_vector.inl:
// 31-43, include/hyperquicksort_common_vector.inl:30-41): p (or k) not a
// power of two runs SampleSort instead, with the same notice.
inline Family Resolve(Family f, const PartitionComm& comm, unsigned k_way) {
  if (f == kHyk && (!IsPowerOfTwo(unsigned(comm.size)) || !IsPowerOfTwo(k_way))) {
    std::cout << "The number of processes or k_way value is not a power of 2. "
              << "We are using SampleSort algorithm instead!" << std::endl;
    return kSample;
  }
  if (f == kHyperQuick && !IsPowerOfTwo(unsigned(comm.size))) {
    std::cout << "The number of processes is not a power of 2. "
              << "We are using SampleSort algorithm instead!" << std::endl;
    return kSample;
  }
  return f;
}

inline gs_opts Options(Family f, const PartitionComm& comm, unsigned k_way) {
  gs_opts o;
  std::memset(&o, 0, sizeof(o));
  o.algo = Strategy(f);
  o.partitions = uint32_t(comm.size > 0 ? comm.size : 1);
  o.k_way = k_way;
  o.oversample = 32;
  o.seed = 0x67707573u;
  return o;
}

template <typename Vector>
inline typename Vector::value_type* Data(Vector* v) {
  return v->size() ? &(*v)[0] : nullptr;
}

template <typename Comp, typename Vector>
void SortKeys(Family f, const PartitionComm& comm, unsigned k_way, Comp, Vector* keys) {
  typedef typename Vector::value_type T;
  static_assert(HasDtype<T>::value,
                "keys must be int, unsigned int, float, double, int64_t or uint64_t "
                "(use the KeyFunc overload for other types)");
  f = Resolve(f, comm, k_way);
  gs_ctx* c = Context(comm.device);
  const gs_opts o = Options(f, comm, k_way);
  const uint32_t flags = GS_FLAG_HOST | (Direction<Comp>::desc ? GS_FLAG_DESCENDING : 0u);
  Check(c, f, gs_sort_keys(c, Dtype<T>::v, Data(keys), Data(keys), keys->size(), flags, &o));
}

// Keys and one value vector: ties on the key ordered by value, as the
// reference's pair path (include/helpers/hyksort_helper.h:224-297).
template <typename Comp, typename VectorK, typename VectorV>
void SortPairs(Family f, const PartitionComm& comm, unsigned k_way, Comp, VectorK* keys,
               VectorV* values) {
  typedef typename VectorK::value_type K;
  typedef typename VectorV::value_type V;
  static_assert(HasDtype<K>::value && HasDtype<V>::value,
                "keys and values must be one of the six primitive types");
  f = Resolve(f, comm, k_way);
  gs_ctx* c = Context(comm.device);
  if (values->size() != keys->size()) Raise(f, GS_ERR_INVALID, "keys and values differ in size");
  const gs_opts o = Options(f, comm, k_way);
  const uint32_t flags = GS_FLAG_HOST | (Direction<Comp>::desc ? GS_FLAG_DESCENDING : 0u);
  Check(c, f, gs_sort_pairs(c, Dtype<K>::v, Dtype<V>::v, Data(keys), Data(values), Data(keys),
                            Data(values), keys->size(), flags, &o));
}

// Sort keys with their global indexes (stable), return the permutation
// (the reference's HykSortWithGlobalIndexes,
// include/hyksort_common_vector.inl:552-565).
template <typename Comp, typename VectorK>
std::vector<uint64_t> SortWithIndexes(Family f, const PartitionComm& comm, unsigned k_way, Comp,
                                      VectorK* keys) {
  typedef typename VectorK::value_type K;
  static_assert(HasDtype<K>::value, "keys must be one of the six primitive types");
  f = Resolve(f, comm, k_way);
  gs_ctx* c = Context(comm.device);
  std::vector<uint64_t> idx(keys->size());
  for (size_t i = 0; i < idx.size(); ++i) idx[i] = i;
  const gs_opts o = Options(f, comm, k_way);
  const uint32_t flags =
      GS_FLAG_HOST | GS_FLAG_PAIRS_STABLE | (Direction<Comp>::desc ? GS_FLAG_DESCENDING : 0u);
  Check(c, f, gs_sort_pairs(c, Dtype<K>::v, GS_U64, Data(keys), idx.data(), Data(keys),
                            idx.data(), keys->size(), flags, &o));
  return idx;
}

// Move one value vector to where its key went (the reference's
// ParUtils::ArrangeValues, include/par/par_utils.h:23-86), on the GPU.
template <typename Vector>
void Arrange(gs_ctx* c, Family f, const std::vector<uint64_t>& perm, Vector* values) {
  typedef typename Vector::value_type V;
  static_assert(std::is_trivially_copyable<V>::value && sizeof(V) <= 64,
                "value vectors hold trivially copyable elements of at most 64 bytes");
  if (values->size() != perm.size()) Raise(f, GS_ERR_INVALID, "value vector size differs from keys");
  if (perm.empty()) return;
  std::vector<V> tmp(values->begin(), values->end());
  Check(c, f, gs_gather(c, tmp.data(), Data(values), perm.size(), uint32_t(sizeof(V)),
                        perm.data(), GS_FLAG_HOST));
}

template <typename Comp, typename VectorK, typename... Vectors>
void SortMulti(Family f, const PartitionComm& comm, unsigned k_way, Comp comp, VectorK* keys,
               Vectors*... values) {
  if (keys->empty()) Raise(Resolve(f, comm, k_way), GS_ERR_EMPTY, "No data to sort.");
  const std::vector<uint64_t> perm = SortWithIndexes(f, comm, k_way, comp, keys);
  gs_ctx* c = Context(comm.device);
  int dummy[] = {0, (Arrange(c, f, perm, values), 0)...};
  (void)dummy;
}

// User-defined records: keys from `key_func`, a stable (key, index) sort on
// the GPU, records permuted on the host (include/helpers/hyksort_helper.h:
// 150-219 does the same with CudaCustomType{key, idx}).
template <typename KeyType, typename Comp, typename KeyFunc, typename Vector>
void SortRecords(Family f, const PartitionComm& comm, unsigned k_way, KeyFunc key_func,
                 Vector* list) {
  static_assert(HasDtype<KeyType>::value, "KeyType must be one of the six primitive types");
  f = Resolve(f, comm, k_way);
  if (list->empty()) Raise(f, GS_ERR_EMPTY, "No data to sort.");
  std::vector<KeyType> keys(list->size());
  for (size_t i = 0; i < keys.size(); ++i) keys[i] = key_func((*list)[i]);
  const std::vector<uint64_t> perm =
      SortWithIndexes(f, comm, k_way, typename std::conditional<Direction<Comp>::desc,
                                                                std::greater<KeyType>,
                                                                std::less<KeyType>>::type(),
                      &keys);
  Vector tmp(*list);
  for (size_t i = 0; i < perm.size(); ++i) (*list)[i] = tmp[perm[i]];
}

}  // namespace detail
}  // namespace gpusort

#endif  // GPUSORT_GB300_ENGINE_HPP_
