// gpusort/hyksort.h - HykSort entry points of gpusort_gb300 (header only).
//
// Same names and overload shapes as the reference's
// include/hyksort_common_vector.h:12-214; the MPI communicator becomes a
// PartitionComm (p partitions of one array on one GPU) and the vector is
// the whole array, sorted globally in place. p or k not a power of two
// runs SampleSort, as the reference does
// (include/hyksort_common_vector.inl:31-43).
#ifndef GPUSORT_GB300_HYKSORT_H_
#define GPUSORT_GB300_HYKSORT_H_

#include "engine.h"
#include "samplesort.h"

namespace gpusort {

template <typename Vector>
void HykSort(MpiComm comm, unsigned int k_way, bool is_using_gpu, Vector* keys) {
  typedef typename Vector::value_type T;
  HykSort(comm, std::less<T>(), k_way, is_using_gpu, keys);
}

template <typename StrictWeakOrdering, typename Vector,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HykSort(MpiComm comm, StrictWeakOrdering comp, unsigned int k_way, bool is_using_gpu,
             Vector* keys) {
  detail::RequireGpu(is_using_gpu);
  detail::SortKeys(detail::kHyk, comm, k_way, comp, keys);
}

// User-defined records sorted by key_func(record) (KeyType: a primitive).
template <typename KeyType, typename KeyFunc, typename Vector>
void HykSort(MpiComm comm, unsigned int k_way, bool is_using_gpu, KeyFunc key_func,
             Vector* list) {
  typedef typename Vector::value_type T;
  HykSort<KeyType>(comm, std::less<T>(), k_way, is_using_gpu, key_func, list);
}

template <typename KeyType, typename StrictWeakOrdering, typename KeyFunc, typename Vector,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HykSort(MpiComm comm, StrictWeakOrdering, unsigned int k_way, bool is_using_gpu,
             KeyFunc key_func, Vector* list) {
  detail::RequireGpu(is_using_gpu);
  detail::SortRecords<KeyType, StrictWeakOrdering>(detail::kHyk, comm, k_way, key_func, list);
}

// Keys and one value vector: ties ordered by value.
template <typename VectorK, typename VectorV>
void HykSort(MpiComm comm, unsigned int k_way, bool is_using_gpu, VectorK* keys,
             VectorV* values) {
  typedef typename VectorK::value_type K;
  HykSort(comm, std::less<K>(), k_way, is_using_gpu, keys, values);
}

template <typename StrictWeakOrdering, typename VectorK, typename VectorV,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HykSort(MpiComm comm, StrictWeakOrdering comp, unsigned int k_way, bool is_using_gpu,
             VectorK* keys, VectorV* values) {
  detail::RequireGpu(is_using_gpu);
  detail::SortPairs(detail::kHyk, comm, k_way, comp, keys, values);
}

// Keys and two or more value vectors: (key, global index) sort, then each
// value vector follows its key.
template <typename VectorK, typename VectorV1, typename VectorV2, typename... Vectors>
void HykSort(MpiComm comm, unsigned int k_way, bool is_using_gpu, VectorK* keys,
             VectorV1* v1, VectorV2* v2, Vectors*... values) {
  typedef typename VectorK::value_type K;
  HykSort(comm, std::less<K>(), k_way, is_using_gpu, keys, v1, v2, values...);
}

template <typename StrictWeakOrdering, typename VectorK, typename VectorV1, typename VectorV2,
          typename... Vectors, typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HykSort(MpiComm comm, StrictWeakOrdering comp, unsigned int k_way, bool is_using_gpu,
             VectorK* keys, VectorV1* v1, VectorV2* v2, Vectors*... values) {
  detail::RequireGpu(is_using_gpu);
  detail::SortMulti(detail::kHyk, comm, k_way, comp, keys, v1, v2, values...);
}

}  // namespace gpusort

#endif  // GPUSORT_GB300_HYKSORT_H_
