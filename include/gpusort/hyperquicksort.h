// gpusort/hyperquicksort.h - HyperQuickSort entry points of gpusort_gb300 (header only).
//
// Same names and overload shapes as the reference's include/hyperquicksort_common_vector.h:12-172; the MPI
// communicator becomes a PartitionComm (p partitions of one array on one
// GPU) and the vector is the whole array, sorted globally in place.
// p not a power of two runs SampleSort, as the reference does
// (include/hyperquicksort_common_vector.inl:30-41).
#ifndef GPUSORT_GB300_HYPERQUICKSORT_H_
#define GPUSORT_GB300_HYPERQUICKSORT_H_

#include "engine.h"

namespace gpusort {

template <typename Vector>
void HyperQuickSort(MpiComm comm, Vector* keys) {
  typedef typename Vector::value_type T;
  HyperQuickSort(comm, std::less<T>(), keys);
}

template <typename StrictWeakOrdering, typename Vector,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HyperQuickSort(MpiComm comm, StrictWeakOrdering comp, Vector* keys) {
  detail::SortKeys(detail::kHyperQuick, comm, 2, comp, keys);
}

// User-defined records sorted by key_func(record): the reference sorts
// records with their own operator< on the CPU; on the GPU the key is
// extracted first, as HykSort's record overload does.
template <typename KeyType, typename StrictWeakOrdering, typename KeyFunc, typename Vector,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HyperQuickSort(MpiComm comm, StrictWeakOrdering, KeyFunc key_func, Vector* list) {
  detail::SortRecords<KeyType, StrictWeakOrdering>(detail::kHyperQuick, comm, 2, key_func, list);
}

template <typename VectorK, typename VectorV>
void HyperQuickSort(MpiComm comm, VectorK* keys, VectorV* values) {
  typedef typename VectorK::value_type K;
  HyperQuickSort(comm, std::less<K>(), keys, values);
}

template <typename StrictWeakOrdering, typename VectorK, typename VectorV,
          typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HyperQuickSort(MpiComm comm, StrictWeakOrdering comp, VectorK* keys, VectorV* values) {
  detail::SortPairs(detail::kHyperQuick, comm, 2, comp, keys, values);
}

template <typename VectorK, typename VectorV1, typename VectorV2, typename... Vectors>
void HyperQuickSort(MpiComm comm, VectorK* keys, VectorV1* v1, VectorV2* v2, Vectors*... values) {
  typedef typename VectorK::value_type K;
  HyperQuickSort(comm, std::less<K>(), keys, v1, v2, values...);
}

template <typename StrictWeakOrdering, typename VectorK, typename VectorV1, typename VectorV2,
          typename... Vectors, typename = detail::EnableIfComparator<StrictWeakOrdering>>
void HyperQuickSort(MpiComm comm, StrictWeakOrdering comp, VectorK* keys, VectorV1* v1, VectorV2* v2,
            Vectors*... values) {
  detail::SortMulti(detail::kHyperQuick, comm, 2, comp, keys, v1, v2, values...);
}

}  // namespace gpusort

#endif  // GPUSORT_GB300_HYPERQUICKSORT_H_
