// ref_driver.cc - runs the reference's OWN sort code on thread-ranks.
// TEST INFRASTRUCTURE: compiled by oracle/ref/Makefile against the
// reference's headers and sources where they lie (nothing is copied) and the
// thread-rank MPI shim in this directory; output goes to oracle/_ref/.
//
// usage: ref_driver ALGO KTYPE NRANKS KWAY THREADS DESC IN OUT [VTYPE VIN VOUT]
//   ALGO   hyk | sample | hquick   (HykSort / SampleSort / HyperQuickSort)
//   KTYPE  u32 i32 f32 u64 i64 f64 (VTYPE: u32 i32 u64 i64 f64)
//   DESC   0 = std::less, 1 = std::greater
//   files  int64 element count, then the raw elements (the layout of the
//          reference's per-rank data files, src/test/utils.h:610-661), here
//          one file for the whole array; rank r gets the r-th block of
//          CalcNumElemsEachBlock elements (src/test/utils.h:629-650).
// The output file is the concatenation of the ranks' results in rank order.
// Rank 0 prints "seconds <t>" (wall time between barriers around the sort)
// and "sizes <n0> <n1> ..." on stderr. With GS_REF_REPEAT=R in the
// environment a keys-only sort runs R times, each on a fresh copy of the
// input, with one "seconds" line per run (the output is the last run's).
#include <omp.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>

#include <algorithm>
#include <functional>
#include <string>
#include <utility>
#include <vector>

#include "hyksort.h"
#include "hyperquicksort.h"
#include "samplesort.h"
#include "mpi.h"

namespace gpusort {
// The reference's GPU local sort lives in src/cuda_utils.cu (Thrust). This
// build runs its CPU path only: report no device, exactly as the reference
// does on a machine without a GPU (src/cuda_utils.cu:81-92 +
// include/helpers/hyksort_helper.h:112).
int CudaUtils::GetDeviceCount() throw(ThrustException) { return 0; }
bool CudaUtils::IsHavingDevices() throw(ThrustException) { return false; }
template<typename StrictWeakOrdering, typename RandomAccessIterator>
void CudaUtils::Sort(StrictWeakOrdering comp, int rank, RandomAccessIterator first,
                     RandomAccessIterator last) throw(ThrustException) {
  throw ThrustException("no GPU in the thread-rank oracle build");
}
template<typename StrictWeakOrdering, typename RandomAccessIterator1,
         typename RandomAccessIterator2>
void CudaUtils::SortByKey(StrictWeakOrdering comp, int rank, RandomAccessIterator1 key_first,
                          RandomAccessIterator1 key_last, RandomAccessIterator2 val_first,
                          void* _out) throw(ThrustException) {
  throw ThrustException("no GPU in the thread-rank oracle build");
}
}  // namespace gpusort

namespace {

double now() {
  struct timeval tv;
  gettimeofday(&tv, 0);
  return tv.tv_sec + tv.tv_usec * 1e-6;
}

template <typename T>
std::vector<T> read_file(const char* path) {
  std::vector<T> v;
  FILE* f = fopen(path, "rb");
  if (!f) { fprintf(stderr, "cannot open %s\n", path); exit(2); }
  int64_t n = 0;
  if (fread(&n, sizeof(n), 1, f) != 1) { fprintf(stderr, "bad file %s\n", path); exit(2); }
  v.resize(n);
  if (n && fread(&v[0], sizeof(T), n, f) != size_t(n)) { fprintf(stderr, "short %s\n", path); exit(2); }
  fclose(f);
  return v;
}

template <typename T>
void write_file(const char* path, const std::vector<T>& v) {
  FILE* f = fopen(path, "wb");
  int64_t n = int64_t(v.size());
  fwrite(&n, sizeof(n), 1, f);
  if (n) fwrite(&v[0], sizeof(T), n, f);
  fclose(f);
}

struct Job {
  std::string algo;
  int nranks, kway, threads, desc;
  double seconds;
  void* keys;    // std::vector<K>* per rank (array of vectors)
  void* vals;    // std::vector<V>* per rank or NULL
};

template <typename K>
void run_keys_rank(Job* j, int rank) {
  omp_set_num_threads(j->threads);
  std::vector<K>& keys = static_cast<std::vector<K>*>(j->keys)[rank];
  MPI_Comm comm = MPI_COMM_WORLD;
  MPI_Barrier(comm);
  double t0 = now();
  if (j->algo == "hyk") {
    if (j->desc) gpusort::HykSort(comm, std::greater<K>(), j->kway, false, &keys);
    else gpusort::HykSort(comm, j->kway, false, &keys);
  } else if (j->algo == "sample") {
    if (j->desc) gpusort::SampleSort(comm, std::greater<K>(), &keys);
    else gpusort::SampleSort(comm, &keys);
  } else {
    if (j->desc) gpusort::HyperQuickSort(comm, std::greater<K>(), &keys);
    else gpusort::HyperQuickSort(comm, &keys);
  }
  MPI_Barrier(comm);
  if (rank == 0) j->seconds = now() - t0;
}

template <typename K, typename V>
void run_pairs_rank(Job* j, int rank) {
  omp_set_num_threads(j->threads);
  std::vector<K>& keys = static_cast<std::vector<K>*>(j->keys)[rank];
  std::vector<V>& vals = static_cast<std::vector<V>*>(j->vals)[rank];
  MPI_Comm comm = MPI_COMM_WORLD;
  MPI_Barrier(comm);
  double t0 = now();
  if (j->algo == "hyk") {
    if (j->desc) gpusort::HykSort(comm, std::greater<K>(), j->kway, false, &keys, &vals);
    else gpusort::HykSort(comm, j->kway, false, &keys, &vals);
  } else if (j->algo == "sample") {
    if (j->desc) gpusort::SampleSort(comm, std::greater<K>(), &keys, &vals);
    else gpusort::SampleSort(comm, &keys, &vals);
  } else {
    if (j->desc) gpusort::HyperQuickSort(comm, std::greater<K>(), &keys, &vals);
    else gpusort::HyperQuickSort(comm, &keys, &vals);
  }
  MPI_Barrier(comm);
  if (rank == 0) j->seconds = now() - t0;
}

template <typename K>
void keys_entry(void* arg, int rank) { run_keys_rank<K>(static_cast<Job*>(arg), rank); }

template <typename K, typename V>
void pairs_entry(void* arg, int rank) { run_pairs_rank<K, V>(static_cast<Job*>(arg), rank); }

template <typename T>
std::vector<std::vector<T> > split(const std::vector<T>& all, int np) {
  std::vector<std::vector<T> > out(np);
  const int64_t total = int64_t(all.size());
  const int64_t each = gpusort::CalcNumElemsEachBlock(total, np);
  for (int i = 0; i < np; ++i) {
    int64_t b = each * i;
    int64_t e = std::min<int64_t>(b + each, total);
    if (i == np - 1) e = total;
    if (b > total) b = total;
    out[i].assign(all.begin() + b, all.begin() + e);
  }
  return out;
}

template <typename T>
std::vector<T> concat(const std::vector<std::vector<T> >& parts, std::string* sizes) {
  std::vector<T> all;
  for (size_t i = 0; i < parts.size(); ++i) {
    all.insert(all.end(), parts[i].begin(), parts[i].end());
    char b[32];
    snprintf(b, sizeof(b), " %lld", (long long)parts[i].size());
    *sizes += b;
  }
  return all;
}

template <typename K>
int do_keys(Job& j, const char* in, const char* out) {
  const std::vector<K> input = read_file<K>(in);
  const char* rep = getenv("GS_REF_REPEAT");
  const int runs = rep ? std::max(1, atoi(rep)) : 1;
  std::vector<std::vector<K> > ranks;
  for (int r = 0; r < runs; ++r) {
    ranks = split(input, j.nranks);
    j.keys = &ranks[0];
    j.vals = 0;
    shim_run_ranks(j.nranks, keys_entry<K>, &j);
    fprintf(stderr, "seconds %.9f\n", j.seconds);
  }
  std::string sizes;
  write_file(out, concat(ranks, &sizes));
  fprintf(stderr, "sizes%s\n", sizes.c_str());
  return 0;
}

template <typename K, typename V>
int do_pairs(Job& j, const char* in, const char* out, const char* vin, const char* vout) {
  std::vector<std::vector<K> > kr = split(read_file<K>(in), j.nranks);
  std::vector<std::vector<V> > vr = split(read_file<V>(vin), j.nranks);
  // Register the pair's MPI type on this thread before the ranks look it up
  // concurrently (the reference caches it in a process-wide map,
  // include/mpi/mpi_common.h:77-95).
  gpusort::MpiDataUtils::GetType<std::pair<K, V> >();
  j.keys = &kr[0];
  j.vals = &vr[0];
  shim_run_ranks(j.nranks, pairs_entry<K, V>, &j);
  std::string sizes, vs;
  write_file(out, concat(kr, &sizes));
  write_file(vout, concat(vr, &vs));
  fprintf(stderr, "seconds %.9f\nsizes%s\n", j.seconds, sizes.c_str());
  return 0;
}

template <typename K>
int dispatch_v(Job& j, const std::string& vt, char** argv) {
  if (vt == "u32") return do_pairs<K, uint32_t>(j, argv[7], argv[8], argv[10], argv[11]);
  if (vt == "i32") return do_pairs<K, int32_t>(j, argv[7], argv[8], argv[10], argv[11]);
  if (vt == "u64") return do_pairs<K, uint64_t>(j, argv[7], argv[8], argv[10], argv[11]);
  if (vt == "i64") return do_pairs<K, int64_t>(j, argv[7], argv[8], argv[10], argv[11]);
  if (vt == "f64") return do_pairs<K, double>(j, argv[7], argv[8], argv[10], argv[11]);
  fprintf(stderr, "unknown value type %s\n", vt.c_str());
  return 2;
}

template <typename K>
int dispatch(Job& j, int argc, char** argv) {
  if (argc >= 12) return dispatch_v<K>(j, argv[9], argv);
  return do_keys<K>(j, argv[7], argv[8]);
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 9 && argc != 12) {
    fprintf(stderr, "usage: %s ALGO KTYPE NRANKS KWAY THREADS DESC IN OUT [VTYPE VIN VOUT]\n",
            argv[0]);
    return 2;
  }
  Job j;
  j.algo = argv[1];
  std::string kt = argv[2];
  j.nranks = atoi(argv[3]);
  j.kway = atoi(argv[4]);
  j.threads = atoi(argv[5]);
  j.desc = atoi(argv[6]);
  j.seconds = 0;
  if (kt == "u32") return dispatch<uint32_t>(j, argc, argv);
  if (kt == "i32") return dispatch<int32_t>(j, argc, argv);
  if (kt == "f32") return dispatch<float>(j, argc, argv);
  if (kt == "u64") return dispatch<uint64_t>(j, argc, argv);
  if (kt == "i64") return dispatch<int64_t>(j, argc, argv);
  if (kt == "f64") return dispatch<double>(j, argc, argv);
  fprintf(stderr, "unknown key type %s\n", kt.c_str());
  return 2;
}
