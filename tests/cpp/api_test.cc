// Exercises the C++ drop-in layer (include/gpusort/) the way the
// reference's test drivers call HykSort / SampleSort / HyperQuickSort
// (src/test/utils.h:776-791,872-887; src/test/test_user_defined.cc:
// 414-427), checking every result against std::sort / std::stable_sort.
// Exit status 0 when every check passes.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <functional>
#include <numeric>
#include <random>
#include <tuple>
#include <vector>

#include "gpusort/gpusort.h"

static int failures = 0;
#define CHECK(cond, what)                                      \
  do {                                                         \
    if (!(cond)) {                                             \
      std::printf("FAIL %s (%s:%d)\n", what, __FILE__, __LINE__); \
      ++failures;                                              \
    } else {                                                   \
      std::printf("ok   %s\n", what);                          \
    }                                                          \
  } while (0)

template <typename T>
std::vector<T> Random(size_t n, uint64_t seed, uint64_t mod = 0) {
  std::mt19937_64 g(seed);
  std::vector<T> v(n);
  for (auto& x : v) {
    const uint64_t r = mod ? g() % mod : g();
    if (std::is_floating_point<T>::value) x = T(double(int64_t(r % 2000001) - 1000000) / 7.0);
    else x = T(r);
  }
  return v;
}

// A user-defined record with a key, like the reference's SampleClass
// (src/test/test_user_defined.cc:23-150).
struct Record {
  int64_t key;
  double v1;
  float v2;
  bool operator<(const Record& o) const { return key < o.key; }
  bool operator>(const Record& o) const { return key > o.key; }
};
static int64_t GetKey(const Record& r) { return r.key; }

int main() {
  gpusort::PartitionComm comm(4);  // four virtual ranks

  {  // HykSort, keys, k = 4
    auto a = Random<uint32_t>(1 << 20, 1), want = a;
    std::sort(want.begin(), want.end());
    gpusort::HykSort(comm, 4, true, &a);
    CHECK(a == want, "HykSort uint32 ascending");
  }
  {  // comparator: std::greater
    auto a = Random<int64_t>(300001, 2, 1000), want = a;
    std::sort(want.begin(), want.end(), std::greater<int64_t>());
    gpusort::HykSort(comm, std::greater<int64_t>(), 4, true, &a);
    CHECK(a == want, "HykSort int64 descending with duplicates");
  }
  {
    auto a = Random<float>(200003, 3), want = a;
    std::sort(want.begin(), want.end());
    gpusort::SampleSort(comm, &a);
    CHECK(a == want, "SampleSort float");
  }
  {
    auto a = Random<double>(100000, 4), want = a;
    std::sort(want.begin(), want.end(), std::greater<double>());
    gpusort::HyperQuickSort(comm, std::greater<double>(), &a);
    CHECK(a == want, "HyperQuickSort double descending");
  }
  {  // keys + values: ties ordered by value, like std::pair
    auto k = Random<int>(100000, 5, 50);
    auto v = Random<unsigned>(100000, 6, 1000);
    std::vector<std::pair<int, unsigned>> p(k.size());
    for (size_t i = 0; i < k.size(); ++i) p[i] = {k[i], v[i]};
    std::sort(p.begin(), p.end(), std::greater<std::pair<int, unsigned>>());
    gpusort::HykSort(comm, std::greater<int>(), 4, true, &k, &v);
    bool ok = true;
    for (size_t i = 0; i < p.size(); ++i) ok &= (k[i] == p[i].first && v[i] == p[i].second);
    CHECK(ok, "HykSort keys + values, ties by value (descending)");
  }
  {  // keys + three value vectors: values follow their key (stable)
    auto k = Random<uint64_t>(50000, 7, 100);
    std::vector<double> v1(k.size());
    std::vector<float> v2(k.size());
    std::vector<int> v3(k.size());
    for (size_t i = 0; i < k.size(); ++i) { v1[i] = double(i) * 0.5; v2[i] = float(i); v3[i] = int(i); }
    std::vector<size_t> order(k.size());
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return k[a] < k[b]; });
    const auto k0 = k;
    gpusort::HykSort(comm, 4, true, &k, &v1, &v2, &v3);
    bool ok = true;
    for (size_t i = 0; i < k.size(); ++i)
      ok &= k[i] == k0[order[i]] && v1[i] == double(order[i]) * 0.5 && v2[i] == float(order[i]) &&
            v3[i] == int(order[i]);
    CHECK(ok, "HykSort keys + 3 value vectors");
    auto s = Random<int>(20000, 8, 9);
    std::vector<long> w1(s.size()), w2(s.size());
    for (size_t i = 0; i < s.size(); ++i) w1[i] = long(i), w2[i] = -long(i);
    gpusort::SampleSort(comm, &s, &w1, &w2);
    bool ok2 = std::is_sorted(s.begin(), s.end());
    for (size_t i = 0; i < s.size(); ++i) ok2 &= w2[i] == -w1[i];
    CHECK(ok2, "SampleSort keys + 2 value vectors");
  }
  {  // user-defined records with a key function
    std::vector<Record> list(100000);
    auto keys = Random<int64_t>(list.size(), 9, 5000);
    for (size_t i = 0; i < list.size(); ++i) list[i] = Record{keys[i], double(i), float(i) * 2};
    auto want = list;
    std::stable_sort(want.begin(), want.end());
    gpusort::HykSort<int64_t>(comm, std::less<Record>(), 4, true, &GetKey, &list);
    bool ok = true;
    for (size_t i = 0; i < list.size(); ++i) ok &= list[i].key == want[i].key && list[i].v1 == want[i].v1;
    CHECK(ok, "HykSort user-defined records (KeyFunc)");
    gpusort::SampleSort<int64_t>(comm, std::greater<Record>(), &GetKey, &list);
    bool desc = true;
    for (size_t i = 1; i < list.size(); ++i) desc &= list[i - 1].key >= list[i].key;
    CHECK(desc, "SampleSort user-defined records descending");
  }
  {  // p or k not a power of two: SampleSort with the reference's notice
    gpusort::PartitionComm six(6);
    auto a = Random<uint32_t>(123457, 10), want = a;
    std::sort(want.begin(), want.end());
    gpusort::HykSort(six, 3, true, &a);
    CHECK(a == want, "HykSort with p = 6, k = 3 falls back to SampleSort");
  }
  {  // empty input and the CPU-path request
    std::vector<uint32_t> e;
    bool thrust = false, mpi = false, cpu = false;
    try { gpusort::HykSort(comm, 4, true, &e); } catch (gpusort::ThrustException& x) {
      thrust = std::string(x.what()) == "No data to sort.";
    }
    try { gpusort::SampleSort(comm, &e); } catch (gpusort::MpiException& x) {
      mpi = std::string(x.what()) == "No data to sort.";
    }
    std::vector<uint32_t> one{3, 1, 2};
    try { gpusort::HykSort(comm, 4, false, &one); } catch (gpusort::ThrustException&) { cpu = true; }
    CHECK(thrust, "HykSort empty input -> ThrustException(\"No data to sort.\")");
    CHECK(mpi, "SampleSort empty input -> MpiException(\"No data to sort.\")");
    CHECK(cpu, "is_using_gpu = false is refused");
  }
  std::printf("%s: %d failure(s)\n", failures ? "FAILED" : "PASSED", failures);
  return failures ? 1 : 0;
}
