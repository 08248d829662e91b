// Host-only stand-in for the small part of the Kokkos Core API that the
// reference's FDTD sources use (Views of double, MDRangePolicy, parallel_for,
// deep_copy, fence, the hwloc/configuration queries of the sample driver).
//
// Test infrastructure only: it exists so that the reference's own, unmodified
// Kokkos-path sources compile on a machine without the Kokkos submodule and
// serve as the oracle against which the CUDA engine is checked.  Dispatch is a
// plain (OpenMP-parallel) loop nest; the reference's functors have no
// cross-iteration dependencies inside one parallel_for, so the iteration order
// does not change any result.
#pragma once

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <initializer_list>
#include <memory>
#include <ostream>
#include <string>
#include <type_traits>
#include <utility>
#ifdef _OPENMP
#include <omp.h>
#endif

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

struct LayoutLeft {};
struct LayoutRight {};
enum MemoryTraitsFlags { Aligned = 1 };
template <unsigned Flags> struct MemoryTraits {};
struct OpenMPSpace {};
using DefaultExecutionSpace = OpenMPSpace;
using HostSpace = OpenMPSpace;

struct WithoutInitializing_t {};
constexpr WithoutInitializing_t WithoutInitializing{};

struct ViewAllocProp {
  std::string label;
  bool initialize = true;
};
inline ViewAllocProp view_alloc(WithoutInitializing_t, const std::string& label) {
  return ViewAllocProp{label, false};
}
inline ViewAllocProp view_alloc(const std::string& label, WithoutInitializing_t) {
  return ViewAllocProp{label, false};
}

template <class DataType, class... Props> class View;

// Rank-1 view of T with shared ownership (copies alias the same storage).
template <class T, class... Props>
class View<T*, Props...> {
 public:
  using value_type = T;
  View() = default;
  // Every allocation is zero-filled, WithoutInitializing included.  The
  // reference's PML class allocates its conductivity and split-field arrays
  // without initialisation and reads them in cells it never sets
  // (src/FDTD_kokkos/FDTD_PML_kokkos.cpp:47-69, first touch commented out);
  // a zero fill gives those reads the values a fresh allocation holds, so the
  // reference's results are defined and repeatable.
  View(const ViewAllocProp& prop, std::size_t n) : label_(prop.label), n_(n) {
    data_ = std::shared_ptr<T[]>(new T[n ? n : 1]);
    (void)prop.initialize;
    std::memset(data_.get(), 0, sizeof(T) * (n ? n : 1));
  }
  View(const std::string& label, std::size_t n) : View(ViewAllocProp{label, true}, n) {}
  T& operator()(long i) const { return data_[i]; }
  T& operator[](long i) const { return data_[i]; }
  T* data() const { return data_.get(); }
  std::size_t size() const { return n_; }
  std::size_t extent(int) const { return n_; }
  const std::string& label() const { return label_; }

 private:
  std::string label_;
  std::size_t n_ = 0;
  std::shared_ptr<T[]> data_;
};

template <class V>
inline void deep_copy(const V& dst, const typename V::value_type& value) {
  const long n = static_cast<long>(dst.size());
  typename V::value_type* p = dst.data();
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) p[i] = value;
}
template <class V1, class V2>
inline auto deep_copy(const V1& dst, const V2& src)
    -> decltype(dst.data(), src.data(), void()) {
  if (dst.data() != src.data())
    std::memcpy(dst.data(), src.data(), sizeof(typename V1::value_type) * dst.size());
}
template <class V>
inline V create_mirror_view(const V& v) { return v; }  // host space: the mirror is the view

namespace Iterate_ns {}
enum class Iterate { Default, Left, Right };

template <unsigned N, Iterate Outer = Iterate::Default, Iterate Inner = Iterate::Default>
struct Rank {
  static constexpr unsigned rank = N;
};

template <class RankT>
struct MDRangePolicy {
  static_assert(RankT::rank == 3, "shim supports rank-3 policies only");
  long lo[3];
  long hi[3];
  MDRangePolicy(std::initializer_list<long> b, std::initializer_list<long> e) {
    int d = 0;
    for (long v : b) lo[d++] = v;
    d = 0;
    for (long v : e) hi[d++] = v;
  }
};

template <class F>
struct RangePolicy {
  long lo, hi;
  RangePolicy(long b, long e) : lo(b), hi(e) {}
};

// The functor is called with the indices in the order the policy lists them;
// the outermost index is split across threads.
template <class RankT, class Functor>
inline void parallel_for(const MDRangePolicy<RankT>& p, const Functor& f) {
  const long a0 = p.lo[0], b0 = p.hi[0];
#pragma omp parallel for schedule(static)
  for (long x0 = a0; x0 < b0; ++x0)
    for (long x1 = p.lo[1]; x1 < p.hi[1]; ++x1)
      for (long x2 = p.lo[2]; x2 < p.hi[2]; ++x2)
        f(static_cast<int>(x0), static_cast<int>(x1), static_cast<int>(x2));
}
template <class RankT, class Functor>
inline void parallel_for(const std::string&, const MDRangePolicy<RankT>& p, const Functor& f) {
  parallel_for(p, f);
}
template <class Functor>
inline void parallel_for(const std::string&, long n, const Functor& f) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) f(static_cast<int>(i));
}

inline void fence() {}
inline void fence(const std::string&) {}
inline void initialize(int&, char**) {}
inline void initialize() {}
inline void finalize() {}

inline void print_configuration(std::ostream& os, bool = false) {
  int threads = 1;
#ifdef _OPENMP
  threads = omp_get_max_threads();
#endif
  os << "Kokkos host shim (OpenMP threads: " << threads << ")" << std::endl;
}

namespace hwloc {
inline bool available() { return false; }
inline unsigned get_available_numa_count() { return 1; }
inline unsigned get_available_cores_per_numa() {
#ifdef _OPENMP
  return static_cast<unsigned>(omp_get_num_procs());
#else
  return 1;
#endif
}
inline unsigned get_available_threads_per_core() { return 1; }
}  // namespace hwloc

}  // namespace Kokkos
