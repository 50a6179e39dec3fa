// Kokkos-subset shim: TEST INFRASTRUCTURE ONLY.
//
// The reference solver (Maccchiatooo/Cylinder-flow) is written against Kokkos
// (Views in CudaUVMSpace, RangePolicy/MDRangePolicy parallel_for, parallel_reduce
// with Sum/Max/Min, Random_XorShift64_Pool, subview/deep_copy).  Kokkos is not
// installed on this machine, so this header re-implements exactly the subset the
// reference sources use, on the host, with OpenMP for parallel_for.  It lets the
// reference's own lbm.cpp / System.cpp compile UNMODIFIED into the CPU oracle
// binaries under oracle/_ref/ (the "reference's own Kokkos OpenMP build").
//
// Semantics kept from Kokkos:
//   * Views are reference-counted handles, zero-initialised on allocation.
//   * Default layout is LayoutRight (last index fastest), as in a Kokkos
//     OpenMP/host build; CudaUVMSpace is an alias of host memory.
//   * parallel_for runs every index exactly once; order is unspecified.
//   * parallel_reduce here runs serially in lexicographic index order so that
//     floating-point sums are reproducible (real Kokkos leaves the order open).
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <initializer_list>
#include <limits>
#include <stdexcept>
#include <cmath>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_CLASS_LAMBDA [=, *this]

namespace Kokkos {

inline void initialize(int &, char **) {}
inline void initialize() {}
inline void finalize() {}
inline void fence() {}

struct LayoutLeft {};
struct LayoutRight {};
struct HostSpace {};
struct CudaUVMSpace {};
struct CudaSpace {};
struct OpenMP {};

struct ALL_t {};
constexpr ALL_t ALL{};

namespace impl {
template <class T> struct strip { using type = T; static constexpr int rank = 0; };
template <class T> struct strip<T *> {
  using type = typename strip<T>::type;
  static constexpr int rank = strip<T>::rank + 1;
};
template <class... P> struct has_left : std::false_type {};
template <class H, class... P>
struct has_left<H, P...>
    : std::integral_constant<bool, std::is_same<H, LayoutLeft>::value || has_left<P...>::value> {};
}  // namespace impl

// Rank-N strided view over a shared buffer.  Used for Views and subviews.
template <class DataType, class... Props>
class View {
 public:
  using value_type = typename impl::strip<DataType>::type;
  static constexpr int Rank = impl::strip<DataType>::rank;
  static constexpr bool left = impl::has_left<Props...>::value;

  View() = default;
  explicit View(const std::string &, size_t n0 = 0, size_t n1 = 0, size_t n2 = 0,
                size_t n3 = 0, size_t n4 = 0, size_t n5 = 0) {
    size_t n[6] = {n0, n1, n2, n3, n4, n5};
    size_t total = 1;
    for (int r = 0; r < Rank; ++r) {
      ext_[r] = n[r];
      total *= n[r];
    }
    if (left) {
      size_t s = 1;
      for (int r = 0; r < Rank; ++r) { stride_[r] = s; s *= ext_[r]; }
    } else {
      size_t s = 1;
      for (int r = Rank - 1; r >= 0; --r) { stride_[r] = s; s *= ext_[r]; }
    }
    mem_ = std::shared_ptr<value_type>(new value_type[total > 0 ? total : 1](),
                                       std::default_delete<value_type[]>());
    ptr_ = mem_.get();
    size_ = total;
  }

  template <class... I>
  inline value_type &operator()(I... idx) const {
    static_assert(sizeof...(I) == (size_t)Rank, "View rank mismatch");
    const long ii[] = {static_cast<long>(idx)...};
    long off = 0;
    for (int r = 0; r < Rank; ++r) off += ii[r] * static_cast<long>(stride_[r]);
    return ptr_[off];
  }

  value_type *data() const { return ptr_; }
  size_t size() const { return size_; }
  size_t span() const { return size_; }
  size_t extent(int r) const { return ext_[r]; }
  int extent_int(int r) const { return static_cast<int>(ext_[r]); }
  size_t stride(int r) const { return stride_[r]; }

  // Element-wise access in logical (lexicographic) order, for deep_copy.
  value_type &flat(size_t k) const {
    long off = 0;
    for (int r = Rank - 1; r >= 0; --r) {
      size_t e = ext_[r] ? ext_[r] : 1;
      off += static_cast<long>(k % e) * static_cast<long>(stride_[r]);
      k /= e;
    }
    return ptr_[off];
  }

  // Internal: build a sub-view.
  std::shared_ptr<value_type> mem_;
  value_type *ptr_ = nullptr;
  size_t ext_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  size_t stride_[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  size_t size_ = 0;
};

// ---- subview ---------------------------------------------------------------
namespace impl {
struct SubState {
  long offset = 0;
  int rank = 0;
  size_t ext[8];
  size_t stride[8];
};
template <class V>
inline void sub_apply(const V &v, SubState &st, int r, ALL_t) {
  st.ext[st.rank] = v.ext_[r];
  st.stride[st.rank] = v.stride_[r];
  ++st.rank;
}
template <class V, class A, class B>
inline void sub_apply(const V &v, SubState &st, int r, const std::pair<A, B> &p) {
  st.offset += static_cast<long>(p.first) * static_cast<long>(v.stride_[r]);
  st.ext[st.rank] = static_cast<size_t>(p.second - p.first);
  st.stride[st.rank] = v.stride_[r];
  ++st.rank;
}
template <class V, class I,
          typename std::enable_if<std::is_integral<I>::value, int>::type = 0>
inline void sub_apply(const V &v, SubState &st, int r, I i) {
  st.offset += static_cast<long>(i) * static_cast<long>(v.stride_[r]);
}
template <class T> struct is_kept : std::true_type {};
template <> struct is_kept<int> : std::false_type {};
template <> struct is_kept<long> : std::false_type {};
template <> struct is_kept<unsigned> : std::false_type {};
template <> struct is_kept<size_t> : std::false_type {};
template <class... A> struct count_kept { static constexpr int value = 0; };
template <class H, class... A> struct count_kept<H, A...> {
  static constexpr int value =
      (is_kept<typename std::decay<H>::type>::value ? 1 : 0) + count_kept<A...>::value;
};
template <class T, int N> struct add_ptr { using type = typename add_ptr<T *, N - 1>::type; };
template <class T> struct add_ptr<T, 0> { using type = T; };
}  // namespace impl

template <class DataType, class... Props, class... Args>
auto subview(const View<DataType, Props...> &v, Args... args)
    -> View<typename impl::add_ptr<typename View<DataType, Props...>::value_type,
                                   impl::count_kept<Args...>::value>::type,
            LayoutRight> {
  using VT = typename View<DataType, Props...>::value_type;
  constexpr int R = impl::count_kept<Args...>::value;
  impl::SubState st;
  int r = 0;
  int dummy[] = {(impl::sub_apply(v, st, r++, args), 0)...};
  (void)dummy;
  View<typename impl::add_ptr<VT, R>::type, LayoutRight> out;
  out.mem_ = v.mem_;
  out.ptr_ = v.ptr_ + st.offset;
  size_t total = 1;
  for (int k = 0; k < R; ++k) {
    out.ext_[k] = st.ext[k];
    out.stride_[k] = st.stride[k];
    total *= st.ext[k];
  }
  out.size_ = total;
  return out;
}

template <class D1, class... P1, class D2, class... P2>
void deep_copy(const View<D1, P1...> &dst, const View<D2, P2...> &src) {
  if (dst.size() != src.size()) {
    std::fprintf(stderr, "Kokkos shim: deep_copy size mismatch %zu vs %zu\n", dst.size(),
                 src.size());
    std::abort();
  }
  for (size_t k = 0; k < dst.size(); ++k) dst.flat(k) = src.flat(k);
}

// ---- execution policies ------------------------------------------------------
template <unsigned N> struct Rank { static constexpr unsigned rank = N; };

template <class... Args>
struct RangePolicy {
  long b, e;
  RangePolicy(long b_, long e_) : b(b_), e(e_) {}
};

template <class R, class... Args>
struct MDRangePolicy {
  static constexpr int N = R::rank;
  long b[8], e[8];
  MDRangePolicy(std::initializer_list<long> lo, std::initializer_list<long> hi) {
    int k = 0;
    for (long x : lo) b[k++] = x;
    k = 0;
    for (long x : hi) e[k++] = x;
  }
};

template <class F, class... A>
void parallel_for(const std::string &, const RangePolicy<A...> &p, const F &f) {
#pragma omp parallel for schedule(static)
  for (long i = p.b; i < p.e; ++i) f(static_cast<int>(i));
}
template <class F>
void parallel_for(const std::string &, long n, const F &f) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < n; ++i) f(static_cast<int>(i));
}
template <class F, class... A>
void parallel_for(const std::string &, const MDRangePolicy<Rank<2>, A...> &p, const F &f) {
#pragma omp parallel for collapse(2) schedule(static)
  for (long i = p.b[0]; i < p.e[0]; ++i)
    for (long j = p.b[1]; j < p.e[1]; ++j) f(static_cast<int>(i), static_cast<int>(j));
}
template <class F, class... A>
void parallel_for(const std::string &, const MDRangePolicy<Rank<3>, A...> &p, const F &f) {
#pragma omp parallel for collapse(2) schedule(static)
  for (long i = p.b[0]; i < p.e[0]; ++i)
    for (long j = p.b[1]; j < p.e[1]; ++j)
      for (long k = p.b[2]; k < p.e[2]; ++k)
        f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k));
}
template <class F, class... A>
void parallel_for(const std::string &, const MDRangePolicy<Rank<4>, A...> &p, const F &f) {
#pragma omp parallel for collapse(3) schedule(static)
  for (long i = p.b[0]; i < p.e[0]; ++i)
    for (long j = p.b[1]; j < p.e[1]; ++j)
      for (long k = p.b[2]; k < p.e[2]; ++k)
        for (long l = p.b[3]; l < p.e[3]; ++l)
          f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k),
            static_cast<int>(l));
}

// ---- reducers -----------------------------------------------------------------
template <class T> struct Max {
  T &ref;
  explicit Max(T &r) : ref(r) {}
  void init(T &v) const { v = std::numeric_limits<T>::lowest(); }
  void join(T &a, const T &b) const { if (b > a) a = b; }
  T &reference() const { return ref; }
};
template <class T> struct Min {
  T &ref;
  explicit Min(T &r) : ref(r) {}
  void init(T &v) const { v = std::numeric_limits<T>::max(); }
  void join(T &a, const T &b) const { if (b < a) a = b; }
  T &reference() const { return ref; }
};
template <class T> struct Sum {
  T &ref;
  explicit Sum(T &r) : ref(r) {}
  void init(T &v) const { v = T(0); }
  void join(T &a, const T &b) const { a += b; }
  T &reference() const { return ref; }
};

namespace impl {
template <class F, class T, class... A>
void serial_reduce(const MDRangePolicy<Rank<2>, A...> &p, const F &f, T &acc) {
  for (long i = p.b[0]; i < p.e[0]; ++i)
    for (long j = p.b[1]; j < p.e[1]; ++j) f(static_cast<int>(i), static_cast<int>(j), acc);
}
template <class F, class T, class... A>
void serial_reduce(const MDRangePolicy<Rank<3>, A...> &p, const F &f, T &acc) {
  for (long i = p.b[0]; i < p.e[0]; ++i)
    for (long j = p.b[1]; j < p.e[1]; ++j)
      for (long k = p.b[2]; k < p.e[2]; ++k)
        f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k), acc);
}
template <class F, class T, class... A>
void serial_reduce(const RangePolicy<A...> &p, const F &f, T &acc) {
  for (long i = p.b; i < p.e; ++i) f(static_cast<int>(i), acc);
}
}  // namespace impl

template <class P, class F, class T>
void parallel_reduce(const std::string &, const P &p, const F &f, Max<T> r) {
  T acc;
  r.init(acc);
  impl::serial_reduce(p, f, acc);
  r.reference() = acc;
}
template <class P, class F, class T>
void parallel_reduce(const std::string &, const P &p, const F &f, Min<T> r) {
  T acc;
  r.init(acc);
  impl::serial_reduce(p, f, acc);
  r.reference() = acc;
}
template <class P, class F, class T>
void parallel_reduce(const std::string &, const P &p, const F &f, Sum<T> r) {
  T acc = T(0);
  impl::serial_reduce(p, f, acc);
  r.reference() = acc;
}
template <class P, class F, class T,
          typename std::enable_if<std::is_arithmetic<T>::value, int>::type = 0>
void parallel_reduce(const std::string &, const P &p, const F &f, T &result) {
  T acc = T(0);
  impl::serial_reduce(p, f, acc);
  result = acc;
}

}  // namespace Kokkos
