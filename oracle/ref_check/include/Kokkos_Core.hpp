// Kokkos_Core.hpp -- TEST INFRASTRUCTURE.  A minimal serial stand-in for the
// handful of Kokkos entry points used by the reference's hot-path headers
// (SimInfo.h, States.h, RiemannSolvers.h, Gravity.h, BoundaryConditions.h,
// Update.h, ThermalConduction.h, Viscosity.h, ComputeDt.h, Init.h).  It lets
// those headers compile unchanged with g++ so that their arithmetic can be run
// on the CPU and compared with the oracle.  Nothing here is Kokkos code; it is
// written for this repository and implements only these semantics (serial,
// or with OpenMP over rows when compiled with -fopenmp, to time the reference's
// own step code on the host cores):
//   - View<double***>: zero-initialised, shallow-copy (shared) storage,
//     operator()(i0, i1, i2) row-major;
//   - MDRangePolicy<Rank<2>>: [b0, e0) x [b1, e1), functor called as f(i0, i1);
//   - parallel_for / parallel_reduce with Max reducers or plain sum targets;
//   - deep_copy, create_mirror, Array<T, N>, math forwards.
// The reference kernels have no cross-iteration dependences, so serial order
// yields the same values as any parallel order.
#pragma once
#include <algorithm>
#include <array>
#include <cmath>
#include <cstddef>
#include <cstdint>
#include <iostream>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]

namespace Kokkos {

inline void initialize(int &, char **) {}
inline void finalize() {}

template <class T, std::size_t N>
struct Array {
  T m_data[N];
  T &operator[](std::size_t k) { return m_data[k]; }
  const T &operator[](std::size_t k) const { return m_data[k]; }
  static constexpr std::size_t size() { return N; }
};

template <class T>
class View;

namespace detail {
// Like Kokkos, views copied while a parallel dispatch runs do not take part in
// reference counting (the kernel's captured views keep the data alive): the
// copies the kernels make per cell then cost a pointer copy, not an atomic.
inline int &tracking_off() {
  static int off = 0;
  return off;
}
}  // namespace detail

template <class T>
class View<T ***> {
 public:
  View() = default;
  View(const std::string &, std::size_t n0, std::size_t n1, std::size_t n2)
      : owner_(std::make_shared<std::vector<T>>(n0 * n1 * n2, T(0))), p_(owner_->data()), n0_(n0), n1_(n1),
        n2_(n2) {}
  View(const View &o) : p_(o.p_), n0_(o.n0_), n1_(o.n1_), n2_(o.n2_) {
    if (!detail::tracking_off()) owner_ = o.owner_;
  }
  View &operator=(const View &o) {
    if (!detail::tracking_off()) owner_ = o.owner_;
    p_ = o.p_;
    n0_ = o.n0_;
    n1_ = o.n1_;
    n2_ = o.n2_;
    return *this;
  }
  T &operator()(std::size_t a, std::size_t b, std::size_t c) const { return p_[(a * n1_ + b) * n2_ + c]; }
  std::size_t extent(int k) const { return k == 0 ? n0_ : (k == 1 ? n1_ : n2_); }
  T *data() const { return p_; }
  std::size_t size() const { return n0_ * n1_ * n2_; }

 private:
  std::shared_ptr<std::vector<T>> owner_;
  T *p_ = nullptr;
  std::size_t n0_ = 0, n1_ = 0, n2_ = 0;
};

template <class V>
V create_mirror(const V &v) {
  return V("mirror", v.extent(0), v.extent(1), v.extent(2));
}
template <class V>
void deep_copy(const V &dst, const V &src) {
  std::copy(src.data(), src.data() + src.size(), dst.data());
}

template <int R>
struct Rank {};

template <class R>
struct MDRangePolicy;
template <>
struct MDRangePolicy<Rank<2>> {
  MDRangePolicy() = default;
  MDRangePolicy(std::array<long, 2> b, std::array<long, 2> e) : b_(b), e_(e) {}
  std::array<long, 2> b_{0, 0}, e_{0, 0};
};

template <class F>
void parallel_for(const std::string &, const MDRangePolicy<Rank<2>> &p, const F &f) {
  detail::tracking_off() = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
  for (long i1 = p.b_[1]; i1 < p.e_[1]; ++i1)
    for (long i0 = p.b_[0]; i0 < p.e_[0]; ++i0) f((int)i0, (int)i1);
  detail::tracking_off() = 0;
}

template <class T>
struct Max {
  T &ref;
  explicit Max(T &r) : ref(r) {}
  static T identity() { return std::numeric_limits<T>::lowest(); }
  static void join(T &dst, const T &src) {
    if (src > dst) dst = src;
  }
};

namespace detail {
template <class X>
struct is_max : std::false_type {};
template <class T>
struct is_max<Max<T>> : std::true_type {};

template <class X>
struct slot {  // plain lvalue target: sum reduction
  using value_type = std::remove_reference_t<X>;
  value_type local;
  value_type &target;
  explicit slot(X &t) : local(0), target(t) {}
  static value_type identity() { return value_type(0); }
  void join(const value_type &v) { local += v; }
  void finish() { target = local; }
};
template <class T>
struct slot<Max<T>> {
  using value_type = T;
  value_type local;
  T &target;
  explicit slot(Max<T> &m) : local(Max<T>::identity()), target(m.ref) {}
  static value_type identity() { return Max<T>::identity(); }
  void join(const value_type &v) { Max<T>::join(local, v); }
  void finish() { target = local; }
};
}  // namespace detail

template <class F, class A, class B, class C>
void parallel_reduce(const std::string &, const MDRangePolicy<Rank<2>> &p, const F &f, A &&a, B &&b, C &&c) {
  using SA = detail::slot<std::remove_cv_t<std::remove_reference_t<A>>>;
  using SB = detail::slot<std::remove_cv_t<std::remove_reference_t<B>>>;
  using SC = detail::slot<std::remove_cv_t<std::remove_reference_t<C>>>;
  SA sa(a);
  SB sb(b);
  SC sc(c);
  detail::tracking_off() = 1;
#ifdef _OPENMP
  // per-thread partial results joined at the end; the reductions used are
  // maxima and integer counts, which do not depend on the order
#pragma omp parallel
  {
    typename SA::value_type la = SA::identity();
    typename SB::value_type lb = SB::identity();
    typename SC::value_type lc = SC::identity();
#pragma omp for schedule(static)
    for (long i1 = p.b_[1]; i1 < p.e_[1]; ++i1)
      for (long i0 = p.b_[0]; i0 < p.e_[0]; ++i0) f((int)i0, (int)i1, la, lb, lc);
#pragma omp critical
    {
      sa.join(la);
      sb.join(lb);
      sc.join(lc);
    }
  }
#else
  for (long i1 = p.b_[1]; i1 < p.e_[1]; ++i1)
    for (long i0 = p.b_[0]; i0 < p.e_[0]; ++i0) f((int)i0, (int)i1, sa.local, sb.local, sc.local);
#endif
  detail::tracking_off() = 0;
  sa.finish();
  sb.finish();
  sc.finish();
}

template <class T>
inline T max(T a, T b) { return (a < b) ? b : a; }
template <class T>
inline T min(T a, T b) { return (b < a) ? b : a; }
inline double abs(double a) { return std::fabs(a); }
inline double sin(double a) { return std::sin(a); }
inline double cos(double a) { return std::cos(a); }
inline double tanh(double a) { return std::tanh(a); }
inline double exp(double a) { return std::exp(a); }
inline double sqrt(double a) { return std::sqrt(a); }

}  // namespace Kokkos
