// Minimal host-only stand-in for the Kokkos API surface used by the ppkMHD
// MUSCL-Hancock MHD functors (src/muscl/MHD*.h, src/shared/BoundariesFunctors.h,
// src/shared/RiemannSolvers_MHD.h, src/shared/mhd_utils.h).
//
// TEST INFRASTRUCTURE ONLY.  This header exists so that the reference's own,
// unmodified functor headers can be compiled with g++ into the CPU oracle
// (oracle/_ref/libppkmhd_ref.so).  Nothing in the product links against it.
//
// Semantics reproduced:
//   * View<T*...> with LayoutRight storage (last index fastest), reference
//     counted, zero-initialised on allocation (as Kokkos does);
//   * MDRangePolicy<Rank<N>> iterated with the last index fastest
//     (Kokkos' default Iterate::Right on host back-ends);
//   * parallel_for / parallel_reduce run SERIALLY by default, which fixes the
//     order of the reference's atomic_add / atomic_sub updates; setting
//     PPKMHD_SHIM_THREADS>1 in the environment parallelises the outermost
//     index with OpenMP (used only to time the reference on many cores);
//   * Max<T> reducer with identity = lowest();
//   * atomic_add / atomic_sub as OpenMP atomics.
#ifndef PPKMHD_KOKKOS_SHIM_CORE_HPP
#define PPKMHD_KOKKOS_SHIM_CORE_HPP

#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cstddef>
#include <limits>
#include <memory>
#include <ostream>
#include <iostream>
#include <sstream>
#include <string>
#include <type_traits>
#include <initializer_list>
#include <algorithm>

#include "Kokkos_Macros.hpp"

#ifdef _OPENMP
#  include <omp.h>
#endif

namespace Kokkos
{

// ---------------------------------------------------------------- spaces
struct HostSpace
{};
struct OpenMP
{};
using DefaultExecutionSpace = OpenMP;
using DefaultHostExecutionSpace = OpenMP;

inline void
initialize(int &, char **)
{}
inline void
initialize()
{}
inline void
finalize()
{}
inline void
fence()
{}
inline void
print_configuration(std::ostream & os, bool = false)
{
  os << "Kokkos API shim (host, serial by default)\n";
}
namespace hwloc
{
inline bool
available()
{
  return false;
}
inline unsigned
get_available_numa_count()
{
  return 1;
}
inline unsigned
get_available_cores_per_numa()
{
  return 1;
}
inline unsigned
get_available_threads_per_core()
{
  return 1;
}
} // namespace hwloc

// ---------------------------------------------------------------- Array
template <class T, size_t N>
struct Array
{
  T m_internal_implementation_private_member_data[N];
  KOKKOS_INLINE_FUNCTION T &
  operator[](size_t i)
  {
    return m_internal_implementation_private_member_data[i];
  }
  KOKKOS_INLINE_FUNCTION const T &
  operator[](size_t i) const
  {
    return m_internal_implementation_private_member_data[i];
  }
  static constexpr size_t
  size()
  {
    return N;
  }
  T *
  data()
  {
    return m_internal_implementation_private_member_data;
  }
};

// ---------------------------------------------------------------- View
namespace shim_detail
{
// Decompose a Kokkos data type like double***[3] into value type, number of
// runtime extents and the static trailing extents.
template <class T>
struct data_type_traits
{
  using value_type = T;
  static constexpr int dyn_rank = 0;
  static constexpr int static_rank = 0;
  static constexpr size_t static_extent(int) { return 1; }
};
template <class T>
struct data_type_traits<T *>
{
  using value_type = typename data_type_traits<T>::value_type;
  static constexpr int dyn_rank = data_type_traits<T>::dyn_rank + 1;
  static constexpr int static_rank = data_type_traits<T>::static_rank;
  static constexpr size_t static_extent(int r) { return data_type_traits<T>::static_extent(r); }
};
template <class T, size_t N>
struct data_type_traits<T[N]>
{
  using value_type = typename data_type_traits<T>::value_type;
  static constexpr int dyn_rank = data_type_traits<T>::dyn_rank;
  static constexpr int static_rank = data_type_traits<T>::static_rank + 1;
  // outermost static extent first
  static constexpr size_t static_extent(int r)
  {
    return r == 0 ? N : data_type_traits<T>::static_extent(r - 1);
  }
};
} // namespace shim_detail

template <class DataType, class... Props>
class View
{
  using traits = shim_detail::data_type_traits<DataType>;

public:
  using value_type = typename traits::value_type;
  using non_const_value_type = typename std::remove_const<value_type>::type;
  static constexpr int rank = traits::dyn_rank + traits::static_rank;
  using HostMirror = View<DataType, Props...>;

  View() = default;

  // Kokkos allows assignment between views of the same value type and total
  // rank whose static extents match at run time (e.g. real_t**** with a last
  // extent of 3 into real_t***[3]); the LayoutRight storage is identical.
  template <class D2, class... P2,
            class = typename std::enable_if<
              !std::is_same<View<D2, P2...>, View<DataType, Props...>>::value &&
              View<D2, P2...>::rank == shim_detail::data_type_traits<DataType>::dyn_rank +
                                         shim_detail::data_type_traits<DataType>::static_rank>::type>
  View(const View<D2, P2...> & o)
    : m_holder(o.m_holder)
    , m_ptr(o.m_ptr)
    , m_size(o.m_size)
    , m_label(o.m_label)
  {
    for (int q = 0; q < 8; ++q)
      m_ext[q] = o.m_ext[q];
  }

  template <class... Ints>
  View(const std::string & label, Ints... n)
  {
    static_assert(sizeof...(Ints) <= 8, "too many extents");
    size_t ext[8] = { static_cast<size_t>(n)... };
    init(label, ext, sizeof...(Ints));
  }

  KOKKOS_INLINE_FUNCTION size_t
  extent(int r) const
  {
    return r < rank ? m_ext[r] : 1;
  }
  KOKKOS_INLINE_FUNCTION int
  extent_int(int r) const
  {
    return static_cast<int>(extent(r));
  }
  size_t
  size() const
  {
    return m_size;
  }
  size_t
  span() const
  {
    return m_size;
  }
  value_type *
  data() const
  {
    return m_ptr;
  }
  const std::string &
  label() const
  {
    return m_label;
  }

  // LayoutRight indexing (last index fastest).
  KOKKOS_INLINE_FUNCTION value_type &
  operator()(int64_t i0) const
  {
    return m_ptr[i0];
  }
  KOKKOS_INLINE_FUNCTION value_type &
  operator()(int64_t i0, int64_t i1) const
  {
    return m_ptr[i0 * m_ext[1] + i1];
  }
  KOKKOS_INLINE_FUNCTION value_type &
  operator()(int64_t i0, int64_t i1, int64_t i2) const
  {
    return m_ptr[(i0 * m_ext[1] + i1) * m_ext[2] + i2];
  }
  KOKKOS_INLINE_FUNCTION value_type &
  operator()(int64_t i0, int64_t i1, int64_t i2, int64_t i3) const
  {
    return m_ptr[((i0 * m_ext[1] + i1) * m_ext[2] + i2) * m_ext[3] + i3];
  }

private:
  void
  init(const std::string & label, const size_t * n, int nargs)
  {
    m_label = label;
    int r = 0;
    for (; r < traits::dyn_rank; ++r)
      m_ext[r] = r < nargs ? n[r] : 1;
    for (int s = 0; s < traits::static_rank; ++s, ++r)
      m_ext[r] = traits::static_extent(s);
    m_size = 1;
    for (int q = 0; q < rank; ++q)
      m_size *= m_ext[q];
    // zero-initialised, as Kokkos::View allocations are
    value_type * p = static_cast<value_type *>(std::calloc(m_size ? m_size : 1, sizeof(value_type)));
    m_holder = std::shared_ptr<value_type>(p, [](value_type * q) { std::free(q); });
    m_ptr = p;
  }

  std::shared_ptr<value_type> m_holder;
  value_type *                m_ptr = nullptr;
  size_t                      m_ext[8] = { 1, 1, 1, 1, 1, 1, 1, 1 };
  size_t                      m_size = 0;
  std::string                 m_label;

  template <class D, class... P>
  friend class View;
};

template <class D, class... P>
typename View<D, P...>::HostMirror
create_mirror(const View<D, P...> & v)
{
  size_t e[4] = { v.extent(0), v.extent(1), v.extent(2), v.extent(3) };
  constexpr int dyn = shim_detail::data_type_traits<D>::dyn_rank;
  if constexpr (dyn == 1)
    return typename View<D, P...>::HostMirror(v.label(), e[0]);
  else if constexpr (dyn == 2)
    return typename View<D, P...>::HostMirror(v.label(), e[0], e[1]);
  else if constexpr (dyn == 3)
    return typename View<D, P...>::HostMirror(v.label(), e[0], e[1], e[2]);
  else
    return typename View<D, P...>::HostMirror(v.label(), e[0], e[1], e[2], e[3]);
}

template <class D, class... P>
typename View<D, P...>::HostMirror
create_mirror_view(const View<D, P...> & v)
{
  return v;
}

template <class D1, class... P1, class D2, class... P2>
void
deep_copy(const View<D1, P1...> & dst, const View<D2, P2...> & src)
{
  if (dst.data() == src.data())
    return;
  std::memcpy(dst.data(), src.data(), std::min(dst.size(), src.size()) * sizeof(*dst.data()));
}

template <class D, class... P>
void
deep_copy(const View<D, P...> & dst, const typename View<D, P...>::value_type & val)
{
  for (size_t n = 0; n < dst.size(); ++n)
    dst.data()[n] = val;
}

// ---------------------------------------------------------------- policies
template <unsigned N>
struct Rank
{
  static constexpr unsigned rank = N;
};

template <class... Args>
struct RangePolicy
{
  int64_t begin, end;
  RangePolicy(int64_t b, int64_t e)
    : begin(b)
    , end(e)
  {}
};

template <class RankT, class... Args>
struct MDRangePolicy
{
  static constexpr unsigned rank = RankT::rank;
  int64_t                   lo[3] = { 0, 0, 0 };
  int64_t                   hi[3] = { 1, 1, 1 };
  MDRangePolicy(std::initializer_list<int64_t> l, std::initializer_list<int64_t> h)
  {
    int q = 0;
    for (auto v : l)
      lo[q++] = v;
    q = 0;
    for (auto v : h)
      hi[q++] = v;
  }
};

namespace shim_detail
{
inline int
shim_threads()
{
  static int n = [] {
    const char * s = std::getenv("PPKMHD_SHIM_THREADS");
    int          v = s ? std::atoi(s) : 1;
    return v < 1 ? 1 : v;
  }();
  return n;
}
} // namespace shim_detail

template <class... A, class F>
void
parallel_for(const RangePolicy<A...> & p, const F & f)
{
  const int nt = shim_detail::shim_threads();
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
  for (int64_t i = p.begin; i < p.end; ++i)
    f(static_cast<int>(i));
}

template <class R, class... A, class F>
void
parallel_for(const MDRangePolicy<R, A...> & p, const F & f)
{
  const int nt = shim_detail::shim_threads();
  if constexpr (R::rank == 2)
  {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
      for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
        f(static_cast<int>(i), static_cast<int>(j));
  }
  else
  {
#pragma omp parallel for schedule(static) num_threads(nt) if (nt > 1)
    for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
      for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
        for (int64_t k = p.lo[2]; k < p.hi[2]; ++k)
          f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k));
  }
}

template <class P, class F>
void
parallel_for(const std::string &, const P & p, const F & f)
{
  parallel_for(p, f);
}

template <class T>
struct Max
{
  T & ref;
  explicit Max(T & r)
    : ref(r)
  {}
  static T
  identity()
  {
    return std::numeric_limits<T>::lowest();
  }
  static void
  join(T & a, const T & b)
  {
    if (b > a)
      a = b;
  }
};

template <class R, class... A, class F, class T>
void
parallel_reduce(const MDRangePolicy<R, A...> & p, const F & f, const Max<T> & red)
{
  const int nt = shim_detail::shim_threads();
  T         result = Max<T>::identity();
#pragma omp parallel num_threads(nt) if (nt > 1)
  {
    T local = Max<T>::identity();
    if constexpr (R::rank == 2)
    {
#pragma omp for schedule(static)
      for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
        for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
          f(static_cast<int>(i), static_cast<int>(j), local);
    }
    else
    {
#pragma omp for schedule(static)
      for (int64_t i = p.lo[0]; i < p.hi[0]; ++i)
        for (int64_t j = p.lo[1]; j < p.hi[1]; ++j)
          for (int64_t k = p.lo[2]; k < p.hi[2]; ++k)
            f(static_cast<int>(i), static_cast<int>(j), static_cast<int>(k), local);
    }
#pragma omp critical
    Max<T>::join(result, local);
  }
  red.ref = result;
}

template <class P, class F, class Red>
void
parallel_reduce(const std::string &, const P & p, const F & f, const Red & r)
{
  parallel_reduce(p, f, r);
}

// ---------------------------------------------------------------- atomics
template <class T>
KOKKOS_INLINE_FUNCTION void
atomic_add(T * p, const T v)
{
#pragma omp atomic
  *p += v;
}
template <class T>
KOKKOS_INLINE_FUNCTION void
atomic_sub(T * p, const T v)
{
#pragma omp atomic
  *p -= v;
}

} // namespace Kokkos

#include "Kokkos_MathematicalFunctions.hpp"

#endif // PPKMHD_KOKKOS_SHIM_CORE_HPP
