// Kokkos macro stand-ins for the host-only API shim (test infrastructure only).
#ifndef PPKMHD_KOKKOS_SHIM_MACROS_HPP
#define PPKMHD_KOKKOS_SHIM_MACROS_HPP
#define KOKKOS_VERSION_MAJOR 4
#define KOKKOS_VERSION 40000
#define KOKKOS_ENABLE_CXX17
#define KOKKOS_ENABLE_OPENMP
#define KOKKOS_INLINE_FUNCTION inline
#define KOKKOS_FORCEINLINE_FUNCTION inline
#define KOKKOS_FUNCTION
#define KOKKOS_LAMBDA [=]
#define KOKKOS_ASSERT(cond) ((void)0)
#endif
