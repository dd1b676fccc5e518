// Kokkos math-constant header stand-in (test infrastructure only).
#ifndef PPKMHD_KOKKOS_SHIM_CONST_HPP
#define PPKMHD_KOKKOS_SHIM_CONST_HPP
#include "Kokkos_Core.hpp"
#endif
