// Kokkos math-function stand-ins: thin aliases of the IEEE <cmath> functions
// (test infrastructure only).
#ifndef PPKMHD_KOKKOS_SHIM_MATH_HPP
#define PPKMHD_KOKKOS_SHIM_MATH_HPP
#include <cmath>
#include <cstdlib>
namespace Kokkos
{
using std::abs;
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::fmod;
using std::isnan;
using std::sqrt;
using std::sin;
using std::cos;
namespace Experimental
{
using std::exp;
using std::fabs;
using std::fmax;
using std::fmin;
using std::fmod;
using std::isnan;
using std::sqrt;
} // namespace Experimental
} // namespace Kokkos
#endif
