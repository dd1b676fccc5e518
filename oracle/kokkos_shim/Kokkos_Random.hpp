// Stand-in for Kokkos_Random.hpp: a 64-bit xorshift pool with the interface
// used by the reference's Kelvin-Helmholtz initial condition.  Only needed so
// that the reference init headers compile; the oracle never draws from it for
// the Orszag-Tang problems (test infrastructure only).
#ifndef PPKMHD_KOKKOS_SHIM_RANDOM_HPP
#define PPKMHD_KOKKOS_SHIM_RANDOM_HPP
#include <cstdint>
#include "Kokkos_Core.hpp"
namespace Kokkos
{
template <class Space>
class Random_XorShift64_Pool
{
public:
  struct generator_type
  {
    uint64_t s;
    uint64_t
    urand64()
    {
      s ^= s << 13;
      s ^= s >> 7;
      s ^= s << 17;
      return s;
    }
    double
    drand()
    {
      return (urand64() >> 11) * (1.0 / 9007199254740992.0);
    }
    double
    drand(double a, double b)
    {
      return a + (b - a) * drand();
    }
  };
  Random_XorShift64_Pool() = default;
  explicit Random_XorShift64_Pool(uint64_t seed)
    : m_seed(seed ? seed : 0x9E3779B97F4A7C15ull)
  {}
  generator_type
  get_state() const
  {
    return generator_type{ m_seed };
  }
  void
  free_state(const generator_type &) const
  {}

private:
  uint64_t m_seed = 0x9E3779B97F4A7C15ull;
};
} // namespace Kokkos
#endif
