/*
 * FP64 operation counter of the reference's MUSCL-Hancock + HLLD + CT step.
 *
 * TEST / MEASUREMENT INFRASTRUCTURE ONLY.  Compiles the C restatement
 * mhd_oracle.c (the reference's operation order, bitwise equal to the
 * reference) as C++ with `double` replaced by a counting scalar type, so
 * every floating-point operation the reference algorithm performs is
 * tallied per stage (ORC_STAGE markers in mhd_oracle.c):
 *   add  additions and subtractions      mul   multiplications
 *   div  divisions                       sqrt  square roots
 *   cmp  comparisons, fmin and fmax (selections; no arithmetic result)
 * Negation, fabs and copysign are sign-bit operations and are not counted.
 * The counts give the algorithmic FP64 work per cell-update of the plain
 * FP64 path (the denominator of its FP64-arithmetic roofline).
 *
 * Built by oracle/Makefile into build/libflop_count.so; driven by
 * oracle/flop_count.py.
 */
#include <cctype>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>
#ifdef _OPENMP
#  include <omp.h>
#endif

enum
{
  OP_ADD = 0,
  OP_MUL,
  OP_DIV,
  OP_SQRT,
  OP_CMP,
  OP_KINDS
};
static const int kStages = 10;
static uint64_t  g_ops[kStages][OP_KINDS];
static int       g_stage = 0;

static inline void
tally(int op)
{
  g_ops[g_stage][op]++;
}

// One FP64 value whose operations are counted.  Same size and alignment as
// double, so arrays of it are the oracle's double arrays.
struct CD
{
  double v;
  CD() = default;
  CD(double x) : v(x) {}
  CD &
  operator+=(CD o)
  {
    tally(OP_ADD);
    v += o.v;
    return *this;
  }
  CD &
  operator-=(CD o)
  {
    tally(OP_ADD);
    v -= o.v;
    return *this;
  }
  CD &
  operator*=(CD o)
  {
    tally(OP_MUL);
    v *= o.v;
    return *this;
  }
  CD &
  operator/=(CD o)
  {
    tally(OP_DIV);
    v /= o.v;
    return *this;
  }
  CD
  operator-() const
  {
    return CD(-v);
  }
  CD
  operator+() const
  {
    return *this;
  }
  explicit operator int() const { return (int)v; }
  explicit operator float() const { return (float)v; }
};
static_assert(sizeof(CD) == sizeof(double), "counting type must alias double");

#define CD_BIN(OP, KIND)                                                                  \
  static inline CD operator OP(CD a, CD b)                                                \
  {                                                                                        \
    tally(KIND);                                                                           \
    return CD(a.v OP b.v);                                                                 \
  }                                                                                        \
  static inline CD operator OP(CD a, double b)                                            \
  {                                                                                        \
    tally(KIND);                                                                           \
    return CD(a.v OP b);                                                                   \
  }                                                                                        \
  static inline CD operator OP(double a, CD b)                                            \
  {                                                                                        \
    tally(KIND);                                                                           \
    return CD(a OP b.v);                                                                   \
  }
CD_BIN(+, OP_ADD)
CD_BIN(-, OP_ADD)
CD_BIN(*, OP_MUL)
CD_BIN(/, OP_DIV)
#undef CD_BIN

#define CD_CMP(OP)                                                                        \
  static inline bool operator OP(CD a, CD b)                                              \
  {                                                                                        \
    tally(OP_CMP);                                                                         \
    return a.v OP b.v;                                                                     \
  }                                                                                        \
  static inline bool operator OP(CD a, double b)                                          \
  {                                                                                        \
    tally(OP_CMP);                                                                         \
    return a.v OP b;                                                                       \
  }                                                                                        \
  static inline bool operator OP(double a, CD b)                                          \
  {                                                                                        \
    tally(OP_CMP);                                                                         \
    return a OP b.v;                                                                       \
  }
CD_CMP(<)
CD_CMP(>)
CD_CMP(<=)
CD_CMP(>=)
CD_CMP(==)
CD_CMP(!=)
#undef CD_CMP

static inline CD
sqrt(CD a)
{
  tally(OP_SQRT);
  return CD(std::sqrt(a.v));
}
static inline CD
fabs(CD a)
{
  return CD(std::fabs(a.v));
}
static inline CD
copysign(CD a, CD b)
{
  return CD(std::copysign(a.v, b.v));
}
static inline CD
fmax(CD a, CD b)
{
  tally(OP_CMP);
  return CD(std::fmax(a.v, b.v));
}
static inline CD
fmin(CD a, CD b)
{
  tally(OP_CMP);
  return CD(std::fmin(a.v, b.v));
}
static inline CD
nextafter(CD a, double b)
{
  return CD(std::nextafter(a.v, b));
}
static inline CD
sin(CD a)
{
  return CD(std::sin(a.v));
}
static inline CD
cos(CD a)
{
  return CD(std::cos(a.v));
}

#define ORC_STAGE(s) (g_stage = (s))
#define double CD
#include "mhd_oracle.c"
#undef double

extern "C"
{
  // Counters of stage s (STG_* of mhd_oracle.c): out[OP_KINDS].
  void
  flop_counts(int s, uint64_t * out)
  {
    for (int k = 0; k < OP_KINDS; ++k)
      out[k] = (s >= 0 && s < kStages) ? g_ops[s][k] : 0;
  }
  void
  flop_reset(void)
  {
    std::memset(g_ops, 0, sizeof g_ops);
    g_stage = 0;
  }
  int
  flop_stage_count(void)
  {
    return STG_COUNT;
  }
}
