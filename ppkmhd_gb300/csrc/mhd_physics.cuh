// Point-wise MHD physics of the MUSCL-Hancock + HLLD + CT step, as device
// functions templated on the real type R (double or float).
//
// Each function keeps the operation order of the reference expression it
// implements (cited per function), so that a build without FMA contraction
// (nvcc --fmad=false, MHD_FP_EXACT) reproduces a serial CPU run of the
// reference bit for bit.  The fast build lets nvcc contract multiply-adds.
#pragma once

#include <cstdint>

#ifndef MHD_VARIANT_TAG
#  define MHD_VARIANT_TAG v_default
#endif

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

enum : int
{
  ID = 0,
  IP = 1,
  IU = 2,
  IV = 3,
  IW = 4,
  IA = 5,
  IB = 6,
  IC = 7,
  NV = 8
};

enum : int
{
  RIEMANN_LLF = 1,
  RIEMANN_HLL = 2,
  RIEMANN_HLLD = 4
};

template <class R>
struct State
{
  R v[NV];
  __device__ __forceinline__ R &
  operator[](int i)
  {
    return v[i];
  }
  __device__ __forceinline__ const R &
  operator[](int i) const
  {
    return v[i];
  }
};

template <class R>
__device__ __forceinline__ void
swap_vals(R & a, R & b)
{
  R t = a;
  a = b;
  b = t;
}

// MHD_EXACT_BUILD = 1 (the FMA-free FP64 build) evaluates every expression in
// the reference's operation order.  The other builds use algebraically equal
// forms with fewer divides and square roots (shared reciprocals, rsqrt for
// |B|/sqrt(rho)); they differ from the reference at round-off level only.
#ifndef MHD_EXACT_BUILD
#  define MHD_EXACT_BUILD 0
#endif
constexpr bool kExactOrder = MHD_EXACT_BUILD != 0;

// Reciprocal, reciprocal square root and square root of the fast builds
// (GB300 issues 2 FP64 FMAs per SM per cycle, so FP64 operation counts set
// the speed of the FP64 kernels).
//  * FP64 reciprocal: the hardware approximation rcp.approx.ftz.f64 (relative
//    error below 2^-18 on 1e6 log-uniform samples) refined by one third-order
//    Newton step y (1 + e + e^2), e = 1 - x y, whose relative error is e^3:
//    at most 0.51 ulp (99.97 % of the samples correctly rounded) in 3 FMAs,
//    against 5 FP64 operations for the correctly rounded library reciprocal.
//    Arguments whose reciprocal is not a normal number (zero, subnormal,
//    |x| >= 2^1021, infinite, NaN) take the library reciprocal.
//  * FP64 rsqrt: the library's (within 0.51 ulp; 5 FP64 operations).
//  * FP64 square root: x times the hardware approximation
//    rsqrt.approx.ftz.f64 (relative error below 2^-20), refined by one
//    third-order correction, for positive normal x: within 0.76 ulp in 5
//    FP64 operations against 8 for the IEEE square root; other arguments
//    take the IEEE square root.
//  * FP32: the hardware approximations alone (about 1 ulp).
__device__ __forceinline__ double
rcp(double x)
{
  const unsigned ex = ((unsigned)__double2hiint(x) >> 20) & 0x7ffu;
  if (ex - 1u < 0x7fbu) // 1 <= biased exponent <= 0x7fb: 2^-1022 <= |x| < 2^1021
  {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
  }
  return __drcp_rn(x);
}
__device__ __forceinline__ float
rcp(float x)
{
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ double
rsq(double x)
{
  return rsqrt(x);
}
__device__ __forceinline__ float
rsq(float x)
{
  float y;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float
fsqrt(float x)
{
  if (x > 0.f && x < INFINITY)
    return x * rsq(x);
  return sqrtf(x);
}
// Square root of a positive normal double from the rsqrt.approx.ftz.f64 seed
// y ~ x^-1/2: s = x y and e = 1 - s y (= 1 - x y^2 up to one rounding), then
// one third-order Householder correction s (1 + e/2 + 3e^2/8), the Taylor
// series of (1 - e)^-1/2 to second order: 5 FP64 operations (x * rsqrt(x)
// takes 6).  Zero, subnormal, negative, infinite and NaN arguments go to sqrt.
__device__ __forceinline__ double
fsqrt(double x)
{
  const unsigned se = (unsigned)__double2hiint(x) >> 20; // sign and biased exponent
  if (se - 1u < 0x7feu)                                  // positive, exponent 1 .. 0x7fe
  {
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double s = x * y;
    const double e = fma(-s, y, 1.0);
    return fma(s * e, fma(e, 0.375, 0.5), s);
  }
  return sqrt(x);
}

// Correctly rounded FP64 quotients that share a denominator, for the
// FMA-free build (whose every operation must round as the reference's):
// y = RN(1/b) from the library's correctly rounded reciprocal, then per
// quotient q0 = a y and two corrections q + (a - b q) y, each with the exact
// FMA remainder.  Markstein's theorem (P. W. Markstein, IBM J. Res. Dev. 34,
// 1990; M. Cornea, J. Harrison, P. T. P. Tang, Scientific Computing on
// Itanium-based Systems, 2002): with y = RN(1/b) and q a faithful quotient,
// RN(q + (a - b q) y) = RN(a / b); the first correction makes q0 (within
// 1.5 ulp) faithful.  Equal to the IEEE quotient bit for bit (checked against
// it on 1.3e8 operand pairs: random magnitudes and signs, quotients near 1,
// all-ones mantissas, exact quotients, signed zeros, random bit patterns).
// Operands whose exponents lie within 100 of either end of the range or
// differ by more than 800 (zeros, subnormals, huge values, inf, NaN) take
// a / b itself; a zero numerator over a normal denominator gives a y, the
// IEEE signed zero.  5 FP64 operations per quotient and one reciprocal per
// denominator, against about 1.3 times that for each IEEE division.
__device__ __forceinline__ double
qrcp(double b)
{
  return __drcp_rn(b);
}
__device__ __forceinline__ double
qdiv(double a, double b, double y)
{
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7ffu;
  const unsigned eb = ((unsigned)__double2hiint(b) >> 20) & 0x7ffu;
  const double   q0 = a * y;
  if (ea - 100u > 1846u || eb - 100u > 1846u || (int)ea - (int)eb > 800 ||
      (int)eb - (int)ea > 800)
    return (a == 0.0 && eb - 1u < 2045u) ? q0 : a / b;
  const double r0 = fma(-b, q0, a);
  const double q1 = fma(r0, y, q0);
  const double r1 = fma(-b, q1, a);
  return fma(r1, y, q1);
}
// FP32 code paths divide directly
__device__ __forceinline__ float
qrcp(float)
{
  return 0.f;
}
__device__ __forceinline__ float
qdiv(float a, float b, float)
{
  return a / b;
}

// Round-to-nearest add, subtract and multiply that the compiler never
// contracts into fused multiply-adds: values computed with them are the same
// bits in every kernel that evaluates them.
__device__ __forceinline__ double
rn_add(double a, double b)
{
  return __dadd_rn(a, b);
}
__device__ __forceinline__ float
rn_add(float a, float b)
{
  return __fadd_rn(a, b);
}
__device__ __forceinline__ double
rn_sub(double a, double b)
{
  return __dsub_rn(a, b);
}
__device__ __forceinline__ float
rn_sub(float a, float b)
{
  return __fsub_rn(a, b);
}
__device__ __forceinline__ double
rn_mul(double a, double b)
{
  return __dmul_rn(a, b);
}
__device__ __forceinline__ float
rn_mul(float a, float b)
{
  return __fmul_rn(a, b);
}

// Selection by comparison.  GB300 runs FP64 comparisons on the narrow FP64
// pipe; the FP64 builds compare the bit patterns as integers instead, on the
// integer pipes.  The fast build's key(x) = bits ^ ((bits >> 63) & 0x7fff...)
// orders like the values for non-NaN doubles, with -0 below +0.  The exact
// build must select exactly what the reference's FP comparison selects
// (mhd_utils.h:36-77) for every input, so its key is the signed magnitude
// (-0 and +0 equal) and a NaN operand makes the comparison false, as the FP
// comparison is.
__device__ __forceinline__ long long
order_key(double x)
{
  const long long b = __double_as_longlong(x);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
// (a > r) and (a < r) of IEEE doubles, bit for bit, on integer operations
__device__ __forceinline__ bool
exact_gt(double a, double r)
{
  const long long ba = __double_as_longlong(a), br = __double_as_longlong(r);
  const long long ma = ba & 0x7fffffffffffffffLL, mr = br & 0x7fffffffffffffffLL;
  const long long inf = 0x7ff0000000000000LL;
  if (ma > inf || mr > inf)
    return false; // a NaN operand
  return (ba < 0 ? -ma : ma) > (br < 0 ? -mr : mr);
}
template <class R>
__device__ __forceinline__ R
sel_max(R r, R a)
{
  if constexpr (sizeof(R) == 8 && !kExactOrder)
    return order_key(a) > order_key(r) ? a : r;
  else if constexpr (sizeof(R) == 8)
    return exact_gt(a, r) ? a : r;
  else
    return (a > r) ? a : r;
}
template <class R>
__device__ __forceinline__ R
sel_min(R r, R a)
{
  if constexpr (sizeof(R) == 8 && !kExactOrder)
    return order_key(a) < order_key(r) ? a : r;
  else if constexpr (sizeof(R) == 8)
    return exact_gt(r, a) ? a : r;
  else
    return (a < r) ? a : r;
}
template <class R>
__device__ __forceinline__ R
max4(R a0, R a1, R a2, R a3)
{
  return sel_max(sel_max(sel_max(a0, a1), a2), a3);
}
template <class R>
__device__ __forceinline__ R
min4(R a0, R a1, R a2, R a3)
{
  return sel_min(sel_min(sel_min(a0, a1), a2), a3);
}
template <class R>
__device__ __forceinline__ R
max5(R a0, R a1, R a2, R a3, R a4)
{
  return sel_max(sel_max(sel_max(sel_max(a0, a1), a2), a3), a4);
}
// max5(|n0|/sqrt(r0), ..., |n3|/sqrt(r3), smallc) of IEEE quotients and
// square roots, bit for bit, with one quotient and one square root instead
// of four of each.  Approximate ratios t_i = |n_i| rsqrt(r_i) (the library
// rsqrt, within 1 ulp: |t_i / (|n_i| / sqrt(r_i)) - 1| <= 3.4e-16) bracket
// the rounded ratios q_i = RN(|n_i| / RN(sqrt(r_i))) (|q_i / (|n_i| /
// sqrt(r_i)) - 1| <= 2.3e-16), so when the largest t_j exceeds every other
// t_i by more than the relative margin 4e-15, q_j is the largest q and is
// the only one computed; a contender within the margin with the same
// operands (the same bits) is the same value.  Other contenders, and
// operands outside the ranges where those bounds hold (r not a positive
// double in [2^-900, 2^900], |n| not 0 or in [2^-500, 2^500)), take the four
// IEEE quotients.  The result is the max5 chain of sel_max on the q_i.
__device__ __forceinline__ bool
alfven_operands_ok(double n, double r)
{
  const unsigned hr = (unsigned)__double2hiint(r), hn = (unsigned)__double2hiint(n) & 0x7fffffffu;
  const unsigned er = hr >> 20, en = hn >> 20;
  return er - 0x07bu <= 0x708u && (en - 0x20bu <= 0x3e7u || (hn | (unsigned)__double2loint(n)) == 0u);
}
__device__ __forceinline__ double
alfven_max5_exact(double n0, double r0, double n1, double r1, double n2, double r2, double n3,
                  double r3, double smallc)
{
  const double n[4] = { fabs(n0), fabs(n1), fabs(n2), fabs(n3) };
  const double r[4] = { r0, r1, r2, r3 };
  bool         ok = true;
#pragma unroll
  for (int i = 0; i < 4; ++i)
    ok = ok && alfven_operands_ok(n[i], r[i]);
  if (ok)
  {
    double t[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      t[i] = n[i] * rsqrt(r[i]);
    int j = 0;
#pragma unroll
    for (int i = 1; i < 4; ++i)
      j = t[i] > t[j] ? i : j;
    const double lim = t[j] * (1.0 - 4e-15);
    bool         amb = false;
#pragma unroll
    for (int i = 0; i < 4; ++i)
      amb = amb || (i != j && t[i] >= lim &&
                    (__double_as_longlong(n[i]) != __double_as_longlong(n[j]) ||
                     __double_as_longlong(r[i]) != __double_as_longlong(r[j])));
    if (!amb)
    {
      const double q = n[j] / sqrt(r[j]);
      return exact_gt(smallc, q) ? smallc : q;
    }
  }
  // the chain of the exact build's sel_max (exact_gt): max5 of the quotients
  double m = n[0] / sqrt(r[0]);
#pragma unroll
  for (int i = 1; i < 4; ++i)
  {
    const double q = n[i] / sqrt(r[i]);
    m = exact_gt(q, m) ? q : m;
  }
  return exact_gt(smallc, m) ? smallc : m;
}

// Sign tests and |d| <= t (t >= 0) of the fast FP64 build on bit patterns
// (integer pipe).  They agree with the FP comparisons for every non-NaN
// argument, -0 included.
template <class R>
__device__ __forceinline__ bool
gt0(R x)
{
  if constexpr (sizeof(R) == 8 && !kExactOrder)
    return __double_as_longlong(x) > 0;
  else
    return x > R(0);
}
template <class R>
__device__ __forceinline__ bool
ge0(R x)
{
  if constexpr (sizeof(R) == 8 && !kExactOrder)
  {
    const long long b = __double_as_longlong(x);
    return b >= 0 || (b & 0x7fffffffffffffffLL) == 0;
  }
  else
    return x >= R(0);
}
template <class R>
__device__ __forceinline__ bool
abs_le(R d, R t)
{
  if constexpr (sizeof(R) == 8 && !kExactOrder)
    return (__double_as_longlong(d) & 0x7fffffffffffffffLL) <= __double_as_longlong(t);
  else
    return fabs(d) <= t;
}


// Squares of both fast magnetosonic speeds (normal field in slot IA, then in
// slot IB) of one state with one reciprocal of the density
// (mhd_utils.h:89-117).  The callers take the square root of the largest
// only: the square root is monotone, so max_i sqrt(x_i) = sqrt(max_i x_i)
// (exactly for a correctly rounded root, within the 0.76 ulp of fsqrt).
template <class R>
__device__ __forceinline__ void
fast_speeds2_xy(const State<R> & q, R gamma0, R & cfx2, R & cfy2)
{
  const R invd = rcp(q[ID]);
  const R a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * q[IP] * invd;
  const R d2 = R(0.5) * (b2 * invd + c2);
  const R cd = c2 * invd;
  cfx2 = d2 + fsqrt(d2 * d2 - cd * a * a);
  cfy2 = d2 + fsqrt(d2 * d2 - cd * b * b);
}

// Fast magnetosonic speed with the normal field in slot IA
// (find_speed_fast<IX>, mhd_utils.h:89-117).
template <class R>
__device__ __forceinline__ R
fast_speed_x(const State<R> & q, R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
}

// Squared fast speeds in the same operation order (everything under the
// outer square root of fast_speed_x / fast_speed_y).  (The three quotients
// over d with one shared reciprocal, qdiv, measured 2 % slower in the exact
// 2D HLLD, whose x and y calls on one state share two of them already.)  The IEEE square root
// is correctly rounded and non-decreasing, so the maximum of the square roots
// of several such values is the square root of their maximum, bit for bit
// (a NaN, from a slightly negative inner argument, is skipped or kept by the
// same comparisons before and after the root).
template <class R>
__device__ __forceinline__ R
fast_speed2_x(const State<R> & q, R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  return d2 + sqrt(d2 * d2 - c2 * a * a / d);
}
template <class R>
__device__ __forceinline__ R
fast_speed2_y(const State<R> & q, R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  return d2 + sqrt(d2 * d2 - c2 * b * b / d);
}

// Same with the normal field in slot IB (find_speed_fast<IY>).
template <class R>
__device__ __forceinline__ R
fast_speed_y(const State<R> & q, R gamma0)
{
  const R d = q[ID], p = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const R b2 = a * a + b * b + c * c;
  const R c2 = gamma0 * p / d;
  const R d2 = R(0.5) * (b2 / d + c2);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
}

// MC-type limited slope of one variable from its two neighbours
// (slope_unsplit_hydro_2d_scalar, MHDBaseFunctor2D.h:370-383; the same
// statement sequence as compute_limited_slope, MHDBaseFunctor2D.h:129-155).
template <class R>
__device__ __forceinline__ R
limited_slope(R q, R qp, R qm, R slope_type)
{
  const R dlft = slope_type * (q - qm);
  const R drgt = slope_type * (qp - q);
  const R dcen = R(0.5) * (qp - qm);
  const R dsgn = (dcen >= R(0)) ? R(1) : R(-1);
  const R slop = fmin(fabs(dlft), fabs(drgt));
  R       dlim = slop;
  if ((dlft * drgt) <= R(0))
    dlim = R(0);
  return dsgn * fmin(dlim, fabs(dcen));
}

// The same limiter with the comparisons, minima and the sign transfer done
// on IEEE bit patterns (integer pipe): magnitudes of doubles order like their
// bit patterns, and the scalings by slope_type (1 or 2) and by 1/2 are exact,
// so the result equals limited_slope except for the sign of a zero result and
// when a product underflows.  5 floating-point operations instead of 11
// (3 in FP64).
__device__ __forceinline__ long long
fbits(double x)
{
  return __double_as_longlong(x);
}
__device__ __forceinline__ int
fbits(float x)
{
  return __float_as_int(x);
}
__device__ __forceinline__ double
from_fbits(long long b, double)
{
  return __longlong_as_double(b);
}
__device__ __forceinline__ float
from_fbits(int b, float)
{
  return __int_as_float(b);
}

template <class R>
__device__ __forceinline__ R
limited_slope_bits(R q, R qp, R qm, R slope_type)
{
  const R a = q - qm, b = qp - q, c = qp - qm;
  const auto ia = fbits(a), ib = fbits(b);
  using I = decltype(ia);
  const I sign = I(1) << (sizeof(I) * 8 - 1);
  const I aa = ia & ~sign, ab = ib & ~sign;
  // dlft * drgt <= 0: opposite signs or a zero
  if (((ia ^ ib) & sign) != 0 || aa == 0 || ab == 0)
    return R(0);
  if constexpr (sizeof(R) == 8)
  {
    // FP64: the doubling and the halving on the exponent field too, so the
    // limiter costs 3 FP64 operations.  Exact for normal numbers; 2m
    // saturates at infinity and |c|/2 below 2^-1022 is taken as zero.
    constexpr long long one = 1LL << 52, inf = 0x7ff0000000000000LL;
    long long mb = aa < ab ? aa : ab;
    if (fbits(slope_type) == fbits(R(2)))
      mb = mb < one ? (mb << 1) : (mb + one < inf ? mb + one : inf);
    const long long cb = fbits(c) & ~sign;
    const long long hc = cb >= 2 * one ? cb - one : 0;
    const long long r = mb < hc ? mb : hc;
    return from_fbits(r | (fbits(c) & sign), R(0));
  }
  else
  {
    R m = from_fbits(aa < ab ? aa : ab, R(0));
    if (slope_type == R(2))
      m = m + m;
    const I hc = fbits(R(0.5) * c) & ~sign;
    const I mb = fbits(m);
    const I r = mb < hc ? mb : hc;
    return from_fbits(r | (fbits(c) & sign), R(0));
  }
}

template <class R>
__device__ __forceinline__ R
slope_limited(R q, R qp, R qm, R slope_type)
{
  if constexpr (kExactOrder)
    return limited_slope(q, qp, qm, slope_type);
  else
    return limited_slope_bits(q, qp, qm, slope_type);
}

// Conservative variables and 1D flux of a primitive state
// (find_mhd_flux, mhd_utils.h:173-231; isothermal branch inactive).
template <class R>
__device__ __forceinline__ void
mhd_flux_and_cons(const State<R> & q, State<R> & u, State<R> & f, R gamma0)
{
  const R p = q[IP];
  const R entho = R(1) / (gamma0 - R(1));
  const R d = q[ID], vu = q[IU], vv = q[IV], vw = q[IW], a = q[IA], b = q[IB], c = q[IC];
  const R ecin = R(0.5) * (vu * vu + vv * vv + vw * vw) * d;
  const R emag = R(0.5) * (a * a + b * b + c * c);
  const R etot = p * entho + ecin + emag;
  const R ptot = p + emag;
  u[ID] = d;
  u[IP] = etot;
  u[IU] = d * vu;
  u[IV] = d * vv;
  u[IW] = d * vw;
  u[IA] = a;
  u[IB] = b;
  u[IC] = c;
  f[ID] = d * vu;
  f[IP] = (etot + ptot) * vu - a * (a * vu + b * vv + c * vw);
  f[IU] = d * vu * vu - a * a + ptot;
  f[IV] = d * vu * vv - a * b;
  f[IW] = d * vu * vw - a * c;
  f[IA] = R(0);
  f[IB] = b * vu - a * vv;
  f[IC] = c * vu - a * vw;
}

// HLL (riemann_hll, RiemannSolvers_MHD.h:27-67).
template <class R>
__device__ void
riemann_hll(State<R> & ql, State<R> & qr, State<R> & flux, R gamma0)
{
  const R bx_mean = R(0.5) * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  State<R> ul, fl, ur, fr;
  mhd_flux_and_cons(ql, ul, fl, gamma0);
  mhd_flux_and_cons(qr, ur, fr, gamma0);
  // fmax(cfl, cfr) as the root of the larger square (fast_speed2_x)
  const R cfm = sqrt(fmax(fast_speed2_x(ql, gamma0), fast_speed2_x(qr, gamma0)));
  const R vl = ql[IU], vr = qr[IU];
  const R sl = fmin(fmin(vl, vr) - cfm, R(0));
  const R sr = fmax(fmax(vl, vr) + cfm, R(0));
#pragma unroll
  for (int v = 0; v < NV; ++v)
    flux[v] = (sr * fl[v] - sl * fr[v] + sr * sl * (ur[v] - ul[v])) / (sr - sl);
}

// Local Lax-Friedrichs (riemann_llf, RiemannSolvers_MHD.h:81-111) with the
// fastest x information speed (find_speed_info, mhd_utils.h:374-401).
template <class R>
__device__ void
riemann_llf(State<R> & ql, State<R> & qr, State<R> & flux, R gamma0)
{
  const R bx_mean = R(0.5) * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  State<R> ul, fl, ur, fr;
  mhd_flux_and_cons(ql, ul, fl, gamma0);
  mhd_flux_and_cons(qr, ur, fr, gamma0);
#pragma unroll
  for (int v = 0; v < NV; ++v)
    flux[v] = (fl[v] + fr[v]) / R(2);
  const R cl = fast_speed_x(ql, gamma0) + fabs(ql[IU]);
  const R cr = fast_speed_x(qr, gamma0) + fabs(qr[IU]);
  const R vel = fmax(cl, cr);
#pragma unroll
  for (int v = 0; v < NV; ++v)
    flux[v] -= vel * (ur[v] - ul[v]) / R(2);
}

// HLLD of Miyoshi & Kusano (2005) in the RAMSES/DUMSES form
// (riemann_hlld, RiemannSolvers_MHD.h:133-367).  States are in the
// face-normal frame (normal velocity IU, normal field IA).
template <class R>
__device__ void
riemann_hlld(State<R> & ql, State<R> & qr, State<R> & flux, R gamma0, R entho)
{
  // entho = 1 / (gamma0 - 1), the caller's IEEE quotient (the same bits as
  // the reference's per-call division)
  const R a = R(0.5) * (ql[IA] + qr[IA]);
  const R sgnm = (a >= R(0)) ? R(1) : R(-1);
  ql[IA] = a;
  qr[IA] = a;

  const R rl = ql[ID], pl = ql[IP], ul = ql[IU], vl = ql[IV], wl = ql[IW], bl = ql[IB],
          cl = ql[IC];
  const R ecinl = R(0.5) * (ul * ul + vl * vl + wl * wl) * rl;
  const R emagl = R(0.5) * (a * a + bl * bl + cl * cl);
  const R etotl = pl * entho + ecinl + emagl;
  const R ptotl = pl + emagl;
  const R vdotbl = ul * a + vl * bl + wl * cl;

  const R rr = qr[ID], pr = qr[IP], ur = qr[IU], vr = qr[IV], wr = qr[IW], br = qr[IB],
          cr = qr[IC];
  const R ecinr = R(0.5) * (ur * ur + vr * vr + wr * wr) * rr;
  const R emagr = R(0.5) * (a * a + br * br + cr * cr);
  const R etotr = pr * entho + ecinr + emagr;
  const R ptotr = pr + emagr;
  const R vdotbr = ur * a + vr * br + wr * cr;

  // fmax(cfastl, cfastr) as the root of the larger square (fast_speed2_x)
  const R cfm = sqrt(fmax(fast_speed2_x(ql, gamma0), fast_speed2_x(qr, gamma0)));

  const R sl = fmin(ul, ur) - cfm;
  const R sr = fmax(ul, ur) + cfm;

  const R rcl = rl * (ul - sl);
  const R rcr = rr * (sr - ur);

  // quotients that share a denominator use its correctly rounded reciprocal
  // (qdiv: bit for bit the IEEE quotients)
  const R drc = rcr + rcl, yrc = qrcp(drc);
  const R ustar = qdiv(rcr * ur + rcl * ul + (ptotl - ptotr), drc, yrc);
  const R ptotstar = qdiv(rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur), drc, yrc);
  const R a2 = a * a, ya2 = qrcp(a2); // estar / a^2, both sides

  // left star state
  const R dsl = sl - ustar, ysl = qrcp(dsl);
  const R rstarl = qdiv(rl * (sl - ul), dsl, ysl);
  R       estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const R el = rl * (sl - ul) * (sl - ul) - a * a;
  R       vstarl, wstarl, bstarl, cstarl;
  if (a2 > R(0) && fabs(qdiv(estar, a2, ya2) - R(1)) <= R(1e-8))
  {
    vstarl = vl;
    bstarl = bl;
    wstarl = wl;
    cstarl = cl;
  }
  else
  {
    // four quotients over estar (qdiv: bit for bit the IEEE ones)
    const R ye = qrcp(estar);
    vstarl = vl - qdiv(a * bl * (ustar - ul), estar, ye);
    bstarl = qdiv(bl * el, estar, ye);
    wstarl = wl - qdiv(a * cl * (ustar - ul), estar, ye);
    cstarl = qdiv(cl * el, estar, ye);
  }
  const R vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  const R etotstarl =
    qdiv((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl), dsl, ysl);
  const R sqrrstarl = sqrt(rstarl);
  const R calfvenl = fabs(a) / sqrrstarl;
  const R sal = ustar - calfvenl;

  // right star state
  const R dsr = sr - ustar, ysr = qrcp(dsr);
  const R rstarr = qdiv(rr * (sr - ur), dsr, ysr);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const R er = rr * (sr - ur) * (sr - ur) - a * a;
  R       vstarr, wstarr, bstarr, cstarr;
  if (a2 > R(0) && fabs(qdiv(estar, a2, ya2) - R(1)) <= R(1e-8))
  {
    vstarr = vr;
    bstarr = br;
    wstarr = wr;
    cstarr = cr;
  }
  else
  {
    // four quotients over estar (qdiv: bit for bit the IEEE ones)
    const R ye = qrcp(estar);
    vstarr = vr - qdiv(a * br * (ustar - ur), estar, ye);
    bstarr = qdiv(br * er, estar, ye);
    wstarr = wr - qdiv(a * cr * (ustar - ur), estar, ye);
    cstarr = qdiv(cr * er, estar, ye);
  }
  const R vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  const R etotstarr =
    qdiv((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr), dsr, ysr);
  const R sqrrstarr = sqrt(rstarr);
  const R calfvenr = fabs(a) / sqrrstarr;
  const R sar = ustar + calfvenr;

  // sample the self-similar solution at x/t = 0, in the reference's order
  R ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > R(0))
  {
    ro = rl; uo = ul; vo = vl; wo = wl; bo = bl; co = cl;
    ptoto = ptotl; etoto = etotl; vdotbo = vdotbl;
  }
  else if (sal > R(0))
  {
    ro = rstarl; uo = ustar; vo = vstarl; wo = wstarl; bo = bstarl; co = cstarl;
    ptoto = ptotstar; etoto = etotstarl; vdotbo = vdotbstarl;
  }
  else if (!(ustar > R(0)) && !(sar > R(0)))
  {
    if (sr > R(0))
    {
      ro = rstarr; uo = ustar; vo = vstarr; wo = wstarr; bo = bstarr; co = cstarr;
      ptoto = ptotstar; etoto = etotstarr; vdotbo = vdotbstarr;
    }
    else
    {
      ro = rr; uo = ur; vo = vr; wo = wr; bo = br; co = cr;
      ptoto = ptotr; etoto = etotr; vdotbo = vdotbr;
    }
  }
  else
  {
    // double-star states, only needed between the two Alfven waves (four
    // quotients over one denominator)
    const R ds = sqrrstarl + sqrrstarr, ys = qrcp(ds);
    const R vstarstar =
      qdiv(sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl), ds, ys);
    const R wstarstar =
      qdiv(sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl), ds, ys);
    const R bstarstar = qdiv(
      sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl), ds,
      ys);
    const R cstarstar = qdiv(
      sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl), ds,
      ys);
    const R vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
    uo = ustar;
    vo = vstarstar;
    wo = wstarstar;
    bo = bstarstar;
    co = cstarstar;
    ptoto = ptotstar;
    vdotbo = vdotbstarstar;
    if (ustar > R(0))
    {
      ro = rstarl;
      etoto = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
    }
    else
    {
      ro = rstarr;
      etoto = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);
    }
  }

  flux[ID] = ro * uo;
  flux[IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[IU] = ro * uo * uo - a * a + ptoto;
  flux[IV] = ro * uo * vo - a * bo;
  flux[IW] = ro * uo * wo - a * co;
  flux[IA] = R(0);
  flux[IB] = bo * uo - a * vo;
  flux[IC] = co * uo - a * wo;
}

// HLLD, same states and sampling as riemann_hlld, with 8 reciprocals, 4
// square roots and 2 rsqrt instead of ~28 divides and 6 square roots.
template <class R>
__device__ void
riemann_hlld_fast(State<R> & ql, State<R> & qr, State<R> & flux, R gamma0, R entho, R p0 = R(0))
{
  // FP32: total pressures are carried minus the constant p0 (the momentum
  // flux comes out shifted by -p0; the energy flux and the wave speeds use
  // the unshifted values), see flux_shift
  constexpr bool shifted = sizeof(R) == 4;
  // the version-2 face stage gives both states the face-centred normal field,
  // and then the mean is that value exactly
  R a = ql[IA];
  if (fbits(ql[IA]) != fbits(qr[IA]))
    a = R(0.5) * (ql[IA] + qr[IA]);
  const R a2 = a * a;
  const R sgnm = ge0(a) ? R(1) : R(-1);

  const R rl = ql[ID], pl = ql[IP], ul = ql[IU], vl = ql[IV], wl = ql[IW], bl = ql[IB],
          cl = ql[IC];
  const R b2l = a2 + bl * bl + cl * cl;
  const R emagl = R(0.5) * b2l;
  const R etotl = pl * entho + R(0.5) * (ul * ul + vl * vl + wl * wl) * rl + emagl;
  const R ptotl = shifted ? (pl - p0) + emagl : pl + emagl;
  const R vdotbl = ul * a + vl * bl + wl * cl;

  const R rr = qr[ID], pr = qr[IP], ur = qr[IU], vr = qr[IV], wr = qr[IW], br = qr[IB],
          cr = qr[IC];
  const R b2r = a2 + br * br + cr * cr;
  const R emagr = R(0.5) * b2r;
  const R etotr = pr * entho + R(0.5) * (ur * ur + vr * vr + wr * wr) * rr + emagr;
  const R ptotr = shifted ? (pr - p0) + emagr : pr + emagr;
  const R vdotbr = ur * a + vr * br + wr * cr;

  R cfastl, cfastr;
  {
    const R id = rcp(rl);
    const R c2 = gamma0 * pl * id;
    const R d2 = R(0.5) * (b2l * id + c2);
    cfastl = d2 + fsqrt(d2 * d2 - c2 * a2 * id); // squared speed
  }
  {
    const R id = rcp(rr);
    const R c2 = gamma0 * pr * id;
    const R d2 = R(0.5) * (b2r * id + c2);
    cfastr = d2 + fsqrt(d2 * d2 - c2 * a2 * id);
  }
  const R cmax = fsqrt(sel_max(cfastl, cfastr)); // = max of the square roots
  const R sl = sel_min(ul, ur) - cmax;
  const R sr = sel_max(ul, ur) + cmax;
  const R rcl = rl * (ul - sl);
  const R rcr = rr * (sr - ur);
  const R irc = rcp(rcr + rcl);
  const R ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) * irc;
  const R ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) * irc;

  // left star state
  const R slu = sl - ul, sls = sl - ustar;
  const R isls = rcp(sls);
  const R rstarl = rl * slu * isls;
  R       vstarl = vl, wstarl = wl, bstarl = bl, cstarl = cl;
  {
    const R estar = rl * slu * sls - a2;
    if (!(gt0(a2) && abs_le(estar - a2, R(1e-8) * a2)))
    {
      const R ie = rcp(estar);
      const R el = rl * slu * slu - a2;
      const R tv = a * (ustar - ul) * ie;
      vstarl = vl - bl * tv;
      wstarl = wl - cl * tv;
      const R fe = el * ie;
      bstarl = bl * fe;
      cstarl = cl * fe;
    }
  }
  const R rsl = rsq(rstarl);
  const R sqrrstarl = rstarl * rsl;
  const R sal = ustar - fabs(a) * rsl;

  // right star state
  const R sru = sr - ur, srs = sr - ustar;
  const R isrs = rcp(srs);
  const R rstarr = rr * sru * isrs;
  R       vstarr = vr, wstarr = wr, bstarr = br, cstarr = cr;
  {
    const R estar = rr * sru * srs - a2;
    if (!(gt0(a2) && abs_le(estar - a2, R(1e-8) * a2)))
    {
      const R ie = rcp(estar);
      const R er = rr * sru * sru - a2;
      const R tv = a * (ustar - ur) * ie;
      vstarr = vr - br * tv;
      wstarr = wr - cr * tv;
      const R fe = er * ie;
      bstarr = br * fe;
      cstarr = cr * fe;
    }
  }
  const R rsr = rsq(rstarr);
  const R sqrrstarr = rstarr * rsr;
  const R sar = ustar + fabs(a) * rsr;

  // Star-state total energy and v.B.  Every star region takes them from one
  // side only: the left star region (sal > 0) from the left, the right ones
  // (ustar <= 0, sar <= 0) from the right, the double-star region from the
  // left iff ustar > 0.  In FP64 (FP64-pipe bound) only that side is
  // computed, with the reference's expressions, and both names below carry
  // it; `left` repeats the region tests (with a number for sal, sal > 0
  // implies ustar > 0).  In FP32 (issue bound) both sides cost fewer
  // instructions than selecting the operands.
  R vdotbstarl, etotstarl, vdotbstarr, etotstarr;
  if constexpr (sizeof(R) == 8)
  {
    const bool left = gt0(sal) || gt0(ustar);
    vdotbstarl = left ? ustar * a + vstarl * bstarl + wstarl * cstarl
                      : ustar * a + vstarr * bstarr + wstarr * cstarr;
    etotstarl = left ? (slu * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) * isls
                     : (sru * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarl)) * isrs;
    vdotbstarr = vdotbstarl;
    etotstarr = etotstarl;
  }
  else
  {
    // with the shift: -ptot ul + ptot* u* = -(ptot - p0) ul + (ptot* - p0) u* + p0 (u* - ul)
    vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
    etotstarl = (slu * etotl - ptotl * ul + ptotstar * ustar + p0 * (ustar - ul) +
                 a * (vdotbl - vdotbstarl)) * isls;
    vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
    etotstarr = (sru * etotr - ptotr * ur + ptotstar * ustar + p0 * (ustar - ur) +
                 a * (vdotbr - vdotbstarr)) * isrs;
  }

  R ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (gt0(sl))
  {
    ro = rl; uo = ul; vo = vl; wo = wl; bo = bl; co = cl;
    ptoto = ptotl; etoto = etotl; vdotbo = vdotbl;
  }
  else if (gt0(sal))
  {
    ro = rstarl; uo = ustar; vo = vstarl; wo = wstarl; bo = bstarl; co = cstarl;
    ptoto = ptotstar; etoto = etotstarl; vdotbo = vdotbstarl;
  }
  else if (!gt0(ustar) && !gt0(sar))
  {
    if (gt0(sr))
    {
      ro = rstarr; uo = ustar; vo = vstarr; wo = wstarr; bo = bstarr; co = cstarr;
      ptoto = ptotstar; etoto = etotstarr; vdotbo = vdotbstarr;
    }
    else
    {
      ro = rr; uo = ur; vo = vr; wo = wr; bo = br; co = cr;
      ptoto = ptotr; etoto = etotr; vdotbo = vdotbr;
    }
  }
  else
  {
    const R is = rcp(sqrrstarl + sqrrstarr);
    const R sq = sgnm * sqrrstarl * sqrrstarr;
    vo = (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) * is;
    wo = (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) * is;
    bo = (sqrrstarl * bstarr + sqrrstarr * bstarl + sq * (vstarr - vstarl)) * is;
    co = (sqrrstarl * cstarr + sqrrstarr * cstarl + sq * (wstarr - wstarl)) * is;
    uo = ustar;
    ptoto = ptotstar;
    vdotbo = ustar * a + vo * bo + wo * co;
    if (gt0(ustar))
    {
      ro = rstarl;
      etoto = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbo);
    }
    else
    {
      ro = rstarr;
      etoto = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbo);
    }
  }
  const R rou = ro * uo;
  flux[ID] = rou;
  flux[IP] = (etoto + (shifted ? ptoto + p0 : ptoto)) * uo - a * vdotbo;
  flux[IU] = rou * uo - a2 + ptoto;
  flux[IV] = rou * vo - a * bo;
  flux[IW] = rou * wo - a * co;
  flux[IA] = R(0);
  flux[IB] = bo * uo - a * vo;
  flux[IC] = co * uo - a * wo;
}

// riemann_mhd dispatch (RiemannSolvers_MHD.h:372-392); entho = 1/(gamma0-1),
// precomputed once per run for the fast HLLD.  p0: the FP32 momentum-flux
// shift (flux_shift); the HLL and LLF fluxes get it subtracted afterwards.
template <class R>
__device__ __forceinline__ void
riemann(int solver, State<R> & ql, State<R> & qr, State<R> & flux, R gamma0, R entho,
        R p0 = R(0))
{
  if (solver == RIEMANN_HLLD)
  {
    if constexpr (kExactOrder)
      riemann_hlld(ql, qr, flux, gamma0, entho);
    else
      riemann_hlld_fast(ql, qr, flux, gamma0, entho, p0);
    return;
  }
  if (solver == RIEMANN_HLL)
    riemann_hll(ql, qr, flux, gamma0);
  else
    riemann_llf(ql, qr, flux, gamma0);
  if constexpr (sizeof(R) == 4)
    flux[IU] = flux[IU] - p0;
}

// Two-dimensional HLLD magnetic Riemann solver giving the edge EMF
// (mag_riemann2d_hlld, RiemannSolvers_MHD.h:398-630).  q[0..3] are the
// LL, RL, LR, RR states; e[0..3] their corner emfs.  The region is selected
// by the signs of SB, ST, SL, SR exactly as the reference's 0/1 masks do
// (copysign based, :569-596); only the selected candidate is evaluated.
template <class R>
__device__ R
mag_riemann2d_hlld(const State<R> (&q)[4], const R (&e)[4], R gamma0, R smallc)
{
  const State<R> &qLL = q[0], &qRL = q[1], &qLR = q[2], &qRR = q[3];
  const R         ELL = e[0], ERL = e[1], ELR = e[2], ERR = e[3];

  const R rLL = qLL[ID], pLL = qLL[IP], uLL = qLL[IU], vLL = qLL[IV], aLL = qLL[IA],
          bLL = qLL[IB], cLL = qLL[IC];
  const R rLR = qLR[ID], pLR = qLR[IP], uLR = qLR[IU], vLR = qLR[IV], aLR = qLR[IA],
          bLR = qLR[IB], cLR = qLR[IC];
  const R rRL = qRL[ID], pRL = qRL[IP], uRL = qRL[IU], vRL = qRL[IV], aRL = qRL[IA],
          bRL = qRL[IB], cRL = qRL[IC];
  const R rRR = qRR[ID], pRR = qRR[IP], uRR = qRR[IU], vRR = qRR[IV], aRR = qRR[IA],
          bRR = qRR[IB], cRR = qRR[IC];

  // FMAX4 of the eight fast speeds as the roots of the largest squares
  // (fast_speed2_x / _y): two square roots instead of eight
  const R cxm = sqrt(max4(fast_speed2_x(qLL, gamma0), fast_speed2_x(qLR, gamma0),
                          fast_speed2_x(qRL, gamma0), fast_speed2_x(qRR, gamma0)));
  const R cym = sqrt(max4(fast_speed2_y(qLL, gamma0), fast_speed2_y(qLR, gamma0),
                          fast_speed2_y(qRL, gamma0), fast_speed2_y(qRR, gamma0)));

  const R SL = min4(uLL, uLR, uRL, uRR) - cxm;
  const R SR = max4(uLL, uLR, uRL, uRR) + cxm;
  const R SB = min4(vLL, vLR, vRL, vRR) - cym;
  const R ST = max4(vLL, vLR, vRL, vRR) + cym;

  // region flags from the sign bits, as (int)(1 + copysign(1, S)) / 2 does
  const bool SB_pos = !signbit(SB), ST_pos = !signbit(ST);
  const bool SL_pos = !signbit(SL), SR_pos = !signbit(SR);

  // Corner regions return an input emf directly.
  if (SB_pos && SL_pos)
    return ELL;
  if (SB_pos && !SR_pos)
    return ERL;
  if (!SB_pos && !ST_pos && SL_pos)
    return ELR;
  if (!SB_pos && !ST_pos && !SR_pos)
    return ERR;

  const R PtotLL = pLL + R(0.5) * (aLL * aLL + bLL * bLL + cLL * cLL);
  const R PtotLR = pLR + R(0.5) * (aLR * aLR + bLR * bLR + cLR * cLR);
  const R PtotRL = pRL + R(0.5) * (aRL * aRL + bRL * bRL + cRL * cRL);
  const R PtotRR = pRR + R(0.5) * (aRR * aRR + bRR * bRR + cRR * cRR);

  const R rcLLx = rLL * (uLL - SL);
  const R rcRLx = rRL * (SR - uRL);
  const R rcLRx = rLR * (uLR - SL);
  const R rcRRx = rRR * (SR - uRR);
  const R rcLLy = rLL * (vLL - SB);
  const R rcLRy = rLR * (ST - vLR);
  const R rcRLy = rRL * (vRL - SB);
  const R rcRRy = rRR * (ST - vRR);

  const R ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  const R vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  // the 24 star-state quotients share four denominators (qdiv: bit for bit
  // the IEEE quotients, in the reference's operation order)
  const R dSL = SL - ustar, dSR = SR - ustar, dSB = SB - vstar, dST = ST - vstar;
  const R ySL = qrcp(dSL), ySR = qrcp(dSR), ySB = qrcp(dSB), yST = qrcp(dST);

  const R rstarLLx = qdiv(rLL * (SL - uLL), dSL, ySL);
  const R BstarLL = qdiv(bLL * (SL - uLL), dSL, ySL);
  const R rstarLLy = qdiv(rLL * (SB - vLL), dSB, ySB);
  const R AstarLL = qdiv(aLL * (SB - vLL), dSB, ySB);
  const R rstarLL = qdiv(rstarLLx * (SB - vLL), dSB, ySB);
  const R EstarLLx = ustar * BstarLL - vLL * aLL;
  const R EstarLLy = uLL * bLL - vstar * AstarLL;
  const R EstarLL = ustar * BstarLL - vstar * AstarLL;

  const R rstarLRx = qdiv(rLR * (SL - uLR), dSL, ySL);
  const R BstarLR = qdiv(bLR * (SL - uLR), dSL, ySL);
  const R rstarLRy = qdiv(rLR * (ST - vLR), dST, yST);
  const R AstarLR = qdiv(aLR * (ST - vLR), dST, yST);
  const R rstarLR = qdiv(rstarLRx * (ST - vLR), dST, yST);
  const R EstarLRx = ustar * BstarLR - vLR * aLR;
  const R EstarLRy = uLR * bLR - vstar * AstarLR;
  const R EstarLR = ustar * BstarLR - vstar * AstarLR;

  const R rstarRLx = qdiv(rRL * (SR - uRL), dSR, ySR);
  const R BstarRL = qdiv(bRL * (SR - uRL), dSR, ySR);
  const R rstarRLy = qdiv(rRL * (SB - vRL), dSB, ySB);
  const R AstarRL = qdiv(aRL * (SB - vRL), dSB, ySB);
  const R rstarRL = qdiv(rstarRLx * (SB - vRL), dSB, ySB);
  const R EstarRLx = ustar * BstarRL - vRL * aRL;
  const R EstarRLy = uRL * bRL - vstar * AstarRL;
  const R EstarRL = ustar * BstarRL - vstar * AstarRL;

  const R rstarRRx = qdiv(rRR * (SR - uRR), dSR, ySR);
  const R BstarRR = qdiv(bRR * (SR - uRR), dSR, ySR);
  const R rstarRRy = qdiv(rRR * (ST - vRR), dST, yST);
  const R AstarRR = qdiv(aRR * (ST - vRR), dST, yST);
  const R rstarRR = qdiv(rstarRRx * (ST - vRR), dST, yST);
  const R EstarRRx = ustar * BstarRR - vRR * aRR;
  const R EstarRRy = uRR * bRR - vstar * AstarRR;
  const R EstarRR = ustar * BstarRR - vstar * AstarRR;

  // FMAX5 of |B| / sqrt(rho) over the corner states (RiemannSolvers_MHD.h:
  // 529-548), one IEEE quotient and square root per maximum
  const R calfvenL = alfven_max5_exact(aLR, rstarLRx, AstarLR, rstarLR, aLL, rstarLLx, AstarLL,
                                       rstarLL, smallc);
  const R calfvenR = alfven_max5_exact(aRR, rstarRRx, AstarRR, rstarRR, aRL, rstarRLx, AstarRL,
                                       rstarRL, smallc);
  const R calfvenB = alfven_max5_exact(bLL, rstarLLy, BstarLL, rstarLL, bRL, rstarRLy, BstarRL,
                                       rstarRL, smallc);
  const R calfvenT = alfven_max5_exact(bLR, rstarLRy, BstarLR, rstarLR, bRR, rstarRRy, BstarRR,
                                       rstarRR, smallc);

  const R SAL = fmin(ustar - calfvenL, R(0));
  const R SAR = fmax(ustar + calfvenR, R(0));
  const R SAB = fmin(vstar - calfvenB, R(0));
  const R SAT = fmax(vstar + calfvenT, R(0));

  if (SB_pos) // SL < 0 < SR
    return (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) / (SAR - SAL);
  if (!ST_pos) // SL < 0 < SR
    return (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) / (SAR - SAL);
  if (SL_pos)
    return (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) / (SAT - SAB);
  if (!SR_pos)
    return (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) / (SAT - SAB);

  // eight quotients over two denominators
  const R dLR = SAR - SAL, dBT = SAT - SAB;
  const R yLR = qrcp(dLR), yBT = qrcp(dBT);
  const R AstarT = qdiv(SAR * AstarRR - SAL * AstarLR, dLR, yLR);
  const R AstarB = qdiv(SAR * AstarRL - SAL * AstarLL, dLR, yLR);
  const R BstarR = qdiv(SAT * BstarRR - SAB * BstarRL, dBT, yBT);
  const R BstarL = qdiv(SAT * BstarLR - SAB * BstarLL, dBT, yBT);
  return qdiv(qdiv(SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR +
                     SAR * SAT * EstarLL,
                   dLR, yLR),
              dBT, yBT) -
         qdiv(SAT * SAB, dBT, yBT) * (AstarT - AstarB) +
         qdiv(SAR * SAL, dLR, yLR) * (BstarR - BstarL);
}

// The Alfven-speed maximum of one side of the 2D HLLD: the largest |n|/sqrt(r)
// over two corners, each with its state (n, r) and its compressed state
// (n f, r f) (for example aLR over rstarLRx and AstarLR = aLR fLRy over
// rstarLR = rstarLRx fLRy).  The compressed candidate squared is the plain
// one times f, so it wins its corner iff f > 1 (an integer-keyed compare);
// the two corner winners meet in one cross-multiplied comparison and only
// the overall winner takes an rsqrt.  nf, rf are the compressed values as
// the caller computed them, so the result is one of the four candidates,
// the largest or within one rounding of it where two tie to the last bits.
template <class R>
__device__ __forceinline__ R
alfven_max2x2(R n0, R r0, R nf0, R rf0, R f0, R n1, R r1, R nf1, R rf1, R f1)
{
  const long long one = order_key(R(1));
  const bool      c0 = order_key(f0) > one, c1 = order_key(f1) > one;
  const R         na = c0 ? nf0 : n0, ra = c0 ? rf0 : r0;
  const R         nb = c1 ? nf1 : n1, rb = c1 ? rf1 : r1;
  const bool      sb = order_key(nb * nb * ra) > order_key(na * na * rb);
  return fabs(sb ? nb : na) * rsq(sb ? rb : ra);
}

// The same 2D HLLD solve with shared reciprocals: 12 reciprocals, 10 square
// roots and 12 rsqrt (4 in FP64, through alfven_max2x2) instead of ~75
// divides and 32 square roots.
template <class R>
__device__ R
mag_riemann2d_hlld_fast(const State<R> (&q)[4], R gamma0, R smallc)
{
  const State<R> &qLL = q[0], &qRL = q[1], &qLR = q[2], &qRR = q[3];
  R               cFastLLx, cFastLLy, cFastLRx, cFastLRy, cFastRLx, cFastRLy, cFastRRx, cFastRRy;
  fast_speeds2_xy(qLL, gamma0, cFastLLx, cFastLLy);
  fast_speeds2_xy(qLR, gamma0, cFastLRx, cFastLRy);
  fast_speeds2_xy(qRL, gamma0, cFastRLx, cFastRLy);
  fast_speeds2_xy(qRR, gamma0, cFastRRx, cFastRRy);
  const R uLL = qLL[IU], uLR = qLR[IU], uRL = qRL[IU], uRR = qRR[IU];
  const R vLL = qLL[IV], vLR = qLR[IV], vRL = qRL[IV], vRR = qRR[IV];
  const R cxm = fsqrt(max4(cFastLLx, cFastLRx, cFastRLx, cFastRRx));
  const R cym = fsqrt(max4(cFastLLy, cFastLRy, cFastRLy, cFastRRy));
  const R SL = min4(uLL, uLR, uRL, uRR) - cxm;
  const R SR = max4(uLL, uLR, uRL, uRR) + cxm;
  const R SB = min4(vLL, vLR, vRL, vRR) - cym;
  const R ST = max4(vLL, vLR, vRL, vRR) + cym;
  const bool SB_pos = !signbit(SB), ST_pos = !signbit(ST);
  const bool SL_pos = !signbit(SL), SR_pos = !signbit(SR);
  // corner regions: the corner state's own emf u b - v a
  if (SB_pos && SL_pos)
    return uLL * qLL[IB] - vLL * qLL[IA];
  if (SB_pos && !SR_pos)
    return uRL * qRL[IB] - vRL * qRL[IA];
  if (!SB_pos && !ST_pos && SL_pos)
    return uLR * qLR[IB] - vLR * qLR[IA];
  if (!SB_pos && !ST_pos && !SR_pos)
    return uRR * qRR[IB] - vRR * qRR[IA];

  const R rLL = qLL[ID], rLR = qLR[ID], rRL = qRL[ID], rRR = qRR[ID];
  const R aLL = qLL[IA], aLR = qLR[IA], aRL = qRL[IA], aRR = qRR[IA];
  const R bLL = qLL[IB], bLR = qLR[IB], bRL = qRL[IB], bRR = qRR[IB];
  const R PtotLL = qLL[IP] + R(0.5) * (aLL * aLL + bLL * bLL + qLL[IC] * qLL[IC]);
  const R PtotLR = qLR[IP] + R(0.5) * (aLR * aLR + bLR * bLR + qLR[IC] * qLR[IC]);
  const R PtotRL = qRL[IP] + R(0.5) * (aRL * aRL + bRL * bRL + qRL[IC] * qRL[IC]);
  const R PtotRR = qRR[IP] + R(0.5) * (aRR * aRR + bRR * bRR + qRR[IC] * qRR[IC]);

  const R rcLLx = rLL * (uLL - SL), rcRLx = rRL * (SR - uRL);
  const R rcLRx = rLR * (uLR - SL), rcRRx = rRR * (SR - uRR);
  const R rcLLy = rLL * (vLL - SB), rcLRy = rLR * (ST - vLR);
  const R rcRLy = rRL * (vRL - SB), rcRRy = rRR * (ST - vRR);
  const R ustar = (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR +
                   (PtotLL - PtotRL + PtotLR - PtotRR)) *
                  rcp(rcLLx + rcLRx + rcRLx + rcRRx);
  const R vstar = (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR +
                   (PtotLL - PtotLR + PtotRL - PtotRR)) *
                  rcp(rcLLy + rcLRy + rcRLy + rcRRy);

  const R iL = rcp(SL - ustar), iR = rcp(SR - ustar);
  const R iB = rcp(SB - vstar), iT = rcp(ST - vstar);
  // x and y compression factors of each corner state
  const R fLLx = (SL - uLL) * iL, fLRx = (SL - uLR) * iL, fRLx = (SR - uRL) * iR, fRRx = (SR - uRR) * iR;
  const R fLLy = (SB - vLL) * iB, fRLy = (SB - vRL) * iB, fLRy = (ST - vLR) * iT, fRRy = (ST - vRR) * iT;

  const R rstarLLx = rLL * fLLx, BstarLL = bLL * fLLx, rstarLLy = rLL * fLLy, AstarLL = aLL * fLLy;
  const R rstarLL = rstarLLx * fLLy;
  const R rstarLRx = rLR * fLRx, BstarLR = bLR * fLRx, rstarLRy = rLR * fLRy, AstarLR = aLR * fLRy;
  const R rstarLR = rstarLRx * fLRy;
  const R rstarRLx = rRL * fRLx, BstarRL = bRL * fRLx, rstarRLy = rRL * fRLy, AstarRL = aRL * fRLy;
  const R rstarRL = rstarRLx * fRLy;
  const R rstarRRx = rRR * fRRx, BstarRR = bRR * fRRx, rstarRRy = rRR * fRRy, AstarRR = aRR * fRRy;
  const R rstarRR = rstarRRx * fRRy;

  R calfvenL, calfvenR, calfvenB, calfvenT;
  if constexpr (sizeof(R) == 8)
  {
    calfvenL = sel_max(alfven_max2x2(aLR, rstarLRx, AstarLR, rstarLR, fLRy,
                                     aLL, rstarLLx, AstarLL, rstarLL, fLLy), smallc);
    calfvenR = sel_max(alfven_max2x2(aRR, rstarRRx, AstarRR, rstarRR, fRRy,
                                     aRL, rstarRLx, AstarRL, rstarRL, fRLy), smallc);
    calfvenB = sel_max(alfven_max2x2(bLL, rstarLLy, BstarLL, rstarLL, fLLx,
                                     bRL, rstarRLy, BstarRL, rstarRL, fRLx), smallc);
    calfvenT = sel_max(alfven_max2x2(bLR, rstarLRy, BstarLR, rstarLR, fLRx,
                                     bRR, rstarRRy, BstarRR, rstarRR, fRRx), smallc);
  }
  else
  {
    calfvenL = max5(fabs(aLR) * rsq(rstarLRx), fabs(AstarLR) * rsq(rstarLR),
                    fabs(aLL) * rsq(rstarLLx), fabs(AstarLL) * rsq(rstarLL), smallc);
    calfvenR = max5(fabs(aRR) * rsq(rstarRRx), fabs(AstarRR) * rsq(rstarRR),
                    fabs(aRL) * rsq(rstarRLx), fabs(AstarRL) * rsq(rstarRL), smallc);
    calfvenB = max5(fabs(bLL) * rsq(rstarLLy), fabs(BstarLL) * rsq(rstarLL),
                    fabs(bRL) * rsq(rstarRLy), fabs(BstarRL) * rsq(rstarRL), smallc);
    calfvenT = max5(fabs(bLR) * rsq(rstarLRy), fabs(BstarLR) * rsq(rstarLR),
                    fabs(bRR) * rsq(rstarRRy), fabs(BstarRR) * rsq(rstarRR), smallc);
  }
  const R SAL = sel_min(ustar - calfvenL, R(0));
  const R SAR = sel_max(ustar + calfvenR, R(0));
  const R SAB = sel_min(vstar - calfvenB, R(0));
  const R SAT = sel_max(vstar + calfvenT, R(0));
  const R iLR = rcp(SAR - SAL), iBT = rcp(SAT - SAB);

  if (SB_pos)
    return (SAR * (ustar * BstarLL - vLL * aLL) - SAL * (ustar * BstarRL - vRL * aRL) +
            SAR * SAL * (bRL - bLL)) * iLR;
  if (!ST_pos)
    return (SAR * (ustar * BstarLR - vLR * aLR) - SAL * (ustar * BstarRR - vRR * aRR) +
            SAR * SAL * (bRR - bLR)) * iLR;
  if (SL_pos)
    return (SAT * (uLL * bLL - vstar * AstarLL) - SAB * (uLR * bLR - vstar * AstarLR) -
            SAT * SAB * (aLR - aLL)) * iBT;
  if (!SR_pos)
    return (SAT * (uRL * bRL - vstar * AstarRL) - SAB * (uRR * bRR - vstar * AstarRR) -
            SAT * SAB * (aRR - aRL)) * iBT;

  const R EstarLL = ustar * BstarLL - vstar * AstarLL;
  const R EstarLR = ustar * BstarLR - vstar * AstarLR;
  const R EstarRL = ustar * BstarRL - vstar * AstarRL;
  const R EstarRR = ustar * BstarRR - vstar * AstarRR;
  const R AstarT = (SAR * AstarRR - SAL * AstarLR) * iLR;
  const R AstarB = (SAR * AstarRL - SAL * AstarLL) * iLR;
  const R BstarR = (SAT * BstarRR - SAB * BstarRL) * iBT;
  const R BstarL = (SAT * BstarLR - SAB * BstarLL) * iBT;
  return (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) *
           iLR * iBT -
         SAT * SAB * iBT * (AstarT - AstarB) + SAR * SAL * iLR * (BstarR - BstarL);
}

// compute_emf<EmfDir> (RiemannSolvers_MHD.h:651-874): rotate the four
// reconstructed edge states (RT, RB, LT, LB) into the 2D frame of the edge,
// average the parallel field components and call the 2D solver.
// edir: 0 = EMFX, 1 = EMFY, 2 = EMFZ.
template <class R>
__device__ __forceinline__ R
compute_emf(int edir, const State<R> (&qe)[4], R gamma0, R smallc)
{
  const State<R> &qRT = qe[0], &qRB = qe[1], &qLT = qe[2], &qLB = qe[3];
  int             iu, iv, iw, ia, ib, ic;
  if (edir == 2)
  {
    iu = IU; iv = IV; iw = IW; ia = IA; ib = IB; ic = IC;
  }
  else if (edir == 1)
  {
    iu = IW; iv = IU; iw = IV; ia = IC; ib = IA; ic = IB;
  }
  else
  {
    iu = IV; iv = IW; iw = IU; ia = IB; ib = IC; ic = IA;
  }
  State<R> q[4]; // LL, RL, LR, RR
  q[0][ID] = qRT[ID]; q[1][ID] = qLT[ID]; q[2][ID] = qRB[ID]; q[3][ID] = qLB[ID];
  q[0][IP] = qRT[IP]; q[1][IP] = qLT[IP]; q[2][IP] = qRB[IP]; q[3][IP] = qLB[IP];
  q[0][IU] = qRT[iu]; q[1][IU] = qLT[iu]; q[2][IU] = qRB[iu]; q[3][IU] = qLB[iu];
  q[0][IV] = qRT[iv]; q[1][IV] = qLT[iv]; q[2][IV] = qRB[iv]; q[3][IV] = qLB[iv];
  q[0][IA] = R(0.5) * (qRT[ia] + qLT[ia]);
  q[1][IA] = q[0][IA];
  q[2][IA] = R(0.5) * (qRB[ia] + qLB[ia]);
  q[3][IA] = q[2][IA];
  q[0][IB] = R(0.5) * (qRT[ib] + qRB[ib]);
  q[1][IB] = R(0.5) * (qLT[ib] + qLB[ib]);
  q[2][IB] = q[0][IB];
  q[3][IB] = q[1][IB];
  q[0][IW] = qRT[iw]; q[1][IW] = qLT[iw]; q[2][IW] = qRB[iw]; q[3][IW] = qLB[iw];
  q[0][IC] = qRT[ic]; q[1][IC] = qLT[ic]; q[2][IC] = qRB[ic]; q[3][IC] = qLB[ic];
  if constexpr (kExactOrder)
  {
    R e[4];
#pragma unroll
    for (int c = 0; c < 4; ++c)
      e[c] = q[c][IU] * q[c][IB] - q[c][IV] * q[c][IA];
    return mag_riemann2d_hlld(q, e, gamma0, smallc);
  }
  else
    return mag_riemann2d_hlld_fast(q, gamma0, smallc);
}

} // namespace MHD_VARIANT_TAG
} // namespace mhd
