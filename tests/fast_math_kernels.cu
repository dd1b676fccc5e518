// Test kernels of tests/test_fast_math.py: the fast builds' FP64 reciprocal
// and square root (mhd_physics.cuh: rcp = one third-order Newton step on
// rcp.approx.ftz.f64, fsqrt = one third-order Householder correction of
// x * rsqrt.approx.ftz.f64) against correctly rounded host references, next
// to the CUDA library's __drcp_rn, sqrt and rsqrt; and, on the arguments that
// take the fallback branches (zeros, subnormals, |x| >= 2^1021, infinities,
// NaN, negative numbers), bit for bit against the library function they fall
// back to.  One thread per element, every access in bounds.  Prints
//   <name> max_ulp <m> correctly_rounded <fraction>      (normal arguments)
//   special_<name> mismatches <count> of <n>             (fallback arguments)
//   special_gt mismatches <count> of <n>                 (exact build's integer
//                                                         comparison, all pairs)
//   special_alfven mismatches <count> of <n>             (exact build's Alfven-speed
//                                                         maximum with one quotient,
//                                                         ties, near ties, specials)
// and exits non-zero on a CUDA error.
//
// Build and run (GB300):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fast_math_kernels tests/fast_math_kernels.cu
//   ./fast_math_kernels
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "../ppkmhd_gb300/csrc/mhd_physics.cuh"

enum Op : int
{
  OP_RCP = 0,      // mhd::rcp(double)
  OP_DRCP_RN = 1,  // __drcp_rn
  OP_FSQRT = 2,    // mhd::fsqrt(double)
  OP_SQRT = 3,     // sqrt
  OP_RSQ = 4,      // mhd::rsq(double) (= rsqrt)
  OP_COUNT = 5
};

template <int OP>
__global__ void
k_apply(const double * __restrict__ x, double * __restrict__ y, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const double v = x[i];
  double       r;
  if constexpr (OP == OP_RCP)
    r = mhd::rcp(v);
  else if constexpr (OP == OP_DRCP_RN)
    r = __drcp_rn(v);
  else if constexpr (OP == OP_FSQRT)
    r = mhd::fsqrt(v);
  else if constexpr (OP == OP_SQRT)
    r = sqrt(v);
  else
    r = mhd::rsq(v);
  y[i] = r;
}

static double
ulp_error(double got, long double ref)
{
  const double r = (double)ref;
  const double u = std::nextafter(std::fabs(r), INFINITY) - std::fabs(r);
  return (double)(std::fabs((long double)got - ref) / (long double)u);
}

template <int OP>
static int
launch(const double * dx, double * dy, int n)
{
  k_apply<OP><<<(n + 255) / 256, 256>>>(dx, dy, n);
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}

static int
apply(int op, const double * dx, double * dy, int n)
{
  switch (op)
  {
  case OP_RCP: return launch<OP_RCP>(dx, dy, n);
  case OP_DRCP_RN: return launch<OP_DRCP_RN>(dx, dy, n);
  case OP_FSQRT: return launch<OP_FSQRT>(dx, dy, n);
  case OP_SQRT: return launch<OP_SQRT>(dx, dy, n);
  default: return launch<OP_RSQ>(dx, dy, n);
  }
}

// exact build's integer comparison against the FP comparison, all pairs
__global__ void
k_gt(const double * __restrict__ v, int n, unsigned * __restrict__ bad)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * n)
    return;
  const double a = v[i / n], b = v[i % n];
  if (mhd::exact_gt(a, b) != (a > b))
    atomicAdd(bad, 1u);
}

static bool
same_bits(double a, double b)
{
  if (std::isnan(a) && std::isnan(b))
    return true;
  uint64_t x, y;
  std::memcpy(&x, &a, 8);
  std::memcpy(&y, &b, 8);
  return x == y;
}

// The exact build's Alfven-speed maximum (one quotient and square root)
// against the four IEEE quotients and the exact sel_max chain, bit for bit.
__global__ void
k_alfven(const double * __restrict__ in, double * __restrict__ out, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n)
    return;
  const double * a = in + 9 * (size_t)i;
  out[2 * i] = mhd::alfven_max5_exact(a[0], a[1], a[2], a[3], a[4], a[5], a[6], a[7], a[8]);
  double m = fabs(a[0]) / sqrt(a[1]);
  for (int q = 1; q < 4; ++q)
  {
    const double v = fabs(a[2 * q]) / sqrt(a[2 * q + 1]);
    m = mhd::exact_gt(v, m) ? v : m;
  }
  out[2 * i + 1] = mhd::exact_gt(a[8], m) ? a[8] : m;
}

static int
check_alfven()
{
  const int           n = 1 << 20;
  std::vector<double> h(9 * (size_t)n);
  uint64_t            s = 0x9e3779b97f4a7c15ull;
  auto rnd = [&]() {
    s ^= s << 13;
    s ^= s >> 7;
    s ^= s << 17;
    return s;
  };
  auto uni = [&]() { return (double)(rnd() >> 11) * (1.0 / 9007199254740992.0); };
  auto logu = [&](double lo, double hi) { return std::exp(std::log(lo) + uni() * std::log(hi / lo)); };
  const double specials[] = { 0.0, -0.0, 1e-310, -1e-310, INFINITY, -INFINITY, NAN, 1e300, 1e-300,
                              -1.0, 2.2250738585072014e-308 };
  for (int i = 0; i < n; ++i)
  {
    double * a = &h[9 * (size_t)i];
    const int kind = (int)(rnd() % 8);
    for (int q = 0; q < 4; ++q)
    {
      a[2 * q] = logu(1e-20, 1e20) * ((rnd() & 1) ? 1.0 : -1.0);
      a[2 * q + 1] = logu(1e-20, 1e20);
    }
    a[8] = logu(1e-12, 1e2);
    if (kind == 1) // identical operands (exact ties)
      for (int q = 1; q < 4; ++q)
      {
        a[2 * q] = a[0];
        a[2 * q + 1] = a[1];
      }
    else if (kind == 2) // equal ratios from different operands: n 2^k, r 4^k
    {
      const int q = 1 + (int)(rnd() % 3);
      a[2 * q] = a[0] * 4.0;
      a[2 * q + 1] = a[1] * 16.0;
    }
    else if (kind == 3) // near ties: one ulp apart
    {
      const int q = 1 + (int)(rnd() % 3);
      a[2 * q] = a[0];
      a[2 * q + 1] = std::nextafter(a[1], (rnd() & 1) ? 0.0 : INFINITY);
    }
    else if (kind == 4) // ratios within 1e-15 of each other
    {
      const int q = 1 + (int)(rnd() % 3);
      a[2 * q] = a[0] * (1.0 + (uni() - 0.5) * 4e-15);
      a[2 * q + 1] = a[1];
    }
    else if (kind == 5) // special operands
    {
      const int q = (int)(rnd() % 9);
      a[q] = specials[rnd() % (sizeof specials / sizeof specials[0])];
    }
    else if (kind == 6) // zero numerators and large smallc
    {
      a[2 * (rnd() % 4)] = 0.0;
      a[8] = logu(1e-3, 1e12);
    }
  }
  double *d_in = nullptr, *d_out = nullptr;
  if (cudaMalloc(&d_in, h.size() * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&d_out, 2 * (size_t)n * sizeof(double)) != cudaSuccess)
    return 1;
  cudaMemcpy(d_in, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice);
  k_alfven<<<(n + 255) / 256, 256>>>(d_in, d_out, n);
  std::vector<double> o(2 * (size_t)n);
  if (cudaMemcpy(o.data(), d_out, o.size() * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess)
    return 1;
  int bad = 0;
  for (int i = 0; i < n; ++i)
  {
    uint64_t x, y;
    std::memcpy(&x, &o[2 * (size_t)i], 8);
    std::memcpy(&y, &o[2 * (size_t)i + 1], 8);
    bad += x != y;
  }
  std::printf("special_alfven mismatches %d of %d\n", bad, n);
  cudaFree(d_in);
  cudaFree(d_out);
  return 0;
}

int
main()
{
  const int           n = 1 << 20;
  std::vector<double> hx(n), hy(n), hz(n);
  // log-uniform over [1e-30, 1e30] from a fixed LCG, plus exact powers of two
  uint64_t s = 0x2545F4914F6CDD1DULL;
  for (int i = 0; i < n; ++i)
  {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    const double u = (double)(s >> 11) / 9007199254740992.0;
    hx[i] = (i % 97 == 0) ? std::ldexp(1.0, (i / 97) % 200 - 100) : std::pow(10.0, -30.0 + 60.0 * u);
  }
  // arguments of the fallback branches and the edges of the fast ranges
  std::vector<double> sp = { 0.0, -0.0, INFINITY, -INFINITY, NAN, -NAN,
                             std::ldexp(1.0, -1074), std::ldexp(1.0, -1073), std::ldexp(3.0, -1050),
                             -std::ldexp(1.0, -1074), std::nextafter(std::ldexp(1.0, -1022), 0.0),
                             std::ldexp(1.0, -1022), std::nextafter(std::ldexp(1.0, -1022), 1.0),
                             std::ldexp(1.0, 1021), std::nextafter(std::ldexp(1.0, 1021), 0.0),
                             std::ldexp(1.5, 1021), std::ldexp(1.0, 1022), std::ldexp(1.0, 1023),
                             std::nextafter(std::ldexp(1.0, 1022), 0.0), -std::ldexp(1.9, 1021),
                             1.7976931348623157e308, -1.0, -2.5e-300, -1e300, 1.0, 2.0, 0.5 };
  for (int e = -1074; e <= 1023; e += 7)
  {
    sp.push_back(std::ldexp(1.0, e));
    sp.push_back(-std::ldexp(1.3, e < 1023 ? e : 1022));
    sp.push_back(std::ldexp(1.7, e < 1023 ? e : 1022));
  }
  const int ns = (int)sp.size();
  double *  dx = nullptr, *dy = nullptr;
  if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dy, n * sizeof(double)) != cudaSuccess)
  {
    std::printf("cudaMalloc failed\n");
    return 1;
  }
  const char * names[OP_COUNT] = { "rcp", "drcp_rn", "fsqrt", "sqrt", "rsq" };
  cudaMemcpy(dx, hx.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  for (int op = 0; op < OP_COUNT; ++op)
  {
    if (apply(op, dx, dy, n))
    {
      std::printf("%s: CUDA error\n", names[op]);
      return 1;
    }
    cudaMemcpy(hy.data(), dy, n * sizeof(double), cudaMemcpyDeviceToHost);
    double maxu = 0.0;
    long   exact = 0;
    for (int i = 0; i < n; ++i)
    {
      const long double xv = hx[i];
      const long double ref = (op == OP_RCP || op == OP_DRCP_RN) ? 1.0L / xv
                              : (op == OP_RSQ)                  ? 1.0L / sqrtl(xv)
                                                                : sqrtl(xv);
      const double u = ulp_error(hy[i], ref);
      maxu = u > maxu ? u : maxu;
      exact += hy[i] == (double)ref;
    }
    std::printf("%s max_ulp %.6f correctly_rounded %.6f\n", names[op], maxu, (double)exact / n);
  }
  // fallback arguments: the fast function against the library one it falls
  // back to (rcp -> __drcp_rn, fsqrt -> sqrt), bit for bit
  cudaMemcpy(dx, sp.data(), ns * sizeof(double), cudaMemcpyHostToDevice);
  const int pairs[2][2] = { { OP_RCP, OP_DRCP_RN }, { OP_FSQRT, OP_SQRT } };
  for (const auto & pr : pairs)
  {
    if (apply(pr[0], dx, dy, ns))
      return 1;
    cudaMemcpy(hy.data(), dy, ns * sizeof(double), cudaMemcpyDeviceToHost);
    if (apply(pr[1], dx, dy, ns))
      return 1;
    cudaMemcpy(hz.data(), dy, ns * sizeof(double), cudaMemcpyDeviceToHost);
    int bad = 0;
    for (int i = 0; i < ns; ++i)
    {
      // inside the fast ranges the fast function may differ by its rounding
      const double v = sp[i];
      const bool   fast_range = (pr[0] == OP_RCP)
                                  ? (std::isfinite(v) && std::fabs(v) >= std::ldexp(1.0, -1022) &&
                                   std::fabs(v) < std::ldexp(1.0, 1021))
                                  : (std::isfinite(v) && v >= std::ldexp(1.0, -1022));
      if (fast_range)
      {
        const long double ref = pr[0] == OP_RCP ? 1.0L / (long double)v : sqrtl((long double)v);
        bad += ulp_error(hy[i], ref) > 0.8;
      }
      else
        bad += !same_bits(hy[i], hz[i]);
    }
    std::printf("special_%s mismatches %d of %d\n", names[pr[0]], bad, ns);
  }
  // the exact build's integer comparison on every pair of the special values
  {
    unsigned * dbad = nullptr;
    if (cudaMalloc(&dbad, sizeof(unsigned)) != cudaSuccess)
      return 1;
    cudaMemset(dbad, 0, sizeof(unsigned));
    k_gt<<<(ns * ns + 255) / 256, 256>>>(dx, ns, dbad);
    unsigned hb = 0;
    if (cudaDeviceSynchronize() != cudaSuccess)
      return 1;
    cudaMemcpy(&hb, dbad, sizeof hb, cudaMemcpyDeviceToHost);
    std::printf("special_gt mismatches %u of %d\n", hb, ns * ns);
    cudaFree(dbad);
  }
  cudaFree(dx);
  cudaFree(dy);
  if (check_alfven())
    return 1;
  return cudaDeviceSynchronize() == cudaSuccess ? 0 : 1;
}
