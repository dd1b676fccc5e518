// Accuracy check of the fast builds' FP64 reciprocal and square root
// (mhd_physics.cuh: rcp = one third-order Newton step on rcp.approx.ftz.f64,
// fsqrt = one third-order Householder correction of x * rsqrt.approx.ftz.f64)
// against correctly rounded host references, next to the CUDA library's
// __drcp_rn, sqrt and rsqrt and the two hardware seeds.  One thread per
// element, every access in bounds.  Prints one line per function:
//   <name> max_ulp <m> correctly_rounded <fraction>
// and exits non-zero on a CUDA error.
//
// Build and run (GB300):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fast_math_probe tests/fast_math_probe.cu
//   ./fast_math_probe
#include <cmath>
#include <cstdint>
#include <cstdio>
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
  OP_RCP_SEED = 5, // rcp.approx.ftz.f64
  OP_RSQ_SEED = 6, // rsqrt.approx.ftz.f64
  OP_COUNT = 7
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
  else if constexpr (OP == OP_RSQ)
    r = mhd::rsq(v);
  else if constexpr (OP == OP_RCP_SEED)
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(v));
  else
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(v));
  y[i] = r;
}

static double
ulp_error(double got, long double ref)
{
  const double r = (double)ref;
  const double u = std::nextafter(std::fabs(r), INFINITY) - std::fabs(r);
  return (double)(std::fabs((long double)got - ref) / (long double)u);
}

int
main()
{
  const int           n = 1 << 20;
  std::vector<double> hx(n), hy(n);
  // log-uniform over [1e-30, 1e30] from a fixed LCG, plus exact powers of two
  uint64_t s = 0x2545F4914F6CDD1DULL;
  for (int i = 0; i < n; ++i)
  {
    s = s * 6364136223846793005ULL + 1442695040888963407ULL;
    const double u = (double)(s >> 11) / 9007199254740992.0;
    hx[i] = (i % 97 == 0) ? std::ldexp(1.0, (i / 97) % 200 - 100) : std::pow(10.0, -30.0 + 60.0 * u);
  }
  double *dx = nullptr, *dy = nullptr;
  if (cudaMalloc(&dx, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&dy, n * sizeof(double)) != cudaSuccess)
  {
    std::printf("cudaMalloc failed\n");
    return 1;
  }
  cudaMemcpy(dx, hx.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  const char * names[OP_COUNT] = { "rcp", "drcp_rn", "fsqrt", "sqrt", "rsq", "rcp_seed", "rsq_seed" };
  for (int op = 0; op < OP_COUNT; ++op)
  {
    const dim3 grid((n + 255) / 256), block(256);
    switch (op)
    {
    case OP_RCP: k_apply<OP_RCP><<<grid, block>>>(dx, dy, n); break;
    case OP_DRCP_RN: k_apply<OP_DRCP_RN><<<grid, block>>>(dx, dy, n); break;
    case OP_FSQRT: k_apply<OP_FSQRT><<<grid, block>>>(dx, dy, n); break;
    case OP_SQRT: k_apply<OP_SQRT><<<grid, block>>>(dx, dy, n); break;
    case OP_RSQ: k_apply<OP_RSQ><<<grid, block>>>(dx, dy, n); break;
    case OP_RCP_SEED: k_apply<OP_RCP_SEED><<<grid, block>>>(dx, dy, n); break;
    default: k_apply<OP_RSQ_SEED><<<grid, block>>>(dx, dy, n); break;
    }
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess)
    {
      std::printf("%s: %s\n", names[op], cudaGetErrorString(e));
      return 1;
    }
    cudaMemcpy(hy.data(), dy, n * sizeof(double), cudaMemcpyDeviceToHost);
    double maxu = 0.0;
    long   exact = 0;
    for (int i = 0; i < n; ++i)
    {
      const long double xv = hx[i];
      const long double ref = (op == OP_RCP || op == OP_DRCP_RN || op == OP_RCP_SEED) ? 1.0L / xv
                              : (op == OP_RSQ || op == OP_RSQ_SEED) ? 1.0L / sqrtl(xv)
                                                                    : sqrtl(xv);
      const double u = ulp_error(hy[i], ref);
      maxu = u > maxu ? u : maxu;
      exact += hy[i] == (double)ref;
    }
    std::printf("%s max_ulp %.6f correctly_rounded %.6f\n", names[op], maxu, (double)exact / n);
  }
  cudaFree(dx);
  cudaFree(dy);
  return 0;
}
