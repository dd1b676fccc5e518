// The HLLD flux surrogate: a 27-64-64-19 multilayer perceptron with GELU
// activations, BF16 weights and activations and FP32 accumulation.
//
// It replaces riemann_hlld (RiemannSolvers_MHD.h:133-367) on faces that a
// jump sensor flags as smooth.  The network does not predict the flux
// itself: the flux is split into the central part
//     Fc = (F(qL) + F(qR)) / 2          (exact, from the physical MHD flux)
// and the upwind dissipation D = Fc - F_HLLD, and the network predicts D in
// units of the face's own scales times the jump size:
//     F = Fc - scale * sJ * Dn.
// Everything is dimensionless per face, so one network serves every
// density, pressure and field level.
//
// Per face, in the face-normal frame (a = normal B, q = [rho, vn, vt1, vt2,
// p, Bt1, Bt2] left and right):
//   rs = (rhoL + rhoR) / 2
//   Ps = (pL + pR) / 2 + (|BL|^2 + |BR|^2) / 4       (total-pressure scale)
//   vs = sqrt(Ps / rs), bs = sqrt(Ps)
//   means   m = (vn, vt1, vt2) / vs, p / Ps, (Bt1, Bt2) / bs, and a / bs
//   jumps   h = (qR - qL) / 2 over (rs, vs, vs, vs, Ps, bs, bs)
//   J = max |h| (the smoothness sensor), sJ = max(J, kJFloor), hn = h / sJ
//   scale = (rs vs, Ps vs, Ps, Ps, Ps, bs vs, bs vs) for the flux
//           components (rho, E, mn, mt1, mt2, Bt1, Bt2)
// The flux is odd in each transverse direction: reflecting t1 (vt1, Bt1 ->
// -vt1, -Bt1 on both sides) flips the mt1 and Bt1 components and leaves the
// others.  The network keeps that exactly: its inputs are invariant under
// both reflections -- the even scalars (mean vn, p, a; jumps of rho, vn, p;
// sJ / kTauRef) and the 10 pairwise products of each transverse set
// u1 = (mean vt1, mean Bt1, hn_vt1, hn_Bt1), u2 likewise -- and its 19
// outputs are the three even components (rho, E, mn) and, for each odd
// component, 4 coefficients c of its basis: Dn_mt1 = sum_k c_k u1_k, etc.
// An odd component therefore vanishes with its transverse set, whatever
// the weights.
// GELU is the tanh form of Hendrycks and Gimpel (2016):
//   gelu(x) = x/2 (1 + tanh(sqrt(2/pi) (x + 0.044715 x^3))).
//
// Parameter vector (FP32 master copy), row = input, column = output unit:
//   W1[32][64] b1[64] W2[64][64] b2[64] W3[64][24] b3[24]   (7832 floats)
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mhd_umma.cuh"

namespace mhd
{
namespace mlp
{

constexpr int kIn = 32;     // 27 invariant inputs + 5 zero pads
constexpr int kInUsed = 27;
constexpr int kHid = 64;
constexpr int kOut = 24;    // 19 raw outputs + 5 pads
constexpr int kRawUsed = 19;
constexpr int kOutUsed = 7; // flux components after the basis combination
constexpr int kBasis = 8;   // u1[4], u2[4]
constexpr int kFeat = kIn + kBasis; // features of one face: inputs then basis

constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kIn * kHid;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid * kOut;
constexpr int kParams = kOffB3 + kOut; // 7832

// mma.m16n8k16 fragments of the three weight matrices, as bf16x2 words:
// [k-tile][n-tile][lane][2]
constexpr int kPackW1 = 0;
constexpr int kPackW2 = kPackW1 + (kIn / 16) * (kHid / 8) * 64;
constexpr int kPackW3 = kPackW2 + (kHid / 16) * (kHid / 8) * 64;
constexpr int kPackWords = kPackW3 + (kHid / 16) * (kOut / 8) * 64; // 3840
constexpr int kBiasFloats = kHid + kHid + kOut;                    // 152

// Image of the network for the tensor-core (tcgen05) batch forward: the
// transposed weight matrices W^T[N][K] of the three layers in BF16, in the
// tensor cores' K-major canonical layout (mhd_umma.cuh), then the biases in
// FP32.  Layer 3's 24 output rows are padded with zero rows to kN3 = 32 (for
// M = 128 the MMA's N is a multiple of 16).
constexpr int kN3 = 32;
constexpr int kTcW1 = 0;                         // byte offsets
constexpr int kTcW2 = kTcW1 + kHid * kIn * 2;    // 4096
constexpr int kTcW3 = kTcW2 + kHid * kHid * 2;   // 12288
constexpr int kTcWBytes = kTcW3 + kN3 * kHid * 2; // 16384
constexpr int kTcPackWords = kTcWBytes / 4 + kBiasFloats;
static_assert(kTcWBytes % 16 == 0 && kHid % 4 == 0 && kOut % 4 == 0, "16-byte bias groups");

constexpr double kJFloor = 1e-4;
constexpr double kTauRef = 0.1;

// Harvested face sample: the public record of MHD_SAMPLE_FLOATS floats.
constexpr int kRecord = 24;
constexpr int kRecQL = 0, kRecQR = 7, kRecA = 14, kRecJ = 15, kRecD = 16, kRecGamma = 23;

// Dimensionless encoding of one face (see the file comment): feat[0..31]
// the network inputs, feat[32..39] the odd bases u1, u2; scale[7] the flux
// units.  q arrays in the order rho, vn, vt1, vt2, p, Bt1, Bt2.  Returns J.
template <class T>
__host__ __device__ inline T
encode(const T * qL, const T * qR, T a, T * feat, T * scale)
{
  const T rs = T(0.5) * (qL[0] + qR[0]);
  const T b2L = a * a + qL[5] * qL[5] + qL[6] * qL[6];
  const T b2R = a * a + qR[5] * qR[5] + qR[6] * qR[6];
  const T Ps = T(0.5) * (qL[4] + qR[4]) + T(0.25) * (b2L + b2R);
  const T irs = T(1) / rs, iPs = T(1) / Ps;
  const T vs = sqrt(Ps * irs), bs = sqrt(Ps);
  const T ivs = T(1) / vs, ibs = T(1) / bs;
  T h[7];
  h[0] = T(0.5) * (qR[0] - qL[0]) * irs;
  h[1] = T(0.5) * (qR[1] - qL[1]) * ivs;
  h[2] = T(0.5) * (qR[2] - qL[2]) * ivs;
  h[3] = T(0.5) * (qR[3] - qL[3]) * ivs;
  h[4] = T(0.5) * (qR[4] - qL[4]) * iPs;
  h[5] = T(0.5) * (qR[5] - qL[5]) * ibs;
  h[6] = T(0.5) * (qR[6] - qL[6]) * ibs;
  T J = T(0);
  for (int q = 0; q < 7; ++q)
    J = fmax(J, fabs(h[q]));
  const T sJ = fmax(J, T(kJFloor));
  const T isJ = T(1) / sJ;
  // even scalars
  feat[0] = T(0.5) * (qL[1] + qR[1]) * ivs;
  feat[1] = T(0.5) * (qL[4] + qR[4]) * iPs;
  feat[2] = a * ibs;
  feat[3] = h[0] * isJ;
  feat[4] = h[1] * isJ;
  feat[5] = h[4] * isJ;
  feat[6] = sJ * T(1.0 / kTauRef);
  // odd bases
  T * u1 = feat + kIn;
  T * u2 = feat + kIn + 4;
  u1[0] = T(0.5) * (qL[2] + qR[2]) * ivs;
  u1[1] = T(0.5) * (qL[5] + qR[5]) * ibs;
  u1[2] = h[2] * isJ;
  u1[3] = h[5] * isJ;
  u2[0] = T(0.5) * (qL[3] + qR[3]) * ivs;
  u2[1] = T(0.5) * (qL[6] + qR[6]) * ibs;
  u2[2] = h[3] * isJ;
  u2[3] = h[6] * isJ;
  // their pairwise products (invariant under the reflections)
  int o = 7;
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      feat[o++] = u1[i] * u1[j];
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      feat[o++] = u2[i] * u2[j];
  for (; o < kIn; ++o)
    feat[o] = T(0);
  scale[0] = rs * vs * sJ;
  scale[1] = Ps * vs * sJ;
  scale[2] = Ps * sJ;
  scale[3] = Ps * sJ;
  scale[4] = Ps * sJ;
  scale[5] = bs * vs * sJ;
  scale[6] = bs * vs * sJ;
  return J;
}

// Raw network outputs -> dimensionless dissipation of the 7 flux components
// (rho, E, mn, mt1, mt2, Bt1, Bt2).
template <class T>
__host__ __device__ inline void
combine(const T * y, const T * u, T * Dn)
{
  const T *u1 = u, *u2 = u + 4;
  Dn[0] = y[0];
  Dn[1] = y[1];
  Dn[2] = y[2];
  Dn[3] = y[3] * u1[0] + y[4] * u1[1] + y[5] * u1[2] + y[6] * u1[3];
  Dn[5] = y[7] * u1[0] + y[8] * u1[1] + y[9] * u1[2] + y[10] * u1[3];
  Dn[4] = y[11] * u2[0] + y[12] * u2[1] + y[13] * u2[2] + y[14] * u2[3];
  Dn[6] = y[15] * u2[0] + y[16] * u2[1] + y[17] * u2[2] + y[18] * u2[3];
}

// Physical ideal-MHD flux in the face-normal frame, components (rho, E, mn,
// mt1, mt2, Bt1, Bt2): the flux vector of riemann_hlld
// (RiemannSolvers_MHD.h:358-366).
template <class T>
__host__ __device__ inline void
physical_flux(const T * q, T a, T gamma0, T * F)
{
  const T r = q[0], u = q[1], v = q[2], w = q[3], p = q[4], b = q[5], c = q[6];
  const T B2 = a * a + b * b + c * c;
  const T Ptot = p + T(0.5) * B2;
  const T E = p / (gamma0 - T(1)) + T(0.5) * r * (u * u + v * v + w * w) + T(0.5) * B2;
  const T vB = u * a + v * b + w * c;
  F[0] = r * u;
  F[1] = (E + Ptot) * u - a * vB;
  F[2] = r * u * u + Ptot - a * a;
  F[3] = r * u * v - a * b;
  F[4] = r * u * w - a * c;
  F[5] = b * u - a * v;
  F[6] = c * u - a * w;
}

template <class T>
__host__ __device__ inline void
central_flux(const T * qL, const T * qR, T a, T gamma0, T * Fc)
{
  T FL[7], FR[7];
  physical_flux(qL, a, gamma0, FL);
  physical_flux(qR, a, gamma0, FR);
  for (int q = 0; q < 7; ++q)
    Fc[q] = T(0.5) * (FL[q] + FR[q]);
}

// |D / scale| above this is treated as a failed prediction.
constexpr float kDissBound = 16.0f;

// ---------------------------------------------------------------- device

#ifdef __CUDACC__

constexpr float kGeluC0 = 0.7978845608028654f; // sqrt(2/pi)
constexpr float kGeluC1 = 0.044715f;

__device__ __forceinline__ float
tanh_hw(float x)
{
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// GELU with the hardware tanh approximation in FP32.
__device__ __forceinline__ float
gelu_hw(float x)
{
  const float u = x * (kGeluC0 + (kGeluC0 * kGeluC1) * x * x);
  const float hx = 0.5f * x;
  return fmaf(hx, tanh_hw(u), hx);
}

// The deployed activation: GELU evaluated in BF16 arithmetic on a BF16
// input, two lanes per instruction (x^2, x (c0 + c0 c1 x^2), tanh, x/2 (1 +
// tanh)).  gelu_bf16 is the same sequence on one value, for training.
__device__ __forceinline__ uint32_t
tanh_bf16x2(uint32_t x)
{
  uint32_t y;
  asm("tanh.approx.bf16x2 %0, %1;" : "=r"(y) : "r"(x));
  return y;
}

__device__ __forceinline__ unsigned short
tanh_bf16(unsigned short x)
{
  unsigned short y;
  asm("tanh.approx.bf16 %0, %1;" : "=h"(y) : "h"(x));
  return y;
}

__device__ __forceinline__ uint32_t
gelu_bf16x2(uint32_t xw)
{
  const __nv_bfloat162 x = *reinterpret_cast<const __nv_bfloat162 *>(&xw);
  const __nv_bfloat162 c0 = __float2bfloat162_rn(kGeluC0);
  const __nv_bfloat162 c01 = __float2bfloat162_rn(kGeluC0 * kGeluC1);
  const __nv_bfloat162 h = __float2bfloat162_rn(0.5f);
  const __nv_bfloat162 u = __hmul2(x, __hfma2(__hmul2(x, x), c01, c0));
  const uint32_t       uw = *reinterpret_cast<const uint32_t *>(&u);
  const uint32_t       tw = tanh_bf16x2(uw);
  const __nv_bfloat162 t = *reinterpret_cast<const __nv_bfloat162 *>(&tw);
  const __nv_bfloat162 hx = __hmul2(x, h);
  const __nv_bfloat162 g = __hfma2(hx, t, hx);
  return *reinterpret_cast<const uint32_t *>(&g);
}

__device__ __forceinline__ float
gelu_bf16(float z)
{
  const __nv_bfloat16 x = __float2bfloat16_rn(z);
  const __nv_bfloat16 c0 = __float2bfloat16_rn(kGeluC0);
  const __nv_bfloat16 c01 = __float2bfloat16_rn(kGeluC0 * kGeluC1);
  const __nv_bfloat16 h = __float2bfloat16_rn(0.5f);
  const __nv_bfloat16 u = __hmul(x, __hfma(__hmul(x, x), c01, c0));
  const __nv_bfloat16 t = __ushort_as_bfloat16(tanh_bf16(__bfloat16_as_ushort(u)));
  const __nv_bfloat16 hx = __hmul(x, h);
  return __bfloat162float(__hfma(hx, t, hx));
}

__device__ __forceinline__ uint32_t
pack_bf16x2(float lo, float hi)
{
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ void
mma_16816(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
  asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 "
               "{%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
               : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
               : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// Shared staging of one warp: 32 input rows of 32 bf16 (row stride 20
// words: conflict-free fragment reads) and 32 output rows of 24 floats.
constexpr int kStageRow = 20;
constexpr int kStageXWords = 32 * kStageRow;
constexpr int kStageORow = kOut + 1;
constexpr int kStageOFloats = 32 * kStageORow;

// C fragments (two adjacent 8-wide n-tiles) -> A fragment of the next layer,
// with the activation applied.
__device__ __forceinline__ void
act_to_a(const float (&c0)[4], const float (&c1)[4], uint32_t (&a)[4])
{
  a[0] = gelu_bf16x2(pack_bf16x2(c0[0], c0[1]));
  a[1] = gelu_bf16x2(pack_bf16x2(c0[2], c0[3]));
  a[2] = gelu_bf16x2(pack_bf16x2(c1[0], c1[1]));
  a[3] = gelu_bf16x2(pack_bf16x2(c1[2], c1[3]));
}

// Forward pass of the network for the 32 faces of a warp (one per lane);
// every lane of the warp must call it.  wp: packed weights (shared), bias:
// b1, b2, b3 (shared), sx / so: this warp's staging; x: this lane's inputs,
// out: its raw outputs.
__device__ __forceinline__ void
warp_forward(const uint32_t * __restrict__ wp, const float * __restrict__ bias, uint32_t * sx,
             float * so, const float (&x)[kIn], float (&out)[kOut])
{
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int q = 0; q < kIn / 2; ++q)
    sx[lane * kStageRow + q] = pack_bf16x2(x[2 * q], x[2 * q + 1]);
  __syncwarp();
  const uint2 * W1 = reinterpret_cast<const uint2 *>(wp + kPackW1);
  const uint2 * W2 = reinterpret_cast<const uint2 *>(wp + kPackW2);
  const uint2 * W3 = reinterpret_cast<const uint2 *>(wp + kPackW3);
  const float * b1 = bias;
  const float * b2 = bias + kHid;
  const float * b3 = bias + 2 * kHid;
#pragma unroll 1
  for (int mt = 0; mt < 2; ++mt)
  {
    const int r0 = mt * 16 + g, r1 = r0 + 8;
    float     c[8][4];
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
      const float x0 = b1[nt * 8 + 2 * t], x1 = b1[nt * 8 + 2 * t + 1];
      c[nt][0] = x0;
      c[nt][1] = x1;
      c[nt][2] = x0;
      c[nt][3] = x1;
    }
#pragma unroll
    for (int kt = 0; kt < kIn / 16; ++kt)
    {
      const int      w0 = kt * 8;
      const uint32_t a[4] = { sx[r0 * kStageRow + w0 + t], sx[r1 * kStageRow + w0 + t],
                              sx[r0 * kStageRow + w0 + t + 4], sx[r1 * kStageRow + w0 + t + 4] };
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
      {
        const uint2 w = W1[(kt * 8 + nt) * 32 + lane];
        mma_16816(c[nt], a, w.x, w.y);
      }
    }
    uint32_t h[4][4];
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
      act_to_a(c[2 * kt], c[2 * kt + 1], h[kt]);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt)
    {
      const float x0 = b2[nt * 8 + 2 * t], x1 = b2[nt * 8 + 2 * t + 1];
      c[nt][0] = x0;
      c[nt][1] = x1;
      c[nt][2] = x0;
      c[nt][3] = x1;
#pragma unroll
      for (int kt = 0; kt < 4; ++kt)
      {
        const uint2 w = W2[(kt * 8 + nt) * 32 + lane];
        mma_16816(c[nt], h[kt], w.x, w.y);
      }
    }
#pragma unroll
    for (int kt = 0; kt < 4; ++kt)
      act_to_a(c[2 * kt], c[2 * kt + 1], h[kt]);
#pragma unroll
    for (int nt = 0; nt < kOut / 8; ++nt)
    {
      float y[4] = { b3[nt * 8 + 2 * t], b3[nt * 8 + 2 * t + 1], b3[nt * 8 + 2 * t],
                     b3[nt * 8 + 2 * t + 1] };
#pragma unroll
      for (int kt = 0; kt < 4; ++kt)
      {
        const uint2 w = W3[(kt * (kOut / 8) + nt) * 32 + lane];
        mma_16816(y, h[kt], w.x, w.y);
      }
      so[r0 * kStageORow + nt * 8 + 2 * t] = y[0];
      so[r0 * kStageORow + nt * 8 + 2 * t + 1] = y[1];
      so[r1 * kStageORow + nt * 8 + 2 * t] = y[2];
      so[r1 * kStageORow + nt * 8 + 2 * t + 1] = y[3];
    }
  }
  __syncwarp();
#pragma unroll
  for (int o = 0; o < kOut; ++o)
    out[o] = so[lane * kStageORow + o];
  __syncwarp();
}

// ---------------------------------------------------------------- tcgen05 batch forward

// Shared memory of one 128-thread block running the network on the 5th-
// generation tensor cores: the tcgen05 network image (kTcWBytes of weights,
// then the biases), the activation tile (128 rows x 64 bf16, canonical
// layout; the 32-wide input tile uses its first half), the mbarrier and the
// TMEM address slot.
constexpr int      kTcRows = 128;
constexpr int      kTcAct = kTcWBytes + ((kBiasFloats * 4 + 127) / 128) * 128;
constexpr int      kTcBar = kTcAct + kTcRows * kHid * 2;
constexpr int      kTcSmemBytes = kTcBar + 16;
constexpr uint32_t kTcCols = 64; // TMEM columns per block (FP32 accumulators)
constexpr int      kTcWaitPolls = 1 << 20;

// The persistent form: 256-thread blocks of two independent 128-row
// pipelines, each with its own activation tile, mbarrier, named barrier
// (1 + pipeline) and kTcCols TMEM columns, sharing one copy of the network
// image.  Shared memory: image, activation tiles 0 and 1, mbarriers 0 and
// 1, the TMEM address slot.  At most 4 blocks fit an SM by shared memory,
// which keeps 4 x kTc2Cols within the SM's 512 TMEM columns.
constexpr int      kTc2Threads = 2 * kTcRows;
constexpr int      kTc2Act = kTcAct;
constexpr int      kTc2ActBytes = kTcRows * kHid * 2;
constexpr int      kTc2Bar = kTc2Act + 2 * kTc2ActBytes;
constexpr int      kTc2SmemBytes = kTc2Bar + 24;
constexpr uint32_t kTc2Cols = 2 * kTcCols;
// (an SM has 228 KB of shared memory, of which each block reserves 1 KB)
static_assert(5 * (kTc2SmemBytes + 1024) > 228 * 1024, "at most 4 blocks of the persistent form per SM");

__device__ __forceinline__ void
stage_network_tc(const uint32_t * __restrict__ pack, unsigned char * smem)
{
  const uint4 * src = reinterpret_cast<const uint4 *>(pack);
  uint4 *       dst = reinterpret_cast<uint4 *>(smem);
  for (int q = threadIdx.x; q < kTcWBytes / 16; q += blockDim.x)
    dst[q] = src[q];
  float *       b = reinterpret_cast<float *>(smem + kTcWBytes);
  const float * bs = reinterpret_cast<const float *>(pack + kTcWBytes / 4);
  for (int q = threadIdx.x; q < kBiasFloats; q += blockDim.x)
    b[q] = bs[q];
}

// Hidden-layer epilogue of row r: z = accumulator + bias, gelu in BF16, the
// result written as row r of the next layer's A tile (K = 64).
__device__ __forceinline__ void
hidden_epilogue(uint32_t trow, const float * bias, unsigned char * act, int r)
{
#pragma unroll
  for (int half = 0; half < 2; ++half)
  {
    uint32_t v[32];
    umma::ld32(trow + 32 * half, v);
    // the biases as 16-byte shared loads (the image's bias block is
    // 16-byte aligned): a quarter of the load instructions
    const float4 * b4 = reinterpret_cast<const float4 *>(bias + 32 * half);
    uint32_t       w[16];
#pragma unroll
    for (int q4 = 0; q4 < 8; ++q4)
    {
      const float4 b = b4[q4];
      w[2 * q4] = gelu_bf16x2(pack_bf16x2(__uint_as_float(v[4 * q4]) + b.x,
                                          __uint_as_float(v[4 * q4 + 1]) + b.y));
      w[2 * q4 + 1] = gelu_bf16x2(pack_bf16x2(__uint_as_float(v[4 * q4 + 2]) + b.z,
                                              __uint_as_float(v[4 * q4 + 3]) + b.w));
    }
#pragma unroll
    for (int kc = 0; kc < 4; ++kc)
      *reinterpret_cast<uint4 *>(act + umma::canon_offset(r, 32 * half + 8 * kc, kHid)) =
        make_uint4(w[4 * kc], w[4 * kc + 1], w[4 * kc + 2], w[4 * kc + 3]);
  }
}

// OR of pred over the 128 threads of one pipeline, which synchronise on the
// named barrier kBarId (0 with a 128-thread block is __syncthreads_or).  The
// id is a compile-time constant so that a kernel reserves only the barriers
// it names.
template <int kBarId>
__device__ __forceinline__ bool
group_sync_or(bool pred)
{
  uint32_t out;
  asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\t"
               "bar.red.or.pred q, %2, 128, p;\n\tselp.u32 %0, 1, 0, q;\n\t}\n"
               : "=r"(out)
               : "r"((uint32_t)pred), "n"(kBarId)
               : "memory");
  return out != 0;
}

// Forward pass of 128 rows on the tensor cores, one row per thread of a
// 128-thread pipeline (row r = TMEM lane r; the pipeline's warps are four
// consecutive warps of the block, so warp w reads lanes 32 (w % 4) ..).
// Every thread of the pipeline must call it.  smem: the network image
// (weights, then biases); act: the pipeline's activation tile; mbar: its
// mbarrier; kBarId: its named barrier.  x: this row's inputs; y: its raw
// outputs (biases included).  tmem: the pipeline's kTcCols TMEM columns;
// parity: the mbarrier phase to wait for next (advanced by three on
// success).  Row 0 issues each layer's MMAs (M = 128, K = 16 per
// instruction) and commits them to the mbarrier; every thread then moves its
// row from TMEM through bias and activation into the next A tile.  Numerics
// are those of warp_forward: BF16 operands, FP32 accumulation, bias added in
// FP32, BF16 GELU.  Returns false, for every thread, when a wait reached its
// limit: the outputs are then invalid, the pending phase has been waited for
// once more (bounded) and the caller must stop using the pipeline and free
// TMEM.  polls bounds each layer's wait (the drain always allows
// kTcWaitPolls).
template <int kBarId>
__device__ __forceinline__ bool
block_forward(unsigned char * smem, unsigned char * act, uint32_t mbar, int r, uint32_t tmem,
              uint32_t & parity, const float (&x)[kIn], float (&y)[kOut],
              int polls = kTcWaitPolls)
{
  const float *   bias = reinterpret_cast<const float *>(smem + kTcWBytes);
  const uint32_t  trow = tmem + ((uint32_t)(r & ~31) << 16); // the warp's lane quarter
  const uint32_t  a0 = umma::smem_addr(act), w0 = umma::smem_addr(smem);
#pragma unroll
  for (int kc = 0; kc < kIn / 8; ++kc)
    *reinterpret_cast<uint4 *>(act + umma::canon_offset(r, 8 * kc, kIn)) =
      make_uint4(pack_bf16x2(x[8 * kc], x[8 * kc + 1]), pack_bf16x2(x[8 * kc + 2], x[8 * kc + 3]),
                 pack_bf16x2(x[8 * kc + 4], x[8 * kc + 5]), pack_bf16x2(x[8 * kc + 6], x[8 * kc + 7]));
  bool ok = true;
#pragma unroll 1
  for (int layer = 0; layer < 3; ++layer)
  {
    // generic stores of the A tile -> tensor-core reads; every thread's
    // TMEM loads of the previous layer -> this layer's accumulator writes
    umma::fence_proxy_async();
    umma::fence_before_sync();
    const bool failed = group_sync_or<kBarId>(!ok);
    umma::fence_after_sync();
    if (failed)
    {
      // drain: a thread whose wait gave up waits once more for that phase
      if (!ok)
        umma::mbar_wait(mbar, parity, kTcWaitPolls);
      return false;
    }
    if (r == 0)
    {
      const int      K = layer == 0 ? kIn : kHid;
      const int      N = layer == 2 ? kN3 : kHid;
      const uint32_t wl = w0 + (layer == 0 ? kTcW1 : layer == 1 ? kTcW2 : kTcW3);
      const uint32_t idesc = umma::idesc_bf16_f32(kTcRows, N);
      for (int ks = 0; ks < K / 16; ++ks)
        umma::mma_bf16(tmem, umma::desc_kmajor(a0 + ks * 2 * umma::kLBO, K * 16),
                       umma::desc_kmajor(wl + ks * 2 * umma::kLBO, K * 16), idesc, ks > 0);
      umma::commit(mbar);
    }
    ok = umma::mbar_wait(mbar, parity, polls);
    umma::fence_after_sync();
    if (ok)
    {
      parity ^= 1u;
      if (layer < 2)
        hidden_epilogue(trow, bias + layer * kHid, act, r);
      else
      {
        uint32_t v[32];
        umma::ld32(trow, v);
        const float4 * b4 = reinterpret_cast<const float4 *>(bias + 2 * kHid);
#pragma unroll
        for (int o4 = 0; o4 < kOut / 4; ++o4)
        {
          const float4 b = b4[o4];
          y[4 * o4] = __uint_as_float(v[4 * o4]) + b.x;
          y[4 * o4 + 1] = __uint_as_float(v[4 * o4 + 1]) + b.y;
          y[4 * o4 + 2] = __uint_as_float(v[4 * o4 + 2]) + b.z;
          y[4 * o4 + 3] = __uint_as_float(v[4 * o4 + 3]) + b.w;
        }
      }
    }
  }
  umma::fence_before_sync();
  const bool failed = group_sync_or<kBarId>(!ok);
  umma::fence_after_sync();
  if (failed && !ok)
    umma::mbar_wait(mbar, parity, kTcWaitPolls);
  return !failed;
}

#endif // __CUDACC__

} // namespace mlp
} // namespace mhd
