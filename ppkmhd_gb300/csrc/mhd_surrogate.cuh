// Solver-side kernels of the HLLD flux surrogate (mhd_mlp.cuh):
//  * k_harvest: face samples of the current iteration for training, each
//    with the FP64 dissipation target D = Fc - F_HLLD;
//  * k_flux_mlp + k_flux_fallback: the face-flux stage of the iteration
//    (replacing k_flux): the network on faces the jump sensor flags as
//    smooth, and HLLD, in a second kernel, on the faces it lists as not.
// Both rebuild the face states exactly as k_flux does (face_states, the
// reconstruction of ComputeFluxAndUpdateAlongDirFunctor, MHDRunFunctors2D.h:
// 1110-1190, 3D:1097-1210).
#pragma once

#include "mhd_kernels.cuh"
#include "mhd_mlp.cuh"

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

// normal-frame State -> (rho, vn, vt1, vt2, p, Bt1, Bt2), a
template <class R, class T>
__device__ __forceinline__ void
to_face7(const State<R> & q, T * o)
{
  o[0] = T(q[ID]);
  o[1] = T(q[IU]);
  o[2] = T(q[IV]);
  o[3] = T(q[IW]);
  o[4] = T(q[IP]);
  o[5] = T(q[IB]);
  o[6] = T(q[IC]);
}

template <class R, int DIM, int d>
__device__ __forceinline__ void
harvest_face(const Grid<R> & G, const Buffers<R> & B, int64_t c, float * rec)
{
  State<R> qL, qR;
  face_states<R, DIM, d>(G, B, c, qL, qR);
  double l7[7], r7[7];
  to_face7(qL, l7);
  to_face7(qR, r7);
  const double a = double(qL[IA]);
  double       f[mlp::kIn], sc[7], Fc[7];
  const double J = mlp::encode(l7, r7, a, f, sc);
  mlp::central_flux(l7, r7, a, double(G.gamma0), Fc);
  // FP64 HLLD of the (working-precision) face states
  State<double> dl, dr, fl;
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    dl[v] = double(qL[v]);
    dr[v] = double(qR[v]);
    fl[v] = 0.0;
  }
  riemann_hlld(dl, dr, fl, double(G.gamma0), 1.0 / (double(G.gamma0) - 1.0));
  const double Fh[7] = { fl[ID], fl[IP], fl[IU], fl[IV], fl[IW], fl[IB], fl[IC] };
#pragma unroll
  for (int q = 0; q < 7; ++q)
  {
    rec[mlp::kRecQL + q] = float(l7[q]);
    rec[mlp::kRecQR + q] = float(r7[q]);
    rec[mlp::kRecD + q] = float(Fc[q] - Fh[q]);
  }
  rec[mlp::kRecA] = float(a);
  rec[mlp::kRecJ] = float(J);
  rec[mlp::kRecGamma] = float(G.gamma0);
}

// One record per `stride`-th face of each direction:
// out[(dir * nslot + s) * kRecord ...] for face index s * stride.
template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_harvest(const Grid<R> G, Buffers<R> B, float * __restrict__ out, int stride, int64_t nslot)
{
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= nslot)
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], s * stride, i, j, k))
    return;
  const int     dir = blockIdx.y;
  const int64_t c = cell_at(G, i, j, k);
  float *       rec = out + ((int64_t)dir * nslot + s) * mlp::kRecord;
  if (dir == 0)
    harvest_face<R, DIM, 0>(G, B, c, rec);
  else if (dir == 1)
    harvest_face<R, DIM, 1>(G, B, c, rec);
  else if constexpr (DIM == 3)
    harvest_face<R, DIM, 2>(G, B, c, rec);
}

// Device parameters of a deployed surrogate.
struct SurrogateDev
{
  const uint32_t *     wpack; // mlp::kPackWords
  const float *        bias;  // mlp::kBiasFloats
  float                tau;   // sensor threshold on J
  unsigned long long * count; // [0] faces given by the network, [1] faces computed
  uint32_t *           list;  // faces left to HLLD: face index * DIM + direction
  unsigned *           nlist; // number of entries (reset before each flux stage)
};

constexpr int kMlpThreads = 128;
constexpr int kStash = 23; // per lane: Fc[7], scale[7], u[8], pad (odd stride)
constexpr int kMlpSmemShared = ((mlp::kPackWords + mlp::kBiasFloats) * 4 + 15) / 16 * 16;
constexpr int kMlpSmemPerWarp = (mlp::kStageXWords + mlp::kStageOFloats + 32 * kStash) * 4;
constexpr int kMlpSmemBytes = kMlpSmemShared + (kMlpThreads / 32) * kMlpSmemPerWarp;

// Encoding of mlp::encode in FP32 with hardware reciprocals and rsqrt:
// feat[0..31] network inputs, feat[32..39] odd bases, scale[7].
__device__ __forceinline__ float
encode_fast(const float * qL, const float * qR, float a, float * feat, float * scale)
{
  const float rs = 0.5f * (qL[0] + qR[0]);
  const float b2L = a * a + qL[5] * qL[5] + qL[6] * qL[6];
  const float b2R = a * a + qR[5] * qR[5] + qR[6] * qR[6];
  const float Ps = 0.5f * (qL[4] + qR[4]) + 0.25f * (b2L + b2R);
  const float irs = rcp(rs), iPs = rcp(Ps);
  const float ibs = rsq(Ps), bs = Ps * ibs;
  const float ivs = rs * rsq(rs) * ibs, vs = Ps * ivs * irs; // sqrt(rs / Ps), sqrt(Ps / rs)
  float       h[7];
  h[0] = 0.5f * (qR[0] - qL[0]) * irs;
  h[1] = 0.5f * (qR[1] - qL[1]) * ivs;
  h[2] = 0.5f * (qR[2] - qL[2]) * ivs;
  h[3] = 0.5f * (qR[3] - qL[3]) * ivs;
  h[4] = 0.5f * (qR[4] - qL[4]) * iPs;
  h[5] = 0.5f * (qR[5] - qL[5]) * ibs;
  h[6] = 0.5f * (qR[6] - qL[6]) * ibs;
  float J = 0.f;
#pragma unroll
  for (int q = 0; q < 7; ++q)
    J = fmaxf(J, fabsf(h[q]));
  const float sJ = fmaxf(J, float(mlp::kJFloor));
  const float isJ = rcp(sJ);
  feat[0] = 0.5f * (qL[1] + qR[1]) * ivs;
  feat[1] = 0.5f * (qL[4] + qR[4]) * iPs;
  feat[2] = a * ibs;
  feat[3] = h[0] * isJ;
  feat[4] = h[1] * isJ;
  feat[5] = h[4] * isJ;
  feat[6] = sJ * float(1.0 / mlp::kTauRef);
  float * u1 = feat + mlp::kIn;
  float * u2 = feat + mlp::kIn + 4;
  u1[0] = 0.5f * (qL[2] + qR[2]) * ivs;
  u1[1] = 0.5f * (qL[5] + qR[5]) * ibs;
  u1[2] = h[2] * isJ;
  u1[3] = h[5] * isJ;
  u2[0] = 0.5f * (qL[3] + qR[3]) * ivs;
  u2[1] = 0.5f * (qL[6] + qR[6]) * ibs;
  u2[2] = h[3] * isJ;
  u2[3] = h[6] * isJ;
  int o = 7;
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i; j < 4; ++j)
      feat[o++] = u1[i] * u1[j];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = i; j < 4; ++j)
      feat[o++] = u2[i] * u2[j];
#pragma unroll
  for (int q = mlp::kInUsed; q < mlp::kIn; ++q)
    feat[q] = 0.f;
  const float rvs = rs * vs * sJ, pvs = Ps * vs * sJ, ps = Ps * sJ, bvs = bs * vs * sJ;
  scale[0] = rvs;
  scale[1] = pvs;
  scale[2] = ps;
  scale[3] = ps;
  scale[4] = ps;
  scale[5] = bvs;
  scale[6] = bvs;
  return J;
}

// Central flux (F(qL) + F(qR)) / 2 with 1 / (gamma - 1) given; the momentum
// component minus the total-pressure shift p0 (flux_shift), as the HLLD
// fallback faces store it.
__device__ __forceinline__ void
central_flux_fast(const float * qL, const float * qR, float a, float igm1, float * Fc, float p0)
{
  float F[7] = { 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f };
#pragma unroll
  for (int side = 0; side < 2; ++side)
  {
    const float * q = side ? qR : qL;
    const float   r = q[0], u = q[1], v = q[2], w = q[3], p = q[4], b = q[5], c = q[6];
    const float   B2 = a * a + b * b + c * c;
    const float   Pt = p + 0.5f * B2;
    const float   Ps = (p - p0) + 0.5f * B2;
    const float   E = p * igm1 + 0.5f * r * (u * u + v * v + w * w) + 0.5f * B2;
    const float   vB = u * a + v * b + w * c;
    F[0] += r * u;
    F[1] += (E + Pt) * u - a * vB;
    F[2] += r * u * u + Ps - a * a;
    F[3] += r * u * v - a * b;
    F[4] += r * u * w - a * c;
    F[5] += b * u - a * v;
    F[6] += c * u - a * w;
  }
#pragma unroll
  for (int q = 0; q < 7; ++q)
    Fc[q] = 0.5f * F[q];
}

// One face of the surrogate flux stage.  Returns true when the face must
// be computed by HLLD (not smooth, at a floor, or a failed prediction).
// Per-lane values (central flux, output scales, odd bases) are kept in
// shared memory across the network evaluation, which frees registers for
// the tensor-core fragments.

template <int DIM, int d>
__device__ __forceinline__ bool
flux_face_mlp(const Grid<float> & G, const Buffers<float> & B, const SurrogateDev & S, bool valid,
              int64_t c, const uint32_t * sw, const float * sb, uint32_t * sx, float * so,
              float * stash)
{
  float     f[mlp::kFeat];
  bool      smooth = false;
  const int lane = threadIdx.x & 31;
  float *   my = stash + lane * kStash;
  if (valid)
  {
    State<float> qL, qR;
    face_states<float, DIM, d>(G, B, c, qL, qR);
    B.H[c + d * G.sv] = qR[IA]; // half-step normal field of the face
    float l7[7], r7[7], sc[7], Fc[7];
    to_face7(qL, l7);
    to_face7(qR, r7);
    const float a = qL[IA];
    const float J = encode_fast(l7, r7, a, f, sc);
    // positivity: no reconstructed density or pressure at its floor
    const float smallR = G.smallr, smallp = G.smallp;
    smooth = J <= S.tau && l7[0] > smallR && r7[0] > smallR && l7[4] > smallp * l7[0] &&
             r7[4] > smallp * r7[0];
    central_flux_fast(l7, r7, a, rcp(G.gamma0 - 1.f), Fc, flux_shift(B.st, 0.f));
#pragma unroll
    for (int q = 0; q < 7; ++q)
    {
      my[q] = Fc[q];
      my[7 + q] = sc[q];
    }
#pragma unroll
    for (int q = 0; q < mlp::kBasis; ++q)
      my[14 + q] = f[mlp::kIn + q];
  }
  if (!__any_sync(0xffffffffu, smooth))
    return valid;
  float x[mlp::kIn];
#pragma unroll
  for (int q = 0; q < mlp::kIn; ++q)
    x[q] = smooth ? f[q] : 0.f;
  float y[mlp::kOut];
  mlp::warp_forward(sw, sb, sx, so, x, y);
  if (!smooth)
    return valid;
  float u[mlp::kBasis], Dn[mlp::kOutUsed];
#pragma unroll
  for (int q = 0; q < mlp::kBasis; ++q)
    u[q] = my[14 + q];
  mlp::combine(y, u, Dn);
  bool ok = true;
#pragma unroll
  for (int q = 0; q < 7; ++q)
    ok = ok && isfinite(Dn[q]) && fabsf(Dn[q]) <= mlp::kDissBound;
  if (!ok)
    return true;
  State<float> fl;
  fl[ID] = my[0] - my[7] * Dn[0];
  fl[IP] = my[1] - my[8] * Dn[1];
  fl[IU] = my[2] - my[9] * Dn[2];
  fl[IV] = my[3] - my[10] * Dn[3];
  fl[IW] = my[4] - my[11] * Dn[4];
  fl[IA] = 0.f;
  fl[IB] = my[5] - my[12] * Dn[5];
  fl[IC] = my[6] - my[13] * Dn[6];
  store_face_flux<float, DIM, d>(G, B, c, fl);
  return false;
}

// Face fluxes by the network; blockIdx.y = direction, grid-stride loop over
// the faces so the weights are staged in shared memory once per block.
// Faces the network does not answer are appended to S.list.
template <int DIM>
__global__ void __launch_bounds__(kMlpThreads, 3)
k_flux_mlp(const Grid<float> G, Buffers<float> B, const SurrogateDev S)
{
  // dynamic shared memory (kMlpSmemBytes): weights, biases, then per warp
  // the input staging, the output staging and the stash
  extern __shared__ __align__(16) unsigned char smem[];
  uint32_t * sw = reinterpret_cast<uint32_t *>(smem);
  float *    sb = reinterpret_cast<float *>(sw + mlp::kPackWords);
  const int  warp = threadIdx.x >> 5;
  unsigned char * wbase = smem + kMlpSmemShared + (size_t)warp * kMlpSmemPerWarp;
  uint32_t * sx = reinterpret_cast<uint32_t *>(wbase);
  float *    so = reinterpret_cast<float *>(sx + mlp::kStageXWords);
  float *    stash = so + mlp::kStageOFloats;
  for (int q = threadIdx.x; q < mlp::kPackWords; q += blockDim.x)
    sw[q] = S.wpack[q];
  for (int q = threadIdx.x; q < mlp::kBiasFloats; q += blockDim.x)
    sb[q] = S.bias[q];
  __syncthreads();
  if (step_finished(B.st))
    return;
  const int     dir = blockIdx.y, lane = threadIdx.x & 31;
  const Box &   bx = G.box[BOX_FACE];
  const int64_t n = bx.count();
  unsigned      used = 0, total = 0;
  for (int64_t base = blockIdx.x * (int64_t)blockDim.x; base < n;
       base += (int64_t)gridDim.x * blockDim.x)
  {
    int           i = 0, j = 0, k = 0;
    const int64_t idx = base + threadIdx.x;
    const bool    valid = box_cell(bx, idx, i, j, k);
    const int64_t c = valid ? cell_at(G, i, j, k) : 0;
    bool          rest;
    if (dir == 0)
      rest = flux_face_mlp<DIM, 0>(G, B, S, valid, c, sw, sb, sx, so, stash);
    else if (dir == 1)
      rest = flux_face_mlp<DIM, 1>(G, B, S, valid, c, sw, sb, sx, so, stash);
    else
      rest = flux_face_mlp<DIM, DIM == 3 ? 2 : 1>(G, B, S, valid, c, sw, sb, sx, so, stash);
    total += valid ? 1u : 0u;
    used += (valid && !rest) ? 1u : 0u;
    // warp-aggregated append of the faces left to HLLD
    const unsigned m = __ballot_sync(0xffffffffu, rest);
    if (m)
    {
      unsigned first = 0;
      if (lane == __ffs(m) - 1)
        first = atomicAdd(S.nlist, (unsigned)__popc(m));
      first = __shfl_sync(0xffffffffu, first, __ffs(m) - 1);
      if (rest)
        S.list[first + __popc(m & ((1u << lane) - 1u))] = (uint32_t)(idx * DIM + dir);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
  {
    used += __shfl_xor_sync(0xffffffffu, used, o);
    total += __shfl_xor_sync(0xffffffffu, total, o);
  }
  if (lane == 0 && S.count)
  {
    atomicAdd(&S.count[0], (unsigned long long)used);
    atomicAdd(&S.count[1], (unsigned long long)total);
  }
}

// HLLD on the faces the network left (the list of k_flux_mlp).
template <int DIM>
__global__ void __launch_bounds__(128)
k_flux_fallback(const Grid<float> G, Buffers<float> B, const uint32_t * __restrict__ list,
                const unsigned * __restrict__ nlist)
{
  if (step_finished(B.st))
    return;
  const unsigned n = *nlist;
  for (unsigned q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x)
  {
    const uint32_t e = list[q];
    const int      dir = (int)(e % DIM);
    int            i, j, k;
    if (!box_cell(G.box[BOX_FACE], (int64_t)(e / DIM), i, j, k))
      continue;
    if (dir == 0)
      flux_face<float, DIM, 0>(G, B, i, j, k);
    else if (dir == 1)
      flux_face<float, DIM, 1>(G, B, i, j, k);
    else if constexpr (DIM == 3)
      flux_face<float, DIM, 2>(G, B, i, j, k);
  }
}

} // namespace MHD_VARIANT_TAG
} // namespace mhd
