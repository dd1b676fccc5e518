// Training and evaluation of the HLLD flux surrogate (mhd_mlp.cuh) on the
// GPU: feature encoding of harvested face samples, forward + backward passes
// with per-block partial gradients reduced in a fixed order, Adam, and the
// tensor-core forward passes (the warp-level one of the flux stage is in
// mhd_mlp.cuh; the tcgen05 batch forward below).  Exposed through the
// mhd_mlp_* entry points of include/ppkmhd_gb300.h.
//
// Training arithmetic: FP32 master weights; in MHD_MLP_TRAIN mode the
// forward pass sees BF16 weights and inputs and the deployed BF16 GELU
// (gelu_bf16: the same operations as the tensor-core path), and the
// backward pass differentiates the FP32 GELU (rounding as the identity).  MHD_MLP_CHECK mode
// is plain FP32 with tanhf (for gradient checks against the CPU oracle).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "mhd_core.h"
#include "mhd_mlp.cuh"
#include "ppkmhd_gb300.h"

using namespace mhd::mlp;

static_assert(mhd::kMlpPackTotal == kPackWords + kBiasFloats, "packed surrogate size");
static_assert(kParams == MHD_MLP_PARAMS, "surrogate parameter count");
static_assert(kRecord == MHD_SAMPLE_FLOATS, "face record size");
static_assert(kFeat == MHD_MLP_FEATURES, "face feature count");
static_assert(kTcWaitPolls == MHD_MLP_WAIT_POLLS, "default tensor-core wait bound");
static_assert(kFeat % 4 == 0 && kIn % 4 == 0 && kBasis % 4 == 0 && kOutUsed == 7,
              "16-byte feature and output groups");

struct mhd_mlp
{
  int          device = 0;
  double       gamma0 = 5.0 / 3.0;
  std::vector<float> params; // host copy of the master weights (kept in sync)
  int          wait_polls = kTcWaitPolls; // bound of the tensor-core completion waits
  int          forward_form = MHD_MLP_FORWARD_PERSISTENT;
  double       last_forward_ms = -1.0; // device time of the last batch forward kernel
  float *      d_params = nullptr;
  float *      d_m = nullptr;
  float *      d_v = nullptr;
  cudaStream_t stream = nullptr;
  std::string  err;
  int64_t      adam_step = 0;
};

namespace
{

constexpr int kTB = 64; // samples per training block
constexpr int kTgt = 8; // target / prediction stride: 7 flux components + pad
constexpr int kRowX = 0;                      // inputs [kIn]
constexpr int kRowZ1 = kRowX + kIn;           // layer-1 pre-activations, then their gradient
constexpr int kRowH1 = kRowZ1 + kHid;         // layer-1 activations
constexpr int kRowZ2 = kRowH1 + kHid;         // layer-2 pre-activations, then their gradient
constexpr int kRowH2 = kRowZ2 + kHid;         // layer-2 activations
constexpr int kRowU = kRowH2 + kHid;          // odd bases [kBasis]
constexpr int kRowY = kRowU + kBasis;         // gradient of the raw outputs [kOut]
constexpr int kRowLoss = kRowY + kOut;
constexpr int kRowStride = kRowLoss + 1;      // 321, odd: conflict-free columns
constexpr int kSmemTrain = (kParams + kTB * kRowStride) * (int)sizeof(float);

__device__ __forceinline__ float
bf16_round(float x)
{
  return __bfloat162float(__float2bfloat16_rn(x));
}

__device__ __forceinline__ float
gelu_exact(float x)
{
  return 0.5f * x * (1.0f + tanhf(kGeluC0 * (x + kGeluC1 * x * x * x)));
}

// d/dx of the tanh-form GELU, with the tanh of the same flavour as the forward pass
__device__ __forceinline__ float
gelu_grad(float x, int train)
{
  const float u = kGeluC0 * (x + kGeluC1 * x * x * x);
  const float t = train ? tanh_hw(u) : tanhf(u);
  return 0.5f * (1.0f + t) + 0.5f * x * (1.0f - t * t) * kGeluC0 * (1.0f + 3.0f * kGeluC1 * x * x);
}

// Records -> features (kFeat: inputs and odd bases) and targets D / scale
// (8: 7 components + pad), in FP64.
__global__ void
k_encode(const float * __restrict__ rec, int64_t n, float * __restrict__ feat,
         float * __restrict__ tgt)
{
  const int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= n)
    return;
  const float * r = rec + s * kRecord;
  double        l7[7], r7[7], f[kFeat], sc[7];
  for (int q = 0; q < 7; ++q)
  {
    l7[q] = r[kRecQL + q];
    r7[q] = r[kRecQR + q];
  }
  encode(l7, r7, (double)r[kRecA], f, sc);
  for (int q = 0; q < kFeat; ++q)
    feat[s * kFeat + q] = (float)f[q];
  for (int q = 0; q < 7; ++q)
    tgt[s * kTgt + q] = (float)((double)r[kRecD + q] / sc[q]);
  tgt[s * kTgt + 7] = 0.f;
}

// Forward + backward of kTB samples per block; writes the block's summed
// gradient (kParams) and summed squared error to partial[block].
// idx (optional) maps sample slots to rows of feat/tgt.  norm = 1 / (N * 7).
__global__ void __launch_bounds__(kTB)
k_fwd_bwd(const float * __restrict__ W, const float * __restrict__ feat,
          const float * __restrict__ tgt, const int * __restrict__ idx, int64_t first, int64_t n,
          float norm, int train, float wpow, float * __restrict__ partial)
{
  extern __shared__ float sm[];
  float *     w = sm;
  float *     rows = sm + kParams;
  const int   s = threadIdx.x;
  for (int p = s; p < kParams; p += kTB)
  {
    const float x = W[p];
    // biases stay FP32 in the deployed network; weights are BF16
    const bool is_bias = (p >= kOffB1 && p < kOffW2) || (p >= kOffB2 && p < kOffW3) || p >= kOffB3;
    w[p] = (train && !is_bias) ? bf16_round(x) : x;
  }
  float *       row = rows + s * kRowStride;
  const int64_t slot = first + (int64_t)blockIdx.x * kTB + s;
  const bool    active = slot < n;
  const int64_t src = active ? (idx ? (int64_t)idx[slot] : slot) : 0;
  for (int q = 0; q < kIn; ++q)
  {
    const float x = active ? feat[src * kFeat + q] : 0.f;
    row[kRowX + q] = train ? bf16_round(x) : x;
  }
  for (int q = 0; q < kBasis; ++q)
    row[kRowU + q] = active ? feat[src * kFeat + kIn + q] : 0.f;
  __syncthreads();
  // layer 1
  for (int k = 0; k < kHid; ++k)
  {
    float acc = w[kOffB1 + k];
    for (int i = 0; i < kIn; ++i)
      acc = fmaf(row[kRowX + i], w[kOffW1 + i * kHid + k], acc);
    row[kRowZ1 + k] = acc;
    row[kRowH1 + k] = train ? gelu_bf16(acc) : gelu_exact(acc);
  }
  // layer 2
  for (int k = 0; k < kHid; ++k)
  {
    float acc = w[kOffB2 + k];
    for (int j = 0; j < kHid; ++j)
      acc = fmaf(row[kRowH1 + j], w[kOffW2 + j * kHid + k], acc);
    row[kRowZ2 + k] = acc;
    row[kRowH2 + k] = train ? gelu_bf16(acc) : gelu_exact(acc);
  }
  // layer 3, basis combination and loss gradient; sample weight
  // (sJ / kTauRef)^wpow emphasises the faces with larger jumps, whose
  // dissipation is larger in physical units
  const float sw = wpow != 0.f ? powf(fmaxf(row[kRowX + 6], 1e-3f), wpow) : 1.f;
  float       y[kOut], Dn[kOutUsed];
  for (int o = 0; o < kOut; ++o)
  {
    float acc = w[kOffB3 + o];
    for (int j = 0; j < kHid; ++j)
      acc = fmaf(row[kRowH2 + j], w[kOffW3 + j * kOut + o], acc);
    y[o] = acc;
  }
  combine(y, row + kRowU, Dn);
  float loss = 0.f, dD[kOutUsed];
  for (int c = 0; c < kOutUsed; ++c)
  {
    const float e = active ? Dn[c] - tgt[src * kTgt + c] : 0.f;
    loss = fmaf(sw * e, e, loss);
    dD[c] = 2.f * sw * e * norm;
  }
  // d(loss)/d(raw outputs): the transpose of combine
  const float * u1 = row + kRowU;
  const float * u2 = row + kRowU + 4;
  float *       dy = row + kRowY;
  for (int o = 0; o < kOut; ++o)
    dy[o] = 0.f;
  dy[0] = dD[0];
  dy[1] = dD[1];
  dy[2] = dD[2];
  for (int k = 0; k < 4; ++k)
  {
    dy[3 + k] = dD[3] * u1[k];
    dy[7 + k] = dD[5] * u1[k];
    dy[11 + k] = dD[4] * u2[k];
    dy[15 + k] = dD[6] * u2[k];
  }
  row[kRowLoss] = loss;
  // back through layer 3 and 2: dz2 overwrites z2, dz1 overwrites z1
  for (int j = 0; j < kHid; ++j)
  {
    float acc = 0.f;
    for (int o = 0; o < kOut; ++o)
      acc = fmaf(row[kRowY + o], w[kOffW3 + j * kOut + o], acc);
    row[kRowZ2 + j] = acc * gelu_grad(row[kRowZ2 + j], train);
  }
  for (int j = 0; j < kHid; ++j)
  {
    float acc = 0.f;
    for (int k = 0; k < kHid; ++k)
      acc = fmaf(row[kRowZ2 + k], w[kOffW2 + j * kHid + k], acc);
    row[kRowZ1 + j] = acc * gelu_grad(row[kRowZ1 + j], train);
  }
  __syncthreads();
  // weight gradients summed over the block's samples (thread s owns column s)
  float * out = partial + (size_t)blockIdx.x * (kParams + 1);
  {
    float acc[kIn], bacc = 0.f;
    for (int i = 0; i < kIn; ++i)
      acc[i] = 0.f;
    for (int r = 0; r < kTB; ++r)
    {
      const float * rr = rows + r * kRowStride;
      const float   dz = rr[kRowZ1 + s];
      bacc += dz;
      for (int i = 0; i < kIn; ++i)
        acc[i] = fmaf(rr[kRowX + i], dz, acc[i]);
    }
    for (int i = 0; i < kIn; ++i)
      out[kOffW1 + i * kHid + s] = acc[i];
    out[kOffB1 + s] = bacc;
  }
  {
    float acc[kHid], bacc = 0.f;
    for (int j = 0; j < kHid; ++j)
      acc[j] = 0.f;
    for (int r = 0; r < kTB; ++r)
    {
      const float * rr = rows + r * kRowStride;
      const float   dz = rr[kRowZ2 + s];
      bacc += dz;
      for (int j = 0; j < kHid; ++j)
        acc[j] = fmaf(rr[kRowH1 + j], dz, acc[j]);
    }
    for (int j = 0; j < kHid; ++j)
      out[kOffW2 + j * kHid + s] = acc[j];
    out[kOffB2 + s] = bacc;
  }
  {
    float acc[kOut];
    for (int o = 0; o < kOut; ++o)
      acc[o] = 0.f;
    for (int r = 0; r < kTB; ++r)
    {
      const float * rr = rows + r * kRowStride;
      const float   h = rr[kRowH2 + s];
      for (int o = 0; o < kOut; ++o)
        acc[o] = fmaf(h, rr[kRowY + o], acc[o]);
    }
    for (int o = 0; o < kOut; ++o)
      out[kOffW3 + s * kOut + o] = acc[o];
  }
  if (s < kOut)
  {
    float b = 0.f;
    for (int r = 0; r < kTB; ++r)
      b += rows[r * kRowStride + kRowY + s];
    out[kOffB3 + s] = b;
  }
  if (s == 0)
  {
    float l = 0.f;
    for (int r = 0; r < kTB; ++r)
      l += rows[r * kRowStride + kRowLoss];
    out[kParams] = l;
  }
}

// Sum of the block partials in block order (deterministic); optionally an
// Adam step.  grad_out / loss_out receive the sums when non-null.
__global__ void
k_reduce_adam(const float * __restrict__ partial, int nblocks, float * __restrict__ W,
              float * __restrict__ m, float * __restrict__ v, int adam, float lr, float bc1,
              float bc2, float * __restrict__ grad_out, double * __restrict__ loss_out)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p > kParams)
    return;
  double g = 0.0;
  for (int b = 0; b < nblocks; ++b)
    g += partial[(size_t)b * (kParams + 1) + p];
  if (p == kParams)
  {
    if (loss_out)
      *loss_out = g;
    return;
  }
  if (grad_out)
    grad_out[p] = (float)g;
  if (adam)
  {
    const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
    const float gf = (float)g;
    const float mm = beta1 * m[p] + (1.f - beta1) * gf;
    const float vv = beta2 * v[p] + (1.f - beta2) * gf * gf;
    m[p] = mm;
    v[p] = vv;
    W[p] -= lr * (mm / bc1) / (sqrtf(vv / bc2) + eps);
  }
}

// Batch forward on the 5th-generation tensor cores (mlp::block_forward,
// tcgen05 with accumulators in TMEM) on features: one face per thread, one
// 128-row tile per block.  status[0] is set when a completion wait reached
// its limit.  (The flux stage keeps the warp-level mma.sync forward: with
// one tile in flight per block, the three dependent MMA -> commit -> TMEM
// round trips per tile made the fused flux stage 2.3x slower.)
__global__ void __launch_bounds__(kTcRows)
k_forward_tc(const uint32_t * __restrict__ pack, const float * __restrict__ feat, int64_t n,
             float * __restrict__ out, int * __restrict__ status, int polls)
{
  extern __shared__ __align__(128) unsigned char smem[];
  uint32_t * slot = reinterpret_cast<uint32_t *>(smem + kTcBar + 8);
  stage_network_tc(pack, smem);
  if (threadIdx.x == 0)
    mhd::umma::mbar_init(mhd::umma::smem_addr(smem + kTcBar), 1);
  if (threadIdx.x < 32)
    mhd::umma::tmem_alloc(mhd::umma::smem_addr(slot), kTcCols);
  mhd::umma::fence_before_sync();
  __syncthreads();
  mhd::umma::fence_after_sync();
  const uint32_t tmem = *slot;
  const int64_t  s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  float          f[kIn], u[kBasis], y[kOut], Dn[kOutUsed];
  for (int q = 0; q < kIn; ++q)
    f[q] = s < n ? feat[s * kFeat + q] : 0.f;
  for (int q = 0; q < kBasis; ++q)
    u[q] = s < n ? feat[s * kFeat + kIn + q] : 0.f;
  uint32_t   parity = 0;
  const bool ok = block_forward<0>(smem, smem + kTcAct, mhd::umma::smem_addr(smem + kTcBar),
                                   threadIdx.x, tmem, parity, f, y, polls);
  if (ok && s < n)
  {
    combine(y, u, Dn);
    for (int c = 0; c < kOutUsed; ++c)
      out[s * kTgt + c] = Dn[c];
    out[s * kTgt + 7] = 0.f;
  }
  if (!ok && threadIdx.x == 0)
    atomicOr(status, 1);
  // every thread's TMEM accesses are complete before warp 0 frees it
  mhd::umma::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32)
  {
    mhd::umma::fence_after_sync();
    mhd::umma::tmem_dealloc(tmem, kTcCols);
  }
}

// The same batch forward as a persistent kernel: each 256-thread block stages
// the network once and runs two 128-row pipelines (threads 0-127 and
// 128-255) over the tiles 2 b + g, 2 b + g + 2 gridDim.x, ...  The pipelines
// synchronise on their own named barriers and wait on their own mbarriers,
// so one pipeline's MMAs run while the other moves its rows through the
// epilogue.  Per row the arithmetic is block_forward's: the outputs are
// bitwise those of k_forward_tc.  status[0] is set when a wait reached its
// limit; that pipeline stops, the other finishes its tiles.
__global__ void __launch_bounds__(kTc2Threads, 3)
k_forward_tc2(const uint32_t * __restrict__ pack, const float * __restrict__ feat, int64_t n,
              float * __restrict__ out, int * __restrict__ status, int polls)
{
  extern __shared__ __align__(128) unsigned char smem[];
  const int  g = threadIdx.x >> 7, r = threadIdx.x & (kTcRows - 1);
  uint32_t * slot = reinterpret_cast<uint32_t *>(smem + kTc2Bar + 16);
  stage_network_tc(pack, smem);
  if (threadIdx.x == 0)
  {
    mhd::umma::mbar_init(mhd::umma::smem_addr(smem + kTc2Bar), 1);
    mhd::umma::mbar_init(mhd::umma::smem_addr(smem + kTc2Bar + 8), 1);
  }
  if (threadIdx.x < 32)
    mhd::umma::tmem_alloc(mhd::umma::smem_addr(slot), kTc2Cols);
  mhd::umma::fence_before_sync();
  __syncthreads();
  mhd::umma::fence_after_sync();
  const uint32_t  tmem_base = *slot;
  const uint32_t  tmem = tmem_base + kTcCols * g;
  unsigned char * act = smem + kTc2Act + g * kTc2ActBytes;
  const uint32_t  mbar = mhd::umma::smem_addr(smem + kTc2Bar + 8 * g);
  uint32_t        parity = 0;
  bool            ok = true;
  for (int64_t tile = 2 * (int64_t)blockIdx.x + g; tile * kTcRows < n;
       tile += 2 * (int64_t)gridDim.x)
  {
    const int64_t s = tile * kTcRows + r;
    float         f[kIn], u[kBasis], y[kOut], Dn[kOutUsed];
    // the pipeline's next tile (its rows are one contiguous block of
    // 128 x 160 bytes, 16-byte aligned) prefetched into L2 while this one
    // computes
    const int64_t next = tile + 2 * (int64_t)gridDim.x;
    if (r == 0 && next * kTcRows < n)
      mhd::umma::bulk_prefetch_l2(
        feat + next * kTcRows * kFeat,
        (uint32_t)(min((int64_t)kTcRows, n - next * kTcRows) * kFeat * sizeof(float)));
    // the row's 40 features as ten 16-byte loads (rows are 160 bytes)
    const float4 * f4 = reinterpret_cast<const float4 *>(feat + (s < n ? s : 0) * kFeat);
#pragma unroll
    for (int q4 = 0; q4 < kIn / 4; ++q4)
    {
      const float4 a = s < n ? __ldg(f4 + q4) : make_float4(0.f, 0.f, 0.f, 0.f);
      f[4 * q4] = a.x;
      f[4 * q4 + 1] = a.y;
      f[4 * q4 + 2] = a.z;
      f[4 * q4 + 3] = a.w;
    }
    ok = g == 0 ? block_forward<1>(smem, act, mbar, r, tmem, parity, f, y, polls)
                : block_forward<2>(smem, act, mbar, r, tmem, parity, f, y, polls);
    if (!ok)
      break;
    if (s < n)
    {
      // the odd bases (the row's last 32 bytes) only now: fewer live
      // registers across the forward pass
#pragma unroll
      for (int q4 = 0; q4 < kBasis / 4; ++q4)
      {
        const float4 a = __ldg(f4 + kIn / 4 + q4);
        u[4 * q4] = a.x;
        u[4 * q4 + 1] = a.y;
        u[4 * q4 + 2] = a.z;
        u[4 * q4 + 3] = a.w;
      }
      combine(y, u, Dn);
      float4 * o4 = reinterpret_cast<float4 *>(out + s * kTgt);
      o4[0] = make_float4(Dn[0], Dn[1], Dn[2], Dn[3]);
      o4[1] = make_float4(Dn[4], Dn[5], Dn[6], 0.f);
    }
  }
  if (!ok && r == 0)
    atomicOr(status, 1);
  // both pipelines' TMEM accesses are complete before warp 0 frees it
  mhd::umma::fence_before_sync();
  __syncthreads();
  if (threadIdx.x < 32)
  {
    mhd::umma::fence_after_sync();
    mhd::umma::tmem_dealloc(tmem_base, kTc2Cols);
  }
}

// ---------------------------------------------------------------- host

uint16_t
bf16_bits_rn(float x)
{
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) // NaN
    return (uint16_t)((u >> 16) | 0x40u);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

void
pack_layer(const float * W, int K, int N, uint32_t * out)
{
  const int KT = K / 16, NT = N / 8;
  for (int kt = 0; kt < KT; ++kt)
    for (int nt = 0; nt < NT; ++nt)
      for (int lane = 0; lane < 32; ++lane)
      {
        const int g = lane >> 2, t = lane & 3, n = nt * 8 + g;
        auto      w = [&](int k) { return (uint32_t)bf16_bits_rn(W[k * N + n]); };
        uint32_t *o = out + ((size_t)(kt * NT + nt) * 32 + lane) * 2;
        o[0] = w(kt * 16 + 2 * t) | (w(kt * 16 + 2 * t + 1) << 16);
        o[1] = w(kt * 16 + 8 + 2 * t) | (w(kt * 16 + 8 + 2 * t + 1) << 16);
      }
}

// W[K][N] (row = input, column = output unit) -> W^T[Npad][K] in BF16 (round
// to nearest even) in the tensor cores' canonical K-major layout; rows
// n >= N are zero.
void
pack_layer_tc(const float * W, int K, int N, int Npad, unsigned char * out)
{
  for (int n = 0; n < Npad; ++n)
    for (int k = 0; k < K; ++k)
    {
      const uint16_t v = n < N ? bf16_bits_rn(W[k * N + n]) : (uint16_t)0;
      std::memcpy(out + mhd::umma::canon_offset(n, k, K), &v, sizeof(v));
    }
}

// The tcgen05 network image (kTcPackWords words).
void
pack_tc(const float * params, uint32_t * out)
{
  unsigned char * w = reinterpret_cast<unsigned char *>(out);
  pack_layer_tc(params + kOffW1, kIn, kHid, kHid, w + kTcW1);
  pack_layer_tc(params + kOffW2, kHid, kHid, kHid, w + kTcW2);
  pack_layer_tc(params + kOffW3, kHid, kOut, kN3, w + kTcW3);
  float * b = reinterpret_cast<float *>(out + kTcWBytes / 4);
  std::memcpy(b, params + kOffB1, kHid * sizeof(float));
  std::memcpy(b + kHid, params + kOffB2, kHid * sizeof(float));
  std::memcpy(b + 2 * kHid, params + kOffB3, kOut * sizeof(float));
}

uint64_t
splitmix64(uint64_t & s)
{
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

double
uniform01(uint64_t & s)
{
  return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0);
}

int
fail(mhd_mlp * m, int rc, const std::string & msg)
{
  if (m)
    m->err = msg;
  return rc;
}

#define MLP_CK(call)                                                                   \
  do                                                                                   \
  {                                                                                    \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return fail(m, MHD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

int
upload_params(mhd_mlp * m)
{
  MLP_CK(cudaMemcpy(m->d_params, m->params.data(), kParams * sizeof(float), cudaMemcpyHostToDevice));
  return MHD_OK;
}

int
download_params(mhd_mlp * m)
{
  MLP_CK(cudaMemcpy(m->params.data(), m->d_params, kParams * sizeof(float), cudaMemcpyDeviceToHost));
  return MHD_OK;
}

// RAII device buffer
template <class T>
struct DevBuf
{
  T * p = nullptr;
  ~DevBuf()
  {
    if (p)
      cudaFree(p);
  }
  cudaError_t
  alloc(size_t n)
  {
    return cudaMalloc(&p, n * sizeof(T));
  }
};

int
encode_on_device(mhd_mlp * m, const float * records, int64_t n, DevBuf<float> & feat,
                 DevBuf<float> & tgt)
{
  DevBuf<float> rec;
  MLP_CK(rec.alloc((size_t)n * kRecord));
  MLP_CK(feat.alloc((size_t)n * kFeat));
  MLP_CK(tgt.alloc((size_t)n * kTgt));
  MLP_CK(cudaMemcpyAsync(rec.p, records, (size_t)n * kRecord * sizeof(float), cudaMemcpyHostToDevice,
                         m->stream));
  k_encode<<<(unsigned)((n + 127) / 128), 128, 0, m->stream>>>(rec.p, n, feat.p, tgt.p);
  MLP_CK(cudaGetLastError());
  MLP_CK(cudaStreamSynchronize(m->stream));
  return MHD_OK;
}

int
set_train_smem()
{
  static bool done = false;
  if (!done)
  {
    if (cudaFuncSetAttribute(k_fwd_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemTrain) !=
        cudaSuccess)
      return MHD_ERR_CUDA;
    done = true;
  }
  return MHD_OK;
}

} // namespace

namespace mhd
{
// Packed weights + biases of a network for the flux stage (used by mhd_capi.cpp).
void
mlp_pack(const float * params, uint32_t * out)
{
  pack_layer(params + kOffW1, kIn, kHid, out + kPackW1);
  pack_layer(params + kOffW2, kHid, kHid, out + kPackW2);
  pack_layer(params + kOffW3, kHid, kOut, out + kPackW3);
  float * b = reinterpret_cast<float *>(out + kPackWords);
  std::memcpy(b, params + kOffB1, kHid * sizeof(float));
  std::memcpy(b + kHid, params + kOffB2, kHid * sizeof(float));
  std::memcpy(b + 2 * kHid, params + kOffB3, kOut * sizeof(float));
}

double
mlp_gamma(const mhd_mlp * m)
{
  return m->gamma0;
}

const float *
mlp_params(const mhd_mlp * m)
{
  return m->params.data();
}
} // namespace mhd

extern "C"
{

  int
  mhd_mlp_create(uint64_t seed, double gamma0, mhd_mlp ** out)
  {
    if (!out || !(gamma0 > 1.0))
      return MHD_ERR_INVALID_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      return MHD_ERR_NO_DEVICE;
    mhd_mlp * m = new mhd_mlp;
    *out = m;
    m->gamma0 = gamma0;
    MLP_CK(cudaGetDevice(&m->device));
    MLP_CK(cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking));
    MLP_CK(cudaMalloc(&m->d_params, kParams * sizeof(float)));
    MLP_CK(cudaMalloc(&m->d_m, kParams * sizeof(float)));
    MLP_CK(cudaMalloc(&m->d_v, kParams * sizeof(float)));
    MLP_CK(cudaMemset(m->d_m, 0, kParams * sizeof(float)));
    MLP_CK(cudaMemset(m->d_v, 0, kParams * sizeof(float)));
    // Glorot-uniform weights, zero biases
    m->params.assign(kParams, 0.f);
    uint64_t  s = seed;
    auto      init = [&](int off, int fan_in, int fan_out, int used_in, int used_out) {
      const double lim = std::sqrt(6.0 / (used_in + used_out));
      for (int i = 0; i < fan_in; ++i)
        for (int o = 0; o < fan_out; ++o)
        {
          const double r = (2.0 * uniform01(s) - 1.0) * lim;
          m->params[off + i * fan_out + o] = (i < used_in && o < used_out) ? (float)r : 0.f;
        }
    };
    init(kOffW1, kIn, kHid, kInUsed, kHid);
    init(kOffW2, kHid, kHid, kHid, kHid);
    init(kOffW3, kHid, kOut, kHid, kRawUsed);
    return upload_params(m);
  }

  int
  mhd_mlp_destroy(mhd_mlp * m)
  {
    if (!m)
      return MHD_ERR_INVALID_ARG;
    if (m->d_params)
      cudaFree(m->d_params);
    if (m->d_m)
      cudaFree(m->d_m);
    if (m->d_v)
      cudaFree(m->d_v);
    if (m->stream)
      cudaStreamDestroy(m->stream);
    delete m;
    return MHD_OK;
  }

  int
  mhd_mlp_set_forward_form(mhd_mlp * m, int form)
  {
    if (!m || (form != MHD_MLP_FORWARD_TILES && form != MHD_MLP_FORWARD_PERSISTENT))
      return MHD_ERR_INVALID_ARG;
    m->forward_form = form;
    return MHD_OK;
  }

  int
  mhd_mlp_last_forward_ms(mhd_mlp * m, double * ms)
  {
    if (!m || !ms)
      return MHD_ERR_INVALID_ARG;
    *ms = m->last_forward_ms;
    return MHD_OK;
  }

  int
  mhd_mlp_set_wait_limit(mhd_mlp * m, int polls)
  {
    if (!m || polls < 0)
      return MHD_ERR_INVALID_ARG;
    m->wait_polls = polls;
    return MHD_OK;
  }

  const char *
  mhd_mlp_last_error(mhd_mlp * m)
  {
    return m ? m->err.c_str() : "null network";
  }

  int
  mhd_mlp_set_params(mhd_mlp * m, const float * params, int n)
  {
    if (!m || !params)
      return MHD_ERR_INVALID_ARG;
    if (n != kParams)
      return fail(m, MHD_ERR_INVALID_ARG, "parameter count must be MHD_MLP_PARAMS");
    MLP_CK(cudaSetDevice(m->device));
    m->params.assign(params, params + kParams);
    MLP_CK(cudaMemset(m->d_m, 0, kParams * sizeof(float)));
    MLP_CK(cudaMemset(m->d_v, 0, kParams * sizeof(float)));
    m->adam_step = 0;
    return upload_params(m);
  }

  int
  mhd_mlp_get_params(mhd_mlp * m, float * params, int n)
  {
    if (!m || !params)
      return MHD_ERR_INVALID_ARG;
    if (n != kParams)
      return fail(m, MHD_ERR_INVALID_ARG, "parameter count must be MHD_MLP_PARAMS");
    std::memcpy(params, m->params.data(), kParams * sizeof(float));
    return MHD_OK;
  }

  int
  mhd_mlp_gamma(mhd_mlp * m, double * gamma0)
  {
    if (!m || !gamma0)
      return MHD_ERR_INVALID_ARG;
    *gamma0 = m->gamma0;
    return MHD_OK;
  }

  int
  mhd_mlp_encode(mhd_mlp * m, const float * records, int64_t n, float * features,
                 float * targets)
  {
    if (!m || !records || n <= 0 || !features || !targets)
      return MHD_ERR_INVALID_ARG;
    MLP_CK(cudaSetDevice(m->device));
    DevBuf<float> feat, tgt;
    if (int rc = encode_on_device(m, records, n, feat, tgt))
      return rc;
    MLP_CK(cudaMemcpy(features, feat.p, (size_t)n * kFeat * sizeof(float), cudaMemcpyDeviceToHost));
    MLP_CK(cudaMemcpy(targets, tgt.p, (size_t)n * kTgt * sizeof(float), cudaMemcpyDeviceToHost));
    return MHD_OK;
  }

  int
  mhd_mlp_gradient(mhd_mlp * m, const float * features, const float * targets, int64_t n,
                   int mode, float * grad, double * loss)
  {
    if (!m || !features || !targets || n <= 0 || !grad ||
        (mode != MHD_MLP_CHECK && mode != MHD_MLP_TRAIN))
      return MHD_ERR_INVALID_ARG;
    MLP_CK(cudaSetDevice(m->device));
    if (set_train_smem())
      return fail(m, MHD_ERR_CUDA, "cannot reserve shared memory for the training kernel");
    DevBuf<float> feat, tgt, partial, g;
    DevBuf<double> l;
    const int     nb = (int)((n + kTB - 1) / kTB);
    MLP_CK(feat.alloc((size_t)n * kFeat));
    MLP_CK(tgt.alloc((size_t)n * kTgt));
    MLP_CK(partial.alloc((size_t)nb * (kParams + 1)));
    MLP_CK(g.alloc(kParams));
    MLP_CK(l.alloc(1));
    MLP_CK(cudaMemcpy(feat.p, features, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice));
    MLP_CK(cudaMemcpy(tgt.p, targets, (size_t)n * kTgt * sizeof(float), cudaMemcpyHostToDevice));
    const float norm = (float)(1.0 / ((double)n * kOutUsed));
    k_fwd_bwd<<<nb, kTB, kSmemTrain, m->stream>>>(m->d_params, feat.p, tgt.p, nullptr, 0, n, norm,
                                                  mode == MHD_MLP_TRAIN, 0.f, partial.p);
    k_reduce_adam<<<(kParams + 1 + 255) / 256, 256, 0, m->stream>>>(
      partial.p, nb, m->d_params, m->d_m, m->d_v, 0, 0.f, 1.f, 1.f, g.p, l.p);
    MLP_CK(cudaGetLastError());
    MLP_CK(cudaStreamSynchronize(m->stream));
    MLP_CK(cudaMemcpy(grad, g.p, kParams * sizeof(float), cudaMemcpyDeviceToHost));
    double lsum = 0.0;
    MLP_CK(cudaMemcpy(&lsum, l.p, sizeof(double), cudaMemcpyDeviceToHost));
    if (loss)
      *loss = lsum * norm;
    return MHD_OK;
  }

  int
  mhd_mlp_train(mhd_mlp * m, const float * records, int64_t n, int epochs, int batch, float lr,
                float weight_power, uint64_t seed, float * loss_history)
  {
    if (!m || !records || n < kTB || epochs <= 0 || batch < kTB || !(lr > 0.f))
      return MHD_ERR_INVALID_ARG;
    MLP_CK(cudaSetDevice(m->device));
    if (set_train_smem())
      return fail(m, MHD_ERR_CUDA, "cannot reserve shared memory for the training kernel");
    batch = (batch / kTB) * kTB;
    DevBuf<float> feat, tgt, partial;
    DevBuf<int>   perm;
    DevBuf<double> l;
    if (int rc = encode_on_device(m, records, n, feat, tgt))
      return rc;
    const int nbb = batch / kTB;
    MLP_CK(partial.alloc((size_t)nbb * (kParams + 1)));
    MLP_CK(perm.alloc((size_t)n));
    MLP_CK(l.alloc(1));
    std::vector<int> h((size_t)n);
    uint64_t         s = seed;
    const int64_t    nbatch = n / batch > 0 ? n / batch : 1;
    const int64_t    total = nbatch * epochs;
    int64_t          it = 0;
    for (int ep = 0; ep < epochs; ++ep)
    {
      for (int64_t q = 0; q < n; ++q)
        h[q] = (int)q;
      for (int64_t q = n - 1; q > 0; --q) // Fisher-Yates
        std::swap(h[q], h[(int64_t)(uniform01(s) * (double)(q + 1)) % (q + 1)]);
      MLP_CK(cudaMemcpyAsync(perm.p, h.data(), (size_t)n * sizeof(int), cudaMemcpyHostToDevice,
                             m->stream));
      double ep_loss = 0.0;
      for (int64_t b = 0; b < nbatch; ++b, ++it)
      {
        const int64_t first = b * batch;
        const int64_t cnt = std::min<int64_t>(batch, n - first);
        const int     nb = (int)((cnt + kTB - 1) / kTB);
        const float   norm = (float)(1.0 / ((double)cnt * kOutUsed));
        // cosine decay to lr / 20
        const double  frac = (double)it / (double)std::max<int64_t>(total - 1, 1);
        const float   lr_t = (float)(lr * (0.05 + 0.95 * 0.5 * (1.0 + std::cos(M_PI * frac))));
        ++m->adam_step;
        const float bc1 = (float)(1.0 - std::pow(0.9, (double)m->adam_step));
        const float bc2 = (float)(1.0 - std::pow(0.999, (double)m->adam_step));
        k_fwd_bwd<<<nb, kTB, kSmemTrain, m->stream>>>(m->d_params, feat.p, tgt.p, perm.p, first,
                                                      first + cnt, norm, 1, weight_power,
                                                      partial.p);
        k_reduce_adam<<<(kParams + 1 + 255) / 256, 256, 0, m->stream>>>(
          partial.p, nb, m->d_params, m->d_m, m->d_v, 1, lr_t, bc1, bc2, nullptr, l.p);
        if (loss_history)
        {
          double lb = 0.0;
          MLP_CK(cudaMemcpyAsync(&lb, l.p, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
          MLP_CK(cudaStreamSynchronize(m->stream));
          ep_loss += lb * norm;
        }
      }
      MLP_CK(cudaGetLastError());
      if (loss_history)
        loss_history[ep] = (float)(ep_loss / (double)nbatch);
    }
    MLP_CK(cudaStreamSynchronize(m->stream));
    return download_params(m);
  }

  int
  mhd_mlp_forward(mhd_mlp * m, const float * features, int64_t n, float * out)
  {
    if (!m || !features || n <= 0 || !out)
      return MHD_ERR_INVALID_ARG;
    MLP_CK(cudaSetDevice(m->device));
    std::vector<uint32_t> pack(kTcPackWords);
    pack_tc(m->params.data(), pack.data());
    DevBuf<uint32_t> dp;
    DevBuf<float>    feat, o;
    DevBuf<int>      status;
    MLP_CK(dp.alloc(pack.size()));
    MLP_CK(feat.alloc((size_t)n * kFeat));
    MLP_CK(o.alloc((size_t)n * kTgt));
    MLP_CK(status.alloc(1));
    MLP_CK(cudaMemcpy(dp.p, pack.data(), pack.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    MLP_CK(cudaMemcpy(feat.p, features, (size_t)n * kFeat * sizeof(float), cudaMemcpyHostToDevice));
    MLP_CK(cudaMemset(status.p, 0, sizeof(int)));
    const int64_t tiles = (n + kTcRows - 1) / kTcRows;
    unsigned      grid = 0;
    if (m->forward_form == MHD_MLP_FORWARD_PERSISTENT)
    {
      // every block resident at once: SMs x blocks per SM, at most one
      // block per two tiles.  Blocks per SM from the kernel's registers, its
      // shared memory and the SM's 512 TMEM columns (cudaOccupancy... gave 1
      // for this kernel on GB300 where 3 fit, and a grid of one block per
      // SM ran 8 warps per SM)
      int                sms = 0, sm_regs = 0, sm_smem = 0, reserved = 0, sm_threads = 0;
      cudaFuncAttributes fa{};
      MLP_CK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device));
      MLP_CK(cudaDeviceGetAttribute(&sm_regs, cudaDevAttrMaxRegistersPerMultiprocessor, m->device));
      MLP_CK(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                    m->device));
      MLP_CK(cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, m->device));
      MLP_CK(cudaDeviceGetAttribute(&sm_threads, cudaDevAttrMaxThreadsPerMultiProcessor,
                                    m->device));
      MLP_CK(cudaFuncSetAttribute(k_forward_tc2, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  kTc2SmemBytes));
      // the whole unified L1 as shared memory
      MLP_CK(cudaFuncSetAttribute(k_forward_tc2, cudaFuncAttributePreferredSharedMemoryCarveout,
                                  (int)cudaSharedmemCarveoutMaxShared));
      MLP_CK(cudaFuncGetAttributes(&fa, k_forward_tc2));
      const int warp_regs = ((fa.numRegs * 32 + 255) / 256) * 256; // 256-register granules
      const int by_regs = warp_regs > 0 ? (sm_regs / warp_regs) / (kTc2Threads / 32) : 0;
      const int by_smem = sm_smem / (kTc2SmemBytes + (int)fa.sharedSizeBytes + reserved);
      const int per_sm = std::min({by_regs, by_smem, sm_threads / kTc2Threads, (int)(512 / kTc2Cols)});
      if (per_sm < 1)
        return fail(m, MHD_ERR_CUDA, "the persistent forward does not fit an SM");
      grid = (unsigned)std::min<int64_t>((tiles + 1) / 2, (int64_t)sms * per_sm);
    }
    cudaEvent_t ev[2] = {nullptr, nullptr};
    MLP_CK(cudaEventCreate(&ev[0]));
    MLP_CK(cudaEventCreate(&ev[1]));
    MLP_CK(cudaEventRecord(ev[0], m->stream));
    if (m->forward_form == MHD_MLP_FORWARD_PERSISTENT)
      k_forward_tc2<<<grid, kTc2Threads, kTc2SmemBytes, m->stream>>>(dp.p, feat.p, n, o.p,
                                                                      status.p, m->wait_polls);
    else
      k_forward_tc<<<(unsigned)tiles, kTcRows, kTcSmemBytes, m->stream>>>(dp.p, feat.p, n, o.p,
                                                                          status.p, m->wait_polls);
    const cudaError_t launch = cudaGetLastError();
    MLP_CK(cudaEventRecord(ev[1], m->stream));
    MLP_CK(cudaStreamSynchronize(m->stream));
    float ms = -1.f;
    if (launch == cudaSuccess)
      MLP_CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
    cudaEventDestroy(ev[0]);
    cudaEventDestroy(ev[1]);
    MLP_CK(launch);
    m->last_forward_ms = ms;
    int st = 0;
    MLP_CK(cudaMemcpy(&st, status.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (st)
      return fail(m, MHD_ERR_CUDA, "a tensor-core completion wait reached its limit");
    MLP_CK(cudaMemcpy(out, o.p, (size_t)n * kTgt * sizeof(float), cudaMemcpyDeviceToHost));
    return MHD_OK;
  }

} // extern "C"
