// Solver core for one arithmetic variant: device buffers, one CUDA stream,
// the launch sequence of an iteration, CUDA-graph replay of whole runs,
// host<->device state transfer in either Kokkos layout, FP64 diagnostics and
// per-kernel timing.  Included by mhd_variant.cu, which fixes R and the
// inline namespace MHD_VARIANT_TAG.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mhd_core.h"
#include "mhd_fused.cuh"
#include "mhd_kernels.cuh"
#include "mhd_surrogate.cuh"
#include "mhd_kernels_v0.cuh"

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

#define MHD_CK(call)                                                                  \
  do                                                                                  \
  {                                                                                   \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
    {                                                                                 \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
      return MHD_ERR_CUDA;                                                            \
    }                                                                                 \
  } while (0)

// LayoutRight <-> LayoutLeft.  dir = 0: right -> left, dir = 1: left -> right.
template <class R>
__global__ void
k_transpose(const Grid<R> G, const R * __restrict__ src, R * __restrict__ dst, int dir)
{
  const int64_t n = G.sv * NV;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= n)
    return;
  // idx enumerates the LayoutLeft index: i + isize*(j + jsize*(k + ksize*v))
  const int64_t v = idx / G.sv;
  const int64_t cell = idx - v * G.sv;
  const int64_t k = cell / G.sk;
  const int64_t rem = cell - k * G.sk;
  const int64_t j = rem / G.sj;
  const int64_t i = rem - j * G.sj;
  const int64_t right = ((i * G.jsize + j) * G.ksize + k) * NV + v;
  if (dir == 0)
    dst[idx] = src[right];
  else
    dst[right] = src[idx];
}

// FP64 sums of the 8 stored variables and of |div B| over interior cells,
// one partial record of 10 doubles per block (sums[8], sum |divB|, max |divB|).
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_diag(const Grid<R> G, const R * __restrict__ U, double * __restrict__ partial)
{
  const int g = G.g;
  const Box & b = G.box[BOX_INTERIOR];
  double    acc[10];
#pragma unroll
  for (int q = 0; q < 10; ++q)
    acc[q] = 0.0;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; idx < b.count(); idx += stride)
  {
    int i, j, k;
    box_cell(b, idx, i, j, k);
    const int64_t c = cell_at(G, i, j, k), sv = G.sv;
#pragma unroll
    for (int v = 0; v < NV; ++v)
      acc[v] += (double)U[c + v * sv];
    double div = ((double)U[c + 1 + IA * sv] - (double)U[c + IA * sv]) / G.dx +
                 ((double)U[c + G.sj + IB * sv] - (double)U[c + IB * sv]) / G.dy;
    if (DIM == 3)
      div += ((double)U[c + G.sk + IC * sv] - (double)U[c + IC * sv]) / G.dz;
    acc[8] += fabs(div);
    acc[9] = fmax(acc[9], fabs(div));
  }
  __shared__ double sh[10][256];
#pragma unroll
  for (int q = 0; q < 10; ++q)
    sh[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1)
  {
    if ((int)threadIdx.x < s)
    {
#pragma unroll
      for (int q = 0; q < 9; ++q)
        sh[q][threadIdx.x] += sh[q][threadIdx.x + s];
      sh[9][threadIdx.x] = fmax(sh[9][threadIdx.x], sh[9][threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x < 10)
    partial[blockIdx.x * 10 + threadIdx.x] = sh[threadIdx.x][0];
}

static __global__ void
k_diag_final(const double * __restrict__ partial, int nblocks, double * __restrict__ out)
{
  const int q = threadIdx.x;
  if (q >= 10)
    return;
  double a = 0.0;
  for (int b = 0; b < nblocks; ++b)
  {
    const double x = partial[b * 10 + q];
    a = (q == 9) ? fmax(a, x) : a + x;
  }
  out[q] = a;
}

template <class R>
class SolverImpl final : public SolverCore
{
public:
  static constexpr int kDiagBlocks = 1024;

  mhd_params   P{};
  Grid<R>      G{};
  int          dim = 2;
  int64_t      ncell = 0; // ghost-inclusive cells
  R *          U = nullptr;
  R *          U2 = nullptr;
  R *          Q = nullptr;
  R *          Q2 = nullptr;
  R *          S = nullptr;
  R *          E = nullptr;
  R *          F = nullptr;
  R *          Em = nullptr;
  R *          H = nullptr;  // version 2: face data (FaceData<DIM>)
  R *          Ulo = nullptr; // FP32 version 2: low parts of the state (Buffers::Ulo)
  R *          T = nullptr;  // versions 0/1: stored trace states
  R *          D = nullptr;  // versions 0/1 in 3D: transverse face-field slopes
  int          version = 2;
  double *     diag = nullptr;
  DevState *   st = nullptr;
  DevState *   st_host = nullptr; // pinned
  cudaStream_t stream = nullptr;
  cudaGraphExec_t graph[2] = { nullptr, nullptr }; // one iteration starting from U / from U2
  cudaGraphExec_t graph_pair[2] = { nullptr, nullptr }; // two iterations
  int64_t launched = 0; // iterations enqueued since the last state reset (parity)
  // host-buffer step: slabs of the edge/update stages whose download overlaps
  // the rest of the edge stage (0 = chosen from the array size)
  static constexpr int kMaxHostSlabs = 16;
  int          host_slabs_req = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t  slab_ev[kMaxHostSlabs] = {};
  cudaEvent_t  up_ev[kMaxHostSlabs] = {};
  cudaEvent_t  copy_ev = nullptr;
  // flux surrogate (FP32 builds only)
  uint32_t *           sur_w = nullptr; // packed weights + biases (mhd_mlp.cuh)
  unsigned long long * sur_count = nullptr;
  uint32_t *           sur_list = nullptr; // faces left to HLLD
  unsigned *           sur_nlist = nullptr;
  float                sur_tau = 0.f;
  bool                 sur_on = false;
  int                  sm_count = 0;
  int                  sur_blocks_per_sm = 1;
  // 2D version 2: the fused tile form (k_dt_only + k_mfused2d, every
  // intermediate in shared memory) or the stage kernels; the same state bit
  // for bit in the FMA-free build, round-off apart in the FMA builds.  The
  // default is a fixed function of the configuration (default_form), so a
  // configuration always runs the same kernels; mhd_set_fused fixes either
  // form or has the next stepping call time both (tune_form).
  static constexpr int kFusedTY = sizeof(R) == 4 ? MFUSED_TILE_ROWS : 8;
  using FusedTile = MTile<R, kFusedTY>;
  bool                 fused = false;
  bool                 tuned = true;
  int                  form_req = -1; // -1: default_form; else the mhd_set_fused request
  std::string          tune_report;

  ~SolverImpl() override
  {
    for (int q = 0; q < 2; ++q)
    {
      if (graph[q])
        cudaGraphExecDestroy(graph[q]);
      if (graph_pair[q])
        cudaGraphExecDestroy(graph_pair[q]);
    }
    for (cudaEvent_t e : slab_ev)
      if (e)
        cudaEventDestroy(e);
    for (cudaEvent_t e : up_ev)
      if (e)
        cudaEventDestroy(e);
    if (copy_ev)
      cudaEventDestroy(copy_ev);
    if (copy_stream)
      cudaStreamDestroy(copy_stream);
    R * bufs[] = { U, U2, Q, Q2, S, E, F, Em, H, T, D, Ulo };
    for (R * b : bufs)
      if (b)
        cudaFree(b);
    if (sur_w)
      cudaFree(sur_w);
    if (sur_count)
      cudaFree(sur_count);
    if (sur_list)
      cudaFree(sur_list);
    if (sur_nlist)
      cudaFree(sur_nlist);
    if (diag)
      cudaFree(diag);
    if (st)
      cudaFree(st);
    if (st_host)
      cudaFreeHost(st_host);
    if (stream)
      cudaStreamDestroy(stream);
  }

  int
  real_bytes() const override
  {
    return (int)sizeof(R);
  }

  int
  bind_device() override
  {
    MHD_CK(cudaSetDevice(P.device));
    return MHD_OK;
  }

  int
  setup(const mhd_params & p)
  {
    P = p;
    dim = p.dim;
    G = make_grid<R>(p);
    ncell = G.sv;

    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    {
      err = "no CUDA device available";
      return MHD_ERR_NO_DEVICE;
    }
    if (p.device < 0 || p.device >= ndev)
    {
      err = "device ordinal " + std::to_string(p.device) + " out of range";
      return MHD_ERR_INVALID_ARG;
    }
    MHD_CK(cudaSetDevice(p.device));
    MHD_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    const size_t n = (size_t)ncell;
    const int    nplanes_e = dim == 3 ? 3 : 1;
    const int    nf = dim == 3 ? 5 : 6;
    version = p.implementation_version;
    // (256 bytes of padding: the fused form's optional bulk copies of the
    // last rows, MFUSED_BULK_STAGING, may run past the last value)
    MHD_CK(cudaMalloc(&U, n * NV * sizeof(R) + 256));
    MHD_CK(cudaMalloc(&U2, n * NV * sizeof(R) + 256));
    MHD_CK(cudaMalloc(&Q, n * NV * sizeof(R)));
    if (version == 2)
    {
      MHD_CK(cudaMalloc(&Q2, n * NV * sizeof(R)));
      MHD_CK(cudaMalloc(&S, n * NV * dim * sizeof(R)));
      MHD_CK(cudaMalloc(&H, n * face_data_planes(dim) * sizeof(R)));
    }
    else
    {
      MHD_CK(cudaMalloc(&T, n * NV * (dim == 3 ? 18 : 8) * sizeof(R)));
      if (dim == 3)
        MHD_CK(cudaMalloc(&D, n * 6 * sizeof(R)));
    }
    MHD_CK(cudaMalloc(&E, n * nplanes_e * sizeof(R)));
    MHD_CK(cudaMalloc(&F, n * nf * dim * sizeof(R)));
    MHD_CK(cudaMalloc(&Em, n * nplanes_e * sizeof(R)));
    MHD_CK(cudaMalloc(&diag, (kDiagBlocks * 10 + 16) * sizeof(double)));
    if (sizeof(R) == 4 && version == 2)
      MHD_CK(cudaMalloc(&Ulo, n * NV * sizeof(R)));
    MHD_CK(cudaMalloc(&st, sizeof(DevState)));
    MHD_CK(cudaMallocHost(&st_host, sizeof(DevState)));
    // zero everything once: halo reads of never-written planes see zeros,
    // as the reference's zero-initialised Kokkos views do
    R * bufs[] = { U, U2, Q, Q2, Ulo };
    for (R * b : bufs)
      if (b)
        MHD_CK(cudaMemsetAsync(b, 0, n * NV * sizeof(R), stream));
    if (S)
      MHD_CK(cudaMemsetAsync(S, 0, n * NV * dim * sizeof(R), stream));
    if (H)
      MHD_CK(cudaMemsetAsync(H, 0, n * face_data_planes(dim) * sizeof(R), stream));
    if (T)
      MHD_CK(cudaMemsetAsync(T, 0, n * NV * (dim == 3 ? 18 : 8) * sizeof(R), stream));
    if (D)
      MHD_CK(cudaMemsetAsync(D, 0, n * 6 * sizeof(R), stream));
    MHD_CK(cudaMemsetAsync(E, 0, n * nplanes_e * sizeof(R), stream));
    MHD_CK(cudaMemsetAsync(F, 0, n * nf * dim * sizeof(R), stream));
    MHD_CK(cudaMemsetAsync(Em, 0, n * nplanes_e * sizeof(R), stream));
    MHD_CK(reset_time_state());
    fused = default_form();
    if (fused_ok())
    {
      MHD_CK(cudaFuncSetAttribute(k_mfused2d<R, kFusedTY, RIEMANN_HLLD>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)FusedTile::SMEM));
      MHD_CK(cudaFuncSetAttribute(k_mfused2d<R, kFusedTY, 0>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)FusedTile::SMEM));
    }
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // the fused form exists for 2D implementation version 2 without the
  // flux surrogate (its tile reads 2 halo layers: ghost >= 2; the tile rows
  // are the launch's grid.y, at most 65535)
  bool
  fused_ok() const
  {
    return dim == 2 && version == 2 && !sur_on && G.g >= 2 &&
           (G.ny + FusedTile::TY - 1) / FusedTile::TY <= 65535;
  }

  int
  fused_form() const override
  {
    return fused ? 1 : 0;
  }

  // The form measured faster on GB300 for the configuration.
  bool
  default_form() const
  {
    return fused_ok() && sizeof(R) == 4;
  }

  int
  set_fused(int on) override
  {
    if (on < MHD_FORM_STAGES || on > MHD_FORM_TIMED)
    {
      err = "form must be MHD_FORM_STAGES, MHD_FORM_FUSED or MHD_FORM_TIMED";
      return MHD_ERR_INVALID_ARG;
    }
    if (on == MHD_FORM_FUSED && !fused_ok())
    {
      err = "the fused form is built for 2D implementation version 2 without the flux surrogate";
      return MHD_ERR_INVALID_ARG;
    }
    MHD_CK(cudaStreamSynchronize(stream));
    drop_graphs();
    form_req = on;
    if (on == MHD_FORM_TIMED)
    {
      tuned = false; // timed by the next stepping call
      return MHD_OK;
    }
    fused = on == MHD_FORM_FUSED;
    tuned = true;
    return MHD_OK;
  }

  size_t
  state_bytes() const
  {
    return (size_t)ncell * NV * sizeof(R);
  }

  // Time one iteration of each form on a snapshot of the current state (the
  // array the next iteration reads, the low parts of an FP32 state and the
  // time-step record), restore the snapshot after each, keep the faster.
  // The FMA-free build gives the same state in both forms bit for bit, the
  // FMA builds to round-off, so the choice changes the speed only.
  int
  tune_form()
  {
    if (tuned)
      return MHD_OK;
    tuned = true;
    if (!fused_ok())
    {
      fused = false;
      return MHD_OK;
    }
    if (int rc = read_state())
      return rc;
    if (step_finished_host())
      return MHD_OK;
    const DevState saved = *st_host;
    const int      parity = (int)(saved.it & 1);
    R *            cur = parity ? U2 : U;
    R *            snap = nullptr;
    const size_t   nb = state_bytes() * (Ulo ? 2 : 1);
    MHD_CK(cudaMalloc(&snap, nb));
    auto restore = [&]() -> cudaError_t {
      cudaError_t e = cudaMemcpyAsync(cur, snap, state_bytes(), cudaMemcpyDeviceToDevice, stream);
      if (e == cudaSuccess && Ulo)
        e = cudaMemcpyAsync(Ulo, snap + ncell * NV, state_bytes(), cudaMemcpyDeviceToDevice,
                            stream);
      *st_host = saved;
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(st, st_host, sizeof(DevState), cudaMemcpyHostToDevice, stream);
      return e;
    };
    cudaEvent_t e0, e1;
    MHD_CK(cudaEventCreate(&e0));
    MHD_CK(cudaEventCreate(&e1));
    float ms[2] = { 0.f, 0.f };
    MHD_CK(cudaMemcpyAsync(snap, cur, state_bytes(), cudaMemcpyDeviceToDevice, stream));
    if (Ulo)
      MHD_CK(cudaMemcpyAsync(snap + ncell * NV, Ulo, state_bytes(), cudaMemcpyDeviceToDevice,
                             stream));
    for (int pass = 0; pass < 3; ++pass) // a warm pass per form, then the timed ones
    {
      for (int f = 0; f < 2; ++f)
      {
        fused = f == 1;
        MHD_CK(restore());
        MHD_CK(cudaEventRecord(e0, stream));
        enqueue_step(parity);
        MHD_CK(cudaEventRecord(e1, stream));
        if (int rc = check_launch())
          return rc;
        MHD_CK(cudaEventSynchronize(e1));
        float t = 0.f;
        MHD_CK(cudaEventElapsedTime(&t, e0, e1));
        if (pass > 0)
          ms[f] += t;
      }
    }
    MHD_CK(restore());
    MHD_CK(cudaStreamSynchronize(stream));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(snap);
    fused = ms[1] <= ms[0];
    char buf[160];
    std::snprintf(buf, sizeof buf, "stages %.3f ms, fused %.3f ms per iteration -> %s",
                  ms[0] / 2, ms[1] / 2, fused ? "fused" : "stages");
    tune_report = buf;
    launched = saved.it;
    return MHD_OK;
  }

  cudaError_t
  reset_time_state()
  {
    DevState h{};
    h.t = P.tCurrent;
    h.dt = 0.0;
    h.tEnd = P.tEnd;
    h.it = 0;
    h.nStepmax = P.nStepmax;
    h.status = 0;
    *st_host = h;
    launched = 0;
    return cudaMemcpyAsync(st, st_host, sizeof(DevState), cudaMemcpyHostToDevice, stream);
  }

  Buffers<R>
  buffers(int parity) const
  {
    Buffers<R> B;
    B.Uin = parity ? U2 : U;
    B.Uout = parity ? U : U2;
    B.Q = Q;
    B.Q2 = Q2;
    B.S = S;
    B.E = E;
    B.F = F;
    B.Em = Em;
    B.H = H;
    B.Ulo = Ulo;
    B.st = st;
    return B;
  }

  static unsigned
  nblocks(int64_t n, int t)
  {
    return (unsigned)((n + t - 1) / t);
  }

  // ---- kernel launchers (dimension dispatch) ----
  void
  launch_boundaries(R * arr, int force)
  {
    if (dim == 2)
      k_boundaries<R, 2><<<nblocks(ghost_count<R, 2>(G), 256), 256, 0, stream>>>(G, arr, st, force);
    else
      k_boundaries<R, 3><<<nblocks(ghost_count<R, 3>(G), 256), 256, 0, stream>>>(G, arr, st, force);
  }
  void
  launch_prim_dt(const R * arr, int force)
  {
    const int64_t n = (int64_t)(G.isize - 1) * (G.jsize - 1) * (dim == 3 ? G.ksize - 1 : 1);
    if (dim == 2)
      k_prim_dt<R, 2><<<nblocks(n, 256), 256, 0, stream>>>(G, arr, Q, st, force);
    else
      k_prim_dt<R, 3><<<nblocks(n, 256), 256, 0, stream>>>(G, arr, Q, st, force);
  }
  void
  launch_finalize(int force)
  {
    k_finalize_dt<R><<<1, 1, 0, stream>>>(G, st, force);
  }
  void
  launch_trace(const Buffers<R> & B)
  {
    const int64_t n = (int64_t)(G.nx + 3) * (G.ny + 3) * (dim == 3 ? G.nz + 3 : 1);
    if (dim == 2)
      k_trace<R, 2><<<nblocks(n, 128), 128, 0, stream>>>(G, B);
    else
      k_trace<R, 3><<<nblocks(n, 128), 128, 0, stream>>>(G, B);
  }
  void
  launch_flux(const Buffers<R> & B)
  {
    const int64_t n = (int64_t)(G.nx + 1) * (G.ny + 1) * (dim == 3 ? G.nz + 1 : 1);
    if constexpr (sizeof(R) == 4)
    {
      if (sur_on)
      {
        SurrogateDev S{ sur_w,     reinterpret_cast<const float *>(sur_w + mlp::kPackWords),
                        sur_tau,   sur_count,
                        sur_list,  sur_nlist };
        // grid-stride: one wave of resident blocks (per direction), each
        // stages the weights once
        const unsigned nb =
          std::min(nblocks(n, kMlpThreads),
                   (unsigned)std::max(1, sur_blocks_per_sm * sm_count / (dim == 2 ? 2 : 3)));
        cudaMemsetAsync(sur_nlist, 0, sizeof(unsigned), stream);
        if (dim == 2)
          k_flux_mlp<2><<<dim3(nb, 2), kMlpThreads, kMlpSmemBytes, stream>>>(G, B, S);
        else
          k_flux_mlp<3><<<dim3(nb, 3), kMlpThreads, kMlpSmemBytes, stream>>>(G, B, S);
        return;
      }
    }
    if (dim == 2)
      k_flux<R, 2><<<dim3(nblocks(n, 128), 2), 128, 0, stream>>>(G, B);
    else
      k_flux<R, 3><<<dim3(nblocks(n, 128), 3), 128, 0, stream>>>(G, B);
  }
  void
  launch_flux_fallback(const Buffers<R> & B)
  {
    if constexpr (sizeof(R) == 4)
    {
      const unsigned nb = (unsigned)std::max(1, 4 * sm_count);
      if (dim == 2)
        k_flux_fallback<2><<<nb, 128, 0, stream>>>(G, B, sur_list, sur_nlist);
      else
        k_flux_fallback<3><<<nb, 128, 0, stream>>>(G, B, sur_list, sur_nlist);
    }
    else
      (void)B;
  }
  // Planes along the slowest axis (z in 3D, y in 2D): the edge box has
  // n + 1 of them, the interior box n.
  int
  slow_cells() const
  {
    return dim == 3 ? G.nz : G.ny;
  }
  // edges p0 <= plane < p1 of BOX_FACE
  void
  launch_emf_planes(const Buffers<R> & B, int p0, int p1)
  {
    const int64_t plane = (int64_t)(G.nx + 1) * (dim == 3 ? G.ny + 1 : 1);
    const int64_t n = (int64_t)(p1 - p0) * plane;
    if (n <= 0)
      return;
    if (dim == 2)
      k_emf<R, 2><<<dim3(nblocks(n, 128), 1), 128, 0, stream>>>(G, B, p0 * plane, p1 * plane);
    else
      k_emf<R, 3><<<dim3(nblocks(n, 128), 3), 128, 0, stream>>>(G, B, p0 * plane, p1 * plane);
  }
  // interior cells p0 <= plane < p1
  void
  launch_update_planes(const Buffers<R> & B, int p0, int p1)
  {
    const int64_t plane = (int64_t)G.nx * (dim == 3 ? G.ny : 1);
    const int64_t n = (int64_t)(p1 - p0) * plane;
    if (n <= 0)
      return;
    if (dim == 2)
      k_update<R, 2><<<nblocks(n, 256), 256, 0, stream>>>(G, B, p0 * plane, p1 * plane);
    else
      k_update<R, 3><<<nblocks(n, 256), 256, 0, stream>>>(G, B, p0 * plane, p1 * plane);
  }
  void
  launch_emf(const Buffers<R> & B)
  {
    launch_emf_planes(B, 0, slow_cells() + 1);
  }
  void
  launch_update(const Buffers<R> & B)
  {
    launch_update_planes(B, 0, slow_cells());
  }
  // ---- versions 0 and 1 ----
  void
  launch_v0_prep(const Buffers<R> & B)
  {
    const int64_t n = (int64_t)(G.isize - 1) * (G.jsize - 1) * (G.ksize - 1);
    k_v0_prep3d<R><<<nblocks(n, 128), 128, 0, stream>>>(G, B.Uin, Q, E, D, st);
  }
  void
  launch_v0_trace(const Buffers<R> & B)
  {
    const int64_t n = (int64_t)(G.isize - 1) * (G.jsize - 1) * (dim == 3 ? G.ksize - 1 : 1);
    if (dim == 2)
      k_v0_trace<R, 2><<<nblocks(n, 128), 128, 0, stream>>>(G, B.Uin, Q, E, D, T, st);
    else
      k_v0_trace<R, 3><<<nblocks(n, 128), 128, 0, stream>>>(G, B.Uin, Q, E, D, T, st);
  }
  void
  launch_v0_flux()
  {
    const int64_t n = (int64_t)(G.nx + 1) * (G.ny + 1) * (dim == 3 ? G.nz + 1 : 1);
    if (dim == 2)
      k_v0_flux<R, 2><<<dim3(nblocks(n, 128), 2), 128, 0, stream>>>(G, T, F, st);
    else
      k_v0_flux<R, 3><<<dim3(nblocks(n, 128), 3), 128, 0, stream>>>(G, T, F, st);
  }
  void
  launch_v0_emf()
  {
    const int64_t n = (int64_t)(G.nx + 1) * (G.ny + 1) * (dim == 3 ? G.nz + 1 : 1);
    if (dim == 2)
      k_v0_emf<R, 2><<<dim3(nblocks(n, 128), 1), 128, 0, stream>>>(G, T, Em, st);
    else
      k_v0_emf<R, 3><<<dim3(nblocks(n, 128), 3), 128, 0, stream>>>(G, T, Em, st);
  }
  void
  launch_v0_update(const Buffers<R> & B)
  {
    const int64_t  n = (int64_t)G.nx * G.ny * (dim == 3 ? G.nz : 1);
    const unsigned nb = nblocks(n, 256);
    if (dim == 2 && version == 0)
      k_v0_update<R, 2, 0><<<nb, 256, 0, stream>>>(G, B.Uin, B.Uout, F, Em, st);
    else if (dim == 2)
      k_v0_update<R, 2, 1><<<nb, 256, 0, stream>>>(G, B.Uin, B.Uout, F, Em, st);
    else if (version == 0)
      k_v0_update<R, 3, 0><<<nb, 256, 0, stream>>>(G, B.Uin, B.Uout, F, Em, st);
    else
      k_v0_update<R, 3, 1><<<nb, 256, 0, stream>>>(G, B.Uin, B.Uout, F, Em, st);
  }

  void
  launch_advance()
  {
    k_advance<R><<<1, 1, 0, stream>>>(st);
  }

  // ---- fused form (2D) ----
  void
  launch_dt_only(const R * arr, int force)
  {
    const int64_t n = (int64_t)G.nx * G.ny;
    k_dt_only<R, 2><<<nblocks(n, 256 * kDtCells), 256, 0, stream>>>(G, arr, st, force);
  }
  int
  fused_tile_rows() const
  {
    return (G.ny + FusedTile::TY - 1) / FusedTile::TY;
  }
  // tile rows r0 <= row < r1 (default: all)
  void
  launch_fused(const Buffers<R> & B, int r0 = 0, int r1 = -1)
  {
    using T = FusedTile;
    if (r1 < 0)
      r1 = fused_tile_rows();
    if (r1 <= r0)
      return;
    const dim3 grid((unsigned)((G.nx + T::TX - 1) / T::TX), (unsigned)(r1 - r0));
    if (G.riemann == RIEMANN_HLLD)
      k_mfused2d<R, kFusedTY, RIEMANN_HLLD>
        <<<grid, T::THREADS, T::SMEM, stream>>>(G, B.Uin, B.Uout, B.Ulo, st, r0);
    else
      k_mfused2d<R, kFusedTY, 0>
        <<<grid, T::THREADS, T::SMEM, stream>>>(G, B.Uin, B.Uout, B.Ulo, st, r0);
  }

  static constexpr int kMaxLaunches = 9;

  // Names of the launches of one iteration, in order.
  int
  step_kernel_names(const char ** names) const
  {
    static const char * v2[] = { "k_boundaries", "k_prim_dt", "k_finalize_dt", "k_trace",
                                  "k_flux",       "k_emf",     "k_update",      "k_advance" };
    static const char * v0_2d[] = { "k_boundaries", "k_prim_dt", "k_finalize_dt", "k_v0_trace",
                                    "k_v0_flux",    "k_v0_emf",  "k_v0_update",   "k_advance" };
    static const char * v0_3d[] = { "k_boundaries", "k_prim_dt", "k_finalize_dt",
                                    "k_v0_prep3d",  "k_v0_trace", "k_v0_flux",
                                    "k_v0_emf",     "k_v0_update", "k_advance" };
    static const char * v2s[] = { "k_boundaries", "k_prim_dt",       "k_finalize_dt",
                                  "k_trace",      "k_flux_mlp",      "k_flux_fallback",
                                  "k_emf",        "k_update",        "k_advance" };
    static const char * v2f[] = { "k_boundaries", "k_dt_only", "k_finalize_dt", "k_mfused2d",
                                  "k_advance" };
    const bool    fz = fused && fused_ok();
    const char ** src =
      fz ? v2f : version == 2 ? (sur_on ? v2s : v2) : (dim == 3 ? v0_3d : v0_2d);
    const int n = fz ? 5 : version == 2 ? (sur_on ? 9 : 8) : (dim == 3 ? 9 : 8);
    for (int q = 0; q < n; ++q)
      names[q] = src[q];
    return n;
  }

  // Launch number q of one iteration in the context's form.
  void
  launch_stage(int q, const Buffers<R> & B)
  {
    if (fused && fused_ok())
    {
      if (q == 0)
        return launch_boundaries(B.Uin, 0);
      if (q == 1)
        return launch_dt_only(B.Uin, 0);
      if (q == 2)
        return launch_finalize(0);
      if (q == 3)
        return launch_fused(B);
      return launch_advance();
    }
    launch_stage_plain(q, B);
  }

  // Launch number q of one iteration of the stage kernels.
  void
  launch_stage_plain(int q, const Buffers<R> & B)
  {
    if (q == 0)
      return launch_boundaries(B.Uin, 0);
    if (q == 1)
      return launch_prim_dt(B.Uin, 0);
    if (q == 2)
      return launch_finalize(0);
    if (version == 2)
    {
      if (q == 3)
        return launch_trace(B);
      if (q == 4)
        return launch_flux(B);
      if (sur_on)
      {
        if (q == 5)
          return launch_flux_fallback(B);
        --q;
      }
      if (q == 5)
        return launch_emf(B);
      if (q == 6)
        return launch_update(B);
      return launch_advance();
    }
    const int r = dim == 3 ? q - 3 : q - 2; // 3D has the extra preparation launch
    if (dim == 3 && q == 3)
      return launch_v0_prep(B);
    if (r == 1)
      return launch_v0_trace(B);
    if (r == 2)
      return launch_v0_flux();
    if (r == 3)
      return launch_v0_emf();
    if (r == 4)
      return launch_v0_update(B);
    return launch_advance();
  }

  // One iteration (godunov_unsplit_impl + next_iteration bookkeeping).
  void
  enqueue_step(int parity)
  {
    const Buffers<R> B = buffers(parity);
    const char *     names[kMaxLaunches];
    const int        n = step_kernel_names(names);
    for (int q = 0; q < n; ++q)
      launch_stage(q, B);
  }

  int
  launches_per_step() override
  {
    const char * names[kMaxLaunches];
    return step_kernel_names(names);
  }

  int
  check_launch()
  {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
    {
      err = std::string("kernel launch: ") + cudaGetErrorString(e);
      return MHD_ERR_CUDA;
    }
    return MHD_OK;
  }

  int
  build_graphs()
  {
    if (graph[0])
      return MHD_OK;
    for (int parity = 0; parity < 2; ++parity)
    {
      for (int pair = 0; pair < 2; ++pair)
      {
        cudaGraph_t g = nullptr;
        MHD_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(parity);
        if (pair)
          enqueue_step(1 - parity);
        cudaError_t le = cudaGetLastError();
        cudaError_t ce = cudaStreamEndCapture(stream, &g);
        if (le != cudaSuccess || ce != cudaSuccess)
        {
          err = std::string("graph capture: ") +
                cudaGetErrorString(le != cudaSuccess ? le : ce);
          if (g)
            cudaGraphDestroy(g);
          return MHD_ERR_CUDA;
        }
        cudaGraphExec_t ex = nullptr;
        cudaError_t     ie = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
        {
          err = std::string("graph instantiate: ") + cudaGetErrorString(ie);
          return MHD_ERR_CUDA;
        }
        (pair ? graph_pair : graph)[parity] = ex;
        // upload now so that the first replay does not pay for it
        MHD_CK(cudaGraphUpload(ex, stream));
      }
    }
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int64_t
  low_part_bytes() override
  {
    return Ulo ? ncell * NV * (int64_t)sizeof(R) : 0;
  }

  int
  get_low_parts(void * host) override
  {
    if (!Ulo)
      return MHD_OK;
    MHD_CK(cudaMemcpyAsync(host, Ulo, (size_t)low_part_bytes(), cudaMemcpyDeviceToHost, stream));
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  set_low_parts(const void * host) override
  {
    if (!Ulo)
      return MHD_OK;
    MHD_CK(cudaMemcpyAsync(Ulo, host, (size_t)low_part_bytes(), cudaMemcpyHostToDevice, stream));
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // the low parts of a state that comes from the host are zero
  int
  clear_low_parts()
  {
    if (Ulo)
      MHD_CK(cudaMemsetAsync(Ulo, 0, (size_t)ncell * NV * sizeof(R), stream));
    return MHD_OK;
  }

  // boundaries + U2 = U + primitives + dt (SolverMHDMuscl.h:393-402)
  int
  apply_init()
  {
    if (int rc = clear_low_parts())
      return rc;
    launch_boundaries(U, 1);
    MHD_CK(cudaMemcpyAsync(U2, U, (size_t)ncell * NV * sizeof(R), cudaMemcpyDeviceToDevice, stream));
    launch_prim_dt(U, 1);
    launch_finalize(1);
    if (int rc = check_launch())
      return rc;
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  upload(const void * host, R * dst, int layout)
  {
    const size_t bytes = (size_t)ncell * NV * sizeof(R);
    if (layout == MHD_LAYOUT_LEFT)
    {
      MHD_CK(cudaMemcpyAsync(dst, host, bytes, cudaMemcpyHostToDevice, stream));
    }
    else
    {
      MHD_CK(cudaMemcpyAsync(Q, host, bytes, cudaMemcpyHostToDevice, stream));
      k_transpose<R><<<nblocks(ncell * NV, 256), 256, 0, stream>>>(G, Q, dst, 0);
      if (int rc = check_launch())
        return rc;
    }
    return MHD_OK;
  }

  int
  download(const R * src, void * host, int layout)
  {
    const size_t bytes = (size_t)ncell * NV * sizeof(R);
    if (layout == MHD_LAYOUT_LEFT)
    {
      MHD_CK(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, stream));
    }
    else
    {
      k_transpose<R><<<nblocks(ncell * NV, 256), 256, 0, stream>>>(G, src, Q, 1);
      if (int rc = check_launch())
        return rc;
      MHD_CK(cudaMemcpyAsync(host, Q, bytes, cudaMemcpyDeviceToHost, stream));
    }
    return MHD_OK;
  }

  int
  init_problem() override
  {
    std::vector<double> h((size_t)ncell * NV);
    init_problem_host(P, h.data());
    if constexpr (sizeof(R) == 8)
    {
      MHD_CK(cudaMemcpy(U, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    else
    {
      std::vector<float> f(h.size());
      for (size_t q = 0; q < h.size(); ++q)
        f[q] = (float)h[q];
      MHD_CK(cudaMemcpy(U, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    MHD_CK(reset_time_state());
    return apply_init();
  }

  int
  set_state(const void * Uh, int layout) override
  {
    if (int rc = upload(Uh, U, layout))
      return rc;
    MHD_CK(reset_time_state());
    return apply_init();
  }

  int
  read_state()
  {
    MHD_CK(cudaMemcpyAsync(st_host, st, sizeof(DevState), cudaMemcpyDeviceToHost, stream));
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  R *
  current()
  {
    return (st_host->it % 2 == 0) ? U : U2;
  }

  int
  get_state(void * Uh, int layout) override
  {
    if (int rc = read_state())
      return rc;
    R * cur = current();
    // ghost cells are refreshed from the current interior (idempotent: the
    // next iteration starts with the same fill)
    launch_boundaries(cur, 1);
    if (int rc = check_launch())
      return rc;
    if (int rc = download(cur, Uh, layout))
      return rc;
    MHD_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  status_check()
  {
    if (st_host->status & STATUS_STAGING)
    {
      err = "a tile's bulk copies into shared memory did not complete within the wait bound";
      return MHD_ERR_CUDA;
    }
    if (st_host->status & STATUS_NUMERIC)
    {
      err = "non-finite or non-positive state detected (density, energy or CFL rate)";
      return MHD_ERR_NUMERIC;
    }
    return MHD_OK;
  }

  int
  step() override
  {
    if (int rc = tune_form())
      return rc;
    enqueue_step((int)(launched & 1));
    ++launched;
    return check_launch();
  }

  // SolverBase::compute_dt (SolverBase.cpp:148-179): the CFL dt, clipped to
  // tEnd, that the next iteration would take; the state is not advanced.
  int
  compute_dt(double * dt) override
  {
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    R * cur = current();
    launch_boundaries(cur, 1);
    launch_prim_dt(cur, 1);
    launch_finalize(1);
    if (int rc = check_launch())
      return rc;
    if (int rc = read_state())
      return rc;
    if (dt)
      *dt = st_host->dt;
    return status_check();
  }

  // One iteration with the caller's dt instead of the CFL dt
  // (godunov_unsplit(dt), then next_iteration's t += dt, iteration += 1).
  int
  step_dt(double dt) override
  {
    if (!(dt > 0.0) || !std::isfinite(dt))
    {
      err = "dt must be positive and finite";
      return MHD_ERR_INVALID_ARG;
    }
    if (int rc = tune_form())
      return rc;
    const Buffers<R> B = buffers((int)(launched & 1));
    const char *     names[kMaxLaunches];
    const int        n = step_kernel_names(names);
    launch_stage(0, B);
    launch_stage(1, B);
    k_set_dt<R><<<1, 1, 0, stream>>>(G, st, dt);
    for (int q = 3; q < n; ++q)
      launch_stage(q, B);
    ++launched;
    return check_launch();
  }

  int
  run(int nsteps, int * done) override
  {
    if (int rc = tune_form())
      return rc;
    if (int rc = build_graphs())
      return rc;
    if (int rc = read_state())
      return rc;
    const int it0 = st_host->it;
    launched = it0;
    int left = nsteps;
    while (left >= 2)
    {
      MHD_CK(cudaGraphLaunch(graph_pair[launched & 1], stream));
      launched += 2;
      left -= 2;
    }
    if (left)
    {
      MHD_CK(cudaGraphLaunch(graph[launched & 1], stream));
      launched += 1;
    }
    if (int rc = read_state())
      return rc;
    if (done)
      *done = st_host->it - it0;
    return status_check();
  }

  // Slabs of the host-buffer step: one per 64 MiB of state, at most 16 (or
  // the count set by set_host_slabs), never more than the planes.
  int
  host_slabs() const
  {
    const size_t bytes = (size_t)ncell * NV * sizeof(R);
    int          n = host_slabs_req > 0 ? host_slabs_req
                                        : (int)std::min<size_t>(16, bytes / ((size_t)64 << 20));
    return std::max(1, std::min(n, slow_cells()));
  }

  int
  set_host_slabs(int n) override
  {
    if (n < 0 || n > kMaxHostSlabs)
    {
      err = "host slabs must be in 0.." + std::to_string(kMaxHostSlabs);
      return MHD_ERR_INVALID_ARG;
    }
    host_slabs_req = n;
    return MHD_OK;
  }

  // One iteration on host arrays with the copies overlapped, in nslab slabs
  // along the slowest axis (z in 3D, y in 2D).
  //  in:  slab s of U_in goes up on a second stream; the main stream fills
  //       the ghost cells of the slab's interior planes along the fast axes
  //       (their sources lie in the same plane) and computes primitives and
  //       CFL rates of every plane whose next plane has arrived (the cell
  //       reads the face field of its +1 neighbour).  After the last slab:
  //       the ghost planes of the slow axis, then their primitives.
  //  out: edge EMFs and the update run slab by slab; update slab [u0, u1)
  //       reads the edges of planes u0 .. u1, so the edge launch before it
  //       covers every plane up to u1; each finished slab of U_out goes down
  //       on the second stream while the next slab computes.
  // Ghost planes travel with the first and last slab.  Every cell is
  // computed once by the kernel bodies of enqueue_step, so the result is
  // bitwise the same; only the order of the CFL atomics differs, and their
  // maximum is order-independent.
  int
  make_copy_stream()
  {
    if (!copy_stream)
    {
      MHD_CK(cudaStreamCreateWithFlags(&copy_stream, cudaStreamNonBlocking));
      MHD_CK(cudaEventCreateWithFlags(&copy_ev, cudaEventDisableTiming));
      for (cudaEvent_t & e : slab_ev)
        MHD_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
      for (cudaEvent_t & e : up_ev)
        MHD_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    return MHD_OK;
  }

  // The host-buffer step of the fused form (2D), in nslab slabs of tile rows:
  //  in:  slab s of U_in goes up on the second stream; the main stream fills
  //       the ghost cells of its rows along x and reduces the CFL rates of
  //       every interior row whose next row has arrived; after the last slab
  //       the ghost rows, the remaining rates and dt;
  //  out: the tile kernel runs slab by slab, each finished slab of U_out
  //       going down while the next one computes.
  // The same kernels on the same cells as enqueue_step: bitwise its result.
  int
  enqueue_step_host_fused(int parity, const void * in_host, void * out_host, int nslab)
  {
    if (int rc = make_copy_stream())
      return rc;
    const Buffers<R> B = buffers(parity);
    const int        ns = G.ny, g = G.g, nplanes = G.jsize, ntr = fused_tile_rows();
    const int64_t    plane = G.sj;
    nslab = std::max(1, std::min(nslab, ntr));
    auto t_lo = [&](int s) { return (int)((int64_t)s * ntr / nslab); }; // tile rows
    auto u_lo = [&](int s) { return std::min(ns, t_lo(s) * FusedTile::TY); };
    auto a_lo = [&](int s) { return s == 0 ? 0 : g + u_lo(s); };
    auto a_hi = [&](int s) { return s == nslab - 1 ? nplanes : g + u_lo(s + 1); };
    auto copy = [&](void * dst, const void * src, int s, cudaMemcpyKind kind) -> int {
      for (int v = 0; v < NV; ++v)
      {
        const int64_t off = v * G.sv + (int64_t)a_lo(s) * plane;
        const size_t  bytes = (size_t)(a_hi(s) - a_lo(s)) * plane * sizeof(R);
        MHD_CK(cudaMemcpyAsync(static_cast<R *>(dst) + off, static_cast<const R *>(src) + off,
                               bytes, kind, copy_stream));
      }
      return MHD_OK;
    };
    auto bound = [&](int p0, int p1, int reset) {
      const int64_t n = (int64_t)(p1 - p0) * plane;
      if (n > 0)
        k_boundaries_range<R, 2>
          <<<nblocks(n, 256), 256, 0, stream>>>(G, B.Uin, st, p0 * plane, p1 * plane, reset);
    };
    auto rates = [&](int r0, int r1) { // interior rows r0 <= row < r1 (0-based)
      const int64_t n = (int64_t)(r1 - r0) * G.nx;
      if (n > 0)
        k_dt_only_range<R, 2><<<nblocks(n, 256), 256, 0, stream>>>(
          G, B.Uin, st, (int64_t)r0 * G.nx, (int64_t)r1 * G.nx);
    };
    MHD_CK(cudaEventRecord(copy_ev, stream));
    MHD_CK(cudaStreamWaitEvent(copy_stream, copy_ev, 0));
    for (int s = 0; s < nslab; ++s)
    {
      if (int rc = copy(B.Uin, in_host, s, cudaMemcpyHostToDevice))
        return rc;
      MHD_CK(cudaEventRecord(up_ev[s], copy_stream));
    }
    int rdone = 0; // interior rows whose rates are reduced
    for (int s = 0; s < nslab; ++s)
    {
      MHD_CK(cudaStreamWaitEvent(stream, up_ev[s], 0));
      bound(g + u_lo(s), g + u_lo(s + 1), s == 0);
      // a row's rate reads the face field of the next row
      const int r1 = s == nslab - 1 ? rdone : std::max(rdone, u_lo(s + 1) - 1);
      rates(rdone, r1);
      rdone = r1;
    }
    bound(0, g, 0);
    bound(g + ns, nplanes, 0);
    rates(rdone, ns);
    launch_finalize(0);
    for (int s = 0; s < nslab; ++s)
    {
      launch_fused(B, t_lo(s), t_lo(s + 1));
      MHD_CK(cudaEventRecord(slab_ev[s], stream));
    }
    launch_advance();
    if (int rc = check_launch())
      return rc;
    for (int s = 0; s < nslab; ++s)
    {
      MHD_CK(cudaStreamWaitEvent(copy_stream, slab_ev[s], 0));
      if (int rc = copy(out_host, B.Uout, s, cudaMemcpyDeviceToHost))
        return rc;
    }
    MHD_CK(cudaEventRecord(copy_ev, copy_stream));
    MHD_CK(cudaStreamWaitEvent(stream, copy_ev, 0));
    return MHD_OK;
  }

  int
  enqueue_step_host(int parity, const void * in_host, void * out_host, int nslab)
  {
    if (int rc = make_copy_stream())
      return rc;
    const Buffers<R> B = buffers(parity);
    const int        ns = slow_cells(), g = G.g;
    const int        nplanes = dim == 3 ? G.ksize : G.jsize;
    const int64_t    plane = dim == 3 ? G.sk : G.sj;      // array cells per plane
    const int64_t    pplane = dim == 3 ? (int64_t)(G.isize - 1) * (G.jsize - 1)
                                       : (int64_t)(G.isize - 1); // BOX_PRIM cells per plane
    auto             u_lo = [&](int s) { return (int)((int64_t)s * ns / nslab); };
    auto             a_lo = [&](int s) { return s == 0 ? 0 : g + u_lo(s); };
    auto             a_hi = [&](int s) { return s == nslab - 1 ? nplanes : g + u_lo(s + 1); };
    auto             copy = [&](void * dst, const void * src, int s, cudaMemcpyKind kind) -> int {
      for (int v = 0; v < NV; ++v)
      {
        const int64_t off = v * G.sv + (int64_t)a_lo(s) * plane;
        const size_t  bytes = (size_t)(a_hi(s) - a_lo(s)) * plane * sizeof(R);
        MHD_CK(cudaMemcpyAsync(static_cast<R *>(dst) + off, static_cast<const R *>(src) + off,
                               bytes, kind, copy_stream));
      }
      return MHD_OK;
    };
    auto bound = [&](int p0, int p1, int reset) {
      const int64_t n = (int64_t)(p1 - p0) * plane;
      if (n <= 0)
        return;
      if (dim == 2)
        k_boundaries_range<R, 2>
          <<<nblocks(n, 256), 256, 0, stream>>>(G, B.Uin, st, p0 * plane, p1 * plane, reset);
      else
        k_boundaries_range<R, 3>
          <<<nblocks(n, 256), 256, 0, stream>>>(G, B.Uin, st, p0 * plane, p1 * plane, reset);
    };
    auto prim = [&](int p0, int p1) {
      const int64_t n = (int64_t)(p1 - p0) * pplane;
      if (n <= 0)
        return;
      if (dim == 2)
        k_prim_dt_range<R, 2>
          <<<nblocks(n, 256), 256, 0, stream>>>(G, B.Uin, Q, st, p0 * pplane, p1 * pplane);
      else
        k_prim_dt_range<R, 3>
          <<<nblocks(n, 256), 256, 0, stream>>>(G, B.Uin, Q, st, p0 * pplane, p1 * pplane);
    };
    // uploads (ordered after everything already on the main stream)
    MHD_CK(cudaEventRecord(copy_ev, stream));
    MHD_CK(cudaStreamWaitEvent(copy_stream, copy_ev, 0));
    for (int s = 0; s < nslab; ++s)
    {
      if (int rc = copy(B.Uin, in_host, s, cudaMemcpyHostToDevice))
        return rc;
      MHD_CK(cudaEventRecord(up_ev[s], copy_stream));
    }
    // the trace stage in two parts over BOX_TRACE, whose plane kb is array
    // plane g - 1 + kb: part 1 (no dt) of array planes p0 .. p1-1, part 2
    const int64_t tplane = dim == 3 ? (int64_t)(G.nx + 3) * (G.ny + 3) : (int64_t)(G.nx + 3);
    auto          trace = [&](int part, int p0, int p1) {
      const int64_t t0 = (int64_t)(p0 - (g - 1)) * tplane, t1 = (int64_t)(p1 - (g - 1)) * tplane;
      if (t1 <= t0)
        return;
      const unsigned nb = nblocks(t1 - t0, 128);
      if (dim == 2 && part == 1)
        k_trace_range<R, 2, 1><<<nb, 128, 0, stream>>>(G, B, t0, t1);
      else if (dim == 2)
        k_trace_range<R, 2, 2><<<nb, 128, 0, stream>>>(G, B, t0, t1);
      else if (part == 1)
        k_trace_range<R, 3, 1><<<nb, 128, 0, stream>>>(G, B, t0, t1);
      else
        k_trace_range<R, 3, 2><<<nb, 128, 0, stream>>>(G, B, t0, t1);
    };
    // ghost fill, primitives, CFL; part 1 of the trace stage on the planes
    // whose primitives on both sides are done (it reads planes k-1 .. k+1)
    int pdone = g;     // BOX_PRIM planes g .. pdone-1 are done
    int tdone = g + 1; // trace part 1 of array planes g+1 .. tdone-1 is done
    for (int s = 0; s < nslab; ++s)
    {
      MHD_CK(cudaStreamWaitEvent(stream, up_ev[s], 0));
      bound(g + u_lo(s), g + u_lo(s + 1), s == 0);
      const int p1 = g + u_lo(s + 1) - 1;
      prim(pdone, p1);
      pdone = std::max(pdone, p1);
      trace(1, tdone, pdone - 1);
      tdone = std::max(tdone, pdone - 1);
    }
    bound(0, g, 0);
    bound(g + ns, nplanes, 0);
    prim(0, g);
    prim(pdone, nplanes - 1);
    trace(1, g - 1, g + 1);
    trace(1, tdone, g + ns + 2);
    // dt, trace part 2, face fluxes
    const char * names[kMaxLaunches];
    const int    n = step_kernel_names(names);
    const int    q_emf = sur_on ? 6 : 5;
    launch_stage(2, B);
    trace(2, g - 1, g + ns + 2);
    for (int q = 4; q < q_emf; ++q)
      launch_stage(q, B);
    // edges and update in slabs
    int e_done = 0;
    for (int s = 0; s < nslab; ++s)
    {
      launch_emf_planes(B, e_done, u_lo(s + 1) + 1);
      e_done = u_lo(s + 1) + 1;
      launch_update_planes(B, u_lo(s), u_lo(s + 1));
      MHD_CK(cudaEventRecord(slab_ev[s], stream));
    }
    for (int q = q_emf + 2; q < n; ++q)
      launch_stage(q, B);
    if (int rc = check_launch())
      return rc;
    // downloads
    for (int s = 0; s < nslab; ++s)
    {
      MHD_CK(cudaStreamWaitEvent(copy_stream, slab_ev[s], 0));
      if (int rc = copy(out_host, B.Uout, s, cudaMemcpyDeviceToHost))
        return rc;
    }
    MHD_CK(cudaEventRecord(copy_ev, copy_stream));
    MHD_CK(cudaStreamWaitEvent(stream, copy_ev, 0));
    return MHD_OK;
  }

  int
  step_host(const void * Uin, void * Uout, int layout) override
  {
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    if (int rc = tune_form())
      return rc;
    const int  nslab = host_slabs();
    const bool overlap = layout == MHD_LAYOUT_LEFT && version == 2 && nslab > 1;
    R *        out = (launched & 1) ? U : U2; // the buffer this iteration writes
    // the host state is one float per value: the step starts without low parts
    if (int rc = clear_low_parts())
      return rc;
    if (overlap)
    {
      const int par = (int)(launched & 1);
      if (int rc = fused ? enqueue_step_host_fused(par, Uin, Uout, nslab)
                         : enqueue_step_host(par, Uin, Uout, nslab))
        return rc;
      ++launched;
    }
    else
    {
      if (int rc = upload(Uin, current(), layout))
        return rc;
      enqueue_step((int)(launched & 1));
      ++launched;
      if (int rc = check_launch())
        return rc;
      if (int rc = download(out, Uout, layout))
        return rc;
    }
    if (int rc = read_state())
      return rc;
    return status_check();
  }

  int
  time(double * t, double * dt, int * it) override
  {
    if (int rc = read_state())
      return rc;
    if (t)
      *t = st_host->t;
    if (dt)
      *dt = st_host->dt;
    if (it)
      *it = st_host->it;
    return MHD_OK;
  }

  int
  diagnostics(double sums[8], double * divb_l1, double * divb_max) override
  {
    if (int rc = read_state())
      return rc;
    R * cur = current();
    launch_boundaries(cur, 1);
    if (dim == 2)
      k_diag<R, 2><<<kDiagBlocks, 256, 0, stream>>>(G, cur, diag);
    else
      k_diag<R, 3><<<kDiagBlocks, 256, 0, stream>>>(G, cur, diag);
    k_diag_final<<<1, 32, 0, stream>>>(diag, kDiagBlocks, diag + kDiagBlocks * 10);
    if (int rc = check_launch())
      return rc;
    double out[10];
    MHD_CK(cudaMemcpyAsync(out, diag + kDiagBlocks * 10, sizeof out, cudaMemcpyDeviceToHost, stream));
    MHD_CK(cudaStreamSynchronize(stream));
    for (int q = 0; q < 8; ++q)
      sums[q] = out[q];
    const double ncells = (double)G.nx * G.ny * (dim == 3 ? G.nz : 1);
    if (divb_l1)
      *divb_l1 = out[8] / ncells;
    if (divb_max)
      *divb_max = out[9];
    return MHD_OK;
  }

  int
  run_timed(int nsteps, float * ms) override
  {
    if (int rc = tune_form())
      return rc;
    if (int rc = build_graphs())
      return rc;
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    cudaEvent_t e0, e1;
    MHD_CK(cudaEventCreate(&e0));
    MHD_CK(cudaEventCreate(&e1));
    MHD_CK(cudaEventRecord(e0, stream));
    int left = nsteps;
    while (left >= 2)
    {
      MHD_CK(cudaGraphLaunch(graph_pair[launched & 1], stream));
      launched += 2;
      left -= 2;
    }
    if (left)
    {
      MHD_CK(cudaGraphLaunch(graph[launched & 1], stream));
      launched += 1;
    }
    MHD_CK(cudaEventRecord(e1, stream));
    MHD_CK(cudaEventSynchronize(e1));
    MHD_CK(cudaEventElapsedTime(ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (int rc = read_state())
      return rc;
    return status_check();
  }

  int
  profile_step(const char ** names, float * ms, int max, int * count) override
  {
    if (int rc = tune_form())
      return rc;
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    const Buffers<R> B = buffers((int)(launched & 1));
    const char *     kn[kMaxLaunches];
    const int        n = step_kernel_names(kn);
    cudaEvent_t      ev[kMaxLaunches + 1];
    for (int q = 0; q <= n; ++q)
      MHD_CK(cudaEventCreate(&ev[q]));
    MHD_CK(cudaEventRecord(ev[0], stream));
    for (int q = 0; q < n; ++q)
    {
      launch_stage(q, B);
      MHD_CK(cudaEventRecord(ev[q + 1], stream));
    }
    ++launched;
    if (int rc = check_launch())
      return rc;
    MHD_CK(cudaEventSynchronize(ev[n]));
    for (int q = 0; q < n && q < max; ++q)
    {
      if (names)
        names[q] = kn[q];
      MHD_CK(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
    }
    for (int q = 0; q <= n; ++q)
      cudaEventDestroy(ev[q]);
    if (count)
      *count = n;
    return MHD_OK;
  }

  void
  drop_graphs()
  {
    for (int q = 0; q < 2; ++q)
    {
      if (graph[q])
        cudaGraphExecDestroy(graph[q]);
      if (graph_pair[q])
        cudaGraphExecDestroy(graph_pair[q]);
      graph[q] = graph_pair[q] = nullptr;
    }
  }

  // Deploy (wpack != nullptr) or remove the flux surrogate; the packed words
  // are followed by the biases (mlp::kBiasFloats floats).
  int
  set_surrogate(const uint32_t * wpack, double tau) override
  {
    if constexpr (sizeof(R) != 4)
    {
      (void)wpack;
      (void)tau;
      err = "the flux surrogate runs in FP32 contexts only";
      return MHD_ERR_INVALID_ARG;
    }
    else
    {
      MHD_CK(cudaStreamSynchronize(stream));
      drop_graphs();
      fused = false; // the fused form has no surrogate
      tuned = true;
      if (!wpack)
      {
        sur_on = false;
        // the form the context had: the requested one, else the default
        if (form_req == MHD_FORM_FUSED)
          fused = true;
        else if (form_req == MHD_FORM_TIMED)
          tuned = false;
        else if (form_req != MHD_FORM_STAGES)
          fused = default_form();
        return MHD_OK;
      }
      if (version != 2 || G.riemann != MHD_RIEMANN_HLLD)
      {
        err = "the flux surrogate needs implementation version 2 and the HLLD solver";
        return MHD_ERR_INVALID_ARG;
      }
      const int64_t nlist = G.box[BOX_FACE].count() * dim;
      if (nlist >= (int64_t)UINT32_MAX)
      {
        err = "grid too large for the surrogate's 32-bit face list";
        return MHD_ERR_TOO_LARGE;
      }
      const size_t bytes = (mlp::kPackWords + mlp::kBiasFloats) * sizeof(uint32_t);
      if (!sur_w)
        MHD_CK(cudaMalloc(&sur_w, bytes));
      if (!sur_count)
        MHD_CK(cudaMalloc(&sur_count, 2 * sizeof(unsigned long long)));
      if (!sur_list)
        MHD_CK(cudaMalloc(&sur_list, nlist * sizeof(uint32_t)));
      if (!sur_nlist)
        MHD_CK(cudaMalloc(&sur_nlist, sizeof(unsigned)));
      MHD_CK(cudaMemcpy(sur_w, wpack, bytes, cudaMemcpyHostToDevice));
      MHD_CK(cudaMemset(sur_count, 0, 2 * sizeof(unsigned long long)));
      MHD_CK(cudaMemset(sur_nlist, 0, sizeof(unsigned)));
      if (!sm_count)
        MHD_CK(cudaDeviceGetAttribute(&sm_count, cudaDevAttrMultiProcessorCount, P.device));
      if (dim == 2)
      {
        MHD_CK(cudaFuncSetAttribute(k_flux_mlp<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMlpSmemBytes));
        MHD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sur_blocks_per_sm, k_flux_mlp<2>,
                                                             kMlpThreads, kMlpSmemBytes));
      }
      else
      {
        MHD_CK(cudaFuncSetAttribute(k_flux_mlp<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    kMlpSmemBytes));
        MHD_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&sur_blocks_per_sm, k_flux_mlp<3>,
                                                             kMlpThreads, kMlpSmemBytes));
      }
      sur_blocks_per_sm = std::max(1, sur_blocks_per_sm);
      sur_tau = (float)tau;
      sur_on = true;
      return MHD_OK;
    }
  }

  int
  surrogate_stats(int64_t * used, int64_t * total, int reset) override
  {
    unsigned long long h[2] = { 0, 0 };
    if (sur_count)
    {
      MHD_CK(cudaMemcpyAsync(h, sur_count, sizeof h, cudaMemcpyDeviceToHost, stream));
      MHD_CK(cudaStreamSynchronize(stream));
      if (reset)
        MHD_CK(cudaMemset(sur_count, 0, sizeof h));
    }
    if (used)
      *used = (int64_t)h[0];
    if (total)
      *total = (int64_t)h[1];
    return MHD_OK;
  }

  // Face samples of the current state (the faces of the next iteration):
  // boundaries, primitives, dt and the trace are computed, nothing is
  // advanced.  One record per `stride`-th face of each direction.
  int
  harvest(int stride, float * host, int64_t capacity, int64_t * count) override
  {
    if (version != 2)
    {
      err = "face harvesting needs implementation version 2";
      return MHD_ERR_INVALID_ARG;
    }
    if (int rc = read_state())
      return rc;
    if (step_finished_host())
    {
      err = "the run is finished: no next iteration to sample";
      return MHD_ERR_INVALID_ARG;
    }
    const int64_t nface = G.box[BOX_FACE].count();
    const int64_t nslot = (nface + stride - 1) / stride;
    const int64_t nrec = nslot * dim;
    if (count)
      *count = nrec;
    if (!host)
      return MHD_OK; // size query
    if (capacity < nrec)
    {
      err = "harvest buffer holds " + std::to_string(capacity) + " records, " +
            std::to_string(nrec) + " needed";
      return MHD_ERR_TOO_LARGE;
    }
    launched = st_host->it;
    const Buffers<R> B = buffers((int)(launched & 1));
    float *          d_out = nullptr;
    MHD_CK(cudaMalloc(&d_out, nrec * mlp::kRecord * sizeof(float)));
    launch_stage_plain(0, B);
    launch_stage_plain(1, B);
    launch_stage_plain(2, B);
    launch_stage_plain(3, B);
    if (dim == 2)
      k_harvest<R, 2><<<dim3(nblocks(nslot, 128), 2), 128, 0, stream>>>(G, B, d_out, stride, nslot);
    else
      k_harvest<R, 3><<<dim3(nblocks(nslot, 128), 3), 128, 0, stream>>>(G, B, d_out, stride, nslot);
    int rc = check_launch();
    cudaError_t e = cudaMemcpyAsync(host, d_out, nrec * mlp::kRecord * sizeof(float),
                                    cudaMemcpyDeviceToHost, stream);
    cudaError_t e2 = cudaStreamSynchronize(stream);
    cudaFree(d_out);
    if (rc)
      return rc;
    if (e != cudaSuccess || e2 != cudaSuccess)
    {
      err = std::string("harvest copy: ") + cudaGetErrorString(e != cudaSuccess ? e : e2);
      return MHD_ERR_CUDA;
    }
    return MHD_OK;
  }

  void
  set_time_origin(double t) override
  {
    P.tCurrent = t;
  }

  bool
  step_finished_host() const
  {
    return st_host->t >= st_host->tEnd - 1e-14 || st_host->it >= st_host->nStepmax;
  }

  int
  cell_counts(int64_t * interior, int64_t * with_ghosts) override
  {
    if (interior)
      *interior = (int64_t)G.nx * G.ny * (dim == 3 ? G.nz : 1);
    if (with_ghosts)
      *with_ghosts = (int64_t)G.isize * G.jsize * (dim == 3 ? G.ksize : 1);
    return MHD_OK;
  }

  int
  sizes(int s[4]) override
  {
    s[0] = G.isize;
    s[1] = G.jsize;
    s[2] = G.ksize;
    s[3] = NV;
    return MHD_OK;
  }
};

#undef MHD_CK

} // namespace MHD_VARIANT_TAG
} // namespace mhd
