// Ensemble of independent MHD problems of uneven size advanced together.
//
// Every launch of an iteration covers all problems at once: a block map
// assigns each CUDA block to one problem and to a block of that problem's
// box, so one set of 8 launches (5 in the fused 2D form: one block per
// problem tile) advances the whole ensemble by one iteration, each problem
// with its own CFL dt, time and stopping rule (SolverBase::finished per
// problem).  Whole runs replay from CUDA graphs
// without host synchronisation.  The launch shape (threads per block) of
// every kernel is picked by a small autotuner that times the candidates on
// the ensemble itself.
//
// The reference has no ensemble mode: each problem is exactly the
// single-problem iteration of mhd_kernels.cuh (implementation version 2),
// and the tests check bitwise agreement with independent single runs.
#pragma once

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mhd_core.h"
#include "mhd_solver.cuh"

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

// (problem, block index inside the problem's box) of every CUDA block
struct BlockRef
{
  int p, b;
};

// The grid and buffers of the block's problem, copied into shared memory
// by the block (the bodies then read them like kernel parameters), with the
// state arrays swapped for odd parities.
template <class R>
struct ProblemView
{
  Grid<R>    G;
  Buffers<R> B;
};

template <class R>
__device__ __forceinline__ void
load_problem(ProblemView<R> & v, const Grid<R> * Gs, const Buffers<R> * Bs, int p, int parity)
{
  static_assert(sizeof(Grid<R>) % 4 == 0 && sizeof(Buffers<R>) % 4 == 0, "word copies");
  const int nG = (int)(sizeof(Grid<R>) / 4), nB = (int)(sizeof(Buffers<R>) / 4);
  const unsigned * gsrc = reinterpret_cast<const unsigned *>(Gs + p);
  const unsigned * bsrc = reinterpret_cast<const unsigned *>(Bs + p);
  unsigned *       gdst = reinterpret_cast<unsigned *>(&v.G);
  unsigned *       bdst = reinterpret_cast<unsigned *>(&v.B);
  for (int q = threadIdx.x; q < nG + nB; q += blockDim.x)
  {
    if (q < nG)
      gdst[q] = gsrc[q];
    else
      bdst[q - nG] = bsrc[q - nG];
  }
  __syncthreads();
  if (parity && threadIdx.x == 0)
  {
    R * t = v.B.Uin;
    v.B.Uin = v.B.Uout;
    v.B.Uout = t;
  }
  __syncthreads();
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_boundaries(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  boundaries_body<R, DIM>(v.G, v.B.Uin, v.B.st, 0, m.b * (int64_t)blockDim.x + threadIdx.x,
                          m.b == 0 && threadIdx.x == 0);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_prim_dt(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  prim_dt_body<R, DIM>(v.G, v.B.Uin, v.B.Q, v.B.st, 0, m.b * (int64_t)blockDim.x + threadIdx.x);
}

template <class R>
__global__ void
kb_finalize_dt(const Grid<R> * Gs, const Buffers<R> * Bs, int nprob)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nprob)
    finalize_dt_body<R>(Gs[p], Bs[p].st, 0);
}

template <class R>
__global__ void
kb_advance(const Buffers<R> * Bs, int nprob)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nprob)
    return;
  DevState * st = Bs[p].st;
  if (step_finished(st))
    return;
  st->it += 1;
  st->t += st->dt;
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_trace(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  trace_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + threadIdx.x);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_flux(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  flux_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + threadIdx.x, blockIdx.y);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_emf(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  emf_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + threadIdx.x, blockIdx.y);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_update(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  update_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + threadIdx.x);
}

// ---------------------------------------------------------------- fused form (2D)

// The CFL reduction of the fused form over all problems: interior cells,
// primitives computed but not stored (each tile computes its own), kDtCells
// cells per thread.
template <class R, int DIM>
__global__ void __launch_bounds__(256)
kb_dt_only(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R> v;
  const BlockRef            m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  dt_cells_body<R, DIM, kDtCells>(v.G, v.B.Uin, v.B.st, 0, m.b);
}

// One iteration of one tile of one problem per block (the block map holds
// (problem, tile) with the tiles of a problem row by row): the
// single-problem tile kernel's body on the problem's grid and arrays.
template <class R, int TY, int RS>
__global__ void __launch_bounds__(MTile<R, TY>::THREADS, MTile<R, TY>::MIN_BLOCKS)
kb_mfused2d(const Grid<R> * Gs, const Buffers<R> * Bs, const BlockRef * map, int parity)
{
  __shared__ ProblemView<R>                   v;
  extern __shared__ __align__(16) unsigned char msm_raw[];
  const BlockRef                              m = map[blockIdx.x];
  load_problem(v, Gs, Bs, m.p, parity);
  const int ntx = (v.G.nx + MTile<R, TY>::TX - 1) / MTile<R, TY>::TX;
  mfused2d_tile<R, TY, RS>(v.G, v.B.Uin, v.B.Uout, v.B.Ulo, v.B.st, m.b % ntx, m.b / ntx,
                           msm_raw);
}

// ---------------------------------------------------------------- persistent form

// One work item of the persistent kernel: a problem, a block of that
// problem's box and, for the face and edge stages, the direction.
struct PersistRef
{
  int p, b, d;
};

// Work lists of the six box stages (boundaries, primitives + CFL, trace,
// faces, edges, update) for blocks of kPersistThreads threads.
constexpr int kPersistThreads = 256;
struct PersistWork
{
  const PersistRef * list[6];
  unsigned           n[6];
};

// Grid-wide barrier state of the persistent kernel.
struct PersistSync
{
  unsigned count, gen; // arrivals at the current barrier, barrier generation
  int      status;     // non-zero: a wait gave up; every block stops
  int      pad;
};

// Grid-wide barrier with a bounded wait.  Thread 0 of every block arrives;
// the last arrival opens the barrier (next generation), the others spin on
// the generation for at most `budget` clock cycles.  A wait that gives up
// sets sync->status and returns false, and so does every wait that sees the
// status set: the kernel then ends early and the host reports the error.
// The launch is cooperative, so all blocks are resident and a normal
// barrier always opens.
__device__ __forceinline__ bool
grid_barrier(PersistSync * s, long long budget)
{
  __shared__ int go;
  __syncthreads();
  if (threadIdx.x == 0)
  {
    volatile unsigned * vgen = &s->gen;
    volatile int *      vst = &s->status;
    int                 ok = 1;
    const unsigned      g = *vgen;
    __threadfence();
    if (atomicAdd(&s->count, 1u) == gridDim.x - 1)
    {
      atomicExch(&s->count, 0u);
      __threadfence();
      atomicAdd(&s->gen, 1u);
    }
    else
    {
      const long long t0 = clock64();
      while (*vgen == g)
      {
        if (*vst != 0 || clock64() - t0 > budget)
        {
          atomicExch(&s->status, 1);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    if (*vst != 0)
      ok = 0;
    go = ok;
  }
  __syncthreads();
  return go != 0;
}

// All iterations of a run in one cooperative launch: the stages of every
// iteration follow each other with grid-wide barriers instead of separate
// launches; each block takes work items of the current stage in turn (the
// same bodies, indices and arithmetic as the per-stage kernels above, so the
// states are the same bit for bit).
template <class R, int DIM>
__global__ void __launch_bounds__(kPersistThreads)
kp_run(const Grid<R> * Gs, const Buffers<R> * Bs, const PersistWork W, int nprob, int parity0,
       int niter, PersistSync * sync, long long budget)
{
  __shared__ ProblemView<R> v;
  const int64_t t = threadIdx.x;
  for (int it = 0; it < niter; ++it)
  {
    const int parity = (parity0 + it) & 1;
    for (unsigned w = blockIdx.x; w < W.n[0]; w += gridDim.x)
    {
      const PersistRef m = W.list[0][w];
      load_problem(v, Gs, Bs, m.p, parity);
      boundaries_body<R, DIM>(v.G, v.B.Uin, v.B.st, 0, m.b * (int64_t)blockDim.x + t,
                              m.b == 0 && t == 0);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (unsigned w = blockIdx.x; w < W.n[1]; w += gridDim.x)
    {
      const PersistRef m = W.list[1][w];
      load_problem(v, Gs, Bs, m.p, parity);
      prim_dt_body<R, DIM>(v.G, v.B.Uin, v.B.Q, v.B.st, 0, m.b * (int64_t)blockDim.x + t);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nprob; p += gridDim.x * blockDim.x)
      finalize_dt_body<R>(Gs[p], Bs[p].st, 0);
    if (!grid_barrier(sync, budget))
      return;
    for (unsigned w = blockIdx.x; w < W.n[2]; w += gridDim.x)
    {
      const PersistRef m = W.list[2][w];
      load_problem(v, Gs, Bs, m.p, parity);
      trace_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + t);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (unsigned w = blockIdx.x; w < W.n[3]; w += gridDim.x)
    {
      const PersistRef m = W.list[3][w];
      load_problem(v, Gs, Bs, m.p, parity);
      flux_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + t, m.d);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (unsigned w = blockIdx.x; w < W.n[4]; w += gridDim.x)
    {
      const PersistRef m = W.list[4][w];
      load_problem(v, Gs, Bs, m.p, parity);
      emf_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + t, m.d);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (unsigned w = blockIdx.x; w < W.n[5]; w += gridDim.x)
    {
      const PersistRef m = W.list[5][w];
      load_problem(v, Gs, Bs, m.p, parity);
      update_body<R, DIM>(v.G, v.B, m.b * (int64_t)blockDim.x + t);
      __syncthreads();
    }
    if (!grid_barrier(sync, budget))
      return;
    for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nprob; p += gridDim.x * blockDim.x)
    {
      DevState * st = Bs[p].st;
      if (!step_finished(st))
      {
        st->it += 1;
        st->t += st->dt;
      }
    }
    if (!grid_barrier(sync, budget))
      return;
  }
}

#define MHD_ECK(call)                                                                 \
  do                                                                                  \
  {                                                                                   \
    cudaError_t e_ = (call);                                                          \
    if (e_ != cudaSuccess)                                                            \
    {                                                                                 \
      err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
      return MHD_ERR_CUDA;                                                            \
    }                                                                                 \
  } while (0)

template <class R>
class EnsembleImpl final : public EnsembleCore
{
public:
  // launch kinds with their own block map and launch shape
  enum Kind
  {
    K_BC = 0,
    K_PRIM,
    K_TRACE,
    K_FLUX,
    K_EMF,
    K_UPDATE,
    K_DT,    // fused form: CFL reduction without stored primitives
    K_FUSED, // fused form: one block per (problem, tile), 256 threads
    K_COUNT
  };
  static constexpr const char * kKindName[K_COUNT] = { "boundaries", "prim_dt", "trace", "flux",
                                                       "emf",        "update",  "dt_only",
                                                       "fused" };
  static constexpr int kFusedTY = sizeof(R) == 4 ? MFUSED_TILE_ROWS : 8;
  using FusedTile = MTile<R, kFusedTY>;

  std::vector<mhd_params> P;
  std::vector<Grid<R>>    G;     // host copies
  std::vector<Buffers<R>> B;     // host copies (parity 0)
  Grid<R> *               dG = nullptr;
  Buffers<R> *            dB = nullptr;
  R *                     arena = nullptr;
  DevState *              st = nullptr;
  DevState *              st_host = nullptr;
  int                     dim = 2, n = 0;
  int                     threads[K_COUNT] = { 256, 256, 128, 128, 128, 256, 256, 256 };
  int                     fused_rs = 0; // RIEMANN_HLLD when every problem uses it
  BlockRef *              map[K_COUNT] = {};
  unsigned                nblk[K_COUNT] = {};
  cudaStream_t            stream = nullptr;
  cudaGraphExec_t         graph_pair[2] = { nullptr, nullptr };
  int64_t                 launched = 0;
  // persistent form: work lists of the six box stages, barrier state,
  // cooperative grid size, wait bound, and the form run() uses
  PersistRef *  plist[6] = {};
  unsigned      pn[6] = {};
  PersistSync * psync = nullptr;
  int           pgrid = 0;
  long long     pbudget = 1LL << 34; // about 8 s at 2 GHz per barrier wait
  int           run_mode = MHD_ENSEMBLE_GRAPHS;

  ~EnsembleImpl() override
  {
    drop_graphs();
    snapshot_free();
    for (auto & m : map)
      if (m)
        cudaFree(m);
    for (auto & m : plist)
      if (m)
        cudaFree(m);
    if (psync)
      cudaFree(psync);
    if (dG)
      cudaFree(dG);
    if (dB)
      cudaFree(dB);
    if (arena)
      cudaFree(arena);
    if (st)
      cudaFree(st);
    if (st_host)
      cudaFreeHost(st_host);
    if (stream)
      cudaStreamDestroy(stream);
  }

  void
  drop_graphs()
  {
    for (auto & g : graph_pair)
      if (g)
      {
        cudaGraphExecDestroy(g);
        g = nullptr;
      }
  }

  int
  real_bytes() const override
  {
    return (int)sizeof(R);
  }

  int
  bind_device() override
  {
    MHD_ECK(cudaSetDevice(P[0].device));
    return MHD_OK;
  }

  static int64_t
  box_count(const Grid<R> & g, Kind k)
  {
    switch (k)
    {
    case K_BC:
      return g.dim == 3 ? ghost_count<R, 3>(g) : ghost_count<R, 2>(g);
    case K_PRIM:
      return g.box[BOX_PRIM].count();
    case K_TRACE:
      return g.box[BOX_TRACE].count();
    case K_FLUX:
    case K_EMF:
      return g.box[BOX_FACE].count();
    case K_DT: // kDtCells cells per thread
      return (g.box[BOX_INTERIOR].count() + kDtCells - 1) / kDtCells;
    case K_FUSED: // tiles, one block of FusedTile::THREADS (= threads[K_FUSED]) each
      return (int64_t)((g.nx + FusedTile::TX - 1) / FusedTile::TX) *
             ((g.ny + FusedTile::TY - 1) / FusedTile::TY) * FusedTile::THREADS;
    default:
      return g.box[BOX_INTERIOR].count();
    }
  }

  // the fused form exists for 2D ensembles (every problem is version 2)
  bool
  fused_ok() const
  {
    return dim == 2;
  }

  int
  build_map(Kind k)
  {
    std::vector<BlockRef> h;
    for (int p = 0; p < n; ++p)
    {
      const int64_t cnt = box_count(G[p], k);
      const int64_t nb = (cnt + threads[k] - 1) / threads[k];
      for (int64_t b = 0; b < nb; ++b)
        h.push_back(BlockRef{ p, (int)b });
    }
    if (map[k])
      MHD_ECK(cudaFree(map[k]));
    MHD_ECK(cudaMalloc(&map[k], h.size() * sizeof(BlockRef)));
    MHD_ECK(cudaMemcpy(map[k], h.data(), h.size() * sizeof(BlockRef), cudaMemcpyHostToDevice));
    nblk[k] = (unsigned)h.size();
    return MHD_OK;
  }

  int
  setup(const mhd_params * params, int nprob)
  {
    n = nprob;
    dim = params[0].dim;
    P.assign(params, params + nprob);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    {
      err = "no CUDA device available";
      return MHD_ERR_NO_DEVICE;
    }
    MHD_ECK(cudaSetDevice(params[0].device));
    MHD_ECK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    // one arena: per problem U, U2, Q, Q2, S (dim x 8), E, F (dim x nf), Em, H
    // and, in FP32, the low parts of the state (Buffers::Ulo, 8 planes)
    const int          ne = dim == 3 ? 3 : 1, nf = dim == 3 ? 5 : 6, nh = face_data_planes(dim);
    const int          nlo = sizeof(R) == 4 ? 8 : 0;
    const int          planes = 8 * 4 + 8 * dim + ne + nf * dim + ne + nh + nlo;
    std::vector<size_t> off(n);
    size_t              total = 0;
    G.resize(n);
    for (int p = 0; p < n; ++p)
    {
      G[p] = make_grid<R>(P[p]);
      off[p] = total;
      const size_t cells = (size_t)G[p].sv;
      total += ((cells * planes + 63) / 64) * 64; // 256-byte aligned problems (FP32)
    }
    // (256 bytes of padding: the fused form's optional bulk copies of a
    // problem's last rows, MFUSED_BULK_STAGING, may run past its last value)
    MHD_ECK(cudaMalloc(&arena, total * sizeof(R) + 256));
    MHD_ECK(cudaMemsetAsync(arena, 0, total * sizeof(R), stream));
    MHD_ECK(cudaMalloc(&st, n * sizeof(DevState)));
    MHD_ECK(cudaMallocHost(&st_host, n * sizeof(DevState)));
    B.resize(n);
    for (int p = 0; p < n; ++p)
    {
      R *          a = arena + off[p];
      const size_t c = (size_t)G[p].sv;
      B[p].Uin = a;
      a += 8 * c;
      B[p].Uout = a;
      a += 8 * c;
      B[p].Q = a;
      a += 8 * c;
      B[p].Q2 = a;
      a += 8 * c;
      B[p].S = a;
      a += 8 * dim * c;
      B[p].E = a;
      a += ne * c;
      B[p].F = a;
      a += nf * dim * c;
      B[p].Em = a;
      a += ne * c;
      B[p].H = a;
      a += nh * c;
      B[p].Ulo = nlo ? a : nullptr;
      B[p].st = st + p;
    }
    MHD_ECK(cudaMalloc(&dG, n * sizeof(Grid<R>)));
    MHD_ECK(cudaMalloc(&dB, n * sizeof(Buffers<R>)));
    MHD_ECK(cudaMemcpy(dG, G.data(), n * sizeof(Grid<R>), cudaMemcpyHostToDevice));
    MHD_ECK(cudaMemcpy(dB, B.data(), n * sizeof(Buffers<R>), cudaMemcpyHostToDevice));
    for (int p = 0; p < n; ++p)
      reset_record(p);
    MHD_ECK(cudaMemcpyAsync(st, st_host, n * sizeof(DevState), cudaMemcpyHostToDevice, stream));
    for (int k = 0; k < K_COUNT; ++k)
      if ((k != K_DT && k != K_FUSED) || fused_ok())
        if (int rc = build_map((Kind)k))
          return rc;
    if (fused_ok())
    {
      fused_rs = RIEMANN_HLLD;
      for (int p = 0; p < n; ++p)
        if (G[p].riemann != RIEMANN_HLLD)
          fused_rs = 0;
      MHD_ECK(cudaFuncSetAttribute(kb_mfused2d<R, kFusedTY, RIEMANN_HLLD>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)FusedTile::SMEM));
      MHD_ECK(cudaFuncSetAttribute(kb_mfused2d<R, kFusedTY, 0>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)FusedTile::SMEM));
      // the default form of a 2D FP32 ensemble is the fused one (the single
      // problem's rule); mhd_ensemble_set_mode / _autotune change it
      if (sizeof(R) == 4)
        run_mode = MHD_ENSEMBLE_FUSED;
    }
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  void
  reset_record(int p)
  {
    DevState h{};
    h.t = P[p].tCurrent;
    h.tEnd = P[p].tEnd;
    h.nStepmax = P[p].nStepmax;
    st_host[p] = h;
  }

  void
  launch_kind(Kind k, int parity)
  {
    const unsigned nb = nblk[k];
    const int      th = threads[k];
    if (dim == 2)
    {
      switch (k)
      {
      case K_BC:
        kb_boundaries<R, 2><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_PRIM:
        kb_prim_dt<R, 2><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_TRACE:
        kb_trace<R, 2><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_FLUX:
        kb_flux<R, 2><<<dim3(nb, 2), th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_EMF:
        kb_emf<R, 2><<<dim3(nb, 1), th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_DT:
        kb_dt_only<R, 2><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_FUSED:
        if (fused_rs == RIEMANN_HLLD)
          kb_mfused2d<R, kFusedTY, RIEMANN_HLLD>
            <<<nb, FusedTile::THREADS, FusedTile::SMEM, stream>>>(dG, dB, map[k], parity);
        else
          kb_mfused2d<R, kFusedTY, 0>
            <<<nb, FusedTile::THREADS, FusedTile::SMEM, stream>>>(dG, dB, map[k], parity);
        break;
      default:
        kb_update<R, 2><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
      }
    }
    else
    {
      switch (k)
      {
      case K_BC:
        kb_boundaries<R, 3><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_PRIM:
        kb_prim_dt<R, 3><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_TRACE:
        kb_trace<R, 3><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_FLUX:
        kb_flux<R, 3><<<dim3(nb, 3), th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      case K_EMF:
        kb_emf<R, 3><<<dim3(nb, 3), th, 0, stream>>>(dG, dB, map[k], parity);
        break;
      default:
        kb_update<R, 3><<<nb, th, 0, stream>>>(dG, dB, map[k], parity);
      }
    }
  }

  void
  enqueue_step(int parity)
  {
    if (run_mode == MHD_ENSEMBLE_FUSED)
    {
      launch_kind(K_BC, parity);
      launch_kind(K_DT, parity);
      kb_finalize_dt<R><<<(n + 127) / 128, 128, 0, stream>>>(dG, dB, n);
      launch_kind(K_FUSED, parity);
      kb_advance<R><<<(n + 127) / 128, 128, 0, stream>>>(dB, n);
      return;
    }
    launch_kind(K_BC, parity);
    launch_kind(K_PRIM, parity);
    kb_finalize_dt<R><<<(n + 127) / 128, 128, 0, stream>>>(dG, dB, n);
    launch_kind(K_TRACE, parity);
    launch_kind(K_FLUX, parity);
    launch_kind(K_EMF, parity);
    launch_kind(K_UPDATE, parity);
    kb_advance<R><<<(n + 127) / 128, 128, 0, stream>>>(dB, n);
  }

  int
  launches_per_step() const override
  {
    return run_mode == MHD_ENSEMBLE_FUSED ? 5 : 8;
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
    if (graph_pair[0])
      return MHD_OK;
    for (int parity = 0; parity < 2; ++parity)
    {
      cudaGraph_t g = nullptr;
      MHD_ECK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
      enqueue_step(parity);
      enqueue_step(1 - parity);
      cudaError_t le = cudaGetLastError();
      cudaError_t ce = cudaStreamEndCapture(stream, &g);
      if (le != cudaSuccess || ce != cudaSuccess)
      {
        err = std::string("graph capture: ") + cudaGetErrorString(le != cudaSuccess ? le : ce);
        if (g)
          cudaGraphDestroy(g);
        return MHD_ERR_CUDA;
      }
      cudaError_t ie = cudaGraphInstantiate(&graph_pair[parity], g, 0);
      cudaGraphDestroy(g);
      if (ie != cudaSuccess)
      {
        err = std::string("graph instantiate: ") + cudaGetErrorString(ie);
        return MHD_ERR_CUDA;
      }
      // upload now so that the first replay does not pay for it
      MHD_ECK(cudaGraphUpload(graph_pair[parity], stream));
    }
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // Per problem: boundaries + U2 = U + primitives + dt (SolverMHDMuscl.h:393-402)
  int
  apply_init(int p)
  {
    const Grid<R> & g = G[p];
    // a state from the host has zero low parts
    if (B[p].Ulo)
      MHD_ECK(cudaMemsetAsync(B[p].Ulo, 0, (size_t)g.sv * NV * sizeof(R), stream));
    const int64_t   nall = dim == 3 ? ghost_count<R, 3>(g) : ghost_count<R, 2>(g),
                    nprim = g.box[BOX_PRIM].count();
    if (dim == 2)
    {
      k_boundaries<R, 2><<<(unsigned)((nall + 255) / 256), 256, 0, stream>>>(g, B[p].Uin, B[p].st, 1);
      k_prim_dt<R, 2><<<(unsigned)((nprim + 255) / 256), 256, 0, stream>>>(g, B[p].Uin, B[p].Q,
                                                                             B[p].st, 1);
    }
    else
    {
      k_boundaries<R, 3><<<(unsigned)((nall + 255) / 256), 256, 0, stream>>>(g, B[p].Uin, B[p].st, 1);
      k_prim_dt<R, 3><<<(unsigned)((nprim + 255) / 256), 256, 0, stream>>>(g, B[p].Uin, B[p].Q,
                                                                             B[p].st, 1);
    }
    k_finalize_dt<R><<<1, 1, 0, stream>>>(g, B[p].st, 1);
    MHD_ECK(cudaMemcpyAsync(B[p].Uout, B[p].Uin, (size_t)g.sv * NV * sizeof(R),
                            cudaMemcpyDeviceToDevice, stream));
    return check_launch();
  }

  int
  check_problem(int p)
  {
    if (p < 0 || p >= n)
    {
      err = "problem index out of range";
      return MHD_ERR_INVALID_ARG;
    }
    return MHD_OK;
  }

  static unsigned
  blocks_for(int64_t cnt, int th)
  {
    return (unsigned)((cnt + th - 1) / th);
  }

  // Host array -> device state of problem p; LayoutRight goes through the
  // problem's primitive array as staging (rewritten by the next iteration).
  int
  upload(int p, const void * host, int layout)
  {
    const size_t bytes = (size_t)G[p].sv * NV * sizeof(R);
    if (layout == MHD_LAYOUT_LEFT)
    {
      MHD_ECK(cudaMemcpyAsync(B[p].Uin, host, bytes, cudaMemcpyHostToDevice, stream));
      return MHD_OK;
    }
    MHD_ECK(cudaMemcpyAsync(B[p].Q, host, bytes, cudaMemcpyHostToDevice, stream));
    k_transpose<R><<<blocks_for(G[p].sv * NV, 256), 256, 0, stream>>>(G[p], B[p].Q, B[p].Uin, 0);
    return check_launch();
  }

  int
  download(int p, const R * src, void * host, int layout)
  {
    const size_t bytes = (size_t)G[p].sv * NV * sizeof(R);
    if (layout == MHD_LAYOUT_LEFT)
    {
      MHD_ECK(cudaMemcpyAsync(host, src, bytes, cudaMemcpyDeviceToHost, stream));
      return MHD_OK;
    }
    k_transpose<R><<<blocks_for(G[p].sv * NV, 256), 256, 0, stream>>>(G[p], src, B[p].Q, 1);
    if (int rc = check_launch())
      return rc;
    MHD_ECK(cudaMemcpyAsync(host, B[p].Q, bytes, cudaMemcpyDeviceToHost, stream));
    return MHD_OK;
  }

  int
  set_state(int p, const void * U, int layout) override
  {
    if (int rc = check_problem(p))
      return rc;
    if (int rc = upload(p, U, layout))
      return rc;
    reset_record(p);
    MHD_ECK(cudaMemcpyAsync(st + p, st_host + p, sizeof(DevState), cudaMemcpyHostToDevice, stream));
    if (int rc = apply_init(p))
      return rc;
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // Every problem's state in one call: uploads, record resets and the
  // per-problem initialisation are queued together and the stream is
  // synchronised once (set_state synchronises per problem).
  int
  set_states(const void * const * U, int layout) override
  {
    for (int p = 0; p < n; ++p)
    {
      if (int rc = upload(p, U[p], layout))
        return rc;
      reset_record(p);
    }
    MHD_ECK(cudaMemcpyAsync(st, st_host, (size_t)n * sizeof(DevState), cudaMemcpyHostToDevice,
                            stream));
    for (int p = 0; p < n; ++p)
      if (int rc = apply_init(p))
        return rc;
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  init_problem(int p) override
  {
    if (int rc = check_problem(p))
      return rc;
    std::vector<double> h((size_t)G[p].sv * NV);
    init_problem_host(P[p], h.data());
    if constexpr (sizeof(R) == 8)
      return set_state(p, h.data(), MHD_LAYOUT_LEFT);
    std::vector<float> f(h.size());
    for (size_t q = 0; q < h.size(); ++q)
      f[q] = (float)h[q];
    return set_state(p, f.data(), MHD_LAYOUT_LEFT);
  }

  int
  read_records()
  {
    MHD_ECK(cudaMemcpyAsync(st_host, st, n * sizeof(DevState), cudaMemcpyDeviceToHost, stream));
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // The array the next iteration of problem p reads (SolverMHDMuscl.h:791-805).
  R *
  current(int p) const
  {
    return (st_host[p].it % 2 == 0) ? B[p].Uin : B[p].Uout;
  }

  int
  get_state(int p, void * U, int layout) override
  {
    if (int rc = check_problem(p))
      return rc;
    if (int rc = read_records())
      return rc;
    R *             cur = current(p);
    const Grid<R> & g = G[p];
    const int64_t   nall = dim == 3 ? ghost_count<R, 3>(g) : ghost_count<R, 2>(g);
    // ghost refresh from the interior: the next iteration starts with the same fill
    if (dim == 2)
      k_boundaries<R, 2><<<blocks_for(nall, 256), 256, 0, stream>>>(g, cur, B[p].st, 1);
    else
      k_boundaries<R, 3><<<blocks_for(nall, 256), 256, 0, stream>>>(g, cur, B[p].st, 1);
    if (int rc = check_launch())
      return rc;
    if (int rc = download(p, cur, U, layout))
      return rc;
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // Every problem's state in one call (one record read, one synchronisation).
  int
  get_states(void * const * U, int layout) override
  {
    if (int rc = read_records())
      return rc;
    for (int p = 0; p < n; ++p)
    {
      R *             cur = current(p);
      const Grid<R> & g = G[p];
      const int64_t   nall = dim == 3 ? ghost_count<R, 3>(g) : ghost_count<R, 2>(g);
      if (dim == 2)
        k_boundaries<R, 2><<<blocks_for(nall, 256), 256, 0, stream>>>(g, cur, B[p].st, 1);
      else
        k_boundaries<R, 3><<<blocks_for(nall, 256), 256, 0, stream>>>(g, cur, B[p].st, 1);
      if (int rc = check_launch())
        return rc;
      if (int rc = download(p, cur, U[p], layout))
        return rc;
    }
    MHD_ECK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // FP64 conserved totals and div B of problem p on the GPU (the conventions
  // of the single-problem diagnostics: plain sums over interior cells, mean
  // and max |div B|); the problem's
  // slope array is the scratch for the block partials (rewritten by the
  // next iteration).
  int
  diagnostics(int p, double sums[8], double * divb_l1, double * divb_max) override
  {
    if (int rc = check_problem(p))
      return rc;
    if (int rc = read_records())
      return rc;
    const Grid<R> & g = G[p];
    const unsigned  nb = std::min(1024u, blocks_for(g.box[BOX_INTERIOR].count(), 256));
    double *        partial = reinterpret_cast<double *>(B[p].S);
    double *        out = partial + (size_t)nb * 10;
    const int64_t   nall = dim == 3 ? ghost_count<R, 3>(g) : ghost_count<R, 2>(g);
    if (dim == 2)
    {
      k_boundaries<R, 2><<<blocks_for(nall, 256), 256, 0, stream>>>(g, current(p), B[p].st, 1);
      k_diag<R, 2><<<nb, 256, 0, stream>>>(g, current(p), partial);
    }
    else
    {
      k_boundaries<R, 3><<<blocks_for(nall, 256), 256, 0, stream>>>(g, current(p), B[p].st, 1);
      k_diag<R, 3><<<nb, 256, 0, stream>>>(g, current(p), partial);
    }
    k_diag_final<<<1, 32, 0, stream>>>(partial, (int)nb, out);
    if (int rc = check_launch())
      return rc;
    double h[10];
    MHD_ECK(cudaMemcpyAsync(h, out, sizeof h, cudaMemcpyDeviceToHost, stream));
    MHD_ECK(cudaStreamSynchronize(stream));
    for (int v = 0; v < 8; ++v)
      sums[v] = h[v];
    if (divb_l1)
      *divb_l1 = h[8] / (double)g.box[BOX_INTERIOR].count();
    if (divb_max)
      *divb_max = h[9];
    return MHD_OK;
  }

  int
  time(int p, double * t, double * dt, int * it) override
  {
    if (int rc = check_problem(p))
      return rc;
    if (int rc = read_records())
      return rc;
    if (t)
      *t = st_host[p].t;
    if (dt)
      *dt = st_host[p].dt;
    if (it)
      *it = st_host[p].it;
    return MHD_OK;
  }

  // All problems start from iteration 0 together; a problem that finishes
  // early keeps its state while the others go on.
  int
  run(int nsteps, float * ms) override
  {
    if (int rc = build_graphs())
      return rc;
    if (int rc = read_records())
      return rc;
    int parity = 0;
    for (int p = 0; p < n; ++p)
      if (st_host[p].it % 2 != st_host[0].it % 2)
      {
        err = "problems are at iterations of different parity; set their states again";
        return MHD_ERR_INVALID_ARG;
      }
    parity = st_host[0].it % 2;
    cudaEvent_t e0, e1;
    MHD_ECK(cudaEventCreate(&e0));
    MHD_ECK(cudaEventCreate(&e1));
    MHD_ECK(cudaEventRecord(e0, stream));
    if (run_mode == MHD_ENSEMBLE_PERSISTENT)
    {
      if (int rc = build_persist())
        return rc;
      if (int rc = enqueue_persistent(parity, nsteps))
        return rc;
    }
    else
    {
      int left = nsteps;
      while (left >= 2)
      {
        MHD_ECK(cudaGraphLaunch(graph_pair[parity], stream));
        left -= 2;
      }
      if (left)
      {
        enqueue_step(parity);
        if (int rc = check_launch())
          return rc;
      }
    }
    MHD_ECK(cudaEventRecord(e1, stream));
    MHD_ECK(cudaEventSynchronize(e1));
    float el = 0.f;
    MHD_ECK(cudaEventElapsedTime(&el, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ms)
      *ms = el;
    if (run_mode == MHD_ENSEMBLE_PERSISTENT && nsteps > 0)
      if (int rc = persistent_status())
        return rc;
    if (int rc = read_records())
      return rc;
    for (int p = 0; p < n; ++p)
      if (st_host[p].status & STATUS_STAGING)
      {
        err = "problem " + std::to_string(p) +
              ": a tile's bulk copies into shared memory did not complete within the wait bound";
        return MHD_ERR_CUDA;
      }
    for (int p = 0; p < n; ++p)
      if (st_host[p].status & STATUS_NUMERIC)
      {
        err = "problem " + std::to_string(p) + ": non-finite or non-positive state detected";
        return MHD_ERR_NUMERIC;
      }
    return MHD_OK;
  }

  int
  set_mode(int m) override
  {
    if (m != MHD_ENSEMBLE_GRAPHS && m != MHD_ENSEMBLE_PERSISTENT && m != MHD_ENSEMBLE_FUSED)
    {
      err = "mode must be MHD_ENSEMBLE_GRAPHS, MHD_ENSEMBLE_PERSISTENT or MHD_ENSEMBLE_FUSED";
      return MHD_ERR_INVALID_ARG;
    }
    if (m == MHD_ENSEMBLE_FUSED && !fused_ok())
    {
      err = "the fused ensemble form is built for 2D ensembles";
      return MHD_ERR_INVALID_ARG;
    }
    if (m == MHD_ENSEMBLE_PERSISTENT)
      if (int rc = build_persist())
        return rc;
    if (m != run_mode)
    {
      MHD_ECK(cudaStreamSynchronize(stream));
      drop_graphs(); // the graphs hold the form's launches
    }
    run_mode = m;
    return MHD_OK;
  }

  int
  mode() const override
  {
    return run_mode;
  }

  int
  set_wait_limit(long long cycles) override
  {
    if (cycles < 0)
    {
      err = "wait limit must be non-negative";
      return MHD_ERR_INVALID_ARG;
    }
    pbudget = cycles;
    return MHD_OK;
  }

  // Work lists of the persistent kernel (blocks of kPersistThreads threads;
  // the face and edge stages direction-major) and its cooperative grid:
  // as many blocks as are resident on the device at once.
  int
  build_persist()
  {
    if (psync)
      return MHD_OK;
    const Kind kinds[6] = { K_BC, K_PRIM, K_TRACE, K_FLUX, K_EMF, K_UPDATE };
    for (int q = 0; q < 6; ++q)
    {
      std::vector<PersistRef> h;
      const int nd = kinds[q] == K_FLUX ? dim : (kinds[q] == K_EMF ? (dim == 3 ? 3 : 1) : 1);
      for (int d = 0; d < nd; ++d)
        for (int p = 0; p < n; ++p)
        {
          const int64_t nb = (box_count(G[p], kinds[q]) + kPersistThreads - 1) / kPersistThreads;
          for (int64_t b = 0; b < nb; ++b)
            h.push_back(PersistRef{ p, (int)b, d });
        }
      MHD_ECK(cudaMalloc(&plist[q], std::max<size_t>(1, h.size()) * sizeof(PersistRef)));
      if (!h.empty())
        MHD_ECK(cudaMemcpy(plist[q], h.data(), h.size() * sizeof(PersistRef),
                           cudaMemcpyHostToDevice));
      pn[q] = (unsigned)h.size();
    }
    int dev = 0, sms = 0, coop = 0, bps = 0;
    MHD_ECK(cudaGetDevice(&dev));
    MHD_ECK(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    MHD_ECK(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop)
    {
      err = "the device does not support cooperative launches (persistent ensemble form)";
      return MHD_ERR_CUDA;
    }
    MHD_ECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, persist_kernel(), kPersistThreads, 0));
    pgrid = bps * sms;
    if (pgrid <= 0)
    {
      err = "persistent ensemble kernel cannot be resident";
      return MHD_ERR_CUDA;
    }
    MHD_ECK(cudaMalloc(&psync, sizeof(PersistSync)));
    return MHD_OK;
  }

  const void *
  persist_kernel() const
  {
    return dim == 2 ? (const void *)kp_run<R, 2> : (const void *)kp_run<R, 3>;
  }

  // nsteps iterations in one cooperative launch (queued on the stream)
  int
  enqueue_persistent(int parity, int nsteps)
  {
    if (nsteps <= 0)
      return MHD_OK;
    MHD_ECK(cudaMemsetAsync(psync, 0, sizeof(PersistSync), stream));
    PersistWork W;
    for (int q = 0; q < 6; ++q)
    {
      W.list[q] = plist[q];
      W.n[q] = pn[q];
    }
    const Grid<R> *    gs = dG;
    const Buffers<R> * bs = dB;
    int                np = n, par = parity, ni = nsteps;
    long long          bud = pbudget;
    void *             args[] = { &gs, &bs, &W, &np, &par, &ni, &psync, &bud };
    MHD_ECK(cudaLaunchCooperativeKernel(persist_kernel(), dim3(pgrid), dim3(kPersistThreads), args,
                                        0, stream));
    return MHD_OK;
  }

  int
  persistent_status()
  {
    PersistSync h{};
    MHD_ECK(cudaMemcpyAsync(&h, psync, sizeof h, cudaMemcpyDeviceToHost, stream));
    MHD_ECK(cudaStreamSynchronize(stream));
    if (h.status)
    {
      err = "persistent ensemble: a grid-barrier wait gave up after " + std::to_string(pbudget) +
            " clock cycles (the states of this run are incomplete)";
      return MHD_ERR_CUDA;
    }
    return MHD_OK;
  }

  // Snapshot of every problem's two state arrays, FP32 low parts and
  // record, for the autotuner's trials.
  R *                 snap = nullptr;
  DevState *          st_snap = nullptr;
  std::vector<size_t> snap_off;

  int
  snapshot(bool back)
  {
    const int nplanes = 8 * (sizeof(R) == 4 ? 3 : 2);
    if (!snap)
    {
      snap_off.assign(n + 1, 0);
      for (int p = 0; p < n; ++p)
        snap_off[p + 1] = snap_off[p] + (size_t)G[p].sv * nplanes;
      MHD_ECK(cudaMalloc(&snap, snap_off[n] * sizeof(R)));
      MHD_ECK(cudaMalloc(&st_snap, n * sizeof(DevState)));
    }
    for (int p = 0; p < n; ++p)
    {
      const size_t c = (size_t)G[p].sv * 8 * sizeof(R);
      R *          bufs[3] = { B[p].Uin, B[p].Uout, B[p].Ulo };
      for (int q = 0; q < nplanes / 8; ++q)
      {
        R * s0 = snap + snap_off[p] + (size_t)q * 8 * G[p].sv;
        MHD_ECK(cudaMemcpyAsync(back ? bufs[q] : s0, back ? s0 : bufs[q], c,
                                cudaMemcpyDeviceToDevice, stream));
      }
    }
    MHD_ECK(cudaMemcpyAsync(back ? st : st_snap, back ? st_snap : st, n * sizeof(DevState),
                            cudaMemcpyDeviceToDevice, stream));
    return MHD_OK;
  }

  void
  snapshot_free()
  {
    cudaStreamSynchronize(stream);
    if (snap)
      cudaFree(snap);
    if (st_snap)
      cudaFree(st_snap);
    snap = nullptr;
    st_snap = nullptr;
  }

  // Time each launch kind with every candidate block size on the current
  // states, keep the fastest, rebuild the block maps; then the form.  The
  // trials rerun the update (which adds into the FP32 low parts) and advance
  // the states, so everything is taken from a snapshot made first and
  // restored at the end: results unchanged.
  int
  autotune(std::string & report) override
  {
    if (int rc = read_records())
      return rc;
    const int parity = st_host[0].it % 2;
    const int cand[3] = { 64, 128, 256 };
    cudaEvent_t e0, e1;
    MHD_ECK(cudaEventCreate(&e0));
    MHD_ECK(cudaEventCreate(&e1));
    int rc = snapshot(false);
    char line[160];
    // primitives and dt are needed by the kernels downstream of them
    launch_kind(K_BC, parity);
    launch_kind(K_PRIM, parity);
    kb_finalize_dt<R><<<(n + 127) / 128, 128, 0, stream>>>(dG, dB, n);
    for (int k = 0; k < K_COUNT && rc == MHD_OK; ++k)
    {
      if (k == K_FUSED || (k == K_DT && !fused_ok()))
        continue; // the tile kernel's shape is fixed
      float best = 1e30f;
      int   best_t = threads[k];
      for (int c : cand)
      {
        threads[k] = c;
        if ((rc = build_map((Kind)k)) != MHD_OK)
          break;
        launch_kind((Kind)k, parity); // warm
        MHD_ECK(cudaEventRecord(e0, stream));
        for (int r = 0; r < 3; ++r)
          launch_kind((Kind)k, parity);
        MHD_ECK(cudaEventRecord(e1, stream));
        MHD_ECK(cudaEventSynchronize(e1));
        float el = 0.f;
        MHD_ECK(cudaEventElapsedTime(&el, e0, e1));
        if ((rc = check_launch()) != MHD_OK)
          break;
        std::snprintf(line, sizeof line, "%s threads=%d: %.3f ms\n", kKindName[k], c, el / 3);
        report += line;
        if (el < best)
        {
          best = el;
          best_t = c;
        }
      }
      threads[k] = best_t;
      if (rc == MHD_OK)
        rc = build_map((Kind)k);
      std::snprintf(line, sizeof line, "-> %s uses %d threads per block\n", kKindName[k], best_t);
      report += line;
    }
    // the form: per-stage launches replayed from graphs, one persistent
    // launch with grid-wide barriers, or (2D) the fused tile form replayed
    // from graphs; two iterations of each from the snapshot
    if (rc == MHD_OK)
      rc = tune_mode(parity, e0, e1, report);
    if (rc == MHD_OK)
      rc = snapshot(true);
    snapshot_free();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != MHD_OK && err.empty())
      err = "ensemble autotune failed";
    return rc;
  }

  int
  tune_mode(int parity, cudaEvent_t e0, cudaEvent_t e1, std::string & report)
  {
    const int modes[3] = { MHD_ENSEMBLE_GRAPHS, MHD_ENSEMBLE_PERSISTENT, MHD_ENSEMBLE_FUSED };
    const int nmodes = fused_ok() ? 3 : 2;
    float     t[3] = { 0.f, 0.f, 0.f };
    int       rc = build_persist();
    for (int q = 0; q < nmodes && rc == MHD_OK; ++q)
    {
      run_mode = modes[q];
      drop_graphs();
      if (run_mode != MHD_ENSEMBLE_PERSISTENT && (rc = build_graphs()) != MHD_OK)
        break;
      for (int rep = 0; rep < 2 && rc == MHD_OK; ++rep) // warm, then timed
      {
        if ((rc = snapshot(true)) != MHD_OK)
          break;
        if (cudaEventRecord(e0, stream) != cudaSuccess)
          rc = MHD_ERR_CUDA;
        if (run_mode != MHD_ENSEMBLE_PERSISTENT)
        {
          if (rc == MHD_OK && cudaGraphLaunch(graph_pair[parity], stream) != cudaSuccess)
            rc = MHD_ERR_CUDA;
        }
        else if (rc == MHD_OK)
          rc = enqueue_persistent(parity, 2);
        if (cudaEventRecord(e1, stream) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess)
          rc = MHD_ERR_CUDA;
        if (rc == MHD_OK && run_mode == MHD_ENSEMBLE_PERSISTENT)
          rc = persistent_status();
        if (rc == MHD_OK)
          cudaEventElapsedTime(&t[q], e0, e1);
      }
    }
    drop_graphs();
    if (rc != MHD_OK)
    {
      run_mode = MHD_ENSEMBLE_GRAPHS;
      return rc;
    }
    char line[240];
    std::snprintf(line, sizeof line,
                  "form graphs: %.3f ms per iteration; persistent (%d blocks x %d threads): %.3f ms "
                  "per iteration",
                  t[0] / 2, pgrid, kPersistThreads, t[1] / 2);
    report += line;
    int best = 0;
    for (int q = 1; q < nmodes; ++q)
      if (t[q] < t[best])
        best = q;
    if (nmodes == 3)
    {
      std::snprintf(line, sizeof line, "; fused tiles: %.3f ms per iteration", t[2] / 2);
      report += line;
    }
    run_mode = modes[best];
    report += run_mode == MHD_ENSEMBLE_PERSISTENT ? "\n-> form persistent\n"
              : run_mode == MHD_ENSEMBLE_FUSED    ? "\n-> form fused\n"
                                                  : "\n-> form graphs\n";
    return MHD_OK;
  }

  // Time each launch of one iteration separately (CUDA events around each
  // launch on the ensemble's stream); the iteration is a real one.
  int
  profile_step(const char ** names, float * ms, int max, int * count) override
  {
    if (int rc = read_records())
      return rc;
    const int   parity = st_host[0].it % 2;
    cudaEvent_t ev[9];
    for (auto & e : ev)
      MHD_ECK(cudaEventCreate(&e));
    static const char * kNames[8] = { "kb_boundaries", "kb_prim_dt", "kb_finalize_dt", "kb_trace",
                                      "kb_flux",       "kb_emf",     "kb_update",      "kb_advance" };
    if (run_mode == MHD_ENSEMBLE_FUSED)
    {
      static const char * kf[5] = { "kb_boundaries", "kb_dt_only", "kb_finalize_dt",
                                    "kb_mfused2d", "kb_advance" };
      MHD_ECK(cudaEventRecord(ev[0], stream));
      launch_kind(K_BC, parity);
      MHD_ECK(cudaEventRecord(ev[1], stream));
      launch_kind(K_DT, parity);
      MHD_ECK(cudaEventRecord(ev[2], stream));
      kb_finalize_dt<R><<<(n + 127) / 128, 128, 0, stream>>>(dG, dB, n);
      MHD_ECK(cudaEventRecord(ev[3], stream));
      launch_kind(K_FUSED, parity);
      MHD_ECK(cudaEventRecord(ev[4], stream));
      kb_advance<R><<<(n + 127) / 128, 128, 0, stream>>>(dB, n);
      MHD_ECK(cudaEventRecord(ev[5], stream));
      if (int rc = check_launch())
        return rc;
      MHD_ECK(cudaEventSynchronize(ev[5]));
      for (int q = 0; q < 5 && q < max; ++q)
      {
        MHD_ECK(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
        if (names)
          names[q] = kf[q];
      }
      for (auto & e : ev)
        cudaEventDestroy(e);
      if (count)
        *count = 5;
      return MHD_OK;
    }
    MHD_ECK(cudaEventRecord(ev[0], stream));
    launch_kind(K_BC, parity);
    MHD_ECK(cudaEventRecord(ev[1], stream));
    launch_kind(K_PRIM, parity);
    MHD_ECK(cudaEventRecord(ev[2], stream));
    kb_finalize_dt<R><<<(n + 127) / 128, 128, 0, stream>>>(dG, dB, n);
    MHD_ECK(cudaEventRecord(ev[3], stream));
    launch_kind(K_TRACE, parity);
    MHD_ECK(cudaEventRecord(ev[4], stream));
    launch_kind(K_FLUX, parity);
    MHD_ECK(cudaEventRecord(ev[5], stream));
    launch_kind(K_EMF, parity);
    MHD_ECK(cudaEventRecord(ev[6], stream));
    launch_kind(K_UPDATE, parity);
    MHD_ECK(cudaEventRecord(ev[7], stream));
    kb_advance<R><<<(n + 127) / 128, 128, 0, stream>>>(dB, n);
    MHD_ECK(cudaEventRecord(ev[8], stream));
    if (int rc = check_launch())
      return rc;
    MHD_ECK(cudaEventSynchronize(ev[8]));
    for (int q = 0; q < 8 && q < max; ++q)
    {
      MHD_ECK(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
      if (names)
        names[q] = kNames[q];
    }
    for (auto & e : ev)
      cudaEventDestroy(e);
    if (count)
      *count = 8;
    return MHD_OK;
  }

  int
  cells(int64_t * interior) override
  {
    int64_t s = 0;
    for (int p = 0; p < n; ++p)
      s += G[p].box[BOX_INTERIOR].count();
    *interior = s;
    return MHD_OK;
  }
};

#undef MHD_ECK

} // namespace MHD_VARIANT_TAG
} // namespace mhd
