// Solver core of the hydro-only MUSCL-Hancock scheme for one arithmetic
// variant: device buffers, one CUDA stream, the launch sequence of an
// iteration, CUDA-graph replay of whole runs and host<->device state
// transfer in either Kokkos layout.  Included by hydro_variant.cu, which
// fixes R and the inline namespace MHD_VARIANT_TAG.  It serves the same C ABI
// as the MHD core (mhd_ctx), selected by mhd_params::solver.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "mhd_core.h"
#include "hydro_kernels.cuh"

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{
namespace hydro
{

#define HY_CK(call)                                                                   \
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
class HydroImpl final : public SolverCore
{
public:
  mhd_params      P{};
  HGrid<R>        G{};
  int             dim = 2, nvar = 4;
  int64_t         ncell = 0;
  R *             U = nullptr;
  R *             U2 = nullptr;
  R *             Q = nullptr;
  R *             S = nullptr; // slopes (DIM blocks of NVAR planes), then trace sources (NVAR)
  R *             F = nullptr; // face fluxes * dt/dx, DIM blocks of NVAR planes
  R *             Gf = nullptr; // gravity field, DIM planes (gravity on only)
  double *        diag = nullptr;
  DevState *      st = nullptr;
  DevState *      st_host = nullptr;
  cudaStream_t    stream = nullptr;
  cudaGraphExec_t graph[2] = { nullptr, nullptr };
  cudaGraphExec_t graph_pair[2] = { nullptr, nullptr };
  int64_t         launched = 0;
  static constexpr int kLaunches = 7;      // stage form
  static constexpr int kFusedLaunches = 5; // fused form
  // the fused plain form (k_hdt + k_hfused, intermediates in shared memory)
  // or the stage kernels; the same state bit for bit in the FMA-free build,
  // round-off apart in the FMA builds.  The default is a fixed function of
  // the configuration (default_form), so a configuration always runs the
  // same kernels; mhd_set_fused fixes either form or has the next stepping
  // call time one iteration of each and keep the faster (tune_form).
  bool fused = false;
  bool tuned = true;
  std::string tune_report;

  ~HydroImpl() override
  {
    drop_graphs();
    R * bufs[] = { U, U2, Q, S, F, Gf };
    for (R * b : bufs)
      if (b)
        cudaFree(b);
    if (diag)
      cudaFree(diag);
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
    for (int q = 0; q < 2; ++q)
    {
      if (graph[q])
        cudaGraphExecDestroy(graph[q]);
      if (graph_pair[q])
        cudaGraphExecDestroy(graph_pair[q]);
      graph[q] = graph_pair[q] = nullptr;
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
    HY_CK(cudaSetDevice(P.device));
    return MHD_OK;
  }

  size_t
  state_bytes() const
  {
    return (size_t)ncell * nvar * sizeof(R);
  }

  // The allocations of SolverHydroMuscl<dim>::SolverHydroMuscl
  // (SolverHydroMuscl.h:177-326): U, U2, Q, slopes and fluxes.
  int
  setup(const mhd_params & p)
  {
    P = p;
    dim = p.dim;
    nvar = dim + 2;
    G = make_hgrid<R>(p);
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
    HY_CK(cudaSetDevice(p.device));
    HY_CK(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    const size_t n = (size_t)ncell;
    HY_CK(cudaMalloc(&U, n * nvar * sizeof(R)));
    HY_CK(cudaMalloc(&U2, n * nvar * sizeof(R)));
    HY_CK(cudaMalloc(&Q, n * nvar * sizeof(R)));
    HY_CK(cudaMalloc(&S, n * nvar * (dim + 1) * sizeof(R)));
    HY_CK(cudaMalloc(&F, n * nvar * dim * sizeof(R)));
    HY_CK(cudaMalloc(&diag, (kDiagBlocks * 10 + 16) * sizeof(double)));
    HY_CK(cudaMalloc(&st, sizeof(DevState)));
    HY_CK(cudaMallocHost(&st_host, sizeof(DevState)));
    R * b3[] = { U, U2, Q };
    for (R * b : b3)
      HY_CK(cudaMemsetAsync(b, 0, n * nvar * sizeof(R), stream));
    HY_CK(cudaMemsetAsync(S, 0, n * nvar * (dim + 1) * sizeof(R), stream));
    HY_CK(cudaMemsetAsync(F, 0, n * nvar * dim * sizeof(R), stream));
    if (p.gravity)
    {
      // the field the problem's initialisation writes (constant in time)
      std::vector<double> gh(n * dim, 0.0);
      init_hydro_gravity_host(P, gh.data());
      std::vector<R> gr(gh.begin(), gh.end());
      HY_CK(cudaMalloc(&Gf, n * dim * sizeof(R)));
      HY_CK(cudaMemcpy(Gf, gr.data(), n * dim * sizeof(R), cudaMemcpyHostToDevice));
      G.gf = Gf;
    }
    HY_CK(reset_time_state());
    fused = default_form();
    if (dim == 2)
      HY_CK(cudaFuncSetAttribute(k_hfused<R, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)HTile<R, 2>::SMEM));
    else
      HY_CK(cudaFuncSetAttribute(k_hfused<R, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)HTile<R, 3>::SMEM));
    HY_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  fused_form() const override
  {
    return fused ? 1 : 0;
  }

  // The form measured faster on GB300 for the configuration: fused for 2D
  // FP32 (2D KH 4096^2: 0.92 vs 1.01 ms), stages otherwise (the halo
  // recomputation costs more than the HBM traffic it saves in 3D and in
  // FP64).
  bool
  default_form() const
  {
    return dim == 2 && sizeof(R) == 4;
  }

  int
  set_fused(int on) override
  {
    if (on < MHD_FORM_STAGES || on > MHD_FORM_TIMED)
    {
      err = "form must be MHD_FORM_STAGES, MHD_FORM_FUSED or MHD_FORM_TIMED";
      return MHD_ERR_INVALID_ARG;
    }
    HY_CK(cudaStreamSynchronize(stream));
    drop_graphs();
    if (on == MHD_FORM_TIMED)
    {
      tuned = false; // timed by the next stepping call
      return MHD_OK;
    }
    fused = on == MHD_FORM_FUSED;
    tuned = true;
    return MHD_OK;
  }

  // Time one iteration of each form on a snapshot of the current state (the
  // array the next iteration reads and the time-step record), restore the
  // snapshot after each, keep the faster form.  Both forms produce the same
  // state, so the choice changes only the speed.
  int
  tune_form()
  {
    if (tuned)
      return MHD_OK;
    tuned = true;
    if (int rc = read_state())
      return rc;
    if (step_finished_host())
      return MHD_OK;
    const DevState saved = *st_host;
    const int      parity = (int)(saved.it & 1);
    R *            cur = parity ? U2 : U;
    R *            snap = nullptr;
    HY_CK(cudaMalloc(&snap, state_bytes()));
    cudaEvent_t e0, e1;
    HY_CK(cudaEventCreate(&e0));
    HY_CK(cudaEventCreate(&e1));
    float ms[2] = { 0.f, 0.f };
    HY_CK(cudaMemcpyAsync(snap, cur, state_bytes(), cudaMemcpyDeviceToDevice, stream));
    for (int pass = 0; pass < 3; ++pass) // a warm pass per form, then the timed ones
    {
      for (int f = 0; f < 2; ++f)
      {
        fused = f == 1;
        HY_CK(cudaMemcpyAsync(cur, snap, state_bytes(), cudaMemcpyDeviceToDevice, stream));
        *st_host = saved;
        HY_CK(cudaMemcpyAsync(st, st_host, sizeof(DevState), cudaMemcpyHostToDevice, stream));
        HY_CK(cudaEventRecord(e0, stream));
        enqueue_step(parity);
        HY_CK(cudaEventRecord(e1, stream));
        if (int rc = check_launch())
          return rc;
        HY_CK(cudaEventSynchronize(e1));
        float t = 0.f;
        HY_CK(cudaEventElapsedTime(&t, e0, e1));
        if (pass > 0)
          ms[f] += t;
      }
    }
    HY_CK(cudaMemcpyAsync(cur, snap, state_bytes(), cudaMemcpyDeviceToDevice, stream));
    *st_host = saved;
    HY_CK(cudaMemcpyAsync(st, st_host, sizeof(DevState), cudaMemcpyHostToDevice, stream));
    HY_CK(cudaStreamSynchronize(stream));
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

  static constexpr int kDiagBlocks = 1024;

  cudaError_t
  reset_time_state()
  {
    DevState h{};
    h.t = P.tCurrent;
    h.tEnd = P.tEnd;
    h.nStepmax = P.nStepmax;
    *st_host = h;
    launched = 0;
    return cudaMemcpyAsync(st, st_host, sizeof(DevState), cudaMemcpyHostToDevice, stream);
  }

  static unsigned
  nblocks(int64_t n, int t)
  {
    return (unsigned)((n + t - 1) / t);
  }

  // ---- launches of one iteration ----
  void
  launch_bound(R * arr, int force)
  {
    if (dim == 2)
      k_hbound<R, 2><<<nblocks(ghost_count<R, 2>(G), 256), 256, 0, stream>>>(G, arr, st, force);
    else
      k_hbound<R, 3><<<nblocks(ghost_count<R, 3>(G), 256), 256, 0, stream>>>(G, arr, st, force);
  }
  void
  launch_prim_dt(const R * arr, int force)
  {
    if (dim == 2)
      k_hprim_dt<R, 2><<<nblocks(ncell, 256), 256, 0, stream>>>(G, arr, Q, st, force);
    else
      k_hprim_dt<R, 3><<<nblocks(ncell, 256), 256, 0, stream>>>(G, arr, Q, st, force);
  }
  void
  launch_finalize(int force)
  {
    k_hfinalize<R><<<1, 1, 0, stream>>>(G, st, force);
  }
  void
  launch_slopes()
  {
    const int64_t n = G.box[BOX_TRACE].count();
    if (dim == 2)
      k_hslopes<R, 2><<<nblocks(n, 128), 128, 0, stream>>>(G, Q, S, st);
    else
      k_hslopes<R, 3><<<nblocks(n, 128), 128, 0, stream>>>(G, Q, S, st);
  }
  void
  launch_flux()
  {
    const int64_t n = G.box[BOX_FACE].count();
    if (dim == 2)
      k_hflux<R, 2><<<dim3(nblocks(n, 128), 2), 128, 0, stream>>>(G, Q, S, F, st);
    else
      k_hflux<R, 3><<<dim3(nblocks(n, 128), 3), 128, 0, stream>>>(G, Q, S, F, st);
  }
  void
  launch_update(const R * in, R * out)
  {
    if (dim == 2)
      k_hupdate<R, 2><<<nblocks(ncell, 256), 256, 0, stream>>>(G, in, out, F, st);
    else
      k_hupdate<R, 3><<<nblocks(ncell, 256), 256, 0, stream>>>(G, in, out, F, st);
  }

  void
  launch_dt(const R * in, R * out, int force)
  {
    const unsigned nr = nblocks(G.box[BOX_INTERIOR].count(), 256 * kHdtCells);
    if (dim == 2)
      k_hdt<R, 2><<<nr + nblocks(ghost_count<R, 2>(G), 256), 256, 0, stream>>>(G, in, out, st,
                                                                                force, nr);
    else
      k_hdt<R, 3><<<nr + nblocks(ghost_count<R, 3>(G), 256), 256, 0, stream>>>(G, in, out, st,
                                                                                force, nr);
  }
  void
  launch_fused(const R * in, R * out)
  {
    if (dim == 2)
    {
      using T = HTile<R, 2>;
      const dim3 grid((G.nx + T::TX - 1) / T::TX, (G.ny + T::TY - 1) / T::TY, 1);
      k_hfused<R, 2><<<grid, T::THREADS, T::SMEM, stream>>>(G, in, out, st);
    }
    else
    {
      using T = HTile<R, 3>;
      const dim3 grid((G.nx + T::TX - 1) / T::TX, (G.ny + T::TY - 1) / T::TY,
                      (G.nz + T::TZ - 1) / T::TZ);
      k_hfused<R, 3><<<grid, T::THREADS, T::SMEM, stream>>>(G, in, out, st);
    }
  }

  int
  step_kernel_names(const char ** names) const
  {
    static const char * nm[kLaunches] = { "k_hbound", "k_hprim_dt", "k_hfinalize", "k_hslopes",
                                          "k_hflux",  "k_hupdate",  "k_advance" };
    static const char * nf[kFusedLaunches] = { "k_hbound", "k_hdt", "k_hfinalize", "k_hfused",
                                               "k_advance" };
    const int n = fused ? kFusedLaunches : kLaunches;
    for (int q = 0; q < n; ++q)
      names[q] = fused ? nf[q] : nm[q];
    return n;
  }

  // launch q of one iteration reading `in` and writing `out`
  void
  launch_stage(int q, R * in, R * out)
  {
    if (fused)
    {
      switch (q)
      {
        case 0: return launch_bound(in, 0);
        case 1: return launch_dt(in, out, 0);
        case 2: return launch_finalize(0);
        case 3: return launch_fused(in, out);
        default: k_advance<R><<<1, 1, 0, stream>>>(st);
      }
      return;
    }
    switch (q)
    {
      case 0: return launch_bound(in, 0);
      case 1: return launch_prim_dt(in, 0);
      case 2: return launch_finalize(0);
      case 3: return launch_slopes();
      case 4: return launch_flux();
      case 5: return launch_update(in, out);
      default: k_advance<R><<<1, 1, 0, stream>>>(st);
    }
  }

  void
  enqueue_step(int parity)
  {
    R * in = parity ? U2 : U;
    R * out = parity ? U : U2;
    const int n = launches_per_step();
    for (int q = 0; q < n; ++q)
      launch_stage(q, in, out);
  }

  int
  launches_per_step() override
  {
    return fused ? kFusedLaunches : kLaunches;
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
      for (int pair = 0; pair < 2; ++pair)
      {
        cudaGraph_t g = nullptr;
        HY_CK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        enqueue_step(parity);
        if (pair)
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
        cudaGraphExec_t ex = nullptr;
        cudaError_t     ie = cudaGraphInstantiate(&ex, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess)
        {
          err = std::string("graph instantiate: ") + cudaGetErrorString(ie);
          return MHD_ERR_CUDA;
        }
        (pair ? graph_pair : graph)[parity] = ex;
        HY_CK(cudaGraphUpload(ex, stream));
      }
    HY_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  // boundaries + U2 = U + dt: the tail of the constructor
  // (SolverHydroMuscl.h:300-312)
  int
  apply_init()
  {
    launch_bound(U, 1);
    HY_CK(cudaMemcpyAsync(U2, U, state_bytes(), cudaMemcpyDeviceToDevice, stream));
    launch_prim_dt(U, 1);
    launch_finalize(1);
    if (int rc = check_launch())
      return rc;
    HY_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  upload(const void * host, R * dst, int layout)
  {
    if (layout == MHD_LAYOUT_LEFT)
    {
      HY_CK(cudaMemcpyAsync(dst, host, state_bytes(), cudaMemcpyHostToDevice, stream));
    }
    else
    {
      HY_CK(cudaMemcpyAsync(Q, host, state_bytes(), cudaMemcpyHostToDevice, stream));
      k_htranspose<R><<<nblocks(ncell * nvar, 256), 256, 0, stream>>>(G, Q, dst, 0);
      if (int rc = check_launch())
        return rc;
    }
    return MHD_OK;
  }

  int
  download(const R * src, void * host, int layout)
  {
    if (layout == MHD_LAYOUT_LEFT)
    {
      HY_CK(cudaMemcpyAsync(host, src, state_bytes(), cudaMemcpyDeviceToHost, stream));
    }
    else
    {
      k_htranspose<R><<<nblocks(ncell * nvar, 256), 256, 0, stream>>>(G, src, Q, 1);
      if (int rc = check_launch())
        return rc;
      HY_CK(cudaMemcpyAsync(host, Q, state_bytes(), cudaMemcpyDeviceToHost, stream));
    }
    return MHD_OK;
  }

  int
  init_problem() override
  {
    std::vector<double> h((size_t)ncell * nvar, 0.0);
    init_problem_host(P, h.data());
    if constexpr (sizeof(R) == 8)
    {
      HY_CK(cudaMemcpy(U, h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    else
    {
      std::vector<float> f(h.size());
      for (size_t q = 0; q < h.size(); ++q)
        f[q] = (float)h[q];
      HY_CK(cudaMemcpy(U, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    HY_CK(reset_time_state());
    return apply_init();
  }

  int
  set_state(const void * Uh, int layout) override
  {
    if (int rc = upload(Uh, U, layout))
      return rc;
    HY_CK(reset_time_state());
    return apply_init();
  }

  int
  read_state()
  {
    HY_CK(cudaMemcpyAsync(st_host, st, sizeof(DevState), cudaMemcpyDeviceToHost, stream));
    HY_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  bool
  step_finished_host() const
  {
    return st_host->t >= st_host->tEnd - 1e-14 || st_host->it >= st_host->nStepmax;
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
    launch_bound(cur, 1);
    if (int rc = check_launch())
      return rc;
    if (int rc = download(cur, Uh, layout))
      return rc;
    HY_CK(cudaStreamSynchronize(stream));
    return MHD_OK;
  }

  int
  status_check()
  {
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

  int
  compute_dt(double * dt) override
  {
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    R * cur = current();
    launch_bound(cur, 1);
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
    const int p = (int)(launched & 1);
    R *       in = p ? U2 : U;
    R *       out = p ? U : U2;
    launch_stage(0, in, out);
    launch_stage(1, in, out);
    k_hset_dt<R><<<1, 1, 0, stream>>>(G, st, dt);
    for (int q = 3; q < launches_per_step(); ++q)
      launch_stage(q, in, out);
    ++launched;
    return check_launch();
  }

  int
  replay(int nsteps)
  {
    int left = nsteps;
    while (left >= 2)
    {
      HY_CK(cudaGraphLaunch(graph_pair[launched & 1], stream));
      launched += 2;
      left -= 2;
    }
    if (left)
    {
      HY_CK(cudaGraphLaunch(graph[launched & 1], stream));
      launched += 1;
    }
    return MHD_OK;
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
    if (int rc = replay(nsteps))
      return rc;
    if (int rc = read_state())
      return rc;
    if (done)
      *done = st_host->it - it0;
    return status_check();
  }

  int
  set_host_slabs(int n) override
  {
    if (n < 0 || n > 16)
    {
      err = "host slabs must be in 0..16";
      return MHD_ERR_INVALID_ARG;
    }
    return MHD_OK; // the hydro host step copies the whole state
  }

  // godunov_unsplit_impl on host arrays: upload, one iteration, download
  int
  step_host(const void * Uin, void * Uout, int layout) override
  {
    if (int rc = read_state())
      return rc;
    launched = st_host->it;
    R * out = (launched & 1) ? U : U2;
    if (int rc = upload(Uin, current(), layout))
      return rc;
    if (int rc = tune_form()) // on the uploaded state
      return rc;
    enqueue_step((int)(launched & 1));
    ++launched;
    if (int rc = check_launch())
      return rc;
    if (int rc = download(out, Uout, layout))
      return rc;
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

  // FP64 sums of the stored variables over interior cells (sums[nvar..7] = 0;
  // there is no magnetic field)
  int
  diagnostics(double sums[8], double * divb_l1, double * divb_max) override
  {
    std::vector<double> h(state_bytes() / sizeof(R));
    if (int rc = get_state_vec(h))
      return rc;
    for (int q = 0; q < 8; ++q)
      sums[q] = 0.0;
    const int g = G.g;
    for (int v = 0; v < nvar; ++v)
      for (int k = (dim == 3 ? g : 0); k < (dim == 3 ? G.ksize - g : 1); ++k)
        for (int j = g; j < G.jsize - g; ++j)
          for (int i = g; i < G.isize - g; ++i)
            sums[v] += h[(size_t)v * G.sv + i + j * G.sj + k * G.sk];
    if (divb_l1)
      *divb_l1 = 0.0;
    if (divb_max)
      *divb_max = 0.0;
    return MHD_OK;
  }

  int
  get_state_vec(std::vector<double> & h)
  {
    if constexpr (sizeof(R) == 8)
      return get_state(h.data(), MHD_LAYOUT_LEFT);
    else
    {
      std::vector<float> f(h.size());
      if (int rc = get_state(f.data(), MHD_LAYOUT_LEFT))
        return rc;
      for (size_t q = 0; q < f.size(); ++q)
        h[q] = f[q];
      return MHD_OK;
    }
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
    HY_CK(cudaEventCreate(&e0));
    HY_CK(cudaEventCreate(&e1));
    HY_CK(cudaEventRecord(e0, stream));
    if (int rc = replay(nsteps))
      return rc;
    HY_CK(cudaEventRecord(e1, stream));
    HY_CK(cudaEventSynchronize(e1));
    HY_CK(cudaEventElapsedTime(ms, e0, e1));
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
    const int   p = (int)(launched & 1);
    R *         in = p ? U2 : U;
    R *         out = p ? U : U2;
    const char *kn[kLaunches];
    const int   n = step_kernel_names(kn);
    cudaEvent_t ev[kLaunches + 1];
    for (int q = 0; q <= n; ++q)
      HY_CK(cudaEventCreate(&ev[q]));
    HY_CK(cudaEventRecord(ev[0], stream));
    for (int q = 0; q < n; ++q)
    {
      launch_stage(q, in, out);
      HY_CK(cudaEventRecord(ev[q + 1], stream));
    }
    ++launched;
    if (int rc = check_launch())
      return rc;
    HY_CK(cudaEventSynchronize(ev[n]));
    for (int q = 0; q < n && q < max; ++q)
    {
      if (names)
        names[q] = kn[q];
      HY_CK(cudaEventElapsedTime(&ms[q], ev[q], ev[q + 1]));
    }
    for (int q = 0; q <= n; ++q)
      cudaEventDestroy(ev[q]);
    if (count)
      *count = n;
    return MHD_OK;
  }

  int
  set_surrogate(const uint32_t *, double) override
  {
    err = "the flux surrogate is an option of the MHD solver";
    return MHD_ERR_INVALID_ARG;
  }

  int
  surrogate_stats(int64_t * used, int64_t * total, int) override
  {
    if (used)
      *used = 0;
    if (total)
      *total = 0;
    return MHD_OK;
  }

  int
  harvest(int, float *, int64_t, int64_t *) override
  {
    err = "face harvesting is an option of the MHD solver";
    return MHD_ERR_INVALID_ARG;
  }

  void
  set_time_origin(double t) override
  {
    P.tCurrent = t;
  }

  int64_t
  low_part_bytes() override
  {
    return 0;
  }
  int
  get_low_parts(void *) override
  {
    return MHD_OK;
  }
  int
  set_low_parts(const void *) override
  {
    return MHD_OK;
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
    s[3] = nvar;
    return MHD_OK;
  }
};

#undef HY_CK

} // namespace hydro
} // namespace MHD_VARIANT_TAG
} // namespace mhd
