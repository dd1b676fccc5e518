// Host-side interface between the C ABI (mhd_capi.cpp) and the solver
// cores, one per arithmetic variant (FP64 exact, FP64 fast, FP32), each
// compiled from mhd_variant.cu into its own inline namespace.
#pragma once

#include <cstdint>
#include <string>

#include "ppkmhd_gb300.h"

namespace mhd
{

class SolverCore
{
public:
  virtual ~SolverCore() {}
  virtual int init_problem() = 0;
  virtual int set_state(const void * U, int layout) = 0;
  virtual int get_state(void * U, int layout) = 0;
  virtual int step() = 0;
  virtual int compute_dt(double * dt) = 0;
  virtual int step_dt(double dt) = 0;
  virtual int run(int nsteps, int * done) = 0;
  virtual int step_host(const void * Uin, void * Uout, int layout) = 0;
  virtual int set_host_slabs(int n) = 0;
  virtual int time(double * t, double * dt, int * it) = 0;
  virtual int diagnostics(double sums[8], double * divb_l1, double * divb_max) = 0;
  virtual int run_timed(int nsteps, float * ms) = 0;
  virtual int profile_step(const char ** names, float * ms, int max, int * count) = 0;
  virtual int cell_counts(int64_t * interior, int64_t * with_ghosts) = 0;
  virtual int sizes(int s[4]) = 0;
  virtual int launches_per_step() = 0;
  virtual int real_bytes() const = 0;
  //! make the context's device current for the calling thread
  virtual int bind_device() = 0;
  //! flux surrogate: packed weights + biases (mhd_mlp.cuh), nullptr = off
  virtual int set_surrogate(const uint32_t * wpack, double tau) = 0;
  virtual int surrogate_stats(int64_t * used, int64_t * total, int reset) = 0;
  //! face samples of the next iteration (mhd_harvest_faces)
  virtual int harvest(int stride, float * host, int64_t capacity, int64_t * count) = 0;
  //! time that set_state / init_problem start from (tCurrent)
  virtual void set_time_origin(double t) = 0;
  //! the fused plain form (hydro solver; 2D MHD solver) or the stage kernels
  virtual int set_fused(int on)
  {
    if (on)
    {
      err = "no fused form for this configuration";
      return MHD_ERR_INVALID_ARG;
    }
    return MHD_OK;
  }
  virtual int fused_form() const { return 0; }
  //! FP32 version-2 contexts keep the low parts of the state (Buffers::Ulo):
  //! their size in bytes (0: none), and host copies for checkpoints
  virtual int64_t low_part_bytes() = 0;
  virtual int     get_low_parts(void * host) = 0;
  virtual int     set_low_parts(const void * host) = 0;
  std::string err;
};

// An ensemble of independent problems of one dimension and precision,
// advanced together (mhd_ensemble.cuh).
class EnsembleCore
{
public:
  virtual ~EnsembleCore() {}
  virtual int init_problem(int p) = 0;
  virtual int set_state(int p, const void * U, int layout) = 0;
  virtual int get_state(int p, void * U, int layout) = 0;
  virtual int set_states(const void * const * U, int layout) = 0;
  virtual int get_states(void * const * U, int layout) = 0;
  virtual int run(int nsteps, float * ms) = 0;
  virtual int time(int p, double * t, double * dt, int * it) = 0;
  virtual int diagnostics(int p, double sums[8], double * divb_l1, double * divb_max) = 0;
  virtual int autotune(std::string & report) = 0;
  virtual int profile_step(const char ** names, float * ms, int max, int * count) = 0;
  virtual int cells(int64_t * interior) = 0;
  virtual int launches_per_step() const = 0;
  //! MHD_ENSEMBLE_GRAPHS or MHD_ENSEMBLE_PERSISTENT (mhd_ensemble_set_mode)
  virtual int set_mode(int mode) = 0;
  virtual int mode() const = 0;
  //! clock-cycle bound of every grid-barrier wait of the persistent form
  virtual int set_wait_limit(long long cycles) = 0;
  virtual int real_bytes() const = 0;
  virtual int bind_device() = 0;
  std::string err;
};

// Factories (return nullptr and fill err on failure).
SolverCore * create_core_f64x(const mhd_params & p, std::string & err);
SolverCore * create_core_f64(const mhd_params & p, std::string & err);
SolverCore * create_core_f32(const mhd_params & p, std::string & err);
// hydro-only MUSCL solver cores (hydro_variant.cu), mhd_params::solver =
// MHD_SOLVER_HYDRO_MUSCL
SolverCore * create_hydro_core_f64x(const mhd_params & p, std::string & err);
SolverCore * create_hydro_core_f64(const mhd_params & p, std::string & err);
SolverCore * create_hydro_core_f32(const mhd_params & p, std::string & err);
EnsembleCore * create_ensemble_f64x(const mhd_params * p, int n, std::string & err);
EnsembleCore * create_ensemble_f64(const mhd_params * p, int n, std::string & err);
EnsembleCore * create_ensemble_f32(const mhd_params * p, int n, std::string & err);

// Flux surrogate helpers (mhd_mlp.cu): packed weights + biases for the
// flux stage (kMlpPackTotal words), the network's gamma0 and parameters.
constexpr int kMlpPackTotal = 3840 + 152;
void          mlp_pack(const float * params, uint32_t * out);
double        mlp_gamma(const mhd_mlp * m);
const float * mlp_params(const mhd_mlp * m);

// Empty string when the parameters can be run, else the reason (mhd_capi.cpp).
std::string validate_params(const mhd_params & p);

// Initial condition of p.problem in FP64 on the host, LayoutLeft, ghosts
// included, into a zeroed array (mhd_init.cpp; hydro problems in
// hydro_init.cpp).
void init_problem_host(const mhd_params & p, double * U);
// Orszag-Tang initial condition (MHDInitFunctors2D.h:241-389,
// MHDInitFunctors3D.h:264-415).
void init_orszag_tang_host(const mhd_params & p, double * U);
// Initial conditions of the hydro-only solver (hydro_init.cpp).
void init_hydro_problem_host(const mhd_params & p, double * U);
// The gravity field the hydro problem's initialisation writes, dim planes
// over the ghost-inclusive cells, LayoutLeft (hydro_init.cpp).
void init_hydro_gravity_host(const mhd_params & p, double * g);

} // namespace mhd
