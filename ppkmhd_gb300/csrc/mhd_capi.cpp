// C ABI of ppkmhd_gb300 (include/ppkmhd_gb300.h): argument checking, variant
// dispatch, .ini parsing, and the host-side Orszag-Tang initial condition.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "mhd_core.h"
#include "ppkmhd_gb300.h"
#include "../host/ConfigMap.h"
#include "../host/HydroParams.h"

struct mhd_ctx
{
  mhd::SolverCore * core = nullptr;
  mhd_params        params{};
  std::string       err;
};

// On-disk header of mhd_checkpoint_save (documented in ppkmhd_gb300.h).
struct CheckpointHeader
{
  char     magic[8];
  uint32_t format, dim, nx, ny, nz, ghost, nbvar, real_bytes;
  double   t, dt;
  int64_t  iteration;
  int32_t  times_saved, pad;
  double   box[7]; // xmin, xmax, ymin, ymax, zmin, zmax, gamma0
};
static_assert(sizeof(CheckpointHeader) == 8 + 8 * 4 + 2 * 8 + 8 + 8 + 7 * 8, "checkpoint header");

struct mhd_ensemble
{
  mhd::EnsembleCore * core = nullptr;
  int                 n = 0;
  std::string         err;
};

namespace
{

int
fail(mhd_ctx * ctx, int rc, const std::string & msg)
{
  if (ctx)
    ctx->err = msg;
  return rc;
}

int
from_core(mhd_ctx * ctx, int rc)
{
  if (rc != MHD_OK)
    ctx->err = ctx->core->err;
  return rc;
}

int
fail(mhd_ensemble * e, int rc, const std::string & msg)
{
  if (e)
    e->err = msg;
  return rc;
}

int
from_core(mhd_ensemble * e, int rc)
{
  if (rc != MHD_OK)
    e->err = e->core->err;
  return rc;
}

} // namespace

namespace mhd
{

// Empty string when the parameters can be run.
// The hydro-only solver's parameters (SolverHydroMuscl<dim>).
std::string
validate_hydro_params(const mhd_params & p)
{
  if (p.dim != 2 && p.dim != 3)
    return "dim must be 2 or 3";
  if (p.ghost != 2)
    return "ghost width must be 2 for the hydro MUSCL scheme";
  if (p.nx < p.ghost || p.ny < p.ghost || (p.dim == 3 && p.nz < p.ghost))
    return "each interior extent must be at least the ghost width (2)";
  const double cells = (double)(p.nx + 4) * (p.ny + 4) * (p.dim == 3 ? p.nz + 4 : 1);
  if (cells * (p.dim + 2) > 4.0e9)
    return "grid too large: ghost-inclusive cells x variables must stay below 4e9";
  if (p.riemann != MHD_RIEMANN_APPROX && p.riemann != MHD_RIEMANN_LLF &&
      p.riemann != MHD_RIEMANN_HLLC && p.riemann != MHD_RIEMANN_HLL)
    return "riemann solver must be approx, llf, hll or hllc for the hydro solver";
  // riemann_hydro's 3D dispatch has no HLL branch (RiemannSolvers.h:608-633):
  // the reference would leave the face flux uninitialised
  if (p.dim == 3 && p.riemann == MHD_RIEMANN_HLL)
    return "the 3D hydro solver has no hll Riemann solver (approx, llf or hllc)";
  // godunov_unsplit_impl has branches for versions 0 and 1 only
  // (SolverHydroMuscl.cpp:277-319, :350-399)
  if (p.implementation_version != 0 && p.implementation_version != 1)
    return "implementationVersion must be 0 or 1 for the hydro solver";
  for (int f = 0; f < (p.dim == 3 ? 6 : 4); ++f)
    if (p.boundary[f] != MHD_BC_REFLECTING && p.boundary[f] != MHD_BC_OUTFLOW &&
        p.boundary[f] != MHD_BC_PERIODIC)
      return "boundary types must be 1 (reflecting), 2 (outflow) or 3 (periodic)";
  // slope_unsplit_hydro_2d/3d: 0 = first order, 1 and 2 limited
  // (HydroBaseFunctor2D.h:487-525); other values leave the slopes unset
  if (p.slope_type != 0.0 && p.slope_type != 1.0 && p.slope_type != 2.0)
    return "slope_type must be 0, 1 (minmod) or 2 (monotonized central)";
  if (!(p.gamma0 > 1.0) || !(p.cfl > 0.0) || !(p.smallr > 0.0) || !(p.smallc > 0.0))
    return "gamma0 must be > 1 and cfl, smallr, smallc > 0";
  if (!(p.xmax > p.xmin) || !(p.ymax > p.ymin) || (p.dim == 3 && !(p.zmax > p.zmin)))
    return "domain bounds must satisfy max > min";
  if (p.precision != MHD_FP64 && p.precision != MHD_FP32)
    return "precision must be 64 or 32";
  if (p.fp_mode != MHD_FP_FAST && p.fp_mode != MHD_FP_EXACT)
    return "fp_mode must be MHD_FP_FAST or MHD_FP_EXACT";
  if (p.precision == MHD_FP32 && p.fp_mode == MHD_FP_EXACT)
    return "MHD_FP_EXACT is only available with MHD_FP64";
  if (p.gravity < 0 || p.gravity > 2)
    return "gravity must be 0, 1 (static) or 2 (point)";
  const int q = p.problem;
  if (q != MHD_PROBLEM_BLAST && q != MHD_PROBLEM_IMPLODE && q != MHD_PROBLEM_KELVIN_HELMHOLTZ &&
      q != MHD_PROBLEM_GRESHO_VORTEX && q != MHD_PROBLEM_FOUR_QUADRANT &&
      q != MHD_PROBLEM_ISENTROPIC_VORTEX && q != MHD_PROBLEM_RAYLEIGH_TAYLOR &&
      q != MHD_PROBLEM_RISING_BUBBLE && q != MHD_PROBLEM_DISK)
    return "unknown problem id for the hydro solver";
  if (p.dim == 3 && (q == MHD_PROBLEM_FOUR_QUADRANT || q == MHD_PROBLEM_ISENTROPIC_VORTEX))
    return "four_quadrant and isentropic_vortex are 2D problems";
  if (q == MHD_PROBLEM_KELVIN_HELMHOLTZ && p.problem_int[3])
    return "kelvin_helmholtz: perturbation_rand draws from Kokkos' own generator; use the sine "
           "perturbation";
  // the hydro functors have the random and the Robertson perturbations only
  // (HydroInitFunctors2D.h:278-332, 3D)
  if (q == MHD_PROBLEM_KELVIN_HELMHOLTZ && !p.problem_int[1])
    return "kelvin_helmholtz: the hydro solver seeds with perturbation_sine_robertson only (the "
           "reference leaves the state empty otherwise)";
  // the init functors of these two write the gravity field, which the
  // reference allocates only with gravity on (SolverHydroMuscl.h:242-246)
  if ((q == MHD_PROBLEM_RAYLEIGH_TAYLOR || q == MHD_PROBLEM_RISING_BUBBLE ||
       q == MHD_PROBLEM_DISK) && !p.gravity)
    return "rayleigh_taylor, rising_bubble and disk need [gravity] static=true or point=true";
  return "";
}

std::string
validate_params(const mhd_params & p)
{
  if (p.solver == MHD_SOLVER_HYDRO_MUSCL)
    return validate_hydro_params(p);
  if (p.solver != MHD_SOLVER_MHD_MUSCL)
    return "solver must be MHD_SOLVER_MHD_MUSCL or MHD_SOLVER_HYDRO_MUSCL";
  if (p.dim != 2 && p.dim != 3)
    return "dim must be 2 or 3";
  if (p.ghost != 3)
    return "ghost width must be 3 for the MHD MUSCL scheme";
  if (p.nx < p.ghost || p.ny < p.ghost || (p.dim == 3 && p.nz < p.ghost))
    return "each interior extent must be at least the ghost width (3)";
  const double cells = (double)(p.nx + 6) * (p.ny + 6) * (p.dim == 3 ? p.nz + 6 : 1);
  if (cells * 8 > 4.0e9)
    return "grid too large: ghost-inclusive cells x 8 variables must stay below 4e9";
  if (p.riemann != MHD_RIEMANN_HLLD && p.riemann != MHD_RIEMANN_HLL && p.riemann != MHD_RIEMANN_LLF)
    return "riemann solver must be hlld, hll or llf for MHD";
  if (p.implementation_version < 0 || p.implementation_version > 2)
    return "implementationVersion must be 0, 1 or 2";
  for (int f = 0; f < (p.dim == 3 ? 6 : 4); ++f)
    if (p.boundary[f] != MHD_BC_REFLECTING && p.boundary[f] != MHD_BC_OUTFLOW &&
        p.boundary[f] != MHD_BC_PERIODIC)
      return "boundary types must be 1 (reflecting), 2 (outflow) or 3 (periodic)";
  // slope_unsplit_hydro_2d/3d compute slopes only for slope_type 1 or 2
  // (MHDBaseFunctor2D.h:464-466, MHDBaseFunctor3D.h:525-526)
  if (p.slope_type != 1.0 && p.slope_type != 2.0)
    return "slope_type must be 1 (minmod) or 2 (monotonized central)";
  if (!(p.gamma0 > 1.0) || !(p.cfl > 0.0) || !(p.smallr > 0.0) || !(p.smallc > 0.0))
    return "gamma0 must be > 1 and cfl, smallr, smallc > 0";
  if (!(p.xmax > p.xmin) || !(p.ymax > p.ymin) || (p.dim == 3 && !(p.zmax > p.zmin)))
    return "domain bounds must satisfy max > min";
  if (p.precision != MHD_FP64 && p.precision != MHD_FP32)
    return "precision must be 64 or 32";
  if (p.fp_mode != MHD_FP_FAST && p.fp_mode != MHD_FP_EXACT)
    return "fp_mode must be MHD_FP_FAST or MHD_FP_EXACT";
  if (p.precision == MHD_FP32 && p.fp_mode == MHD_FP_EXACT)
    return "MHD_FP_EXACT is only available with MHD_FP64";
  if (p.problem < MHD_PROBLEM_ORSZAG_TANG || p.problem > MHD_PROBLEM_WAVE)
    return "unknown problem id";
  if (p.problem == MHD_PROBLEM_KELVIN_HELMHOLTZ && p.problem_int[3])
    return "kelvin_helmholtz: perturbation_rand draws from Kokkos' own generator; use the sine "
           "perturbations";
  if (p.problem == MHD_PROBLEM_KELVIN_HELMHOLTZ && !p.problem_int[0] && !p.problem_int[1])
    return "kelvin_helmholtz: no perturbation selected (the reference leaves the state empty)";
  if (p.problem == MHD_PROBLEM_WAVE && (p.problem_int[0] < 0 || p.problem_int[0] > 3))
    return "wave: type must be 0 (fast), 1 (Alfven), 2 (slow) or 3 (contact)";
  return "";
}

} // namespace mhd

namespace
{
using mhd::validate_params;
} // namespace

namespace mhd
{


} // namespace mhd

namespace
{

// restart_upscale (IO_HDF5.h:1603-1694 of the reference, copy_buffer): a
// state of half the resolution, ghost cells included (isize_c = nx/2 + 2g),
// onto the context's grid.  Fine cell i (ghost-inclusive) takes coarse cell
// (i + g) / 2 (integer division) along every axis; the face-centred normal
// field takes the coarse face value where i + g is even and the mean of the
// two coarse faces around it otherwise, so the discrete div B stays zero.
template <class T>
void
upscale_state(const T * c, T * f, int dim, int isize, int jsize, int ksize, int g, int nx, int ny,
              int nvar)
{
  const int64_t iL = nx / 2 + 2 * g, jL = ny / 2 + 2 * g;
  const int64_t cv = iL * jL * (dim == 3 ? (ksize - 2 * g) / 2 + 2 * g : 1);
  const int64_t fv = (int64_t)isize * jsize * ksize;
  const bool mhd = nvar == 8; // the hydro solver has no face-centred field
  for (int v = 0; v < nvar; ++v)
    for (int k = 0; k < ksize; ++k)
    {
      const int kl = dim == 3 ? (k + g) / 2 : 0;
      for (int j = 0; j < jsize; ++j)
      {
        const int jl = (j + g) / 2;
        for (int i = 0; i < isize; ++i)
        {
          const int      il = (i + g) / 2;
          const T *      src = c + v * cv;
          const int64_t  a = il + iL * jl + iL * jL * kl;
          T              x = src[a];
          if (mhd && v == 5 && i + g - 2 * il != 0)
            x = (src[a] + src[a + 1]) / 2;
          else if (mhd && v == 6 && j + g - 2 * jl != 0)
            x = (src[a] + src[a + iL]) / 2;
          else if (mhd && dim == 3 && v == 7 && k + g - 2 * kl != 0)
            x = (src[a] + src[a + iL * jL]) / 2;
          f[v * fv + i + (int64_t)isize * (j + (int64_t)jsize * k)] = x;
        }
      }
    }
}

int
checkpoint_load(mhd_ctx * ctx, const char * path, int reset_time, int * times_saved, bool upscale)
{
  if (!ctx || !ctx->core)
    return MHD_ERR_INVALID_ARG;
  if (!path)
    return fail(ctx, MHD_ERR_INVALID_ARG, "null path");
  FILE * f = std::fopen(path, "rb");
  if (!f)
    return fail(ctx, MHD_ERR_INVALID_ARG, std::string("cannot open ") + path);
  CheckpointHeader   h{};
  const bool         got = std::fread(&h, sizeof h, 1, f) == 1;
  int                sz[4];
  ctx->core->sizes(sz);
  const mhd_params & p = ctx->params;
  const int          k = upscale ? 2 : 1; // file resolution = context / k
  std::string        bad;
  if (!got || std::memcmp(h.magic, "PPKMHDCK", 8) != 0 || (h.format != 1 && h.format != 2))
    bad = "not a checkpoint file (format 1 or 2)";
  else if (upscale && (p.nx % 2 || p.ny % 2 || (p.dim == 3 && p.nz % 2)))
    bad = "restart_upscale needs even nx, ny, nz";
  else if ((int)h.dim != p.dim || (int)h.nx * k != p.nx || (int)h.ny * k != p.ny ||
           (p.dim == 3 && (int)h.nz * k != p.nz) || (int)h.ghost != p.ghost ||
           (int)h.nbvar != sz[3])
    bad = upscale ? "checkpoint grid is not half the context's (restart_upscale)"
                  : "checkpoint grid does not match the context";
  else if ((int)h.real_bytes != ctx->core->real_bytes())
    bad = "checkpoint precision does not match the context";
  const int                  g = p.ghost;
  const size_t               nfile = (size_t)(h.nx + 2 * g) * (h.ny + 2 * g) *
                         (p.dim == 3 ? h.nz + 2 * g : 1) * sz[3];
  std::vector<unsigned char> U, lo;
  if (bad.empty())
  {
    U.resize(nfile * h.real_bytes);
    if (std::fread(U.data(), 1, U.size(), f) != U.size())
      bad = "checkpoint file is truncated";
    // the low parts of a compensated FP32 state carry over at the same
    // resolution only (an upscaled state starts without them)
    if (bad.empty() && h.format == 2 && !upscale)
    {
      lo.resize((size_t)ctx->core->low_part_bytes());
      if (lo.empty())
        bad = "checkpoint has low parts the context does not keep";
      else if (std::fread(lo.data(), 1, lo.size(), f) != lo.size())
        bad = "checkpoint file is truncated";
    }
  }
  std::fclose(f);
  if (!bad.empty())
    return fail(ctx, MHD_ERR_INVALID_ARG, bad);
  if (upscale)
  {
    std::vector<unsigned char> fine((size_t)sz[0] * sz[1] * sz[2] * sz[3] * h.real_bytes);
    if (h.real_bytes == 8)
      upscale_state((const double *)U.data(), (double *)fine.data(), p.dim, sz[0], sz[1],
                    p.dim == 3 ? sz[2] : 1, g, p.nx, p.ny, sz[3]);
    else
      upscale_state((const float *)U.data(), (float *)fine.data(), p.dim, sz[0], sz[1],
                    p.dim == 3 ? sz[2] : 1, g, p.nx, p.ny, sz[3]);
    U.swap(fine);
  }
  ctx->core->set_time_origin(reset_time ? 0.0 : h.t);
  int rc = ctx->core->set_state(U.data(), MHD_LAYOUT_LEFT);
  ctx->core->set_time_origin(p.tCurrent);
  if (rc == MHD_OK && !lo.empty())
    rc = ctx->core->set_low_parts(lo.data());
  if (rc)
    return from_core(ctx, rc);
  if (times_saved)
    *times_saved = h.times_saved;
  return MHD_OK;
}

} // namespace

extern "C"
{

  const char *
  mhd_version(void)
  {
    return "ppkmhd_gb300 1.0 (sm_103a)";
  }

  int
  mhd_params_default(mhd_params * p)
  {
    if (!p)
      return MHD_ERR_INVALID_ARG;
    std::memset(p, 0, sizeof *p);
    p->dim = 2;
    p->nx = p->ny = p->nz = 1;
    p->ghost = 3;
    p->xmin = p->ymin = p->zmin = 0.0;
    p->xmax = p->ymax = p->zmax = 1.0;
    p->gamma0 = 1.4;
    p->cfl = 1.0;
    p->slope_type = 2.0;
    p->smallr = 1e-8;
    p->smallc = 1e-8;
    p->riemann = MHD_RIEMANN_HLLD;
    p->implementation_version = 2;
    for (int f = 0; f < 6; ++f)
      p->boundary[f] = MHD_BC_PERIODIC;
    p->tEnd = 1.0;
    p->tCurrent = 0.0;
    p->nStepmax = 1000;
    p->problem = MHD_PROBLEM_ORSZAG_TANG;
    p->ot_kt = 0.0;
    p->precision = MHD_FP64;
    p->fp_mode = MHD_FP_FAST;
    p->device = 0;
    return MHD_OK;
  }

  int
  mhd_params_from_ini(const char * ini_text, mhd_params * p, char * err, size_t errlen)
  {
    auto set_err = [&](const std::string & m) {
      if (err && errlen)
        std::snprintf(err, errlen, "%s", m.c_str());
    };
    if (!ini_text || !p)
    {
      set_err("null argument");
      return MHD_ERR_INVALID_ARG;
    }
    ConfigMap                 map(ini_text, (int)std::strlen(ini_text));
    ppkmhd_gb300::HydroParams hp;
    hp.setup(map);
    if (!hp.valid_solver)
    {
      set_err("[run] solver_name must be MHD_Muscl_2D, MHD_Muscl_3D, Hydro_Muscl_2D or "
              "Hydro_Muscl_3D");
      return MHD_ERR_PARSE;
    }
    // back-end options (not in the reference): [gb300] precision = 64|32,
    // [gb300] fp_mode = fast|exact
    const int         precision = (int)map.getInteger("gb300", "precision", 64);
    const std::string mode = map.getString("gb300", "fp_mode", "fast");
    *p = hp.to_mhd_params(map, precision, mode == "exact" ? MHD_FP_EXACT : MHD_FP_FAST);
    set_err("");
    return MHD_OK;
  }

  int
  mhd_create(const mhd_params * p, mhd_ctx ** out)
  {
    if (!p || !out)
      return MHD_ERR_INVALID_ARG;
    *out = nullptr;
    const std::string bad = validate_params(*p);
    mhd_ctx *         ctx = new (std::nothrow) mhd_ctx;
    if (!ctx)
      return MHD_ERR_CUDA;
    ctx->params = *p;
    if (!bad.empty())
    {
      ctx->err = bad;
      *out = ctx; // so that mhd_last_error can report; the context has no core
      return MHD_ERR_INVALID_ARG;
    }
    std::string err;
    const bool  hydro = p->solver == MHD_SOLVER_HYDRO_MUSCL;
    if (p->precision == MHD_FP32)
      ctx->core = hydro ? mhd::create_hydro_core_f32(*p, err) : mhd::create_core_f32(*p, err);
    else if (p->fp_mode == MHD_FP_EXACT)
      ctx->core = hydro ? mhd::create_hydro_core_f64x(*p, err) : mhd::create_core_f64x(*p, err);
    else
      ctx->core = hydro ? mhd::create_hydro_core_f64(*p, err) : mhd::create_core_f64(*p, err);
    *out = ctx;
    if (!ctx->core && err.find("out of range") != std::string::npos)
    {
      ctx->err = err;
      return MHD_ERR_INVALID_ARG;
    }
    if (!ctx->core)
    {
      ctx->err = err;
      return err.find("no CUDA device") != std::string::npos ? MHD_ERR_NO_DEVICE : MHD_ERR_CUDA;
    }
    return MHD_OK;
  }

  int
  mhd_destroy(mhd_ctx * ctx)
  {
    if (!ctx)
      return MHD_ERR_INVALID_ARG;
    delete ctx->core;
    delete ctx;
    return MHD_OK;
  }

#define NEED_CORE(ctx)                                                   \
  do                                                                     \
  {                                                                      \
    if (!(ctx))                                                          \
      return MHD_ERR_INVALID_ARG;                                        \
    if (!(ctx)->core)                                                    \
      return fail((ctx), MHD_ERR_INVALID_ARG, "context was not created"); \
    if (int rc_ = (ctx)->core->bind_device())                            \
      return from_core((ctx), rc_);                                      \
  } while (0)

  int
  mhd_initial_state(const mhd_params * p, double * U)
  {
    if (!p || !U || !validate_params(*p).empty())
      return MHD_ERR_INVALID_ARG;
    const int    nvar = p->solver == MHD_SOLVER_HYDRO_MUSCL ? p->dim + 2 : 8;
    const size_t n = (size_t)(p->nx + 2 * p->ghost) * (p->ny + 2 * p->ghost) *
                     (p->dim == 3 ? p->nz + 2 * p->ghost : 1) * nvar;
    std::memset(U, 0, n * sizeof(double));
    mhd::init_problem_host(*p, U);
    return MHD_OK;
  }

  int
  mhd_init_problem(mhd_ctx * ctx)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->init_problem());
  }

  static int
  check_array(mhd_ctx * ctx, const void * U, int layout, int real_bytes)
  {
    if (!U)
      return fail(ctx, MHD_ERR_INVALID_ARG, "null state array");
    if (layout != MHD_LAYOUT_LEFT && layout != MHD_LAYOUT_RIGHT)
      return fail(ctx, MHD_ERR_INVALID_ARG, "layout must be MHD_LAYOUT_LEFT or MHD_LAYOUT_RIGHT");
    if (real_bytes != ctx->core->real_bytes())
      return fail(ctx, MHD_ERR_INVALID_ARG,
                  "real_bytes " + std::to_string(real_bytes) + " does not match the context precision");
    return MHD_OK;
  }

  int
  mhd_set_state(mhd_ctx * ctx, const void * U, int layout, int real_bytes)
  {
    NEED_CORE(ctx);
    if (int rc = check_array(ctx, U, layout, real_bytes))
      return rc;
    return from_core(ctx, ctx->core->set_state(U, layout));
  }

  int
  mhd_get_state(mhd_ctx * ctx, void * U, int layout, int real_bytes)
  {
    NEED_CORE(ctx);
    if (int rc = check_array(ctx, U, layout, real_bytes))
      return rc;
    return from_core(ctx, ctx->core->get_state(U, layout));
  }

  int
  mhd_step(mhd_ctx * ctx)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->step());
  }

  int
  mhd_compute_dt(mhd_ctx * ctx, double * dt)
  {
    NEED_CORE(ctx);
    if (!dt)
      return fail(ctx, MHD_ERR_INVALID_ARG, "dt must not be NULL");
    return from_core(ctx, ctx->core->compute_dt(dt));
  }

  int
  mhd_step_dt(mhd_ctx * ctx, double dt)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->step_dt(dt));
  }

  int
  mhd_run(mhd_ctx * ctx, int nsteps, int * done)
  {
    NEED_CORE(ctx);
    if (nsteps < 0)
      return fail(ctx, MHD_ERR_INVALID_ARG, "nsteps must be >= 0");
    return from_core(ctx, ctx->core->run(nsteps, done));
  }

  int
  mhd_step_host(mhd_ctx * ctx, const void * U_in, void * U_out, int layout, int real_bytes)
  {
    NEED_CORE(ctx);
    if (int rc = check_array(ctx, U_in, layout, real_bytes))
      return rc;
    if (int rc = check_array(ctx, U_out, layout, real_bytes))
      return rc;
    return from_core(ctx, ctx->core->step_host(U_in, U_out, layout));
  }

  int
  mhd_set_host_slabs(mhd_ctx * ctx, int nslabs)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->set_host_slabs(nslabs));
  }

  int
  mhd_set_fused(mhd_ctx * ctx, int fused)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->set_fused(fused));
  }

  int
  mhd_get_fused(mhd_ctx * ctx, int * fused)
  {
    NEED_CORE(ctx);
    if (!fused)
      return fail(ctx, MHD_ERR_INVALID_ARG, "null pointer");
    *fused = ctx->core->fused_form();
    return MHD_OK;
  }

  int
  mhd_time(mhd_ctx * ctx, double * t, double * dt, int * iteration)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->time(t, dt, iteration));
  }

  int
  mhd_diagnostics(mhd_ctx * ctx, double sums[8], double * divb_l1, double * divb_max)
  {
    NEED_CORE(ctx);
    if (!sums)
      return fail(ctx, MHD_ERR_INVALID_ARG, "null sums");
    return from_core(ctx, ctx->core->diagnostics(sums, divb_l1, divb_max));
  }

  int
  mhd_run_timed(mhd_ctx * ctx, int nsteps, float * ms)
  {
    NEED_CORE(ctx);
    if (!ms || nsteps < 0)
      return fail(ctx, MHD_ERR_INVALID_ARG, "bad arguments");
    return from_core(ctx, ctx->core->run_timed(nsteps, ms));
  }

  int
  mhd_profile_step(mhd_ctx * ctx, const char ** names, float * ms, int max, int * count)
  {
    NEED_CORE(ctx);
    if (!ms)
      return fail(ctx, MHD_ERR_INVALID_ARG, "null ms");
    return from_core(ctx, ctx->core->profile_step(names, ms, max, count));
  }

  int
  mhd_cell_counts(mhd_ctx * ctx, int64_t * interior, int64_t * with_ghosts)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->cell_counts(interior, with_ghosts));
  }

  int
  mhd_sizes(mhd_ctx * ctx, int sizes[4])
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->sizes(sizes));
  }

  int
  mhd_launches_per_step(mhd_ctx * ctx, int * n)
  {
    NEED_CORE(ctx);
    if (n)
      *n = ctx->core->launches_per_step();
    return MHD_OK;
  }

  int
  mhd_checkpoint_save(mhd_ctx * ctx, const char * path, int times_saved)
  {
    NEED_CORE(ctx);
    if (!path)
      return fail(ctx, MHD_ERR_INVALID_ARG, "null path");
    int sz[4];
    ctx->core->sizes(sz);
    const size_t n = (size_t)sz[0] * sz[1] * sz[2] * sz[3];
    const int    rb = ctx->core->real_bytes();
    std::vector<unsigned char> U(n * rb);
    if (int rc = ctx->core->get_state(U.data(), MHD_LAYOUT_LEFT))
      return from_core(ctx, rc);
    // format 2: format 1 followed by the FP32 low parts of the state
    std::vector<unsigned char> lo((size_t)ctx->core->low_part_bytes());
    if (!lo.empty())
      if (int rc = ctx->core->get_low_parts(lo.data()))
        return from_core(ctx, rc);
    double t = 0, dt = 0;
    int    it = 0;
    if (int rc = ctx->core->time(&t, &dt, &it))
      return from_core(ctx, rc);
    const mhd_params & p = ctx->params;
    CheckpointHeader   h{};
    std::memcpy(h.magic, "PPKMHDCK", 8);
    h.format = lo.empty() ? 1 : 2;
    h.dim = (uint32_t)p.dim;
    h.nx = (uint32_t)p.nx;
    h.ny = (uint32_t)p.ny;
    h.nz = (uint32_t)(p.dim == 3 ? p.nz : 1);
    h.ghost = (uint32_t)p.ghost;
    h.nbvar = (uint32_t)sz[3];
    h.real_bytes = (uint32_t)rb;
    h.t = t;
    h.dt = dt;
    h.iteration = it;
    h.times_saved = times_saved;
    const double box[7] = { p.xmin, p.xmax, p.ymin, p.ymax, p.zmin, p.zmax, p.gamma0 };
    std::memcpy(h.box, box, sizeof box);
    FILE * f = std::fopen(path, "wb");
    if (!f)
      return fail(ctx, MHD_ERR_INVALID_ARG, std::string("cannot open ") + path + " for writing");
    const bool ok = std::fwrite(&h, sizeof h, 1, f) == 1 &&
                    std::fwrite(U.data(), 1, U.size(), f) == U.size() &&
                    std::fwrite(lo.data(), 1, lo.size(), f) == lo.size();
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed)
      return fail(ctx, MHD_ERR_INVALID_ARG, std::string("short write to ") + path);
    return MHD_OK;
  }

  int
  mhd_checkpoint_load(mhd_ctx * ctx, const char * path, int reset_time, int * times_saved)
  {
    return checkpoint_load(ctx, path, reset_time, times_saved, false);
  }

  int
  mhd_checkpoint_load_upscaled(mhd_ctx * ctx, const char * path, int reset_time, int * times_saved)
  {
    return checkpoint_load(ctx, path, reset_time, times_saved, true);
  }

  int
  mhd_harvest_faces(mhd_ctx * ctx, int stride, float * records, int64_t capacity, int64_t * count)
  {
    NEED_CORE(ctx);
    if (stride < 1 || !count)
      return fail(ctx, MHD_ERR_INVALID_ARG, "stride must be >= 1 and count non-null");
    return from_core(ctx, ctx->core->harvest(stride, records, capacity, count));
  }

  int
  mhd_set_surrogate(mhd_ctx * ctx, const mhd_mlp * mlp, double tau)
  {
    NEED_CORE(ctx);
    if (!mlp)
      return from_core(ctx, ctx->core->set_surrogate(nullptr, 0.0));
    if (!(tau > 0.0) || tau > 0.1)
      return fail(ctx, MHD_ERR_INVALID_ARG, "tau must be in (0, 0.1]");
    if (std::fabs(mhd::mlp_gamma(mlp) - ctx->params.gamma0) > 1e-6 * ctx->params.gamma0)
      return fail(ctx, MHD_ERR_INVALID_ARG,
                  "the network was trained for another adiabatic index (gamma0)");
    std::vector<uint32_t> pack(mhd::kMlpPackTotal);
    mhd::mlp_pack(mhd::mlp_params(mlp), pack.data());
    return from_core(ctx, ctx->core->set_surrogate(pack.data(), tau));
  }

  int
  mhd_surrogate_stats(mhd_ctx * ctx, int64_t * faces_network, int64_t * faces_total, int reset)
  {
    NEED_CORE(ctx);
    return from_core(ctx, ctx->core->surrogate_stats(faces_network, faces_total, reset));
  }

  const char *
  mhd_last_error(mhd_ctx * ctx)
  {
    return ctx ? ctx->err.c_str() : "null context";
  }

  // ---------------------------------------------------------------- ensembles

  int
  mhd_ensemble_create(const mhd_params * p, int n, mhd_ensemble ** out)
  {
    if (!p || !out || n <= 0)
      return MHD_ERR_INVALID_ARG;
    *out = nullptr;
    mhd_ensemble * e = new (std::nothrow) mhd_ensemble;
    if (!e)
      return MHD_ERR_CUDA;
    e->n = n;
    *out = e;
    for (int q = 0; q < n; ++q)
    {
      const std::string bad = validate_params(p[q]);
      if (!bad.empty())
        return fail(e, MHD_ERR_INVALID_ARG, "problem " + std::to_string(q) + ": " + bad);
      if (p[q].solver != MHD_SOLVER_MHD_MUSCL)
        return fail(e, MHD_ERR_INVALID_ARG,
                    "problem " + std::to_string(q) + ": ensembles run the MHD solver");
      if (p[q].implementation_version != 2)
        return fail(e, MHD_ERR_INVALID_ARG,
                    "problem " + std::to_string(q) + ": ensembles use implementation version 2");
      if (p[q].dim != p[0].dim || p[q].precision != p[0].precision ||
          p[q].fp_mode != p[0].fp_mode || p[q].device != p[0].device)
        return fail(e, MHD_ERR_INVALID_ARG,
                    "problem " + std::to_string(q) +
                      ": dim, precision, fp_mode and device must be the same for all problems");
    }
    std::string err;
    if (p[0].precision == MHD_FP32)
      e->core = mhd::create_ensemble_f32(p, n, err);
    else if (p[0].fp_mode == MHD_FP_EXACT)
      e->core = mhd::create_ensemble_f64x(p, n, err);
    else
      e->core = mhd::create_ensemble_f64(p, n, err);
    if (!e->core)
      return fail(e, err.find("no CUDA device") != std::string::npos ? MHD_ERR_NO_DEVICE : MHD_ERR_CUDA,
                  err);
    return MHD_OK;
  }

  int
  mhd_ensemble_destroy(mhd_ensemble * e)
  {
    if (!e)
      return MHD_ERR_INVALID_ARG;
    delete e->core;
    delete e;
    return MHD_OK;
  }

#define NEED_ENSEMBLE(e)                                                   \
  do                                                                       \
  {                                                                        \
    if (!(e))                                                              \
      return MHD_ERR_INVALID_ARG;                                          \
    if (!(e)->core)                                                        \
      return fail((e), MHD_ERR_INVALID_ARG, "ensemble was not created");   \
    if (int rc_ = (e)->core->bind_device())                                \
      return from_core((e), rc_);                                          \
  } while (0)

  static int
  check_problem_array(mhd_ensemble * e, int prob, const void * U, int layout, int real_bytes)
  {
    if (prob < 0 || prob >= e->n)
      return fail(e, MHD_ERR_INVALID_ARG, "problem index out of range");
    if (!U)
      return fail(e, MHD_ERR_INVALID_ARG, "null state array");
    if (layout != MHD_LAYOUT_LEFT && layout != MHD_LAYOUT_RIGHT)
      return fail(e, MHD_ERR_INVALID_ARG, "layout must be MHD_LAYOUT_LEFT or MHD_LAYOUT_RIGHT");
    if (real_bytes != e->core->real_bytes())
      return fail(e, MHD_ERR_INVALID_ARG,
                  "real_bytes " + std::to_string(real_bytes) + " does not match the ensemble precision");
    return MHD_OK;
  }

  int
  mhd_ensemble_init_problem(mhd_ensemble * e, int prob)
  {
    NEED_ENSEMBLE(e);
    return from_core(e, e->core->init_problem(prob));
  }

  int
  mhd_ensemble_set_state(mhd_ensemble * e, int prob, const void * U, int layout, int real_bytes)
  {
    NEED_ENSEMBLE(e);
    if (int rc = check_problem_array(e, prob, U, layout, real_bytes))
      return rc;
    return from_core(e, e->core->set_state(prob, U, layout));
  }

  int
  mhd_ensemble_get_state(mhd_ensemble * e, int prob, void * U, int layout, int real_bytes)
  {
    NEED_ENSEMBLE(e);
    if (int rc = check_problem_array(e, prob, U, layout, real_bytes))
      return rc;
    return from_core(e, e->core->get_state(prob, U, layout));
  }

  static int
  check_problem_arrays(mhd_ensemble * e, const void * const * U, int layout, int real_bytes)
  {
    if (!U)
      return fail(e, MHD_ERR_INVALID_ARG, "null array of state pointers");
    for (int p = 0; p < e->n; ++p)
      if (int rc = check_problem_array(e, p, U[p], layout, real_bytes))
        return rc;
    return MHD_OK;
  }

  int
  mhd_ensemble_set_states(mhd_ensemble * e, const void * const * U, int layout, int real_bytes)
  {
    NEED_ENSEMBLE(e);
    if (int rc = check_problem_arrays(e, U, layout, real_bytes))
      return rc;
    return from_core(e, e->core->set_states(U, layout));
  }

  int
  mhd_ensemble_get_states(mhd_ensemble * e, void * const * U, int layout, int real_bytes)
  {
    NEED_ENSEMBLE(e);
    if (int rc = check_problem_arrays(e, U, layout, real_bytes))
      return rc;
    return from_core(e, e->core->get_states(U, layout));
  }

  int
  mhd_ensemble_run(mhd_ensemble * e, int nsteps, float * ms)
  {
    NEED_ENSEMBLE(e);
    if (nsteps < 0)
      return fail(e, MHD_ERR_INVALID_ARG, "nsteps must be non-negative");
    return from_core(e, e->core->run(nsteps, ms));
  }

  int
  mhd_ensemble_time(mhd_ensemble * e, int prob, double * t, double * dt, int * iteration)
  {
    NEED_ENSEMBLE(e);
    return from_core(e, e->core->time(prob, t, dt, iteration));
  }

  int
  mhd_ensemble_diagnostics(mhd_ensemble * e, int prob, double sums[8], double * divb_l1,
                           double * divb_max)
  {
    NEED_ENSEMBLE(e);
    if (!sums)
      return fail(e, MHD_ERR_INVALID_ARG, "null sums");
    return from_core(e, e->core->diagnostics(prob, sums, divb_l1, divb_max));
  }

  int
  mhd_ensemble_autotune(mhd_ensemble * e, char * report, size_t report_len)
  {
    NEED_ENSEMBLE(e);
    std::string text;
    const int   rc = e->core->autotune(text);
    if (report && report_len)
    {
      std::strncpy(report, text.c_str(), report_len - 1);
      report[report_len - 1] = 0;
    }
    return from_core(e, rc);
  }

  int
  mhd_ensemble_set_mode(mhd_ensemble * e, int mode)
  {
    NEED_ENSEMBLE(e);
    return from_core(e, e->core->set_mode(mode));
  }

  int
  mhd_ensemble_get_mode(mhd_ensemble * e, int * mode)
  {
    NEED_ENSEMBLE(e);
    if (!mode)
      return fail(e, MHD_ERR_INVALID_ARG, "null output");
    *mode = e->core->mode();
    return MHD_OK;
  }

  int
  mhd_ensemble_set_wait_limit(mhd_ensemble * e, long long cycles)
  {
    NEED_ENSEMBLE(e);
    return from_core(e, e->core->set_wait_limit(cycles));
  }

  int
  mhd_ensemble_profile_step(mhd_ensemble * e, const char ** names, float * ms, int max, int * count)
  {
    NEED_ENSEMBLE(e);
    if (!ms)
      return fail(e, MHD_ERR_INVALID_ARG, "null ms");
    return from_core(e, e->core->profile_step(names, ms, max, count));
  }

  int
  mhd_ensemble_cell_count(mhd_ensemble * e, int64_t * interior)
  {
    NEED_ENSEMBLE(e);
    if (!interior)
      return fail(e, MHD_ERR_INVALID_ARG, "null output");
    return from_core(e, e->core->cells(interior));
  }

  int
  mhd_ensemble_launches_per_step(mhd_ensemble * e, int * n)
  {
    NEED_ENSEMBLE(e);
    if (n)
      *n = e->core->launches_per_step();
    return MHD_OK;
  }

  const char *
  mhd_ensemble_last_error(mhd_ensemble * e)
  {
    return e ? e->err.c_str() : "null ensemble";
  }

} // extern "C"
