/*
 * ppkmhd_gb300 -- C ABI of the GB300-native (sm_103a) MUSCL-Hancock + HLLD +
 * constrained-transport MHD step.
 *
 * Drop-in boundary: this ABI replaces the device side of ppkMHD's
 * SolverMHDMuscl<dim> (src/muscl/SolverMHDMuscl.h, .cpp).  The C++ host layer
 * in ppkmhd_gb300/host (ConfigMap, HydroParams, SolverBase, SolverFactory,
 * SolverMHDMusclGPU) keeps the reference's plugin interface and calls these
 * functions.  All functions return an int status (MHD_OK = 0); on error the
 * message is available from mhd_last_error().  No function aborts, traps or
 * prints.  A context is used by one host thread at a time; it owns one CUDA
 * stream and all device buffers.  Host arrays are owned by the caller and
 * only copied.
 *
 * State arrays hold the 8 conservative variables of the reference
 * (enums.h:17-34: rho, E, rho*u, rho*v, rho*w, Bx, By, Bz), ghost cells
 * included (ghost width 3), with face-centred magnetic field components
 * (U(i,j,k,IA) is Bx on the face at i-1/2).
 */
#ifndef PPKMHD_GB300_H
#define PPKMHD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MHD_ABI_VERSION 2

/* status codes */
#define MHD_OK 0
#define MHD_ERR_INVALID_ARG -1  /* bad pointer, size, enum value or unsupported option */
#define MHD_ERR_CUDA -2         /* a CUDA runtime call failed (message has the CUDA error) */
#define MHD_ERR_NO_DEVICE -3    /* no CUDA device / the CUDA kernels are missing */
#define MHD_ERR_NUMERIC -4      /* device status word: non-finite or non-positive state */
#define MHD_ERR_PARSE -5        /* .ini text rejected */
#define MHD_ERR_TOO_LARGE -6    /* request larger than a fixed limit */
#define MHD_FINISHED 1          /* mhd_step_noalloc: t >= tEnd, nothing was computed */

/* enums.h:136-143 (RiemannSolverType).  The MHD solver takes LLF, HLL and
 * HLLD; the hydro solver takes APPROX, LLF, HLLC and, in 2D, HLL (the
 * reference's 3D hydro dispatch has no HLL branch, RiemannSolvers.h:608-633) */
#define MHD_RIEMANN_APPROX 0
#define MHD_RIEMANN_LLF 1
#define MHD_RIEMANN_HLL 2
#define MHD_RIEMANN_HLLC 3
#define MHD_RIEMANN_HLLD 4

/* mhd_params::solver: [run] solver_name MHD_Muscl_2D/3D or Hydro_Muscl_2D/3D */
#define MHD_SOLVER_MHD_MUSCL 0
#define MHD_SOLVER_HYDRO_MUSCL 1

/* enums.h:105-112 (BoundaryConditionType) */
#define MHD_BC_REFLECTING 1 /* BC_DIRICHLET */
#define MHD_BC_OUTFLOW 2    /* BC_NEUMANN */
#define MHD_BC_PERIODIC 3   /* BC_PERIODIC */

/* arithmetic of the step */
#define MHD_FP64 64
#define MHD_FP32 32
/* FP64 only: MHD_FP_EXACT compiles without FMA contraction and keeps every
 * operation of the reference in its order, so results are bitwise equal to a
 * serial run of the reference built without FMA; MHD_FP_FAST lets the
 * compiler contract multiply-adds. */
#define MHD_FP_FAST 0
#define MHD_FP_EXACT 1

/* host array layouts */
#define MHD_LAYOUT_LEFT 0  /* [var][k][j][i], i fastest (Kokkos LayoutLeft, the CUDA build) */
#define MHD_LAYOUT_RIGHT 1 /* [i][j][k][var], var fastest (Kokkos LayoutRight, the OpenMP build) */

/* initial conditions: [hydro] problem (SolverMHDMuscl.h:649-710) and the
 * layout of mhd_params::problem_real / problem_int for each
 * (src/shared/problems/*Params.h, values float-rounded as ConfigMap reads
 * them) */
#define MHD_PROBLEM_ORSZAG_TANG 0      /* ot_kt */
#define MHD_PROBLEM_BLAST 1            /* real: radius, center_x, _y, _z, density_in, density_out,
                                          pressure_in, pressure_out */
#define MHD_PROBLEM_IMPLODE 2          /* real: outer rho, p, vx, vy, vz, Bx, By, Bz, then inner;
                                          int: shape_region */
#define MHD_PROBLEM_KELVIN_HELMHOLTZ 3 /* real: d_in, d_out, pressure, vflow_in, vflow_out,
                                          amplitude, w0, delta; int: perturbation_sine,
                                          perturbation_sine_robertson, mode */
#define MHD_PROBLEM_ROTOR 4            /* real: r0, r1, u0, p0, b0 */
#define MHD_PROBLEM_FIELD_LOOP 5       /* real: radius, density_in, amplitude, vflow */
#define MHD_PROBLEM_WAVE 6             /* real: amplitude, V0, rev[7], d0, p0, sin_a2, cos_a2,
                                          sin_a3, cos_a3, dby, dbz, bx0, by0, bz0, k_par
                                          (WaveParams.h); int: type */
/* hydro solver problems (SolverHydroMuscl.cpp:110-250; blast, implode and
 * kelvin_helmholtz take the layouts above; unknown names give implode) */
#define MHD_PROBLEM_GRESHO_VORTEX 7     /* real: rho0, Ma */
#define MHD_PROBLEM_FOUR_QUADRANT 8     /* real: x, y; int: config_number (2D) */
#define MHD_PROBLEM_ISENTROPIC_VORTEX 9 /* real: rho_a, T_a, u_a, v_a, center_x, center_y,
                                           strength (2D) */
#define MHD_PROBLEM_RAYLEIGH_TAYLOR 10  /* real: amplitude, d0, d1, gx, gy, gz */
#define MHD_PROBLEM_RISING_BUBBLE 11    /* real: R, x0, y0, z0, din, dout, gx, gy, gz */
#define MHD_PROBLEM_DISK 12             /* real: radius, radius_inner, xc, yc, zc, ref_density,
                                           contrast_density, contrast_width, ref_sound_speed,
                                           then the point source xs, ys, zs, G M, soften */

/*
 * Run/mesh/scheme parameters.  Mirrors the fields of HydroParams /
 * HydroSettings (src/shared/HydroParams.h:28-234) that the MHD MUSCL step
 * reads, plus SolverBase's tEnd/tCurrent (SolverBase.cpp:119-120).  Real
 * parameters are doubles; mhd_params_from_ini() rounds them through float as
 * ConfigMap::getFloat does (ConfigMap.cpp:38-46).
 */
typedef struct mhd_params
{
  int    dim;        /* 2 or 3 */
  int    nx, ny, nz; /* interior cells (nz ignored in 2D) */
  int    ghost;      /* ghost width, must be 3 */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double gamma0, cfl, slope_type, smallr, smallc;
  int    riemann;    /* MHD_RIEMANN_* */
  int    implementation_version; /* [OTHER] implementationVersion: 0, 1 or 2 */
  int    boundary[6];            /* xmin, xmax, ymin, ymax, zmin, zmax: MHD_BC_* */
  double tEnd, tCurrent;
  int    nStepmax;
  int    problem;    /* MHD_PROBLEM_* */
  double ot_kt;      /* [OrszagTang] kt */
  int    precision;  /* MHD_FP64 or MHD_FP32 */
  int    fp_mode;    /* MHD_FP_FAST or MHD_FP_EXACT */
  int    device;     /* CUDA device ordinal the context binds (default 0) */
  double problem_real[24]; /* per-problem parameters, see MHD_PROBLEM_* */
  int    problem_int[4];
  int    solver;     /* MHD_SOLVER_MHD_MUSCL (default) or MHD_SOLVER_HYDRO_MUSCL */
  int    gravity;    /* hydro solver: 0 off, 1 [gravity] static, 2 [gravity] point
                        (SolverBase.cpp:138-141; either switches gravity on) */
  double gravity_field[3]; /* hydro solver: the uniform static field the problem's
                              initialisation sets (zero for problems that set none;
                              the disk sets the point-source field instead) */
} mhd_params;

typedef struct mhd_ctx mhd_ctx;

/* Fill defaults: HydroParams()/HydroSettings() constructors (HydroParams.h:41-58,
 * :156-204), with the MHD solver's 3 ghost cells.  The hydro-only solver
 * (solver = MHD_SOLVER_HYDRO_MUSCL, SolverHydroMuscl<dim>) uses 2 ghost cells
 * and state arrays of dim + 2 variables (rho, E, rho u, rho v[, rho w]);
 * every entry point below serves both solvers unless it says otherwise. */
int mhd_params_default(mhd_params *p);

/* Parse .ini text with the reference's rules: INIReader (lower-cased
 * "section.name" keys, inline ';' comments, continuation lines),
 * ConfigMap::getFloat (strtof, float-rounded), getInteger (strtol base 0), and
 * HydroParams::setup (HydroParams.cpp:27-217).  Replaces
 * broadcast_parameters() + HydroParams::setup() (main.cpp:133-137). */
int mhd_params_from_ini(const char *ini_text, mhd_params *p, char *err, size_t errlen);

/* Allocate device buffers for one problem and set up the stream.
 * Replaces the allocations of SolverMHDMuscl<dim>::SolverMHDMuscl
 * (SolverMHDMuscl.h:211-387).  The state is zero until mhd_init_problem or
 * mhd_set_state.
 * MHD_FP32 with implementation version 2 keeps the device state compensated:
 * next to the float state the context holds its low parts (8 more float
 * planes, to about 48 significant bits together), each iteration adds its
 * FP32 increment to the pair without rounding loss, and the momentum fluxes
 * are computed and stored relative to one constant total pressure per
 * iteration.  The arithmetic stays FP32; what no longer accumulates is the
 * rounding of the state itself.  mhd_get_state returns the float state (the
 * pair rounded once); a state set from the host (mhd_set_state,
 * mhd_step_host) starts with zero low parts; checkpoints carry them
 * (format 2). */
int mhd_create(const mhd_params *p, mhd_ctx **ctx);
int mhd_destroy(mhd_ctx *ctx);

/* Initial condition + boundaries + U2 = U + primitives + dt, i.e. the tail of
 * the solver constructor (SolverMHDMuscl.h:390-402). */
int mhd_init_problem(mhd_ctx *ctx);

/* The initial condition of p->problem alone, computed on the host in FP64
 * (no device needed): U receives the ghost-inclusive LayoutLeft state that
 * the reference's init functor writes, before any boundary fill. */
int mhd_initial_state(const mhd_params *p, double *U);

/* Inject a full ghost-inclusive state (real_bytes 8 or 4, matching the
 * context precision) and redo boundaries, primitives and dt; resets the
 * iteration count to 0 and t to tCurrent. */
int mhd_set_state(mhd_ctx *ctx, const void *U, int layout, int real_bytes);

/* Copy out the current solution (the array the next step reads: U when the
 * iteration count is even, U2 otherwise -- SolverMHDMuscl.h:791-805). */
int mhd_get_state(mhd_ctx *ctx, void *U, int layout, int real_bytes);

/* One SolverBase::next_iteration (SolverBase.cpp:205-220) = one
 * godunov_unsplit (SolverMHDMuscl.h:791-805, .cpp:373-572): boundaries,
 * primitives, CFL dt (clipped to tEnd), slopes, half step, edge fields, HLLD
 * face fluxes, CT edge EMFs and the update; then iteration += 1, t += dt.
 * Does nothing when finished() holds.  Asynchronous (dt stays on device). */
int mhd_step(mhd_ctx *ctx);

/* SolverBase::compute_dt (SolverBase.cpp:148-179): the CFL time step of the
 * current state, clipped to tEnd — the dt the next mhd_step will take.  The
 * state, t and the iteration count are unchanged.  Synchronises the stream. */
int mhd_compute_dt(mhd_ctx *ctx, double *dt);

/* godunov_unsplit(dt) with the caller's dt (dt > 0, not clipped), then
 * t += dt and iteration += 1; mhd_step is mhd_compute_dt followed by this
 * with the CFL dt.  Does nothing when finished() holds.  Asynchronous. */
int mhd_step_dt(mhd_ctx *ctx, double dt);

/* Up to nsteps iterations of main.cpp:154-159 from a CUDA graph, stopping
 * (on device) when t >= tEnd - 1e-14 or iteration >= nStepmax.  Returns after
 * the stream is synchronised; *done = iterations executed. */
int mhd_run(mhd_ctx *ctx, int nsteps, int *done);

/* godunov_unsplit_impl(data_in, data_out) on HOST arrays: copy U_in to the
 * device, run one iteration, copy the result back.  The state inside the
 * context is replaced by U_in first, so t/dt bookkeeping continues.  With
 * MHD_LAYOUT_LEFT and implementation version 2 the copies overlap the step
 * in slabs along the slowest axis: each uploaded slab gets its ghost fill,
 * primitives, slopes and edge field while the next one arrives, and each
 * finished slab of U_out is copied back while the next one's edges compute
 * (same result, bitwise).  Pinned host buffers make the copies asynchronous. */
int mhd_step_host(mhd_ctx *ctx, const void *U_in, void *U_out, int layout, int real_bytes);

/* Slab count of mhd_step_host: 0 (default) = one slab per 64 MiB of state,
 * at most 16; 1 = no overlap; never more than the grid's planes or 16.
 * No counterpart in the reference, which copies no state per step. */
int mhd_set_host_slabs(mhd_ctx *ctx, int nslabs);

/* The form of an iteration.  MHD_FORM_FUSED: the plain form fused into one
 * tile kernel per iteration after the CFL reduction: each block loads a tile
 * of the state with two halo layers and computes primitives, slopes (and
 * half step, edge field), face fluxes (and edge EMFs) and the update in
 * shared memory, writing only the new state to HBM (hydro solver: k_hdt +
 * k_hfused; MHD solver, 2D implementation version 2 without the flux
 * surrogate: k_dt_only + k_mfused2d).  MHD_FORM_STAGES: the stage kernels,
 * which keep the intermediates in HBM.  Both give the same state bit for bit
 * in the MHD_FP_EXACT build; the FMA builds contract each kernel's
 * expressions independently (round-off differences).  Without this call a
 * context runs the form its configuration maps to (the faster one on GB300
 * for that configuration: fused for 2D FP32, stages otherwise), so the same
 * configuration always runs the same kernels.  MHD_FORM_TIMED: the next
 * stepping call times one iteration of each form on the current state and
 * keeps the faster.  MHD_FORM_FUSED where the configuration has no fused
 * form returns MHD_ERR_INVALID_ARG.  mhd_get_fused: 1 when the fused form
 * runs. */
#define MHD_FORM_STAGES 0
#define MHD_FORM_FUSED 1
#define MHD_FORM_TIMED 2
int mhd_set_fused(mhd_ctx *ctx, int fused);
int mhd_get_fused(mhd_ctx *ctx, int *fused);

/* t, the dt of the last computed CFL condition, and the iteration count
 * (SolverBase m_t, m_dt, m_iteration).  Synchronises the stream. */
int mhd_time(mhd_ctx *ctx, double *t, double *dt, int *iteration);

/* FP64 diagnostics of the current state over interior cells: sums[8] of the
 * conservative variables (cell-centred B for the field components), and the
 * L1 / max norms of the discrete divergence of the face-centred field. */
int mhd_diagnostics(mhd_ctx *ctx, double sums[8], double *divb_l1, double *divb_max);

/* Device-resident stepping for timing: run nsteps iterations (no early stop
 * check on the host) and return the elapsed device time measured with CUDA
 * events on the context's stream. */
int mhd_run_timed(mhd_ctx *ctx, int nsteps, float *ms);

/* Time each kernel of one iteration separately (CUDA events around every
 * launch, on the context's stream).  names/ms receive up to max entries;
 * *count = number of kernels in an iteration. */
int mhd_profile_step(mhd_ctx *ctx, const char **names, float *ms, int max, int *count);

/* Cells updated per iteration (interior) and per the reference's own count
 * (ghost cells included, SolverMHDMuscl.h:256 + solver_utils.h:55-56). */
int mhd_cell_counts(mhd_ctx *ctx, int64_t *interior, int64_t *with_ghosts);

/* Sizes of the ghost-inclusive arrays: isize, jsize, ksize (1 in 2D), nbvar. */
int mhd_sizes(mhd_ctx *ctx, int sizes[4]);

/* Number of kernel launches one iteration makes. */
int mhd_launches_per_step(mhd_ctx *ctx, int *n);

const char *mhd_last_error(mhd_ctx *ctx);
const char *mhd_version(void);

/*
 * Ensembles: many independent problems of uneven size advanced together.
 * The reference runs such problems one at a time, each through its own
 * solver object (main.cpp:133-159 per .ini); here one context holds them
 * all, and every kernel launch of an iteration covers every problem, each
 * with its own CFL dt, time and stopping rule (SolverBase::finished), with
 * whole runs replayed from CUDA graphs.  Each problem is exactly the
 * single-problem iteration above (implementation version 2): results are
 * bitwise those of separate mhd_ctx runs of the same parameters.
 */
typedef struct mhd_ensemble mhd_ensemble;

/* p[0..n-1]: one parameter set per problem; all share dim, precision,
 * fp_mode and device, and use implementation version 2.  States start at
 * zero until mhd_ensemble_init_problem / mhd_ensemble_set_state.  On a
 * parameter error *ens is still set, so mhd_ensemble_last_error can report. */
int mhd_ensemble_create(const mhd_params *p, int n, mhd_ensemble **ens);
int mhd_ensemble_destroy(mhd_ensemble *ens);

/* Orszag-Tang initial condition of problem `prob`, then boundaries,
 * primitives and dt (as mhd_init_problem). */
int mhd_ensemble_init_problem(mhd_ensemble *ens, int prob);

/* As mhd_set_state / mhd_get_state, for problem `prob`. */
int mhd_ensemble_set_state(mhd_ensemble *ens, int prob, const void *U, int layout, int real_bytes);
int mhd_ensemble_get_state(mhd_ensemble *ens, int prob, void *U, int layout, int real_bytes);

/* Every problem at once: U[p] is problem p's array (n pointers, one layout
 * and precision for all).  The copies and per-problem set-up are queued
 * together and the stream is synchronised once per call, where the
 * per-problem calls synchronise once per problem. */
int mhd_ensemble_set_states(mhd_ensemble *ens, const void *const *U, int layout, int real_bytes);
int mhd_ensemble_get_states(mhd_ensemble *ens, void *const *U, int layout, int real_bytes);

/* nsteps iterations of every problem that is not finished (problems stop
 * on device at their own tEnd / nStepmax); *ms = elapsed device time (CUDA
 * events on the ensemble's stream; may be NULL).  All problems must be at
 * iterations of the same parity (true after set_state/init of each). */
int mhd_ensemble_run(mhd_ensemble *ens, int nsteps, float *ms);

int mhd_ensemble_time(mhd_ensemble *ens, int prob, double *t, double *dt, int *iteration);
int mhd_ensemble_diagnostics(mhd_ensemble *ens, int prob, double sums[8], double *divb_l1,
                             double *divb_max);

/* Pick the threads per block of every batched kernel by timing candidates
 * on the current states, then the form (graphs, persistent and, in 2D,
 * fused: two timed iterations of each); every trial starts from a snapshot
 * of the states taken first and restored at the end, so results are
 * unchanged; report = one line per candidate (may be NULL). */
int mhd_ensemble_autotune(mhd_ensemble *ens, char *report, size_t report_len);

/* The form mhd_ensemble_run takes (the ensemble has no counterpart in the
 * reference).  MHD_ENSEMBLE_GRAPHS: the eight per-stage launches of an
 * iteration, each over all problems, replayed from CUDA graphs (the
 * default, except for 2D FP32 ensembles).  MHD_ENSEMBLE_PERSISTENT: the
 * whole run in one cooperative launch of as many blocks as are resident,
 * the stages of every iteration separated by grid-wide barriers; same kernel
 * bodies, same states bit for bit.  MHD_ENSEMBLE_FUSED (2D only; the default
 * of 2D FP32 ensembles): the fused tile form of mhd_set_fused over all
 * problems, five launches per iteration replayed from CUDA graphs, the same
 * states bit for bit in the MHD_FP_EXACT build.  mhd_ensemble_autotune times
 * the forms on the current states and keeps the fastest. */
#define MHD_ENSEMBLE_GRAPHS 0
#define MHD_ENSEMBLE_PERSISTENT 1
#define MHD_ENSEMBLE_FUSED 2
int mhd_ensemble_set_mode(mhd_ensemble *ens, int mode);
int mhd_ensemble_get_mode(mhd_ensemble *ens, int *mode);

/* Bound, in clock cycles, of every grid-barrier wait of the persistent form
 * (default 2^34).  A wait that runs out stops the launch early: the run
 * returns MHD_ERR_CUDA, the states of that run are incomplete (set them
 * again) and the ensemble stays usable.  0 makes every wait give up at once:
 * the way to exercise that path. */
int mhd_ensemble_set_wait_limit(mhd_ensemble *ens, long long cycles);

/* As mhd_profile_step, for one iteration of the whole ensemble. */
int mhd_ensemble_profile_step(mhd_ensemble *ens, const char **names, float *ms, int max,
                              int *count);

/* Interior cells over all problems (cell-updates per ensemble iteration). */
int mhd_ensemble_cell_count(mhd_ensemble *ens, int64_t *interior);
int mhd_ensemble_launches_per_step(mhd_ensemble *ens, int *n);
const char *mhd_ensemble_last_error(mhd_ensemble *ens);

/*
 * Checkpoint / restart.  The reference restarts from its HDF5 output
 * ([run] restart_enabled, restart_filename, restart_reset_totaltime;
 * SolverMHDMuscl<dim>::init_restart, SolverMHDMuscl.h:613-643), which drops
 * the magnetic field (the HDF5 writers pass 4 or 5 variables,
 * IO_ReadWrite.cpp:102-106, :150-154).  Here a checkpoint is one binary file:
 *   char magic[8] = "PPKMHDCK"; uint32 format = 1 or 2, dim, nx, ny, nz,
 *   ghost, nbvar = 8, real_bytes; double t, dt; int64 iteration; int32
 *   times_saved, pad; double xmin, xmax, ymin, ymax, zmin, zmax, gamma0;
 * followed by the ghost-inclusive state, LayoutLeft, in the context's
 * precision (all fields little-endian); format 2 (FP32, implementation
 * version 2) then holds the same number of floats again: the low parts of
 * the compensated FP32 state (see mhd_create).  Loading restores the state and t
 * (0 with reset_time, as restart_reset_totaltime); the iteration count
 * restarts at 0 as in the reference.  Continuing from a checkpoint is
 * bitwise equal to the uninterrupted run.
 */
/* VTK ImageData output of a host state (save_VTK_2D / save_VTK_3D,
 * src/utils/io/IO_VTK.cpp:24-209, :212-410 of the reference): interior cells,
 * one cell-data array per variable named as SolverBase does (rho, energy,
 * rho_vx, rho_vy, rho_vz, bx, by, bz), raw appended binary with a UInt64 byte
 * count before each array (or ASCII with [output] outputVtkAscii), written to
 * [output] outputDir/outputPrefix_NNNNNNN.vti for the mesh of ini_text.
 * U: ghost-inclusive LayoutLeft FP64 state.  The file name is copied to path
 * (pathlen bytes, may be NULL).  Host only: needs no device. */
int mhd_write_vtk(const char *ini_text, const double *U, int iStep, char *path, size_t pathlen);

int mhd_checkpoint_save(mhd_ctx *ctx, const char *path, int times_saved);
int mhd_checkpoint_load(mhd_ctx *ctx, const char *path, int reset_time, int *times_saved);
/* [run] restart_upscale (copy_buffer of the HDF5 restart reader, IO_HDF5.h:
 * 1603-1694): load a checkpoint of half the context's resolution (nx/2,
 * ny/2[, nz/2]; nx, ny, nz even).  Fine cell i (ghost-inclusive) takes coarse
 * cell (i + g) / 2 along every axis; the face-centred normal field takes the
 * coarse face value where i + g is even and the mean of the two coarse faces
 * around it otherwise, which keeps the discrete div B at zero.  A format-2
 * file's low parts are not carried over. */
int mhd_checkpoint_load_upscaled(mhd_ctx *ctx, const char *path, int reset_time, int *times_saved);

/*
 * HLLD flux surrogate.  The reference has no learned component; this is the
 * GB300 build's FP32 option for the face-flux stage (riemann_hlld,
 * RiemannSolvers_MHD.h:133-367, at the call site of
 * ComputeFluxAndUpdateAlongDirFunctor, MHDRunFunctors{2D,3D}.h).
 *
 * A 27-64-64-19 perceptron (GELU, BF16 weights, FP32 accumulation) predicts
 * the upwind dissipation D = (F(qL) + F(qR))/2 - F_HLLD of a face in the
 * face's own dimensionless units, odd in each transverse direction by
 * construction (reflection-invariant inputs; the odd components are the
 * network's coefficients times odd bases); it is used on faces whose largest
 * normalised half-jump J is at most tau, whose reconstructed density and
 * pressure are above their floors and whose prediction is finite and
 * bounded; every other face gets HLLD.  Training runs on the GPU with the
 * library's own forward/backward kernels.
 */
#define MHD_MLP_PARAMS 7832      /* W1[32][64] b1[64] W2[64][64] b2[64] W3[64][24] b3[24] */
#define MHD_MLP_FEATURES 40      /* per face: 32 network inputs, then the 8 odd bases */
#define MHD_SAMPLE_FLOATS 24     /* one harvested face record, see mhd_harvest_faces */
#define MHD_MLP_TRAIN 0          /* BF16 weights/activations, hardware tanh (deployed numerics) */
#define MHD_MLP_CHECK 1          /* plain FP32, tanhf: for gradient checks */

typedef struct mhd_mlp mhd_mlp;

/* Face samples of the context's next iteration (boundaries, primitives, dt
 * and trace are computed; the state is not advanced): one record per
 * stride-th face of each direction, records[q * MHD_SAMPLE_FLOATS + ...] =
 * qL[7], qR[7] (rho, vn, vt1, vt2, p, Bt1, Bt2 in the face-normal frame), a
 * (normal B), J (sensor value), D[7] (FP64 central flux minus FP64 HLLD of
 * the same states: rho, E, mn, mt1, mt2, Bt1, Bt2), gamma0.  With
 * records == NULL only *count is set. */
int mhd_harvest_faces(mhd_ctx *ctx, int stride, float *records, int64_t capacity,
                      int64_t *count);

/* A network with Glorot-uniform weights from `seed`, for adiabatic index gamma0. */
int mhd_mlp_create(uint64_t seed, double gamma0, mhd_mlp **mlp);
int mhd_mlp_destroy(mhd_mlp *mlp);
int mhd_mlp_set_params(mhd_mlp *mlp, const float *params, int n);
int mhd_mlp_get_params(mhd_mlp *mlp, float *params, int n);
int mhd_mlp_gamma(mhd_mlp *mlp, double *gamma0);

/* Records -> features[n][MHD_MLP_FEATURES] and targets[n][8] (D / scale:
 * rho, E, mn, mt1, mt2, Bt1, Bt2, pad; FP64 on the GPU). */
int mhd_mlp_encode(mhd_mlp *mlp, const float *records, int64_t n, float *features,
                   float *targets);

/* Gradient of the mean squared error (over n samples and the 7 used
 * outputs) with respect to the MHD_MLP_PARAMS parameters; *loss = the error. */
int mhd_mlp_gradient(mhd_mlp *mlp, const float *features, const float *targets, int64_t n,
                     int mode, float *grad, double *loss);

/* Adam on the harvested records (seeded shuffles, cosine learning-rate
 * decay to lr/20); each sample's squared error is weighted by
 * (sJ / 0.1)^weight_power (sJ = max(J, 1e-4); 0 = unweighted);
 * loss_history[epochs] = mean batch loss (may be NULL). */
int mhd_mlp_train(mhd_mlp *mlp, const float *records, int64_t n, int epochs, int batch,
                  float lr, float weight_power, uint64_t seed, float *loss_history);

/* Batch forward pass on features[n][MHD_MLP_FEATURES] -> out[n][8] (the 7
 * dimensionless dissipation components and a pad), on the 5th-generation
 * tensor cores (tcgen05, FP32 accumulators in TMEM) with the deployed
 * numerics: BF16 weights and activations, FP32 accumulation, BF16 GELU. */
int mhd_mlp_forward(mhd_mlp *mlp, const float *features, int64_t n, float *out);

/* Bound (number of polls, >= 0; default MHD_MLP_WAIT_POLLS) of each wait of
 * mhd_mlp_forward for a tensor-core completion.  A wait that reaches it makes
 * the call return MHD_ERR_CUDA after the pending work has drained (with the
 * default bound); the network and the device stay usable.  0 makes every
 * wait give up at once: the way to exercise that error path. */
#define MHD_MLP_WAIT_POLLS (1 << 20)
int mhd_mlp_set_wait_limit(mhd_mlp *mlp, int polls);

/* Kernel form of mhd_mlp_forward (both give bitwise the same outputs):
 * MHD_MLP_FORWARD_PERSISTENT (the default) keeps SMs x resident blocks of
 * two 128-row pipelines each, the network staged once per block, one
 * pipeline's MMAs running while the other's rows go through the epilogue;
 * MHD_MLP_FORWARD_TILES launches one 128-thread block per 128-row tile. */
#define MHD_MLP_FORWARD_TILES 0
#define MHD_MLP_FORWARD_PERSISTENT 1
int mhd_mlp_set_forward_form(mhd_mlp *mlp, int form);
/* Device time (CUDA events around the launch, ms) of the last
 * mhd_mlp_forward kernel; -1 before the first. */
int mhd_mlp_last_forward_ms(mhd_mlp *mlp, double *ms);
const char *mhd_mlp_last_error(mhd_mlp *mlp);

/* Use the network in the flux stage of an FP32, version-2, HLLD context
 * (mlp == NULL: back to HLLD everywhere).  The network's gamma0 must match
 * the context's.  tau: sensor threshold on J (0 < tau <= 0.1). */
int mhd_set_surrogate(mhd_ctx *ctx, const mhd_mlp *mlp, double tau);

/* Faces given by the network and faces computed since the surrogate was
 * set or the last reset (reset != 0 clears the counters). */
int mhd_surrogate_stats(mhd_ctx *ctx, int64_t *faces_network, int64_t *faces_total, int reset);

/* Device scratch reserved by mhd_step_noalloc on every GPU that loads this
 * library, for the process lifetime. */
#define MHD_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)

/*
 * One iteration that allocates nothing.  This entry point has no counterpart
 * in the reference; it is for callers that cannot call cudaMalloc (a host
 * that owns all device memory through its own pool, a latency-bounded loop
 * where an allocation may stall or fail, a job that must keep a fixed device
 * footprint after start-up).
 *
 * U_in and U_out are the caller's DEVICE arrays on GPU p->device
 * (LayoutLeft, ghost cells included, real type per p->precision).  U_in is
 * written too: its ghost cells are refilled in place, as the reference's
 * make_boundaries(data_in) does; its interior is only read.  Every
 * intermediate lives in a file-scope __device__ array of
 * MHD_NOALLOC_SCRATCH_BYTES, cleared by each call (cudaMemsetAsync, no
 * allocation); grids that need more return MHD_ERR_TOO_LARGE (32 MiB holds
 * about 280^2 interior cells in 2D or 33^3 in 3D in FP64, twice as many in
 * FP32).  t is the current time and dt is clipped to p->tEnd.  When
 * t >= tEnd - 1e-14 the call returns MHD_FINISHED with *dt = 0 and U_out
 * untouched (no GPU work).  Otherwise, on MHD_OK, *dt holds the dt of the
 * iteration and U_out the new state; the call synchronises `stream` (a
 * cudaStream_t of p->device, NULL for the legacy default stream).  The
 * kernels run on p->device; the calling thread's current device is restored
 * before the call returns.  Only MHD_FP_FAST and implementation version 2
 * are accepted.
 * The first call on a device looks up the scratch array's device address
 * (cudaGetSymbolAddress) and keeps it for the process; make that call before
 * any stream capture.  Calls after a cudaDeviceReset of that device are not
 * supported (the address goes stale).  All calls share the array: calls that
 * overlap on the GPU race and must be serialised.  Errors are reported by
 * the status code only (no context exists).
 */
int mhd_step_noalloc(const mhd_params *p, void *U_in, void *U_out, double t, double *dt,
                     void *stream);

#ifdef __cplusplus
}
#endif
#endif /* PPKMHD_GB300_H */
