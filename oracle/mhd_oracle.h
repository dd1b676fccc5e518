/*
 * CPU oracle for the ppkMHD MUSCL-Hancock + HLLD + constrained-transport MHD
 * step (implementation version 2, 2D and 3D, FP64).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm, used (a) by tests/ as the parity checker for the CUDA kernels,
 * (b) by bench.py as the timed CPU baseline ("port").  It is never linked into
 * or called by the product library.
 *
 * Every function cites the reference file:line it restates.  Floating-point
 * expressions keep the reference's operation order, and the atomic face/edge
 * updates of the reference are replayed as a deterministic gather in the order
 * a serial execution of the reference applies them, so that the oracle is
 * bitwise equal to the reference built without FMA contraction
 * (oracle/_ref, see tests/test_oracle_pinning.py).
 *
 * Array layout ("LayoutLeft", the layout Kokkos uses on CUDA):
 *   U[i + isize*(j + jsize*(k + ksize*var))], ghost cells included.
 */
#ifndef PPKMHD_ORACLE_H
#define PPKMHD_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_ID = 0, ORC_IP = 1, ORC_IU = 2, ORC_IV = 3, ORC_IW = 4, ORC_IA = 5, ORC_IB = 6, ORC_IC = 7 };
/* src/shared/enums.h:94-101 (RiemannSolverType) and :105-112 (BoundaryConditionType) */
enum { ORC_RIEMANN_APPROX = 0, ORC_RIEMANN_LLF = 1, ORC_RIEMANN_HLL = 2, ORC_RIEMANN_HLLC = 3, ORC_RIEMANN_HLLD = 4 };
enum { ORC_BC_UNDEFINED = 0, ORC_BC_DIRICHLET = 1, ORC_BC_NEUMANN = 2, ORC_BC_PERIODIC = 3 };

typedef struct orc_params
{
  int    dim;                 /* 2 or 3 */
  int    nx, ny, nz, ghost;   /* interior sizes, ghost width (3 for MHD) */
  int    isize, jsize, ksize; /* ghost-inclusive sizes (ksize = 1 in 2D) */
  double xmin, xmax, ymin, ymax, zmin, zmax;
  double dx, dy, dz;
  double gamma0, cfl, slope_type, smallr, smallc, smallp, cIso;
  int    riemann;             /* ORC_RIEMANN_* */
  int    version;             /* implementationVersion */
  int    bc[6];               /* xmin, xmax, ymin, ymax, zmin, zmax */
  double tEnd, tCurrent;
  int    nStepmax;
  double ot_kt;               /* [OrszagTang] kt */
  int    problem_is_ot;       /* 1 when [hydro] problem = orszag_tang */
} orc_params;

/* INI text -> parameters, with the reference's parsing rules. Returns 0 on success. */
int orc_params_from_ini(const char *ini_text, orc_params *p);

/* Orszag-Tang initial condition into U (LayoutLeft, ghosts included). */
void orc_init_orszag_tang(const orc_params *p, double *U);

/* Ghost-cell fill (periodic / reflecting / outflow), X then Y then Z faces. */
void orc_make_boundaries(const orc_params *p, double *U);

typedef struct orc_solver orc_solver;

orc_solver *orc_create(const orc_params *p, int nthreads);
void        orc_destroy(orc_solver *s);
/* Inject U (LayoutLeft), then boundaries, U2 = U, primitives, dt (as the reference constructor does). */
void orc_set_state(orc_solver *s, const double *U);
/* Current solution (the array the next step reads). */
void orc_get_state(const orc_solver *s, double *U);
/* Run up to n iterations of the main loop; returns the number executed. */
int  orc_run(orc_solver *s, int n);
void orc_time(const orc_solver *s, double *t, double *dt, int *iteration);
/* Test hook: move every later dt up by `ulps` ulps (0: the reference's dt). */
void orc_set_dt_ulps(orc_solver *s, int ulps);
int64_t orc_nelem(const orc_params *p);

/* Function-level probes (normal-frame 8-component states). */
void   orc_riemann(const orc_params *p, const double *qL, const double *qR, double *flux);
/* qEdge: 4 states ordered RT, RB, LT, LB; emf_dir: 0 = EMFX, 1 = EMFY, 2 = EMFZ */
double orc_compute_emf(const orc_params *p, int emf_dir, const double *qEdge);

#ifdef __cplusplus
}
#endif
#endif
