/*
 * CPU oracle for ppkMHD's hydro-only MUSCL-Hancock solver
 * (SolverHydroMuscl<dim>, Hydro_Muscl_2D / Hydro_Muscl_3D), FP64.
 *
 * TEST INFRASTRUCTURE ONLY.  A plain-C restatement of the reference
 * algorithm, used by tests/ as the parity checker of the CUDA kernels and by
 * bench.py as the timed CPU baseline of the hydro workload.  The product
 * library never links or calls it.
 *
 * Every function cites the reference file:line it restates and keeps the
 * reference's operation order, so the oracle is bitwise equal to the
 * reference built without FMA contraction (oracle/_ref, checked by
 * tests/test_hydro_oracle.py).  It restates implementation version 0
 * (ComputeAndStoreFluxes + Update).  Version 1 (stored slopes, per-direction
 * trace, flux and update) computes every face flux from the same slopes and
 * traces and applies the same additions in the same order, so the same code
 * serves it, with its one difference: in 3D with gravity its z faces' right
 * states get no gravity predictor.
 *
 * Array layout ("LayoutLeft"): U[i + isize*(j + jsize*(k + ksize*var))],
 * ghost cells included (ghost width 2), 4 variables in 2D (rho, E, rho u,
 * rho v), 5 in 3D (+ rho w).
 */
#ifndef PPKMHD_HYDRO_ORACLE_H
#define PPKMHD_HYDRO_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* src/shared/enums.h:136-143 (RiemannSolverType) */
enum { HORC_APPROX = 0, HORC_LLF = 1, HORC_HLL = 2, HORC_HLLC = 3 };

typedef struct horc_params
{
  int    dim, nx, ny, nz, ghost, nvar;
  int    isize, jsize, ksize;
  double xmin, xmax, ymin, ymax, zmin, zmax, dx, dy, dz;
  double gamma0, gamma6, cfl, slope_type, smallr, smallc, smallp, smallpp;
  int    riemann, version, bc[6];
  double tEnd, tCurrent;
  int    nStepmax;
  int    gravity;    /* [gravity] static or point */
  double grav[3];    /* the uniform field the problem's init sets (0 otherwise) */
  int    point;      /* the disk problem: the point-source field instead */
  double xs, ys, zs, GM, eps; /* [gravity] x, y, z, G * M, soften */
  double xc, yc, zc;          /* [disk] centre (the field is evaluated relative to it) */
} horc_params;

/* INI text -> parameters (HydroParams::setup + init, SolverBase's gravity
 * keys).  Returns 0, or -1 when the solver is not Hydro_Muscl_2D/3D. */
int     horc_params_from_ini(const char *ini_text, horc_params *p);
int64_t horc_nelem(const horc_params *p);
/* The gravity field the problem's initialisation writes (dim planes,
 * LayoutLeft, ghosts included; zero for problems that write none). */
void horc_gravity_field(const horc_params *p, double *g);

typedef struct horc_solver horc_solver;
horc_solver *horc_create(const horc_params *p, int nthreads);
void         horc_destroy(horc_solver *s);
/* U (LayoutLeft) as the initial condition, then what the constructor does
 * after init: boundaries, U2 = U, dt. */
void horc_set_state(horc_solver *s, const double *U);
void horc_get_state(const horc_solver *s, double *U);
/* up to n iterations of the main loop (stops when finished); returns the count */
int  horc_run(horc_solver *s, int n);
void horc_time(const horc_solver *s, double *t, double *dt, int *iteration);

/* One Riemann problem (nvar-component primitive states rho, p, u, v[, w]). */
void horc_riemann(const horc_params *p, const double *qL, const double *qR, double *flux);

#ifdef __cplusplus
}
#endif
#endif
