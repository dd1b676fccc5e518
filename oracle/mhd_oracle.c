/*
 * CPU oracle: plain-C restatement of ppkMHD's MUSCL-Hancock + HLLD + CT MHD
 * step (implementation version 2), 2D and 3D, FP64.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU baseline).
 * The product library never links or calls this file.
 *
 * Reference files restated (paths relative to the ppkMHD source tree):
 *   src/utils/config/ConfigMap.cpp, src/utils/config/inih/{ini,INIReader}.cpp
 *   src/shared/HydroParams.cpp, src/shared/SolverBase.cpp
 *   src/shared/mhd_utils.h, src/shared/RiemannSolvers_MHD.h
 *   src/shared/BoundariesFunctors.h
 *   src/muscl/MHDBaseFunctor{2D,3D}.h, src/muscl/MHDRunFunctors{2D,3D}.h
 *   src/muscl/MHDInitFunctors{2D,3D}.h, src/muscl/SolverMHDMuscl.{h,cpp}
 *
 * Parity rules kept here: the operation order of every floating-point
 * expression is the reference's; the reference's atomic face/edge updates are
 * replayed as a gather in the order a serial run of the reference applies
 * them.  Compile with -ffp-contract=off.
 */
#include "mhd_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#  include <omp.h>
#endif

#define NV 8
enum { ID = 0, IP = 1, IU = 2, IV = 3, IW = 4, IA = 5, IB = 6, IC = 7 };

/* Stage markers of the FP64 operation counter (oracle/flop_count.cpp
 * compiles this file with a counting scalar type and defines ORC_STAGE);
 * no-ops in the oracle itself. */
#ifndef ORC_STAGE
#  define ORC_STAGE(s) ((void)0)
#endif
enum { STG_OTHER = 0, STG_PRIM, STG_DT, STG_SLOPES, STG_HALF, STG_EFIELD, STG_FACEB, STG_FLUX,
       STG_EMF, STG_UPDATE, STG_COUNT };

/* INI parsing with the reference's rules (inih + INIReader + ConfigMap) */
#include "ini_text.h"

/* HydroParams::setup (HydroParams.cpp:27-217) + init (:420-453) */
int
orc_params_from_ini(const char *ini_text, orc_params *p)
{
  ini_map m = { 0 };
  ini_parse_text(&m, ini_text);
  memset(p, 0, sizeof *p);

  const char *solver = ini_str(&m, "run", "solver_name", "unknown");
  if (!strcmp(solver, "MHD_Muscl_2D"))
    p->dim = 2;
  else if (!strcmp(solver, "MHD_Muscl_3D"))
    p->dim = 3;
  else
  {
    free(m.kv);
    return -1;
  }
  p->ghost = 3;
  p->nStepmax = (int)ini_int(&m, "run", "nstepmax", 1000);
  p->tEnd = (double)(float)ini_float(&m, "run", "tend", 0.0f);
  p->tCurrent = ini_float(&m, "run", "tCurrent", 0.0f);
  p->nx = (int)ini_int(&m, "mesh", "nx", 1);
  p->ny = (int)ini_int(&m, "mesh", "ny", 1);
  p->nz = (int)ini_int(&m, "mesh", "nz", 1);
  p->xmin = ini_float(&m, "mesh", "xmin", 0.0f);
  p->ymin = ini_float(&m, "mesh", "ymin", 0.0f);
  p->zmin = ini_float(&m, "mesh", "zmin", 0.0f);
  p->xmax = ini_float(&m, "mesh", "xmax", 1.0f);
  p->ymax = ini_float(&m, "mesh", "ymax", 1.0f);
  p->zmax = ini_float(&m, "mesh", "zmax", 1.0f);
  static const char *bcn[6] = { "boundary_type_xmin", "boundary_type_xmax", "boundary_type_ymin",
                                "boundary_type_ymax", "boundary_type_zmin", "boundary_type_zmax" };
  for (int f = 0; f < 6; ++f)
    p->bc[f] = (int)ini_int(&m, "mesh", bcn[f], ORC_BC_DIRICHLET);
  p->gamma0 = ini_float(&m, "hydro", "gamma0", 1.4f);
  p->cfl = ini_float(&m, "hydro", "cfl", 0.5f);
  p->slope_type = ini_float(&m, "hydro", "slope_type", 1.0f);
  p->smallc = ini_float(&m, "hydro", "smallc", 1e-10f);
  p->smallr = ini_float(&m, "hydro", "smallr", 1e-10f);
  p->cIso = 0.0; /* HydroSettings default; not read from the .ini */
  const char *rs = ini_str(&m, "hydro", "riemann", "approx");
  if (!strcmp(rs, "llf"))
    p->riemann = ORC_RIEMANN_LLF;
  else if (!strcmp(rs, "hll"))
    p->riemann = ORC_RIEMANN_HLL;
  else if (!strcmp(rs, "hllc"))
    p->riemann = ORC_RIEMANN_HLLC;
  else if (!strcmp(rs, "hlld"))
    p->riemann = ORC_RIEMANN_HLLD;
  else
    p->riemann = ORC_RIEMANN_APPROX;
  p->version = (int)ini_float(&m, "OTHER", "implementationVersion", 0.0f);
  if (p->version != 0 && p->version != 1 && p->version != 2)
    p->version = 0;
  const char *prob = ini_str(&m, "hydro", "problem", "unknown");
  p->problem_is_ot = !strcmp(prob, "orszag_tang");
  p->ot_kt = ini_float(&m, "OrszagTang", "kt", 0.0f);
  free(m.kv);

  /* HydroParams::init */
  p->isize = p->nx + 2 * p->ghost;
  p->jsize = p->ny + 2 * p->ghost;
  p->ksize = p->dim == 3 ? p->nz + 2 * p->ghost : 1;
  p->dx = (p->xmax - p->xmin) / p->nx;
  p->dy = (p->ymax - p->ymin) / p->ny;
  p->dz = (p->zmax - p->zmin) / p->nz;
  p->smallp = p->smallc * p->smallc / p->gamma0;
  return 0;
}

int64_t
orc_nelem(const orc_params *p)
{
  return (int64_t)p->isize * p->jsize * p->ksize * NV;
}

/* ====================================================================== */
/* indexing */
/* ====================================================================== */

typedef struct
{
  int64_t sj, sk, sv; /* strides of j, k, var (i stride = 1) */
} layout;

static inline layout
mk_layout(const orc_params *p)
{
  layout L;
  L.sj = p->isize;
  L.sk = (int64_t)p->isize * p->jsize;
  L.sv = L.sk * p->ksize;
  return L;
}

#define AT(L, i, j, k) ((int64_t)(i) + (int64_t)(j) * (L).sj + (int64_t)(k) * (L).sk)

/* ====================================================================== */
/* initial condition: MHDInitFunctors2D.h:241-389, MHDInitFunctors3D.h:264-415 */
/* ====================================================================== */

void
orc_init_orszag_tang(const orc_params *p, double *U)
{
  const layout L = mk_layout(p);
  const double TWOPI = 2 * 3.141592653589793238462643383279502884;
  const double gamma0 = p->gamma0;
  const int    g = p->ghost;
  if (p->dim == 2)
  {
    const double B0 = 1.0 / sqrt(2 * TWOPI);
    const double p0 = gamma0 / (2 * TWOPI);
    const double d0 = gamma0 * p0;
    const double v0 = 1.0;
    for (int j = 0; j < p->jsize; ++j)
      for (int i = 0; i < p->isize; ++i)
      {
        const double xPos = p->xmin + p->dx / 2 + (i - g) * p->dx;
        const double yPos = p->ymin + p->dy / 2 + (j - g) * p->dy;
        const int64_t c = AT(L, i, j, 0);
        U[c + ID * L.sv] = d0;
        U[c + IU * L.sv] = -d0 * v0 * sin(yPos * TWOPI);
        U[c + IV * L.sv] = d0 * v0 * sin(xPos * TWOPI);
        U[c + IW * L.sv] = 0.0;
        U[c + IA * L.sv] = -B0 * sin(yPos * TWOPI);
        U[c + IB * L.sv] = B0 * sin(2.0 * xPos * TWOPI);
        U[c + IC * L.sv] = 0.0;
      }
    const double TwoPi = 4.0 * asin(1.0);
    const double p0e = gamma0 / (2.0 * TwoPi);
    for (int j = 0; j < p->jsize - 1; ++j)
      for (int i = 0; i < p->isize - 1; ++i)
      {
        const int64_t c = AT(L, i, j, 0);
        const double  bxs = U[c + IA * L.sv] + U[c + 1 + IA * L.sv];
        const double  bys = U[c + IB * L.sv] + U[c + L.sj + IB * L.sv];
        U[c + IP * L.sv] = p0e / (gamma0 - 1.0) +
                           0.5 * (U[c + IU * L.sv] * U[c + IU * L.sv] / U[c + ID * L.sv] +
                                  U[c + IV * L.sv] * U[c + IV * L.sv] / U[c + ID * L.sv] +
                                  0.25 * (bxs * bxs) + 0.25 * (bys * bys));
      }
  }
  else
  {
    const double PI = 3.141592653589793238462643383279502884;
    const double B0 = 1.0 / sqrt(4 * PI);
    const double p0 = gamma0 / (4 * PI);
    const double d0 = gamma0 * p0;
    const double v0 = 1.0;
    const double kt = p->ot_kt;
    for (int k = 0; k < p->ksize; ++k)
      for (int j = 0; j < p->jsize; ++j)
        for (int i = 0; i < p->isize; ++i)
        {
          const double xPos = p->xmin + p->dx / 2 + (i - g) * p->dx;
          const double yPos = p->ymin + p->dy / 2 + (j - g) * p->dy;
          const double zPos = p->zmin + p->dz / 2 + (k - g) * p->dz;
          const double zfac = cos(2 * TWOPI * kt * (zPos - p->zmin) / (p->zmax - p->zmin));
          const int64_t c = AT(L, i, j, k);
          U[c + ID * L.sv] = d0;
          U[c + IU * L.sv] = -d0 * v0 * sin(yPos * TWOPI);
          U[c + IV * L.sv] = d0 * v0 * sin(xPos * TWOPI);
          U[c + IW * L.sv] = 0.0;
          U[c + IA * L.sv] = -B0 * zfac * sin(yPos * TWOPI);
          U[c + IB * L.sv] = B0 * zfac * sin(2.0 * xPos * TWOPI);
          U[c + IC * L.sv] = 0.0;
        }
    for (int k = 0; k < p->ksize; ++k)
      for (int j = 0; j < p->jsize - 1; ++j)
        for (int i = 0; i < p->isize - 1; ++i)
        {
          const int64_t c = AT(L, i, j, k);
          const double  bxs = U[c + IA * L.sv] + U[c + 1 + IA * L.sv];
          const double  bys = U[c + IB * L.sv] + U[c + L.sj + IB * L.sv];
          U[c + IP * L.sv] = p0 / (gamma0 - 1.0) +
                             0.5 * (U[c + IU * L.sv] * U[c + IU * L.sv] / U[c + ID * L.sv] +
                                    U[c + IV * L.sv] * U[c + IV * L.sv] / U[c + ID * L.sv] +
                                    0.25 * (bxs * bxs) + 0.25 * (bys * bys));
        }
  }
}

/* ====================================================================== */
/* boundaries: BoundariesFunctors.h:535-748 (2D), :750-1057 (3D);          */
/* SolverBase.cpp:513-537 (face order X, Y, Z)                             */
/* ====================================================================== */

/* Source index and sign for ghost index `c` along an axis of `n` interior
 * cells with ghost width g; `hi` selects the max face. */
static inline int
bc_src(int c, int n, int g, int type, int hi, int *flip)
{
  *flip = 0;
  if (!hi)
  {
    if (type == ORC_BC_DIRICHLET)
    {
      *flip = 1;
      return 2 * g - 1 - c;
    }
    if (type == ORC_BC_NEUMANN)
      return g;
    return n + c;
  }
  if (type == ORC_BC_DIRICHLET)
  {
    *flip = 1;
    return 2 * n + 2 * g - 1 - c;
  }
  if (type == ORC_BC_NEUMANN)
    return n + g - 1;
  return c - n;
}

void
orc_make_boundaries(const orc_params *p, double *U)
{
  const layout L = mk_layout(p);
  const int    g = p->ghost;
  const int    ks = p->ksize;
  /* X faces: normal velocity IU and normal field IA flip sign when reflecting */
  for (int face = 0; face < 2; ++face)
  {
    const int type = p->bc[face];
    for (int k = 0; k < ks; ++k)
      for (int j = 0; j < p->jsize; ++j)
        for (int q = 0; q < g; ++q)
        {
          const int i = face ? q + p->nx + g : q;
          int       flip;
          const int i0 = bc_src(i, p->nx, g, type, face, &flip);
          for (int v = 0; v < NV; ++v)
          {
            const double s = (flip && (v == IU || v == IA)) ? -1.0 : 1.0;
            U[AT(L, i, j, k) + v * L.sv] = U[AT(L, i0, j, k) + v * L.sv] * s;
          }
        }
  }
  for (int face = 2; face < 4; ++face)
  {
    const int type = p->bc[face];
    for (int k = 0; k < ks; ++k)
      for (int q = 0; q < g; ++q)
        for (int i = 0; i < p->isize; ++i)
        {
          const int j = face == 3 ? q + p->ny + g : q;
          int       flip;
          const int j0 = bc_src(j, p->ny, g, type, face == 3, &flip);
          for (int v = 0; v < NV; ++v)
          {
            const double s = (flip && (v == IV || v == IB)) ? -1.0 : 1.0;
            U[AT(L, i, j, k) + v * L.sv] = U[AT(L, i, j0, k) + v * L.sv] * s;
          }
        }
  }
  if (p->dim == 3)
    for (int face = 4; face < 6; ++face)
    {
      const int type = p->bc[face];
      for (int q = 0; q < g; ++q)
        for (int j = 0; j < p->jsize; ++j)
          for (int i = 0; i < p->isize; ++i)
          {
            const int k = face == 5 ? q + p->nz + g : q;
            int       flip;
            const int k0 = bc_src(k, p->nz, g, type, face == 5, &flip);
            for (int v = 0; v < NV; ++v)
            {
              const double s = (flip && (v == IW || v == IC)) ? -1.0 : 1.0;
              U[AT(L, i, j, k) + v * L.sv] = U[AT(L, i, j, k0) + v * L.sv] * s;
            }
          }
    }
}

/* ====================================================================== */
/* point-wise physics                                                      */
/* ====================================================================== */

/* mhd_utils.h:89-117, normal direction = slot IA of the state */
static inline double
fast_speed_x(const double *q, double gamma0)
{
  const double d = q[ID], pr = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const double b2 = a * a + b * b + c * c;
  const double c2 = gamma0 * pr / d;
  const double d2 = 0.5 * (b2 / d + c2);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
}

/* same, normal direction = slot IB */
static inline double
fast_speed_y(const double *q, double gamma0)
{
  const double d = q[ID], pr = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const double b2 = a * a + b * b + c * c;
  const double c2 = gamma0 * pr / d;
  const double d2 = 0.5 * (b2 / d + c2);
  return sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d));
}

/* mhd_utils.h:173-231 (cIso = 0) */
static void
mhd_flux_and_cons(const double *q, double *u, double *f, double gamma0)
{
  const double pr = q[IP];
  const double entho = 1.0 / (gamma0 - 1.0);
  const double d = q[ID], vu = q[IU], vv = q[IV], vw = q[IW], a = q[IA], b = q[IB], c = q[IC];
  const double ecin = 0.5 * (vu * vu + vv * vv + vw * vw) * d;
  const double emag = 0.5 * (a * a + b * b + c * c);
  const double etot = pr * entho + ecin + emag;
  const double ptot = pr + emag;
  u[ID] = d;
  u[IP] = etot;
  u[IU] = d * vu;
  u[IV] = d * vv;
  u[IW] = d * vw;
  u[IA] = a;
  u[IB] = b;
  u[IC] = c;
  f[ID] = d * vu;
  f[IP] = (etot + ptot) * vu - a * (a * vu + b * vv + c * vw);
  f[IU] = d * vu * vu - a * a + ptot;
  f[IV] = d * vu * vv - a * b;
  f[IW] = d * vu * vw - a * c;
  f[IA] = 0.0;
  f[IB] = b * vu - a * vv;
  f[IC] = c * vu - a * vw;
}

/* RiemannSolvers_MHD.h:27-67 */
static void
riemann_hll(double *ql, double *qr, double *flux, double gamma0)
{
  const double bx_mean = 0.5 * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  double ul[NV], fl[NV], ur[NV], fr[NV];
  mhd_flux_and_cons(ql, ul, fl, gamma0);
  mhd_flux_and_cons(qr, ur, fr, gamma0);
  const double cfl = fast_speed_x(ql, gamma0);
  const double cfr = fast_speed_x(qr, gamma0);
  const double vl = ql[IU], vr = qr[IU];
  const double sl = fmin(fmin(vl, vr) - fmax(cfl, cfr), 0.0);
  const double sr = fmax(fmax(vl, vr) + fmax(cfl, cfr), 0.0);
  for (int v = 0; v < NV; ++v)
    flux[v] = (sr * fl[v] - sl * fr[v] + sr * sl * (ur[v] - ul[v])) / (sr - sl);
}

/* mhd_utils.h:283-317 (x direction only) */
static inline double
info_speed_x(const double *q, double gamma0)
{
  const double d = q[ID], pr = q[IP], a = q[IA], b = q[IB], c = q[IC];
  const double b2 = a * a + b * b + c * c;
  const double c2 = gamma0 * pr / d;
  const double d2 = 0.5 * (b2 / d + c2);
  const double cf = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d));
  return cf + fabs(q[IU]);
}

/* RiemannSolvers_MHD.h:81-111 */
static void
riemann_llf(double *ql, double *qr, double *flux, double gamma0)
{
  const double bx_mean = 0.5 * (ql[IA] + qr[IA]);
  ql[IA] = bx_mean;
  qr[IA] = bx_mean;
  double ul[NV], fl[NV], ur[NV], fr[NV];
  mhd_flux_and_cons(ql, ul, fl, gamma0);
  mhd_flux_and_cons(qr, ur, fr, gamma0);
  for (int v = 0; v < NV; ++v)
    flux[v] = (fl[v] + fr[v]) / 2;
  const double cl = info_speed_x(ql, gamma0);
  const double cr = info_speed_x(qr, gamma0);
  const double vel = fmax(cl, cr);
  for (int v = 0; v < NV; ++v)
    flux[v] -= vel * (ur[v] - ul[v]) / 2;
}

/* RiemannSolvers_MHD.h:133-367 (HLLD of Miyoshi & Kusano 2005, RAMSES/DUMSES form) */
static void
riemann_hlld(double *ql, double *qr, double *flux, double gamma0)
{
  const double entho = 1.0 / (gamma0 - 1.0);
  const double a = 0.5 * (ql[IA] + qr[IA]);
  const double sgnm = (a >= 0) ? 1.0 : -1.0;
  ql[IA] = a;
  qr[IA] = a;

  const double rl = ql[ID], pl = ql[IP], ul = ql[IU], vl = ql[IV], wl = ql[IW], bl = ql[IB],
               cl = ql[IC];
  const double ecinl = 0.5 * (ul * ul + vl * vl + wl * wl) * rl;
  const double emagl = 0.5 * (a * a + bl * bl + cl * cl);
  const double etotl = pl * entho + ecinl + emagl;
  const double ptotl = pl + emagl;
  const double vdotbl = ul * a + vl * bl + wl * cl;

  const double rr = qr[ID], pr = qr[IP], ur = qr[IU], vr = qr[IV], wr = qr[IW], br = qr[IB],
               cr = qr[IC];
  const double ecinr = 0.5 * (ur * ur + vr * vr + wr * wr) * rr;
  const double emagr = 0.5 * (a * a + br * br + cr * cr);
  const double etotr = pr * entho + ecinr + emagr;
  const double ptotr = pr + emagr;
  const double vdotbr = ur * a + vr * br + wr * cr;

  const double cfastl = fast_speed_x(ql, gamma0);
  const double cfastr = fast_speed_x(qr, gamma0);

  const double sl = fmin(ul, ur) - fmax(cfastl, cfastr);
  const double sr = fmax(ul, ur) + fmax(cfastl, cfastr);

  const double rcl = rl * (ul - sl);
  const double rcr = rr * (sr - ur);

  const double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);

  /* left star region */
  const double rstarl = rl * (sl - ul) / (sl - ustar);
  double       estar = rl * (sl - ul) * (sl - ustar) - a * a;
  const double el = rl * (sl - ul) * (sl - ul) - a * a;
  double       vstarl, wstarl, bstarl, cstarl;
  if (a * a > 0 && fabs(estar / (a * a) - 1.0) <= 1e-8)
  {
    vstarl = vl;
    bstarl = bl;
    wstarl = wl;
    cstarl = cl;
  }
  else
  {
    vstarl = vl - a * bl * (ustar - ul) / estar;
    bstarl = bl * el / estar;
    wstarl = wl - a * cl * (ustar - ul) / estar;
    cstarl = cl * el / estar;
  }
  const double vdotbstarl = ustar * a + vstarl * bstarl + wstarl * cstarl;
  const double etotstarl =
    ((sl - ul) * etotl - ptotl * ul + ptotstar * ustar + a * (vdotbl - vdotbstarl)) / (sl - ustar);
  const double sqrrstarl = sqrt(rstarl);
  const double calfvenl = fabs(a) / sqrrstarl;
  const double sal = ustar - calfvenl;

  /* right star region */
  const double rstarr = rr * (sr - ur) / (sr - ustar);
  estar = rr * (sr - ur) * (sr - ustar) - a * a;
  const double er = rr * (sr - ur) * (sr - ur) - a * a;
  double       vstarr, wstarr, bstarr, cstarr;
  if (a * a > 0 && fabs(estar / (a * a) - 1.0) <= 1e-8)
  {
    vstarr = vr;
    bstarr = br;
    wstarr = wr;
    cstarr = cr;
  }
  else
  {
    vstarr = vr - a * br * (ustar - ur) / estar;
    bstarr = br * er / estar;
    wstarr = wr - a * cr * (ustar - ur) / estar;
    cstarr = cr * er / estar;
  }
  const double vdotbstarr = ustar * a + vstarr * bstarr + wstarr * cstarr;
  const double etotstarr =
    ((sr - ur) * etotr - ptotr * ur + ptotstar * ustar + a * (vdotbr - vdotbstarr)) / (sr - ustar);
  const double sqrrstarr = sqrt(rstarr);
  const double calfvenr = fabs(a) / sqrrstarr;
  const double sar = ustar + calfvenr;

  /* double star region */
  const double vstarstar =
    (sqrrstarl * vstarl + sqrrstarr * vstarr + sgnm * (bstarr - bstarl)) / (sqrrstarl + sqrrstarr);
  const double wstarstar =
    (sqrrstarl * wstarl + sqrrstarr * wstarr + sgnm * (cstarr - cstarl)) / (sqrrstarl + sqrrstarr);
  const double bstarstar =
    (sqrrstarl * bstarr + sqrrstarr * bstarl + sgnm * sqrrstarl * sqrrstarr * (vstarr - vstarl)) /
    (sqrrstarl + sqrrstarr);
  const double cstarstar =
    (sqrrstarl * cstarr + sqrrstarr * cstarl + sgnm * sqrrstarl * sqrrstarr * (wstarr - wstarl)) /
    (sqrrstarl + sqrrstarr);
  const double vdotbstarstar = ustar * a + vstarstar * bstarstar + wstarstar * cstarstar;
  const double etotstarstarl = etotstarl - sgnm * sqrrstarl * (vdotbstarl - vdotbstarstar);
  const double etotstarstarr = etotstarr + sgnm * sqrrstarr * (vdotbstarr - vdotbstarstar);

  double ro, uo, vo, wo, bo, co, ptoto, etoto, vdotbo;
  if (sl > 0)
  {
    ro = rl; uo = ul; vo = vl; wo = wl; bo = bl; co = cl;
    ptoto = ptotl; etoto = etotl; vdotbo = vdotbl;
  }
  else if (sal > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarl; wo = wstarl; bo = bstarl; co = cstarl;
    ptoto = ptotstar; etoto = etotstarl; vdotbo = vdotbstarl;
  }
  else if (ustar > 0)
  {
    ro = rstarl; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarl; vdotbo = vdotbstarstar;
  }
  else if (sar > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarstar; wo = wstarstar; bo = bstarstar; co = cstarstar;
    ptoto = ptotstar; etoto = etotstarstarr; vdotbo = vdotbstarstar;
  }
  else if (sr > 0)
  {
    ro = rstarr; uo = ustar; vo = vstarr; wo = wstarr; bo = bstarr; co = cstarr;
    ptoto = ptotstar; etoto = etotstarr; vdotbo = vdotbstarr;
  }
  else
  {
    ro = rr; uo = ur; vo = vr; wo = wr; bo = br; co = cr;
    ptoto = ptotr; etoto = etotr; vdotbo = vdotbr;
  }

  flux[ID] = ro * uo;
  flux[IP] = (etoto + ptoto) * uo - a * vdotbo;
  flux[IU] = ro * uo * uo - a * a + ptoto;
  flux[IV] = ro * uo * vo - a * bo;
  flux[IW] = ro * uo * wo - a * co;
  flux[IA] = 0.0;
  flux[IB] = bo * uo - a * vo;
  flux[IC] = co * uo - a * wo;
}

/* RiemannSolvers_MHD.h:372-392 */
static void
riemann_dispatch(int solver, double *ql, double *qr, double *flux, double gamma0)
{
  if (solver == ORC_RIEMANN_HLLD)
    riemann_hlld(ql, qr, flux, gamma0);
  else if (solver == ORC_RIEMANN_HLL)
    riemann_hll(ql, qr, flux, gamma0);
  else if (solver == ORC_RIEMANN_LLF)
    riemann_llf(ql, qr, flux, gamma0);
}

void
orc_riemann(const orc_params *p, const double *qL, const double *qR, double *flux)
{
  double l[NV], r[NV];
  memcpy(l, qL, sizeof l);
  memcpy(r, qR, sizeof r);
  for (int v = 0; v < NV; ++v)
    flux[v] = 0.0;
  riemann_dispatch(p->riemann, l, r, flux, p->gamma0);
}

static inline double
max4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  return r;
}
static inline double
min4(double a0, double a1, double a2, double a3)
{
  double r = a0;
  r = (a1 < r) ? a1 : r;
  r = (a2 < r) ? a2 : r;
  r = (a3 < r) ? a3 : r;
  return r;
}
static inline double
max5(double a0, double a1, double a2, double a3, double a4)
{
  double r = a0;
  r = (a1 > r) ? a1 : r;
  r = (a2 > r) ? a2 : r;
  r = (a3 > r) ? a3 : r;
  r = (a4 > r) ? a4 : r;
  return r;
}

/* 2D magnetic HLLD Riemann solver, RiemannSolvers_MHD.h:398-630.
 * q[4] ordered LL, RL, LR, RR; e[4] the corner emfs in the same order. */
static double
mag_riemann2d_hlld(const double q[4][NV], const double e[4], double gamma0, double smallc)
{
  const double *qLL = q[0], *qRL = q[1], *qLR = q[2], *qRR = q[3];
  const double  ELL = e[0], ERL = e[1], ELR = e[2], ERR = e[3];

  const double rLL = qLL[ID], pLL = qLL[IP], uLL = qLL[IU], vLL = qLL[IV], aLL = qLL[IA],
               bLL = qLL[IB], cLL = qLL[IC];
  const double rLR = qLR[ID], pLR = qLR[IP], uLR = qLR[IU], vLR = qLR[IV], aLR = qLR[IA],
               bLR = qLR[IB], cLR = qLR[IC];
  const double rRL = qRL[ID], pRL = qRL[IP], uRL = qRL[IU], vRL = qRL[IV], aRL = qRL[IA],
               bRL = qRL[IB], cRL = qRL[IC];
  const double rRR = qRR[ID], pRR = qRR[IP], uRR = qRR[IU], vRR = qRR[IV], aRR = qRR[IA],
               bRR = qRR[IB], cRR = qRR[IC];

  const double cFastLLx = fast_speed_x(qLL, gamma0);
  const double cFastLRx = fast_speed_x(qLR, gamma0);
  const double cFastRLx = fast_speed_x(qRL, gamma0);
  const double cFastRRx = fast_speed_x(qRR, gamma0);
  const double cFastLLy = fast_speed_y(qLL, gamma0);
  const double cFastLRy = fast_speed_y(qLR, gamma0);
  const double cFastRLy = fast_speed_y(qRL, gamma0);
  const double cFastRRy = fast_speed_y(qRR, gamma0);

  const double SL = min4(uLL, uLR, uRL, uRR) - max4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const double SR = max4(uLL, uLR, uRL, uRR) + max4(cFastLLx, cFastLRx, cFastRLx, cFastRRx);
  const double SB = min4(vLL, vLR, vRL, vRR) - max4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);
  const double ST = max4(vLL, vLR, vRL, vRR) + max4(cFastLLy, cFastLRy, cFastRLy, cFastRRy);

  const double PtotLL = pLL + 0.5 * (aLL * aLL + bLL * bLL + cLL * cLL);
  const double PtotLR = pLR + 0.5 * (aLR * aLR + bLR * bLR + cLR * cLR);
  const double PtotRL = pRL + 0.5 * (aRL * aRL + bRL * bRL + cRL * cRL);
  const double PtotRR = pRR + 0.5 * (aRR * aRR + bRR * bRR + cRR * cRR);

  const double rcLLx = rLL * (uLL - SL);
  const double rcRLx = rRL * (SR - uRL);
  const double rcLRx = rLR * (uLR - SL);
  const double rcRRx = rRR * (SR - uRR);
  const double rcLLy = rLL * (vLL - SB);
  const double rcLRy = rLR * (ST - vLR);
  const double rcRLy = rRL * (vRL - SB);
  const double rcRRy = rRR * (ST - vRR);

  const double ustar =
    (rcLLx * uLL + rcLRx * uLR + rcRLx * uRL + rcRRx * uRR + (PtotLL - PtotRL + PtotLR - PtotRR)) /
    (rcLLx + rcLRx + rcRLx + rcRRx);
  const double vstar =
    (rcLLy * vLL + rcLRy * vLR + rcRLy * vRL + rcRRy * vRR + (PtotLL - PtotLR + PtotRL - PtotRR)) /
    (rcLLy + rcLRy + rcRLy + rcRRy);

  const double rstarLLx = rLL * (SL - uLL) / (SL - ustar);
  const double BstarLL = bLL * (SL - uLL) / (SL - ustar);
  const double rstarLLy = rLL * (SB - vLL) / (SB - vstar);
  const double AstarLL = aLL * (SB - vLL) / (SB - vstar);
  const double rstarLL = rLL * (SL - uLL) / (SL - ustar) * (SB - vLL) / (SB - vstar);
  const double EstarLLx = ustar * BstarLL - vLL * aLL;
  const double EstarLLy = uLL * bLL - vstar * AstarLL;
  const double EstarLL = ustar * BstarLL - vstar * AstarLL;

  const double rstarLRx = rLR * (SL - uLR) / (SL - ustar);
  const double BstarLR = bLR * (SL - uLR) / (SL - ustar);
  const double rstarLRy = rLR * (ST - vLR) / (ST - vstar);
  const double AstarLR = aLR * (ST - vLR) / (ST - vstar);
  const double rstarLR = rLR * (SL - uLR) / (SL - ustar) * (ST - vLR) / (ST - vstar);
  const double EstarLRx = ustar * BstarLR - vLR * aLR;
  const double EstarLRy = uLR * bLR - vstar * AstarLR;
  const double EstarLR = ustar * BstarLR - vstar * AstarLR;

  const double rstarRLx = rRL * (SR - uRL) / (SR - ustar);
  const double BstarRL = bRL * (SR - uRL) / (SR - ustar);
  const double rstarRLy = rRL * (SB - vRL) / (SB - vstar);
  const double AstarRL = aRL * (SB - vRL) / (SB - vstar);
  const double rstarRL = rRL * (SR - uRL) / (SR - ustar) * (SB - vRL) / (SB - vstar);
  const double EstarRLx = ustar * BstarRL - vRL * aRL;
  const double EstarRLy = uRL * bRL - vstar * AstarRL;
  const double EstarRL = ustar * BstarRL - vstar * AstarRL;

  const double rstarRRx = rRR * (SR - uRR) / (SR - ustar);
  const double BstarRR = bRR * (SR - uRR) / (SR - ustar);
  const double rstarRRy = rRR * (ST - vRR) / (ST - vstar);
  const double AstarRR = aRR * (ST - vRR) / (ST - vstar);
  const double rstarRR = rRR * (SR - uRR) / (SR - ustar) * (ST - vRR) / (ST - vstar);
  const double EstarRRx = ustar * BstarRR - vRR * aRR;
  const double EstarRRy = uRR * bRR - vstar * AstarRR;
  const double EstarRR = ustar * BstarRR - vstar * AstarRR;

  const double calfvenL = max5(fabs(aLR) / sqrt(rstarLRx), fabs(AstarLR) / sqrt(rstarLR),
                               fabs(aLL) / sqrt(rstarLLx), fabs(AstarLL) / sqrt(rstarLL), smallc);
  const double calfvenR = max5(fabs(aRR) / sqrt(rstarRRx), fabs(AstarRR) / sqrt(rstarRR),
                               fabs(aRL) / sqrt(rstarRLx), fabs(AstarRL) / sqrt(rstarRL), smallc);
  const double calfvenB = max5(fabs(bLL) / sqrt(rstarLLy), fabs(BstarLL) / sqrt(rstarLL),
                               fabs(bRL) / sqrt(rstarRLy), fabs(BstarRL) / sqrt(rstarRL), smallc);
  const double calfvenT = max5(fabs(bLR) / sqrt(rstarLRy), fabs(BstarLR) / sqrt(rstarLR),
                               fabs(bRR) / sqrt(rstarRRy), fabs(BstarRR) / sqrt(rstarRR), smallc);

  const double SAL = fmin(ustar - calfvenL, 0.0);
  const double SAR = fmax(ustar + calfvenR, 0.0);
  const double SAB = fmin(vstar - calfvenB, 0.0);
  const double SAT = fmax(vstar + calfvenT, 0.0);

  const double AstarT = (SAR * AstarRR - SAL * AstarLR) / (SAR - SAL);
  const double AstarB = (SAR * AstarRL - SAL * AstarLL) / (SAR - SAL);
  const double BstarR = (SAT * BstarRR - SAB * BstarRL) / (SAT - SAB);
  const double BstarL = (SAT * BstarLR - SAB * BstarLL) / (SAT - SAB);

  /* 0/1 region masks from the sign bits of SB, ST, SL, SR (:569-572) */
  const int SB_pos = (int)(1 + copysign(1.0, SB)) / 2, SB_neg = 1 - SB_pos;
  const int ST_pos = (int)(1 + copysign(1.0, ST)) / 2, ST_neg = 1 - ST_pos;
  const int SL_pos = (int)(1 + copysign(1.0, SL)) / 2, SL_neg = 1 - SL_pos;
  const int SR_pos = (int)(1 + copysign(1.0, SR)) / 2, SR_neg = 1 - SR_pos;

  double E = 0, t;
  t = (SAL * SAB * EstarRR - SAL * SAT * EstarRL - SAR * SAB * EstarLR + SAR * SAT * EstarLL) /
        (SAR - SAL) / (SAT - SAB) -
      SAT * SAB / (SAT - SAB) * (AstarT - AstarB) + SAR * SAL / (SAR - SAL) * (BstarR - BstarL);
  E += (SB_neg * ST_pos * SL_neg * SR_pos) * t;

  t = (SAR * EstarLLx - SAL * EstarRLx + SAR * SAL * (bRL - bLL)) / (SAR - SAL);
  t = SL_pos * ELL + SL_neg * SR_neg * ERL + SL_neg * SR_pos * t;
  E += SB_pos * t;

  t = (SAR * EstarLRx - SAL * EstarRRx + SAR * SAL * (bRR - bLR)) / (SAR - SAL);
  t = SL_pos * ELR + SL_neg * SR_neg * ERR + SL_neg * SR_pos * t;
  E += (SB_neg * ST_neg) * t;

  t = (SAT * EstarLLy - SAB * EstarLRy - SAT * SAB * (aLR - aLL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_pos) * t;

  t = (SAT * EstarRLy - SAB * EstarRRy - SAT * SAB * (aRR - aRL)) / (SAT - SAB);
  E += (SB_neg * ST_pos * SL_neg * SR_neg) * t;
  return E;
}

/* compute_emf<EmfDir>, RiemannSolvers_MHD.h:651-874.
 * qEdge ordered RT, RB, LT, LB (EdgeIndex, enums.h:176-182). */
static double
compute_emf(int emf_dir, const double qEdge[4][NV], double gamma0, double smallc)
{
  const double *qRT = qEdge[0], *qRB = qEdge[1], *qLT = qEdge[2], *qLB = qEdge[3];
  double        q[4][NV]; /* LL, RL, LR, RR */
  double       *qLL = q[0], *qRL = q[1], *qLR = q[2], *qRR = q[3];
  qLL[ID] = qRT[ID]; qRL[ID] = qLT[ID]; qLR[ID] = qRB[ID]; qRR[ID] = qLB[ID];
  qLL[IP] = qRT[IP]; qRL[IP] = qLT[IP]; qLR[IP] = qRB[IP]; qRR[IP] = qLB[IP];
  /* (first parallel, second parallel, orthogonal) slots of velocity and field */
  int iu, iv, iw, ia, ib, ic;
  if (emf_dir == 2)
  { iu = IU; iv = IV; iw = IW; ia = IA; ib = IB; ic = IC; }
  else if (emf_dir == 1)
  { iu = IW; iv = IU; iw = IV; ia = IC; ib = IA; ic = IB; }
  else
  { iu = IV; iv = IW; iw = IU; ia = IB; ib = IC; ic = IA; }
  qLL[IU] = qRT[iu]; qRL[IU] = qLT[iu]; qLR[IU] = qRB[iu]; qRR[IU] = qLB[iu];
  qLL[IV] = qRT[iv]; qRL[IV] = qLT[iv]; qLR[IV] = qRB[iv]; qRR[IV] = qLB[iv];
  qLL[IA] = 0.5 * (qRT[ia] + qLT[ia]);
  qRL[IA] = 0.5 * (qRT[ia] + qLT[ia]);
  qLR[IA] = 0.5 * (qRB[ia] + qLB[ia]);
  qRR[IA] = 0.5 * (qRB[ia] + qLB[ia]);
  qLL[IB] = 0.5 * (qRT[ib] + qRB[ib]);
  qRL[IB] = 0.5 * (qLT[ib] + qLB[ib]);
  qLR[IB] = 0.5 * (qRT[ib] + qRB[ib]);
  qRR[IB] = 0.5 * (qLT[ib] + qLB[ib]);
  qLL[IW] = qRT[iw]; qRL[IW] = qLT[iw]; qLR[IW] = qRB[iw]; qRR[IW] = qLB[iw];
  qLL[IC] = qRT[ic]; qRL[IC] = qLT[ic]; qLR[IC] = qRB[ic]; qRR[IC] = qLB[ic];
  double e[4];
  for (int c = 0; c < 4; ++c)
    e[c] = q[c][IU] * q[c][IB] - q[c][IV] * q[c][IA];
  return mag_riemann2d_hlld((const double(*)[NV])q, e, gamma0, smallc);
}

double
orc_compute_emf(const orc_params *p, int emf_dir, const double *qEdge)
{
  return compute_emf(emf_dir, (const double(*)[NV])qEdge, p->gamma0, p->smallc);
}

/* MHDBaseFunctor2D.h:370-383 (slope_unsplit_hydro_2d_scalar, 3-point form):
 * MC-type limiter controlled by slope_type */
static inline double
limited_slope(double q, double qp, double qm, double slope_type)
{
  const double dlft = slope_type * (q - qm);
  const double drgt = slope_type * (qp - q);
  const double dcen = 0.5 * (qp - qm);
  const double dsgn = (dcen >= 0.0) ? 1.0 : -1.0;
  const double slop = fmin(fabs(dlft), fabs(drgt));
  double       dlim = slop;
  if ((dlft * drgt) <= 0.0)
    dlim = 0.0;
  return dsgn * fmin(dlim, fabs(dcen));
}

/* ====================================================================== */
/* solver                                                                  */
/* ====================================================================== */

struct orc_solver
{
  orc_params p;
  layout     L;
  int        nthreads;
  double    *U, *U2, *Q, *Q2, *Sx, *Sy, *Sz, *E, *sF, *Fx, *Fy, *Fz, *Em;
  double     t, dt;
  int        it;
  int        dt_ulps; /* test hook: dt moved by this many ulps (orc_set_dt_ulps) */
};

static double *
zalloc(int64_t n)
{
  return (double *)calloc((size_t)n, sizeof(double));
}

orc_solver *
orc_create(const orc_params *p, int nthreads)
{
  orc_solver *s = (orc_solver *)calloc(1, sizeof *s);
  s->p = *p;
  s->L = mk_layout(p);
  s->nthreads = nthreads < 1 ? 1 : nthreads;
  const int64_t n8 = orc_nelem(p), n1 = n8 / NV;
  s->U = zalloc(n8);
  s->U2 = zalloc(n8);
  s->Q = zalloc(n8);
  s->Q2 = zalloc(n8);
  s->Sx = zalloc(n8);
  s->Sy = zalloc(n8);
  s->Sz = p->dim == 3 ? zalloc(n8) : NULL;
  s->E = zalloc(3 * n1);
  s->sF = zalloc(3 * n1);
  s->Fx = zalloc(n8);
  s->Fy = zalloc(n8);
  s->Fz = p->dim == 3 ? zalloc(n8) : NULL;
  s->Em = zalloc(3 * n1);
  s->t = p->tCurrent;
  s->it = 0;
  orc_init_orszag_tang(p, s->U);
  orc_set_state(s, s->U);
  return s;
}

void
orc_destroy(orc_solver *s)
{
  if (!s)
    return;
  double *a[] = { s->U, s->U2, s->Q, s->Q2, s->Sx, s->Sy, s->Sz, s->E, s->sF, s->Fx, s->Fy, s->Fz, s->Em };
  for (size_t q = 0; q < sizeof a / sizeof a[0]; ++q)
    free(a[q]);
  free(s);
}

/* ConvertToPrimitivesFunctor{2D,3D}_MHD (MHDRunFunctors2D.h:85-159, 3D:88-163)
 * + constoprim_mhd (MHDBaseFunctor2D.h:194-242) over [0, size-1)^dim */
static void
convert_to_primitives(orc_solver *s, const double *U)
{
  const orc_params *p = &s->p;
  const layout      L = s->L;
  const int         kmax = p->dim == 3 ? p->ksize - 1 : 1;
  const double      smallr = p->smallr, gamma0 = p->gamma0, smallp = p->smallp;
  double           *Q = s->Q;
#pragma omp parallel for collapse(2) schedule(static) num_threads(s->nthreads)
  for (int k = 0; k < kmax; ++k)
    for (int j = 0; j < p->jsize - 1; ++j)
      for (int i = 0; i < p->isize - 1; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        const double  nbx = U[c + 1 + IA * L.sv];
        const double  nby = U[c + L.sj + IB * L.sv];
        const double  nbz = p->dim == 3 ? U[c + L.sk + IC * L.sv] : 0.0;
        const double  d = fmax(U[c + ID * L.sv], smallr);
        const double  vu = U[c + IU * L.sv] / d;
        const double  vv = U[c + IV * L.sv] / d;
        const double  vw = U[c + IW * L.sv] / d;
        const double  a = 0.5 * (U[c + IA * L.sv] + nbx);
        const double  b = 0.5 * (U[c + IB * L.sv] + nby);
        const double  cz = 0.5 * (U[c + IC * L.sv] + nbz);
        const double  eken = 0.5 * (vu * vu + vv * vv + vw * vw);
        const double  emag = 0.5 * (a * a + b * b + cz * cz);
        const double  eint = (U[c + IP * L.sv] - emag) / d - eken;
        Q[c + ID * L.sv] = d;
        Q[c + IP * L.sv] = fmax((gamma0 - 1.0) * d * eint, d * smallp);
        Q[c + IU * L.sv] = vu;
        Q[c + IV * L.sv] = vv;
        Q[c + IW * L.sv] = vw;
        Q[c + IA * L.sv] = a;
        Q[c + IB * L.sv] = b;
        Q[c + IC * L.sv] = cz;
      }
}

/* ComputeDtFunctor{2D,3D}_MHD (MHDRunFunctors2D.h:16-80, 3D:16-83) with
 * find_speed_info<NDIM> (mhd_utils.h:319-366); SolverMHDMuscl.h:722-741 and
 * SolverBase.cpp:148-179 (clip to tEnd) */
static void
compute_dt(orc_solver *s)
{
  const orc_params *p = &s->p;
  const layout      L = s->L;
  const int         g = p->ghost;
  const int         k0 = p->dim == 3 ? g : 0, k1 = p->dim == 3 ? p->ksize - g : 1;
  const double      gamma0 = p->gamma0;
  const double     *Q = s->Q;
  double            invDt = -1.0 / 0.0;
#pragma omp parallel for collapse(2) schedule(static) reduction(max : invDt) num_threads(s->nthreads)
  for (int k = k0; k < k1; ++k)
    for (int j = g; j < p->jsize - g; ++j)
      for (int i = g; i < p->isize - g; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        const double  d = Q[c + ID * L.sv], pr = Q[c + IP * L.sv];
        const double  u = Q[c + IU * L.sv], v = Q[c + IV * L.sv], w = Q[c + IW * L.sv];
        const double  a = Q[c + IA * L.sv], b = Q[c + IB * L.sv], cz = Q[c + IC * L.sv];
        const double  b2 = a * a + b * b + cz * cz;
        const double  c2 = gamma0 * pr / d;
        const double  d2 = 0.5 * (b2 / d + c2);
        const double  vx = sqrt(d2 + sqrt(d2 * d2 - c2 * a * a / d)) + fabs(u);
        const double  vy = sqrt(d2 + sqrt(d2 * d2 - c2 * b * b / d)) + fabs(v);
        double        val;
        if (p->dim == 3)
        {
          const double vz = sqrt(d2 + sqrt(d2 * d2 - c2 * cz * cz / d)) + fabs(w);
          val = vx / p->dx + vy / p->dy + vz / p->dz;
        }
        else
          val = vx / p->dx + vy / p->dy;
        invDt = fmax(invDt, val);
      }
  s->dt = p->cfl / invDt;
  for (int u = 0; u < s->dt_ulps; ++u)
    s->dt = nextafter(s->dt, INFINITY);
  if (s->t + s->dt > p->tEnd)
    s->dt = p->tEnd - s->t;
}

/* Test hook: every later dt of the solver is moved up by `ulps` units in the
 * last place (0 restores the reference's dt).  Used to measure how far one
 * rounding difference carries (tests/test_oracle_pinning.py). */
void
orc_set_dt_ulps(orc_solver *s, int ulps)
{
  s->dt_ulps = ulps;
}

void
orc_set_state(orc_solver *s, const double *U)
{
  const int64_t n8 = orc_nelem(&s->p);
  if (U != s->U)
    memcpy(s->U, U, (size_t)n8 * sizeof(double));
  s->it = 0;
  s->t = s->p.tCurrent;
  orc_make_boundaries(&s->p, s->U);
  memcpy(s->U2, s->U, (size_t)n8 * sizeof(double));
  convert_to_primitives(s, s->U);
  compute_dt(s);
}

void
orc_get_state(const orc_solver *s, double *U)
{
  const double *cur = (s->it % 2 == 0) ? s->U : s->U2;
  memcpy(U, cur, (size_t)orc_nelem(&s->p) * sizeof(double));
}

void
orc_time(const orc_solver *s, double *t, double *dt, int *iteration)
{
  *t = s->t;
  *dt = s->dt;
  *iteration = s->it;
}

/* ---------------------------------------------------------------------- */
/* 2D, implementation version 2 (SolverMHDMuscl.cpp:373-458)               */
/* ---------------------------------------------------------------------- */

static void
step2d(orc_solver *s, double *Uin, double *Uout)
{
  const orc_params *p = &s->p;
  const layout      L = s->L;
  const int64_t     sv = L.sv, sj = L.sj;
  const int         g = p->ghost, isize = p->isize, jsize = p->jsize;
  const double      st = p->slope_type, gamma = p->gamma0;
  const double      smallR = p->smallr, smallp = p->smallp;
  double           *Q = s->Q, *Q2 = s->Q2, *Sx = s->Sx, *Sy = s->Sy, *E = s->E, *sF = s->sF;
  double           *Fx = s->Fx, *Fy = s->Fy, *Em = s->Em;
  const int         nt = s->nthreads;

  orc_make_boundaries(p, Uin);
  memcpy(Uout, Uin, (size_t)orc_nelem(p) * sizeof(double));
  convert_to_primitives(s, Uin);
  compute_dt(s);
  const double dtdx = s->dt / p->dx;
  const double dtdy = s->dt / p->dy;

  /* ComputeSlopesFunctor2D_MHD (MHDRunFunctors2D.h:164-248), [1, size-1) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = 1; j < jsize - 1; ++j)
    for (int i = 1; i < isize - 1; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      for (int v = 0; v < NV; ++v)
      {
        const double q = Q[c + v * sv];
        Sx[c + v * sv] = limited_slope(q, Q[c + 1 + v * sv], Q[c - 1 + v * sv], st);
        Sy[c + v * sv] = limited_slope(q, Q[c + sj + v * sv], Q[c - sj + v * sv], st);
      }
      Sx[c + IA * sv] = Uin[c + 1 + IA * sv] - Uin[c + IA * sv];
      Sy[c + IB * sv] = Uin[c + sj + IB * sv] - Uin[c + IB * sv];
    }

  /* ComputeUpdatedPrimVarFunctor2D_MHD (MHDRunFunctors2D.h:920-1051), [g-2, size-g+1) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = g - 2; j < jsize - g + 1; ++j)
    for (int i = g - 2; i < isize - g + 1; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      const double  r = Q[c + ID * sv], pr = Q[c + IP * sv], u = Q[c + IU * sv],
                   v = Q[c + IV * sv], w = Q[c + IW * sv], A = Q[c + IA * sv],
                   B = Q[c + IB * sv], C = Q[c + IC * sv];
      const double drx = Sx[c + ID * sv], dpx = Sx[c + IP * sv], dux = Sx[c + IU * sv],
                   dvx = Sx[c + IV * sv], dwx = Sx[c + IW * sv], dBx = Sx[c + IB * sv],
                   dCx = Sx[c + IC * sv];
      const double dry = Sy[c + ID * sv], dpy = Sy[c + IP * sv], duy = Sy[c + IU * sv],
                   dvy = Sy[c + IV * sv], dwy = Sy[c + IW * sv], dAy = Sy[c + IA * sv],
                   dCy = Sy[c + IC * sv];
      const double dAx = Uin[c + 1 + IA * sv] - Uin[c + IA * sv];
      const double dBy = Uin[c + sj + IB * sv] - Uin[c + IB * sv];
      const double sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
      const double su0 =
        (-u * dux - dpx / r - B * dBx / r - C * dCx / r) * dtdx + (-v * duy + B * dAy / r) * dtdy;
      const double sv0 =
        (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - C * dCy / r) * dtdy;
      const double sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy;
      const double sp0 = (-u * dpx - dux * gamma * pr) * dtdx + (-v * dpy - dvy * gamma * pr) * dtdy;
      const double sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy;
      const double sB0 = (-u * dBx - B * dux + v * dAx + A * dvx) * dtdx;
      const double sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx +
                         (-v * dCy - C * dvy + w * dBy + B * dwy) * dtdy;
      Q2[c + ID * sv] = r + 0.5 * sr0;
      Q2[c + IU * sv] = u + 0.5 * su0;
      Q2[c + IV * sv] = v + 0.5 * sv0;
      Q2[c + IW * sv] = w + 0.5 * sw0;
      Q2[c + IP * sv] = pr + 0.5 * sp0;
      Q2[c + IA * sv] = A + 0.5 * sA0;
      Q2[c + IB * sv] = B + 0.5 * sB0;
      Q2[c + IC * sv] = C + 0.5 * sC0;
    }

  /* ComputeElecFieldFunctor2D (MHDRunFunctors2D.h:253-314), [1, size) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = 1; j < jsize; ++j)
    for (int i = 1; i < isize; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      const double  u = 0.25 * (Q[c - 1 - sj + IU * sv] + Q[c - 1 + IU * sv] +
                               Q[c - sj + IU * sv] + Q[c + IU * sv]);
      const double  v = 0.25 * (Q[c - 1 - sj + IV * sv] + Q[c - 1 + IV * sv] +
                               Q[c - sj + IV * sv] + Q[c + IV * sv]);
      const double  A = 0.5 * (Uin[c - sj + IA * sv] + Uin[c + IA * sv]);
      const double  B = 0.5 * (Uin[c - 1 + IB * sv] + Uin[c + IB * sv]);
      E[c] = u * B - v * A;
    }

  /* ComputeSourceFaceMagFunctor2D (MHDRunFunctors2D.h:319-370), [1, size-1) */
  const int64_t n1 = L.sv;
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = 1; j < jsize - 1; ++j)
    for (int i = 1; i < isize - 1; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      sF[c] = (E[c + sj] - E[c]) * 0.5 * dtdy;
      sF[c + n1] = -(E[c + 1] - E[c]) * 0.5 * dtdx;
    }

  /* ComputeFluxAndUpdateAlongDirFunctor2D_MHD<dir> flux part
   * (MHDRunFunctors2D.h:1110-1229), faces [g, size-g] */
  for (int dir = 0; dir < 2; ++dir)
  {
    double       *F = dir == 0 ? Fx : Fy;
    const double *S = dir == 0 ? Sx : Sy;
    const int64_t off = dir == 0 ? 1 : sj;
#pragma omp parallel for schedule(static) num_threads(nt)
    for (int j = g; j < jsize - g + 1; ++j)
      for (int i = g; i < isize - g + 1; ++i)
      {
        const int64_t c = AT(L, i, j, 0), cn = c - off;
        double        qR[NV], qL[NV], fl[NV];
        for (int v = 0; v < 5; ++v)
        {
          qR[v] = Q2[c + v * sv] - 0.5 * S[c + v * sv];
          qL[v] = Q2[cn + v * sv] + 0.5 * S[cn + v * sv];
        }
        qR[ID] = fmax(smallR, qR[ID]);
        qR[IP] = fmax(smallp * qR[ID], qR[IP]);
        qL[ID] = fmax(smallR, qL[ID]);
        qL[IP] = fmax(smallp * qL[ID], qL[IP]);
        if (dir == 0)
        {
          const double AL = Uin[c + IA * sv] + sF[c];
          qR[IA] = AL;
          qR[IB] = Q2[c + IB * sv] - 0.5 * S[c + IB * sv];
          qR[IC] = Q2[c + IC * sv] - 0.5 * S[c + IC * sv];
          qL[IA] = qR[IA];
          qL[IB] = Q2[cn + IB * sv] + 0.5 * S[cn + IB * sv];
          qL[IC] = Q2[cn + IC * sv] + 0.5 * S[cn + IC * sv];
        }
        else
        {
          const double BL = Uin[c + IB * sv] + sF[c + n1];
          qR[IA] = Q2[c + IA * sv] - 0.5 * S[c + IA * sv];
          qR[IB] = BL;
          qR[IC] = Q2[c + IC * sv] - 0.5 * S[c + IC * sv];
          qL[IA] = Q2[cn + IA * sv] + 0.5 * S[cn + IA * sv];
          qL[IB] = qR[IB];
          qL[IC] = Q2[cn + IC * sv] + 0.5 * S[cn + IC * sv];
          double tmp;
          tmp = qL[IU]; qL[IU] = qL[IV]; qL[IV] = tmp;
          tmp = qL[IA]; qL[IA] = qL[IB]; qL[IB] = tmp;
          tmp = qR[IU]; qR[IU] = qR[IV]; qR[IV] = tmp;
          tmp = qR[IA]; qR[IA] = qR[IB]; qR[IB] = tmp;
        }
        for (int v = 0; v < NV; ++v)
          fl[v] = 0.0;
        riemann_dispatch(p->riemann, qL, qR, fl, gamma);
        if (dir == 1)
        {
          double tmp;
          tmp = fl[IU]; fl[IU] = fl[IV]; fl[IV] = tmp;
          tmp = fl[IA]; fl[IA] = fl[IB]; fl[IB] = tmp;
        }
        for (int v = 0; v < NV; ++v)
          F[c + v * sv] = fl[v];
      }
  }

  /* ReconstructEdgeComputeEmfAndUpdateFunctor2D (MHDRunFunctors2D.h:1291-1534),
   * edges [g, size-g] */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = g; j < jsize - g + 1; ++j)
    for (int i = g; i < isize - g + 1; ++i)
    {
      double qe[4][NV]; /* RT, RB, LT, LB */
      /* (cell offset di, dj; sign_x, sign_y, sign_a, sign_b) per corner state,
       * reconstruct_state_at_edge (MHDRunFunctors2D.h:1347-1435) */
      static const int corner[4][6] = {
        { -1, -1, 1, 1, 1, 1 },   /* RT from cell (i-1, j-1) */
        { -1, 0, 1, -1, -1, 1 },  /* RB from cell (i-1, j)   */
        { 0, -1, -1, 1, 1, -1 },  /* LT from cell (i, j-1)   */
        { 0, 0, -1, -1, -1, -1 }, /* LB from cell (i, j)     */
      };
      for (int e = 0; e < 4; ++e)
      {
        const int     i0 = i + corner[e][0], j0 = j + corner[e][1];
        const int     sx = corner[e][2], sy = corner[e][3], sa = corner[e][4], sb = corner[e][5];
        /* face of Bx: (i0+1, j0) for RT/RB, (i0, j0) for LT/LB; face of By:
         * (i0, j0+1) for RT/LT, (i0, j0) for RB/LB */
        const int     ia = (e == 0 || e == 1) ? i0 + 1 : i0, ja = j0;
        const int     ib = i0, jb = (e == 0 || e == 2) ? j0 + 1 : j0;
        const int64_t c0 = AT(L, i0, j0, 0), ca = AT(L, ia, ja, 0), cb = AT(L, ib, jb, 0);
        const double  A = Uin[ca + IA * sv] + sF[ca];
        const double  dAy = limited_slope(Uin[ca + IA * sv], Uin[ca + sj + IA * sv],
                                         Uin[ca - sj + IA * sv], st);
        const double  B = Uin[cb + IB * sv] + sF[cb + n1];
        const double  dBx = limited_slope(Uin[cb + IB * sv], Uin[cb + 1 + IB * sv],
                                         Uin[cb - 1 + IB * sv], st);
        double *q = qe[e];
        for (int v = 0; v < NV; ++v)
          q[v] = Q2[c0 + v * sv];
        q[ID] += 0.5 * (sx * Sx[c0 + ID * sv] + sy * Sy[c0 + ID * sv]);
        q[IU] += 0.5 * (sx * Sx[c0 + IU * sv] + sy * Sy[c0 + IU * sv]);
        q[IV] += 0.5 * (sx * Sx[c0 + IV * sv] + sy * Sy[c0 + IV * sv]);
        q[IW] += 0.5 * (sx * Sx[c0 + IW * sv] + sy * Sy[c0 + IW * sv]);
        q[IP] += 0.5 * (sx * Sx[c0 + IP * sv] + sy * Sy[c0 + IP * sv]);
        q[IA] = A + 0.5 * (sa * dAy);
        q[IB] = B + 0.5 * (sb * dBx);
        q[IC] += 0.5 * (sx * Sx[c0 + IC * sv] + sy * Sy[c0 + IC * sv]);
        q[ID] = fmax(smallR, q[ID]);
        q[IP] = fmax(smallp * q[ID], q[IP]);
      }
      Em[AT(L, i, j, 0)] = compute_emf(2, (const double(*)[NV])qe, gamma, p->smallc);
    }

  /* update: the atomic adds/subs of the flux and emf functors, in the order a
   * serial run applies them (MHDRunFunctors2D.h:1231-1273, :1519-1523) */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = g; j < jsize - g; ++j)
    for (int i = g; i < isize - g; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      static const int hv[6] = { ID, IP, IU, IV, IW, IC };
      for (int q = 0; q < 6; ++q)
      {
        const int v = hv[q];
        double    x = Uout[c + v * sv];
        x += Fx[c + v * sv] * dtdx;
        x -= Fx[c + 1 + v * sv] * dtdx;
        x += Fy[c + v * sv] * dtdy;
        x -= Fy[c + sj + v * sv] * dtdy;
        Uout[c + v * sv] = x;
      }
    }
  /* face fields: Bx faces i in [g, isize-g], By faces j in [g, jsize-g] */
#pragma omp parallel for schedule(static) num_threads(nt)
  for (int j = g; j < jsize - g + 1; ++j)
    for (int i = g; i < isize - g + 1; ++i)
    {
      const int64_t c = AT(L, i, j, 0);
      if (j < jsize - g)
      {
        double x = Uout[c + IA * sv];
        x -= Em[c] * dtdy;
        x += Em[c + sj] * dtdy;
        Uout[c + IA * sv] = x;
      }
      if (i < isize - g)
      {
        double x = Uout[c + IB * sv];
        x += Em[c] * dtdx;
        x -= Em[c + 1] * dtdx;
        Uout[c + IB * sv] = x;
      }
    }
}

/* ---------------------------------------------------------------------- */
/* 3D, implementation version 2 (SolverMHDMuscl.cpp:465-572)               */
/* ---------------------------------------------------------------------- */

/* compute_limited_slope<dir> on face-centred field (MHDBaseFunctor3D.h:128-158).
 * For dir = z the reference samples the minus neighbour at k + 1 (not k - 1),
 * so the z slope is identically zero; that is reproduced here. */
static inline double
face_slope3(const double *U, layout L, int64_t c, int comp, int dir, double st)
{
  const int64_t cv = c + comp * L.sv;
  if (dir == 0)
    return limited_slope(U[cv], U[cv + 1], U[cv - 1], st);
  if (dir == 1)
    return limited_slope(U[cv], U[cv + L.sj], U[cv - L.sj], st);
  return limited_slope(U[cv], U[cv + L.sk], U[cv + L.sk], st);
}

static void
step3d(orc_solver *s, double *Uin, double *Uout)
{
  const orc_params *p = &s->p;
  const layout      L = s->L;
  const int64_t     sv = L.sv, sj = L.sj, sk = L.sk;
  const int         g = p->ghost, isize = p->isize, jsize = p->jsize, ksize = p->ksize;
  const double      st = p->slope_type, gamma = p->gamma0;
  const double      smallR = p->smallr, smallp = p->smallp;
  double           *Q = s->Q, *Q2 = s->Q2, *Sx = s->Sx, *Sy = s->Sy, *Sz = s->Sz, *E = s->E;
  double           *sF = s->sF, *Em = s->Em;
  double           *Fd[3] = { s->Fx, s->Fy, s->Fz };
  const double     *Sd[3] = { s->Sx, s->Sy, s->Sz };
  const int64_t     n1 = sv;
  const int         nt = s->nthreads;
  const int64_t     stride[3] = { 1, sj, sk };

  ORC_STAGE(STG_OTHER);
  orc_make_boundaries(p, Uin);
  memcpy(Uout, Uin, (size_t)orc_nelem(p) * sizeof(double));
  ORC_STAGE(STG_PRIM);
  convert_to_primitives(s, Uin);
  ORC_STAGE(STG_DT);
  compute_dt(s);
  ORC_STAGE(STG_OTHER);
  const double dtdx = s->dt / p->dx;
  const double dtdy = s->dt / p->dy;
  const double dtdz = s->dt / p->dz;

  ORC_STAGE(STG_SLOPES);
  /* ComputeSlopesFunctor3D_MHD (MHDRunFunctors3D.h:168-273), [1, size-1) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = 1; k < ksize - 1; ++k)
    for (int j = 1; j < jsize - 1; ++j)
      for (int i = 1; i < isize - 1; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        for (int v = 0; v < NV; ++v)
        {
          const double q = Q[c + v * sv];
          Sx[c + v * sv] = limited_slope(q, Q[c + 1 + v * sv], Q[c - 1 + v * sv], st);
          Sy[c + v * sv] = limited_slope(q, Q[c + sj + v * sv], Q[c - sj + v * sv], st);
          Sz[c + v * sv] = limited_slope(q, Q[c + sk + v * sv], Q[c - sk + v * sv], st);
        }
        Sx[c + IA * sv] = Uin[c + 1 + IA * sv] - Uin[c + IA * sv];
        Sy[c + IB * sv] = Uin[c + sj + IB * sv] - Uin[c + IB * sv];
        Sz[c + IC * sv] = Uin[c + sk + IC * sv] - Uin[c + IC * sv];
      }

  ORC_STAGE(STG_HALF);
  /* ComputeUpdatedPrimVarFunctor3D_MHD (MHDRunFunctors3D.h:865-1022), [g-2, size-g+1) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = g - 2; k < ksize - g + 1; ++k)
    for (int j = g - 2; j < jsize - g + 1; ++j)
      for (int i = g - 2; i < isize - g + 1; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        const double  r = Q[c + ID * sv], pr = Q[c + IP * sv], u = Q[c + IU * sv],
                     v = Q[c + IV * sv], w = Q[c + IW * sv], A = Q[c + IA * sv],
                     B = Q[c + IB * sv], C = Q[c + IC * sv];
        const double drx = Sx[c + ID * sv], dpx = Sx[c + IP * sv], dux = Sx[c + IU * sv],
                     dvx = Sx[c + IV * sv], dwx = Sx[c + IW * sv], dCx = Sx[c + IC * sv],
                     dBx = Sx[c + IB * sv];
        const double dry = Sy[c + ID * sv], dpy = Sy[c + IP * sv], duy = Sy[c + IU * sv],
                     dvy = Sy[c + IV * sv], dwy = Sy[c + IW * sv], dCy = Sy[c + IC * sv],
                     dAy = Sy[c + IA * sv];
        const double drz = Sz[c + ID * sv], dpz = Sz[c + IP * sv], duz = Sz[c + IU * sv],
                     dvz = Sz[c + IV * sv], dwz = Sz[c + IW * sv], dAz = Sz[c + IA * sv],
                     dBz = Sz[c + IB * sv];
        const double dAx = Uin[c + 1 + IA * sv] - Uin[c + IA * sv];
        const double dBy = Uin[c + sj + IB * sv] - Uin[c + IB * sv];
        const double dCz = Uin[c + sk + IC * sv] - Uin[c + IC * sv];
        const double sr0 =
          (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
        const double su0 = (-u * dux - (dpx + B * dBx + C * dCx) / r) * dtdx +
                           (-v * duy + B * dAy / r) * dtdy + (-w * duz + C * dAz / r) * dtdz;
        const double sv0 = (-u * dvx + A * dBx / r) * dtdx +
                           (-v * dvy - (dpy + A * dAy + C * dCy) / r) * dtdy +
                           (-w * dvz + C * dBz / r) * dtdz;
        const double sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + B * dCy / r) * dtdy +
                           (-w * dwz - (dpz + A * dAz + B * dBz) / r) * dtdz;
        const double sp0 = (-u * dpx - dux * gamma * pr) * dtdx +
                           (-v * dpy - dvy * gamma * pr) * dtdy +
                           (-w * dpz - dwz * gamma * pr) * dtdz;
        const double sA0 = (u * dBy + B * duy - v * dAy - A * dvy) * dtdy +
                           (u * dCz + C * duz - w * dAz - A * dwz) * dtdz;
        const double sB0 = (v * dAx + A * dvx - u * dBx - B * dux) * dtdx +
                           (v * dCz + C * dvz - w * dBz - B * dwz) * dtdz;
        const double sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx +
                           (w * dBy + B * dwy - v * dCy - C * dvy) * dtdy;
        Q2[c + ID * sv] = r + 0.5 * sr0;
        Q2[c + IU * sv] = u + 0.5 * su0;
        Q2[c + IV * sv] = v + 0.5 * sv0;
        Q2[c + IW * sv] = w + 0.5 * sw0;
        Q2[c + IP * sv] = pr + 0.5 * sp0;
        Q2[c + IA * sv] = A + 0.5 * sA0;
        Q2[c + IB * sv] = B + 0.5 * sB0;
        Q2[c + IC * sv] = C + 0.5 * sC0;
      }

  ORC_STAGE(STG_EFIELD);
  /* ComputeElecFieldFunctor3D (MHDRunFunctors3D.h:278-362), [1, size-1) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = 1; k < ksize - 1; ++k)
    for (int j = 1; j < jsize - 1; ++j)
      for (int i = 1; i < isize - 1; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        double        u, v, w, A, B, C;
        v = 0.25 * (Q[c - sj - sk + IV * sv] + Q[c - sj + IV * sv] + Q[c - sk + IV * sv] +
                    Q[c + IV * sv]);
        w = 0.25 * (Q[c - sj - sk + IW * sv] + Q[c - sj + IW * sv] + Q[c - sk + IW * sv] +
                    Q[c + IW * sv]);
        B = 0.5 * (Uin[c - sk + IB * sv] + Uin[c + IB * sv]);
        C = 0.5 * (Uin[c - sj + IC * sv] + Uin[c + IC * sv]);
        E[c] = v * C - w * B;
        u = 0.25 * (Q[c - 1 - sk + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sk + IU * sv] +
                    Q[c + IU * sv]);
        w = 0.25 * (Q[c - 1 - sk + IW * sv] + Q[c - 1 + IW * sv] + Q[c - sk + IW * sv] +
                    Q[c + IW * sv]);
        A = 0.5 * (Uin[c - sk + IA * sv] + Uin[c + IA * sv]);
        C = 0.5 * (Uin[c - 1 + IC * sv] + Uin[c + IC * sv]);
        E[c + n1] = w * A - u * C;
        u = 0.25 * (Q[c - 1 - sj + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sj + IU * sv] +
                    Q[c + IU * sv]);
        v = 0.25 * (Q[c - 1 - sj + IV * sv] + Q[c - 1 + IV * sv] + Q[c - sj + IV * sv] +
                    Q[c + IV * sv]);
        A = 0.5 * (Uin[c - sj + IA * sv] + Uin[c + IA * sv]);
        B = 0.5 * (Uin[c - 1 + IB * sv] + Uin[c + IB * sv]);
        E[c + 2 * n1] = u * B - v * A;
      }

  ORC_STAGE(STG_FACEB);
  /* ComputeSourceFaceMagFunctor3D (MHDRunFunctors3D.h:367-436), [1, size-1) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = 1; k < ksize - 1; ++k)
    for (int j = 1; j < jsize - 1; ++j)
      for (int i = 1; i < isize - 1; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        const double *Ex = E, *Ey = E + n1, *Ez = E + 2 * n1;
        sF[c] = (Ez[c + sj] - Ez[c]) * 0.5 * dtdy - (Ey[c + sk] - Ey[c]) * 0.5 * dtdz;
        sF[c + n1] = -(Ez[c + 1] - Ez[c]) * 0.5 * dtdx + (Ex[c + sk] - Ex[c]) * 0.5 * dtdz;
        sF[c + 2 * n1] = (Ey[c + 1] - Ey[c]) * 0.5 * dtdx - (Ex[c + sj] - Ex[c]) * 0.5 * dtdy;
      }

  ORC_STAGE(STG_FLUX);
  /* ComputeFluxAndUpdateAlongDirFunctor3D_MHD<dir> flux part
   * (MHDRunFunctors3D.h:1100-1253), faces [g, size-g] */
  for (int dir = 0; dir < 3; ++dir)
  {
    double       *F = Fd[dir];
    const double *S = Sd[dir];
    const int64_t off = stride[dir];
    const int     nrm = IA + dir; /* slot of the face-normal field */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
    for (int k = g; k < ksize - g + 1; ++k)
      for (int j = g; j < jsize - g + 1; ++j)
        for (int i = g; i < isize - g + 1; ++i)
        {
          const int64_t c = AT(L, i, j, k), cn = c - off;
          double        qR[NV], qL[NV], fl[NV];
          for (int v = 0; v < 5; ++v)
          {
            qR[v] = Q2[c + v * sv] - 0.5 * S[c + v * sv];
            qL[v] = Q2[cn + v * sv] + 0.5 * S[cn + v * sv];
          }
          qR[ID] = fmax(smallR, qR[ID]);
          qR[IP] = fmax(smallp * qR[ID], qR[IP]);
          qL[ID] = fmax(smallR, qL[ID]);
          qL[IP] = fmax(smallp * qL[ID], qL[IP]);
          for (int v = IA; v <= IC; ++v)
          {
            if (v == nrm)
            {
              qR[v] = Uin[c + v * sv] + sF[c + dir * n1];
              qL[v] = qR[v];
            }
            else
            {
              qR[v] = Q2[c + v * sv] - 0.5 * S[c + v * sv];
              qL[v] = Q2[cn + v * sv] + 0.5 * S[cn + v * sv];
            }
          }
          if (dir > 0)
          {
            const int tv = IU + dir, tb = IA + dir;
            double    tmp;
            tmp = qL[IU]; qL[IU] = qL[tv]; qL[tv] = tmp;
            tmp = qL[IA]; qL[IA] = qL[tb]; qL[tb] = tmp;
            tmp = qR[IU]; qR[IU] = qR[tv]; qR[tv] = tmp;
            tmp = qR[IA]; qR[IA] = qR[tb]; qR[tb] = tmp;
          }
          for (int v = 0; v < NV; ++v)
            fl[v] = 0.0;
          riemann_dispatch(p->riemann, qL, qR, fl, gamma);
          if (dir > 0)
          {
            const int tv = IU + dir, tb = IA + dir;
            double    tmp;
            tmp = fl[IU]; fl[IU] = fl[tv]; fl[tv] = tmp;
            tmp = fl[IA]; fl[IA] = fl[tb]; fl[tb] = tmp;
          }
          for (int v = 0; v < NV; ++v)
            F[c + v * sv] = fl[v];
        }
  }

  ORC_STAGE(STG_EMF);
  /* ReconstructEdgeComputeEmfAndUpdateFunctor3D<dir> (MHDRunFunctors3D.h:1331-1778),
   * edges [g, size-g]; edge direction edir, transverse directions d0 < d1. */
  for (int edir = 0; edir < 3; ++edir)
  {
    const int     d0 = edir == 0 ? 1 : 0, d1 = edir == 2 ? 1 : 2;
    const double *S0 = Sd[d0], *S1 = Sd[d1];
    const int64_t o0 = stride[d0], o1 = stride[d1];
    double       *Eo = Em + edir * n1;
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
    for (int k = g; k < ksize - g + 1; ++k)
      for (int j = g; j < jsize - g + 1; ++j)
        for (int i = g; i < isize - g + 1; ++i)
        {
          const int64_t c = AT(L, i, j, k);
          double        qe[4][NV]; /* RT, RB, LT, LB */
          /* corner state e: cell offset (-o0 if e in {RT,RB}) + (-o1 if e in {RT,LT});
           * reconstruct_state_at_edge<d0,d1> (MHDRunFunctors3D.h:1406-1529) */
          for (int e = 0; e < 4; ++e)
          {
            const int    r0 = (e == 0 || e == 1), r1 = (e == 0 || e == 2);
            const int    sdq0 = r0 ? 1 : -1, sdq1 = r1 ? 1 : -1;
            /* sign of the normal-field slopes: LB(-,-), RT(+,+), RB(-,+), LT(+,-) */
            const int    sb0 = (e == 0 || e == 2) ? 1 : -1, sb1 = (e == 0 || e == 1) ? 1 : -1;
            const int64_t cc = c - (r0 ? o0 : 0) - (r1 ? o1 : 0);
            const int64_t c0 = cc + (r0 ? o0 : 0); /* face of B_{d0} */
            const int64_t c1 = cc + (r1 ? o1 : 0); /* face of B_{d1} */
            const double B0 = Uin[c0 + (IA + d0) * sv] + sF[c0 + d0 * n1];
            const double dB0d1 = face_slope3(Uin, L, c0, IA + d0, d1, st);
            const double B1 = Uin[c1 + (IA + d1) * sv] + sF[c1 + d1 * n1];
            const double dB1d0 = face_slope3(Uin, L, c1, IA + d1, d0, st);
            double      *q = qe[e];
            for (int v = 0; v < NV; ++v)
              q[v] = Q2[cc + v * sv];
            q[ID] += 0.5 * (sdq0 * S0[cc + ID * sv] + sdq1 * S1[cc + ID * sv]);
            q[IU] += 0.5 * (sdq0 * S0[cc + IU * sv] + sdq1 * S1[cc + IU * sv]);
            q[IV] += 0.5 * (sdq0 * S0[cc + IV * sv] + sdq1 * S1[cc + IV * sv]);
            q[IW] += 0.5 * (sdq0 * S0[cc + IW * sv] + sdq1 * S1[cc + IW * sv]);
            q[IP] += 0.5 * (sdq0 * S0[cc + IP * sv] + sdq1 * S1[cc + IP * sv]);
            /* field slots in the reference's statement order (:1490-1524),
             * including the double transverse increment of IB on Y and X edges */
            if (d0 == 0)
              q[IA] = B0 + 0.5 * (sb0 * dB0d1);
            else
              q[IA] += 0.5 * (sdq0 * S0[cc + IA * sv] + sdq1 * S1[cc + IA * sv]);
            if (d0 == 1)
              q[IB] = B0 + 0.5 * (sb0 * dB0d1);
            else
              q[IB] += 0.5 * (sdq0 * S0[cc + IB * sv] + sdq1 * S1[cc + IB * sv]);
            if (d1 == 1)
              q[IB] = B1 + 0.5 * (sb1 * dB1d0);
            else
              q[IB] += 0.5 * (sdq0 * S0[cc + IB * sv] + sdq1 * S1[cc + IB * sv]);
            if (d1 == 2)
              q[IC] = B1 + 0.5 * (sb1 * dB1d0);
            else
              q[IC] += 0.5 * (sdq0 * S0[cc + IC * sv] + sdq1 * S1[cc + IC * sv]);
            q[ID] = fmax(smallR, q[ID]);
            q[IP] = fmax(smallp * q[ID], q[IP]);
          }
          if (edir == 1)
          {
            /* Y edges: RB and LT are exchanged before the solve (:1688-1698) */
            for (int v = 0; v < NV; ++v)
            {
              const double tmp = qe[1][v];
              qe[1][v] = qe[2][v];
              qe[2][v] = tmp;
            }
          }
          Eo[c] = compute_emf(edir, (const double(*)[NV])qe, gamma, p->smallc);
        }
  }

  ORC_STAGE(STG_UPDATE);
  /* update: hydro variables by X, then Y, then Z fluxes (atomic updates of
   * MHDRunFunctors3D.h:1255-1313 in serial order) */
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = g; k < ksize - g; ++k)
    for (int j = g; j < jsize - g; ++j)
      for (int i = g; i < isize - g; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        for (int v = 0; v < 5; ++v)
        {
          double x = Uout[c + v * sv];
          x += Fd[0][c + v * sv] * dtdx;
          x -= Fd[0][c + 1 + v * sv] * dtdx;
          x += Fd[1][c + v * sv] * dtdy;
          x -= Fd[1][c + sj + v * sv] * dtdy;
          x += Fd[2][c + v * sv] * dtdz;
          x -= Fd[2][c + sk + v * sv] * dtdz;
          Uout[c + v * sv] = x;
        }
      }
  /* face fields: EMF passes X, then Y, then Z (MHDRunFunctors3D.h:1638-1766).
   * Bx face (i,j,k): Y pass (+eY(k), -eY(k+1))*dtdz, Z pass (-eZ(j), +eZ(j+1))*dtdy
   * By face:         X pass (-eX(k), +eX(k+1))*dtdz, Z pass (+eZ(i), -eZ(i+1))*dtdx
   * Bz face:         X pass (+eX(j), -eX(j+1))*dtdy, Y pass (-eY(i), +eY(i+1))*dtdx
   * The reference guards every one of these updates to interior cells. */
  const double *eX = Em, *eY = Em + n1, *eZ = Em + 2 * n1;
#pragma omp parallel for collapse(2) schedule(static) num_threads(nt)
  for (int k = g; k < ksize - g; ++k)
    for (int j = g; j < jsize - g; ++j)
      for (int i = g; i < isize - g; ++i)
      {
        const int64_t c = AT(L, i, j, k);
        {
          double x = Uout[c + IA * sv];
          x += eY[c] * dtdz;
          x -= eY[c + sk] * dtdz;
          x -= eZ[c] * dtdy;
          x += eZ[c + sj] * dtdy;
          Uout[c + IA * sv] = x;
        }
        {
          double x = Uout[c + IB * sv];
          x -= eX[c] * dtdz;
          x += eX[c + sk] * dtdz;
          x += eZ[c] * dtdx;
          x -= eZ[c + 1] * dtdx;
          Uout[c + IB * sv] = x;
        }
        {
          double x = Uout[c + IC * sv];
          x += eX[c] * dtdy;
          x -= eX[c + sj] * dtdy;
          x -= eY[c] * dtdx;
          x += eY[c + 1] * dtdx;
          Uout[c + IC * sv] = x;
        }
      }
  ORC_STAGE(STG_OTHER);
}

/* SolverBase.cpp:195-220 (finished, next_iteration) and
 * SolverMHDMuscl.h:791-805 (ping-pong between U and U2) */
int
orc_run(orc_solver *s, int n)
{
  int done = 0;
  while (done < n && !(s->t >= (s->p.tEnd - 1e-14) || s->it >= s->p.nStepmax))
  {
    double *in = (s->it % 2 == 0) ? s->U : s->U2;
    double *out = (s->it % 2 == 0) ? s->U2 : s->U;
    if (s->p.dim == 2)
      step2d(s, in, out);
    else
      step3d(s, in, out);
    s->it++;
    s->t += s->dt;
    done++;
  }
  return done;
}
