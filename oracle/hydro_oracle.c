/*
 * CPU oracle: plain-C restatement of ppkMHD's hydro-only MUSCL-Hancock
 * solver (SolverHydroMuscl<2>/<3>), FP64.
 *
 * TEST INFRASTRUCTURE ONLY (the parity checker and the timed CPU baseline of
 * the hydro workload).  The product library never links or calls this file.
 *
 * Reference files restated (paths relative to the ppkMHD source tree):
 *   src/shared/HydroParams.cpp, src/shared/SolverBase.cpp,
 *   src/shared/BoundariesFunctors.h, src/shared/RiemannSolvers.h,
 *   src/muscl/HydroBaseFunctor{2D,3D}.h, src/muscl/HydroRunFunctors{2D,3D}.h,
 *   src/muscl/SolverHydroMuscl.{h,cpp}
 * Every floating-point expression keeps the reference's operation order.
 * Compile with -ffp-contract=off.
 */
#include "hydro_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#  include <omp.h>
#endif

#include "ini_text.h"

enum { ID = 0, IP = 1, IU = 2, IV = 3, IW = 4 };
#define HALF 0.5
#define MAXV 5

/* ---------------------------------------------------------------- parameters */

/* HydroParams::setup (HydroParams.cpp:27-217) for the Hydro_Muscl solvers,
 * HydroParams::init (:420-453), SolverBase::read_config's gravity switches
 * (SolverBase.cpp:138-141) and the uniform field that the Rayleigh-Taylor and
 * rising-bubble initialisations write (HydroInitFunctors2D.h:668-902,
 * HydroInitFunctors3D.h), RayleighTaylorInstabilityParams.h,
 * RisingBubbleParams.h. */
int
horc_params_from_ini(const char *ini_text, horc_params *p)
{
  ini_map m = { 0 };
  ini_parse_text(&m, ini_text);
  memset(p, 0, sizeof *p);
  const char *solver = ini_str(&m, "run", "solver_name", "unknown");
  if (!strcmp(solver, "Hydro_Muscl_2D"))
    p->dim = 2;
  else if (!strcmp(solver, "Hydro_Muscl_3D"))
    p->dim = 3;
  else
  {
    free(m.kv);
    return -1;
  }
  p->ghost = 2;
  p->nvar = p->dim == 2 ? 4 : 5;
  p->nStepmax = (int)ini_int(&m, "run", "nstepmax", 1000);
  p->tEnd = ini_float(&m, "run", "tend", 0.0f);
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
    p->bc[f] = (int)ini_int(&m, "mesh", bcn[f], 1);
  p->gamma0 = ini_float(&m, "hydro", "gamma0", 1.4f);
  p->cfl = ini_float(&m, "hydro", "cfl", 0.5f);
  p->slope_type = ini_float(&m, "hydro", "slope_type", 1.0f);
  p->smallc = ini_float(&m, "hydro", "smallc", 1e-10f);
  p->smallr = ini_float(&m, "hydro", "smallr", 1e-10f);
  const char *rs = ini_str(&m, "hydro", "riemann", "approx");
  p->riemann = !strcmp(rs, "llf")    ? HORC_LLF
               : !strcmp(rs, "hll")  ? HORC_HLL
               : !strcmp(rs, "hllc") ? HORC_HLLC
                                     : HORC_APPROX;
  p->version = (int)ini_float(&m, "OTHER", "implementationVersion", 0.0f);
  if (p->version != 0 && p->version != 1 && p->version != 2)
    p->version = 0;
  const int point = ini_bool(&m, "gravity", "point", 0);
  p->gravity = ini_bool(&m, "gravity", "static", 0) || point;
  const char *prob = ini_str(&m, "hydro", "problem", "unknown");
  if (!strcmp(prob, "disk"))
  {
    /* PointSourceGravity.h and the disk centre of DiskParams.h (mesh
     * defaults -0.5 .. 0.5 there) */
    p->point = 1;
    p->xs = ini_float(&m, "gravity", "x", 0.0f);
    p->ys = ini_float(&m, "gravity", "y", 0.0f);
    p->zs = ini_float(&m, "gravity", "z", 0.0f);
    p->GM = ini_float(&m, "gravity", "G", 1.0f) * ini_float(&m, "gravity", "M", 1.0f);
    p->eps = ini_float(&m, "gravity", "soften", 0.01f);
    const double x0 = ini_float(&m, "mesh", "xmin", -0.5f), x1 = ini_float(&m, "mesh", "xmax", 0.5f);
    const double y0 = ini_float(&m, "mesh", "ymin", -0.5f), y1 = ini_float(&m, "mesh", "ymax", 0.5f);
    const double z0 = ini_float(&m, "mesh", "zmin", -0.5f), z1 = ini_float(&m, "mesh", "zmax", 0.5f);
    p->xc = ini_float(&m, "disk", "xc", (float)((x0 + x1) / 2));
    p->yc = ini_float(&m, "disk", "yc", (float)((y0 + y1) / 2));
    p->zc = ini_float(&m, "disk", "zc", (float)((z0 + z1) / 2));
  }
  if (!strcmp(prob, "rayleigh_taylor"))
  {
    p->grav[0] = ini_float(&m, "rayleigh_taylor", "gx", 0.0f);
    p->grav[1] = ini_float(&m, "rayleigh_taylor", "gy", -0.1f);
    p->grav[2] = ini_float(&m, "rayleigh_taylor", "gz", 0.0f);
  }
  else if (!strcmp(prob, "rising_bubble"))
  {
    p->grav[0] = ini_float(&m, "rising_bubble", "gx", 0.0f);
    p->grav[1] = ini_float(&m, "rising_bubble", "gy", -0.1f);
    p->grav[2] = ini_float(&m, "rising_bubble", "gz", 0.0f);
  }
  if (p->dim == 2)
    p->grav[2] = 0.0;
  free(m.kv);
  if (p->version == 2 || (p->dim == 3 && p->riemann == HORC_HLL))
    return -1; /* version 2 and 3D HLL are not restated */

  p->isize = p->nx + 2 * p->ghost;
  p->jsize = p->ny + 2 * p->ghost;
  p->ksize = p->dim == 3 ? p->nz + 2 * p->ghost : 1;
  p->dx = (p->xmax - p->xmin) / p->nx;
  p->dy = (p->ymax - p->ymin) / p->ny;
  p->dz = (p->zmax - p->zmin) / p->nz;
  p->smallp = p->smallc * p->smallc / p->gamma0;
  p->smallpp = p->smallr * p->smallp;
  p->gamma6 = (p->gamma0 + 1.0) / (2.0 * p->gamma0);
  return 0;
}

int64_t
horc_nelem(const horc_params *p)
{
  return (int64_t)p->isize * p->jsize * p->ksize * p->nvar;
}

/* ---------------------------------------------------------------- gravity field */

/* The field the init functors write: uniform (RayleighTaylorInstabilityFunctor,
 * RisingBubbleFunctor) or, for the disk (InitDiskFunctor2D/3D,
 * HydroInitFunctors2D.h:907-1060), PointSourceGravity::eval at the cell centre
 * relative to the disk centre (z = 0 in 2D). */
void
horc_gravity_field(const horc_params *p, double *g)
{
  const int64_t sk = (int64_t)p->isize * p->jsize, sv = sk * p->ksize;
  for (int k = 0; k < p->ksize; ++k)
    for (int j = 0; j < p->jsize; ++j)
      for (int i = 0; i < p->isize; ++i)
      {
        const int64_t c = i + (int64_t)j * p->isize + k * sk;
        double        gx = p->grav[0], gy = p->grav[1], gz = p->grav[2];
        if (!p->gravity)
          gx = gy = gz = 0.0;
        else if (p->point)
        {
          const double x = p->xmin + p->dx / 2 + (i - p->ghost) * p->dx - p->xc;
          const double y = p->ymin + p->dy / 2 + (j - p->ghost) * p->dy - p->yc;
          const double z = p->dim == 3 ? p->zmin + p->dz / 2 + (k - p->ghost) * p->dz - p->zc : 0.0;
          const double r = sqrt((x - p->xs) * (x - p->xs) + (y - p->ys) * (y - p->ys) +
                                (z - p->zs) * (z - p->zs) + p->eps * p->eps);
          const double GM2 = p->GM / (r * r * r);
          gx = GM2 * (p->xs - x);
          gy = GM2 * (p->ys - y);
          gz = GM2 * (p->zs - z);
        }
        g[c] = gx;
        g[c + sv] = gy;
        if (p->dim == 3)
          g[c + 2 * sv] = gz;
      }
}

/* ---------------------------------------------------------------- indexing */

typedef struct
{
  int64_t sj, sk, sv;
} hlayout;

static inline hlayout
mk_layout(const horc_params *p)
{
  hlayout L;
  L.sj = p->isize;
  L.sk = (int64_t)p->isize * p->jsize;
  L.sv = L.sk * p->ksize;
  return L;
}

/* ---------------------------------------------------------------- boundaries */

/* MakeBoundariesFunctor2D/3D<faceId> (BoundariesFunctors.h:18-530): the X
 * faces over the full j (and k) range, then Y, then Z; reflecting walls flip
 * the normal velocity.  SolverBase::make_boundaries_serial (SolverBase.cpp:
 * 338-410) applies the faces in that order. */
static void
make_boundaries(const horc_params *p, double *U)
{
  const hlayout L = mk_layout(p);
  const int     g = p->ghost, nv = p->nvar;
  const int     n[3] = { p->nx, p->ny, p->nz };
  const int     size[3] = { p->isize, p->jsize, p->ksize };
  const int     vel[3] = { IU, IV, IW };
  const int64_t stride[3] = { 1, L.sj, L.sk };
  for (int d = 0; d < p->dim; ++d)
  {
    /* the two axes other than d, over their full ghost-inclusive range */
    const int a = d == 0 ? 1 : 0, b = d == 2 ? 1 : 2;
    const int na = size[a], nb = p->dim == 3 ? size[b] : 1;
    for (int side = 0; side < 2; ++side)
    {
      const int type = p->bc[2 * d + side];
      for (int ib = 0; ib < nb; ++ib)
        for (int ia = 0; ia < na; ++ia)
          for (int c = 0; c < g; ++c)
          {
            const int dst = side == 0 ? c : n[d] + g + c;
            int       src;
            double    sign = 1.0;
            if (type == 1)
              src = side == 0 ? 2 * g - 1 - dst : 2 * n[d] + 2 * g - 1 - dst;
            else if (type == 2)
              src = side == 0 ? g : n[d] + g - 1;
            else
              src = side == 0 ? n[d] + dst : dst - n[d];
            const int64_t base = (int64_t)ia * stride[a] + (p->dim == 3 ? (int64_t)ib * stride[b] : 0);
            for (int v = 0; v < nv; ++v)
            {
              sign = (type == 1 && v == vel[d]) ? -1.0 : 1.0;
              U[base + (int64_t)dst * stride[d] + v * L.sv] =
                U[base + (int64_t)src * stride[d] + v * L.sv] * sign;
            }
          }
    }
  }
}

/* ---------------------------------------------------------------- point-wise physics */

/* computePrimitives (HydroBaseFunctor2D.h:82-112, HydroBaseFunctor3D.h:79-117) */
static inline void
prim(const horc_params *p, const double *u, double *c, double *q)
{
  const double d = fmax(u[ID], p->smallr);
  const double ux = u[IU] / d;
  const double uy = u[IV] / d;
  double       eken;
  double       uz = 0.0;
  if (p->dim == 3)
  {
    uz = u[IW] / d;
    eken = HALF * (ux * ux + uy * uy + uz * uz);
  }
  else
    eken = HALF * (ux * ux + uy * uy);
  const double e = u[IP] / d - eken;
  const double pr = fmax((p->gamma0 - 1.0) * d * e, d * p->smallp);
  *c = sqrt(p->gamma0 * (pr) / d);
  q[ID] = d;
  q[IP] = pr;
  q[IU] = ux;
  q[IV] = uy;
  if (p->dim == 3)
    q[IW] = uz;
}

/* slope_unsplit_hydro_2d_scalar (HydroBaseFunctor2D.h:432-470) and the 3D
 * scalar version (HydroBaseFunctor3D.h:411-480): one direction */
static inline double
slope1(double slope_type, double q, double qp, double qm)
{
  const double dlft = slope_type * (q - qm);
  const double drgt = slope_type * (qp - q);
  const double dcen = HALF * (qp - qm);
  const double dsgn = (dcen >= 0.0) ? 1.0 : -1.0;
  const double slop = fmin(fabs(dlft), fabs(drgt));
  double       dlim = slop;
  if ((dlft * drgt) <= 0.0)
    dlim = 0.0;
  return dsgn * fmin(dlim, fabs(dcen));
}

/* slope_unsplit_hydro_2d/3d (HydroBaseFunctor2D.h:487-525, 3D:482-540) of
 * cell c: dq[d * 5 + v], zero for slope_type 0 */
static void
slopes(const horc_params *p, const hlayout *L, const double *Q, int64_t c, double *dq)
{
  const int64_t st[3] = { 1, L->sj, L->sk };
  for (int d = 0; d < p->dim; ++d)
    for (int v = 0; v < p->nvar; ++v)
    {
      if (p->slope_type == 0.0)
      {
        dq[d * MAXV + v] = 0.0;
        continue;
      }
      const double *Qv = Q + v * L->sv;
      dq[d * MAXV + v] = slope1(p->slope_type, Qv[c], Qv[c + st[d]], Qv[c - st[d]]);
    }
}

/* trace_unsplit_2d_along_dir (HydroBaseFunctor2D.h:225-311) and
 * trace_unsplit_3d_along_dir (HydroBaseFunctor3D.h:274-400): the state on
 * face (dir, side) of a cell, side -1 = the minus face (FACE_XMIN ...),
 * +1 = the plus face */
static void
trace_face(const horc_params *p, const double *q, const double *dq, const double dtd[3], int dir,
           int side, double *qf)
{
  const double g0 = p->gamma0;
  const double r = q[ID], pr = q[IP], u = q[IU], v = q[IV];
  const double drx = dq[0 * MAXV + ID], dpx = dq[0 * MAXV + IP], dux = dq[0 * MAXV + IU],
               dvx = dq[0 * MAXV + IV];
  const double dry = dq[1 * MAXV + ID], dpy = dq[1 * MAXV + IP], duy = dq[1 * MAXV + IU],
               dvy = dq[1 * MAXV + IV];
  double sr0, sp0, su0, sv0, sw0 = 0.0, w = 0.0;
  double dwx = 0, dwy = 0, drz = 0, dpz = 0, duz = 0, dvz = 0, dwz = 0;
  if (p->dim == 2)
  {
    sr0 = -u * drx - v * dry - (dux + dvy) * r;
    sp0 = -u * dpx - v * dpy - (dux + dvy) * g0 * pr;
    su0 = -u * dux - v * duy - (dpx) / r;
    sv0 = -u * dvx - v * dvy - (dpy) / r;
  }
  else
  {
    w = q[IW];
    dwx = dq[0 * MAXV + IW];
    dwy = dq[1 * MAXV + IW];
    drz = dq[2 * MAXV + ID];
    dpz = dq[2 * MAXV + IP];
    duz = dq[2 * MAXV + IU];
    dvz = dq[2 * MAXV + IV];
    dwz = dq[2 * MAXV + IW];
    sr0 = -u * drx - v * dry - w * drz - (dux + dvy + dwz) * r;
    sp0 = -u * dpx - v * dpy - w * dpz - (dux + dvy + dwz) * g0 * pr;
    su0 = -u * dux - v * duy - w * duz - (dpx) / r;
    sv0 = -u * dvx - v * dvy - w * dvz - (dpy) / r;
    sw0 = -u * dwx - v * dwy - w * dwz - (dpz) / r;
  }
  const double t = dtd[dir];
  const double dr = dir == 0 ? drx : dir == 1 ? dry : drz;
  const double dp = dir == 0 ? dpx : dir == 1 ? dpy : dpz;
  const double du = dir == 0 ? dux : dir == 1 ? duy : duz;
  const double dv = dir == 0 ? dvx : dir == 1 ? dvy : dvz;
  const double dw = dir == 0 ? dwx : dir == 1 ? dwy : dwz;
  if (side < 0)
  {
    qf[ID] = r - HALF * dr + sr0 * t * HALF;
    qf[IP] = pr - HALF * dp + sp0 * t * HALF;
    qf[IU] = u - HALF * du + su0 * t * HALF;
    qf[IV] = v - HALF * dv + sv0 * t * HALF;
    if (p->dim == 3)
      qf[IW] = w - HALF * dw + sw0 * t * HALF;
  }
  else
  {
    qf[ID] = r + HALF * dr + sr0 * t * HALF;
    qf[IP] = pr + HALF * dp + sp0 * t * HALF;
    qf[IU] = u + HALF * du + su0 * t * HALF;
    qf[IV] = v + HALF * dv + sv0 * t * HALF;
    if (p->dim == 3)
      qf[IW] = w + HALF * dw + sw0 * t * HALF;
  }
  qf[ID] = fmax(p->smallr, qf[ID]);
}

/* cmpflx (RiemannSolvers.h:19-48) */
static void
cmpflx(const horc_params *p, const double *qg, double *flux)
{
  flux[ID] = qg[ID] * qg[IU];
  flux[IU] = flux[ID] * qg[IU] + qg[IP];
  flux[IV] = flux[ID] * qg[IV];
  if (p->dim == 3)
    flux[IW] = flux[ID] * qg[IW];
  const double entho = 1.0 / (p->gamma0 - 1.0);
  double       ekin = HALF * qg[ID] * (qg[IU] * qg[IU] + qg[IV] * qg[IV]);
  if (p->dim == 3)
    ekin += HALF * qg[ID] * (qg[IW] * qg[IW]);
  const double etot = qg[IP] * entho + ekin;
  flux[IP] = qg[IU] * (etot + qg[IP]);
}

/* riemann_approx (RiemannSolvers.h:50-199) */
static void
riemann_approx(const horc_params *p, const double *ql_, const double *qr_, double *flux)
{
  const double gamma0 = p->gamma0, gamma6 = p->gamma6, smallr = p->smallr, smallc = p->smallc,
               smallp = p->smallp, smallpp = p->smallpp;
  const double rl = fmax(ql_[ID], smallr);
  const double ul = ql_[IU];
  const double pl = fmax(ql_[IP], rl * smallp);
  const double rr = fmax(qr_[ID], smallr);
  const double ur = qr_[IU];
  const double pr = fmax(qr_[IP], rr * smallp);
  const double cl = gamma0 * pl * rl;
  const double cr = gamma0 * pr * rr;
  double       wl = sqrt(cl);
  double       wr = sqrt(cr);
  double       pstar = fmax(((wr * pl + wl * pr) + wl * wr * (ul - ur)) / (wl + wr), 0.0);
  double       pold = pstar;
  double       conv = 1.0;
  for (int iter = 0; (iter < 10) && (conv > 1e-6); ++iter)
  {
    const double wwl = sqrt(cl * (1.0 + gamma6 * (pold - pl) / pl));
    const double wwr = sqrt(cr * (1.0 + gamma6 * (pold - pr) / pr));
    const double qlw = 2.0 * wwl * wwl * wwl / (wwl * wwl + cl);
    const double qrw = 2.0 * wwr * wwr * wwr / (wwr * wwr + cr);
    const double usl = ul - (pold - pl) / wwl;
    const double usr = ur + (pold - pr) / wwr;
    const double delp = fmax(qrw * qlw / (qrw + qlw) * (usl - usr), -pold);
    pold = pold + delp;
    conv = fabs(delp / (pold + smallpp));
  }
  pstar = pold;
  wl = sqrt(cl * (1.0 + gamma6 * (pstar - pl) / pl));
  wr = sqrt(cr * (1.0 + gamma6 * (pstar - pr) / pr));
  const double ustar = HALF * (ul + (pl - pstar) / wl + ur - (pr - pstar) / wr);
  const double sgnm = copysign(1.0, ustar);
  double       ro, uo, po, wo;
  if (sgnm > 0.0)
  {
    ro = rl;
    uo = ul;
    po = pl;
    wo = wl;
  }
  else
  {
    ro = rr;
    uo = ur;
    po = pr;
    wo = wr;
  }
  const double co = fmax(smallc, sqrt(fabs(gamma0 * po / ro)));
  const double rstar = fmax(ro / (1.0 + ro * (po - pstar) / (wo * wo)), smallr);
  const double cstar = fmax(smallc, sqrt(fabs(gamma0 * pstar / rstar)));
  double       spout = co - sgnm * uo;
  double       spin = cstar - sgnm * ustar;
  const double ushock = wo / ro - sgnm * uo;
  if (pstar >= po)
  {
    spin = ushock;
    spout = ushock;
  }
  const double scr = fmax(spout - spin, smallc + fabs(spout + spin));
  double       frac = HALF * (1.0 + (spout + spin) / scr);
  if (frac != frac)
    frac = 0.0;
  else
    frac = frac >= 1.0 ? 1.0 : frac <= 0.0 ? 0.0 : frac;
  double qg[MAXV];
  qg[ID] = frac * rstar + (1.0 - frac) * ro;
  qg[IU] = frac * ustar + (1.0 - frac) * uo;
  qg[IP] = frac * pstar + (1.0 - frac) * po;
  if (spout < 0.0)
  {
    qg[ID] = ro;
    qg[IU] = uo;
    qg[IP] = po;
  }
  if (spin > 0.0)
  {
    qg[ID] = rstar;
    qg[IU] = ustar;
    qg[IP] = pstar;
  }
  if (sgnm > 0.0)
  {
    qg[IV] = ql_[IV];
    if (p->dim == 3)
      qg[IW] = ql_[IW];
  }
  else
  {
    qg[IV] = qr_[IV];
    if (p->dim == 3)
      qg[IW] = qr_[IW];
  }
  cmpflx(p, qg, flux);
}

/* conservative variables and physical fluxes of riemann_llf / riemann_hll
 * (RiemannSolvers.h:249-309, :374-425); hll takes fleft[ID] = uleft[IU] */
static void
cons_and_flux(const horc_params *p, const double *q, double entho, int hll, double *u, double *f)
{
  u[ID] = q[ID];
  u[IP] = q[IP] * entho + HALF * q[ID] * q[IU] * q[IU];
  u[IP] += HALF * q[ID] * q[IV] * q[IV];
  if (p->dim == 3)
    u[IP] += HALF * q[ID] * q[IW] * q[IW];
  u[IU] = q[ID] * q[IU];
  u[IV] = q[ID] * q[IV];
  if (p->dim == 3)
    u[IW] = q[ID] * q[IW];
  f[ID] = hll ? u[IU] : u[ID] * q[IU];
  f[IP] = q[IU] * (u[IP] + q[IP]);
  f[IU] = q[IP] + u[IU] * q[IU];
  f[IV] = f[ID] * q[IV];
  if (p->dim == 3)
    f[IW] = f[ID] * q[IW];
}

/* riemann_llf (RiemannSolvers.h:201-327) */
static void
riemann_llf(const horc_params *p, const double *ql, const double *qr, double *flux)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp;
  const double entho = 1.0 / (gamma0 - 1.0);
  const double rl = fmax(ql[ID], smallr);
  const double ul = ql[IU];
  const double pl = fmax(ql[IP], rl * smallp);
  const double rr = fmax(qr[ID], smallr);
  const double ur = qr[IU];
  const double pr = fmax(qr[IP], rr * smallp);
  const double cl = sqrt(gamma0 * pl / rl);
  const double cr = sqrt(gamma0 * pr / rr);
  const double cmax = fmax(fabs(ul) + cl, fabs(ur) + cr);
  double       uleft[MAXV], uright[MAXV], fleft[MAXV], fright[MAXV];
  cons_and_flux(p, ql, entho, 0, uleft, fleft);
  cons_and_flux(p, qr, entho, 0, uright, fright);
  for (int v = 0; v < p->nvar; ++v)
    flux[v] = HALF * (fleft[v] + fright[v] - cmax * (uright[v] - uleft[v]));
}

/* riemann_hll (RiemannSolvers.h:329-435) */
static void
riemann_hll(const horc_params *p, const double *ql, const double *qr, double *flux)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp;
  const double entho = 1.0 / (gamma0 - 1.0);
  const double rl = fmax(ql[ID], smallr);
  const double ul = ql[IU];
  const double pl = fmax(ql[IP], rl * smallp);
  const double rr = fmax(qr[ID], smallr);
  const double ur = qr[IU];
  const double pr = fmax(qr[IP], rr * smallp);
  const double cl = sqrt(gamma0 * pl / rl);
  const double cr = sqrt(gamma0 * pr / rr);
  const double SL = fmin(fmin(ul, ur) - fmax(cl, cr), 0.0);
  const double SR = fmax(fmax(ul, ur) + fmax(cl, cr), 0.0);
  double       uleft[MAXV], uright[MAXV], fleft[MAXV], fright[MAXV];
  cons_and_flux(p, ql, entho, 1, uleft, fleft);
  cons_and_flux(p, qr, entho, 1, uright, fright);
  for (int v = 0; v < p->nvar; ++v)
    flux[v] = (SR * fleft[v] - SL * fright[v] + SR * SL * (uright[v] - uleft[v])) / (SR - SL);
}

/* riemann_hllc (RiemannSolvers.h:437-568) */
static void
riemann_hllc(const horc_params *p, const double *ql, const double *qr, double *flux)
{
  const double gamma0 = p->gamma0, smallr = p->smallr, smallp = p->smallp, smallc = p->smallc;
  const double entho = 1.0 / (gamma0 - 1.0);
  const double rl = fmax(ql[ID], smallr);
  const double pl = fmax(ql[IP], rl * smallp);
  const double ul = ql[IU];
  double       ecinl = HALF * rl * ul * ul;
  ecinl += HALF * rl * ql[IV] * ql[IV];
  if (p->dim == 3)
    ecinl += HALF * rl * ql[IW] * ql[IW];
  const double etotl = pl * entho + ecinl;
  const double ptotl = pl;
  const double rr = fmax(qr[ID], smallr);
  const double pr = fmax(qr[IP], rr * smallp);
  const double ur = qr[IU];
  double       ecinr = HALF * rr * ur * ur;
  ecinr += HALF * rr * qr[IV] * qr[IV];
  if (p->dim == 3)
    ecinr += HALF * rr * qr[IW] * qr[IW];
  const double etotr = pr * entho + ecinr;
  const double ptotr = pr;
  const double cfastl = sqrt(fmax(gamma0 * pl / rl, smallc * smallc));
  const double cfastr = sqrt(fmax(gamma0 * pr / rr, smallc * smallc));
  const double SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  const double SR = fmax(ul, ur) + fmax(cfastl, cfastr);
  const double rcl = rl * (ul - SL);
  const double rcr = rr * (SR - ur);
  const double ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
  const double ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
  const double rstarl = rl * (SL - ul) / (SL - ustar);
  const double etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
  const double rstarr = rr * (SR - ur) / (SR - ustar);
  const double etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
  double       ro, uo, ptoto, etoto;
  if (SL > 0.0)
  {
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (ustar > 0.0)
  {
    ro = rstarl;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarl;
  }
  else if (SR > 0.0)
  {
    ro = rstarr;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarr;
  }
  else
  {
    ro = rr;
    uo = ur;
    ptoto = ptotr;
    etoto = etotr;
  }
  flux[ID] = ro * uo;
  flux[IU] = ro * uo * uo + ptoto;
  flux[IP] = (etoto + ptoto) * uo;
  flux[IV] = flux[ID] > 0.0 ? flux[ID] * ql[IV] : flux[ID] * qr[IV];
  if (p->dim == 3)
    flux[IW] = flux[ID] > 0.0 ? flux[ID] * ql[IW] : flux[ID] * qr[IW];
}

/* riemann_hydro (RiemannSolvers.h:570-633) */
void
horc_riemann(const horc_params *p, const double *qL, const double *qR, double *flux)
{
  if (p->riemann == HORC_HLL)
    riemann_hll(p, qL, qR, flux);
  else if (p->riemann == HORC_HLLC)
    riemann_hllc(p, qL, qR, flux);
  else if (p->riemann == HORC_LLF)
    riemann_llf(p, qL, qR, flux);
  else
    riemann_approx(p, qL, qR, flux);
}

/* ---------------------------------------------------------------- solver */

struct horc_solver
{
  horc_params P;
  double     *U, *U2, *Q, *F[3], *g; /* g: gravity field, dim planes */
  double      t, dt;
  int         it, nthreads;
};

horc_solver *
horc_create(const horc_params *p, int nthreads)
{
  horc_solver *s = (horc_solver *)calloc(1, sizeof *s);
  s->P = *p;
  const size_t n = (size_t)horc_nelem(p);
  s->U = (double *)calloc(n, sizeof(double));
  s->U2 = (double *)calloc(n, sizeof(double));
  s->Q = (double *)calloc(n, sizeof(double));
  for (int d = 0; d < p->dim; ++d)
    s->F[d] = (double *)calloc(n, sizeof(double));
  s->g = (double *)calloc((size_t)p->isize * p->jsize * p->ksize * p->dim, sizeof(double));
  horc_gravity_field(p, s->g);
  s->t = p->tCurrent;
  s->nthreads = nthreads > 0 ? nthreads : 1;
  return s;
}

void
horc_destroy(horc_solver *s)
{
  if (!s)
    return;
  free(s->U);
  free(s->U2);
  free(s->Q);
  for (int d = 0; d < 3; ++d)
    free(s->F[d]);
  free(s->g);
  free(s);
}

/* ComputeDtFunctor2D/3D (HydroRunFunctors2D.h:13-82, 3D:14-88) and
 * ComputeDtGravityFunctor2D/3D (2D:84-175, 3D:90-190) over interior cells,
 * then dt = cfl / invDt (SolverHydroMuscl.h:649-690) clipped to tEnd
 * (SolverBase.cpp:148-179) */
static void
compute_dt(horc_solver *s)
{
  const horc_params *p = &s->P;
  const hlayout      L = mk_layout(p);
  const double      *U = (s->it % 2 == 0) ? s->U : s->U2;
  const int          g = p->ghost;
  const int          k0 = p->dim == 3 ? g : 0, k1 = p->dim == 3 ? p->ksize - g : 1;
  double             dxg = fmin(p->dx, p->dy);
  if (p->dim == 3)
    dxg = fmin(dxg, p->dz);
  double invDt = 0.0;
#pragma omp parallel for reduction(max : invDt) num_threads(s->nthreads) collapse(2)
  for (int k = k0; k < k1; ++k)
    for (int j = g; j < p->jsize - g; ++j)
      for (int i = g; i < p->isize - g; ++i)
      {
        const int64_t c = i + j * L.sj + k * L.sk;
        double        u[MAXV], q[MAXV], cs;
        for (int v = 0; v < p->nvar; ++v)
          u[v] = U[c + v * L.sv];
        prim(p, u, &cs, q);
        double val;
        if (p->gravity)
        {
          double velocity = 0.0;
          velocity += cs + fabs(q[IU]);
          velocity += cs + fabs(q[IV]);
          if (p->dim == 3)
            velocity += cs + fabs(q[IW]);
          const double *gf = s->g;
          double kk = fabs(gf[c]) + fabs(gf[c + L.sv]);
          if (p->dim == 3)
            kk = kk + fabs(gf[c + 2 * L.sv]);
          kk *= p->cfl * dxg / (velocity * velocity);
          kk = fmax(kk, 1e-4);
          velocity *= kk / (sqrt(1.0 + 2.0 * kk) - 1.0);
          val = velocity / dxg;
        }
        else
        {
          const double vx = cs + fabs(q[IU]);
          const double vy = cs + fabs(q[IV]);
          if (p->dim == 3)
          {
            const double vz = cs + fabs(q[IW]);
            val = vx / p->dx + vy / p->dy + vz / p->dz;
          }
          else
            val = vx / p->dx + vy / p->dy;
        }
        invDt = fmax(invDt, val);
      }
  s->dt = p->cfl / invDt;
  if (s->t + s->dt > p->tEnd)
    s->dt = p->tEnd - s->t;
}

void
horc_set_state(horc_solver *s, const double *U)
{
  const size_t n = (size_t)horc_nelem(&s->P);
  memcpy(s->U, U, n * sizeof(double));
  make_boundaries(&s->P, s->U);
  memcpy(s->U2, s->U, n * sizeof(double));
  s->it = 0;
  s->t = s->P.tCurrent;
  compute_dt(s);
}

void
horc_get_state(const horc_solver *s, double *U)
{
  memcpy(U, (s->it % 2 == 0) ? s->U : s->U2, (size_t)horc_nelem(&s->P) * sizeof(double));
}

void
horc_time(const horc_solver *s, double *t, double *dt, int *iteration)
{
  if (t)
    *t = s->t;
  if (dt)
    *dt = s->dt;
  if (iteration)
    *iteration = s->it;
}

/* godunov_unsplit_impl (SolverHydroMuscl.cpp:257-320 / :327-400), version 0:
 * boundaries of data_in, data_out = data_in, primitives over the whole array
 * (ConvertToPrimitivesFunctor2D/3D), ComputeAndStoreFluxesFunctor2D/3D
 * (HydroRunFunctors2D.h:490-755, 3D:300-705), UpdateFunctor2D/3D, then the
 * gravity source term (GravitySourceTermFunctor2D/3D). */
static void
godunov(horc_solver *s, double *in, double *out, double dt)
{
  const horc_params *p = &s->P;
  const hlayout      L = mk_layout(p);
  const int          g = p->ghost, nv = p->nvar, dim = p->dim;
  const size_t       n = (size_t)horc_nelem(p);
  make_boundaries(p, in);
  memcpy(out, in, n * sizeof(double));
  const int64_t ncell = (int64_t)p->isize * p->jsize * p->ksize;
#pragma omp parallel for num_threads(s->nthreads)
  for (int64_t c = 0; c < ncell; ++c)
  {
    double u[MAXV], q[MAXV], cs;
    for (int v = 0; v < nv; ++v)
      u[v] = in[c + v * L.sv];
    prim(p, u, &cs, q);
    for (int v = 0; v < nv; ++v)
      s->Q[c + v * L.sv] = q[v];
  }
  const double  dtd[3] = { dt / p->dx, dt / p->dy, dt / p->dz };
  const int64_t st[3] = { 1, L.sj, L.sk };
  const int     k0 = dim == 3 ? g : 0, k1 = dim == 3 ? p->ksize - g : 0;
  /* faces of cells [g, size-g] (inclusive) along each axis */
#pragma omp parallel for num_threads(s->nthreads) collapse(2)
  for (int k = k0; k <= k1; ++k)
    for (int j = g; j <= p->jsize - g; ++j)
      for (int i = g; i <= p->isize - g; ++i)
      {
        const int64_t c = i + j * L.sj + k * L.sk;
        double        qc[MAXV], dqc[3 * MAXV];
        for (int v = 0; v < nv; ++v)
          qc[v] = s->Q[c + v * L.sv];
        slopes(p, &L, s->Q, c, dqc);
        for (int d = 0; d < dim; ++d)
        {
          const int64_t nb = c - st[d];
          double        qn[MAXV], dqn[3 * MAXV], qleft[MAXV], qright[MAXV], flux[MAXV];
          for (int v = 0; v < nv; ++v)
            qn[v] = s->Q[nb + v * L.sv];
          slopes(p, &L, s->Q, nb, dqn);
          trace_face(p, qc, dqc, dtd, d, -1, qright);
          trace_face(p, qn, dqn, dtd, d, +1, qleft);
          if (p->gravity)
          {
            /* gravity predictor (half time step), the field at each cell */
            const double *gf = s->g;
            qleft[IU] += 0.5 * dt * gf[nb];
            qleft[IV] += 0.5 * dt * gf[nb + L.sv];
            if (dim == 3)
              qleft[IW] += 0.5 * dt * gf[nb + 2 * L.sv];
            /* version 1 in 3D gives the right state of z faces no
             * predictor (HydroRunFunctors3D.h:1344-1346, where the x and y
             * faces have it at :1198-1206 and :1272-1280) */
            if (!(p->version == 1 && dim == 3 && d == 2))
            {
              qright[IU] += 0.5 * dt * gf[c];
              qright[IV] += 0.5 * dt * gf[c + L.sv];
              if (dim == 3)
                qright[IW] += 0.5 * dt * gf[c + 2 * L.sv];
            }
          }
          /* rotate to the face-normal frame: swap the normal velocity into IU */
          const int vn = d == 0 ? IU : d == 1 ? IV : IW;
          if (d > 0)
          {
            double x = qleft[IU];
            qleft[IU] = qleft[vn];
            qleft[vn] = x;
            x = qright[IU];
            qright[IU] = qright[vn];
            qright[vn] = x;
          }
          horc_riemann(p, qleft, qright, flux);
          double *F = s->F[d];
          for (int v = 0; v < nv; ++v)
          {
            const int src = v == IU ? vn : v == vn ? IU : v;
            F[c + v * L.sv] = flux[src] * dtd[d];
          }
        }
      }
  const int kk0 = dim == 3 ? g : 0, kk1 = dim == 3 ? p->ksize - g : 1;
#pragma omp parallel for num_threads(s->nthreads) collapse(2)
  for (int k = kk0; k < kk1; ++k)
    for (int j = g; j < p->jsize - g; ++j)
      for (int i = g; i < p->isize - g; ++i)
      {
        const int64_t c = i + j * L.sj + k * L.sk;
        for (int v = 0; v < nv; ++v)
        {
          double x = out[c + v * L.sv];
          for (int d = 0; d < dim; ++d)
          {
            x += s->F[d][c + v * L.sv];
            x -= s->F[d][c + st[d] + v * L.sv];
          }
          out[c + v * L.sv] = x;
        }
        if (p->gravity)
        {
          /* GravitySourceTermFunctor2D (HydroRunFunctors2D.h:1262-1340,
           * rhoNew floored at smallr) / 3D (HydroRunFunctors3D.h:1440-1510,
           * not floored) */
          const double rhoOld = in[c + ID * L.sv];
          const double rhoNew = dim == 2 ? fmax(p->smallr, out[c + ID * L.sv]) : out[c + ID * L.sv];
          double       rhou = out[c + IU * L.sv];
          double       rhov = out[c + IV * L.sv];
          double       rhow = dim == 3 ? out[c + IW * L.sv] : 0.0;
          double       ekin_old;
          if (dim == 3)
            ekin_old = 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rhoNew;
          else
            ekin_old = 0.5 * (rhou * rhou + rhov * rhov) / rhoNew;
          const double *gf = s->g;
          rhou += 0.5 * dt * gf[c] * (rhoOld + rhoNew);
          rhov += 0.5 * dt * gf[c + L.sv] * (rhoOld + rhoNew);
          if (dim == 3)
            rhow += 0.5 * dt * gf[c + 2 * L.sv] * (rhoOld + rhoNew);
          out[c + IU * L.sv] = rhou;
          out[c + IV * L.sv] = rhov;
          if (dim == 3)
            out[c + IW * L.sv] = rhow;
          double ekin_new;
          if (dim == 3)
            ekin_new = 0.5 * (rhou * rhou + rhov * rhov + rhow * rhow) / rhoNew;
          else
            ekin_new = 0.5 * (rhou * rhou + rhov * rhov) / rhoNew;
          out[c + IP * L.sv] += (ekin_new - ekin_old);
        }
      }
}

/* main loop (main.cpp:154-159): while !finished(): next_iteration ->
 * next_iteration_impl (SolverHydroMuscl.h:695-735: compute_dt, then
 * godunov_unsplit(m_dt) ping-ponging U and U2), m_iteration++, m_t += m_dt
 * (SolverBase.cpp:205-220) */
int
horc_run(horc_solver *s, int n)
{
  int done = 0;
  while (done < n && !(s->t >= (s->P.tEnd - 1e-14) || s->it >= s->P.nStepmax))
  {
    compute_dt(s);
    if (s->it % 2 == 0)
      godunov(s, s->U, s->U2, s->dt);
    else
      godunov(s, s->U2, s->U, s->dt);
    s->it += 1;
    s->t += s->dt;
    ++done;
  }
  return done;
}
