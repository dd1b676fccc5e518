// Kernels of one iteration of the hydro-only MUSCL-Hancock solver
// (ppkMHD's SolverHydroMuscl<dim>, solver names Hydro_Muscl_2D/3D),
// templated on the real type R and the dimension DIM (NVAR = DIM + 2
// conservative variables: rho, E, rho u, rho v[, rho w]; ghost width 2).
//
// One iteration is 7 launches on one stream, every face flux computed once
// by one thread and every cell updated by the thread that owns it (gather
// form, no atomics except the CFL maximum, bitwise deterministic):
//
//   k_hbound     ghost fill of U_in (periodic / reflecting / outflow)
//   k_hprim_dt   primitives Q over the whole array + CFL max-reduction
//   k_hfinalize  dt = cfl / max, clipped to tEnd; dt/dx, dt/dy, dt/dz
//   k_hslopes    limited slopes S_d and trace source terms of every cell the
//                faces read
//   k_hflux      per face: both traced states, gravity predictor, Riemann
//                solver (approx / LLF / HLL / HLLC), flux * dt/dx stored
//   k_hupdate    U_out = U_in + flux differences (interior), gravity source
//                term; ghost cells copied (the reference's deep_copy)
//   k_advance    iteration += 1, t += dt
//
// Implementation versions 0 (ComputeAndStoreFluxes + Update) and 1 (stored
// slopes, per-direction trace/flux/update) compute the same face fluxes from
// the same slopes and apply the same additions in the same order, so both
// run these kernels; their one difference (version 1 in 3D gives the right
// state of z faces no gravity predictor) is a flag of k_hflux.
//
// Device layout: SoA planes, i fastest, ghost cells included:
//   U[i + isize*(j + jsize*(k + ksize*var))]   (Kokkos LayoutLeft)
#pragma once

#include <cstdint>
#include <type_traits>
#include <cuda_runtime.h>

#include "mhd_kernels.cuh"

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{
namespace hydro
{

constexpr int MAXV = 5;

template <class R>
struct HGrid
{
  int     dim, nx, ny, nz, g, nvar;
  int     isize, jsize, ksize;
  int64_t sj, sk, sv;
  int     bc[6];
  int     riemann;   // MHD_RIEMANN_APPROX / LLF / HLL / HLLC
  int     gravity;   // [gravity] static or point: the predictor and source terms
  int     zgrav_right; // 0: version 1 in 3D (no predictor on the right state of z faces)
  R       gamma0, gamma6, smallr, smallc, smallp, smallpp, slope_type, entho;
  const R * gf;      // gravity field (dim planes of sv cells) when gravity is on
  double  cfl, dx, dy, dz, dxg; // dxg = min(dx, dy[, dz]) (ComputeDtGravityFunctor)
  double  idx, idy, idz, idxg;  // host IEEE reciprocals
  Box     box[BOX_COUNT];
};

template <class R>
__device__ __forceinline__ int64_t
hcell(const HGrid<R> & G, int i, int j, int k)
{
  return (int64_t)i + (int64_t)j * G.sj + (int64_t)k * G.sk;
}

// Quotient of the builds: the FMA-free FP64 build divides as the reference
// does (IEEE); the fast builds multiply by the approximate reciprocal (FP64:
// rcp with one third-order refinement, within 0.51 ulp; FP32: rcp.approx).
template <class R>
__device__ __forceinline__ R
hdiv(R a, R b)
{
  if constexpr (kExactOrder)
    return a / b;
  else
    return a * rcp(b);
}
template <class R>
__device__ __forceinline__ R
hsqrt(R x)
{
  if constexpr (kExactOrder)
    return sqrt(x);
  else
    return fsqrt(x);
}

// ---------------------------------------------------------------- point-wise physics

// computePrimitives (HydroBaseFunctor2D.h:82-112, HydroBaseFunctor3D.h:79-117):
// q = (rho, p, u, v[, w]) and the sound speed c
template <class R, int DIM>
__device__ __forceinline__ void
hprim(const HGrid<R> & G, const R * u, R & c, R * q)
{
  const R d = fmax(u[ID], G.smallr);
  R       ux, uy, uz = R(0), eken, e;
  if constexpr (kExactOrder)
  {
    ux = u[IU] / d;
    uy = u[IV] / d;
    if constexpr (DIM == 3)
    {
      uz = u[IW] / d;
      eken = R(0.5) * (ux * ux + uy * uy + uz * uz);
    }
    else
      eken = R(0.5) * (ux * ux + uy * uy);
    e = u[IP] / d - eken;
  }
  else
  {
    const R id = rcp(d);
    ux = u[IU] * id;
    uy = u[IV] * id;
    if constexpr (DIM == 3)
    {
      uz = u[IW] * id;
      eken = R(0.5) * (ux * ux + uy * uy + uz * uz);
    }
    else
      eken = R(0.5) * (ux * ux + uy * uy);
    e = u[IP] * id - eken;
  }
  const R p = fmax((G.gamma0 - R(1)) * d * e, d * G.smallp);
  c = hsqrt(hdiv(G.gamma0 * (p), d));
  q[ID] = d;
  q[IP] = p;
  q[IU] = ux;
  q[IV] = uy;
  if constexpr (DIM == 3)
    q[IW] = uz;
}

// Source terms of the half-step prediction of trace_unsplit_2d_along_dir
// (HydroBaseFunctor2D.h:225-311) / trace_unsplit_3d_along_dir
// (HydroBaseFunctor3D.h:274-400): sr0, sp0, su0, sv0[, sw0] of a cell from
// its primitives q and limited slopes dq[d][v].  They do not depend on the
// face, so each cell's are computed once (by the slopes stage) for its 2 DIM
// face states; the expressions are the reference's, so the values are the
// ones every trace call of the reference recomputes.
template <class R, int DIM>
__device__ __forceinline__ void
hsources(const HGrid<R> & G, const R * q, const R (*dq)[MAXV], R * src)
{
  const R r = q[ID], p = q[IP], u = q[IU], v = q[IV];
  if constexpr (DIM == 2)
  {
    src[ID] = -u * dq[0][ID] - v * dq[1][ID] - (dq[0][IU] + dq[1][IV]) * r;
    src[IP] = -u * dq[0][IP] - v * dq[1][IP] - (dq[0][IU] + dq[1][IV]) * G.gamma0 * p;
    if constexpr (kExactOrder)
    {
      src[IU] = -u * dq[0][IU] - v * dq[1][IU] - (dq[0][IP]) / r;
      src[IV] = -u * dq[0][IV] - v * dq[1][IV] - (dq[1][IP]) / r;
    }
    else
    {
      const R ir = rcp(r);
      src[IU] = -u * dq[0][IU] - v * dq[1][IU] - dq[0][IP] * ir;
      src[IV] = -u * dq[0][IV] - v * dq[1][IV] - dq[1][IP] * ir;
    }
  }
  else
  {
    const R w = q[IW];
    src[ID] =
      -u * dq[0][ID] - v * dq[1][ID] - w * dq[2][ID] - (dq[0][IU] + dq[1][IV] + dq[2][IW]) * r;
    src[IP] = -u * dq[0][IP] - v * dq[1][IP] - w * dq[2][IP] -
              (dq[0][IU] + dq[1][IV] + dq[2][IW]) * G.gamma0 * p;
    if constexpr (kExactOrder)
    {
      src[IU] = -u * dq[0][IU] - v * dq[1][IU] - w * dq[2][IU] - (dq[0][IP]) / r;
      src[IV] = -u * dq[0][IV] - v * dq[1][IV] - w * dq[2][IV] - (dq[1][IP]) / r;
      src[IW] = -u * dq[0][IW] - v * dq[1][IW] - w * dq[2][IW] - (dq[2][IP]) / r;
    }
    else
    {
      const R ir = rcp(r);
      src[IU] = -u * dq[0][IU] - v * dq[1][IU] - w * dq[2][IU] - dq[0][IP] * ir;
      src[IV] = -u * dq[0][IV] - v * dq[1][IV] - w * dq[2][IV] - dq[1][IP] * ir;
      src[IW] = -u * dq[0][IW] - v * dq[1][IW] - w * dq[2][IW] - dq[2][IP] * ir;
    }
  }
}

// The face state of trace_unsplit_*_along_dir on the minus (MINUS) or plus
// face of a cell: q -/+ dq_DIR / 2 + src * t / 2 with t = dt/dx_DIR, density
// floored at smallr.
template <class R, int DIM, bool MINUS>
__device__ __forceinline__ void
htrace(const HGrid<R> & G, const R * q, const R * d, const R * src, R t, R * qf)
{
#pragma unroll
  for (int v = 0; v < DIM + 2; ++v)
  {
    if constexpr (MINUS)
      qf[v] = q[v] - R(0.5) * d[v] + src[v] * t * R(0.5);
    else
      qf[v] = q[v] + R(0.5) * d[v] + src[v] * t * R(0.5);
  }
  qf[ID] = fmax(G.smallr, qf[ID]);
}

// cmpflx (RiemannSolvers.h:19-48)
template <class R, int DIM>
__device__ __forceinline__ void
hcmpflx(const HGrid<R> & G, const R * qg, R * flux)
{
  flux[ID] = qg[ID] * qg[IU];
  flux[IU] = flux[ID] * qg[IU] + qg[IP];
  flux[IV] = flux[ID] * qg[IV];
  if constexpr (DIM == 3)
    flux[IW] = flux[ID] * qg[IW];
  R ekin = R(0.5) * qg[ID] * (qg[IU] * qg[IU] + qg[IV] * qg[IV]);
  if constexpr (DIM == 3)
    ekin += R(0.5) * qg[ID] * (qg[IW] * qg[IW]);
  const R etot = qg[IP] * G.entho + ekin;
  flux[IP] = qg[IU] * (etot + qg[IP]);
}

// riemann_approx (RiemannSolvers.h:50-199): two-shock approximate solver,
// Newton iterations on the star pressure (at most 10, to |dp / p| <= 1e-6)
template <class R, int DIM>
__device__ __forceinline__ void
riemann_approx(const HGrid<R> & G, const R * ql, const R * qr, R * flux)
{
  const R gamma0 = G.gamma0, gamma6 = G.gamma6, smallr = G.smallr, smallc = G.smallc;
  const R rl = fmax(ql[ID], smallr);
  const R ul = ql[IU];
  const R pl = fmax(ql[IP], rl * G.smallp);
  const R rr = fmax(qr[ID], smallr);
  const R ur = qr[IU];
  const R pr = fmax(qr[IP], rr * G.smallp);
  const R cl = gamma0 * pl * rl;
  const R cr = gamma0 * pr * rr;
  R       wl = hsqrt(cl);
  R       wr = hsqrt(cr);
  R       pstar = fmax(hdiv((wr * pl + wl * pr) + wl * wr * (ul - ur), wl + wr), R(0));
  R       pold = pstar;
  R       conv = R(1);
  // the divisions by pl and pr of every iteration: one reciprocal each in
  // the fast builds
  const R ipl = kExactOrder ? R(0) : rcp(pl);
  const R ipr = kExactOrder ? R(0) : rcp(pr);
  for (int iter = 0; (iter < 10) && (conv > R(1e-6)); ++iter)
  {
    R wwl, wwr, qlw, qrw, usl, usr, delp;
    if constexpr (kExactOrder)
    {
      wwl = sqrt(cl * (R(1) + gamma6 * (pold - pl) / pl));
      wwr = sqrt(cr * (R(1) + gamma6 * (pold - pr) / pr));
      qlw = R(2) * wwl * wwl * wwl / (wwl * wwl + cl);
      qrw = R(2) * wwr * wwr * wwr / (wwr * wwr + cr);
      usl = ul - (pold - pl) / wwl;
      usr = ur + (pold - pr) / wwr;
      delp = fmax(qrw * qlw / (qrw + qlw) * (usl - usr), -pold);
      pold = pold + delp;
      conv = fabs(delp / (pold + G.smallpp));
    }
    else
    {
      wwl = fsqrt(cl * (R(1) + gamma6 * (pold - pl) * ipl));
      wwr = fsqrt(cr * (R(1) + gamma6 * (pold - pr) * ipr));
      const R iwl = rcp(wwl), iwr = rcp(wwr);
      qlw = R(2) * wwl * wwl * wwl * rcp(wwl * wwl + cl);
      qrw = R(2) * wwr * wwr * wwr * rcp(wwr * wwr + cr);
      usl = ul - (pold - pl) * iwl;
      usr = ur + (pold - pr) * iwr;
      delp = fmax(qrw * qlw * rcp(qrw + qlw) * (usl - usr), -pold);
      pold = pold + delp;
      conv = fabs(delp * rcp(pold + G.smallpp));
    }
  }
  pstar = pold;
  if constexpr (kExactOrder)
  {
    wl = sqrt(cl * (R(1) + gamma6 * (pstar - pl) / pl));
    wr = sqrt(cr * (R(1) + gamma6 * (pstar - pr) / pr));
  }
  else
  {
    wl = fsqrt(cl * (R(1) + gamma6 * (pstar - pl) * ipl));
    wr = fsqrt(cr * (R(1) + gamma6 * (pstar - pr) * ipr));
  }
  const R ustar = R(0.5) * (ul + hdiv(pl - pstar, wl) + ur - hdiv(pr - pstar, wr));
  const R sgnm = copysign(R(1), ustar);
  R       ro, uo, po, wo;
  if (sgnm > R(0))
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
  const R co = fmax(smallc, hsqrt(fabs(hdiv(gamma0 * po, ro))));
  const R rstar = fmax(hdiv(ro, R(1) + hdiv(ro * (po - pstar), wo * wo)), smallr);
  const R cstar = fmax(smallc, hsqrt(fabs(hdiv(gamma0 * pstar, rstar))));
  R       spout = co - sgnm * uo;
  R       spin = cstar - sgnm * ustar;
  const R ushock = hdiv(wo, ro) - sgnm * uo;
  if (pstar >= po)
  {
    spin = ushock;
    spout = ushock;
  }
  const R scr = fmax(spout - spin, smallc + fabs(spout + spin));
  R       frac = R(0.5) * (R(1) + hdiv(spout + spin, scr));
  if (frac != frac)
    frac = R(0);
  else
    frac = frac >= R(1) ? R(1) : frac <= R(0) ? R(0) : frac;
  R qg[MAXV];
  qg[ID] = frac * rstar + (R(1) - frac) * ro;
  qg[IU] = frac * ustar + (R(1) - frac) * uo;
  qg[IP] = frac * pstar + (R(1) - frac) * po;
  if (spout < R(0))
  {
    qg[ID] = ro;
    qg[IU] = uo;
    qg[IP] = po;
  }
  if (spin > R(0))
  {
    qg[ID] = rstar;
    qg[IU] = ustar;
    qg[IP] = pstar;
  }
  if (sgnm > R(0))
  {
    qg[IV] = ql[IV];
    if constexpr (DIM == 3)
      qg[IW] = ql[IW];
  }
  else
  {
    qg[IV] = qr[IV];
    if constexpr (DIM == 3)
      qg[IW] = qr[IW];
  }
  hcmpflx<R, DIM>(G, qg, flux);
}

// conservative state and physical flux of riemann_llf / riemann_hll
// (RiemannSolvers.h:249-309, :374-425); HLL takes fleft[ID] = uleft[IU]
template <class R, int DIM>
__device__ __forceinline__ void
hcons_flux(const HGrid<R> & G, const R * q, bool hll, R * u, R * f)
{
  u[ID] = q[ID];
  u[IP] = q[IP] * G.entho + R(0.5) * q[ID] * q[IU] * q[IU];
  u[IP] += R(0.5) * q[ID] * q[IV] * q[IV];
  if constexpr (DIM == 3)
    u[IP] += R(0.5) * q[ID] * q[IW] * q[IW];
  u[IU] = q[ID] * q[IU];
  u[IV] = q[ID] * q[IV];
  if constexpr (DIM == 3)
    u[IW] = q[ID] * q[IW];
  f[ID] = hll ? u[IU] : u[ID] * q[IU];
  f[IP] = q[IU] * (u[IP] + q[IP]);
  f[IU] = q[IP] + u[IU] * q[IU];
  f[IV] = f[ID] * q[IV];
  if constexpr (DIM == 3)
    f[IW] = f[ID] * q[IW];
}

// riemann_llf (RiemannSolvers.h:201-327) and riemann_hll (:329-435)
template <class R, int DIM>
__device__ __forceinline__ void
riemann_llf_hll(const HGrid<R> & G, const R * ql, const R * qr, bool hll, R * flux)
{
  constexpr int NVAR = DIM + 2;
  const R       rl = fmax(ql[ID], G.smallr);
  const R       ul = ql[IU];
  const R       pl = fmax(ql[IP], rl * G.smallp);
  const R       rr = fmax(qr[ID], G.smallr);
  const R       ur = qr[IU];
  const R       pr = fmax(qr[IP], rr * G.smallp);
  const R       cl = hsqrt(hdiv(G.gamma0 * pl, rl));
  const R       cr = hsqrt(hdiv(G.gamma0 * pr, rr));
  R             uleft[MAXV], uright[MAXV], fleft[MAXV], fright[MAXV];
  hcons_flux<R, DIM>(G, ql, hll, uleft, fleft);
  hcons_flux<R, DIM>(G, qr, hll, uright, fright);
  if (!hll)
  {
    const R cmax = fmax(fabs(ul) + cl, fabs(ur) + cr);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      flux[v] = R(0.5) * (fleft[v] + fright[v] - cmax * (uright[v] - uleft[v]));
    return;
  }
  const R SL = fmin(fmin(ul, ur) - fmax(cl, cr), R(0));
  const R SR = fmax(fmax(ul, ur) + fmax(cl, cr), R(0));
  if constexpr (kExactOrder)
  {
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      flux[v] = (SR * fleft[v] - SL * fright[v] + SR * SL * (uright[v] - uleft[v])) / (SR - SL);
  }
  else
  {
    const R is = rcp(SR - SL);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      flux[v] = (SR * fleft[v] - SL * fright[v] + SR * SL * (uright[v] - uleft[v])) * is;
  }
}

// riemann_hllc (RiemannSolvers.h:437-568)
template <class R, int DIM>
__device__ __forceinline__ void
riemann_hllc(const HGrid<R> & G, const R * ql, const R * qr, R * flux)
{
  const R gamma0 = G.gamma0, smallc = G.smallc;
  const R rl = fmax(ql[ID], G.smallr);
  const R pl = fmax(ql[IP], rl * G.smallp);
  const R ul = ql[IU];
  R       ecinl = R(0.5) * rl * ul * ul;
  ecinl += R(0.5) * rl * ql[IV] * ql[IV];
  if constexpr (DIM == 3)
    ecinl += R(0.5) * rl * ql[IW] * ql[IW];
  const R etotl = pl * G.entho + ecinl;
  const R ptotl = pl;
  const R rr = fmax(qr[ID], G.smallr);
  const R pr = fmax(qr[IP], rr * G.smallp);
  const R ur = qr[IU];
  R       ecinr = R(0.5) * rr * ur * ur;
  ecinr += R(0.5) * rr * qr[IV] * qr[IV];
  if constexpr (DIM == 3)
    ecinr += R(0.5) * rr * qr[IW] * qr[IW];
  const R etotr = pr * G.entho + ecinr;
  const R ptotr = pr;
  const R cfastl = hsqrt(fmax(hdiv(gamma0 * pl, rl), smallc * smallc));
  const R cfastr = hsqrt(fmax(hdiv(gamma0 * pr, rr), smallc * smallc));
  const R SL = fmin(ul, ur) - fmax(cfastl, cfastr);
  const R SR = fmax(ul, ur) + fmax(cfastl, cfastr);
  const R rcl = rl * (ul - SL);
  const R rcr = rr * (SR - ur);
  R       ustar, ptotstar, rstarl, etotstarl, rstarr, etotstarr;
  if constexpr (kExactOrder)
  {
    ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) / (rcr + rcl);
    ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) / (rcr + rcl);
    rstarl = rl * (SL - ul) / (SL - ustar);
    etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) / (SL - ustar);
    rstarr = rr * (SR - ur) / (SR - ustar);
    etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) / (SR - ustar);
  }
  else
  {
    const R irc = rcp(rcr + rcl);
    ustar = (rcr * ur + rcl * ul + (ptotl - ptotr)) * irc;
    ptotstar = (rcr * ptotl + rcl * ptotr + rcl * rcr * (ul - ur)) * irc;
    const R isl = rcp(SL - ustar), isr = rcp(SR - ustar);
    rstarl = rl * (SL - ul) * isl;
    etotstarl = ((SL - ul) * etotl - ptotl * ul + ptotstar * ustar) * isl;
    rstarr = rr * (SR - ur) * isr;
    etotstarr = ((SR - ur) * etotr - ptotr * ur + ptotstar * ustar) * isr;
  }
  R ro, uo, ptoto, etoto;
  if (SL > R(0))
  {
    ro = rl;
    uo = ul;
    ptoto = ptotl;
    etoto = etotl;
  }
  else if (ustar > R(0))
  {
    ro = rstarl;
    uo = ustar;
    ptoto = ptotstar;
    etoto = etotstarl;
  }
  else if (SR > R(0))
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
  flux[IV] = flux[ID] > R(0) ? flux[ID] * ql[IV] : flux[ID] * qr[IV];
  if constexpr (DIM == 3)
    flux[IW] = flux[ID] > R(0) ? flux[ID] * ql[IW] : flux[ID] * qr[IW];
}

// riemann_hydro (RiemannSolvers.h:570-633)
template <class R, int DIM>
__device__ __forceinline__ void
hriemann(const HGrid<R> & G, const R * ql, const R * qr, R * flux)
{
  if (G.riemann == MHD_RIEMANN_HLLC)
    riemann_hllc<R, DIM>(G, ql, qr, flux);
  else if (G.riemann == MHD_RIEMANN_LLF)
    riemann_llf_hll<R, DIM>(G, ql, qr, false, flux);
  else if (G.riemann == MHD_RIEMANN_HLL)
    riemann_llf_hll<R, DIM>(G, ql, qr, true, flux);
  else
    riemann_approx<R, DIM>(G, ql, qr, flux);
}

// ---------------------------------------------------------------- kernels
// The CFL rate of one interior cell: ComputeDtFunctor2D/3D
// (HydroRunFunctors2D.h:13-82, 3D:14-88), sum_d (c + |v_d|) / dx_d, or with
// static gravity ComputeDtGravityFunctor2D/3D (2D:84-175, 3D:90-190); a NaN
// rate counts as 0 (fmax ignores NaN operands).
template <class R, int DIM>
__device__ __forceinline__ R
hrate(const HGrid<R> & G, const R * q, R cs, int64_t c)
{
  R val;
  if (G.gravity)
  {
    R velocity = R(0);
    velocity += cs + fabs(q[IU]);
    velocity += cs + fabs(q[IV]);
    if constexpr (DIM == 3)
      velocity += cs + fabs(q[IW]);
    R kk = fabs(G.gf[c]) + fabs(G.gf[c + G.sv]);
    if constexpr (DIM == 3)
      kk = kk + fabs(G.gf[c + 2 * G.sv]);
    kk *= hdiv(R(G.cfl) * R(G.dxg), velocity * velocity);
    kk = fmax(kk, R(1e-4));
    velocity *= hdiv(kk, hsqrt(R(1) + R(2) * kk) - R(1));
    if constexpr (kExactOrder)
      val = qdiv(velocity, R(G.dxg), R(G.idxg));
    else
      val = velocity * R(G.idxg);
  }
  else
  {
    const R vx = cs + fabs(q[IU]);
    const R vy = cs + fabs(q[IV]);
    if constexpr (kExactOrder)
    {
      if constexpr (DIM == 3)
      {
        const R vz = cs + fabs(q[IW]);
        val = qdiv(vx, R(G.dx), R(G.idx)) + qdiv(vy, R(G.dy), R(G.idy)) +
              qdiv(vz, R(G.dz), R(G.idz));
      }
      else
        val = qdiv(vx, R(G.dx), R(G.idx)) + qdiv(vy, R(G.dy), R(G.idy));
    }
    else
    {
      if constexpr (DIM == 3)
        val = vx * R(G.idx) + vy * R(G.idy) + (cs + fabs(q[IW])) * R(G.idz);
      else
        val = vx * R(G.idx) + vy * R(G.idy);
    }
  }
  return (val >= R(0)) ? val : R(0);
}

// U_out of one interior cell: the flux additions in the reference's order
// (xf/xp: the flux * dt/dx of the cell's minus and plus faces per direction
// and variable), then the gravity source term (GravitySourceTermFunctor2D,
// HydroRunFunctors2D.h:1262-1340, new density floored at smallr; 3D,
// 3D:1440-1510, not floored).
template <class R, int DIM>
__device__ __forceinline__ void
hupdate_cell(const HGrid<R> & G, const DevState * st, const R * uin, const R (*fm)[MAXV],
             const R (*fp)[MAXV], R * u, int64_t c)
{
#pragma unroll
  for (int v = 0; v < DIM + 2; ++v)
  {
    R x = uin[v];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
      x = rn_add(x, fm[d][v]);
      x = rn_sub(x, fp[d][v]);
    }
    u[v] = x;
  }
  if (G.gravity)
  {
    const R rhoOld = uin[ID];
    const R rhoNew = DIM == 2 ? fmax(G.smallr, u[ID]) : u[ID];
    R       rhou = u[IU], rhov = u[IV], rhow = DIM == 3 ? u[IW] : R(0);
    R       ekin_old, ekin_new;
    if constexpr (DIM == 3)
      ekin_old = hdiv(R(0.5) * (rhou * rhou + rhov * rhov + rhow * rhow), rhoNew);
    else
      ekin_old = hdiv(R(0.5) * (rhou * rhou + rhov * rhov), rhoNew);
    const R hdt = R(0.5 * st->dt);
    rhou += hdt * G.gf[c] * (rhoOld + rhoNew);
    rhov += hdt * G.gf[c + G.sv] * (rhoOld + rhoNew);
    if constexpr (DIM == 3)
      rhow += hdt * G.gf[c + 2 * G.sv] * (rhoOld + rhoNew);
    u[IU] = rhou;
    u[IV] = rhov;
    if constexpr (DIM == 3)
      u[IW] = rhow;
    if constexpr (DIM == 3)
      ekin_new = hdiv(R(0.5) * (rhou * rhou + rhov * rhov + rhow * rhow), rhoNew);
    else
      ekin_new = hdiv(R(0.5) * (rhou * rhou + rhov * rhov), rhoNew);
    u[IP] += (ekin_new - ekin_old);
  }
}


// Ghost fill.  The reference fills the X faces (over the full j, k range),
// then Y, then Z (MakeBoundariesFunctor2D/3D, BoundariesFunctors.h:18-530;
// SolverBase.cpp:338-410): a ghost cell ends up with the interior value at
// the composition of the per-axis source maps, times the reflection signs of
// the normal velocities.  The iteration's first thread clears the CFL word.
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_hbound(const HGrid<R> G, R * __restrict__ U, DevState * st, int force)
{
  if (!force && step_finished(st))
    return;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx == 0)
    st->invdt_bits = 0ull;
  int i, j, k; // idx enumerates the ghost cells only
  if (!ghost_cell<R, DIM>(G, idx, i, j, k))
    return;
  const int  g = G.g;
  const bool gx = i < g || i >= G.nx + g;
  const bool gy = j < g || j >= G.ny + g;
  const bool gz = DIM == 3 && (k < g || k >= G.nz + g);
  if (!gx && !gy && !gz)
    return;
  bool fx = false, fy = false, fz = false;
  int  i0 = i, j0 = j, k0 = k;
  if (gx)
    i0 = bc_source(i, G.nx, g, G.bc[i < g ? 0 : 1], i >= g, fx);
  if (gy)
    j0 = bc_source(j, G.ny, g, G.bc[j < g ? 2 : 3], j >= g, fy);
  if (gz)
    k0 = bc_source(k, G.nz, g, G.bc[k < g ? 4 : 5], k >= g, fz);
  const int64_t dst = hcell(G, i, j, k), src = hcell(G, i0, j0, k0);
#pragma unroll
  for (int v = 0; v < DIM + 2; ++v)
  {
    R x = U[src + v * G.sv];
    if (fx && v == IU)
      x = x * R(-1);
    if (fy && v == IV)
      x = x * R(-1);
    if (fz && v == IW)
      x = x * R(-1);
    U[dst + v * G.sv] = x;
  }
}

// ConvertToPrimitivesFunctor2D/3D over the whole array
// (HydroRunFunctors2D.h:184-240), fused with the CFL reduction over the
// interior cells: ComputeDtFunctor2D/3D (2D:13-82, 3D:14-88),
// max of sum_d (c + |v_d|) / dx_d, or with static gravity
// ComputeDtGravityFunctor2D/3D (2D:84-175, 3D:90-190).  The max is reduced
// in FP64 (one atomicMax per block on the bit pattern, which orders like the
// value for non-negative doubles): order-independent, so dt is the
// reference's bit for bit in the FMA-free build.
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_hprim_dt(const HGrid<R> G, const R * __restrict__ U, R * __restrict__ Q, DevState * st,
           int force)
{
  if (!force && step_finished(st))
    return;
  constexpr int NVAR = DIM + 2;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  R             rate = R(0);
  bool          bad = false;
  int           i, j, k;
  if (box_cell(G.box[BOX_ALL], idx, i, j, k))
  {
    const int64_t c = hcell(G, i, j, k);
    R             u[MAXV], q[MAXV], cs;
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      u[v] = U[c + v * G.sv];
    hprim<R, DIM>(G, u, cs, q);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Q[c + v * G.sv] = q[v];
    const int  g = G.g;
    const bool interior = i >= g && i < G.nx + g && j >= g && j < G.ny + g &&
                          (DIM == 2 || (k >= g && k < G.nz + g));
    if (interior)
    {
      rate = hrate<R, DIM>(G, q, cs, c);
      bad = !(u[ID] > R(0)) || !isfinite(u[IP]);
    }
  }
  __shared__ R red[32];
  rate = warp_max(rate);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    red[wid] = rate;
  if (__syncthreads_or(bad) && threadIdx.x == 0)
    atomicOr(&st->status, STATUS_NUMERIC);
  if (wid == 0)
  {
    rate = lane < (int)(blockDim.x >> 5) ? red[lane] : R(0);
    rate = warp_max(rate);
    const unsigned long long rb = (unsigned long long)__double_as_longlong((double)rate);
    if (lane == 0 && rate > R(0) && rb > *(volatile unsigned long long *)&st->invdt_bits)
      atomicMax(&st->invdt_bits, rb);
  }
}

// dt = cfl / invDt (SolverHydroMuscl.h:649-690) clipped to tEnd
// (SolverBase.cpp:148-179); dt/dx of ComputeAndStoreFluxesFunctor
// (HydroRunFunctors2D.h:505-507) in the working precision.
template <class R>
__global__ void
k_hfinalize(const HGrid<R> G, DevState * st, int force)
{
  if (!force && step_finished(st))
    return;
  const double invDt = __longlong_as_double((long long)st->invdt_bits);
  double       dt = G.cfl / invDt;
  if (st->t + dt > st->tEnd)
    dt = st->tEnd - st->t;
  st->dt = dt;
  st->dtdx = dt / G.dx;
  st->dtdy = dt / G.dy;
  st->dtdz = dt / G.dz;
  st->fdtdx = (float)((float)dt / (float)G.dx);
  st->fdtdy = (float)((float)dt / (float)G.dy);
  st->fdtdz = (float)((float)dt / (float)G.dz);
  if (!(invDt > 0.0) || !isfinite(dt))
    st->status |= STATUS_NUMERIC;
}

// godunov_unsplit(dt) with the caller's dt
template <class R>
__global__ void
k_hset_dt(const HGrid<R> G, DevState * st, double dt)
{
  if (step_finished(st))
    return;
  st->dt = dt;
  st->dtdx = dt / G.dx;
  st->dtdy = dt / G.dy;
  st->dtdz = dt / G.dz;
  st->fdtdx = (float)((float)dt / (float)G.dx);
  st->fdtdy = (float)((float)dt / (float)G.dy);
  st->fdtdz = (float)((float)dt / (float)G.dz);
}

// ComputeSlopesFunctor2D/3D (HydroRunFunctors2D.h:900-985, 3D:930-1040) with
// slope_unsplit_hydro_2d/3d (HydroBaseFunctor2D.h:432-525, 3D:411-540) over
// [g-1, size-g] per axis: S[(d * NVAR + v) * sv + cell]; slope_type 0 gives
// zero slopes (first order).  The cell's trace source terms follow in planes
// S[(DIM * NVAR + v) * sv + cell] (hsources).
template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_hslopes(const HGrid<R> G, const R * __restrict__ Q, R * __restrict__ S, const DevState * st)
{
  if (step_finished(st))
    return;
  constexpr int NVAR = DIM + 2;
  int           i, j, k;
  if (!box_cell(G.box[BOX_TRACE], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  const int64_t c = hcell(G, i, j, k);
  const int64_t str[3] = { 1, G.sj, G.sk };
  R             q[MAXV], dq[DIM][MAXV], src[MAXV];
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
    q[v] = Q[c + v * G.sv];
#pragma unroll
  for (int d = 0; d < DIM; ++d)
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
    {
      const R * Qv = Q + v * G.sv;
      R         sl = R(0);
      if (G.slope_type != R(0))
      {
        if constexpr (kExactOrder)
          sl = limited_slope(q[v], Qv[c + str[d]], Qv[c - str[d]], G.slope_type);
        else
          sl = limited_slope_bits(q[v], Qv[c + str[d]], Qv[c - str[d]], G.slope_type);
      }
      dq[d][v] = sl;
      S[(d * NVAR + v) * G.sv + c] = sl;
    }
  hsources<R, DIM>(G, q, dq, src);
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
    S[(DIM * NVAR + v) * G.sv + c] = src[v];
}

// Face flux along direction D of the face at the minus side of every cell
// of [g, size-g] per axis (ComputeAndStoreFluxesFunctor2D/3D,
// HydroRunFunctors2D.h:490-755, 3D:300-705; ComputeTraceAndFluxes_Functor,
// 2D:988-1255, 3D:1044-1420): right state = the cell traced to its minus
// face, left state = the minus neighbour traced to its plus face, the gravity
// predictor 0.5 dt g on both, the normal velocity swapped into IU, the
// Riemann solver, the flux swapped back and scaled by dt/dx_D.
// The flux of one face along D from the register copies of its two cells:
// right cell (primitives qc, slopes along D dc, sources sc) and its minus
// neighbour (qn, dn, sn); returns flux * t, t = dt/dx_D.
template <class R, int DIM, int D>
__device__ __forceinline__ void
hface_flux(const HGrid<R> & G, const DevState * st, const R * qc, const R * dc, const R * sc,
           const R * qn, const R * dn, const R * sn, R * out, int64_t c, int64_t nb)
{
  constexpr int NVAR = DIM + 2;
  constexpr int VN = D == 0 ? IU : D == 1 ? IV : IW; // normal velocity
  R             tx, ty, tz;
  dt_over_dx(st, tx, ty, tz);
  const R t = D == 0 ? tx : D == 1 ? ty : tz;
  R       qleft[MAXV], qright[MAXV], flux[MAXV];
  htrace<R, DIM, true>(G, qc, dc, sc, t, qright);
  htrace<R, DIM, false>(G, qn, dn, sn, t, qleft);
  if (G.gravity)
  {
    // the gravity predictor with the field at each cell (left state: the
    // minus neighbour nb, right state: the cell c)
    const R hdt = R(0.5 * st->dt);
    const R * g = G.gf;
    qleft[IU] += hdt * g[nb];
    qleft[IV] += hdt * g[nb + G.sv];
    if constexpr (DIM == 3)
      qleft[IW] += hdt * g[nb + 2 * G.sv];
    if (D != 2 || G.zgrav_right)
    {
      qright[IU] += hdt * g[c];
      qright[IV] += hdt * g[c + G.sv];
      if constexpr (DIM == 3)
        qright[IW] += hdt * g[c + 2 * G.sv];
    }
  }
  if constexpr (D > 0)
  {
    swap_vals(qleft[IU], qleft[VN]);
    swap_vals(qright[IU], qright[VN]);
  }
  hriemann<R, DIM>(G, qleft, qright, flux);
  if constexpr (D > 0)
    swap_vals(flux[IU], flux[VN]);
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
    out[v] = flux[v] * t;
}

template <class R, int DIM, int D>
__device__ __forceinline__ void
hflux_face(const HGrid<R> & G, const R * __restrict__ Q, const R * __restrict__ S,
           R * __restrict__ F, const DevState * st, int64_t c)
{
  constexpr int NVAR = DIM + 2;
  const int64_t nb = c - (D == 0 ? 1 : D == 1 ? G.sj : G.sk);
  // the cell and its minus neighbour: primitives, slopes along D, sources
  R qc[MAXV], qn[MAXV], dc[MAXV], dn[MAXV], sc[MAXV], sn[MAXV], f[MAXV];
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
  {
    qc[v] = Q[c + v * G.sv];
    qn[v] = Q[nb + v * G.sv];
    dc[v] = S[(D * NVAR + v) * G.sv + c];
    dn[v] = S[(D * NVAR + v) * G.sv + nb];
    sc[v] = S[(DIM * NVAR + v) * G.sv + c];
    sn[v] = S[(DIM * NVAR + v) * G.sv + nb];
  }
  hface_flux<R, DIM, D>(G, st, qc, dc, sc, qn, dn, sn, f, c, nb);
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
    F[(D * NVAR + v) * G.sv + c] = f[v];
}

// grid (faces / 128, DIM): blockIdx.y is the direction
template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_hflux(const HGrid<R> G, const R * __restrict__ Q, const R * __restrict__ S, R * __restrict__ F,
        const DevState * st)
{
  if (step_finished(st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  const int64_t c = hcell(G, i, j, k);
  if (blockIdx.y == 0)
    hflux_face<R, DIM, 0>(G, Q, S, F, st, c);
  else if (blockIdx.y == 1)
    hflux_face<R, DIM, 1>(G, Q, S, F, st, c);
  else if constexpr (DIM == 3)
    hflux_face<R, DIM, 2>(G, Q, S, F, st, c);
}

// UpdateFunctor2D/3D (HydroRunFunctors2D.h:765-840, 3D:715-800) or
// UpdateDirFunctor per direction (same additions in the same order),
// then GravitySourceTermFunctor2D (HydroRunFunctors2D.h:1262-1340, new density
// floored at smallr) / 3D (3D:1440-1510, not floored); ghost cells are the
// boundary-filled input (Kokkos::deep_copy(data_out, data_in)).
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_hupdate(const HGrid<R> G, const R * __restrict__ Uin, R * __restrict__ Uout,
          const R * __restrict__ F, const DevState * st)
{
  if (step_finished(st))
    return;
  constexpr int NVAR = DIM + 2;
  int           i, j, k;
  if (!box_cell(G.box[BOX_ALL], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  const int64_t c = hcell(G, i, j, k);
  const int     g = G.g;
  const bool    interior = i >= g && i < G.nx + g && j >= g && j < G.ny + g &&
                        (DIM == 2 || (k >= g && k < G.nz + g));
  if (!interior)
  {
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Uout[c + v * G.sv] = Uin[c + v * G.sv];
    return;
  }
  const int64_t str[3] = { 1, G.sj, G.sk };
  R             uin[MAXV], u[MAXV], fm[DIM][MAXV], fp[DIM][MAXV];
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
  {
    uin[v] = Uin[c + v * G.sv];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
      const R * Fd = F + (d * NVAR + v) * G.sv;
      fm[d][v] = Fd[c];
      fp[d][v] = Fd[c + str[d]];
    }
  }
  hupdate_cell<R, DIM>(G, st, uin, fm, fp, u, c);
#pragma unroll
  for (int v = 0; v < NVAR; ++v)
    Uout[c + v * G.sv] = u[v];
}

// ---------------------------------------------------------------- fused form

// The CFL reduction of the fused form (no primitive array is written): the
// rates of the interior cells as k_hprim_dt computes them, kHdtCells cells
// per thread in the first nrate blocks; the ghost cells of U_in, just
// filled by k_hbound, are copied to U_out by the blocks after them (the
// reference's deep_copy(data_out, data_in) of the ghost layers; the tile
// kernel writes the interior).
constexpr int kHdtCells = 4;

template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_hdt(const HGrid<R> G, const R * __restrict__ U, R * __restrict__ Uout, DevState * st, int force,
      unsigned nrate)
{
  if (!force && step_finished(st))
    return;
  constexpr int NVAR = DIM + 2;
  if (blockIdx.x >= nrate)
  {
    // the ghost layers copied to U_out (blocks nrate.. of the launch)
    int i, j, k;
    if (!Uout ||
        !ghost_cell<R, DIM>(G, (blockIdx.x - nrate) * (int64_t)blockDim.x + threadIdx.x, i, j, k))
      return;
    const int64_t c = hcell(G, i, j, k);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Uout[c + v * G.sv] = U[c + v * G.sv];
    return;
  }
  // the rates of kHdtCells interior cells per thread (blocks 0..nrate-1)
  R    rate = R(0);
  bool bad = false;
#pragma unroll
  for (int q = 0; q < kHdtCells; ++q)
  {
    int i, j, k;
    if (box_cell(G.box[BOX_INTERIOR], (blockIdx.x * (int64_t)kHdtCells + q) * blockDim.x +
                                        threadIdx.x, i, j, k))
    {
      const int64_t c = hcell(G, i, j, k);
      R             u[MAXV], qv[MAXV], cs;
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
        u[v] = U[c + v * G.sv];
      hprim<R, DIM>(G, u, cs, qv);
      const R r = hrate<R, DIM>(G, qv, cs, c);
      rate = r > rate ? r : rate;
      bad = bad || !(u[ID] > R(0)) || !isfinite(u[IP]);
    }
  }
  __shared__ R red[32];
  rate = warp_max(rate);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0)
    red[wid] = rate;
  if (__syncthreads_or(bad) && threadIdx.x == 0)
    atomicOr(&st->status, STATUS_NUMERIC);
  if (wid == 0)
  {
    rate = lane < (int)(blockDim.x >> 5) ? red[lane] : R(0);
    rate = warp_max(rate);
    const unsigned long long rb = (unsigned long long)__double_as_longlong((double)rate);
    if (lane == 0 && rate > R(0) && rb > *(volatile unsigned long long *)&st->invdt_bits)
      atomicMax(&st->invdt_bits, rb);
  }
}

// Tile shape of the fused form: TX x TY x TZ interior cells per block (TZ = 1
// in 2D), chosen so that the block's shared-memory working set (below) fits
// in 227 KB.
template <class R, int DIM>
struct HTile
{
  static constexpr int TX = DIM == 2 ? 32 : (sizeof(R) == 4 ? 16 : 8);
  static constexpr int TY = DIM == 2 ? 16 : 8;
  static constexpr int TZ = DIM == 2 ? 1 : 4;
  static constexpr int NVAR = DIM + 2;
  // primitives over the tile and 2 halo layers
  static constexpr int MX = TX + 4, MY = TY + 4, MZ = DIM == 2 ? 1 : TZ + 4;
  static constexpr int NM = MX * MY * MZ;
  // slopes and sources over the tile and 1 halo layer
  static constexpr int SX = TX + 2, SY = TY + 2, SZ = DIM == 2 ? 1 : TZ + 2;
  static constexpr int NS = SX * SY * SZ;
  static constexpr int NSC = NVAR; // the trace sources (slopes are recomputed per face)
  // faces along d of the tile: one extra layer along d
  static constexpr int NF0 = (TX + 1) * TY * TZ;
  static constexpr int NF1 = TX * (TY + 1) * TZ;
  static constexpr int NF2 = DIM == 2 ? 0 : TX * TY * (TZ + 1);
  static constexpr int NF = NF0 + NF1 + NF2;
  static constexpr int THREADS = 256;
  static constexpr size_t SMEM = sizeof(R) * ((size_t)NM * NVAR + (size_t)NS * NSC + (size_t)NF * NVAR);
};

// One whole iteration but the CFL reduction for one tile of interior cells
// (the plain form fused: primitives, slopes, trace sources, face fluxes,
// update), every intermediate in shared memory:
//   1. primitives of the tile and 2 halo layers, from U_in (ghost cells
//      filled by k_hbound) — ConvertToPrimitivesFunctor;
//   2. trace source terms of the tile and 1 halo layer (from the limited
//      slopes of ComputeSlopesFunctor, kept in registers);
//   3. the flux * dt/dx of every face of the tile's cells (both faces of the
//      boundary layer), the two cells' slopes along the face normal taken
//      again from the primitives — ComputeAndStoreFluxes /
//      ComputeTraceAndFluxes;
//   4. the update of the tile's cells, gravity source included, written to
//      U_out — UpdateFunctor / UpdateDirFunctor, GravitySourceTermFunctor.
// Each value is computed by the same device functions from the same
// operands as in the unfused kernels, so U_out is bitwise theirs; halo cells
// are recomputed by neighbouring tiles instead of being written to and read
// back from HBM.  Loads along x are coalesced (i fastest in shared memory as
// in HBM).
template <class R, int DIM>
__global__ void __launch_bounds__(HTile<R, DIM>::THREADS)
k_hfused(const HGrid<R> G, const R * __restrict__ U, R * __restrict__ Uout, const DevState * st)
{
  using T = HTile<R, DIM>;
  constexpr int NVAR = T::NVAR;
  if (step_finished(st))
    return;
  extern __shared__ __align__(16) unsigned char hsm_raw[];
  R * Qs = reinterpret_cast<R *>(hsm_raw);       // [NVAR][NM]
  R * Ss = Qs + (size_t)NVAR * T::NM;             // [NSC][NS]
  R * Fs = Ss + (size_t)T::NSC * T::NS;           // [NVAR][NF]
  const int g = G.g;
  const int i0 = g + blockIdx.x * T::TX, j0 = g + blockIdx.y * T::TY;
  const int k0 = DIM == 3 ? g + blockIdx.z * T::TZ : 0;
  const int tid = threadIdx.x;

  // 1. primitives over global [i0-2, i0+TX+2) x ... (inside the array)
  for (int m = tid; m < T::NM; m += T::THREADS)
  {
    const int a = m % T::MX, b = (m / T::MX) % T::MY, cz = m / (T::MX * T::MY);
    const int i = i0 - 2 + a, j = j0 - 2 + b, k = DIM == 3 ? k0 - 2 + cz : 0;
    R         q[MAXV];
    if (i < G.isize && j < G.jsize && k < G.ksize)
    {
      const int64_t c = hcell(G, i, j, k);
      R             u[MAXV], cs;
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
        u[v] = U[c + v * G.sv];
      hprim<R, DIM>(G, u, cs, q);
    }
    else
    {
      // beyond the array (a partial last tile): a neutral state that only
      // cells outside the interior read
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
        q[v] = (v == ID || v == IP) ? R(1) : R(0);
    }
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Qs[v * T::NM + m] = q[v];
  }
  __syncthreads();

  // 2. slopes and sources over the tile and 1 halo layer
  constexpr int mstr[3] = { 1, T::MX, T::MX * T::MY };
  // (2D: warps on 32-column rows of the item grid, contiguous shared-memory
  // reads whatever the row pitch; ItemGrid)
  using IS = ItemGrid<T::SX, T::SY>;
  for (int w = tid; w < (DIM == 2 ? IS::COUNT : T::NS); w += T::THREADS)
  {
    int a, b, cz = 0, sidx;
    if constexpr (DIM == 2)
    {
      if (!IS::at(w, a, b))
        continue;
      sidx = a + T::SX * b;
    }
    else
    {
      sidx = w;
      a = sidx % T::SX;
      b = (sidx / T::SX) % T::SY;
      cz = sidx / (T::SX * T::SY);
    }
    const int m = (a + 1) + T::MX * ((b + 1) + T::MY * (DIM == 3 ? cz + 1 : 0));
    R         q[MAXV], dq[DIM][MAXV], src[MAXV];
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      q[v] = Qs[v * T::NM + m];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
      {
        R sl = R(0);
        if (G.slope_type != R(0))
        {
          const R qp = Qs[v * T::NM + m + mstr[d]], qm = Qs[v * T::NM + m - mstr[d]];
          if constexpr (kExactOrder)
            sl = limited_slope(q[v], qp, qm, G.slope_type);
          else
            sl = limited_slope_bits(q[v], qp, qm, G.slope_type);
        }
        dq[d][v] = sl;
      }
    hsources<R, DIM>(G, q, dq, src);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Ss[v * T::NS + sidx] = src[v];
  }
  __syncthreads();

  // 3. face fluxes: faces of direction d of the tile's cells, one extra
  // layer along d (the plus faces of the last cells)
  auto face_dir = [&](auto dtag) {
    constexpr int D = decltype(dtag)::value;
    constexpr int FX = T::TX + (D == 0), FY = T::TY + (D == 1), FZ = T::TZ + (D == 2);
    constexpr int NFD = FX * FY * FZ;
    constexpr int off = D == 0 ? 0 : D == 1 ? T::NF0 : T::NF0 + T::NF1;
    constexpr int sstr[3] = { 1, T::SX, T::SX * T::SY };
    using IF = ItemGrid<FX, FY>;
    for (int w = tid; w < (DIM == 2 ? IF::COUNT : NFD); w += T::THREADS)
    {
      int a, b, cz = 0, f;
      if constexpr (DIM == 2)
      {
        if (!IF::at(w, a, b))
          continue;
        f = a + FX * b;
      }
      else
      {
        f = w;
        a = f % FX;
        b = (f / FX) % FY;
        cz = f / (FX * FY);
      }
      // the face's right cell in the slopes box and in the primitives box
      const int sc_ = (a + 1) + T::SX * ((b + 1) + T::SY * (DIM == 3 ? cz + 1 : 0));
      const int mc = (a + 2) + T::MX * ((b + 2) + T::MY * (DIM == 3 ? cz + 2 : 0));
      const int sn_ = sc_ - sstr[D], mn = mc - mstr[D];
      R         qc[MAXV], qn[MAXV], dc[MAXV], dn[MAXV], scv[MAXV], snv[MAXV], fl[MAXV];
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
      {
        const R * Qv = Qs + v * T::NM;
        qc[v] = Qv[mc];
        qn[v] = Qv[mn];
        // the slopes along D of both cells again (the same limiter on the
        // same primitives as the slopes stage)
        dc[v] = R(0);
        dn[v] = R(0);
        if (G.slope_type != R(0))
        {
          const R qcp = Qv[mc + mstr[D]], qnm = Qv[mn - mstr[D]];
          if constexpr (kExactOrder)
          {
            dc[v] = limited_slope(qc[v], qcp, qn[v], G.slope_type);
            dn[v] = limited_slope(qn[v], qc[v], qnm, G.slope_type);
          }
          else
          {
            dc[v] = limited_slope_bits(qc[v], qcp, qn[v], G.slope_type);
            dn[v] = limited_slope_bits(qn[v], qc[v], qnm, G.slope_type);
          }
        }
        scv[v] = Ss[v * T::NS + sc_];
        snv[v] = Ss[v * T::NS + sn_];
      }
      // global cells of the face for the gravity field in HBM, clamped to
      // the array: a partial last tile's faces beyond it are computed but
      // never used
      const int     gi = min(i0 + a, G.isize - 1), gj = min(j0 + b, G.jsize - 1);
      const int     gk = DIM == 3 ? min(k0 + cz, G.ksize - 1) : 0;
      const int64_t gc = hcell(G, gi, gj, gk);
      const int64_t gn = gc - (D == 0 ? 1 : D == 1 ? G.sj : G.sk);
      hface_flux<R, DIM, D>(G, st, qc, dc, scv, qn, dn, snv, fl, gc, gn);
#pragma unroll
      for (int v = 0; v < NVAR; ++v)
        Fs[v * T::NF + off + f] = fl[v];
    }
  };
  face_dir(std::integral_constant<int, 0>{});
  face_dir(std::integral_constant<int, 1>{});
  if constexpr (DIM == 3)
    face_dir(std::integral_constant<int, 2>{});
  __syncthreads();

  // 4. update of the tile's interior cells
  constexpr int NT = T::TX * T::TY * T::TZ;
  for (int o = tid; o < NT; o += T::THREADS)
  {
    const int a = o % T::TX, b = (o / T::TX) % T::TY, cz = o / (T::TX * T::TY);
    const int i = i0 + a, j = j0 + b, k = DIM == 3 ? k0 + cz : 0;
    if (i >= G.nx + g || j >= G.ny + g || (DIM == 3 && k >= G.nz + g))
      continue;
    const int64_t c = hcell(G, i, j, k);
    // face index of the cell's minus face along d, and of its plus face
    const int f0 = a + (T::TX + 1) * (b + T::TY * cz);
    const int f1 = T::NF0 + a + T::TX * (b + (T::TY + 1) * cz);
    const int f2 = T::NF0 + T::NF1 + a + T::TX * (b + T::TY * cz);
    const int fm_[3] = { f0, f1, f2 };
    const int fstep[3] = { 1, T::TX, T::TX * T::TY };
    R         uin[MAXV], u[MAXV], fm[DIM][MAXV], fp[DIM][MAXV];
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
    {
      uin[v] = U[c + v * G.sv];
#pragma unroll
      for (int d = 0; d < DIM; ++d)
      {
        fm[d][v] = Fs[v * T::NF + fm_[d]];
        fp[d][v] = Fs[v * T::NF + fm_[d] + fstep[d]];
      }
    }
    hupdate_cell<R, DIM>(G, st, uin, fm, fp, u, c);
#pragma unroll
    for (int v = 0; v < NVAR; ++v)
      Uout[c + v * G.sv] = u[v];
  }
}

// LayoutRight <-> LayoutLeft of an NVAR-variable array.  dir = 0: right ->
// left, dir = 1: left -> right.
template <class R>
__global__ void
k_htranspose(const HGrid<R> G, const R * __restrict__ src, R * __restrict__ dst, int dir)
{
  const int64_t n = G.sv * G.nvar;
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= n)
    return;
  const int64_t v = idx / G.sv;
  const int64_t cell = idx - v * G.sv;
  const int64_t k = cell / G.sk;
  const int64_t rem = cell - k * G.sk;
  const int64_t j = rem / G.sj;
  const int64_t i = rem - j * G.sj;
  const int64_t right = ((i * G.jsize + j) * G.ksize + k) * G.nvar + v;
  if (dir == 0)
    dst[idx] = src[right];
  else
    dst[right] = src[idx];
}

template <class R>
HGrid<R>
make_hgrid(const mhd_params & p)
{
  HGrid<R> G{};
  G.dim = p.dim;
  G.nx = p.nx;
  G.ny = p.ny;
  G.nz = p.dim == 3 ? p.nz : 1;
  G.g = p.ghost;
  G.nvar = p.dim + 2;
  G.isize = p.nx + 2 * p.ghost;
  G.jsize = p.ny + 2 * p.ghost;
  G.ksize = p.dim == 3 ? p.nz + 2 * p.ghost : 1;
  G.sj = G.isize;
  G.sk = (int64_t)G.isize * G.jsize;
  G.sv = G.sk * G.ksize;
  for (int f = 0; f < 6; ++f)
    G.bc[f] = p.boundary[f];
  G.riemann = p.riemann;
  G.gravity = p.gravity != 0;
  G.gf = nullptr; // set by the solver core once the field is on the device
  G.zgrav_right = !(p.dim == 3 && p.implementation_version == 1);
  // HydroParams::init (HydroParams.cpp:436-443) in real_t
  G.gamma0 = R(p.gamma0);
  G.entho = R(1) / (G.gamma0 - R(1));
  G.smallr = R(p.smallr);
  G.smallc = R(p.smallc);
  G.smallp = R(R(p.smallc) * R(p.smallc) / R(p.gamma0));
  G.smallpp = R(G.smallr * G.smallp);
  G.gamma6 = R((G.gamma0 + R(1)) / (R(2) * G.gamma0));
  G.slope_type = R(p.slope_type);
  G.cfl = p.cfl;
  G.dx = (double)R(R(p.xmax - p.xmin) / R(p.nx));
  G.dy = (double)R(R(p.ymax - p.ymin) / R(p.ny));
  G.dz = p.dim == 3 ? (double)R(R(p.zmax - p.zmin) / R(p.nz)) : 1.0;
  G.dxg = std::fmin(G.dx, G.dy);
  if (p.dim == 3)
    G.dxg = std::fmin(G.dxg, G.dz);
  G.idx = 1.0 / G.dx;
  G.idy = 1.0 / G.dy;
  G.idz = 1.0 / G.dz;
  G.idxg = 1.0 / G.dxg;
  const bool d3 = p.dim == 3;
  const int  g = G.g;
  G.box[BOX_ALL] = Box(0, 0, 0, G.isize, G.jsize, d3 ? G.ksize : 1);
  G.box[BOX_PRIM] = G.box[BOX_ALL];
  G.box[BOX_TRACE] = Box(g - 1, g - 1, d3 ? g - 1 : 0, G.nx + 2, G.ny + 2, d3 ? G.nz + 2 : 1);
  G.box[BOX_FACE] = Box(g, g, d3 ? g : 0, G.nx + 1, G.ny + 1, d3 ? G.nz + 1 : 1);
  G.box[BOX_INTERIOR] = Box(g, g, d3 ? g : 0, G.nx, G.ny, d3 ? G.nz : 1);
  return G;
}

} // namespace hydro
} // namespace MHD_VARIANT_TAG
} // namespace mhd
