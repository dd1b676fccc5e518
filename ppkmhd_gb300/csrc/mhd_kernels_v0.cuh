// Kernels of implementation versions 0 and 1 of ppkMHD's MHD MUSCL step
// (SolverMHDMuscl.cpp:401-429 in 2D, :494-539 in 3D): a full trace to face
// and edge states, stored; Riemann fluxes and edge EMFs from the stored
// states; then the update.  Version 0 stores fluxes and EMFs and gathers
// (UpdateFunctor / UpdateEmfFunctor); version 1 adds them with atomics from
// the face / edge threads.  Both are evaluated here as a gather; for version
// 1 the contributions of a cell are applied in the order a serial run of
// the reference applies them.
//
// Stored trace states (T buffer), NS states of 8 planes each:
//   2D (NS = 8):  qm_x, qp_x, qm_y, qp_y, qRT, qRB, qLT, qLB
//   3D (NS = 18): qm_x, qp_x, qm_y, qp_y, qm_z, qp_z,
//                 qRT_X, qRB_X, qLT_X, qLB_X, qRT_Y, ..., qLB_Z
#pragma once

#include "mhd_kernels.cuh"

#ifndef MHD_VARIANT_TAG
#  define MHD_VARIANT_TAG v_default
#endif

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

template <int DIM>
struct TraceLayout
{
  static constexpr int NS = DIM == 2 ? 8 : 18;
  __device__ static constexpr int qm(int d) { return 2 * d; }
  __device__ static constexpr int qp(int d) { return 2 * d + 1; }
  // corner e in {RT, RB, LT, LB} = {0, 1, 2, 3} of the edges along dir (3D)
  __device__ static constexpr int edge(int e, int dir) { return DIM == 2 ? 4 + e : 6 + 4 * dir + e; }
};

template <class R>
__device__ __forceinline__ R
div_r(R a, R r, R ir)
{
  if constexpr (kExactOrder)
    return a / r;
  else
    return a * ir;
}

// ---------------------------------------------------------------- 3D preparation

// Edge electric field (ComputeElecFieldFunctor3D, MHDRunFunctors3D.h:278-362)
// and transverse face-field slopes (ComputeMagSlopesFunctor3D,
// MHDRunFunctors3D.h:441-538 with slope_unsplit_mhd_3d,
// MHDBaseFunctor3D.h:563-668) over [1, size-1)^3.  Stored slopes (D buffer,
// 6 planes): dBx/dy, dBx/dz, dBy/dx, dBy/dz, dBz/dx, dBz/dy.
template <class R>
__global__ void __launch_bounds__(128)
k_v0_prep3d(const Grid<R> G, const R * __restrict__ U, const R * __restrict__ Q,
            R * __restrict__ E, R * __restrict__ D, const DevState * st)
{
  if (step_finished(st))
    return;
  const Box & b = G.box[BOX_PRIM];
  int         i, j, k;
  if (!box_cell(b, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  if (i < 1 || j < 1 || k < 1)
    return;
  const int64_t sv = G.sv, sj = G.sj, sk = G.sk;
  const int64_t c = cell_at(G, i, j, k);
  R             u, v, w, A, Bf, C;
  v = R(0.25) * (Q[c - sj - sk + IV * sv] + Q[c - sj + IV * sv] + Q[c - sk + IV * sv] + Q[c + IV * sv]);
  w = R(0.25) * (Q[c - sj - sk + IW * sv] + Q[c - sj + IW * sv] + Q[c - sk + IW * sv] + Q[c + IW * sv]);
  Bf = R(0.5) * (U[c - sk + IB * sv] + U[c + IB * sv]);
  C = R(0.5) * (U[c - sj + IC * sv] + U[c + IC * sv]);
  E[c] = v * C - w * Bf;
  u = R(0.25) * (Q[c - 1 - sk + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sk + IU * sv] + Q[c + IU * sv]);
  w = R(0.25) * (Q[c - 1 - sk + IW * sv] + Q[c - 1 + IW * sv] + Q[c - sk + IW * sv] + Q[c + IW * sv]);
  A = R(0.5) * (U[c - sk + IA * sv] + U[c + IA * sv]);
  C = R(0.5) * (U[c - 1 + IC * sv] + U[c + IC * sv]);
  E[c + sv] = w * A - u * C;
  u = R(0.25) * (Q[c - 1 - sj + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sj + IU * sv] + Q[c + IU * sv]);
  v = R(0.25) * (Q[c - 1 - sj + IV * sv] + Q[c - 1 + IV * sv] + Q[c - sj + IV * sv] + Q[c + IV * sv]);
  A = R(0.5) * (U[c - sj + IA * sv] + U[c + IA * sv]);
  Bf = R(0.5) * (U[c - 1 + IB * sv] + U[c + IB * sv]);
  E[c + 2 * sv] = u * Bf - v * A;
  // xslope_type = min(slope_type, 2) (MHDBaseFunctor3D.h:596)
  const R       xst = fmin(G.slope_type, R(2));
  const R *     Ua = U + IA * sv, *Ub = U + IB * sv, *Uc = U + IC * sv;
  D[c + 0 * sv] = slope_limited(Ua[c], Ua[c + sj], Ua[c - sj], xst);
  D[c + 1 * sv] = slope_limited(Ua[c], Ua[c + sk], Ua[c - sk], xst);
  D[c + 2 * sv] = slope_limited(Ub[c], Ub[c + 1], Ub[c - 1], xst);
  D[c + 3 * sv] = slope_limited(Ub[c], Ub[c + sk], Ub[c - sk], xst);
  D[c + 4 * sv] = slope_limited(Uc[c], Uc[c + 1], Uc[c - 1], xst);
  D[c + 5 * sv] = slope_limited(Uc[c], Uc[c + sj], Uc[c - sj], xst);
}

// Store state q (8 planes) as trace state s of cell c, with the density and
// pressure floors of the trace (smallp * rho in 2D; smallp in the 3D trace,
// MHDBaseFunctor3D.h:908-1112).
template <class R, int DIM>
__device__ __forceinline__ void
put_state(R * __restrict__ T, int64_t sv, int64_t c, int s, R (&q)[NV], R smallR, R smallp)
{
  q[ID] = fmax(smallR, q[ID]);
  if constexpr (DIM == 2)
    q[IP] = fmax(smallp * q[ID], q[IP]);
  else
    q[IP] = fmax(smallp, q[IP]);
  R * dst = T + (int64_t)s * NV * sv + c;
#pragma unroll
  for (int v = 0; v < NV; ++v)
    dst[v * sv] = q[v];
}

// ---------------------------------------------------------------- trace

// ComputeTraceFunctor{2D,3D}_MHD (MHDRunFunctors2D.h:782-911,
// MHDRunFunctors3D.h:543-856) with trace_unsplit_mhd_2d
// (MHDBaseFunctor2D.h:775-1109) / trace_unsplit_mhd_3d_simpler
// (MHDBaseFunctor3D.h:690-1114), over [g-2, size-g+1)^DIM.
template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_v0_trace(const Grid<R> G, const R * __restrict__ U, const R * __restrict__ Q,
           const R * __restrict__ E, const R * __restrict__ D, R * __restrict__ T,
           const DevState * st)
{
  if (step_finished(st))
    return;
  const Box & b = G.box[BOX_PRIM];
  int         i, j, k;
  if (!box_cell(b, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  const int g = G.g;
  if (i < g - 2 || i >= G.isize - g + 1 || j < g - 2 || j >= G.jsize - g + 1)
    return;
  if (DIM == 3 && (k < g - 2 || k >= G.ksize - g + 1))
    return;
  const int64_t sv = G.sv, sj = G.sj, sk = G.sk;
  const int64_t c = cell_at(G, i, j, k);
  R             dtdx, dtdy, dtdz;
  dt_over_dx(st, dtdx, dtdy, dtdz);
  const R smallR = G.smallr, smallp = G.smallp, gamma = G.gamma0, sl = G.slope_type;
  using TL = TraceLayout<DIM>;

  R q[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
    q[v] = Q[c + v * sv];
  // hydro slopes (slope_unsplit_hydro_{2,3}d); only the ones the trace reads
  R dqx[NV], dqy[NV], dqz[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    dqx[v] = slope_limited(q[v], Q[c + 1 + v * sv], Q[c - 1 + v * sv], sl);
    dqy[v] = slope_limited(q[v], Q[c + sj + v * sv], Q[c - sj + v * sv], sl);
    if constexpr (DIM == 3)
      dqz[v] = slope_limited(q[v], Q[c + sk + v * sv], Q[c - sk + v * sv], sl);
    else
      dqz[v] = R(0);
  }
  R r = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW], A = q[IA], Bc = q[IB], C = q[IC];
  const R drx = dqx[ID] * R(0.5), dpx = dqx[IP] * R(0.5), dux = dqx[IU] * R(0.5),
          dvx = dqx[IV] * R(0.5), dwx = dqx[IW] * R(0.5), dCx = dqx[IC] * R(0.5),
          dBx = dqx[IB] * R(0.5);
  const R dry = dqy[ID] * R(0.5), dpy = dqy[IP] * R(0.5), duy = dqy[IU] * R(0.5),
          dvy = dqy[IV] * R(0.5), dwy = dqy[IW] * R(0.5), dCy = dqy[IC] * R(0.5),
          dAy = dqy[IA] * R(0.5);
  const R ir = kExactOrder ? R(0) : rcp(r);

  if constexpr (DIM == 2)
  {
    // Ez at the four corners from the 3x3 primitive and 4x4 face neighbourhoods
    R Ez[2][2];
#pragma unroll
    for (int di = 0; di < 2; ++di)
#pragma unroll
      for (int dj = 0; dj < 2; ++dj)
      {
        const int64_t cc = c + di + dj * sj;
        const R uu = R(0.25) * (Q[cc - 1 - sj + IU * sv] + Q[cc - 1 + IU * sv] +
                                Q[cc - sj + IU * sv] + Q[cc + IU * sv]);
        const R vv = R(0.25) * (Q[cc - 1 - sj + IV * sv] + Q[cc - 1 + IV * sv] +
                                Q[cc - sj + IV * sv] + Q[cc + IV * sv]);
        const R AA = R(0.5) * (U[cc - sj + IA * sv] + U[cc + IA * sv]);
        const R BB = R(0.5) * (U[cc - 1 + IB * sv] + U[cc + IB * sv]);
        Ez[di][dj] = uu * BB - vv * AA;
      }
    const R ELL = Ez[0][0], ELR = Ez[0][1], ERL = Ez[1][0], ERR = Ez[1][1];
    R       AL = U[c + IA * sv], AR = U[c + 1 + IA * sv];
    R       BL = U[c + IB * sv], BR = U[c + sj + IB * sv];
    // transverse face-field slopes (slope_unsplit_mhd_2d, MHDBaseFunctor2D.h:450-509)
    const R *Ua = U + IA * sv, *Ub = U + IB * sv;
    const R  dALy = R(0.5) * slope_limited(Ua[c], Ua[c + sj], Ua[c - sj], sl);
    const R  dBLx = R(0.5) * slope_limited(Ub[c], Ub[c + 1], Ub[c - 1], sl);
    const R  dARy = R(0.5) * slope_limited(Ua[c + 1], Ua[c + 1 + sj], Ua[c + 1 - sj], sl);
    const R  dBRx = R(0.5) * slope_limited(Ub[c + sj], Ub[c + sj + 1], Ub[c + sj - 1], sl);
    const R  dAx = R(0.5) * (AR - AL);
    const R  dBy = R(0.5) * (BR - BL);
    const R  sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
    R        su0, sv0, sw0;
    if constexpr (kExactOrder)
    {
      su0 = (-u * dux - dpx / r - Bc * dBx / r - C * dCx / r) * dtdx + (-v * duy + Bc * dAy / r) * dtdy;
      sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - C * dCy / r) * dtdy;
      sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + Bc * dCy / r) * dtdy;
    }
    else
    {
      su0 = (-u * dux - (dpx + Bc * dBx + C * dCx) * ir) * dtdx + (-v * duy + Bc * dAy * ir) * dtdy;
      sv0 = (-u * dvx + A * dBx * ir) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) * ir) * dtdy;
      sw0 = (-u * dwx + A * dCx * ir) * dtdx + (-v * dwy + Bc * dCy * ir) * dtdy;
    }
    const R sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
    const R sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy;
    const R sB0 = (-u * dBx - Bc * dux + v * dAx + A * dvx) * dtdx;
    const R sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx + (-v * dCy - C * dvy + w * dBy + Bc * dwy) * dtdy;
    const R sAL0 = +(ELR - ELL) * R(0.5) * dtdy;
    const R sAR0 = +(ERR - ERL) * R(0.5) * dtdy;
    const R sBL0 = -(ERL - ELL) * R(0.5) * dtdx;
    const R sBR0 = -(ERR - ELR) * R(0.5) * dtdx;
    r = r + sr0;
    u = u + su0;
    v = v + sv0;
    w = w + sw0;
    p = p + sp0;
    A = A + sA0;
    Bc = Bc + sB0;
    C = C + sC0;
    AL = AL + sAL0;
    AR = AR + sAR0;
    BL = BL + sBL0;
    BR = BR + sBR0;
    R s[NV];
    // qp / qm along x and y
    s[ID] = r - drx; s[IU] = u - dux; s[IV] = v - dvx; s[IW] = w - dwx; s[IP] = p - dpx;
    s[IA] = AL; s[IB] = Bc - dBx; s[IC] = C - dCx;
    put_state<R, 2>(T, sv, c, TL::qp(0), s, smallR, smallp);
    s[ID] = r + drx; s[IU] = u + dux; s[IV] = v + dvx; s[IW] = w + dwx; s[IP] = p + dpx;
    s[IA] = AR; s[IB] = Bc + dBx; s[IC] = C + dCx;
    put_state<R, 2>(T, sv, c, TL::qm(0), s, smallR, smallp);
    s[ID] = r - dry; s[IU] = u - duy; s[IV] = v - dvy; s[IW] = w - dwy; s[IP] = p - dpy;
    s[IA] = A - dAy; s[IB] = BL; s[IC] = C - dCy;
    put_state<R, 2>(T, sv, c, TL::qp(1), s, smallR, smallp);
    s[ID] = r + dry; s[IU] = u + duy; s[IV] = v + dvy; s[IW] = w + dwy; s[IP] = p + dpy;
    s[IA] = A + dAy; s[IB] = BR; s[IC] = C + dCy;
    put_state<R, 2>(T, sv, c, TL::qm(1), s, smallR, smallp);
    // corner states
    s[ID] = r + (+drx + dry); s[IU] = u + (+dux + duy); s[IV] = v + (+dvx + dvy);
    s[IW] = w + (+dwx + dwy); s[IP] = p + (+dpx + dpy);
    s[IA] = AR + (+dARy); s[IB] = BR + (+dBRx); s[IC] = C + (+dCx + dCy);
    put_state<R, 2>(T, sv, c, TL::edge(0, 2), s, smallR, smallp);
    s[ID] = r + (+drx - dry); s[IU] = u + (+dux - duy); s[IV] = v + (+dvx - dvy);
    s[IW] = w + (+dwx - dwy); s[IP] = p + (+dpx - dpy);
    s[IA] = AR + (-dARy); s[IB] = BL + (+dBLx); s[IC] = C + (+dCx - dCy);
    put_state<R, 2>(T, sv, c, TL::edge(1, 2), s, smallR, smallp);
    s[ID] = r + (-drx + dry); s[IU] = u + (-dux + duy); s[IV] = v + (-dvx + dvy);
    s[IW] = w + (-dwx + dwy); s[IP] = p + (-dpx + dpy);
    s[IA] = AL + (+dALy); s[IB] = BR + (-dBRx); s[IC] = C + (-dCx + dCy);
    put_state<R, 2>(T, sv, c, TL::edge(2, 2), s, smallR, smallp);
    s[ID] = r + (-drx - dry); s[IU] = u + (-dux - duy); s[IV] = v + (-dvx - dvy);
    s[IW] = w + (-dwx - dwy); s[IP] = p + (-dpx - dpy);
    s[IA] = AL + (-dALy); s[IB] = BL + (-dBLx); s[IC] = C + (-dCx - dCy);
    put_state<R, 2>(T, sv, c, TL::edge(3, 2), s, smallR, smallp);
  }
  else
  {
    const R drz = dqz[ID] * R(0.5), dpz = dqz[IP] * R(0.5), duz = dqz[IU] * R(0.5),
            dvz = dqz[IV] * R(0.5), dwz = dqz[IW] * R(0.5), dAz = dqz[IA] * R(0.5),
            dBz = dqz[IB] * R(0.5);
    const R *Ex = E, *Ey = E + sv, *Ez = E + 2 * sv;
    const R  ELL = Ex[c], ELR = Ex[c + sk], ERL = Ex[c + sj], ERR = Ex[c + sj + sk];
    const R  FLL = Ey[c], FLR = Ey[c + sk], FRL = Ey[c + 1], FRR = Ey[c + 1 + sk];
    const R  GLL = Ez[c], GLR = Ez[c + sj], GRL = Ez[c + 1], GRR = Ez[c + 1 + sj];
    R        AL = U[c + IA * sv], AR = U[c + 1 + IA * sv];
    R        BL = U[c + IB * sv], BR = U[c + sj + IB * sv];
    R        CL = U[c + IC * sv], CR = U[c + sk + IC * sv];
    const R dALy = R(0.5) * D[c], dALz = R(0.5) * D[c + sv];
    const R dBLx = R(0.5) * D[c + 2 * sv], dBLz = R(0.5) * D[c + 3 * sv];
    const R dCLx = R(0.5) * D[c + 4 * sv], dCLy = R(0.5) * D[c + 5 * sv];
    const R dARy = R(0.5) * D[c + 1], dARz = R(0.5) * D[c + 1 + sv];
    const R dBRx = R(0.5) * D[c + sj + 2 * sv], dBRz = R(0.5) * D[c + sj + 3 * sv];
    const R dCRx = R(0.5) * D[c + sk + 4 * sv], dCRy = R(0.5) * D[c + sk + 5 * sv];
    const R dAx = R(0.5) * (AR - AL), dBy = R(0.5) * (BR - BL), dCz = R(0.5) * (CR - CL);
    const R sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
    const R su0 = (-u * dux - div_r(dpx + Bc * dBx + C * dCx, r, ir)) * dtdx +
                  (-v * duy + div_r(Bc * dAy, r, ir)) * dtdy + (-w * duz + div_r(C * dAz, r, ir)) * dtdz;
    const R sv0 = (-u * dvx + div_r(A * dBx, r, ir)) * dtdx +
                  (-v * dvy - div_r(dpy + A * dAy + C * dCy, r, ir)) * dtdy +
                  (-w * dvz + div_r(C * dBz, r, ir)) * dtdz;
    const R sw0 = (-u * dwx + div_r(A * dCx, r, ir)) * dtdx + (-v * dwy + div_r(Bc * dCy, r, ir)) * dtdy +
                  (-w * dwz - div_r(dpz + A * dAz + Bc * dBz, r, ir)) * dtdz;
    const R sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
                  (-w * dpz - dwz * gamma * p) * dtdz;
    const R sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy + (u * dCz + C * duz - w * dAz - A * dwz) * dtdz;
    const R sB0 = (v * dAx + A * dvx - u * dBx - Bc * dux) * dtdx + (v * dCz + C * dvz - w * dBz - Bc * dwz) * dtdz;
    const R sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx + (w * dBy + Bc * dwy - v * dCy - C * dvy) * dtdy;
    const R sAL0 = +(GLR - GLL) * dtdy * R(0.5) - (FLR - FLL) * dtdz * R(0.5);
    const R sAR0 = +(GRR - GRL) * dtdy * R(0.5) - (FRR - FRL) * dtdz * R(0.5);
    const R sBL0 = -(GRL - GLL) * dtdx * R(0.5) + (ELR - ELL) * dtdz * R(0.5);
    const R sBR0 = -(GRR - GLR) * dtdx * R(0.5) + (ERR - ERL) * dtdz * R(0.5);
    const R sCL0 = +(FRL - FLL) * dtdx * R(0.5) - (ERL - ELL) * dtdy * R(0.5);
    const R sCR0 = +(FRR - FLR) * dtdx * R(0.5) - (ERR - ELR) * dtdy * R(0.5);
    r = r + sr0;
    u = u + su0;
    v = v + sv0;
    w = w + sw0;
    p = p + sp0;
    A = A + sA0;
    Bc = Bc + sB0;
    C = C + sC0;
    AL = AL + sAL0;
    AR = AR + sAR0;
    BL = BL + sBL0;
    BR = BR + sBR0;
    CL = CL + sCL0;
    CR = CR + sCR0;
    R s[NV];
    // face states
    s[ID] = r - drx; s[IU] = u - dux; s[IV] = v - dvx; s[IW] = w - dwx; s[IP] = p - dpx;
    s[IA] = AL; s[IB] = Bc - dBx; s[IC] = C - dCx;
    put_state<R, 3>(T, sv, c, TL::qp(0), s, smallR, smallp);
    s[ID] = r + drx; s[IU] = u + dux; s[IV] = v + dvx; s[IW] = w + dwx; s[IP] = p + dpx;
    s[IA] = AR; s[IB] = Bc + dBx; s[IC] = C + dCx;
    put_state<R, 3>(T, sv, c, TL::qm(0), s, smallR, smallp);
    s[ID] = r - dry; s[IU] = u - duy; s[IV] = v - dvy; s[IW] = w - dwy; s[IP] = p - dpy;
    s[IA] = A - dAy; s[IB] = BL; s[IC] = C - dCy;
    put_state<R, 3>(T, sv, c, TL::qp(1), s, smallR, smallp);
    s[ID] = r + dry; s[IU] = u + duy; s[IV] = v + dvy; s[IW] = w + dwy; s[IP] = p + dpy;
    s[IA] = A + dAy; s[IB] = BR; s[IC] = C + dCy;
    put_state<R, 3>(T, sv, c, TL::qm(1), s, smallR, smallp);
    s[ID] = r - drz; s[IU] = u - duz; s[IV] = v - dvz; s[IW] = w - dwz; s[IP] = p - dpz;
    s[IA] = A - dAz; s[IB] = Bc - dBz; s[IC] = CL;
    put_state<R, 3>(T, sv, c, TL::qp(2), s, smallR, smallp);
    s[ID] = r + drz; s[IU] = u + duz; s[IV] = v + dvz; s[IW] = w + dwz; s[IP] = p + dpz;
    s[IA] = A + dAz; s[IB] = Bc + dBz; s[IC] = CR;
    put_state<R, 3>(T, sv, c, TL::qm(2), s, smallR, smallp);
    // X-edge corner states
    s[ID] = r + (+dry + drz); s[IU] = u + (+duy + duz); s[IV] = v + (+dvy + dvz);
    s[IW] = w + (+dwy + dwz); s[IP] = p + (+dpy + dpz);
    s[IA] = A + (+dAy + dAz); s[IB] = BR + (+dBRz); s[IC] = CR + (+dCRy);
    put_state<R, 3>(T, sv, c, TL::edge(0, 0), s, smallR, smallp);
    s[ID] = r + (+dry - drz); s[IU] = u + (+duy - duz); s[IV] = v + (+dvy - dvz);
    s[IW] = w + (+dwy - dwz); s[IP] = p + (+dpy - dpz);
    s[IA] = A + (+dAy - dAz); s[IB] = BR + (-dBRz); s[IC] = CL + (+dCLy);
    put_state<R, 3>(T, sv, c, TL::edge(1, 0), s, smallR, smallp);
    s[ID] = r + (-dry + drz); s[IU] = u + (-duy + duz); s[IV] = v + (-dvy + dvz);
    s[IW] = w + (-dwy + dwz); s[IP] = p + (-dpy + dpz);
    s[IA] = A + (-dAy + dAz); s[IB] = BL + (+dBLz); s[IC] = CR + (-dCRy);
    put_state<R, 3>(T, sv, c, TL::edge(2, 0), s, smallR, smallp);
    s[ID] = r + (-dry - drz); s[IU] = u + (-duy - duz); s[IV] = v + (-dvy - dvz);
    s[IW] = w + (-dwy - dwz); s[IP] = p + (-dpy - dpz);
    s[IA] = A + (-dAy - dAz); s[IB] = BL + (-dBLz); s[IC] = CL + (-dCLy);
    put_state<R, 3>(T, sv, c, TL::edge(3, 0), s, smallR, smallp);
    // Y-edge corner states
    s[ID] = r + (+drx + drz); s[IU] = u + (+dux + duz); s[IV] = v + (+dvx + dvz);
    s[IW] = w + (+dwx + dwz); s[IP] = p + (+dpx + dpz);
    s[IA] = AR + (+dARz); s[IB] = Bc + (+dBx + dBz); s[IC] = CR + (+dCRx);
    put_state<R, 3>(T, sv, c, TL::edge(0, 1), s, smallR, smallp);
    s[ID] = r + (+drx - drz); s[IU] = u + (+dux - duz); s[IV] = v + (+dvx - dvz);
    s[IW] = w + (+dwx - dwz); s[IP] = p + (+dpx - dpz);
    s[IA] = AR + (-dARz); s[IB] = Bc + (+dBx - dBz); s[IC] = CL + (+dCLx);
    put_state<R, 3>(T, sv, c, TL::edge(1, 1), s, smallR, smallp);
    s[ID] = r + (-drx + drz); s[IU] = u + (-dux + duz); s[IV] = v + (-dvx + dvz);
    s[IW] = w + (-dwx + dwz); s[IP] = p + (-dpx + dpz);
    s[IA] = AL + (+dALz); s[IB] = Bc + (-dBx + dBz); s[IC] = CR + (-dCRx);
    put_state<R, 3>(T, sv, c, TL::edge(2, 1), s, smallR, smallp);
    s[ID] = r + (-drx - drz); s[IU] = u + (-dux - duz); s[IV] = v + (-dvx - dvz);
    s[IW] = w + (-dwx - dwz); s[IP] = p + (-dpx - dpz);
    s[IA] = AL + (-dALz); s[IB] = Bc + (-dBx - dBz); s[IC] = CL + (-dCLx);
    put_state<R, 3>(T, sv, c, TL::edge(3, 1), s, smallR, smallp);
    // Z-edge corner states
    s[ID] = r + (+drx + dry); s[IU] = u + (+dux + duy); s[IV] = v + (+dvx + dvy);
    s[IW] = w + (+dwx + dwy); s[IP] = p + (+dpx + dpy);
    s[IA] = AR + (+dARy); s[IB] = BR + (+dBRx); s[IC] = C + (+dCx + dCy);
    put_state<R, 3>(T, sv, c, TL::edge(0, 2), s, smallR, smallp);
    s[ID] = r + (+drx - dry); s[IU] = u + (+dux - duy); s[IV] = v + (+dvx - dvy);
    s[IW] = w + (+dwx - dwy); s[IP] = p + (+dpx - dpy);
    s[IA] = AR + (-dARy); s[IB] = BL + (+dBLx); s[IC] = C + (+dCx - dCy);
    put_state<R, 3>(T, sv, c, TL::edge(1, 2), s, smallR, smallp);
    s[ID] = r + (-drx + dry); s[IU] = u + (-dux + duy); s[IV] = v + (-dvx + dvy);
    s[IW] = w + (-dwx + dwy); s[IP] = p + (-dpx + dpy);
    s[IA] = AL + (+dALy); s[IB] = BR + (-dBRx); s[IC] = C + (-dCx + dCy);
    put_state<R, 3>(T, sv, c, TL::edge(2, 2), s, smallR, smallp);
    s[ID] = r + (-drx - dry); s[IU] = u + (-dux - duy); s[IV] = v + (-dvx - dvy);
    s[IW] = w + (-dwx - dwy); s[IP] = p + (-dpx - dpy);
    s[IA] = AL + (-dALy); s[IB] = BL + (-dBLx); s[IC] = C + (-dCx - dCy);
    put_state<R, 3>(T, sv, c, TL::edge(3, 2), s, smallR, smallp);
  }
}

// ---------------------------------------------------------------- fluxes and EMFs

// ComputeFluxesAndStoreFunctor / ComputeFluxesAndUpdateFunctor flux part
// (MHDRunFunctors2D.h:375-607, 3D:1783-2095): Riemann problem between
// qm_d of the left cell and qp_d of the right cell, in the face-normal
// frame; stored in the physical frame (as UpdateFunctor reads it).
template <class R, int DIM, int d>
__device__ __forceinline__ void
v0_flux_face(const Grid<R> & G, const R * __restrict__ T, R * __restrict__ F, int i, int j, int k)
{
  using TL = TraceLayout<DIM>;
  const int64_t sv = G.sv;
  const int64_t off = d == 0 ? 1 : (d == 1 ? G.sj : G.sk);
  const int64_t c = cell_at(G, i, j, k);
  State<R>      qL, qR, fl;
  const R *     Tm = T + (int64_t)TL::qm(d) * NV * sv + c - off;
  const R *     Tp = T + (int64_t)TL::qp(d) * NV * sv + c;
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    qL[v] = Tm[v * sv];
    qR[v] = Tp[v * sv];
  }
  if constexpr (d > 0)
  {
    swap_vals(qL[IU], qL[IU + d]);
    swap_vals(qL[IA], qL[IA + d]);
    swap_vals(qR[IU], qR[IU + d]);
    swap_vals(qR[IA], qR[IA + d]);
  }
#pragma unroll
  for (int v = 0; v < NV; ++v)
    fl[v] = R(0);
  riemann(G.riemann, qL, qR, fl, G.gamma0, G.entho);
  if constexpr (d > 0)
  {
    swap_vals(fl[IU], fl[IU + d]);
    swap_vals(fl[IA], fl[IA + d]);
  }
  constexpr int NF = FluxComps<DIM>::NF;
  R * Fd = F + (int64_t)d * NF * sv;
#pragma unroll
  for (int q = 0; q < NF; ++q)
    Fd[c + q * sv] = fl[FluxComps<DIM>::var(q)];
}

template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_v0_flux(const Grid<R> G, const R * __restrict__ T, R * __restrict__ F, const DevState * st)
{
  if (step_finished(st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  if (blockIdx.y == 0)
    v0_flux_face<R, DIM, 0>(G, T, F, i, j, k);
  else if (blockIdx.y == 1)
    v0_flux_face<R, DIM, 1>(G, T, F, i, j, k);
  else if constexpr (DIM == 3)
    v0_flux_face<R, DIM, 2>(G, T, F, i, j, k);
}

// ComputeEmfAndStoreFunctor (MHDRunFunctors2D.h:612-686, 3D:2100-2238):
// the four stored corner states around the edge, with RB and LT exchanged
// for y edges.
template <class R, int DIM, int edir>
__device__ __forceinline__ void
v0_emf_edge(const Grid<R> & G, const R * __restrict__ T, R * __restrict__ Em, int i, int j, int k)
{
  using TL = TraceLayout<DIM>;
  const int64_t sv = G.sv;
  constexpr int d0 = edir == 0 ? 1 : 0, d1 = edir == 2 ? 1 : 2;
  const int64_t stride[3] = { 1, G.sj, G.sk };
  const int64_t o0 = stride[d0], o1 = DIM == 2 ? G.sj : stride[d1];
  const int64_t c = cell_at(G, i, j, k);
  // (source corner, cell) for slots RT, RB, LT, LB
  const int64_t cell[4] = { c - o0 - o1, c - o0, c - o1, c };
  int           corner[4] = { 0, 1, 2, 3 };
  if constexpr (DIM == 3 && edir == 1)
  {
    // y edges: slot RB reads the LT state of cell c - o1, slot LT the RB
    // state of cell c - o0 (MHDRunFunctors3D.h:2212-2217)
    corner[1] = 2;
    corner[2] = 1;
  }
  State<R> qe[4];
#pragma unroll
  for (int e = 0; e < 4; ++e)
  {
    const int64_t cc = (DIM == 3 && edir == 1 && (e == 1 || e == 2)) ? cell[3 - e] : cell[e];
    const R *     src = T + (int64_t)TL::edge(corner[e], edir) * NV * sv + cc;
#pragma unroll
    for (int v = 0; v < NV; ++v)
      qe[e][v] = src[v * sv];
  }
  Em[c + (DIM == 2 ? 0 : (int64_t)edir * sv)] = compute_emf(edir, qe, G.gamma0, G.smallc);
}

template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_v0_emf(const Grid<R> G, const R * __restrict__ T, R * __restrict__ Em, const DevState * st)
{
  if (step_finished(st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  if constexpr (DIM == 2)
    v0_emf_edge<R, 2, 2>(G, T, Em, i, j, k);
  else if (blockIdx.y == 0)
    v0_emf_edge<R, 3, 0>(G, T, Em, i, j, k);
  else if (blockIdx.y == 1)
    v0_emf_edge<R, 3, 1>(G, T, Em, i, j, k);
  else
    v0_emf_edge<R, 3, 2>(G, T, Em, i, j, k);
}

// ---------------------------------------------------------------- update

// Version 0: UpdateFunctor (MHDRunFunctors2D.h:1539-1641, 3D:2430-2544) and
// UpdateEmfFunctor (2D:1646-1699, 3D:2549-2628).
// Version 1: the atomic updates of ComputeFluxesAndUpdateFunctor and
// ComputeEmfAndUpdateFunctor (2D:475-777, 3D:1914-2424) in serial order:
// a cell first receives the faces it owns (x, y, z), then the far faces in
// the order their threads run (z, y, x); face fields likewise.
template <class R, int DIM, int VERSION>
__global__ void __launch_bounds__(256)
k_v0_update(const Grid<R> G, const R * __restrict__ Uin, R * __restrict__ Uout,
            const R * __restrict__ F, const R * __restrict__ Em, const DevState * st)
{
  if (step_finished(st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_INTERIOR], blockIdx.x * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    return;
  const int64_t sv = G.sv, sj = G.sj, sk = G.sk;
  const int64_t c = cell_at(G, i, j, k);
  R             dtd[3];
  dt_over_dx(st, dtd[0], dtd[1], dtd[2]);
  const int64_t off[3] = { 1, sj, sk };
  constexpr int NF = FluxComps<DIM>::NF;
#pragma unroll
  for (int q = 0; q < NF; ++q)
  {
    const int v = FluxComps<DIM>::var(q);
    R         x = Uin[c + v * sv];
    if constexpr (VERSION == 0)
    {
#pragma unroll
      for (int d = 0; d < DIM; ++d)
      {
        const R * Fd = F + ((int64_t)d * NF + q) * sv;
        x += Fd[c] * dtd[d];
        x -= Fd[c + off[d]] * dtd[d];
      }
    }
    else
    {
#pragma unroll
      for (int d = 0; d < DIM; ++d)
        x += F[((int64_t)d * NF + q) * sv + c] * dtd[d];
#pragma unroll
      for (int d = DIM - 1; d >= 0; --d)
        x -= F[((int64_t)d * NF + q) * sv + c + off[d]] * dtd[d];
    }
    Uout[c + v * sv] = x;
  }
  if constexpr (DIM == 2)
  {
    R a = Uin[c + IA * sv], b = Uin[c + IB * sv];
    if constexpr (VERSION == 0)
    {
      a += (Em[c + sj] - Em[c]) * dtd[1];
      b -= (Em[c + 1] - Em[c]) * dtd[0];
    }
    else
    {
      a -= Em[c] * dtd[1];
      a += Em[c + sj] * dtd[1];
      b += Em[c] * dtd[0];
      b -= Em[c + 1] * dtd[0];
    }
    Uout[c + IA * sv] = a;
    Uout[c + IB * sv] = b;
  }
  else
  {
    // Em planes: x edges, y edges, z edges
    const R *eX = Em, *eY = Em + sv, *eZ = Em + 2 * sv;
    R        a = Uin[c + IA * sv], b = Uin[c + IB * sv], cz = Uin[c + IC * sv];
    if constexpr (VERSION == 0)
    {
      a += (eZ[c + sj] - eZ[c]) * dtd[1];
      b -= (eZ[c + 1] - eZ[c]) * dtd[0];
      a -= (eY[c + sk] - eY[c]) * dtd[2];
      b += (eX[c + sk] - eX[c]) * dtd[2];
      cz += (eY[c + 1] - eY[c]) * dtd[0];
      cz -= (eX[c + sj] - eX[c]) * dtd[1];
    }
    else
    {
      a -= eZ[c] * dtd[1];
      a += eY[c] * dtd[2];
      a -= eY[c + sk] * dtd[2];
      a += eZ[c + sj] * dtd[1];
      b += eZ[c] * dtd[0];
      b -= eX[c] * dtd[2];
      b += eX[c + sk] * dtd[2];
      b -= eZ[c + 1] * dtd[0];
      cz -= eY[c] * dtd[0];
      cz += eX[c] * dtd[1];
      cz -= eX[c + sj] * dtd[1];
      cz += eY[c + 1] * dtd[0];
    }
    Uout[c + IA * sv] = a;
    Uout[c + IB * sv] = b;
    Uout[c + IC * sv] = cz;
  }
}

} // namespace MHD_VARIANT_TAG
} // namespace mhd
