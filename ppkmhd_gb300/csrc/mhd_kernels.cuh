// Kernels of one MUSCL-Hancock + HLLD + CT iteration (implementation
// version 2 of ppkMHD), templated on the real type R and the dimension DIM.
//
// One iteration is 8 launches on one stream, all in gather form (every face
// flux and edge EMF is computed once by one thread and every cell is updated
// by the thread that owns it; no atomics, bitwise deterministic):
//
//   k_boundaries  ghost fill of U_in (periodic / reflecting / outflow)
//   k_prim_dt     primitives Q over [0,size-1)^DIM + CFL max-reduction (FP64)
//   k_finalize_dt dt = cfl / max, clipped to tEnd; dt/dx, dt/dy, dt/dz
//   k_trace       limited slopes S_d, half-step primitives Q2, edge fields E,
//                 transverse face-field slopes (H)
//   k_flux        HLLD face fluxes F_d (face-normal B predicted with curl E,
//                 stored in H for the edge stage)
//   k_emf         reconstructed edge states -> 2D HLLD EMFs
//   k_update      U_out = U_in - div F (hydro), U_out = U_in + curl EMF (face B)
//   k_advance     iteration += 1, t += dt
//
// Device layout: SoA var-planes, i fastest, ghost cells included:
//   U[i + isize*(j + jsize*(k + ksize*var))]   (Kokkos LayoutLeft)
// The time-step state (t, dt, iteration, the reduction word) lives in device
// memory so that whole runs replay from a CUDA graph without host syncs.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "mhd_physics.cuh"
#include "ppkmhd_gb300.h"

#ifndef MHD_VARIANT_TAG
#  define MHD_VARIANT_TAG v_default
#endif

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

// Device-resident time-step bookkeeping (SolverBase m_t, m_dt, m_iteration).
struct DevState
{
  double             t, dt, tEnd;
  double             dtdx, dtdy, dtdz;
  unsigned long long invdt_bits; // max of the CFL rate, as the bits of a non-negative double
  int                it, nStepmax;
  int                status; // bit 0: non-finite or non-positive state seen
  int                pad;
  float              fdtdx, fdtdy, fdtdz; // dt/dx... rounded once for the FP32 kernels
  // FP32 kernels: the momentum fluxes of this iteration are stored minus the
  // constant fp0 = (max + min) / 2 of the interior cells' total pressure
  // p + B^2/2 (bit patterns of positive floats order like the values)
  float              fp0;
  unsigned           ptmax_bits, ptmin_bits;
};

// The total-pressure shift of the momentum fluxes: the flux divergence only
// sees differences of fluxes of one direction, so subtracting one constant
// from all of them leaves the update unchanged, while the FP32 rounding of
// the Riemann solver's total pressure and of the stored flux applies to
// |p_tot - fp0| instead of p_tot.  FP64 kernels take no shift.
__device__ __forceinline__ double
flux_shift(const DevState *, double)
{
  return 0.0;
}
__device__ __forceinline__ float
flux_shift(const DevState * st, float)
{
  return st->fp0;
}

// dt/dx, dt/dy, dt/dz in the working precision
__device__ __forceinline__ void
dt_over_dx(const DevState * st, double & x, double & y, double & z)
{
  x = st->dtdx;
  y = st->dtdy;
  z = st->dtdz;
}
__device__ __forceinline__ void
dt_over_dx(const DevState * st, float & x, float & y, float & z)
{
  x = st->fdtdx;
  y = st->fdtdy;
  z = st->fdtdz;
}

enum : int
{
  STATUS_NUMERIC = 1,
  STATUS_STAGING = 2 // a tile's bulk copies did not complete within the wait bound
};


template <class R>
struct Buffers
{
  R *       Uin;
  R *       Uout;
  R *       Q;   // primitives, 8 planes
  R *       Q2;  // half-step primitives, 8 planes
  R *       S;   // limited slopes, DIM blocks of 8 planes
  R *       E;   // edge electric field (1 plane in 2D, Ex/Ey/Ez in 3D)
  R *       F;   // face fluxes, DIM blocks of NF planes
  R *       Em;  // edge EMFs (1 plane in 2D, 3 in 3D)
  R *       H;   // face data, FaceData<DIM>::NPLANES planes (below)
  // FP32 contexts: the low parts of the state (8 planes; U = U_in + Ulo to
  // about 48 bits), updated in place by k_update; nullptr: plain FP32 state
  R *       Ulo;
  DevState *st;
};

// Face-centred quantities the edge reconstruction reads many times, stored
// once: planes [0, DIM) hold the half-step face-normal field
// B_d + (curl E)_d dt/2 of face (c, d), written by the flux stage on the
// face box (the edge stage evaluates the layer below it with the same
// expression, face_field); planes [DIM, NPLANES) the limited slopes of the
// face-centred field along the transverse directions the edges use, written
// by the trace stage.  Every stored value is the expression the edge stage
// would otherwise evaluate, so the edge EMFs are unchanged bit for bit.
template <int DIM>
struct FaceData
{
  static constexpr int NSLOPE = DIM == 2 ? 2 : 4;
  static constexpr int NPLANES = DIM + NSLOPE;
  // plane holding the slope of face field f (0 = Bx, 1 = By, 2 = Bz) along
  // direction t; -1 for the slopes along z, which are identically zero
  // (compute_limited_slope<IZ> samples its minus neighbour at k + 1,
  // MHDBaseFunctor3D.h:128-158)
  __host__ __device__ static constexpr int
  slope_plane(int f, int t)
  {
    return (f == 0 && t == 1)   ? DIM
           : (f == 1 && t == 0) ? DIM + 1
           : (f == 2 && t == 0) ? DIM + 2
           : (f == 2 && t == 1) ? DIM + 3
                                : -1;
  }
};

inline int
face_data_planes(int dim)
{
  return dim == 3 ? FaceData<3>::NPLANES : FaceData<2>::NPLANES;
}

template <int DIM>
struct FluxComps
{
  // hydro components updated by the face fluxes: 2D also updates Bz
  // (MHDRunFunctors2D.h:1231-1273), 3D none of B (MHDRunFunctors3D.h:1255-1313)
  static constexpr int NF = DIM == 2 ? 6 : 5;
  __device__ static constexpr int var(int c) { return c < 5 ? c : IC; }
};

__device__ __forceinline__ bool
step_finished(const DevState * st)
{
  // SolverBase::finished (SolverBase.cpp:195-201)
  return st->t >= (st->tEnd - 1e-14) || st->it >= st->nStepmax;
}

// Unsigned 32-bit division by a run-time constant d >= 1 through a
// multiply-high (Granlund & Montgomery, 1994): with s = ceil(log2 d) and
// m = ceil(2^(32+s) / d) - 2^32, q = (umulhi(x, m) + x) >> s for every 32-bit x.
// The constants are computed on the host.
struct FastDiv
{
  unsigned d = 1, m = 0, s = 0;
  FastDiv() = default;
  explicit FastDiv(unsigned dv)
    : d(dv)
  {
    s = 0;
    while ((1ull << s) < dv)
      ++s;
    m = (unsigned)(((1ull << (32 + s)) + dv - 1) / dv - (1ull << 32));
  }
  __device__ __forceinline__ unsigned
  div(unsigned x) const
  {
    const unsigned hi = __umulhi(x, m);
    return (unsigned)(((unsigned long long)hi + x) >> s);
  }
};

// A box of cells [lo, lo+n) flattened with i fastest.
struct Box
{
  int     i0 = 0, j0 = 0, k0 = 0, ni = 1, nj = 1, nk = 1;
  FastDiv di, dj;
  Box() = default;
  Box(int a, int b, int c, int n0, int n1, int n2)
    : i0(a)
    , j0(b)
    , k0(c)
    , ni(n0)
    , nj(n1)
    , nk(n2)
    , di((unsigned)n0)
    , dj((unsigned)n1)
  {}
  __host__ __device__ int64_t
  count() const
  {
    return (int64_t)ni * nj * nk;
  }
};

// The boxes the kernels iterate over (filled on the host by make_grid).
enum BoxId : int
{
  BOX_ALL = 0,      // every cell (boundaries)
  BOX_PRIM = 1,     // [0, size-1)^DIM (primitives)
  BOX_TRACE = 2,    // [g-1, size-g+1]^DIM (slopes, half step, edge field)
  BOX_FACE = 3,     // [g, size-g]^DIM (faces and edges)
  BOX_INTERIOR = 4, // interior cells (update, diagnostics)
  BOX_COUNT = 5
};

__device__ __forceinline__ bool
box_cell(const Box & b, int64_t idx, int & i, int & j, int & k)
{
  if (idx >= b.count())
    return false;
  // counts stay below 2^31 (grids are limited to 4e9 values, i.e. 5e8 cells)
  const unsigned x = (unsigned)idx;
  const unsigned r = b.di.div(x);
  i = b.i0 + (int)(x - r * (unsigned)b.ni);
  const unsigned kk = b.dj.div(r);
  j = b.j0 + (int)(r - kk * (unsigned)b.nj);
  k = b.k0 + (int)kk;
  return true;
}

// The items of a W x H grid (W >= 32) in warp order: the first 32 columns
// row by row, one row per warp, so that a warp reads a contiguous run of a
// shared-memory row (no bank conflicts whatever the row pitch), then the
// W - 32 remaining columns; the count is rounded up to whole warps, so that
// consecutive item ranges start on a warp boundary.
template <int W, int H>
struct ItemGrid
{
  static constexpr int MAIN = 32 * H, XW = W - 32;
  static constexpr int COUNT = MAIN + (XW * H + 31) / 32 * 32;
  __device__ __forceinline__ static bool
  at(int w, int & a, int & b)
  {
    if (w < MAIN)
    {
      a = w & 31;
      b = w >> 5;
      return true;
    }
    if constexpr (XW == 0)
      return false;
    else
    {
      w -= MAIN;
      if (w >= XW * H)
        return false;
      a = 32 + w % XW;
      b = w / XW;
      return true;
    }
  }
};

template <class R>
struct Grid
{
  int     dim, nx, ny, nz, g;
  int     isize, jsize, ksize;
  int64_t sj, sk, sv; // strides of j, k and var (i stride is 1)
  int     bc[6];
  int     riemann;
  R       gamma0, smallr, smallp, smallc, slope_type;
  R       entho; // 1 / (gamma0 - 1)
  double  cfl, dx, dy, dz;
  double  idx, idy, idz; // 1/dx, 1/dy, 1/dz (host IEEE quotients, correctly rounded)
  Box     box[BOX_COUNT];
};

template <class R>
__device__ __forceinline__ int64_t
cell_at(const Grid<R> & G, int i, int j, int k)
{
  return (int64_t)i + (int64_t)j * G.sj + (int64_t)k * G.sk;
}

// ---------------------------------------------------------------- boundaries

// Source index along one axis for ghost index c (BoundariesFunctors.h:535-1057).
__device__ __forceinline__ int
bc_source(int c, int n, int g, int type, bool hi, bool & flip)
{
  flip = false;
  if (!hi)
  {
    if (type == 1)
    {
      flip = true;
      return 2 * g - 1 - c;
    }
    if (type == 2)
      return g;
    return n + c;
  }
  if (type == 1)
  {
    flip = true;
    return 2 * n + 2 * g - 1 - c;
  }
  if (type == 2)
    return n + g - 1;
  return c - n;
}

// Ghost fill.  The reference fills the X faces, then Y, then Z, each over
// the full extent of the other axes; a ghost cell therefore ends up with the
// interior value at the composition of the per-axis source maps, multiplied
// by the per-axis reflection signs (normal velocity and normal field).
// Interior cells are left alone.
template <class R, int DIM>
__device__ __forceinline__ void
fill_ghost(const Grid<R> & G, R * __restrict__ U, int i, int j, int k)
{
  const int g = G.g;
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
  const int64_t dst = cell_at(G, i, j, k), src = cell_at(G, i0, j0, k0);
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    R x = U[src + v * G.sv];
    if (fx && (v == IU || v == IA))
      x = x * R(-1);
    if (fy && (v == IV || v == IB))
      x = x * R(-1);
    if (fz && (v == IW || v == IC))
      x = x * R(-1);
    U[dst + v * G.sv] = x;
  }
}

// The ghost cells of the array, enumerated without the interior: the
// ghost layers of the slowest axis whole, then the ghost rows of the
// interior planes (3D), then the ghost columns of the interior rows.  GR:
// any grid description with nx, ny, nz, g, isize, jsize, ksize (the MHD and
// the hydro solvers').
template <class R, int DIM, class GR>
__host__ __device__ __forceinline__ int64_t
ghost_count(const GR & G)
{
  const int64_t all = (int64_t)G.isize * G.jsize * (DIM == 3 ? G.ksize : 1);
  return all - (int64_t)G.nx * G.ny * (DIM == 3 ? G.nz : 1);
}

template <class R, int DIM, class GR>
__device__ __forceinline__ bool
ghost_cell(const GR & G, int64_t idx, int & i, int & j, int & k)
{
  if (idx >= ghost_count<R, DIM>(G))
    return false;
  const int g = G.g, g2 = 2 * G.g;
  // counts stay below 2^31 (grids are limited to 4e9 values)
  unsigned x = (unsigned)idx;
  k = 0;
  if constexpr (DIM == 3)
  {
    const unsigned plane = (unsigned)(G.isize * G.jsize);
    const unsigned nA = (unsigned)g2 * plane;
    if (x < nA)
    {
      const unsigned r = x / plane, rem = x - r * plane;
      k = (int)r < g ? (int)r : G.nz + (int)r;
      j = (int)(rem / (unsigned)G.isize);
      i = (int)(rem - (unsigned)j * (unsigned)G.isize);
      return true;
    }
    x -= nA;
    const unsigned nB = (unsigned)G.nz * (unsigned)g2 * (unsigned)G.isize;
    if (x < nB)
    {
      const unsigned t = x / (unsigned)G.isize;
      i = (int)(x - t * (unsigned)G.isize);
      const unsigned kk = t / (unsigned)g2, r = t - kk * (unsigned)g2;
      k = g + (int)kk;
      j = (int)r < g ? (int)r : G.ny + (int)r;
      return true;
    }
    x -= nB;
    const unsigned t = x / (unsigned)g2, c = x - t * (unsigned)g2;
    i = (int)c < g ? (int)c : G.nx + (int)c;
    const unsigned kk = t / (unsigned)G.ny;
    j = g + (int)(t - kk * (unsigned)G.ny);
    k = g + (int)kk;
    return true;
  }
  else
  {
    const unsigned nA = (unsigned)g2 * (unsigned)G.isize;
    if (x < nA)
    {
      const unsigned r = x / (unsigned)G.isize;
      i = (int)(x - r * (unsigned)G.isize);
      j = (int)r < g ? (int)r : G.ny + (int)r;
      return true;
    }
    x -= nA;
    const unsigned t = x / (unsigned)g2, c = x - t * (unsigned)g2;
    i = (int)c < g ? (int)c : G.nx + (int)c;
    j = g + (int)t;
    return true;
  }
}

// Ghost cell number idx (0 <= idx < ghost_count) of U; first: the launch's
// first thread, which also clears the iteration's CFL reduction.
template <class R, int DIM>
__device__ __forceinline__ void
boundaries_body(const Grid<R> & G, R * __restrict__ U, DevState * st, int force, int64_t idx,
                bool first)
{
  if (!force && step_finished(st))
    return;
  if (first)
  {
    st->invdt_bits = 0ull; // reset the CFL reduction of this iteration
    st->ptmax_bits = 0u;
    st->ptmin_bits = 0x7f800000u; // +inf
  }
  int i, j, k;
  if (ghost_cell<R, DIM>(G, idx, i, j, k))
    fill_ghost<R, DIM>(G, U, i, j, k);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_boundaries(const Grid<R> G, R * __restrict__ U, DevState * st, int force)
{
  boundaries_body<R, DIM>(G, U, st, force, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
                          blockIdx.x == 0 && threadIdx.x == 0);
}

// Ghost fill of the cells base <= index < end of BOX_ALL (a range of planes
// of the slowest axis); reset: this launch is the iteration's first and
// clears the CFL reduction.
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_boundaries_range(const Grid<R> G, R * __restrict__ U, DevState * st, int64_t base, int64_t end,
                   int reset)
{
  const int64_t idx = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= end || step_finished(st))
    return;
  if (reset && blockIdx.x == 0 && threadIdx.x == 0)
  {
    st->invdt_bits = 0ull;
    st->ptmax_bits = 0u;
    st->ptmin_bits = 0x7f800000u;
  }
  int i, j, k;
  if (box_cell(G.box[BOX_ALL], idx, i, j, k))
    fill_ghost<R, DIM>(G, U, i, j, k);
}

// ---------------------------------------------------------------- primitives + CFL

template <class T>
__device__ __forceinline__ T
warp_max(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
    v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ConvertToPrimitivesFunctor (MHDRunFunctors2D.h:85-159, 3D:88-163) with
// constoprim_mhd (MHDBaseFunctor2D.h:194-242), fused with the CFL reduction
// of ComputeDtFunctor (MHDRunFunctors2D.h:16-80, 3D:16-83): for interior
// cells, max over sum_d (c_fast,d + |v_d|)/dx_d.  The max is reduced in FP64
// (warp shuffles, then one atomicMax per block on the bit pattern, which
// orders like the value for non-negative doubles) and is order-independent,
// so dt is bitwise the reference's.
// constoprim_mhd (MHDBaseFunctor2D.h:194-242, MHDBaseFunctor3D.h:194-242)
// of cell c: the cell-centred field is the mean of the cell's two faces per
// direction (the +1 neighbour's face field is read), the density floored at
// smallr, the pressure at d * smallp.  Shared by the stage kernels and the
// fused tile kernel, so both evaluate the same expressions (cell_prim_v: on
// the cell's values u and the +1 neighbours' face fields nbx, nby, nbz).
template <class R>
struct CellPrim
{
  R d, p, vu, vv, vw, a, bb, cc;
  R emag, invd; // 0.5 |B|^2 and the reciprocal of d the quotients used
};

template <class R, int DIM>
__device__ __forceinline__ CellPrim<R>
cell_prim_v(const Grid<R> & G, const R (&u)[NV], R nbx, R nby, R nbz)
{
  const R       d = fmax(u[ID], G.smallr);
  R             vu, vv, vw;
  // exact build: the nine quotients over d share its correctly rounded
  // reciprocal (qdiv: bit for bit the IEEE quotients); fast builds multiply
  // by an approximate reciprocal
  const R       invd = kExactOrder ? qrcp(d) : rcp(d);
  if constexpr (kExactOrder)
  {
    vu = qdiv(u[IU], d, invd);
    vv = qdiv(u[IV], d, invd);
    vw = qdiv(u[IW], d, invd);
  }
  else
  {
    vu = u[IU] * invd;
    vv = u[IV] * invd;
    vw = u[IW] * invd;
  }
  const R       a = R(0.5) * (u[IA] + nbx);
  const R       bb = R(0.5) * (u[IB] + nby);
  const R       cc = R(0.5) * (u[IC] + nbz);
  const R       eken = R(0.5) * (vu * vu + vv * vv + vw * vw);
  const R       emag = R(0.5) * (a * a + bb * bb + cc * cc);
  const R       eint = kExactOrder ? qdiv(u[IP] - emag, d, invd) - eken
                                   : (u[IP] - emag) * invd - eken;
  const R       p = fmax((G.gamma0 - R(1)) * d * eint, d * G.smallp);
  return CellPrim<R>{ d, p, vu, vv, vw, a, bb, cc, emag, invd };
}

template <class R, int DIM>
__device__ __forceinline__ CellPrim<R>
cell_prim(const Grid<R> & G, const R * __restrict__ U, int64_t c)
{
  const int64_t sv = G.sv;
  R             u[NV];
#pragma unroll
  for (int v = 0; v < NV; ++v)
    u[v] = U[c + v * sv];
  const R nbx = U[c + 1 + IA * sv];
  const R nby = U[c + G.sj + IB * sv];
  const R nbz = DIM == 3 ? U[c + G.sk + IC * sv] : R(0);
  return cell_prim_v<R, DIM>(G, u, nbx, nby, nbz);
}

// find_speed_info<NDIM> (mhd_utils.h:319-366) of an interior cell from its
// primitives: the CFL rate sum_d (c_fast,d + |v_d|)/dx_d (0 for NaN), the
// FP32 total pressure p + B^2/2 (the momentum-flux shift), and whether the
// conservative state is non-positive or non-finite.
template <class R, int DIM>
__device__ __forceinline__ void
cell_rate(const Grid<R> & G, const R * __restrict__ U, int64_t c, const CellPrim<R> & P,
          R & rate, R & ptot, bool & bad)
{
  const int64_t sv = G.sv;
  const R d = P.d, p = P.p, vu = P.vu, vv = P.vv, vw = P.vw, a = P.a, bb = P.bb, cc = P.cc;
  const R emag = P.emag, invd = P.invd;
  (void)vw;
  (void)emag;
  const R b2 = a * a + bb * bb + cc * cc;
  R       val;
  if constexpr (kExactOrder)
  {
    // 1/dx.. are the host's IEEE reciprocals (correctly rounded)
    const R c2 = qdiv(G.gamma0 * p, d, invd);
    const R d2 = R(0.5) * (qdiv(b2, d, invd) + c2);
    const R sx = sqrt(d2 + sqrt(d2 * d2 - qdiv(c2 * a * a, d, invd))) + fabs(vu);
    const R sy = sqrt(d2 + sqrt(d2 * d2 - qdiv(c2 * bb * bb, d, invd))) + fabs(vv);
    if constexpr (DIM == 3)
    {
      const R sz = sqrt(d2 + sqrt(d2 * d2 - qdiv(c2 * cc * cc, d, invd))) + fabs(vw);
      val = qdiv(sx, R(G.dx), R(G.idx)) + qdiv(sy, R(G.dy), R(G.idy)) +
            qdiv(sz, R(G.dz), R(G.idz));
    }
    else
      val = qdiv(sx, R(G.dx), R(G.idx)) + qdiv(sy, R(G.dy), R(G.idy));
  }
  else
  {
    const R c2 = G.gamma0 * p * invd;
    const R d2 = R(0.5) * (b2 * invd + c2);
    const R cd = c2 * invd;
    const R sx = fsqrt(d2 + fsqrt(d2 * d2 - cd * a * a)) + fabs(vu);
    const R sy = fsqrt(d2 + fsqrt(d2 * d2 - cd * bb * bb)) + fabs(vv);
    if constexpr (DIM == 3)
    {
      const R sz = fsqrt(d2 + fsqrt(d2 * d2 - cd * cc * cc)) + fabs(vw);
      val = sx * R(G.idx) + sy * R(G.idy) + sz * R(G.idz);
    }
    else
      val = sx * R(G.idx) + sy * R(G.idy);
  }
  // fmax in the reference ignores NaN operands; a NaN rate is dropped
  // (it arises legitimately when round-off makes the inner root of the
  // fast speed slightly negative, e.g. for a field along one axis)
  rate = (val >= R(0)) ? val : R(0);
  if constexpr (sizeof(R) == 4)
    ptot = p + emag;
  const R Ein = U[c + IP * sv];
  bad = !(U[c + ID * sv] > R(0)) || !isfinite(Ein);
}

// The block's part of the CFL reduction (every thread of the block calls
// it): rate, the thread's maximum rate; thi / tlo, the bit patterns of the
// largest / smallest positive finite FP32 total pressure it saw (0 / +inf
// for none); bad, a non-positive or non-finite state seen.
template <class R>
__device__ __forceinline__ void
reduce_dt(DevState * st, R rate, unsigned thi, unsigned tlo, bool bad)
{
  // block max in the working precision (max is exact in any precision), then
  // one FP64 atomicMax per block; FP32 also reduces the range of the
  // positive, finite interior total pressures (bit patterns of positive
  // floats order like the values; max and min are order-independent, so the
  // momentum-flux shift is deterministic), in the same block step
  __shared__ R        red[32];
  __shared__ unsigned rhi[32], rlo[32];
  rate = warp_max(rate);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned  phi = 0u, plo = 0x7f800000u;
  if constexpr (sizeof(R) == 4)
  {
    phi = __reduce_max_sync(0xffffffffu, thi);
    plo = __reduce_min_sync(0xffffffffu, tlo);
  }
  if (lane == 0)
  {
    red[wid] = rate;
    rhi[wid] = phi;
    rlo[wid] = plo;
  }
  if (__syncthreads_or(bad) && threadIdx.x == 0)
    atomicOr(&st->status, STATUS_NUMERIC);
  if (wid == 0)
  {
    const bool in = lane < (int)(blockDim.x >> 5);
    rate = in ? red[lane] : R(0);
    rate = warp_max(rate);
    // one atomic per block, and none when the running maximum (minimum),
    // read first, already covers the block's value: most blocks then skip
    // the atomics that all target the same word (the result is the same)
    const unsigned long long rb = (unsigned long long)__double_as_longlong((double)rate);
    if (lane == 0 && rate > R(0) && rb > *(volatile unsigned long long *)&st->invdt_bits)
      atomicMax(&st->invdt_bits, rb);
    if constexpr (sizeof(R) == 4)
    {
      phi = __reduce_max_sync(0xffffffffu, in ? rhi[lane] : 0u);
      plo = __reduce_min_sync(0xffffffffu, in ? rlo[lane] : 0x7f800000u);
      if (lane == 0 && phi != 0u && phi > *(volatile unsigned *)&st->ptmax_bits)
        atomicMax(&st->ptmax_bits, phi);
      if (lane == 0 && plo != 0x7f800000u && plo < *(volatile unsigned *)&st->ptmin_bits)
        atomicMin(&st->ptmin_bits, plo);
    }
  }
}

// positive finite FP32 total pressures as ordered bit patterns
__device__ __forceinline__ void
ptot_range(float ptot, unsigned & thi, unsigned & tlo)
{
  if (ptot > 0.f && ptot < INFINITY)
  {
    thi = max(thi, __float_as_uint(ptot));
    tlo = min(tlo, __float_as_uint(ptot));
  }
}
__device__ __forceinline__ void
ptot_range(double, unsigned &, unsigned &)
{
}

template <class R, int DIM, bool STORE_Q = true>
__device__ __forceinline__ void
prim_dt_body(const Grid<R> & G, const R * __restrict__ U, R * __restrict__ Q, DevState * st,
             int force, int64_t idx, int64_t end = INT64_MAX)
{
  if (!force && step_finished(st))
    return;
  const Box & b = G.box[STORE_Q ? BOX_PRIM : BOX_INTERIOR];
  int       i, j, k;
  R         rate = R(0);
  R         ptot = R(-1); // FP32: interior total pressure, -1 elsewhere
  bool      bad = false;
  if (idx < end && box_cell(b, idx, i, j, k))
  {
    const int64_t c = cell_at(G, i, j, k);
    const int64_t sv = G.sv;
    const CellPrim<R> P = cell_prim<R, DIM>(G, U, c);
    if constexpr (STORE_Q)
    {
      Q[c + ID * sv] = P.d;
      Q[c + IP * sv] = P.p;
      Q[c + IU * sv] = P.vu;
      Q[c + IV * sv] = P.vv;
      Q[c + IW * sv] = P.vw;
      Q[c + IA * sv] = P.a;
      Q[c + IB * sv] = P.bb;
      Q[c + IC * sv] = P.cc;
    }
    const int g = G.g;
    const bool interior = i >= g && i < G.isize - g && j >= g && j < G.jsize - g &&
                          (DIM == 2 || (k >= g && k < G.ksize - g));
    if (interior)
      cell_rate<R, DIM>(G, U, c, P, rate, ptot, bad);
  }
  unsigned thi = 0u, tlo = 0x7f800000u;
  ptot_range(ptot, thi, tlo);
  reduce_dt<R>(st, rate, thi, tlo, bad);
}

// The CFL reduction alone over CPT cells per thread (the cells of block blk
// of BOX_INTERIOR, CPT consecutive runs of blockDim.x cells): more loads in
// flight per thread and one block reduction per CPT x blockDim.x cells.
template <class R, int DIM, int CPT>
__device__ __forceinline__ void
dt_cells_body(const Grid<R> & G, const R * __restrict__ U, DevState * st, int force, int64_t blk)
{
  if (!force && step_finished(st))
    return;
  const Box & b = G.box[BOX_INTERIOR];
  R           rate = R(0);
  unsigned    thi = 0u, tlo = 0x7f800000u;
  bool        bad = false;
#pragma unroll
  for (int q = 0; q < CPT; ++q)
  {
    int i, j, k;
    if (box_cell(b, (blk * CPT + q) * (int64_t)blockDim.x + threadIdx.x, i, j, k))
    {
      const int64_t     c = cell_at(G, i, j, k);
      const CellPrim<R> P = cell_prim<R, DIM>(G, U, c);
      R                 r = R(0), pt = R(-1);
      bool              bd = false;
      cell_rate<R, DIM>(G, U, c, P, r, pt, bd);
      rate = r > rate ? r : rate;
      ptot_range(pt, thi, tlo);
      bad = bad || bd;
    }
  }
  reduce_dt<R>(st, rate, thi, tlo, bad);
}

template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_prim_dt(const Grid<R> G, const R * __restrict__ U, R * __restrict__ Q, DevState * st, int force)
{
  prim_dt_body<R, DIM>(G, U, Q, st, force, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// cells base <= index < end of BOX_PRIM (threads past end still join the
// block reduction)
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_prim_dt_range(const Grid<R> G, const R * __restrict__ U, R * __restrict__ Q, DevState * st,
                int64_t base, int64_t end)
{
  prim_dt_body<R, DIM>(G, U, Q, st, 0, base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x, end);
}

// compute_dt_local (SolverMHDMuscl.h:722-741) and the clip of
// SolverBase::compute_dt (SolverBase.cpp:148-179); dtdx = m_dt / dx
// (SolverMHDMuscl.cpp:390-391).
template <class R>
__device__ __forceinline__ void
finalize_dt_body(const Grid<R> & G, DevState * st, int force)
{
  if (!force && step_finished(st))
    return;
  const double invDt = __longlong_as_double((long long)st->invdt_bits);
  double       dt;
  if constexpr (sizeof(R) == 8)
    dt = G.cfl / invDt;
  else
    dt = G.cfl / invDt; // FP64 dt for the FP32 storage path
  if (st->t + dt > st->tEnd)
    dt = st->tEnd - st->t;
  st->dt = dt;
  st->dtdx = dt / G.dx;
  st->dtdy = dt / G.dy;
  st->dtdz = dt / G.dz;
  st->fdtdx = (float)st->dtdx;
  st->fdtdy = (float)st->dtdy;
  st->fdtdz = (float)st->dtdz;
  if constexpr (sizeof(R) == 4)
    st->fp0 = st->ptmax_bits >= st->ptmin_bits && st->ptmin_bits < 0x7f800000u
                ? 0.5f * (__uint_as_float(st->ptmax_bits) + __uint_as_float(st->ptmin_bits))
                : 0.f;
  if (!(invDt > 0.0) || !isfinite(dt))
    st->status |= STATUS_NUMERIC;
}

template <class R>
__global__ void
k_finalize_dt(const Grid<R> G, DevState * st, int force)
{
  finalize_dt_body<R>(G, st, force);
}

// godunov_unsplit(dt) with the caller's dt (SolverMHDMuscl.cpp:390-391:
// dtdx = dt / dx): the dt of this iteration instead of the CFL one.
template <class R>
__global__ void
k_set_dt(const Grid<R> G, DevState * st, double dt)
{
  if (step_finished(st))
    return;
  st->dt = dt;
  st->dtdx = dt / G.dx;
  st->dtdy = dt / G.dy;
  st->dtdz = dt / G.dz;
  st->fdtdx = (float)st->dtdx;
  st->fdtdy = (float)st->dtdy;
  st->fdtdz = (float)st->dtdz;
}

template <class R>
__global__ void
k_advance(DevState * st)
{
  if (step_finished(st))
    return;
  st->it += 1;
  st->t += st->dt;
}

// ---------------------------------------------------------------- trace

// compute_limited_slope<dir> of a face-centred field component
// (MHDBaseFunctor2D.h:129-155, MHDBaseFunctor3D.h:128-158).  In 3D the
// reference samples the minus neighbour along z at k + 1, so the z slope is
// identically zero; that is kept.
template <class R, int DIM>
__device__ __forceinline__ R
face_field_slope(const Grid<R> & G, const R * __restrict__ U, uint32_t c, int comp, int dir)
{
  const uint32_t cv = c + (uint32_t)comp * (uint32_t)G.sv;
  const uint32_t sj = (uint32_t)G.sj, sk = (uint32_t)G.sk;
  if (dir == 0)
    return slope_limited(U[cv], U[cv + 1], U[cv - 1], G.slope_type);
  if (dir == 1)
    return slope_limited(U[cv], U[cv + sj], U[cv - sj], G.slope_type);
  // the reference takes the minus sample at k + 1 as well
  // (compute_limited_slope, MHDBaseFunctor3D.h:142), so the z slope is zero;
  // the edge stage uses that zero directly and never calls this for z
  return slope_limited(U[cv], U[cv + sk], U[cv + sk], G.slope_type);
}


// Hancock half step of one cell (ComputeUpdatedPrimVarFunctor,
// MHDRunFunctors2D.h:920-1051, 3D:865-1022): q2 = q + (dt/2) times the
// primitive MHD source terms built from the limited slopes s.  Shared by the
// trace stage and the fused tile kernel.
template <class R, int DIM>
__device__ __forceinline__ void
hancock(const R (&q)[NV], const R (&s)[DIM][NV], R gamma, R dtdx, R dtdy, R dtdz, R (&q2)[NV])
{
  (void)dtdz;
  const R r = q[ID], p = q[IP], u = q[IU], v = q[IV], w = q[IW], A = q[IA], Bc = q[IB], C = q[IC];
  const R drx = s[0][ID], dpx = s[0][IP], dux = s[0][IU], dvx = s[0][IV], dwx = s[0][IW],
          dBx = s[0][IB], dCx = s[0][IC];
  const R dry = s[1][ID], dpy = s[1][IP], duy = s[1][IU], dvy = s[1][IV], dwy = s[1][IW],
          dAy = s[1][IA], dCy = s[1][IC];
  const R dAx = s[0][IA], dBy = s[1][IB];
  R       sr0, su0, sv0, sw0, sp0, sA0, sB0, sC0;
  if constexpr (!kExactOrder)
  {
    // same source terms with one reciprocal of the density
    const R ir = rcp(r);
    if constexpr (DIM == 2)
    {
      sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
      su0 = (-u * dux - (dpx + Bc * dBx + C * dCx) * ir) * dtdx + (-v * duy + Bc * dAy * ir) * dtdy;
      sv0 = (-u * dvx + A * dBx * ir) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) * ir) * dtdy;
      sw0 = (-u * dwx + A * dCx * ir) * dtdx + (-v * dwy + Bc * dCy * ir) * dtdy;
      sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
      sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy;
      sB0 = (-u * dBx - Bc * dux + v * dAx + A * dvx) * dtdx;
      sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx +
            (-v * dCy - C * dvy + w * dBy + Bc * dwy) * dtdy;
    }
    else
    {
      const R drz = s[DIM - 1][ID], dpz = s[DIM - 1][IP], duz = s[DIM - 1][IU],
              dvz = s[DIM - 1][IV], dwz = s[DIM - 1][IW], dAz = s[DIM - 1][IA],
              dBz = s[DIM - 1][IB], dCz = s[DIM - 1][IC];
      sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
      su0 = (-u * dux - (dpx + Bc * dBx + C * dCx) * ir) * dtdx + (-v * duy + Bc * dAy * ir) * dtdy +
            (-w * duz + C * dAz * ir) * dtdz;
      sv0 = (-u * dvx + A * dBx * ir) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) * ir) * dtdy +
            (-w * dvz + C * dBz * ir) * dtdz;
      sw0 = (-u * dwx + A * dCx * ir) * dtdx + (-v * dwy + Bc * dCy * ir) * dtdy +
            (-w * dwz - (dpz + A * dAz + Bc * dBz) * ir) * dtdz;
      sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
            (-w * dpz - dwz * gamma * p) * dtdz;
      sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy + (u * dCz + C * duz - w * dAz - A * dwz) * dtdz;
      sB0 = (v * dAx + A * dvx - u * dBx - Bc * dux) * dtdx + (v * dCz + C * dvz - w * dBz - Bc * dwz) * dtdz;
      sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx + (w * dBy + Bc * dwy - v * dCy - C * dvy) * dtdy;
    }
  }
  else if constexpr (DIM == 2)
  {
    sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy;
    su0 = (-u * dux - dpx / r - Bc * dBx / r - C * dCx / r) * dtdx + (-v * duy + Bc * dAy / r) * dtdy;
    sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - dpy / r - A * dAy / r - C * dCy / r) * dtdy;
    sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + Bc * dCy / r) * dtdy;
    sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy;
    sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy;
    sB0 = (-u * dBx - Bc * dux + v * dAx + A * dvx) * dtdx;
    sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx +
          (-v * dCy - C * dvy + w * dBy + Bc * dwy) * dtdy;
  }
  else
  {
    const R drz = s[DIM - 1][ID], dpz = s[DIM - 1][IP], duz = s[DIM - 1][IU],
            dvz = s[DIM - 1][IV], dwz = s[DIM - 1][IW], dAz = s[DIM - 1][IA],
            dBz = s[DIM - 1][IB], dCz = s[DIM - 1][IC];
    // (IEEE quotients here: in this register-heavy stage the shared
    // reciprocal form measured 5 % slower)
    sr0 = (-u * drx - dux * r) * dtdx + (-v * dry - dvy * r) * dtdy + (-w * drz - dwz * r) * dtdz;
    su0 = (-u * dux - (dpx + Bc * dBx + C * dCx) / r) * dtdx + (-v * duy + Bc * dAy / r) * dtdy +
          (-w * duz + C * dAz / r) * dtdz;
    sv0 = (-u * dvx + A * dBx / r) * dtdx + (-v * dvy - (dpy + A * dAy + C * dCy) / r) * dtdy +
          (-w * dvz + C * dBz / r) * dtdz;
    sw0 = (-u * dwx + A * dCx / r) * dtdx + (-v * dwy + Bc * dCy / r) * dtdy +
          (-w * dwz - (dpz + A * dAz + Bc * dBz) / r) * dtdz;
    sp0 = (-u * dpx - dux * gamma * p) * dtdx + (-v * dpy - dvy * gamma * p) * dtdy +
          (-w * dpz - dwz * gamma * p) * dtdz;
    sA0 = (u * dBy + Bc * duy - v * dAy - A * dvy) * dtdy + (u * dCz + C * duz - w * dAz - A * dwz) * dtdz;
    sB0 = (v * dAx + A * dvx - u * dBx - Bc * dux) * dtdx + (v * dCz + C * dvz - w * dBz - Bc * dwz) * dtdz;
    sC0 = (w * dAx + A * dwx - u * dCx - C * dux) * dtdx + (w * dBy + Bc * dwy - v * dCy - C * dvy) * dtdy;
  }
  q2[ID] = r + R(0.5) * sr0;
  q2[IU] = u + R(0.5) * su0;
  q2[IV] = v + R(0.5) * sv0;
  q2[IW] = w + R(0.5) * sw0;
  q2[IP] = p + R(0.5) * sp0;
  q2[IA] = A + R(0.5) * sA0;
  q2[IB] = Bc + R(0.5) * sB0;
  q2[IC] = C + R(0.5) * sC0;
}

// Slopes, half step and edge field over the box [g-1, size-g+1]^DIM:
//  * ComputeSlopesFunctor (MHDRunFunctors2D.h:164-248, 3D:168-273): MC-type
//    limited slopes per direction; the face-normal field slope is the
//    unlimited face difference;
//  * ComputeUpdatedPrimVarFunctor (MHDRunFunctors2D.h:920-1051,
//    3D:865-1022): Q2 = Q + S/2 with the primitive MHD source terms;
//  * ComputeElecFieldFunctor (MHDRunFunctors2D.h:253-314, 3D:278-362):
//    E = v x B at the lower edges of the cell.
// Slopes and Q2 are only consumed on [g-1, size-g]^DIM, the edge field on
// [g-1, size-g+1]^DIM.
//
// PART 0 does all of it.  The host-buffer step splits it where the time step
// is first needed: PART 1 (edge field, slopes, face-field slopes: no dt) runs
// while the state is still arriving, PART 2 (half step) after the CFL
// reduction, reading the slopes back from S (the two normal-field slopes S
// does not keep are the same face differences, taken again).
template <class R, int DIM, int PART = 0>
__device__ __forceinline__ void
trace_body(const Grid<R> & G, const Buffers<R> & B, int64_t idx)
{
  if (step_finished(B.st))
    return;
  const int g = G.g;
  const Box & b = G.box[BOX_TRACE];
  int       i, j, k;
  if (!box_cell(b, idx, i, j, k))
    return;
  // 32-bit element offsets inside arrays of at most 8 planes (grids hold
  // fewer than 4e9 values, checked at context creation)
  const uint32_t sv = (uint32_t)G.sv, sj = (uint32_t)G.sj, sk = (uint32_t)G.sk;
  const uint32_t c = (uint32_t)cell_at(G, i, j, k);
  const R * __restrict__ Q = B.Q;
  const R * __restrict__ U = B.Uin;
  R dtdx, dtdy, dtdz;
  dt_over_dx(B.st, dtdx, dtdy, dtdz);
  (void)dtdz;

  // edge electric field
  if constexpr (PART == 2)
  {
  }
  else if constexpr (!kExactOrder)
  {
    // E = u B - v A with u, v the means of 4 cells and A, B of 2 faces, as
    // 0.125 (sum u sum B - sum v sum A): scaling by a power of two commutes
    // with rounding, so this is the same value with 3 fewer FP64 operations
    auto s4 = [&](uint32_t d1, uint32_t d2, int v) {
      return Q[c - d1 - d2 + v * sv] + Q[c - d1 + v * sv] + Q[c - d2 + v * sv] + Q[c + v * sv];
    };
    auto s2 = [&](uint32_t d, int v) { return U[c - d + v * sv] + U[c + v * sv]; };
    if constexpr (DIM == 2)
      B.E[c] = R(0.125) * (s4(1u, sj, IU) * s2(1u, IB) - s4(1u, sj, IV) * s2(sj, IA));
    else
    {
      B.E[c] = R(0.125) * (s4(sj, sk, IV) * s2(sj, IC) - s4(sj, sk, IW) * s2(sk, IB));
      B.E[c + sv] = R(0.125) * (s4(1u, sk, IW) * s2(sk, IA) - s4(1u, sk, IU) * s2(1u, IC));
      B.E[c + 2 * sv] = R(0.125) * (s4(1u, sj, IU) * s2(1u, IB) - s4(1u, sj, IV) * s2(sj, IA));
    }
  }
  else if constexpr (DIM == 2)
  {
    const R u = R(0.25) * (Q[c - 1 - sj + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sj + IU * sv] +
                           Q[c + IU * sv]);
    const R v = R(0.25) * (Q[c - 1 - sj + IV * sv] + Q[c - 1 + IV * sv] + Q[c - sj + IV * sv] +
                           Q[c + IV * sv]);
    const R A = R(0.5) * (U[c - sj + IA * sv] + U[c + IA * sv]);
    const R Bf = R(0.5) * (U[c - 1 + IB * sv] + U[c + IB * sv]);
    B.E[c] = u * Bf - v * A;
  }
  else
  {
    R u, v, w, A, Bf, C;
    v = R(0.25) * (Q[c - sj - sk + IV * sv] + Q[c - sj + IV * sv] + Q[c - sk + IV * sv] +
                   Q[c + IV * sv]);
    w = R(0.25) * (Q[c - sj - sk + IW * sv] + Q[c - sj + IW * sv] + Q[c - sk + IW * sv] +
                   Q[c + IW * sv]);
    Bf = R(0.5) * (U[c - sk + IB * sv] + U[c + IB * sv]);
    C = R(0.5) * (U[c - sj + IC * sv] + U[c + IC * sv]);
    B.E[c] = v * C - w * Bf;
    u = R(0.25) * (Q[c - 1 - sk + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sk + IU * sv] +
                   Q[c + IU * sv]);
    w = R(0.25) * (Q[c - 1 - sk + IW * sv] + Q[c - 1 + IW * sv] + Q[c - sk + IW * sv] +
                   Q[c + IW * sv]);
    A = R(0.5) * (U[c - sk + IA * sv] + U[c + IA * sv]);
    C = R(0.5) * (U[c - 1 + IC * sv] + U[c + IC * sv]);
    B.E[c + sv] = w * A - u * C;
    u = R(0.25) * (Q[c - 1 - sj + IU * sv] + Q[c - 1 + IU * sv] + Q[c - sj + IU * sv] +
                   Q[c + IU * sv]);
    v = R(0.25) * (Q[c - 1 - sj + IV * sv] + Q[c - 1 + IV * sv] + Q[c - sj + IV * sv] +
                   Q[c + IV * sv]);
    A = R(0.5) * (U[c - sj + IA * sv] + U[c + IA * sv]);
    Bf = R(0.5) * (U[c - 1 + IB * sv] + U[c + IB * sv]);
    B.E[c + 2 * sv] = u * Bf - v * A;
  }

  if (i > G.isize - g || j > G.jsize - g || (DIM == 3 && k > G.ksize - g))
    return;

  // limited slopes in each direction
  R         q[NV], s[DIM][NV];
  const uint32_t off[3] = { 1u, sj, sk };
#pragma unroll
  for (int v = 0; v < NV; ++v)
    q[v] = Q[c + v * sv];
  if constexpr (PART == 2)
  {
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
      const R * Sd = B.S + (int64_t)d * NV * sv;
#pragma unroll
      for (int v = 0; v < NV; ++v)
        s[d][v] = v == IA + d ? U[c + off[d] + (IA + d) * sv] - U[c + (IA + d) * sv] : Sd[c + v * sv];
    }
  }
  else
  {
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
#pragma unroll
      for (int v = 0; v < NV; ++v)
        s[d][v] = slope_limited(q[v], Q[c + off[d] + v * sv], Q[c - off[d] + v * sv], G.slope_type);
      s[d][IA + d] = U[c + off[d] + (IA + d) * sv] - U[c + (IA + d) * sv];
    }
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
      R * Sd = B.S + (int64_t)d * NV * sv; // the 8 slope planes of direction d
#pragma unroll
      for (int v = 0; v < NV; ++v)
      {
        // the normal-field slope of directions x (and z in 3D, y in 2D) is
        // read by no later stage: the face states take the face field, the
        // edge states the face fields (only the y slope of By is read, by the
        // 3D x edges' double increment)
        if (v == IA + d && (d == 0 || d == DIM - 1))
          continue;
        Sd[c + v * sv] = s[d][v];
      }
    }
    // transverse slopes of the face-centred field for the edge stage
    R * H = B.H;
    H[c + FaceData<DIM>::slope_plane(0, 1) * sv] = face_field_slope<R, DIM>(G, U, c, IA, 1);
    H[c + FaceData<DIM>::slope_plane(1, 0) * sv] = face_field_slope<R, DIM>(G, U, c, IB, 0);
    if constexpr (DIM == 3)
    {
      H[c + FaceData<DIM>::slope_plane(2, 0) * sv] = face_field_slope<R, DIM>(G, U, c, IC, 0);
      H[c + FaceData<DIM>::slope_plane(2, 1) * sv] = face_field_slope<R, DIM>(G, U, c, IC, 1);
    }
    if constexpr (PART == 1)
      return;
  }

  // Hancock half step
  R q2[NV];
  hancock<R, DIM>(q, s, G.gamma0, dtdx, dtdy, dtdz, q2);
  R * Q2 = B.Q2;
#pragma unroll
  for (int v = 0; v < NV; ++v)
    Q2[c + v * sv] = q2[v];
}

// FP32 3D: blocks of 128 threads per SM the register allocation is bounded
// for (80 registers without a bound leave 24 warps per SM for a kernel that
// waits on its loads)
#ifndef MTRACE_MIN_BLOCKS
#  define MTRACE_MIN_BLOCKS 8
#endif
template <class R, int DIM>
__global__ void __launch_bounds__(128, sizeof(R) == 4 && DIM == 3 ? MTRACE_MIN_BLOCKS : 1)
k_trace(const Grid<R> G, Buffers<R> B)
{
  trace_body<R, DIM>(G, B, blockIdx.x * (int64_t)blockDim.x + threadIdx.x);
}

// Cells base <= index < end of BOX_TRACE, one part of trace_body (1: edge
// field and slopes, 2: half step).
template <class R, int DIM, int PART>
__global__ void __launch_bounds__(128)
k_trace_range(const Grid<R> G, Buffers<R> B, int64_t base, int64_t end)
{
  const int64_t idx = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < end)
    trace_body<R, DIM, PART>(G, B, idx);
}

// Half-step predictor of the face-centred field on face c normal to d
// (ComputeSourceFaceMagFunctor2D, MHDRunFunctors2D.h:319-370;
// ComputeSourceFaceMagFunctor3D, MHDRunFunctors3D.h:367-436), evaluated
// on the fly from the stored edge field.
template <class R, int DIM>
__device__ __forceinline__ R
face_source(const Grid<R> & G, const R * __restrict__ E, int64_t c, int d, R dtdx, R dtdy, R dtdz)
{
  const int64_t sj = G.sj, sk = G.sk, n1 = G.sv;
  if constexpr (DIM == 2)
  {
    if (d == 0)
      return (E[c + sj] - E[c]) * R(0.5) * dtdy;
    return -(E[c + 1] - E[c]) * R(0.5) * dtdx;
  }
  else
  {
    const R *Ex = E, *Ey = E + n1, *Ez = E + 2 * n1;
    if (d == 0)
      return (Ez[c + sj] - Ez[c]) * R(0.5) * dtdy - (Ey[c + sk] - Ey[c]) * R(0.5) * dtdz;
    if (d == 1)
      return -(Ez[c + 1] - Ez[c]) * R(0.5) * dtdx + (Ex[c + sk] - Ex[c]) * R(0.5) * dtdz;
    return (Ey[c + 1] - Ey[c]) * R(0.5) * dtdx - (Ex[c + sj] - Ex[c]) * R(0.5) * dtdy;
  }
}

// Half-step normal field of face (c, d): B_d + face_source.  The fast builds
// evaluate it with explicitly rounded operations (no contraction, the exact
// factor 1/2 folded into dt/dx), so that every kernel that evaluates it
// obtains the same bits whatever the surrounding code; the exact build keeps
// the reference's statement.
template <class R, int DIM>
__device__ __forceinline__ R
face_field(const Grid<R> & G, const R * __restrict__ U, const R * __restrict__ E, int64_t c, int d,
           R dtdx, R dtdy, R dtdz)
{
  const R b = U[c + (IA + d) * G.sv];
  if constexpr (kExactOrder)
    return b + face_source<R, DIM>(G, E, c, d, dtdx, dtdy, dtdz);
  else
  {
    const int64_t sj = G.sj, sk = G.sk, n1 = G.sv;
    const R       hx = R(0.5) * dtdx, hy = R(0.5) * dtdy, hz = R(0.5) * dtdz;
    R             s;
    if constexpr (DIM == 2)
    {
      if (d == 0)
        s = rn_mul(rn_sub(E[c + sj], E[c]), hy);
      else
        s = rn_mul(rn_sub(E[c], E[c + 1]), hx);
    }
    else
    {
      const R *Ex = E, *Ey = E + n1, *Ez = E + 2 * n1;
      if (d == 0)
        s = rn_sub(rn_mul(rn_sub(Ez[c + sj], Ez[c]), hy), rn_mul(rn_sub(Ey[c + sk], Ey[c]), hz));
      else if (d == 1)
        s = rn_sub(rn_mul(rn_sub(Ex[c + sk], Ex[c]), hz), rn_mul(rn_sub(Ez[c + 1], Ez[c]), hx));
      else
        s = rn_sub(rn_mul(rn_sub(Ey[c + 1], Ey[c]), hx), rn_mul(rn_sub(Ex[c + sj], Ex[c]), hy));
    }
    return rn_add(b, s);
  }
}

// ---------------------------------------------------------------- face fluxes

// Reconstruction + Riemann solve of ComputeFluxAndUpdateAlongDirFunctor<dir>
// (MHDRunFunctors2D.h:1110-1229, 3D:1097-1253) for faces [g, size-g]^DIM;
// blockIdx.y selects the direction.  The reference adds the flux into cell i
// and subtracts it from cell i-1 with atomics; here it is stored once and
// gathered by k_update.
// Left/right states of the face at the lower side of cell (i,j,k) along d,
// floored and rotated into the face-normal frame (normal velocity -> IU,
// normal field -> IA): MHDRunFunctors2D.h:1110-1190, 3D:1097-1210.
template <class R, int DIM, int d>
__device__ __forceinline__ void
face_states(const Grid<R> & G, const Buffers<R> & B, int64_t c, State<R> & qL, State<R> & qR)
{
  // 32-bit element offsets inside arrays of at most 8 planes
  const uint32_t sv = (uint32_t)G.sv;
  const uint32_t cu = (uint32_t)c;
  const uint32_t cn = cu - (uint32_t)(d == 0 ? 1 : (d == 1 ? G.sj : G.sk));
  const R * __restrict__ Q2 = B.Q2;
  const R * __restrict__ S = B.S + (int64_t)d * NV * sv;
  R dtdx, dtdy, dtdz;
  dt_over_dx(B.st, dtdx, dtdy, dtdz);
  const R smallR = G.smallr, smallp = G.smallp;
  constexpr int nrm = IA + d;
#pragma unroll
  for (int v = 0; v < NV; ++v)
  {
    if (v == nrm)
      continue;
    qR[v] = Q2[cu + v * sv] - R(0.5) * S[cu + v * sv];
    qL[v] = Q2[cn + v * sv] + R(0.5) * S[cn + v * sv];
  }
  qR[ID] = sel_max(smallR, qR[ID]);
  qR[IP] = sel_max(smallp * qR[ID], qR[IP]);
  qL[ID] = sel_max(smallR, qL[ID]);
  qL[IP] = sel_max(smallp * qL[ID], qL[IP]);
  qR[nrm] = face_field<R, DIM>(G, B.Uin, B.E, c, d, dtdx, dtdy, dtdz);
  qL[nrm] = qR[nrm];
  if constexpr (d > 0)
  {
    swap_vals(qL[IU], qL[IU + d]);
    swap_vals(qL[IA], qL[IA + d]);
    swap_vals(qR[IU], qR[IU + d]);
    swap_vals(qR[IA], qR[IA + d]);
  }
}

// Rotate a normal-frame flux back and store the components the update reads.
template <class R, int DIM, int d>
__device__ __forceinline__ void
store_face_flux(const Grid<R> & G, const Buffers<R> & B, int64_t c, State<R> & fl)
{
  if constexpr (d > 0)
  {
    swap_vals(fl[IU], fl[IU + d]);
    swap_vals(fl[IA], fl[IA + d]);
  }
  constexpr int NF = FluxComps<DIM>::NF;
  R * F = B.F + (int64_t)d * NF * G.sv;
#pragma unroll
  for (int q = 0; q < NF; ++q)
    F[c + q * G.sv] = fl[FluxComps<DIM>::var(q)];
}

template <class R, int DIM, int d>
__device__ __forceinline__ void
flux_face(const Grid<R> & G, const Buffers<R> & B, int i, int j, int k)
{
  const int64_t c = cell_at(G, i, j, k);
  State<R>      qR, qL, fl;
  face_states<R, DIM, d>(G, B, c, qL, qR);
  B.H[c + d * G.sv] = qR[IA]; // half-step normal field of the face
#pragma unroll
  for (int v = 0; v < NV; ++v)
    fl[v] = R(0);
  riemann(G.riemann, qL, qR, fl, G.gamma0, G.entho, flux_shift(B.st, R(0)));
  store_face_flux<R, DIM, d>(G, B, c, fl);
}

template <class R, int DIM>
__device__ __forceinline__ void
flux_body(const Grid<R> & G, const Buffers<R> & B, int64_t idx, int dir)
{
  if (step_finished(B.st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], idx, i, j, k))
    return;
  if (dir == 0)
    flux_face<R, DIM, 0>(G, B, i, j, k);
  else if (dir == 1)
    flux_face<R, DIM, 1>(G, B, i, j, k);
  else if constexpr (DIM == 3)
    flux_face<R, DIM, 2>(G, B, i, j, k);
}

template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_flux(const Grid<R> G, Buffers<R> B)
{
  flux_body<R, DIM>(G, B, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, blockIdx.y);
}

// ---------------------------------------------------------------- edge EMFs

// ReconstructEdgeComputeEmfAndUpdateFunctor (MHDRunFunctors2D.h:1291-1534,
// 3D:1331-1778) for edges [g, size-g]^DIM; blockIdx.y is the edge direction
// (0 = x, 1 = y, 2 = z; 2D has z edges only).  The corner states RT, RB,
// LT, LB come from the cells (c - o0 - o1), (c - o0), (c - o1), c where
// o0, o1 are the strides of the two transverse directions d0 < d1
// (reconstruct_state_at_edge, MHDRunFunctors3D.h:1406-1529).
template <class R, int DIM, int edir>
__device__ __forceinline__ void
emf_edge(const Grid<R> & G, const Buffers<R> & B, int i, int j, int k)
{
  constexpr int d0 = edir == 0 ? 1 : 0, d1 = edir == 2 ? 1 : 2;
  // 32-bit element offsets inside arrays of at most 8 planes (grids hold
  // fewer than 4e9 values, checked at context creation)
  const uint32_t sv = (uint32_t)G.sv;
  const uint32_t stride[3] = { 1u, (uint32_t)G.sj, (uint32_t)G.sk };
  const uint32_t o0 = stride[d0], o1 = stride[d1];
  const uint32_t c = (uint32_t)cell_at(G, i, j, k);
  const R * __restrict__ Q2 = B.Q2;
  const R * __restrict__ U = B.Uin;
  const R * __restrict__ S0 = B.S + (int64_t)d0 * NV * sv;
  const R * __restrict__ S1 = B.S + (int64_t)(DIM == 2 ? 1 : d1) * NV * sv;
  R dtdx, dtdy, dtdz;
  dt_over_dx(B.st, dtdx, dtdy, dtdz);
  const R smallR = G.smallr, smallp = G.smallp;

  // Corner cells and face data of the four corners (RT, RB, LT, LB)
  constexpr int dd1 = DIM == 2 ? 1 : d1;
  constexpr int p0 = FaceData<DIM>::slope_plane(d0, dd1);
  constexpr int p1 = FaceData<DIM>::slope_plane(dd1, d0);
  const int     id0 = d0 == 0 ? i : j;
  const int     id1 = dd1 == 1 ? j : k;
  uint32_t      cc[4];
  R             fb0[4], fb1[4]; // B_{d0} + slope term, B_{d1} + slope term
#pragma unroll
  for (int e = 0; e < 4; ++e)
  {
    const bool     r0 = (e == 0 || e == 1), r1 = (e == 0 || e == 2);
    const R        sb0 = (e == 0 || e == 2) ? R(1) : R(-1);
    const R        sb1 = (e == 0 || e == 1) ? R(1) : R(-1);
    cc[e] = c - (r0 ? o0 : 0u) - (r1 ? o1 : 0u);
    const uint32_t c0 = cc[e] + (r0 ? o0 : 0u); // face carrying B_{d0}
    const uint32_t c1 = cc[e] + (r1 ? o1 : 0u); // face carrying B_{d1}
    // half-step face fields: stored by the flux stage on the face box; the
    // layer below it (index g-1 along the other transverse direction) is
    // evaluated here with the same expression
    const R B0 = (r1 && id1 == G.g) ? face_field<R, DIM>(G, U, B.E, c0, d0, dtdx, dtdy, dtdz)
                                    : B.H[c0 + d0 * sv];
    const R B1 = (r0 && id0 == G.g) ? face_field<R, DIM>(G, U, B.E, c1, dd1, dtdx, dtdy, dtdz)
                                    : B.H[c1 + dd1 * sv];
    // transverse face-field slopes from the trace stage (zero along z)
    const R dB0d1 = p0 < 0 ? R(0) : B.H[c0 + p0 * sv];
    const R dB1d0 = p1 < 0 ? R(0) : B.H[c1 + p1 * sv];
    fb0[e] = B0 + R(0.5) * (sb0 * dB0d1);
    fb1[e] = B1 + R(0.5) * (sb1 * dB1d0);
  }
  // Corner states, one variable at a time for the four corners (one plane
  // base per variable): q = Q2 + (+-S0 +- S1)/2, the face-normal fields from
  // the face data, in the statement order of reconstruct_state_at_edge
  State<R> qe[4];
  auto hydro = [&](int v, bool twice = false) {
    const R * __restrict__ q2 = Q2 + v * sv;
    const R * __restrict__ s0 = S0 + v * sv;
    const R * __restrict__ s1 = S1 + v * sv;
#pragma unroll
    for (int e = 0; e < 4; ++e)
    {
      const bool r0 = (e == 0 || e == 1), r1 = (e == 0 || e == 2);
      const R    sdq0 = r0 ? R(1) : R(-1), sdq1 = r1 ? R(1) : R(-1);
      const R    inc = R(0.5) * (sdq0 * s0[cc[e]] + sdq1 * s1[cc[e]]);
      qe[e][v] = q2[cc[e]] + inc;
      if (twice)
        qe[e][v] += inc;
    }
  };
  hydro(ID);
  hydro(IU);
  hydro(IV);
  hydro(IW);
  hydro(IP);
  if constexpr (DIM == 2)
  {
    // MHDRunFunctors2D.h:1424-1432
#pragma unroll
    for (int e = 0; e < 4; ++e)
    {
      qe[e][IA] = fb0[e];
      qe[e][IB] = fb1[e];
    }
    hydro(IC);
  }
  else
  {
    // statement order of MHDRunFunctors3D.h:1490-1524, including the double
    // transverse increment of IB on y and x edges
    if constexpr (d0 == 0)
    {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        qe[e][IA] = fb0[e];
    }
    else
      hydro(IA);
    if constexpr (d0 == 1)
    {
      if constexpr (d1 == 1)
      {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          qe[e][IB] = fb1[e];
      }
      else
      {
        // q[IB] = B0 term, then += the IB slope increment
#pragma unroll
        for (int e = 0; e < 4; ++e)
        {
          const bool r0 = (e == 0 || e == 1), r1 = (e == 0 || e == 2);
          const R    sdq0 = r0 ? R(1) : R(-1), sdq1 = r1 ? R(1) : R(-1);
          qe[e][IB] = fb0[e] + R(0.5) * (sdq0 * S0[cc[e] + IB * sv] + sdq1 * S1[cc[e] + IB * sv]);
        }
      }
    }
    else
    {
      if constexpr (d1 == 1)
      {
#pragma unroll
        for (int e = 0; e < 4; ++e)
          qe[e][IB] = fb1[e];
      }
      else
        hydro(IB, true); // Q2 + inc, then += inc again
    }
    if constexpr (d1 == 2)
    {
#pragma unroll
      for (int e = 0; e < 4; ++e)
        qe[e][IC] = fb1[e];
    }
    else
      hydro(IC);
  }
#pragma unroll
  for (int e = 0; e < 4; ++e)
  {
    qe[e][ID] = sel_max(smallR, qe[e][ID]);
    qe[e][IP] = sel_max(smallp * qe[e][ID], qe[e][IP]);
  }
  if constexpr (DIM == 3 && edir == 1)
  {
    // y edges: RB and LT are exchanged before the solve (MHDRunFunctors3D.h:1688-1698)
#pragma unroll
    for (int v = 0; v < NV; ++v)
      swap_vals(qe[1][v], qe[2][v]);
  }
  B.Em[c + (DIM == 2 ? 0u : (uint32_t)edir * sv)] = compute_emf(edir, qe, G.gamma0, G.smallc);
}

template <class R, int DIM>
__device__ __forceinline__ void
emf_body(const Grid<R> & G, const Buffers<R> & B, int64_t idx, int dir)
{
  if (step_finished(B.st))
    return;
  int i, j, k;
  if (!box_cell(G.box[BOX_FACE], idx, i, j, k))
    return;
  if constexpr (DIM == 2)
    emf_edge<R, 2, 2>(G, B, i, j, k);
  else if (dir == 0)
    emf_edge<R, 3, 0>(G, B, i, j, k);
  else if (dir == 1)
    emf_edge<R, 3, 1>(G, B, i, j, k);
  else
    emf_edge<R, 3, 2>(G, B, i, j, k);
}

// Edges base <= index < end of BOX_FACE (a whole launch: 0 and the box's
// count; slab launches of the host-buffer step cover a range of planes)
template <class R, int DIM>
__global__ void __launch_bounds__(128)
k_emf(const Grid<R> G, Buffers<R> B, int64_t base, int64_t end)
{
  const int64_t idx = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < end)
    emf_body<R, DIM>(G, B, idx, blockIdx.y);
}

// ---------------------------------------------------------------- update

// U_out from U_in for interior cells, replaying the reference's atomic
// updates in the order a serial run applies them: per direction x, y(, z)
// "+ F(face i) dt/dx, - F(face i+1) dt/dx" for the hydro variables
// (MHDRunFunctors2D.h:1231-1273, 3D:1255-1313), then the CT update of the
// face-centred field (MHDRunFunctors2D.h:1519-1523, 3D:1638-1766):
//   2D  Bx: - Ez(j) dt/dy + Ez(j+1) dt/dy;   By: + Ez(i) dt/dx - Ez(i+1) dt/dx
//   3D  Bx: + Ey(k) dt/dz - Ey(k+1) dt/dz - Ez(j) dt/dy + Ez(j+1) dt/dy
//       By: - Ex(k) dt/dz + Ex(k+1) dt/dz + Ez(i) dt/dx - Ez(i+1) dt/dx
//       Bz: + Ex(j) dt/dy - Ex(j+1) dt/dy - Ey(i) dt/dx + Ey(i+1) dt/dx
//
// FP32 takes another operation order, with the same values in exact
// arithmetic: the flux (EMF) differences of each direction are summed into
// one increment d before it meets the state, so the rounding of the update
// is relative to d rather than to the O(1) fluxes; and the state is kept as
// a float pair (U_in, Ulo) whose sum carries about 48 bits: the increment
// is added with an error-free two-sum and the pair renormalised, so the
// state's own rounding no longer accumulates over the iterations.  Without
// an Ulo array (the no-allocation path) U_out = U_in + d.
//
// compensated_sum: h + d into the pair (hn, ln) given the low part l.
__device__ __forceinline__ void
compensated_sum(float h, float d, float l, float & hn, float & ln)
{
  // two-sum h + d = s + e exactly (Knuth), then the low parts
  const float s = __fadd_rn(h, d);
  const float bb = __fsub_rn(s, h);
  const float e = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(d, bb));
  const float t = __fadd_rn(e, l);
  // fast two-sum renormalisation (|s| >= |t|)
  hn = __fadd_rn(s, t);
  ln = __fsub_rn(t, __fsub_rn(hn, s));
}

// Every load of the cell (fluxes, EMFs, state, low parts) is issued before
// its first store, through restrict-qualified pointers, so that the loads
// overlap instead of waiting for each variable's stores.
template <int DIM>
__device__ __forceinline__ void
update_fp32(const Grid<float> & G, const Buffers<float> & B, int64_t c)
{
  const int64_t sv = G.sv, sj = G.sj, sk = G.sk;
  float         dtd[3];
  dt_over_dx(B.st, dtd[0], dtd[1], dtd[2]);
  const int64_t off[3] = { 1, sj, sk };
  constexpr int NF = FluxComps<DIM>::NF;
  constexpr int NB = DIM == 2 ? 2 : 3; // face-field components the EMFs update
  constexpr int NU = NF + NB;          // = NV
  const float * __restrict__ F = B.F;
  const float * __restrict__ Em = B.Em;
  const float * __restrict__ Uin = B.Uin;
  float * __restrict__       Uout = B.Uout;
  float * __restrict__       lo = B.Ulo;
  int   var[NU];
  float d[NU];
#pragma unroll
  for (int q = 0; q < NF; ++q)
  {
    var[q] = FluxComps<DIM>::var(q);
    float x = 0.f;
#pragma unroll
    for (int dd = 0; dd < DIM; ++dd)
    {
      const float * Fq = F + ((int64_t)dd * NF + q) * sv;
      x = x + (Fq[c] - Fq[c + off[dd]]) * dtd[dd];
    }
    d[q] = x;
  }
  if constexpr (DIM == 2)
  {
    var[NF] = IA;
    var[NF + 1] = IB;
    d[NF] = (Em[c + sj] - Em[c]) * dtd[1];
    d[NF + 1] = (Em[c] - Em[c + 1]) * dtd[0];
  }
  else
  {
    const float *eX = Em, *eY = Em + sv, *eZ = Em + 2 * sv;
    var[NF] = IA;
    var[NF + 1] = IB;
    var[NF + 2] = IC;
    d[NF] = (eY[c] - eY[c + sk]) * dtd[2] + (eZ[c + sj] - eZ[c]) * dtd[1];
    d[NF + 1] = (eX[c + sk] - eX[c]) * dtd[2] + (eZ[c] - eZ[c + 1]) * dtd[0];
    d[NF + 2] = (eX[c] - eX[c + sj]) * dtd[1] + (eY[c + 1] - eY[c]) * dtd[0];
  }
  float h[NU], l[NU];
#pragma unroll
  for (int k = 0; k < NU; ++k)
  {
    h[k] = Uin[c + var[k] * sv];
    l[k] = lo ? lo[c + var[k] * sv] : 0.f;
  }
#pragma unroll
  for (int k = 0; k < NU; ++k)
  {
    const int64_t cv = c + var[k] * sv;
    if (!lo)
    {
      Uout[cv] = __fadd_rn(h[k], d[k]);
      continue;
    }
    float hn, ln;
    compensated_sum(h[k], d[k], l[k], hn, ln);
    Uout[cv] = hn;
    lo[cv] = ln;
  }
}

template <class R, int DIM>
__device__ __forceinline__ void
update_body(const Grid<R> & G, const Buffers<R> & B, int64_t idx)
{
  if (step_finished(B.st))
    return;
  const Box & b = G.box[BOX_INTERIOR];
  int       i, j, k;
  if (!box_cell(b, idx, i, j, k))
    return;
  const int64_t sv = G.sv, sj = G.sj, sk = G.sk;
  const int64_t c = cell_at(G, i, j, k);
  if constexpr (sizeof(R) == 4)
  {
    update_fp32<DIM>(G, B, c);
    return;
  }
  R             dtd[3];
  dt_over_dx(B.st, dtd[0], dtd[1], dtd[2]);
  const int64_t off[3] = { 1, sj, sk };
  constexpr int NF = FluxComps<DIM>::NF;
  // restrict-qualified: the stores of one variable do not hold back the
  // loads of the next
  const R * __restrict__ Uin = B.Uin;
  const R * __restrict__ Fl = B.F;
  R * __restrict__       Uout = B.Uout;
#pragma unroll
  for (int q = 0; q < NF; ++q)
  {
    const int v = FluxComps<DIM>::var(q);
    R         x = Uin[c + v * sv];
#pragma unroll
    for (int d = 0; d < DIM; ++d)
    {
      const R * F = Fl + ((int64_t)d * NF + q) * sv;
      x += F[c] * dtd[d];
      x -= F[c + off[d]] * dtd[d];
    }
    Uout[c + v * sv] = x;
  }
  const R * __restrict__ Em = B.Em;
  if constexpr (DIM == 2)
  {
    R x = Uin[c + IA * sv];
    x -= Em[c] * dtd[1];
    x += Em[c + sj] * dtd[1];
    Uout[c + IA * sv] = x;
    x = Uin[c + IB * sv];
    x += Em[c] * dtd[0];
    x -= Em[c + 1] * dtd[0];
    Uout[c + IB * sv] = x;
    if constexpr (NF == 6)
    {
    }
  }
  else
  {
    const R *eX = Em, *eY = Em + sv, *eZ = Em + 2 * sv;
    R        x = Uin[c + IA * sv];
    x += eY[c] * dtd[2];
    x -= eY[c + sk] * dtd[2];
    x -= eZ[c] * dtd[1];
    x += eZ[c + sj] * dtd[1];
    Uout[c + IA * sv] = x;
    x = Uin[c + IB * sv];
    x -= eX[c] * dtd[2];
    x += eX[c + sk] * dtd[2];
    x += eZ[c] * dtd[0];
    x -= eZ[c + 1] * dtd[0];
    Uout[c + IB * sv] = x;
    x = Uin[c + IC * sv];
    x += eX[c] * dtd[1];
    x -= eX[c + sj] * dtd[1];
    x -= eY[c] * dtd[0];
    x += eY[c + 1] * dtd[0];
    Uout[c + IC * sv] = x;
  }
}

// interior cells base <= index < end of BOX_INTERIOR
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_update(const Grid<R> G, Buffers<R> B, int64_t base, int64_t end)
{
  const int64_t idx = base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx < end)
    update_body<R, DIM>(G, B, idx);
}

// Grid description of one problem for the kernels (host side):
// HydroParams::init (HydroParams.cpp:420-453) in the working precision R,
// plus the iteration boxes and their divisors.
template <class R>
inline Grid<R>
make_grid(const mhd_params & p)
{
  Grid<R> G{};
  G.dim = p.dim;
  G.nx = p.nx;
  G.ny = p.ny;
  G.nz = p.dim == 3 ? p.nz : 1;
  G.g = p.ghost;
  G.isize = p.nx + 2 * p.ghost;
  G.jsize = p.ny + 2 * p.ghost;
  G.ksize = p.dim == 3 ? p.nz + 2 * p.ghost : 1;
  G.sj = G.isize;
  G.sk = (int64_t)G.isize * G.jsize;
  G.sv = G.sk * G.ksize;
  for (int f = 0; f < 6; ++f)
    G.bc[f] = p.boundary[f];
  G.riemann = p.riemann;
  G.gamma0 = R(p.gamma0);
  G.entho = R(1) / (G.gamma0 - R(1));
  G.smallr = R(p.smallr);
  G.smallc = R(p.smallc);
  // smallp = smallc^2 / gamma0 in real_t (HydroParams.cpp:438)
  G.smallp = R(R(p.smallc) * R(p.smallc) / R(p.gamma0));
  G.slope_type = R(p.slope_type);
  G.cfl = p.cfl;
  // dx = (xmax - xmin) / nx in real_t (HydroParams.cpp:433-435)
  G.dx = (double)R(R(p.xmax - p.xmin) / R(p.nx));
  G.dy = (double)R(R(p.ymax - p.ymin) / R(p.ny));
  G.dz = p.dim == 3 ? (double)R(R(p.zmax - p.zmin) / R(p.nz)) : 1.0;
  G.idx = 1.0 / G.dx;
  G.idy = 1.0 / G.dy;
  G.idz = 1.0 / G.dz;
  const bool d3 = p.dim == 3;
  const int  g = G.g;
  G.box[BOX_ALL] = Box(0, 0, 0, G.isize, G.jsize, d3 ? G.ksize : 1);
  G.box[BOX_PRIM] = Box(0, 0, 0, G.isize - 1, G.jsize - 1, d3 ? G.ksize - 1 : 1);
  G.box[BOX_TRACE] = Box(g - 1, g - 1, d3 ? g - 1 : 0, G.nx + 3, G.ny + 3, d3 ? G.nz + 3 : 1);
  G.box[BOX_FACE] = Box(g, g, d3 ? g : 0, G.nx + 1, G.ny + 1, d3 ? G.nz + 1 : 1);
  G.box[BOX_INTERIOR] = Box(g, g, d3 ? g : 0, G.nx, G.ny, d3 ? G.nz : 1);
  return G;
}

} // namespace MHD_VARIANT_TAG
} // namespace mhd
