// The 2D plain form fused into one tile kernel (implementation version 2):
// after the ghost fill and the CFL reduction, one launch computes a whole
// iteration of a TX x TY tile of interior cells with every intermediate in
// shared memory:
//
//   1. primitives and the face-centred field of the tile and 2 halo layers
//      (ConvertToPrimitivesFunctor, MHDRunFunctors2D.h:85-159);
//   2. the edge electric field (ComputeElecFieldFunctor, :253-314) of the
//      tile's lower-left corners and 2 more layers, and the limited slopes
//      and half-step primitives (ComputeSlopesFunctor, :164-248;
//      ComputeUpdatedPrimVarFunctor, :920-1051) of the tile and 1 halo layer;
//   3. the HLLD fluxes of every face of the tile's cells
//      (ComputeFluxAndUpdateAlongDirFunctor, :1110-1229) and the 2D HLLD EMF
//      of every corner (ReconstructEdgeComputeEmfAndUpdateFunctor,
//      :1291-1534), the half-step face fields (ComputeSourceFaceMagFunctor2D,
//      :319-370) and the transverse face-field slopes taken from phase 2;
//   4. the update of the tile's cells from the fluxes and EMFs (the
//      reference's atomic adds in their serial order, MHDRunFunctors2D.h:
//      1231-1273 and 1519-1523), written to U_out.
//
// Every value is computed by the same device functions, from the same
// operands, as in the stage kernels (k_prim_dt, k_trace, k_flux, k_emf,
// k_update), so the FMA-free build gives U_out bit for bit theirs; the halo
// is recomputed by neighbouring tiles instead of being written to and read
// back from HBM (the stage form moves about 6.8 GB per 4096^2 FP32
// iteration through Q, Q2, S, H, E, F and Em, the fused form reads the state
// once and writes it once).
#pragma once

#include "mhd_kernels.cuh"

// FP32 tiles are 32 x MFUSED_TILE_ROWS cells with one thread per cell;
// MFUSED_MIN_BLOCKS blocks of 32 x 8 per SM (the register bound the compiler
// keeps to: 64 per thread), fewer of the taller tiles for the same warps.
// 32 x 16 tiles of 512 threads recompute less halo but measured 3.6 %
// slower on GB300 (Kelvin-Helmholtz 4096^2: 1.776 against 1.714 ms).
#ifndef MFUSED_MIN_BLOCKS
#  define MFUSED_MIN_BLOCKS 4
#endif
#ifndef MFUSED_TILE_ROWS
#  define MFUSED_TILE_ROWS 8
#endif
// 1: the tile's state rows reach shared memory by bulk copies (the TMA
// engine, cp.async.bulk: one per variable and row, issued by a warp and
// completed on an mbarrier) before the primitives are computed; 0 (the
// default): each thread loads its cells' values itself.  Both give the same
// state bit for bit; the bulk copies measured 20 % slower on GB300
// (Kelvin-Helmholtz 4096^2 FP32: 2.05 against 1.72 ms), the block waiting
// for its whole tile where the loads of the plain form overlap with the
// other warps' arithmetic.
#ifndef MFUSED_BULK_STAGING
#  define MFUSED_BULK_STAGING 0
#endif

namespace mhd
{
inline namespace MHD_VARIANT_TAG
{

template <class R, int TY_>
struct MTile
{
  static constexpr int TX = 32, TY = TY_;
  static constexpr int THREADS = TX * TY; // one thread per tile cell
  // blocks per SM the FP32 kernels are compiled for (the same 32 warps)
  static constexpr int MIN_BLOCKS = sizeof(R) == 4 ? MFUSED_MIN_BLOCKS * 8 / TY : 1;
  // primitives and face fields: tile + 2 halo layers
  static constexpr int MX = TX + 4, MY = TY + 4, NM = MX * MY;
  // slopes and half-step primitives: tile + 1 halo layer
  static constexpr int SX = TX + 2, SY = TY + 2, NT = SX * SY;
  // edge field at the lower-left corner of cells [i0-1, i0+TX+2) x ..
  static constexpr int EX = TX + 3, EY = TY + 3, NE = EX * EY;
  // x faces, y faces and corners of the tile's cells
  static constexpr int NFX = (TX + 1) * TY, NFY = TX * (TY + 1), NEM = (TX + 1) * (TY + 1);
  static constexpr int NF = FluxComps<2>::NF;
  static constexpr int NFLUX = NF * (NFX + NFY) + NEM;
  // region A holds the primitives until the fluxes replace them
  static constexpr int NA = NV * NM > NFLUX ? NV * NM : NFLUX;
  static constexpr int NREAL = NA + 2 * NM + 3 * NV * NT + NE;
  static constexpr size_t SMEM = sizeof(R) * (size_t)NREAL;
};

// ---- bulk copies into shared memory (cp.async.bulk, completed on an mbarrier)

__device__ __forceinline__ uint32_t
smem_u32(const void * p)
{
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void
stage_bar_init(uint32_t bar)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void
stage_expect(uint32_t bar, uint32_t bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

// bytes (a multiple of 16) from a 16-byte aligned global address to a
// 16-byte aligned shared address
__device__ __forceinline__ void
stage_copy(uint32_t dst, const void * src, uint32_t bytes, uint32_t bar)
{
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, "
               "[%3];" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}

// at most `limit` polls of the phase-0 completion; false when it ran out
__device__ __forceinline__ bool
stage_wait(uint32_t bar, int limit)
{
  uint32_t done = 0;
  for (int it = 0; it < limit && !done; ++it)
    asm volatile("{\n\t.reg .pred q;\n\tmbarrier.try_wait.parity.shared::cta.b64 q, [%1], 0;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}\n"
                 : "=r"(done)
                 : "r"(bar)
                 : "memory");
  return done != 0;
}

constexpr int kStageWaitPolls = 1 << 22;

// half-step normal field of an x face (B_x + (E(j+1) - E(j)) dt/(2 dy)) and
// of a y face (B_y - (E(i+1) - E(i)) dt/(2 dx)) from the values; the same
// expressions as face_field
template <class R>
__device__ __forceinline__ R
face_field_x2(R b, R e_lo, R e_hi, R dtdy)
{
  if constexpr (kExactOrder)
    return b + (e_hi - e_lo) * R(0.5) * dtdy;
  else
    return rn_add(b, rn_mul(rn_sub(e_hi, e_lo), R(0.5) * dtdy));
}
template <class R>
__device__ __forceinline__ R
face_field_y2(R b, R e_lo, R e_hi, R dtdx)
{
  if constexpr (kExactOrder)
    return b + -(e_hi - e_lo) * R(0.5) * dtdx;
  else
    return rn_add(b, rn_mul(rn_sub(e_lo, e_hi), R(0.5) * dtdx));
}

// One iteration of tile (tx, ty) of a problem (the block's whole work; smem:
// MTile::SMEM bytes of dynamic shared memory).  RS: the Riemann solver fixed
// at compile time (RIEMANN_HLLD, the common case: the other solvers' code is
// left out of the kernel), or 0 for the run-time choice of G.riemann.
template <class R, int TY, int RS>
__device__ __forceinline__ void
mfused2d_tile(const Grid<R> & G, const R * __restrict__ Uin, R * __restrict__ Uout,
              R * __restrict__ Ulo, DevState * __restrict__ st, int tx, int ty,
              unsigned char * msm_raw)
{
  using T = MTile<R, TY>;
  if (step_finished(st))
    return;
  R * As = reinterpret_cast<R *>(msm_raw); // primitives [NV][NM], later the fluxes
  R * Ua = As + T::NA;                      // face field B_x [NM]
  R * Ub = Ua + T::NM;                      // face field B_y [NM]
  R * Q2s = Ub + T::NM;                     // half-step primitives [NV][NT]
  R * S0s = Q2s + NV * T::NT;               // slopes along x [NV][NT]
  R * S1s = S0s + NV * T::NT;               // slopes along y [NV][NT]
  R * Es = S1s + NV * T::NT;                // edge field [NE]
  const int g = G.g;
  const int i0 = g + tx * T::TX, j0 = g + ty * T::TY;
  const int tid = threadIdx.x;
  const int64_t sv = G.sv, sj = G.sj;
  R dtdx, dtdy, dtdz;
  dt_over_dx(st, dtdx, dtdy, dtdz);

  // 1. primitives and face fields of cells [i0-2, i0+TX+2) x [j0-2, j0+TY+2);
  // cells whose +1 neighbour lies beyond the array (only in a partial last
  // tile, and read by nothing the tile's interior cells need) get a neutral
  // state.
#if MFUSED_BULK_STAGING
  // The state rows arrive first by bulk copies: per variable, rows j0-2 ..
  // j0+TY+1 (and row j0+TY+2 of B_y, the +1 neighbours' face field), each a
  // run of SW values from the 16-byte boundary at or before column i0-2, so
  // that it holds columns i0-2 .. i0+TX+2; rows beyond the array are not
  // copied.  They land in the half-step region, unused until phase 2.  A
  // copy may run past the last row of the last variable: the arrays carry
  // 256 bytes of padding.
  constexpr int VPC = 16 / (int)sizeof(R);                     // values per 16 bytes
  constexpr int SW = (T::MX + 1 + VPC - 1 + VPC - 1) / VPC * VPC; // staged row width
  constexpr int SR = T::MY + 1;                                // staged rows per variable
  __shared__ alignas(8) unsigned long long stg_bar;
  R * stg = reinterpret_cast<R *>((reinterpret_cast<uintptr_t>(Q2s) + 15) & ~uintptr_t(15));
  static_assert(NV * SR * SW + VPC <= 3 * NV * T::NT, "staging fits the half-step region");
  const int jlo = j0 - 2;
  const int nrows = min(SR, G.jsize - jlo); // rows that exist in the array
  auto      row_src = [&](int v, int b) { return Uin + (int64_t)(jlo + b) * sj + (i0 - 2) + v * sv; };
  if (tid < 32)
  {
    // warp 0: lane 0 sets up the barrier, then the lanes issue the copies
    const int nmain = min(nrows, T::MY);
    const int ncopy = NV * nmain + (nrows > T::MY ? 1 : 0);
    if (tid == 0)
    {
      stage_bar_init(smem_u32(&stg_bar));
      stage_expect(smem_u32(&stg_bar), (uint32_t)ncopy * (uint32_t)(SW * sizeof(R)));
    }
    __syncwarp();
    for (int k = tid; k < ncopy; k += 32)
    {
      const int       v = k < NV * nmain ? k / nmain : IB;
      const int       b = k < NV * nmain ? k - v * nmain : T::MY;
      const uintptr_t src = reinterpret_cast<uintptr_t>(row_src(v, b));
      stage_copy(smem_u32(stg + (v * SR + b) * SW),
                 reinterpret_cast<const void *>(src & ~uintptr_t(15)), (uint32_t)(SW * sizeof(R)),
                 smem_u32(&stg_bar));
    }
  }
  __syncthreads();
  if (!__syncthreads_and(stage_wait(smem_u32(&stg_bar), kStageWaitPolls)))
  {
    // the copies did not complete within the bound: report it, give them a
    // second bound to land, and leave the tile
    if (tid == 0)
      atomicOr(&st->status, STATUS_STAGING);
    stage_wait(smem_u32(&stg_bar), kStageWaitPolls);
    return;
  }
  // the first staged value of row b of variable v
  auto staged = [&](int v, int b) {
    const uintptr_t src = reinterpret_cast<uintptr_t>(row_src(v, b));
    return stg + (v * SR + b) * SW + (int)((src & 15u) / sizeof(R));
  };
#endif
  for (int m = tid; m < T::NM; m += T::THREADS)
  {
    const int i = i0 - 2 + m % T::MX, j = j0 - 2 + m / T::MX;
    R         q[NV], fa = R(0), fb = R(0);
    if (i < G.isize - 1 && j < G.jsize - 1)
    {
#if MFUSED_BULK_STAGING
      const int a = m % T::MX, b = m / T::MX;
      R         u[NV];
#  pragma unroll
      for (int v = 0; v < NV; ++v)
        u[v] = staged(v, b)[a];
      const CellPrim<R> P =
        cell_prim_v<R, 2>(G, u, staged(IA, b)[a + 1], staged(IB, b + 1)[a], R(0));
      fa = u[IA];
      fb = u[IB];
#else
      const int64_t     c = cell_at(G, i, j, 0);
      const CellPrim<R> P = cell_prim<R, 2>(G, Uin, c);
      fa = Uin[c + IA * sv];
      fb = Uin[c + IB * sv];
#endif
      q[ID] = P.d; q[IP] = P.p; q[IU] = P.vu; q[IV] = P.vv; q[IW] = P.vw;
      q[IA] = P.a; q[IB] = P.bb; q[IC] = P.cc;
    }
    else
    {
#pragma unroll
      for (int v = 0; v < NV; ++v)
        q[v] = (v == ID || v == IP) ? R(1) : R(0);
    }
#pragma unroll
    for (int v = 0; v < NV; ++v)
      As[v * T::NM + m] = q[v];
    Ua[m] = fa;
    Ub[m] = fb;
  }
  __syncthreads();

  // 2. edge field, and slopes + half step (two item grids)
  {
    using IE = ItemGrid<T::EX, T::EY>;
    using IT = ItemGrid<T::SX, T::SY>;
    const R * Qs = As;
    for (int w = tid; w < IE::COUNT + IT::COUNT; w += T::THREADS)
    {
      int a, b;
      if (w < IE::COUNT)
      {
        if (IE::at(w, a, b))
        {
          // E of cell (i0-1+a, j0-1+b): primitives box cell (a+1, b+1)
          const int m = (a + 1) + T::MX * (b + 1);
          const int m1 = m - 1, mj = m - T::MX, m1j = m - 1 - T::MX;
          R         e;
          if constexpr (!kExactOrder)
          {
            const R su = Qs[IU * T::NM + m1j] + Qs[IU * T::NM + m1] + Qs[IU * T::NM + mj] +
                         Qs[IU * T::NM + m];
            const R svv = Qs[IV * T::NM + m1j] + Qs[IV * T::NM + m1] + Qs[IV * T::NM + mj] +
                          Qs[IV * T::NM + m];
            e = R(0.125) * (su * (Ub[m1] + Ub[m]) - svv * (Ua[mj] + Ua[m]));
          }
          else
          {
            const R u = R(0.25) * (Qs[IU * T::NM + m1j] + Qs[IU * T::NM + m1] +
                                   Qs[IU * T::NM + mj] + Qs[IU * T::NM + m]);
            const R v = R(0.25) * (Qs[IV * T::NM + m1j] + Qs[IV * T::NM + m1] +
                                   Qs[IV * T::NM + mj] + Qs[IV * T::NM + m]);
            const R A = R(0.5) * (Ua[mj] + Ua[m]);
            const R Bf = R(0.5) * (Ub[m1] + Ub[m]);
            e = u * Bf - v * A;
          }
          Es[a + T::EX * b] = e;
        }
      }
      else if (IT::at(w - IE::COUNT, a, b))
      {
        // slopes and half step of cell (i0-1+a, j0-1+b)
        const int t = a + T::SX * b;
        const int m = (a + 1) + T::MX * (b + 1);
        R         q[NV], s[2][NV], q2[NV];
#pragma unroll
        for (int v = 0; v < NV; ++v)
          q[v] = Qs[v * T::NM + m];
        constexpr int mo[2] = { 1, T::MX };
#pragma unroll
        for (int d = 0; d < 2; ++d)
        {
#pragma unroll
          for (int v = 0; v < NV; ++v)
            s[d][v] = slope_limited(q[v], Qs[v * T::NM + m + mo[d]], Qs[v * T::NM + m - mo[d]],
                                    G.slope_type);
        }
        s[0][IA] = Ua[m + 1] - Ua[m];
        s[1][IB] = Ub[m + T::MX] - Ub[m];
        hancock<R, 2>(q, s, G.gamma0, dtdx, dtdy, dtdz, q2);
#pragma unroll
        for (int v = 0; v < NV; ++v)
        {
          Q2s[v * T::NT + t] = q2[v];
          S0s[v * T::NT + t] = s[0][v];
          S1s[v * T::NT + t] = s[1][v];
        }
      }
    }
  }
  __syncthreads();

  // 3. face fluxes (x faces, y faces) and corner EMFs into region A
  R * Fx = As;                      // [NF][NFX], x faces (i0+fa, j0+fb), pitch TX+1
  R * Fy = Fx + T::NF * T::NFX;     // [NF][NFY], y faces, pitch TX
  R * Ems = Fy + T::NF * T::NFY;    // [NEM], corners, pitch TX+1
  {
    using IX = ItemGrid<T::TX + 1, T::TY>;
    using IY = ItemGrid<T::TX, T::TY + 1>;
    using IK = ItemGrid<T::TX + 1, T::TY + 1>; // corners
    const R smallR = G.smallr, smallp = G.smallp;
    const R shift = flux_shift(st, R(0));
    for (int w = tid; w < IX::COUNT + IY::COUNT + IK::COUNT; w += T::THREADS)
    {
      if (w < IX::COUNT + IY::COUNT)
      {
        const bool xdir = w < IX::COUNT;
        int        fa, fb;
        if (xdir ? IX::at(w, fa, fb) : IY::at(w - IX::COUNT, fa, fb))
        {
          const int f = xdir ? fa + (T::TX + 1) * fb : fa + T::TX * fb;
          // the face's right (upper) cell and its left (lower) neighbour in
          // the slopes box; its face field and edge fields
          const int tr = (fa + 1) + T::SX * (fb + 1);
          const int tl = tr - (xdir ? 1 : T::SX);
          const int m = (fa + 2) + T::MX * (fb + 2);
          const int e0 = (fa + 1) + T::EX * (fb + 1);
          const R * Sd = xdir ? S0s : S1s;
          State<R>  qL, qR, fl;
          // (the normal field, IA for x faces and IB for y faces, is the face
          // field below; indices stay compile-time constants)
#pragma unroll
          for (int v = 0; v < NV; ++v)
          {
            if (xdir ? v == IA : v == IB)
              continue;
            qR[v] = Q2s[v * T::NT + tr] - R(0.5) * Sd[v * T::NT + tr];
            qL[v] = Q2s[v * T::NT + tl] + R(0.5) * Sd[v * T::NT + tl];
          }
          qR[ID] = sel_max(smallR, qR[ID]);
          qR[IP] = sel_max(smallp * qR[ID], qR[IP]);
          qL[ID] = sel_max(smallR, qL[ID]);
          qL[IP] = sel_max(smallp * qL[ID], qL[IP]);
          if (xdir)
          {
            qR[IA] = face_field_x2(Ua[m], Es[e0], Es[e0 + T::EX], dtdy);
            qL[IA] = qR[IA];
          }
          else
          {
            qR[IB] = face_field_y2(Ub[m], Es[e0], Es[e0 + 1], dtdx);
            qL[IB] = qR[IB];
          }
          if (!xdir)
          {
            swap_vals(qL[IU], qL[IV]);
            swap_vals(qL[IA], qL[IB]);
            swap_vals(qR[IU], qR[IV]);
            swap_vals(qR[IA], qR[IB]);
          }
#pragma unroll
          for (int v = 0; v < NV; ++v)
            fl[v] = R(0);
          riemann(RS ? RS : G.riemann, qL, qR, fl, G.gamma0, G.entho, shift);
          if (!xdir)
          {
            swap_vals(fl[IU], fl[IV]);
            swap_vals(fl[IA], fl[IB]);
          }
          R * Fd = xdir ? Fx : Fy;
          const int nfd = xdir ? T::NFX : T::NFY;
#pragma unroll
          for (int q = 0; q < T::NF; ++q)
            Fd[q * nfd + f] = fl[FluxComps<2>::var(q)];
        }
      }
      else
      {
        int ea, eb;
        if (IK::at(w - IX::COUNT - IY::COUNT, ea, eb))
        {
          // corner (i0+ea, j0+eb): cells RT (i-1, j-1), RB (i-1, j),
          // LT (i, j-1), LB (i, j) in the slopes box
          const int q = ea + (T::TX + 1) * eb;
          int       cc[4];
          cc[0] = ea + T::SX * eb;
          cc[1] = cc[0] + T::SX;
          cc[2] = cc[0] + 1;
          cc[3] = cc[0] + 1 + T::SX;
          // half-step x-face fields at (i, j-1), (i, j) and y-face fields at
          // (i-1, j), (i, j), with their transverse limited slopes
          const int ml = (ea + 2) + T::MX * (eb + 1); // x face (i, j-1)
          const int mh = ml + T::MX;                  // x face (i, j)
          const int nl = (ea + 1) + T::MX * (eb + 2); // y face (i-1, j)
          const int nh = nl + 1;                      // y face (i, j)
          const int ec = (ea + 1) + T::EX * (eb + 1); // E(i, j)
          const R   bxl = face_field_x2(Ua[ml], Es[ec - T::EX], Es[ec], dtdy);
          const R   bxh = face_field_x2(Ua[mh], Es[ec], Es[ec + T::EX], dtdy);
          const R   byl = face_field_y2(Ub[nl], Es[ec - 1], Es[ec], dtdx);
          const R   byh = face_field_y2(Ub[nh], Es[ec], Es[ec + 1], dtdx);
          const R   sxl = slope_limited(Ua[ml], Ua[ml + T::MX], Ua[ml - T::MX], G.slope_type);
          const R   sxh = slope_limited(Ua[mh], Ua[mh + T::MX], Ua[mh - T::MX], G.slope_type);
          const R   syl = slope_limited(Ub[nl], Ub[nl + 1], Ub[nl - 1], G.slope_type);
          const R   syh = slope_limited(Ub[nh], Ub[nh + 1], Ub[nh - 1], G.slope_type);
          R         fb0[4], fb1[4];
#pragma unroll
          for (int e = 0; e < 4; ++e)
          {
            const R sb0 = (e == 0 || e == 2) ? R(1) : R(-1);
            const R sb1 = (e == 0 || e == 1) ? R(1) : R(-1);
            const R B0 = (e == 0 || e == 2) ? bxl : bxh, dB0 = (e == 0 || e == 2) ? sxl : sxh;
            const R B1 = (e == 0 || e == 1) ? byl : byh, dB1 = (e == 0 || e == 1) ? syl : syh;
            fb0[e] = B0 + R(0.5) * (sb0 * dB0);
            fb1[e] = B1 + R(0.5) * (sb1 * dB1);
          }
          State<R> qe[4];
          auto hydro = [&](int v) {
#pragma unroll
            for (int e = 0; e < 4; ++e)
            {
              const bool r0 = (e == 0 || e == 1), r1 = (e == 0 || e == 2);
              const R    sdq0 = r0 ? R(1) : R(-1), sdq1 = r1 ? R(1) : R(-1);
              const R    inc = R(0.5) * (sdq0 * S0s[v * T::NT + cc[e]] + sdq1 * S1s[v * T::NT + cc[e]]);
              qe[e][v] = Q2s[v * T::NT + cc[e]] + inc;
            }
          };
          hydro(ID);
          hydro(IU);
          hydro(IV);
          hydro(IW);
          hydro(IP);
#pragma unroll
          for (int e = 0; e < 4; ++e)
          {
            qe[e][IA] = fb0[e];
            qe[e][IB] = fb1[e];
          }
          hydro(IC);
#pragma unroll
          for (int e = 0; e < 4; ++e)
          {
            qe[e][ID] = sel_max(smallR, qe[e][ID]);
            qe[e][IP] = sel_max(smallp * qe[e][ID], qe[e][IP]);
          }
          Ems[q] = compute_emf(2, qe, G.gamma0, G.smallc);
        }
      }
    }
  }
  __syncthreads();

  // 4. update of the tile's interior cells (update_body / update_fp32)
  for (int t = tid; t < T::TX * T::TY; t += T::THREADS)
  {
    const int ua = t % T::TX, ub = t / T::TX;
    const int i = i0 + ua, j = j0 + ub;
    if (i >= G.nx + g || j >= G.ny + g)
      continue;
    const int64_t c = cell_at(G, i, j, 0);
    const int     fx = ua + (T::TX + 1) * ub, fy = ua + T::TX * ub;
    const R       dtd[2] = { dtdx, dtdy };
    if constexpr (sizeof(R) == 4)
    {
      // (update_fp32's arithmetic; every load before the first store)
      int   var[NV];
      float d[NV], h[NV], l[NV];
#pragma unroll
      for (int q = 0; q < T::NF; ++q)
      {
        var[q] = FluxComps<2>::var(q);
        float x = 0.f;
        x = x + (Fx[q * T::NFX + fx] - Fx[q * T::NFX + fx + 1]) * dtd[0];
        x = x + (Fy[q * T::NFY + fy] - Fy[q * T::NFY + fy + T::TX]) * dtd[1];
        d[q] = x;
      }
      var[T::NF] = IA;
      var[T::NF + 1] = IB;
      d[T::NF] = (Ems[fx + T::TX + 1] - Ems[fx]) * dtd[1];
      d[T::NF + 1] = (Ems[fx] - Ems[fx + 1]) * dtd[0];
#pragma unroll
      for (int k = 0; k < NV; ++k)
      {
        h[k] = Uin[c + var[k] * sv];
        l[k] = Ulo ? Ulo[c + var[k] * sv] : 0.f;
      }
#pragma unroll
      for (int k = 0; k < NV; ++k)
      {
        const int64_t cv = c + var[k] * sv;
        if (!Ulo)
        {
          Uout[cv] = __fadd_rn(h[k], d[k]);
          continue;
        }
        float hn, ln;
        compensated_sum(h[k], d[k], l[k], hn, ln);
        Uout[cv] = hn;
        Ulo[cv] = ln;
      }
    }
    else
    {
#pragma unroll
      for (int q = 0; q < T::NF; ++q)
      {
        const int v = FluxComps<2>::var(q);
        R         x = Uin[c + v * sv];
        x += Fx[q * T::NFX + fx] * dtd[0];
        x -= Fx[q * T::NFX + fx + 1] * dtd[0];
        x += Fy[q * T::NFY + fy] * dtd[1];
        x -= Fy[q * T::NFY + fy + T::TX] * dtd[1];
        Uout[c + v * sv] = x;
      }
      R x = Uin[c + IA * sv];
      x -= Ems[fx] * dtd[1];
      x += Ems[fx + T::TX + 1] * dtd[1];
      Uout[c + IA * sv] = x;
      x = Uin[c + IB * sv];
      x += Ems[fx] * dtd[0];
      x -= Ems[fx + 1] * dtd[0];
      Uout[c + IB * sv] = x;
    }
  }
  (void)sj;
}

// Tile (blockIdx.x, row0 + blockIdx.y) of the problem (a launch may cover a
// range of tile rows)
template <class R, int TY, int RS>
__global__ void __launch_bounds__(MTile<R, TY>::THREADS, MTile<R, TY>::MIN_BLOCKS)
k_mfused2d(const Grid<R> G, const R * __restrict__ Uin, R * __restrict__ Uout,
           R * __restrict__ Ulo, DevState * __restrict__ st, int row0)
{
  extern __shared__ __align__(16) unsigned char msm_raw[];
  mfused2d_tile<R, TY, RS>(G, Uin, Uout, Ulo, st, (int)blockIdx.x, row0 + (int)blockIdx.y,
                           msm_raw);
}

// The CFL reduction of the fused form: the rates of the interior cells
// without storing the primitives (the tile kernel computes its own),
// kDtCells cells per thread.
constexpr int kDtCells = 4;

template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_dt_only(const Grid<R> G, const R * __restrict__ U, DevState * st, int force)
{
  dt_cells_body<R, DIM, kDtCells>(G, U, st, force, blockIdx.x);
}

// interior cells base <= index < end (threads past end still join the block
// reduction)
template <class R, int DIM>
__global__ void __launch_bounds__(256)
k_dt_only_range(const Grid<R> G, const R * __restrict__ U, DevState * st, int64_t base,
                int64_t end)
{
  prim_dt_body<R, DIM, false>(G, U, nullptr, st, 0,
                              base + blockIdx.x * (int64_t)blockDim.x + threadIdx.x, end);
}

} // namespace MHD_VARIANT_TAG
} // namespace mhd
