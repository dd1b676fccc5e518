// Driver that runs the REFERENCE's own, unmodified MHD functors on the CPU.
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh from the sources
// of ppkMHD (src/shared, src/muscl, src/utils/config) against the Kokkos-API
// shim in oracle/kokkos_shim, into oracle/_ref/libppkmhd_ref.so.  It is the
// checker used to pin the C restatement (oracle/mhd_oracle.c) and to generate
// the golden fixtures under tests/golden/; the product never links it.
//
// The call sequence restates, line for line, what the reference solver does:
//   * construction: SolverMHDMuscl.h:211-403 (allocate by implementation
//     version, init, make_boundaries, deep_copy(U2,U), convertToPrimitives,
//     compute_dt);
//   * one step: SolverBase.cpp:205-220 (next_iteration) ->
//     SolverMHDMuscl.h:791-805 (godunov_unsplit ping-pong) ->
//     SolverMHDMuscl.cpp:373-458 (2D) / :465-572 (3D);
//   * dt: SolverMHDMuscl.h:722-741 + SolverBase.cpp:148-179 (clip to tEnd);
//   * boundaries: SolverBase.cpp:513-537 (X, then Y, then Z faces).
// The drivers are restated because SolverMHDMuscl.h drags in the I/O and
// timer subsystems; the functors themselves are the reference's code.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "shared/kokkos_shared.h"
#include "shared/HydroParams.h"
#include "shared/HydroState.h"
#include "shared/BoundariesFunctors.h"
#include "shared/RiemannSolvers_MHD.h"
#include "muscl/MHDInitFunctors2D.h"
#include "muscl/MHDInitFunctors3D.h"
#include "muscl/MHDRunFunctors2D.h"
#include "muscl/MHDRunFunctors3D.h"
#include "utils/config/ConfigMap.h"
#include "utils/io/IO_VTK.h"

#include "ref_harness_base.h"

using namespace ppkMHD;
using namespace ppkMHD::muscl;

namespace
{

// SolverMHDMuscl<dim>::init (SolverMHDMuscl.h:649-710): the reference's init
// functor for [hydro] problem, Orszag-Tang for unknown names.
template <class DA>
void
init_problem_2d(ConfigMap & cfg, HydroParams & params, DA U)
{
  const std::string problem = cfg.getString("hydro", "problem", "unknown");
  if (problem == "blast")
    InitBlastFunctor2D_MHD::apply(params, BlastParams(cfg), U);
  else if (problem == "implode")
    InitImplodeFunctor2D_MHD::apply(params, ImplodeParams(cfg), U);
  else if (problem == "kelvin_helmholtz")
    InitKelvinHelmholtzFunctor2D_MHD::apply(params, KHParams(cfg), U);
  else if (problem == "rotor")
    InitRotorFunctor2D_MHD::apply(params, RotorParams(cfg), U);
  else if (problem == "field_loop" || problem == "field loop")
    InitFieldLoopFunctor2D_MHD::apply(params, FieldLoopParams(cfg), U);
  else if (problem == "wave")
    InitWaveFunctor2D_MHD::apply(params, WaveParams(cfg), U);
  else
    InitOrszagTangFunctor2D::apply(params, OrszagTangParams(cfg), U);
}

template <class DA>
void
init_problem_3d(ConfigMap & cfg, HydroParams & params, DA U)
{
  const std::string problem = cfg.getString("hydro", "problem", "unknown");
  if (problem == "blast")
    InitBlastFunctor3D_MHD::apply(params, BlastParams(cfg), U);
  else if (problem == "implode")
    InitImplodeFunctor3D_MHD::apply(params, ImplodeParams(cfg), U);
  else if (problem == "kelvin_helmholtz")
    InitKelvinHelmholtzFunctor3D_MHD::apply(params, KHParams(cfg), U);
  else if (problem == "rotor")
    InitRotorFunctor3D_MHD::apply(params, RotorParams(cfg), U);
  else if (problem == "field_loop" || problem == "field loop")
    InitFieldLoopFunctor3D_MHD::apply(params, FieldLoopParams(cfg), U);
  else if (problem == "wave")
    InitWaveFunctor3D_MHD::apply(params, WaveParams(cfg), U);
  else
    InitOrszagTangFunctor3D::apply(params, OrszagTangParams(cfg), U);
}

struct Ref2D : RefBase
{
  using DA = DataArray2d;
  DA               U, U2, Q, Q2, sFaceMag, Slopes_x, Slopes_y, ElecField;
  DA               Qm_x, Qm_y, Qp_x, Qp_y, QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB;
  DA               Fluxes_x, Fluxes_y;
  DataArrayScalar  Emf1;
  int              isize, jsize, nbvar;

  Ref2D(char *& buf, int n)
    : RefBase(buf, n)
  {
    isize = params.isize;
    jsize = params.jsize;
    nbvar = params.nbvar;
    // SolverMHDMuscl.h:270-305
    U = DA("U", isize, jsize, nbvar);
    U2 = DA("U2", isize, jsize, nbvar);
    Q = DA("Q", isize, jsize, nbvar);
    if (params.implementationVersion == 0 || params.implementationVersion == 1)
    {
      Qm_x = DA("Qm_x", isize, jsize, nbvar);
      Qm_y = DA("Qm_y", isize, jsize, nbvar);
      Qp_x = DA("Qp_x", isize, jsize, nbvar);
      Qp_y = DA("Qp_y", isize, jsize, nbvar);
      QEdge_RT = DA("QEdge_RT", isize, jsize, nbvar);
      QEdge_RB = DA("QEdge_RB", isize, jsize, nbvar);
      QEdge_LT = DA("QEdge_LT", isize, jsize, nbvar);
      QEdge_LB = DA("QEdge_LB", isize, jsize, nbvar);
    }
    else
    {
      Q2 = DA("Q2", isize, jsize, nbvar);
      sFaceMag = DA("sFaceMag", isize, jsize, 2);
      Slopes_x = DA("Slope_x", isize, jsize, nbvar);
      Slopes_y = DA("Slope_y", isize, jsize, nbvar);
      ElecField = DA("ElecField", isize, jsize, 1);
    }
    if (params.implementationVersion == 0)
    {
      Fluxes_x = DA("Fluxes_x", isize, jsize, nbvar);
      Fluxes_y = DA("Fluxes_y", isize, jsize, nbvar);
      Emf1 = DataArrayScalar("Emf", isize, jsize);
    }
    // SolverMHDMuscl.h:390-402 (initial condition by [hydro] problem,
    // dispatched as SolverMHDMuscl<dim>::init, SolverMHDMuscl.h:649-710)
    init_problem_2d(cfg, params, U);
    finish_init();
  }
  void
  finish_init()
  {
    make_boundaries(U);
    Kokkos::deep_copy(U2, U);
    ConvertToPrimitivesFunctor2D_MHD::apply(params, U, Q);
    compute_dt();
  }
  size_t
  nelem() const override
  {
    return U.size();
  }
  void
  set_state(const real_t * u) override
  {
    std::memcpy(U.data(), u, U.size() * sizeof(real_t));
    finish_init();
  }
  void
  get_state(real_t * u) const override
  {
    const DA & cur = (m_iteration % 2 == 0) ? U : U2;
    std::memcpy(u, cur.data(), cur.size() * sizeof(real_t));
  }
  // SolverBase.cpp:338-410, :513-521
  void
  make_boundaries(DA Udata)
  {
    const int nbIter = params.ghostWidth * std::max(params.isize, params.jsize);
    MakeBoundariesFunctor2D_MHD<FACE_XMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D_MHD<FACE_XMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D_MHD<FACE_YMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D_MHD<FACE_YMAX>::apply(params, Udata, nbIter);
  }
  double
  compute_dt_local() override
  {
    real_t invDt = ZERO_F;
    ComputeDtFunctor2D_MHD::apply(params, Q, invDt);
    real_t dt = params.settings.cfl / invDt;
    return dt;
  }
  void
  step() override
  {
    if (m_iteration % 2 == 0)
      godunov(U, U2);
    else
      godunov(U2, U);
  }
  // SolverMHDMuscl.cpp:373-458
  void
  godunov(DA data_in, DA data_out)
  {
    make_boundaries(data_in);
    Kokkos::deep_copy(data_out, data_in);
    ConvertToPrimitivesFunctor2D_MHD::apply(params, data_in, Q);
    compute_dt();
    const auto dtdx = m_dt / params.dx;
    const auto dtdy = m_dt / params.dy;
    if (params.implementationVersion == 0)
    {
      real_t dt = m_dt;
      ComputeTraceFunctor2D_MHD::apply(params, data_in, Q, Qm_x, Qm_y, Qp_x, Qp_y, QEdge_RT,
                                       QEdge_RB, QEdge_LT, QEdge_LB, (real_t)(dt / params.dx),
                                       (real_t)(dt / params.dy));
      ComputeFluxesAndStoreFunctor2D_MHD::apply(params, Qm_x, Qm_y, Qp_x, Qp_y, Fluxes_x, Fluxes_y,
                                                (real_t)(dt / params.dx), (real_t)(dt / params.dy));
      ComputeEmfAndStoreFunctor2D::apply(params, QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB, Emf1,
                                         (real_t)(dt / params.dx), (real_t)(dt / params.dy));
      UpdateFunctor2D_MHD::apply(params, data_out, Fluxes_x, Fluxes_y, dtdx, dtdy);
      UpdateEmfFunctor2D::apply(params, data_out, Emf1, dtdx, dtdy);
    }
    else if (params.implementationVersion == 1)
    {
      real_t dt = m_dt;
      ComputeTraceFunctor2D_MHD::apply(params, data_in, Q, Qm_x, Qm_y, Qp_x, Qp_y, QEdge_RT,
                                       QEdge_RB, QEdge_LT, QEdge_LB, (real_t)(dt / params.dx),
                                       (real_t)(dt / params.dy));
      ComputeFluxesAndUpdateFunctor2D_MHD::apply(params, Qm_x, Qm_y, Qp_x, Qp_y, data_out,
                                                 (real_t)(dt / params.dx),
                                                 (real_t)(dt / params.dy));
      ComputeEmfAndUpdateFunctor2D::apply(params, QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB, data_out,
                                          (real_t)(dt / params.dx), (real_t)(dt / params.dy));
    }
    else
    {
      ComputeSlopesFunctor2D_MHD::apply(params, data_in, Q, Slopes_x, Slopes_y);
      ComputeUpdatedPrimVarFunctor2D_MHD::apply(params, data_in, Q, Slopes_x, Slopes_y, Q2, dtdx,
                                                dtdy);
      ComputeElecFieldFunctor2D::apply(params, data_in, Q, ElecField);
      ComputeSourceFaceMagFunctor2D::apply(params, ElecField, sFaceMag, dtdx, dtdy);
      ComputeFluxAndUpdateAlongDirFunctor2D_MHD<DIR_X>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, sFaceMag, dtdx, dtdy);
      ComputeFluxAndUpdateAlongDirFunctor2D_MHD<DIR_Y>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, sFaceMag, dtdx, dtdy);
      ReconstructEdgeComputeEmfAndUpdateFunctor2D::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, sFaceMag, dtdx, dtdy);
    }
  }
};

struct Ref3D : RefBase
{
  using DA = DataArray3d;
  DA               U, U2, Q, Q2, sFaceMag, Slopes_x, Slopes_y, Slopes_z, ElecField;
  DA               Qm_x, Qm_y, Qm_z, Qp_x, Qp_y, Qp_z;
  DA               QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB;
  DA               QEdge_RT2, QEdge_RB2, QEdge_LT2, QEdge_LB2;
  DA               QEdge_RT3, QEdge_RB3, QEdge_LT3, QEdge_LB3;
  DA               Fluxes_x, Fluxes_y, Fluxes_z;
  DataArrayVector3 Emf, DeltaA, DeltaB, DeltaC;
  int              isize, jsize, ksize, nbvar;

  Ref3D(char *& buf, int n)
    : RefBase(buf, n)
  {
    isize = params.isize;
    jsize = params.jsize;
    ksize = params.ksize;
    nbvar = params.nbvar;
    // SolverMHDMuscl.h:312-386
    U = DA("U", isize, jsize, ksize, nbvar);
    U2 = DA("U2", isize, jsize, ksize, nbvar);
    Q = DA("Q", isize, jsize, ksize, nbvar);
    if (params.implementationVersion == 0 || params.implementationVersion == 1)
    {
      Qm_x = DA("Qm_x", isize, jsize, ksize, nbvar);
      Qm_y = DA("Qm_y", isize, jsize, ksize, nbvar);
      Qm_z = DA("Qm_z", isize, jsize, ksize, nbvar);
      Qp_x = DA("Qp_x", isize, jsize, ksize, nbvar);
      Qp_y = DA("Qp_y", isize, jsize, ksize, nbvar);
      Qp_z = DA("Qp_z", isize, jsize, ksize, nbvar);
      QEdge_RT = DA("QEdge_RT", isize, jsize, ksize, nbvar);
      QEdge_RB = DA("QEdge_RB", isize, jsize, ksize, nbvar);
      QEdge_LT = DA("QEdge_LT", isize, jsize, ksize, nbvar);
      QEdge_LB = DA("QEdge_LB", isize, jsize, ksize, nbvar);
      QEdge_RT2 = DA("QEdge_RT2", isize, jsize, ksize, nbvar);
      QEdge_RB2 = DA("QEdge_RB2", isize, jsize, ksize, nbvar);
      QEdge_LT2 = DA("QEdge_LT2", isize, jsize, ksize, nbvar);
      QEdge_LB2 = DA("QEdge_LB2", isize, jsize, ksize, nbvar);
      QEdge_RT3 = DA("QEdge_RT3", isize, jsize, ksize, nbvar);
      QEdge_RB3 = DA("QEdge_RB3", isize, jsize, ksize, nbvar);
      QEdge_LT3 = DA("QEdge_LT3", isize, jsize, ksize, nbvar);
      QEdge_LB3 = DA("QEdge_LB3", isize, jsize, ksize, nbvar);
      ElecField = DA("ElecField", isize, jsize, ksize, 3);
      DeltaA = DataArrayVector3("DeltaA", isize, jsize, ksize);
      DeltaB = DataArrayVector3("DeltaB", isize, jsize, ksize);
      DeltaC = DataArrayVector3("DeltaC", isize, jsize, ksize);
    }
    else
    {
      Q2 = DA("Q2", isize, jsize, ksize, nbvar);
      sFaceMag = DA("sFaceMag", isize, jsize, ksize, 3);
      Slopes_x = DA("Slope_x", isize, jsize, ksize, nbvar);
      Slopes_y = DA("Slope_y", isize, jsize, ksize, nbvar);
      Slopes_z = DA("Slope_z", isize, jsize, ksize, nbvar);
      ElecField = DA("ElecField", isize, jsize, ksize, 3);
    }
    if (params.implementationVersion == 0)
    {
      Fluxes_x = DA("Fluxes_x", isize, jsize, ksize, nbvar);
      Fluxes_y = DA("Fluxes_y", isize, jsize, ksize, nbvar);
      Fluxes_z = DA("Fluxes_z", isize, jsize, ksize, nbvar);
      Emf = DataArrayVector3("Emf", isize, jsize, ksize);
    }
    init_problem_3d(cfg, params, U);
    finish_init();
  }
  void
  finish_init()
  {
    make_boundaries(U);
    Kokkos::deep_copy(U2, U);
    ConvertToPrimitivesFunctor3D_MHD::apply(params, U, Q);
    compute_dt();
  }
  size_t
  nelem() const override
  {
    return U.size();
  }
  void
  set_state(const real_t * u) override
  {
    std::memcpy(U.data(), u, U.size() * sizeof(real_t));
    finish_init();
  }
  void
  get_state(real_t * u) const override
  {
    const DA & cur = (m_iteration % 2 == 0) ? U : U2;
    std::memcpy(u, cur.data(), cur.size() * sizeof(real_t));
  }
  // SolverBase.cpp:413-509, :524-537
  void
  make_boundaries(DA Udata)
  {
    int max_size = std::max(params.isize, params.jsize);
    max_size = std::max(max_size, params.ksize);
    const int nbIter = params.ghostWidth * max_size * max_size;
    MakeBoundariesFunctor3D_MHD<FACE_XMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D_MHD<FACE_XMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D_MHD<FACE_YMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D_MHD<FACE_YMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D_MHD<FACE_ZMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D_MHD<FACE_ZMAX>::apply(params, Udata, nbIter);
  }
  double
  compute_dt_local() override
  {
    real_t invDt = ZERO_F;
    ComputeDtFunctor3D_MHD::apply(params, Q, invDt);
    real_t dt = params.settings.cfl / invDt;
    return dt;
  }
  void
  step() override
  {
    if (m_iteration % 2 == 0)
      godunov(U, U2);
    else
      godunov(U2, U);
  }
  // SolverMHDMuscl.cpp:465-572
  void
  godunov(DA data_in, DA data_out)
  {
    make_boundaries(data_in);
    Kokkos::deep_copy(data_out, data_in);
    ConvertToPrimitivesFunctor3D_MHD::apply(params, data_in, Q);
    compute_dt();
    const auto dtdx = m_dt / params.dx;
    const auto dtdy = m_dt / params.dy;
    const auto dtdz = m_dt / params.dz;
    if (params.implementationVersion == 0 || params.implementationVersion == 1)
    {
      // SolverMHDMuscl.cpp:93-105 (computeElectricField, computeMagSlopes), :124-173 (trace)
      ComputeElecFieldFunctor3D::apply(params, data_in, Q, ElecField);
      ComputeMagSlopesFunctor3D::apply(params, data_in, DeltaA, DeltaB, DeltaC);
      real_t dt = m_dt;
      const real_t tdx = dt / params.dx, tdy = dt / params.dy, tdz = dt / params.dz;
      ComputeTraceFunctor3D_MHD::apply(params, data_in, Q, DeltaA, DeltaB, DeltaC, ElecField, Qm_x,
                                       Qm_y, Qm_z, Qp_x, Qp_y, Qp_z, QEdge_RT, QEdge_RB, QEdge_LT,
                                       QEdge_LB, QEdge_RT2, QEdge_RB2, QEdge_LT2, QEdge_LB2,
                                       QEdge_RT3, QEdge_RB3, QEdge_LT3, QEdge_LB3, tdx, tdy, tdz);
      if (params.implementationVersion == 0)
      {
        ComputeFluxesAndStoreFunctor3D_MHD::apply(params, Qm_x, Qm_y, Qm_z, Qp_x, Qp_y, Qp_z,
                                                  Fluxes_x, Fluxes_y, Fluxes_z, tdx, tdy, tdz);
        ComputeEmfAndStoreFunctor3D::apply(params, QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB,
                                           QEdge_RT2, QEdge_RB2, QEdge_LT2, QEdge_LB2, QEdge_RT3,
                                           QEdge_RB3, QEdge_LT3, QEdge_LB3, Emf, tdx, tdy, tdz);
        UpdateFunctor3D_MHD::apply(params, data_out, Fluxes_x, Fluxes_y, Fluxes_z, dtdx, dtdy,
                                   dtdz);
        UpdateEmfFunctor3D::apply(params, data_out, Emf, dtdx, dtdy, dtdz);
      }
      else
      {
        ComputeFluxesAndUpdateFunctor3D_MHD::apply(params, Qm_x, Qm_y, Qm_z, Qp_x, Qp_y, Qp_z,
                                                   data_out, tdx, tdy, tdz);
        ComputeEmfAndUpdateFunctor3D::apply(params, QEdge_RT, QEdge_RB, QEdge_LT, QEdge_LB,
                                            QEdge_RT2, QEdge_RB2, QEdge_LT2, QEdge_LB2, QEdge_RT3,
                                            QEdge_RB3, QEdge_LT3, QEdge_LB3, data_out, tdx, tdy,
                                            tdz);
      }
    }
    else
    {
      ComputeSlopesFunctor3D_MHD::apply(params, data_in, Q, Slopes_x, Slopes_y, Slopes_z);
      ComputeUpdatedPrimVarFunctor3D_MHD::apply(
        params, data_in, Q, Slopes_x, Slopes_y, Slopes_z, Q2, dtdx, dtdy, dtdz);
      ComputeElecFieldFunctor3D::apply(params, data_in, Q, ElecField);
      ComputeSourceFaceMagFunctor3D::apply(params, ElecField, sFaceMag, dtdx, dtdy, dtdz);
      ComputeFluxAndUpdateAlongDirFunctor3D_MHD<DIR_X>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
      ComputeFluxAndUpdateAlongDirFunctor3D_MHD<DIR_Y>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
      ComputeFluxAndUpdateAlongDirFunctor3D_MHD<DIR_Z>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
      ReconstructEdgeComputeEmfAndUpdateFunctor3D<DIR_X>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
      ReconstructEdgeComputeEmfAndUpdateFunctor3D<DIR_Y>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
      ReconstructEdgeComputeEmfAndUpdateFunctor3D<DIR_Z>::apply(
        params, data_in, data_out, Q2, Slopes_x, Slopes_y, Slopes_z, sFaceMag, dtdx, dtdy, dtdz);
    }
  }
};

HydroParams
params_from_ini(const char * ini)
{
  std::string s(ini);
  char *      buf = &s[0];
  ConfigMap   cfg(buf, (int)s.size());
  HydroParams p;
  p.setup(cfg);
  return p;
}

} // namespace

extern "C"
{

  int
  ref_real_bytes()
  {
    return (int)sizeof(real_t);
  }

  void *
  ref_create(const char * ini_text)
  {
    std::string s(ini_text);
    char *      buf = &s[0];
    ConfigMap   probe(buf, (int)s.size());
    std::string solver = probe.getString("run", "solver_name", "unknown");
    buf = &s[0];
    if (solver == "MHD_Muscl_2D")
      return new Ref2D(buf, (int)s.size());
    if (solver == "MHD_Muscl_3D")
      return new Ref3D(buf, (int)s.size());
    if (solver == "Hydro_Muscl_2D" || solver == "Hydro_Muscl_3D")
      return ref_hydro_new(buf, (int)s.size(), solver == "Hydro_Muscl_3D");
    return nullptr;
  }

  void
  ref_destroy(void * h)
  {
    delete static_cast<RefBase *>(h);
  }

  // The init functor's output alone (no boundary fill), LayoutRight, for the
  // sizes of ref_create on the same text.  Returns the element count, 0 on
  // an unknown solver.
  long
  ref_initial_state(const char * ini_text, real_t * out)
  {
    std::string s(ini_text);
    char *      buf = &s[0];
    ConfigMap   cfg(buf, (int)s.size());
    HydroParams params;
    params.setup(cfg);
    const std::string solver = cfg.getString("run", "solver_name", "unknown");
    if (solver == "MHD_Muscl_2D")
    {
      DataArray2d U("U", params.isize, params.jsize, params.nbvar);
      init_problem_2d(cfg, params, U);
      if (out)
        std::memcpy(out, U.data(), U.size() * sizeof(real_t));
      return (long)U.size();
    }
    if (solver == "MHD_Muscl_3D")
    {
      DataArray3d U("U", params.isize, params.jsize, params.ksize, params.nbvar);
      init_problem_3d(cfg, params, U);
      if (out)
        std::memcpy(out, U.data(), U.size() * sizeof(real_t));
      return (long)U.size();
    }
    if (solver == "Hydro_Muscl_2D" || solver == "Hydro_Muscl_3D")
      return ref_hydro_initial_state(ini_text, out);
    return 0;
  }

  // sizes: isize, jsize, ksize, nbvar, dim, ghostWidth
  void
  ref_sizes(void * h, int * out)
  {
    auto * r = static_cast<RefBase *>(h);
    out[0] = r->params.isize;
    out[1] = r->params.jsize;
    out[2] = r->params.dimType == THREE_D ? r->params.ksize : 1;
    out[3] = r->params.nbvar;
    out[4] = r->params.dimType == THREE_D ? 3 : 2;
    out[5] = r->params.ghostWidth;
  }

  // State in the reference's host layout (LayoutRight: (i,j[,k],var), var fastest).
  void
  ref_get_state(void * h, real_t * u)
  {
    static_cast<RefBase *>(h)->get_state(u);
  }

  // Inject U (LayoutRight) as the initial condition, then redo what the
  // constructor does after init(): boundaries, U2=U, primitives, dt.
  void
  ref_set_state(void * h, const real_t * u)
  {
    static_cast<RefBase *>(h)->set_state(u);
  }

  // Run n iterations of the main loop (main.cpp:154-159), stopping early when
  // finished().  Returns the number of iterations executed.
  int
  ref_run(void * h, int n)
  {
    auto * r = static_cast<RefBase *>(h);
    int    done = 0;
    while (done < n && !r->finished())
    {
      r->next_iteration();
      ++done;
    }
    return done;
  }

  // t, dt (for the NEXT step's... as the reference holds it), iteration
  void
  ref_time(void * h, double * t, double * dt, int * it)
  {
    auto * r = static_cast<RefBase *>(h);
    *t = r->m_t;
    *dt = r->m_dt;
    *it = r->m_iteration;
  }

  // ---- function-level probes (normal-frame states, 8 reals each) ----
  void
  ref_riemann(const char * ini_text, const real_t * qL, const real_t * qR, real_t * flux)
  {
    HydroParams p = params_from_ini(ini_text);
    MHDState    l, r, f;
    for (int v = 0; v < 8; ++v)
    {
      l[v] = qL[v];
      r[v] = qR[v];
      f[v] = 0;
    }
    riemann_mhd(l, r, f, p);
    for (int v = 0; v < 8; ++v)
      flux[v] = f[v];
  }

  // qEdge: 4 states in the order RT, RB, LT, LB (EdgeIndex), 8 reals each.
  real_t
  ref_compute_emf(const char * ini_text, int emf_dir, const real_t * qEdge)
  {
    HydroParams p = params_from_ini(ini_text);
    MHDState    q[4];
    for (int e = 0; e < 4; ++e)
      for (int v = 0; v < 8; ++v)
        q[e][v] = qEdge[e * 8 + v];
    if (emf_dir == EMFZ)
      return compute_emf<EMFZ>(q, p);
    if (emf_dir == EMFY)
      return compute_emf<EMFY>(q, p);
    return compute_emf<EMFX>(q, p);
  }

  // The reference's VTK writer (save_VTK_2D / save_VTK_3D, IO_VTK.cpp) on the
  // state u (LayoutRight, the sizes of the .ini), with SolverBase's variable
  // names (SolverBase.cpp:48-55) and no debug name.  Returns 0, or -1 on an
  // unknown solver.
  int
  ref_save_vtk(const char * ini_text, const real_t * u, int iStep)
  {
    std::string s(ini_text);
    char *      buf = &s[0];
    ConfigMap   cfg(buf, (int)s.size());
    HydroParams params;
    params.setup(cfg);
    const std::map<int, std::string> names = { { ID, "rho" },    { IP, "energy" }, { IU, "rho_vx" },
                                               { IV, "rho_vy" }, { IW, "rho_vz" }, { IA, "bx" },
                                               { IB, "by" },     { IC, "bz" } };
    const std::string solver = cfg.getString("run", "solver_name", "unknown");
    if (solver == "MHD_Muscl_2D" || solver == "Hydro_Muscl_2D")
    {
      DataArray2d U("U", params.isize, params.jsize, params.nbvar);
      std::memcpy(U.data(), u, U.size() * sizeof(real_t));
      DataArray2d::HostMirror Uh = Kokkos::create_mirror(U);
      ppkMHD::io::save_VTK_2D(U, Uh, params, cfg, params.nbvar, names, iStep, "");
      return 0;
    }
    if (solver == "MHD_Muscl_3D" || solver == "Hydro_Muscl_3D")
    {
      DataArray3d U("U", params.isize, params.jsize, params.ksize, params.nbvar);
      std::memcpy(U.data(), u, U.size() * sizeof(real_t));
      DataArray3d::HostMirror Uh = Kokkos::create_mirror(U);
      ppkMHD::io::save_VTK_3D(U, Uh, params, cfg, params.nbvar, names, iStep, "");
      return 0;
    }
    return -1;
  }

  // Effective (float-rounded, as ConfigMap::getFloat parses) parameters:
  // gamma0, cfl, slope_type, smallr, smallc, smallp, dx, dy, dz, tEnd
  void
  ref_params(const char * ini_text, double * out)
  {
    HydroParams p = params_from_ini(ini_text);
    out[0] = p.settings.gamma0;
    out[1] = p.settings.cfl;
    out[2] = p.settings.slope_type;
    out[3] = p.settings.smallr;
    out[4] = p.settings.smallc;
    out[5] = p.settings.smallp;
    out[6] = p.dx;
    out[7] = p.dy;
    out[8] = p.dz;
    out[9] = p.tEnd;
  }

} // extern "C"
