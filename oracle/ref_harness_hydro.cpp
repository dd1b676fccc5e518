// Driver that runs the REFERENCE's own, unmodified hydro MUSCL functors on
// the CPU (SolverHydroMuscl<2>/<3>, solver names Hydro_Muscl_2D/3D).
//
// TEST INFRASTRUCTURE ONLY.  Compiled by oracle/build_ref.sh into
// oracle/_ref/libppkmhd_ref{64,32}.so next to ref_harness.cpp (its own
// translation unit, as SolverHydroMuscl.cpp is in the reference, so the hydro
// and MHD functor headers never meet).  It pins the C restatement
// oracle/hydro_oracle.c and generates the hydro golden fixtures.
//
// The call sequence restates the reference solver's driver:
//   * construction: SolverHydroMuscl.h:177-326 (allocate by implementation
//     version, the gravity field when [gravity] static/point is on, init,
//     make_boundaries, deep_copy(U2, U), compute_dt);
//   * init dispatch: SolverHydroMuscl.cpp:110-244 (unknown problems fall
//     back to implode; the disk writes the point-source gravity field);
//   * one iteration: SolverHydroMuscl.h:695-735 (compute_dt, then
//     godunov_unsplit(m_dt) ping-ponging U/U2) -> SolverHydroMuscl.cpp:
//     257-320 (2D) / :327-400 (3D);
//   * dt: SolverHydroMuscl.h:649-690 + SolverBase.cpp:148-179;
//   * boundaries: SolverBase.cpp:338-410 (X, then Y, then Z faces).
#include <cstring>
#include <string>

#include "shared/kokkos_shared.h"
#include "shared/HydroParams.h"
#include "shared/HydroState.h"
#include "shared/BoundariesFunctors.h"
#include "shared/RiemannSolvers.h"
#include "muscl/HydroInitFunctors2D.h"
#include "muscl/HydroInitFunctors3D.h"
#include "muscl/HydroRunFunctors2D.h"
#include "muscl/HydroRunFunctors3D.h"
#include "utils/config/ConfigMap.h"

using namespace ppkMHD;
using namespace ppkMHD::muscl;

#include "ref_harness_base.h"

namespace
{

bool
gravity_on(ConfigMap & cfg)
{
  // SolverBase.cpp:138-141
  return cfg.getBool("gravity", "static", false) || cfg.getBool("gravity", "point", false);
}

// SolverHydroMuscl<2>::init (SolverHydroMuscl.cpp:110-178) and
// init_four_quadrant (:60-82)
void
init_problem_2d(ConfigMap & cfg, HydroParams & params, DataArray2d U, VectorField2d gravity)
{
  const std::string problem = cfg.getString("hydro", "problem", "unknown");
  if (problem == "blast")
    InitBlastFunctor2D::apply(params, BlastParams(cfg), U);
  else if (problem == "kelvin_helmholtz")
    InitKelvinHelmholtzFunctor2D::apply(params, KHParams(cfg), U);
  else if (problem == "gresho_vortex")
    InitGreshoVortexFunctor2D::apply(params, GreshoParams(cfg), U);
  else if (problem == "four_quadrant")
  {
    int          configNumber = cfg.getInteger("riemann2d", "config_number", 0);
    real_t       xt = cfg.getFloat("riemann2d", "x", 0.8);
    real_t       yt = cfg.getFloat("riemann2d", "y", 0.8);
    HydroState2d U0, U1, U2, U3;
    getRiemannConfig2d(configNumber, U0, U1, U2, U3);
    primToCons_2D(U0, params.settings.gamma0);
    primToCons_2D(U1, params.settings.gamma0);
    primToCons_2D(U2, params.settings.gamma0);
    primToCons_2D(U3, params.settings.gamma0);
    InitFourQuadrantFunctor2D::apply(params, U, configNumber, U0, U1, U2, U3, xt, yt);
  }
  else if (problem == "isentropic_vortex")
    InitIsentropicVortexFunctor2D::apply(params, IsentropicVortexParams(cfg), U);
  else if (problem == "rayleigh_taylor")
    RayleighTaylorInstabilityFunctor2D::apply(params, RayleighTaylorInstabilityParams(cfg), U,
                                              gravity);
  else if (problem == "rising_bubble")
    RisingBubbleFunctor2D::apply(params, RisingBubbleParams(cfg), U, gravity);
  else if (problem == "disk")
    InitDiskFunctor2D::apply(params, DiskParams(cfg), PointSourceGravity(cfg), U, gravity);
  else
    InitImplodeFunctor2D::apply(params, ImplodeParams(cfg), U);
}

// SolverHydroMuscl<3>::init (SolverHydroMuscl.cpp:184-250)
void
init_problem_3d(ConfigMap & cfg, HydroParams & params, DataArray3d U, VectorField3d gravity)
{
  const std::string problem = cfg.getString("hydro", "problem", "unknown");
  if (problem == "blast")
    InitBlastFunctor3D::apply(params, BlastParams(cfg), U);
  else if (problem == "kelvin_helmholtz")
    InitKelvinHelmholtzFunctor3D::apply(params, KHParams(cfg), U);
  else if (problem == "gresho_vortex")
    InitGreshoVortexFunctor3D::apply(params, GreshoParams(cfg), U);
  else if (problem == "rayleigh_taylor")
    RayleighTaylorInstabilityFunctor3D::apply(params, RayleighTaylorInstabilityParams(cfg), U,
                                              gravity);
  else if (problem == "rising_bubble")
    RisingBubbleFunctor3D::apply(params, RisingBubbleParams(cfg), U, gravity);
  else if (problem == "disk")
    InitDiskFunctor3D::apply(params, DiskParams(cfg), PointSourceGravity(cfg), U, gravity);
  else
    InitImplodeFunctor3D::apply(params, ImplodeParams(cfg), U);
}

struct RefHydro2D : RefBase
{
  using DA = DataArray2d;
  DA            U, U2, Q, Fluxes_x, Fluxes_y, Slopes_x, Slopes_y;
  VectorField2d gravity;
  bool          gravity_enabled;

  RefHydro2D(char *& buf, int n)
    : RefBase(buf, n)
  {
    const int isize = params.isize, jsize = params.jsize, nbvar = params.nbvar;
    gravity_enabled = gravity_on(cfg);
    U = DA("U", isize, jsize, nbvar);
    U2 = DA("U2", isize, jsize, nbvar);
    Q = DA("Q", isize, jsize, nbvar);
    if (params.implementationVersion == 0)
    {
      Fluxes_x = DA("Fluxes_x", isize, jsize, nbvar);
      Fluxes_y = DA("Fluxes_y", isize, jsize, nbvar);
    }
    else
    {
      Slopes_x = DA("Slope_x", isize, jsize, nbvar);
      Slopes_y = DA("Slope_y", isize, jsize, nbvar);
      Fluxes_x = DA("Fluxes_x", isize, jsize, nbvar);
      Fluxes_y = Fluxes_x;
    }
    // the init functors of the gravity problems write the field; it exists
    // in the reference only when gravity is on
    gravity = VectorField2d("gravity field", isize, jsize);
    init_problem_2d(cfg, params, U, gravity);
    finish_init();
  }
  void
  finish_init()
  {
    make_boundaries(U);
    Kokkos::deep_copy(U2, U);
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
  void
  make_boundaries(DA Udata)
  {
    const int nbIter = params.ghostWidth * std::max(params.isize, params.jsize);
    MakeBoundariesFunctor2D<FACE_XMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D<FACE_XMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D<FACE_YMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor2D<FACE_YMAX>::apply(params, Udata, nbIter);
  }
  double
  compute_dt_local() override
  {
    real_t invDt = ZERO_F;
    DA     Udata = (m_iteration % 2 == 0) ? U : U2;
    if (gravity_enabled)
      ComputeDtGravityFunctor2D::apply(params, params.settings.cfl, gravity, Udata, invDt);
    else
      ComputeDtFunctor2D::apply(params, Udata, invDt);
    real_t dt = params.settings.cfl / invDt;
    return dt;
  }
  void
  step() override
  {
    compute_dt();
    if (m_iteration % 2 == 0)
      godunov(U, U2, m_dt);
    else
      godunov(U2, U, m_dt);
  }
  void
  godunov(DA data_in, DA data_out, real_t dt)
  {
    make_boundaries(data_in);
    Kokkos::deep_copy(data_out, data_in);
    ConvertToPrimitivesFunctor2D::apply(params, data_in, Q);
    if (params.implementationVersion == 0)
    {
      ComputeAndStoreFluxesFunctor2D::apply(params, Q, Fluxes_x, Fluxes_y, dt, gravity_enabled,
                                            gravity);
      UpdateFunctor2D::apply(params, data_out, Fluxes_x, Fluxes_y);
    }
    else
    {
      ComputeSlopesFunctor2D::apply(params, Q, Slopes_x, Slopes_y);
      ComputeTraceAndFluxes_Functor2D<XDIR>::apply(params, Q, Slopes_x, Slopes_y, Fluxes_x, dt,
                                                   gravity_enabled, gravity);
      UpdateDirFunctor2D<XDIR>::apply(params, data_out, Fluxes_x);
      ComputeTraceAndFluxes_Functor2D<YDIR>::apply(params, Q, Slopes_x, Slopes_y, Fluxes_y, dt,
                                                   gravity_enabled, gravity);
      UpdateDirFunctor2D<YDIR>::apply(params, data_out, Fluxes_y);
    }
    if (gravity_enabled)
      GravitySourceTermFunctor2D::apply(params, data_in, data_out, gravity, dt);
  }
};

struct RefHydro3D : RefBase
{
  using DA = DataArray3d;
  DA            U, U2, Q, Fluxes_x, Fluxes_y, Fluxes_z, Slopes_x, Slopes_y, Slopes_z;
  VectorField3d gravity;
  bool          gravity_enabled;

  RefHydro3D(char *& buf, int n)
    : RefBase(buf, n)
  {
    const int isize = params.isize, jsize = params.jsize, ksize = params.ksize;
    const int nbvar = params.nbvar;
    gravity_enabled = gravity_on(cfg);
    U = DA("U", isize, jsize, ksize, nbvar);
    U2 = DA("U2", isize, jsize, ksize, nbvar);
    Q = DA("Q", isize, jsize, ksize, nbvar);
    if (params.implementationVersion == 0)
    {
      Fluxes_x = DA("Fluxes_x", isize, jsize, ksize, nbvar);
      Fluxes_y = DA("Fluxes_y", isize, jsize, ksize, nbvar);
      Fluxes_z = DA("Fluxes_z", isize, jsize, ksize, nbvar);
    }
    else
    {
      Slopes_x = DA("Slope_x", isize, jsize, ksize, nbvar);
      Slopes_y = DA("Slope_y", isize, jsize, ksize, nbvar);
      Slopes_z = DA("Slope_z", isize, jsize, ksize, nbvar);
      Fluxes_x = DA("Fluxes_x", isize, jsize, ksize, nbvar);
      Fluxes_y = Fluxes_x;
      Fluxes_z = Fluxes_x;
    }
    gravity = VectorField3d("gravity field", isize, jsize, ksize);
    init_problem_3d(cfg, params, U, gravity);
    finish_init();
  }
  void
  finish_init()
  {
    make_boundaries(U);
    Kokkos::deep_copy(U2, U);
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
  void
  make_boundaries(DA Udata)
  {
    int max_size = std::max(params.isize, params.jsize);
    max_size = std::max(max_size, params.ksize);
    const int nbIter = params.ghostWidth * max_size * max_size;
    MakeBoundariesFunctor3D<FACE_XMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D<FACE_XMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D<FACE_YMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D<FACE_YMAX>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D<FACE_ZMIN>::apply(params, Udata, nbIter);
    MakeBoundariesFunctor3D<FACE_ZMAX>::apply(params, Udata, nbIter);
  }
  double
  compute_dt_local() override
  {
    real_t invDt = ZERO_F;
    DA     Udata = (m_iteration % 2 == 0) ? U : U2;
    if (gravity_enabled)
      ComputeDtGravityFunctor3D::apply(params, params.settings.cfl, gravity, Udata, invDt);
    else
      ComputeDtFunctor3D::apply(params, Udata, invDt);
    real_t dt = params.settings.cfl / invDt;
    return dt;
  }
  void
  step() override
  {
    compute_dt();
    if (m_iteration % 2 == 0)
      godunov(U, U2, m_dt);
    else
      godunov(U2, U, m_dt);
  }
  void
  godunov(DA data_in, DA data_out, real_t dt)
  {
    make_boundaries(data_in);
    Kokkos::deep_copy(data_out, data_in);
    ConvertToPrimitivesFunctor3D::apply(params, data_in, Q);
    if (params.implementationVersion == 0)
    {
      ComputeAndStoreFluxesFunctor3D::apply(params, Q, Fluxes_x, Fluxes_y, Fluxes_z, dt,
                                            gravity_enabled, gravity);
      UpdateFunctor3D::apply(params, data_out, Fluxes_x, Fluxes_y, Fluxes_z);
    }
    else
    {
      ComputeSlopesFunctor3D::apply(params, Q, Slopes_x, Slopes_y, Slopes_z);
      ComputeTraceAndFluxes_Functor3D<XDIR>::apply(params, Q, Slopes_x, Slopes_y, Slopes_z,
                                                   Fluxes_x, dt, gravity_enabled, gravity);
      UpdateDirFunctor3D<XDIR>::apply(params, data_out, Fluxes_x);
      ComputeTraceAndFluxes_Functor3D<YDIR>::apply(params, Q, Slopes_x, Slopes_y, Slopes_z,
                                                   Fluxes_y, dt, gravity_enabled, gravity);
      UpdateDirFunctor3D<YDIR>::apply(params, data_out, Fluxes_y);
      ComputeTraceAndFluxes_Functor3D<ZDIR>::apply(params, Q, Slopes_x, Slopes_y, Slopes_z,
                                                   Fluxes_z, dt, gravity_enabled, gravity);
      UpdateDirFunctor3D<ZDIR>::apply(params, data_out, Fluxes_z);
    }
    if (gravity_enabled)
      GravitySourceTermFunctor3D::apply(params, data_in, data_out, gravity, dt);
  }
};

} // namespace

RefBase *
ref_hydro_new(char *& buf, int n, bool three_d)
{
  if (three_d)
    return new RefHydro3D(buf, n);
  return new RefHydro2D(buf, n);
}

long
ref_hydro_initial_state(const char * ini_text, real_t * out)
{
  std::string s(ini_text);
  char *      buf = &s[0];
  ConfigMap   cfg(buf, (int)s.size());
  HydroParams params;
  params.setup(cfg);
  const std::string solver = cfg.getString("run", "solver_name", "unknown");
  if (solver == "Hydro_Muscl_2D")
  {
    DataArray2d   U("U", params.isize, params.jsize, params.nbvar);
    VectorField2d g("gravity field", params.isize, params.jsize);
    init_problem_2d(cfg, params, U, g);
    if (out)
      std::memcpy(out, U.data(), U.size() * sizeof(real_t));
    return (long)U.size();
  }
  if (solver == "Hydro_Muscl_3D")
  {
    DataArray3d   U("U", params.isize, params.jsize, params.ksize, params.nbvar);
    VectorField3d g("gravity field", params.isize, params.jsize, params.ksize);
    init_problem_3d(cfg, params, U, g);
    if (out)
      std::memcpy(out, U.data(), U.size() * sizeof(real_t));
    return (long)U.size();
  }
  return 0;
}

extern "C"
{
  // The gravity field the init functor writes (dim planes, LayoutRight
  // (i, j[, k], comp)), element count or 0
  long
  ref_hydro_gravity_field(const char * ini_text, real_t * out)
  {
    std::string s(ini_text);
    char *      buf = &s[0];
    ConfigMap   cfg(buf, (int)s.size());
    HydroParams params;
    params.setup(cfg);
    const std::string solver = cfg.getString("run", "solver_name", "unknown");
    if (solver == "Hydro_Muscl_2D")
    {
      DataArray2d   U("U", params.isize, params.jsize, params.nbvar);
      VectorField2d g("gravity field", params.isize, params.jsize);
      init_problem_2d(cfg, params, U, g);
      if (out)
        std::memcpy(out, g.data(), g.size() * sizeof(real_t));
      return (long)g.size();
    }
    if (solver == "Hydro_Muscl_3D")
    {
      DataArray3d   U("U", params.isize, params.jsize, params.ksize, params.nbvar);
      VectorField3d g("gravity field", params.isize, params.jsize, params.ksize);
      init_problem_3d(cfg, params, U, g);
      if (out)
        std::memcpy(out, g.data(), g.size() * sizeof(real_t));
      return (long)g.size();
    }
    return 0;
  }

  // riemann_hydro (RiemannSolvers.h:570-633) on nvar-component primitive
  // states; dim from the .ini's solver
  void
  ref_hydro_riemann(const char * ini_text, const real_t * qL, const real_t * qR, real_t * flux)
  {
    std::string s(ini_text);
    char *      buf = &s[0];
    ConfigMap   cfg(buf, (int)s.size());
    HydroParams p;
    p.setup(cfg);
    if (p.dimType == THREE_D)
    {
      HydroState3d l, r, g, f;
      for (int v = 0; v < 5; ++v)
      {
        l[v] = qL[v];
        r[v] = qR[v];
        g[v] = f[v] = 0;
      }
      riemann_hydro(l, r, g, f, p);
      for (int v = 0; v < 5; ++v)
        flux[v] = f[v];
    }
    else
    {
      HydroState2d l, r, g, f;
      for (int v = 0; v < 4; ++v)
      {
        l[v] = qL[v];
        r[v] = qR[v];
        g[v] = f[v] = 0;
      }
      riemann_hydro(l, r, g, f, p);
      for (int v = 0; v < 4; ++v)
        flux[v] = f[v];
    }
  }
}
