#include "HydroParams.h"

#include <cmath>

#include <cstdio>
#include <iostream>

namespace ppkmhd_gb300
{

// Reals go through ConfigMap::getFloat, i.e. they are rounded to float and
// widened back, defaults included (HydroParams.cpp:27-217).
void
HydroParams::setup(const ConfigMap & map)
{
  nStepmax = (int)map.getInteger("run", "nstepmax", 1000);
  tEnd = map.getFloat("run", "tend", 0.0f);
  nOutput = (int)map.getInteger("run", "noutput", 100);
  if (nOutput == 0)
    enableOutput = false;
  nlog = (int)map.getInteger("run", "nlog", 10);

  solver_name = map.getString("run", "solver_name", "unknown");
  valid_solver = true;
  if (solver_name == "MHD_Muscl_2D" || solver_name == "MHD_Muscl_2D_gpu")
  {
    dimType = TWO_D;
    nbvar = 8;
    ghostWidth = 3;
    mhdEnabled = true;
  }
  else if (solver_name == "MHD_Muscl_3D" || solver_name == "MHD_Muscl_3D_gpu")
  {
    dimType = THREE_D;
    nbvar = 8;
    ghostWidth = 3;
    mhdEnabled = true;
  }
  else if (solver_name == "Hydro_Muscl_2D" || solver_name == "Hydro_Muscl_2D_gpu")
  {
    dimType = TWO_D;
    nbvar = 4;
    ghostWidth = 2;
  }
  else if (solver_name == "Hydro_Muscl_3D" || solver_name == "Hydro_Muscl_3D_gpu")
  {
    dimType = THREE_D;
    nbvar = 5;
    ghostWidth = 2;
  }
  else
  {
    std::cerr << "Solver name not valid : " << solver_name << "\n";
    valid_solver = false;
  }

  nx = (int)map.getInteger("mesh", "nx", 1);
  ny = (int)map.getInteger("mesh", "ny", 1);
  nz = (int)map.getInteger("mesh", "nz", 1);
  xmin = map.getFloat("mesh", "xmin", 0.0f);
  ymin = map.getFloat("mesh", "ymin", 0.0f);
  zmin = map.getFloat("mesh", "zmin", 0.0f);
  xmax = map.getFloat("mesh", "xmax", 1.0f);
  ymax = map.getFloat("mesh", "ymax", 1.0f);
  zmax = map.getFloat("mesh", "zmax", 1.0f);
  static const char * bc_keys[6] = { "boundary_type_xmin", "boundary_type_xmax",
                                     "boundary_type_ymin", "boundary_type_ymax",
                                     "boundary_type_zmin", "boundary_type_zmax" };
  for (int f = 0; f < 6; ++f)
    boundary_type[f] = (int)map.getInteger("mesh", bc_keys[f], MHD_BC_REFLECTING);

  settings.gamma0 = map.getFloat("hydro", "gamma0", 1.4f);
  settings.cfl = map.getFloat("hydro", "cfl", 0.5f);
  settings.iorder = (int)map.getInteger("hydro", "iorder", 2);
  settings.slope_type = map.getFloat("hydro", "slope_type", 1.0f);
  settings.smallc = map.getFloat("hydro", "smallc", 1e-10f);
  settings.smallr = map.getFloat("hydro", "smallr", 1e-10f);

  niter_riemann = (int)map.getInteger("hydro", "niter_riemann", 10);
  const std::string rs = map.getString("hydro", "riemann", "approx");
  if (rs == "approx")
    riemannSolverType = MHD_RIEMANN_APPROX;
  else if (rs == "llf")
    riemannSolverType = MHD_RIEMANN_LLF;
  else if (rs == "hll")
    riemannSolverType = MHD_RIEMANN_HLL;
  else if (rs == "hllc")
    riemannSolverType = MHD_RIEMANN_HLLC;
  else if (rs == "hlld")
    riemannSolverType = MHD_RIEMANN_HLLD;
  else
  {
    std::cout << "Riemann Solver specified in parameter file is invalid\n";
    std::cout << "Use the default one : approx\n";
    riemannSolverType = MHD_RIEMANN_APPROX;
  }

  implementationVersion = (int)map.getFloat("OTHER", "implementationVersion", 0.0f);
  if (implementationVersion != 0 && implementationVersion != 1 && implementationVersion != 2)
  {
    std::cout << "Implementation version is invalid (must be 0, 1 or 2)\n";
    std::cout << "Use the default : 0\n";
    implementationVersion = 0;
  }
  init();
}

void
HydroParams::init()
{
  imin = jmin = kmin = 0;
  imax = nx - 1 + 2 * ghostWidth;
  jmax = ny - 1 + 2 * ghostWidth;
  kmax = nz - 1 + 2 * ghostWidth;
  isize = imax - imin + 1;
  jsize = jmax - jmin + 1;
  ksize = kmax - kmin + 1;
  dx = (xmax - xmin) / nx;
  dy = (ymax - ymin) / ny;
  dz = (zmax - zmin) / nz;
  settings.smallp = settings.smallc * settings.smallc / settings.gamma0;
  settings.smallpp = settings.smallr * settings.smallp;
  settings.gamma6 = (settings.gamma0 + 1.0) / (2.0 * settings.gamma0);
}

void
HydroParams::print() const
{
  std::printf("##########################\n");
  std::printf("Simulation run parameters:\n");
  std::printf("##########################\n");
  std::printf("nx         : %d\n", nx);
  std::printf("ny         : %d\n", ny);
  std::printf("nz         : %d\n", nz);
  std::printf("dx         : %f\n", dx);
  std::printf("dy         : %f\n", dy);
  std::printf("dz         : %f\n", dz);
  std::printf("imin       : %d\n", imin);
  std::printf("imax       : %d\n", imax);
  std::printf("jmin       : %d\n", jmin);
  std::printf("jmax       : %d\n", jmax);
  std::printf("kmin       : %d\n", kmin);
  std::printf("kmax       : %d\n", kmax);
  std::printf("ghostWidth : %d\n", ghostWidth);
  std::printf("nbvar      : %d\n", nbvar);
  std::printf("nStepmax   : %d\n", nStepmax);
  std::printf("tEnd       : %f\n", tEnd);
  std::printf("nOutput    : %d\n", nOutput);
  std::printf("gamma0     : %f\n", settings.gamma0);
  std::printf("cfl        : %f\n", settings.cfl);
  std::printf("smallr     : %12.10f\n", settings.smallr);
  std::printf("smallc     : %12.10f\n", settings.smallc);
  std::printf("slope_type : %f\n", settings.slope_type);
  std::printf("riemann    : %d\n", riemannSolverType);
  std::printf("implementationVersion : %d\n", implementationVersion);
  std::printf("##########################\n");
}

mhd_params
HydroParams::to_mhd_params(const ConfigMap & map, int precision, int fp_mode) const
{
  mhd_params p;
  mhd_params_default(&p);
  p.dim = dimType == THREE_D ? 3 : 2;
  p.nx = nx;
  p.ny = ny;
  p.nz = dimType == THREE_D ? nz : 1;
  p.ghost = ghostWidth;
  p.xmin = xmin;
  p.xmax = xmax;
  p.ymin = ymin;
  p.ymax = ymax;
  p.zmin = zmin;
  p.zmax = zmax;
  p.gamma0 = settings.gamma0;
  p.cfl = settings.cfl;
  p.slope_type = settings.slope_type;
  p.smallr = settings.smallr;
  p.smallc = settings.smallc;
  p.riemann = riemannSolverType;
  p.implementation_version = implementationVersion;
  for (int f = 0; f < 6; ++f)
    p.boundary[f] = boundary_type[f];
  // SolverBase::read_config (SolverBase.cpp:119-120)
  p.tEnd = map.getFloat("run", "tEnd", 0.0f);
  p.tCurrent = map.getFloat("run", "tCurrent", 0.0f);
  p.nStepmax = nStepmax;
  std::string problem = map.getString("hydro", "problem", "unknown");
  p.solver = mhdEnabled ? MHD_SOLVER_MHD_MUSCL : MHD_SOLVER_HYDRO_MUSCL;
  if (!mhdEnabled)
  {
    // the names SolverHydroMuscl<dim>::init dispatches (SolverHydroMuscl.cpp:
    // 123-177 in 2D, :202-244 in 3D); any other name runs implode with its
    // parameters
    const bool two = dimType == TWO_D;
    const bool known = problem == "implode" || problem == "blast" ||
                       problem == "kelvin_helmholtz" || problem == "gresho_vortex" ||
                       problem == "rayleigh_taylor" || problem == "rising_bubble" ||
                       problem == "disk" ||
                       (two && (problem == "four_quadrant" || problem == "isentropic_vortex"));
    if (!known)
      problem = "implode";
  }
  // unknown problems default to Orszag-Tang in the MHD solver
  // (SolverMHDMuscl.h:700-708) and to implode in the hydro solver
  // (SolverHydroMuscl.cpp:170-177)
  p.problem = mhdEnabled ? MHD_PROBLEM_ORSZAG_TANG : MHD_PROBLEM_IMPLODE;
  // SolverBase::read_config (SolverBase.cpp:138-141): static or point
  // gravity switches gravity on (2 marks point)
  p.gravity = map.getBool("gravity", "static", false) ? 1 : 0;
  if (map.getBool("gravity", "point", false))
    p.gravity = 2;
  p.ot_kt = map.getFloat("OrszagTang", "kt", 0.0f);
  double * r = p.problem_real;
  int *    n = p.problem_int;
  if (problem == "blast")
  {
    // BlastParams (src/shared/problems/BlastParams.h)
    p.problem = MHD_PROBLEM_BLAST;
    const double x0 = map.getFloat("mesh", "xmin", 0.0f), y0 = map.getFloat("mesh", "ymin", 0.0f);
    const double z0 = map.getFloat("mesh", "zmin", 0.0f), x1 = map.getFloat("mesh", "xmax", 1.0f);
    const double y1 = map.getFloat("mesh", "ymax", 1.0f), z1 = map.getFloat("mesh", "zmax", 1.0f);
    r[0] = map.getFloat("blast", "radius", (float)((x0 + x1) / 2.0 / 10));
    r[1] = map.getFloat("blast", "center_x", (float)((x0 + x1) / 2));
    r[2] = map.getFloat("blast", "center_y", (float)((y0 + y1) / 2));
    r[3] = map.getFloat("blast", "center_z", (float)((z0 + z1) / 2));
    r[4] = map.getFloat("blast", "density_in", 1.0f);
    r[5] = map.getFloat("blast", "density_out", 1.2f);
    r[6] = map.getFloat("blast", "pressure_in", 10.0f);
    r[7] = map.getFloat("blast", "pressure_out", 0.1f);
  }
  else if (problem == "implode")
  {
    // ImplodeParams (src/shared/problems/ImplodeParams.h)
    p.problem = MHD_PROBLEM_IMPLODE;
    const char * side[2] = { "outer", "inner" };
    const float  dflt[2][8] = { { 1.0f, 1.0f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f },
                                { 0.125f, 0.14f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f } };
    const char * key[8] = { "density_", "pressure_", "vx_", "vy_", "vz_", "Bx_", "By_", "Bz_" };
    for (int s = 0; s < 2; ++s)
      for (int q = 0; q < 8; ++q)
        r[8 * s + q] = map.getFloat("implode", std::string(key[q]) + side[s], dflt[s][q]);
    n[0] = (int)map.getInteger("implode", "shape_region", 0);
  }
  else if (problem == "kelvin_helmholtz")
  {
    // KHParams (src/shared/problems/KHParams.h)
    p.problem = MHD_PROBLEM_KELVIN_HELMHOLTZ;
    r[0] = map.getFloat("KH", "d_in", 1.0f);
    r[1] = map.getFloat("KH", "d_out", 1.0f);
    r[2] = map.getFloat("KH", "pressure", 10.0f);
    r[3] = map.getFloat("KH", "vflow_in", -0.5f);
    r[4] = map.getFloat("KH", "vflow_out", 0.5f);
    r[5] = map.getFloat("KH", "amplitude", 0.1f);
    r[6] = map.getFloat("KH", "w0", 0.1f);
    r[7] = map.getFloat("KH", "delta", 0.03f);
    n[0] = map.getBool("KH", "perturbation_sine", false) ? 1 : 0;
    n[1] = map.getBool("KH", "perturbation_sine_robertson", true) ? 1 : 0;
    n[2] = (int)map.getInteger("KH", "mode", 2);
    n[3] = map.getBool("KH", "perturbation_rand", false) ? 1 : 0;
  }
  else if (mhdEnabled && problem == "rotor")
  {
    // RotorParams (src/shared/problems/RotorParams.h)
    p.problem = MHD_PROBLEM_ROTOR;
    r[0] = map.getFloat("rotor", "r0", 0.1f);
    r[1] = map.getFloat("rotor", "r1", 0.115f);
    r[2] = map.getFloat("rotor", "u0", 2.0f);
    r[3] = map.getFloat("rotor", "p0", 1.0f);
    r[4] = map.getFloat("rotor", "b0", (float)(5.0 / std::sqrt(4 * M_PI)));
  }
  else if (mhdEnabled && (problem == "field_loop" || problem == "field loop"))
  {
    // FieldLoopParams (src/shared/problems/FieldLoopParams.h)
    p.problem = MHD_PROBLEM_FIELD_LOOP;
    r[0] = map.getFloat("FieldLoop", "radius", 1.0f);
    r[1] = map.getFloat("FieldLoop", "density_in", 1.0f);
    r[2] = map.getFloat("FieldLoop", "amplitude", 1.0f);
    r[3] = map.getFloat("FieldLoop", "vflow", 1.0f);
  }
  else if (mhdEnabled && problem == "wave")
  {
    // WaveParams (src/shared/problems/WaveParams.h): right eigenvectors of
    // the fast, Alfven, slow and contact waves and the rotated wave vector
    p.problem = MHD_PROBLEM_WAVE;
    const double xmn = map.getFloat("mesh", "xmin", 0.0f), ymn = map.getFloat("mesh", "ymin", 0.0f);
    const double zmn = map.getFloat("mesh", "zmin", 0.0f), xmx = map.getFloat("mesh", "xmax", 3.0f);
    const double ymx = map.getFloat("mesh", "ymax", 1.5f), zmx = map.getFloat("mesh", "zmax", 1.5f);
    const double Lx = xmx - xmn, Ly = ymx - ymn, Lz = zmx - zmn;
    const double g = map.getFloat("hydro", "gamma0", 1.66667f);
    const double amp = map.getFloat("wave", "amplitude", 1.0e-6f);
    const int    type = (int)map.getInteger("wave", "type", 0);
    static const double ev[4][7] = {
      { 4.472136e-01, -8.944272e-01, 4.216370e-01, 1.490712e-01, 2.012461e+00, 8.432740e-01,
        2.981424e-01 },
      { 0.0, 0.0, -3.333333e-01, 9.428090e-01, 0.0, -3.333333e-01, 9.428090e-01 },
      { 8.944272e-01, -4.472136e-01, -8.432740e-01, -2.981424e-01, 6.708204e-01, -4.216370e-01,
        -1.490712e-01 },
      { 1.0, 1.0, 0.0, 0.0, 0.5, 0.0, 0.0 } };
    n[0] = type;
    if (type >= 0 && type <= 3)
    {
      r[0] = amp;
      r[1] = type == 3 ? 1.0 : 0.0;
      for (int q = 0; q < 7; ++q)
        r[2 + q] = ev[type][q];
      r[9] = 1.0;
      r[10] = 1.0 / g;
      const double TwoPi = 4.0 * std::asin(1.0);
      const double ang_3 = std::atan(Lx / Ly);
      r[13] = std::sin(ang_3);
      r[14] = std::cos(ang_3);
      const double ang_2 = std::atan(0.5 * (Lx * r[14] + Ly * r[13]) / Lz);
      r[11] = std::sin(ang_2);
      r[12] = std::cos(ang_2);
      const double x1 = Lx * r[12] * r[14], x2 = Ly * r[12] * r[13], x3 = Lz * r[11];
      double       lambda = x1;
      if (ang_3 != 0.0)
        lambda = std::fmin(lambda, x2);
      if (ang_2 != 0.)
        lambda = std::fmin(lambda, x3);
      r[20] = TwoPi / lambda;
      r[15] = amp * r[2 + 5];
      r[16] = amp * r[2 + 6];
      r[17] = 1.0;
      r[18] = std::sqrt(2.0);
      r[19] = 0.5;
    }
  }
  else if (!mhdEnabled && problem == "gresho_vortex")
  {
    // GreshoParams (src/shared/problems/GreshoParams.h)
    p.problem = MHD_PROBLEM_GRESHO_VORTEX;
    r[0] = map.getFloat("Gresho", "rho0", 1.0f);
    r[1] = map.getFloat("Gresho", "Ma", 0.1f);
  }
  else if (!mhdEnabled && problem == "four_quadrant")
  {
    // SolverHydroMuscl<2>::init_four_quadrant (SolverHydroMuscl.cpp:60-82)
    p.problem = MHD_PROBLEM_FOUR_QUADRANT;
    n[0] = (int)map.getInteger("riemann2d", "config_number", 0);
    r[0] = map.getFloat("riemann2d", "x", 0.8f);
    r[1] = map.getFloat("riemann2d", "y", 0.8f);
  }
  else if (!mhdEnabled && problem == "isentropic_vortex")
  {
    // IsentropicVortexParams (src/shared/problems/IsentropicVortexParams.h)
    p.problem = MHD_PROBLEM_ISENTROPIC_VORTEX;
    const double x0 = map.getFloat("mesh", "xmin", 0.0f), x1 = map.getFloat("mesh", "xmax", 1.0f);
    const double y0 = map.getFloat("mesh", "ymin", 0.0f), y1 = map.getFloat("mesh", "ymax", 1.0f);
    r[0] = map.getFloat("isentropic_vortex", "density_ambient", 1.0f);
    r[1] = map.getFloat("isentropic_vortex", "temperature_ambient", 1.0f);
    r[2] = map.getFloat("isentropic_vortex", "vx_ambient", 1.0f);
    r[3] = map.getFloat("isentropic_vortex", "vy_ambient", 1.0f);
    r[4] = map.getFloat("isentropic_vortex", "center_x", (float)((x0 + x1) / 2));
    r[5] = map.getFloat("isentropic_vortex", "center_y", (float)((y0 + y1) / 2));
    r[6] = map.getFloat("isentropic_vortex", "strength", 5.0f);
  }
  else if (!mhdEnabled && problem == "rayleigh_taylor")
  {
    // RayleighTaylorInstabilityParams (src/shared/problems/RayleighTaylorInstabilityParams.h)
    p.problem = MHD_PROBLEM_RAYLEIGH_TAYLOR;
    r[0] = map.getFloat("rayleigh_taylor", "amplitude", 0.01f);
    r[1] = map.getFloat("rayleigh_taylor", "d0", 1.0f);
    r[2] = map.getFloat("rayleigh_taylor", "d1", 2.0f);
    r[3] = map.getFloat("rayleigh_taylor", "gx", 0.0f);
    r[4] = map.getFloat("rayleigh_taylor", "gy", -0.1f);
    r[5] = map.getFloat("rayleigh_taylor", "gz", 0.0f);
    for (int q = 0; q < 3; ++q)
      p.gravity_field[q] = r[3 + q];
  }
  else if (!mhdEnabled && problem == "rising_bubble")
  {
    // RisingBubbleParams (src/shared/problems/RisingBubbleParams.h)
    p.problem = MHD_PROBLEM_RISING_BUBBLE;
    r[0] = map.getFloat("rising_bubble", "R", 0.1f);
    r[1] = map.getFloat("rising_bubble", "x0", 0.5f);
    r[2] = map.getFloat("rising_bubble", "y0", 0.25f);
    r[3] = map.getFloat("rising_bubble", "z0", 0.5f);
    r[4] = map.getFloat("rising_bubble", "din", 1.0f);
    r[5] = map.getFloat("rising_bubble", "dout", 2.0f);
    r[6] = map.getFloat("rising_bubble", "gx", 0.0f);
    r[7] = map.getFloat("rising_bubble", "gy", -0.1f);
    r[8] = map.getFloat("rising_bubble", "gz", 0.0f);
    for (int q = 0; q < 3; ++q)
      p.gravity_field[q] = r[6 + q];
  }
  else if (!mhdEnabled && problem == "disk")
  {
    // DiskParams (src/shared/problems/DiskParams.h; its mesh defaults are
    // -0.5 .. 0.5) and PointSourceGravity (PointSourceGravity.h)
    p.problem = MHD_PROBLEM_DISK;
    const double x0 = map.getFloat("mesh", "xmin", -0.5f), y0 = map.getFloat("mesh", "ymin", -0.5f);
    const double z0 = map.getFloat("mesh", "zmin", -0.5f), x1 = map.getFloat("mesh", "xmax", 0.5f);
    const double y1 = map.getFloat("mesh", "ymax", 0.5f), z1 = map.getFloat("mesh", "zmax", 0.5f);
    r[0] = map.getFloat("disk", "radius", (float)((x1 - x0) * 0.125));
    r[1] = map.getFloat("disk", "radius_inner", (float)(r[0] / 10));
    r[2] = map.getFloat("disk", "xc", (float)((x0 + x1) / 2));
    r[3] = map.getFloat("disk", "yc", (float)((y0 + y1) / 2));
    r[4] = map.getFloat("disk", "zc", (float)((z0 + z1) / 2));
    r[5] = map.getFloat("disk", "ref_density", 1.0f);
    r[6] = map.getFloat("disk", "contrast_density", 100.0f);
    r[7] = map.getFloat("disk", "contrast_width", 0.01f);
    r[8] = map.getFloat("disk", "ref_sound_speed", 0.2f);
    r[9] = map.getFloat("gravity", "x", 0.0f);
    r[10] = map.getFloat("gravity", "y", 0.0f);
    r[11] = map.getFloat("gravity", "z", 0.0f);
    r[12] = (double)map.getFloat("gravity", "G", 1.0f) * (double)map.getFloat("gravity", "M", 1.0f);
    r[13] = map.getFloat("gravity", "soften", 0.01f);
  }
  if (p.dim == 2)
    p.gravity_field[2] = 0.0;
  p.precision = precision;
  p.fp_mode = fp_mode;
  return p;
}

} // namespace ppkmhd_gb300
