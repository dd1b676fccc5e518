#include "HydroParams.h"

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
    riemannSolverType = 0;
  else if (rs == "llf")
    riemannSolverType = MHD_RIEMANN_LLF;
  else if (rs == "hll")
    riemannSolverType = MHD_RIEMANN_HLL;
  else if (rs == "hllc")
    riemannSolverType = 3;
  else if (rs == "hlld")
    riemannSolverType = MHD_RIEMANN_HLLD;
  else
  {
    std::cout << "Riemann Solver specified in parameter file is invalid\n";
    std::cout << "Use the default one : approx\n";
    riemannSolverType = 0;
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
  const std::string problem = map.getString("hydro", "problem", "unknown");
  p.problem = MHD_PROBLEM_ORSZAG_TANG; // unknown problems default to Orszag-Tang (SolverMHDMuscl.h:700-708)
  p.ot_kt = map.getFloat("OrszagTang", "kt", 0.0f);
  p.precision = precision;
  p.fp_mode = fp_mode;
  return p;
}

} // namespace ppkmhd_gb300
