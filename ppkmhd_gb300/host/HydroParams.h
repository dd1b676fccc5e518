// Run / mesh / scheme parameters of the MHD MUSCL solver, filled from a
// ConfigMap with the rules of ppkMHD's HydroParams::setup
// (src/shared/HydroParams.cpp:27-217) and HydroParams::init (:420-453).
// Only the fields the MHD MUSCL-Hancock step reads are kept.
#pragma once

#include <string>

#include "ConfigMap.h"
#include "ppkmhd_gb300.h"

namespace ppkmhd_gb300
{

enum DimensionType
{
  TWO_D = 2,
  THREE_D = 3
};

struct HydroSettings
{
  double gamma0 = 1.4;
  double gamma6 = 1.0;
  double cfl = 1.0;
  double slope_type = 2.0;
  int    iorder = 1;
  double smallr = 1e-8;
  double smallc = 1e-8;
  double smallp = 1e-6;
  double smallpp = 1e-6;
  double cIso = 0;
};

struct HydroParams
{
  // run
  int    nStepmax = 0;
  double tEnd = 0.0;
  int    nOutput = 0;
  bool   enableOutput = true;
  bool   mhdEnabled = false;
  int    nlog = 10;
  // mesh
  int           nx = 0, ny = 0, nz = 0;
  int           ghostWidth = 2;
  int           nbvar = 4;
  DimensionType dimType = TWO_D;
  int           imin = 0, imax = 0, jmin = 0, jmax = 0, kmin = 0, kmax = 0;
  int           isize = 0, jsize = 0, ksize = 0;
  double        xmin = 0.0, xmax = 1.0, ymin = 0.0, ymax = 1.0, zmin = 0.0, zmax = 1.0;
  double        dx = 0.0, dy = 0.0, dz = 0.0;
  int           boundary_type[6] = { 0, 0, 0, 0, 0, 0 };
  // scheme
  HydroSettings settings;
  int           niter_riemann = 10;
  int           riemannSolverType = 0;
  int           implementationVersion = 0;
  std::string   solver_name;
  bool          valid_solver = false;

  //! HydroParams::setup: read everything from the map, then init().
  void
  setup(const ConfigMap & map);
  //! HydroParams::init: derived sizes, dx, smallp, gamma6.
  void
  init();
  //! Parameter dump in the spirit of HydroParams::print (HydroParams.cpp:458-506).
  void
  print() const;
  //! The C-ABI parameter block for this configuration.
  mhd_params
  to_mhd_params(const ConfigMap & map, int precision, int fp_mode) const;
};

} // namespace ppkmhd_gb300
