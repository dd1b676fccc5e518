// Solver registry with the interface of ppkMHD's SolverFactory
// (src/shared/SolverFactory.h:43-116): name -> SolverCreateFn.  The MHD
// MUSCL names MHD_Muscl_2D / MHD_Muscl_3D (SolverFactory.cpp:29-30), plus
// the explicit aliases MHD_Muscl_2D_gpu / MHD_Muscl_3D_gpu, create the
// GB300 solver.  An unknown name prints the registered list and returns
// nullptr (the reference aborts).
#pragma once

#include <map>
#include <string>

#include "ConfigMap.h"
#include "HydroParams.h"
#include "SolverBase.h"

namespace ppkmhd_gb300
{

using SolverCreateFn = SolverBase * (*)(HydroParams & params, ConfigMap & configMap);

class SolverFactory
{
public:
  static SolverFactory &
  Instance();
  void
  registerSolver(const std::string & key, SolverCreateFn fn);
  SolverBase *
  create(const std::string & key, HydroParams & params, ConfigMap & configMap);
  void
  printValidSolversNames() const;

private:
  SolverFactory();
  std::map<std::string, SolverCreateFn> m_map;
};

} // namespace ppkmhd_gb300
