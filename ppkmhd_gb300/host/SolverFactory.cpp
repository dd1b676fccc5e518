#include "SolverFactory.h"

#include <iostream>

#include "SolverMHDMusclGPU.h"

namespace ppkmhd_gb300
{

SolverFactory &
SolverFactory::Instance()
{
  static SolverFactory instance;
  return instance;
}

SolverFactory::SolverFactory()
{
  registerSolver("MHD_Muscl_2D", &SolverMHDMusclGPU<2>::create);
  registerSolver("MHD_Muscl_3D", &SolverMHDMusclGPU<3>::create);
  registerSolver("MHD_Muscl_2D_gpu", &SolverMHDMusclGPU<2>::create);
  registerSolver("MHD_Muscl_3D_gpu", &SolverMHDMusclGPU<3>::create);
  // the hydro-only MUSCL solver (SolverHydroMuscl<dim> of the reference) runs
  // through the same context: mhd_params::solver selects the scheme
  registerSolver("Hydro_Muscl_2D", &SolverMHDMusclGPU<2>::create);
  registerSolver("Hydro_Muscl_3D", &SolverMHDMusclGPU<3>::create);
  registerSolver("Hydro_Muscl_2D_gpu", &SolverMHDMusclGPU<2>::create);
  registerSolver("Hydro_Muscl_3D_gpu", &SolverMHDMusclGPU<3>::create);
}

void
SolverFactory::registerSolver(const std::string & key, SolverCreateFn fn)
{
  m_map[key] = fn;
}

void
SolverFactory::printValidSolversNames() const
{
  std::cout << "Valid solver names are:\n";
  for (const auto & kv : m_map)
    std::cout << kv.first << "\n";
}

SolverBase *
SolverFactory::create(const std::string & key, HydroParams & params, ConfigMap & configMap)
{
  auto it = m_map.find(key);
  if (it == m_map.end())
  {
    std::cout << "The solver you requested (" << key << ") does not exist.\n";
    printValidSolversNames();
    return nullptr;
  }
  SolverBase * solver = it->second(params, configMap);
  if (solver && !solver->ok())
  {
    std::cerr << "solver creation failed: " << solver->error() << "\n";
    delete solver;
    return nullptr;
  }
  return solver;
}

} // namespace ppkmhd_gb300
