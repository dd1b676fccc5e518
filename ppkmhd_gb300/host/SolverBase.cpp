#include "SolverBase.h"

#include <cmath>

namespace ppkmhd_gb300
{

SolverBase::SolverBase(HydroParams & p, ConfigMap & cfg)
  : params(p)
  , configMap(cfg)
{
  for (auto & t : timers)
    t.reset(new Timer());
  // variable names of SolverBase.cpp:48-55
  m_variables_names[0] = "rho";
  m_variables_names[1] = "energy";
  m_variables_names[2] = "rho_vx";
  m_variables_names[3] = "rho_vy";
  m_variables_names[4] = "rho_vz";
  m_variables_names[5] = "bx";
  m_variables_names[6] = "by";
  m_variables_names[7] = "bz";
  read_config();
}

SolverBase::~SolverBase() {}

void
SolverBase::read_config()
{
  m_t = configMap.getFloat("run", "tCurrent", 0.0f);
  m_tEnd = configMap.getFloat("run", "tEnd", 0.0f);
  m_dt = m_tEnd;
  m_cfl = configMap.getFloat("hydro", "cfl", 1.0f);
  m_nlog = (int)configMap.getFloat("run", "nlog", 10.0f);
  m_problem_name = configMap.getString("hydro", "problem", "unknown");
  m_solver_name = configMap.getString("run", "solver_name", "unknown");
}

void
SolverBase::compute_dt()
{
  m_dt = compute_dt_local();
  if (m_t + m_dt > m_tEnd)
    m_dt = m_tEnd - m_t;
}

double
SolverBase::compute_dt_local()
{
  return m_tEnd;
}

int
SolverBase::finished()
{
  return m_t >= (m_tEnd - 1e-14) || m_iteration >= params.nStepmax;
}

void
SolverBase::next_iteration()
{
  next_iteration_impl();
  ++m_iteration;
  m_t += m_dt;
}

void
SolverBase::next_iteration_impl()
{}

int
SolverBase::should_save_solution()
{
  const double interval = m_tEnd / params.nOutput;
  if (params.nOutput < 0)
    return 1;
  if ((m_t - (m_times_saved - 1) * interval) > interval)
    return 1;
  if (std::fabs(m_t - m_tEnd) < 1e-12) // ISFUZZYNULL (utils.h:21)
    return 1;
  return 0;
}

void
SolverBase::save_solution()
{
  save_solution_impl();
  ++m_times_saved;
}

void
SolverBase::save_solution_impl()
{}

} // namespace ppkmhd_gb300
