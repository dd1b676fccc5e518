// Driver state shared by the reference harness translation units
// (ref_harness.cpp: MHD solvers, ref_harness_hydro.cpp: hydro solvers).
// TEST INFRASTRUCTURE ONLY: restates SolverBase's time-step bookkeeping
// (SolverBase.cpp:148-220) around the reference's own functors.
#pragma once

#include "shared/HydroParams.h"
#include "utils/config/ConfigMap.h"

struct RefBase
{
  ConfigMap   cfg;
  ppkMHD::HydroParams params;
  double      m_t = 0, m_dt = 0, m_tEnd = 0;
  int         m_iteration = 0;
  RefBase(char *& buf, int n)
    : cfg(buf, n)
  {
    params.setup(cfg);
    m_tEnd = cfg.getFloat("run", "tEnd", 0.0);
    m_t = cfg.getFloat("run", "tCurrent", 0.0);
  }
  virtual ~RefBase() {}
  virtual void
  step() = 0;
  virtual void
  set_state(const ppkMHD::real_t * u) = 0;
  virtual void
  get_state(ppkMHD::real_t * u) const = 0;
  virtual size_t
  nelem() const = 0;
  virtual double
  compute_dt_local() = 0;
  // SolverBase.cpp:148-179
  void
  compute_dt()
  {
    m_dt = compute_dt_local();
    if (m_t + m_dt > m_tEnd)
      m_dt = m_tEnd - m_t;
  }
  // SolverBase.cpp:195-201
  int
  finished() const
  {
    return m_t >= (m_tEnd - 1e-14) || m_iteration >= params.nStepmax;
  }
  // SolverBase.cpp:205-220
  void
  next_iteration()
  {
    step();
    ++m_iteration;
    m_t += m_dt;
  }
};


// ref_harness_hydro.cpp: a Hydro_Muscl_2D/3D driver on the .ini text
RefBase * ref_hydro_new(char *& buf, int n, bool three_d);
// the hydro init functor's output alone (LayoutRight), element count or 0
long ref_hydro_initial_state(const char * ini_text, ppkMHD::real_t * out);
