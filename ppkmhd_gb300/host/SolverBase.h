// Abstract solver with the semantics of ppkMHD's SolverBase
// (src/shared/SolverBase.{h,cpp}): time loop bookkeeping, dt clip to tEnd,
// finished(), output cadence and the five phase timers.  MPI parts of the
// reference are not part of this single-GPU back-end.
#pragma once

#include <chrono>
#include <map>
#include <memory>
#include <string>

#include "ConfigMap.h"
#include "HydroParams.h"

namespace ppkmhd_gb300
{

enum TimerIds
{
  TIMER_TOTAL = 0,
  TIMER_IO = 1,
  TIMER_DT = 2,
  TIMER_BOUNDARIES = 3,
  TIMER_NUM_SCHEME = 4
};

//! Accumulating wall-clock timer (OpenMPTimer semantics: start/stop/elapsed seconds).
class Timer
{
public:
  void
  start()
  {
    m_t0 = std::chrono::steady_clock::now();
    m_running = true;
  }
  void
  stop()
  {
    if (m_running)
      m_total += std::chrono::duration<double>(std::chrono::steady_clock::now() - m_t0).count();
    m_running = false;
  }
  double
  elapsed() const
  {
    return m_total;
  }

private:
  std::chrono::steady_clock::time_point m_t0;
  double                                m_total = 0.0;
  bool                                  m_running = false;
};

class SolverBase
{
public:
  SolverBase(HydroParams & params, ConfigMap & configMap);
  virtual ~SolverBase();

  HydroParams & params;
  ConfigMap &   configMap;

  double      m_t = 0.0;
  double      m_dt = 0.0;
  int         m_iteration = 0;
  double      m_tEnd = 0.0;
  double      m_cfl = 0.0;
  int         m_nlog = 10;
  long long   m_nCells = 0;
  long long   m_nDofsPerCell = 1;
  std::string m_problem_name;
  std::string m_solver_name;
  int         m_times_saved = 0;
  std::map<int, std::string> m_variables_names;
  std::unique_ptr<Timer>     timers[5];

  //! SolverBase::read_config (SolverBase.cpp:113-142)
  virtual void
  read_config();
  //! compute_dt + clip to tEnd (SolverBase.cpp:148-179)
  virtual void
  compute_dt();
  virtual double
  compute_dt_local();
  //! t >= tEnd - 1e-14 or iteration >= nStepmax (SolverBase.cpp:195-201)
  virtual int
  finished();
  //! next_iteration_impl, then ++iteration, t += dt (SolverBase.cpp:205-220)
  virtual void
  next_iteration();
  virtual void
  next_iteration_impl();
  //! output cadence (SolverBase.cpp:264-290)
  virtual int
  should_save_solution();
  virtual void
  save_solution();
  virtual void
  save_solution_impl();
  //! Whether construction succeeded (the reference aborts instead).
  virtual bool
  ok() const
  {
    return true;
  }
  virtual std::string
  error() const
  {
    return "";
  }
};

} // namespace ppkmhd_gb300
