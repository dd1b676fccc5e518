// GB300 solver behind ppkMHD's plugin interface: the replacement of
// SolverMHDMuscl<dim> (src/muscl/SolverMHDMuscl.h, .cpp).  All state lives
// on the GPU inside an mhd_ctx (include/ppkmhd_gb300.h); this class keeps
// the SolverBase bookkeeping (t, dt, iteration, output cadence, timers) in
// step with the device.
#pragma once

#include <string>
#include <vector>

#include "SolverBase.h"
#include "ppkmhd_gb300.h"

namespace ppkmhd_gb300
{

template <int dim>
class SolverMHDMusclGPU : public SolverBase
{
public:
  SolverMHDMusclGPU(HydroParams & params, ConfigMap & configMap);
  ~SolverMHDMusclGPU() override;

  //! SolverFactory hook (SolverMHDMuscl.h:65-71)
  static SolverBase *
  create(HydroParams & params, ConfigMap & configMap)
  {
    return new SolverMHDMusclGPU<dim>(params, configMap);
  }

  double
  compute_dt_local() override;
  void
  next_iteration() override;
  void
  next_iteration_impl() override;
  void
  save_solution_impl() override;
  bool
  ok() const override
  {
    return m_ok;
  }
  std::string
  error() const override
  {
    return m_err;
  }

  //! Run up to n iterations from a CUDA graph (no output or logging inside);
  //! returns the number executed.
  int
  run(int n);
  //! Copy the current conservative state to the host (LayoutLeft).
  bool
  copy_state(std::vector<double> & out);

  mhd_ctx * ctx = nullptr;

private:
  void
  sync_time();
  bool        m_ok = false;
  std::string m_err;
};

extern template class SolverMHDMusclGPU<2>;
extern template class SolverMHDMusclGPU<3>;

} // namespace ppkmhd_gb300
