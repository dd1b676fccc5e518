#include "SolverMHDMusclGPU.h"

#include <cstdio>
#include <iostream>

#include "IO_VTK.h"

namespace ppkmhd_gb300
{

template <int dim>
SolverMHDMusclGPU<dim>::SolverMHDMusclGPU(HydroParams & p, ConfigMap & cfg)
  : SolverBase(p, cfg)
{
  const int         precision = (int)cfg.getInteger("gb300", "precision", 64);
  const std::string mode = cfg.getString("gb300", "fp_mode", "fast");
  mhd_params        mp = p.to_mhd_params(cfg, precision, mode == "exact" ? MHD_FP_EXACT : MHD_FP_FAST);
  int               rc = mhd_create(&mp, &ctx);
  // restart from a checkpoint (SolverMHDMuscl<dim>::init_restart,
  // SolverMHDMuscl.h:613-643; keys of SolverBase.cpp:130-132)
  const bool restart = cfg.getInteger("run", "restart_enabled", 0) != 0;
  if (rc == MHD_OK && restart)
  {
    const std::string file = cfg.getString("run", "restart_filename", "");
    const bool        reset = cfg.getBool("run", "restart_reset_totaltime", false);
    // restart_upscale: the file holds half the resolution (IO_HDF5.h:1603-1694)
    const bool        upscale = cfg.getBool("run", "restart_upscale", false);
    rc = upscale ? mhd_checkpoint_load_upscaled(ctx, file.c_str(), reset ? 1 : 0, &m_times_saved)
                 : mhd_checkpoint_load(ctx, file.c_str(), reset ? 1 : 0, &m_times_saved);
    if (rc == MHD_OK)
      std::cout << "### This is a restarted run ! ###\n";
  }
  else if (rc == MHD_OK)
    rc = mhd_init_problem(ctx); // init + boundaries + U2 = U + primitives + dt
  if (rc != MHD_OK)
  {
    m_err = ctx ? mhd_last_error(ctx) : "mhd_create failed";
    return;
  }
  m_nCells = dim == 2 ? (long long)p.isize * p.jsize : (long long)p.isize * p.jsize * p.ksize;
  m_nDofsPerCell = 1;
  sync_time();
  m_ok = true;
  std::cout << "##########################\n";
  std::cout << "Solver is " << m_solver_name << " (GB300 back-end, "
            << (precision == 32 ? "FP32" : "FP64") << ")\n";
  std::cout << "Problem (init condition) is " << m_problem_name << "\n";
  std::cout << "##########################\n";
  p.print();
}

template <int dim>
SolverMHDMusclGPU<dim>::~SolverMHDMusclGPU()
{
  if (ctx)
    mhd_destroy(ctx);
}

template <int dim>
void
SolverMHDMusclGPU<dim>::sync_time()
{
  double t = 0, dt = 0;
  int    it = 0;
  if (mhd_time(ctx, &t, &dt, &it) == MHD_OK)
  {
    m_t = t;
    m_dt = dt;
    m_iteration = it;
  }
}

template <int dim>
double
SolverMHDMusclGPU<dim>::compute_dt_local()
{
  // the CFL dt of the current state from the device reduction (already
  // clipped to tEnd, which SolverBase::compute_dt does again); every
  // iteration recomputes it on the device
  double dt = 0.0;
  if (mhd_compute_dt(ctx, &dt) == MHD_OK)
    return dt;
  sync_time();
  return m_dt;
}

template <int dim>
void
SolverMHDMusclGPU<dim>::next_iteration_impl()
{
  // SolverMHDMuscl.h:745-784
  if (m_nlog > 0 && m_iteration % m_nlog == 0)
    std::printf("time step=%7d (dt=% 10.8f t=% 10.8f)\n", m_iteration, m_dt, m_t);
  if (params.enableOutput && should_save_solution())
  {
    std::cout << "Output results at time t=" << m_t << " step " << m_iteration << " dt=" << m_dt
              << std::endl;
    save_solution();
  }
  timers[TIMER_NUM_SCHEME]->start();
  mhd_step(ctx);
}

template <int dim>
void
SolverMHDMusclGPU<dim>::next_iteration()
{
  next_iteration_impl();
  sync_time(); // iteration and t were advanced on the device
  timers[TIMER_NUM_SCHEME]->stop();
}

template <int dim>
int
SolverMHDMusclGPU<dim>::run(int n)
{
  int done = 0;
  timers[TIMER_NUM_SCHEME]->start();
  mhd_run(ctx, n, &done);
  timers[TIMER_NUM_SCHEME]->stop();
  sync_time();
  return done;
}

template <int dim>
bool
SolverMHDMusclGPU<dim>::copy_state(std::vector<double> & out)
{
  int s[4];
  mhd_sizes(ctx, s);
  const size_t n = (size_t)s[0] * s[1] * s[2] * s[3];
  out.resize(n);
  if (params.settings.gamma0 > 0 && mhd_get_state(ctx, out.data(), MHD_LAYOUT_LEFT, 8) == MHD_OK)
    return true;
  // FP32 context: read floats and widen
  std::vector<float> f(n);
  if (mhd_get_state(ctx, f.data(), MHD_LAYOUT_LEFT, 4) != MHD_OK)
    return false;
  for (size_t q = 0; q < n; ++q)
    out[q] = f[q];
  return true;
}

template <int dim>
void
SolverMHDMusclGPU<dim>::save_solution_impl()
{
  timers[TIMER_IO]->start();
  std::vector<double> U;
  if (copy_state(U))
    save_VTK(U.data(), params, configMap, m_variables_names, m_times_saved, dim);
  // restartable checkpoint beside each output ([gb300] checkpoint = true)
  if (configMap.getBool("gb300", "checkpoint", false))
  {
    char num[16];
    std::snprintf(num, sizeof num, "%07d", m_times_saved);
    const std::string file = configMap.getString("output", "outputDir", "./") + "/" +
                             configMap.getString("output", "outputPrefix", "output") + "_" + num +
                             ".ckpt";
    if (mhd_checkpoint_save(ctx, file.c_str(), m_times_saved) != MHD_OK)
      std::cerr << "checkpoint: " << mhd_last_error(ctx) << "\n";
  }
  timers[TIMER_IO]->stop();
}

template class SolverMHDMusclGPU<2>;
template class SolverMHDMusclGPU<3>;

} // namespace ppkmhd_gb300
