// Command-line driver with the flow of ppkMHD's main (src/main.cpp:51-189):
// read the .ini, set up HydroParams, create the solver through the factory,
// run the time loop, print the timer summary and the Mcell-updates/s line
// (solver_utils.h:17-60).  Between log/output points the loop advances with
// whole CUDA-graph runs instead of one host round trip per iteration.
#include <cstdio>
#include <iostream>
#include <string>

#include "ConfigMap.h"
#include "HydroParams.h"
#include "SolverFactory.h"
#include "SolverMHDMusclGPU.h"

using namespace ppkmhd_gb300;

int
main(int argc, char * argv[])
{
  if (argc < 2)
  {
    std::cerr << "usage: " << argv[0] << " <file.ini>\n";
    return 1;
  }
  ConfigMap configMap(argv[1]);
  if (configMap.ParseError() < 0)
  {
    std::cerr << "cannot read " << argv[1] << "\n";
    return 1;
  }
  HydroParams params;
  params.setup(configMap);
  const std::string solver_name = configMap.getString("run", "solver_name", "Unknown");
  SolverBase *      solver = SolverFactory::Instance().create(solver_name, params, configMap);
  if (!solver)
    return 1;

  if (params.nOutput != 0)
    solver->save_solution();
  std::cout << "Start computation....\n";
  solver->timers[TIMER_TOTAL]->start();
  auto * gpu2 = dynamic_cast<SolverMHDMusclGPU<2> *>(solver);
  auto * gpu3 = dynamic_cast<SolverMHDMusclGPU<3> *>(solver);
  while (!solver->finished())
  {
    const bool io_now = (solver->m_nlog > 0 && solver->m_iteration % solver->m_nlog == 0) ||
                        (params.enableOutput && solver->should_save_solution());
    if (io_now || (!gpu2 && !gpu3))
    {
      solver->next_iteration();
      continue;
    }
    // advance to the next logging iteration in one graph replay
    int chunk = solver->m_nlog > 0 ? solver->m_nlog - solver->m_iteration % solver->m_nlog : 64;
    if (params.enableOutput)
      chunk = 1; // output cadence depends on t, which is only known step by step
    const int done = gpu2 ? gpu2->run(chunk) : gpu3->run(chunk);
    if (done == 0)
      break;
  }
  solver->timers[TIMER_TOTAL]->stop();
  if (params.nOutput != 0)
    solver->save_solution();
  std::printf("final time is %f\n", solver->m_t);

  const double t_tot = solver->timers[TIMER_TOTAL]->elapsed();
  const double t_comp = solver->timers[TIMER_NUM_SCHEME]->elapsed();
  const double t_io = solver->timers[TIMER_IO]->elapsed();
  std::printf("total       time : %5.3f secondes\n", t_tot);
  std::printf("godunov     time : %5.3f secondes %5.2f%%\n", t_comp, 100 * t_comp / t_tot);
  std::printf("io          time : %5.3f secondes %5.2f%%\n", t_io, 100 * t_io / t_tot);
  std::printf("Perf             : %5.3f number of Mcell-updates/s\n",
              solver->m_iteration * (double)solver->m_nCells / t_tot * 1e-6);
  delete solver;
  return 0;
}
