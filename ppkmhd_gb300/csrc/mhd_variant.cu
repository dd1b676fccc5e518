// One arithmetic variant of the solver core.  Compiled three times by
// ppkmhd_gb300/build.py with
//   -DMHD_VARIANT_TAG=v_f64x -DMHD_REAL=double -DMHD_FACTORY=create_core_f64x --fmad=false
//   -DMHD_VARIANT_TAG=v_f64  -DMHD_REAL=double -DMHD_FACTORY=create_core_f64
//   -DMHD_VARIANT_TAG=v_f32  -DMHD_REAL=float  -DMHD_FACTORY=create_core_f32
// Each build lives in its own inline namespace so the three sets of kernels
// coexist in one shared library.
#include "mhd_solver.cuh"

#if !defined(MHD_VARIANT_TAG) || !defined(MHD_REAL) || !defined(MHD_FACTORY)
#  error "mhd_variant.cu needs MHD_VARIANT_TAG, MHD_REAL and MHD_FACTORY"
#endif

namespace mhd
{

SolverCore *
MHD_FACTORY(const mhd_params & p, std::string & err)
{
  auto * s = new SolverImpl<MHD_REAL>();
  const int rc = s->setup(p);
  if (rc != MHD_OK)
  {
    err = s->err;
    delete s;
    return nullptr;
  }
  return s;
}

} // namespace mhd
