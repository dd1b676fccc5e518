// One arithmetic variant of the hydro-only MUSCL solver core.  Compiled three
// times by ppkmhd_gb300/build.py, like mhd_variant.cu:
//   -DMHD_VARIANT_TAG=v_f64x -DMHD_REAL=double -DMHD_HYDRO_FACTORY=create_hydro_core_f64x --fmad=false
//   -DMHD_VARIANT_TAG=v_f64  -DMHD_REAL=double -DMHD_HYDRO_FACTORY=create_hydro_core_f64
//   -DMHD_VARIANT_TAG=v_f32  -DMHD_REAL=float  -DMHD_HYDRO_FACTORY=create_hydro_core_f32
#include "hydro_solver.cuh"

#if !defined(MHD_VARIANT_TAG) || !defined(MHD_REAL) || !defined(MHD_HYDRO_FACTORY)
#  error "hydro_variant.cu needs MHD_VARIANT_TAG, MHD_REAL and MHD_HYDRO_FACTORY"
#endif

namespace mhd
{

SolverCore *
MHD_HYDRO_FACTORY(const mhd_params & p, std::string & err)
{
  auto * s = new hydro::HydroImpl<MHD_REAL>();
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
