// The ensemble engine of one arithmetic variant.  Compiled three times by
// ppkmhd_gb300/build.py, beside mhd_variant.cu and with the same
// MHD_VARIANT_TAG / MHD_REAL / fmad settings, and
//   -DMHD_ENSEMBLE_FACTORY=create_ensemble_f64x | create_ensemble_f64 | create_ensemble_f32
#include "mhd_ensemble.cuh"

#if !defined(MHD_VARIANT_TAG) || !defined(MHD_REAL) || !defined(MHD_ENSEMBLE_FACTORY)
#  error "mhd_ensemble.cu needs MHD_VARIANT_TAG, MHD_REAL and MHD_ENSEMBLE_FACTORY"
#endif

namespace mhd
{

EnsembleCore *
MHD_ENSEMBLE_FACTORY(const mhd_params * p, int n, std::string & err)
{
  auto * s = new EnsembleImpl<MHD_REAL>();
  const int rc = s->setup(p, n);
  if (rc != MHD_OK)
  {
    err = s->err;
    delete s;
    return nullptr;
  }
  return s;
}

} // namespace mhd
