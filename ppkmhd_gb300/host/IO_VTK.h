// VTK ImageData (.vti) output with the layout of ppkMHD's save_VTK_2D /
// save_VTK_3D (src/utils/io/IO_VTK.cpp:24-410): interior cells only, one
// cell-data array per variable, raw appended binary (UInt64 byte count
// before each array, x fastest) or ASCII, file name
// outputDir/outputPrefix_NNNNNNN.vti.
#pragma once

#include <map>
#include <string>

#include "ConfigMap.h"
#include "HydroParams.h"

namespace ppkmhd_gb300
{

//! U: LayoutLeft FP64 state with ghosts.  Values are written in FP64
//! (Float64).  Returns the file name written, or "" on failure.
std::string
save_VTK(const double * U, const HydroParams & params, const ConfigMap & configMap,
         const std::map<int, std::string> & names, int iStep, int dim);

} // namespace ppkmhd_gb300
