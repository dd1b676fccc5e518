#include "IO_VTK.h"

#include <cstdint>
#include <cstring>
#include <fstream>
#include <sstream>

#include "ppkmhd_gb300.h"

namespace ppkmhd_gb300
{

std::string
save_VTK(const double * U, const HydroParams & params, const ConfigMap & configMap,
         const std::map<int, std::string> & names, int iStep, int dim)
{
  const int   nx = params.nx, ny = params.ny, nz = dim == 3 ? params.nz : 0;
  const int   g = params.ghostWidth;
  const int   isize = params.isize, jsize = params.jsize, ksize = dim == 3 ? params.ksize : 1;
  const std::string outputDir = configMap.getString("output", "outputDir", "./");
  const std::string outputPrefix = configMap.getString("output", "outputPrefix", "output");
  const bool  ascii = configMap.getBool("output", "outputVtkAscii", false);

  std::ostringstream stepNum;
  stepNum.width(7);
  stepNum.fill('0');
  stepNum << iStep;
  const std::string filename = outputDir + "/" + outputPrefix + "_" + stepNum.str() + ".vti";
  std::ofstream out(filename, std::ios::out | std::ios::binary);
  if (!out)
    return "";

  const uint16_t probe = 1;
  const bool     big = *(const uint8_t *)&probe == 0;
  if (ascii)
    out << "<?xml version=\"1.0\"?>\n";
  out << "<VTKFile type=\"ImageData\" version=\"" << (dim == 3 ? "0.1" : "1.0")
      << "\" byte_order=\"" << (big ? "BigEndian" : "LittleEndian")
      << "\" header_type=\"UInt64\">\n";
  out << "  <ImageData WholeExtent=\"0 " << nx << " 0 " << ny << " 0 " << nz << "\" Origin=\""
      << params.xmin << " " << params.ymin << " " << (dim == 3 ? params.zmin : 0) << "\" Spacing=\""
      << params.dx << " " << params.dy << " " << (dim == 3 ? params.dz : 0.0) << "\">\n";
  out << "  <Piece Extent=\"0 " << nx << " 0 " << ny << " 0 " << nz << " \">\n";
  out << "    <PointData>\n";
  out << "    </PointData>\n";
  const int64_t sj = isize, sk = (int64_t)isize * jsize, sv = sk * ksize;
  const int     nvar = params.nbvar;
  const int64_t ncell = (int64_t)nx * ny * (dim == 3 ? params.nz : 1);
  auto          interior = [&](int v, auto && fn) {
    for (int k = (dim == 3 ? g : 0); k < (dim == 3 ? ksize - g : 1); ++k)
      for (int j = g; j < jsize - g; ++j)
        for (int i = g; i < isize - g; ++i)
          fn(U[i + j * sj + k * sk + v * sv]);
  };
  if (ascii)
  {
    out << "    <CellData>\n";
    for (int v = 0; v < nvar; ++v)
    {
      out << "    <DataArray type=\"Float64\" Name=\"" << names.at(v) << "\" format=\"ascii\" >\n";
      interior(v, [&](double x) { out << x << " "; });
      out << "\n    </DataArray>\n";
    }
    out << "    </CellData>\n  </Piece>\n  </ImageData>\n</VTKFile>\n";
  }
  else
  {
    out << "    <CellData>" << std::endl;
    for (int v = 0; v < nvar; ++v)
      out << "     <DataArray type=\"Float64\" Name=\"" << names.at(v)
          << "\" format=\"appended\" offset=\""
          << (uint64_t)v * ncell * sizeof(double) + (uint64_t)v * sizeof(uint64_t) << "\" />"
          << std::endl;
    out << "    </CellData>" << std::endl;
    out << "  </Piece>" << std::endl;
    out << "  </ImageData>" << std::endl;
    out << "  <AppendedData encoding=\"raw\">" << std::endl;
    out << "_";
    const uint64_t nbytes = (uint64_t)ncell * sizeof(double);
    for (int v = 0; v < nvar; ++v)
    {
      out.write((const char *)&nbytes, sizeof nbytes);
      interior(v, [&](double x) { out.write((const char *)&x, sizeof x); });
    }
    out << "  </AppendedData>" << std::endl;
    out << "</VTKFile>" << std::endl;
  }
  return filename;
}

} // namespace ppkmhd_gb300

extern "C"
{

  // The .ini's [output] outputDir / outputPrefix / outputVtkAscii and mesh
  // decide the file; U is the ghost-inclusive LayoutLeft FP64 state; the
  // variable names are SolverBase's (SolverBase.cpp:48-55 of the reference).
  int
  mhd_write_vtk(const char * ini_text, const double * U, int iStep, char * path, size_t pathlen)
  {
    if (!ini_text || !U || iStep < 0)
      return MHD_ERR_INVALID_ARG;
    const ConfigMap map(ini_text, (int)std::strlen(ini_text));
    if (map.ParseError() != 0)
      return MHD_ERR_PARSE;
    ppkmhd_gb300::HydroParams params;
    params.setup(map);
    const std::map<int, std::string> names = { { 0, "rho" },    { 1, "energy" }, { 2, "rho_vx" },
                                               { 3, "rho_vy" }, { 4, "rho_vz" }, { 5, "bx" },
                                               { 6, "by" },     { 7, "bz" } };
    const int         dim = params.dimType == ppkmhd_gb300::THREE_D ? 3 : 2;
    const std::string file = ppkmhd_gb300::save_VTK(U, params, map, names, iStep, dim);
    if (file.empty())
      return MHD_ERR_INVALID_ARG;
    if (path && pathlen)
    {
      std::strncpy(path, file.c_str(), pathlen - 1);
      path[pathlen - 1] = '\0';
    }
    return MHD_OK;
  }

} // extern "C"
