// Initial conditions of the MHD problems, in FP64 on the host, LayoutLeft
// with ghost cells (U[i + isize*(j + jsize*(k + ksize*v))]).  Each follows
// the reference's init functor for [hydro] problem (dispatch of
// SolverMHDMuscl<dim>::init, SolverMHDMuscl.h:649-710; unknown names fall
// back to Orszag-Tang), operation for operation so that the initial state
// is bitwise the reference's:
//   orszag_tang       MHDInitFunctors2D.h:241-389, 3D:264-415
//   blast             MHDInitFunctors2D.h:144-236, 3D:155-260
//   implode           MHDInitFunctors2D.h:36-139, 3D:34-150
//   kelvin_helmholtz  MHDInitFunctors2D.h:394-583, 3D:420-622 (sine seeds;
//                     the random seed needs Kokkos' own generator and is
//                     rejected by validation)
//   rotor             MHDInitFunctors2D.h:588-710, 3D:627-754
//   field_loop        MHDInitFunctors2D.h:715-945, 3D:759-1029
//   wave              MHDInitFunctors3D.h:1034-1314 (the 2D functor leaves U
//                     untouched, MHDInitFunctors2D.h:950-986)
// The problem parameters arrive in mhd_params::problem_real/problem_int in
// the layout documented in ppkmhd_gb300.h (filled by HydroParams::
// to_mhd_params from the reference's parameter structs,
// src/shared/problems/*Params.h).
#include <cmath>
#include <cstdint>
#include <vector>

#include "mhd_core.h"

namespace mhd
{
namespace
{

enum
{
  ID = 0,
  IP = 1,
  IU = 2,
  IV = 3,
  IW = 4,
  IA = 5,
  IB = 6,
  IC = 7
};

constexpr double kPi = 3.141592653589793238462643383279502884;

struct Mesh
{
  int     g, nx, ny, nz, isize, jsize, ksize, dim;
  int64_t sj, sk, sv;
  double  xmin, xmax, ymin, ymax, zmin, zmax, dx, dy, dz;
  explicit Mesh(const mhd_params & p)
  {
    dim = p.dim;
    g = p.ghost;
    nx = p.nx;
    ny = p.ny;
    nz = p.dim == 3 ? p.nz : 1;
    isize = nx + 2 * g;
    jsize = ny + 2 * g;
    ksize = p.dim == 3 ? nz + 2 * g : 1;
    sj = isize;
    sk = (int64_t)isize * jsize;
    sv = sk * ksize;
    xmin = p.xmin;
    xmax = p.xmax;
    ymin = p.ymin;
    ymax = p.ymax;
    zmin = p.zmin;
    zmax = p.zmax;
    dx = (xmax - xmin) / nx;
    dy = (ymax - ymin) / ny;
    dz = p.dim == 3 ? (zmax - zmin) / nz : 1.0;
  }
  int64_t
  at(int i, int j, int k = 0) const
  {
    return i + j * sj + k * sk;
  }
  double
  x(int i) const
  {
    return xmin + dx / 2 + (i - g) * dx;
  }
  double
  y(int j) const
  {
    return ymin + dy / 2 + (j - g) * dy;
  }
  double
  z(int k) const
  {
    return zmin + dz / 2 + (k - g) * dz;
  }
  bool
  interior(int i, int j, int k) const
  {
    return i >= g && i < isize - g && j >= g && j < jsize - g &&
           (dim == 2 || (k >= g && k < ksize - g));
  }
};

inline double
sqr(double x)
{
  return x * x;
}

void
orszag_tang(const mhd_params & p, const Mesh & m, double * U)
{
  const double TWOPI = 2 * kPi;
  const double gamma0 = p.gamma0;
  double       B0, p0, p0e;
  if (p.dim == 2)
  {
    B0 = 1.0 / std::sqrt(2 * TWOPI);
    p0 = gamma0 / (2 * TWOPI);
    p0e = gamma0 / (2.0 * (4.0 * std::asin(1.0)));
  }
  else
  {
    B0 = 1.0 / std::sqrt(4 * kPi);
    p0 = gamma0 / (4 * kPi);
    p0e = p0;
  }
  const double  d0 = gamma0 * p0;
  const double  v0 = 1.0;
  const int64_t sv = m.sv;
#pragma omp parallel for schedule(static)
  for (int k = 0; k < m.ksize; ++k)
  {
    double zfac = 1.0;
    if (p.dim == 3)
      zfac = std::cos(2 * TWOPI * p.ot_kt * (m.z(k) - m.zmin) / (m.zmax - m.zmin));
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double  xPos = m.x(i), yPos = m.y(j);
        const int64_t c = m.at(i, j, k);
        U[c + ID * sv] = d0;
        U[c + IU * sv] = -d0 * v0 * std::sin(yPos * TWOPI);
        U[c + IV * sv] = d0 * v0 * std::sin(xPos * TWOPI);
        U[c + IW * sv] = 0.0;
        if (p.dim == 2)
        {
          U[c + IA * sv] = -B0 * std::sin(yPos * TWOPI);
          U[c + IB * sv] = B0 * std::sin(2.0 * xPos * TWOPI);
        }
        else
        {
          U[c + IA * sv] = -B0 * zfac * std::sin(yPos * TWOPI);
          U[c + IB * sv] = B0 * zfac * std::sin(2.0 * xPos * TWOPI);
        }
        U[c + IC * sv] = 0.0;
      }
  }
#pragma omp parallel for schedule(static)
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize - 1; ++j)
      for (int i = 0; i < m.isize - 1; ++i)
      {
        const int64_t c = m.at(i, j, k);
        const double  bxs = U[c + IA * sv] + U[c + 1 + IA * sv];
        const double  bys = U[c + IB * sv] + U[c + m.sj + IB * sv];
        U[c + IP * sv] = p0e / (gamma0 - 1.0) +
                         0.5 * (U[c + IU * sv] * U[c + IU * sv] / U[c + ID * sv] +
                                U[c + IV * sv] * U[c + IV * sv] / U[c + ID * sv] +
                                0.25 * (bxs * bxs) + 0.25 * (bys * bys));
      }
}

// problem_real: radius, center x, y, z, density in, out, pressure in, out
void
blast(const mhd_params & p, const Mesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   radius2 = r[0] * r[0];
  const double   g1 = p.gamma0 - 1.0;
  const int64_t  sv = m.sv;
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double x = m.x(i), y = m.y(j);
        double       d2 = (x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]);
        if (p.dim == 3)
        {
          const double z = m.z(k);
          d2 = (x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]) + (z - r[3]) * (z - r[3]);
        }
        const bool    in = d2 < radius2;
        const int64_t c = m.at(i, j, k);
        U[c + ID * sv] = in ? r[4] : r[5];
        U[c + IU * sv] = 0.0;
        U[c + IV * sv] = 0.0;
        U[c + IW * sv] = 0.0;
        U[c + IA * sv] = 0.5;
        U[c + IB * sv] = 0.5;
        U[c + IC * sv] = 0.5;
        U[c + IP * sv] = (in ? r[6] : r[7]) / g1 + 0.5 * (sqr(0.5) + sqr(0.5) + sqr(0.5));
      }
}

// problem_real: outer rho, p, u, v, w, Bx, By, Bz, inner rho, p, u, v, w,
// Bx, By, Bz; problem_int[0] = shape_region
void
implode(const mhd_params & p, const Mesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   g1 = p.gamma0 - 1.0;
  const int64_t  sv = m.sv;
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double x = m.x(i), y = m.y(j);
        bool         outer;
        if (p.dim == 2)
          outer = p.problem_int[0] == 1 ? (x + y > 0.5 && x + y < 2.5)
                                        : (x + y > (m.xmin + m.xmax) / 2. + m.ymin);
        else
        {
          const double z = m.z(k);
          outer = p.problem_int[0] == 1 ? (x + y + z > 0.5 && x + y + z < 2.5)
                                        : (x + y + z > (m.xmin + m.xmax) / 2. + m.ymin + m.zmin);
        }
        const double * s = outer ? r : r + 8;
        const int64_t  c = m.at(i, j, k);
        // the reference stores the velocities (not the momenta) in IU..IW
        U[c + ID * sv] = s[0];
        if (p.dim == 2)
          U[c + IP * sv] =
            s[1] / g1 + 0.5 * s[0] * (s[2] * s[2] + s[3] * s[3]) + 0.5 * (s[5] * s[5] + s[6] * s[6]);
        else
          U[c + IP * sv] = s[1] / g1 + 0.5 * s[0] * (s[2] * s[2] + s[3] * s[3] + s[4] * s[4]) +
                           0.5 * (s[5] * s[5] + s[6] * s[6] + s[7] * s[7]);
        U[c + IU * sv] = s[2];
        U[c + IV * sv] = s[3];
        U[c + IW * sv] = p.dim == 2 ? 0.0 : s[4];
        U[c + IA * sv] = s[5];
        U[c + IB * sv] = s[6];
        U[c + IC * sv] = p.dim == 2 ? 0.0 : s[7];
      }
}

// problem_real: d_in, d_out, pressure, vflow_in, vflow_out, amplitude, w0,
// delta; problem_int: perturbation_sine, perturbation_sine_robertson, mode
void
kelvin_helmholtz(const mhd_params & p, const Mesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   d_in = r[0], d_out = r[1], pressure = r[2], vin = r[3], vout = r[4];
  const double   w0 = r[6], delta = r[7];
  const int      n = p.problem_int[2];
  const double   g1 = p.gamma0 - 1.0;
  const int64_t  sv = m.sv;
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double  x = m.x(i), y = m.y(j);
        const int64_t c = m.at(i, j, k);
        double        d, u, v, w = 0.0;
        const double  bx = 0.5, by = 0.0, bz = 0.0;
        if (p.dim == 2)
        {
          if (p.problem_int[1]) // Robertson et al. smooth profile
          {
            const double ramp = 1.0 / (1.0 + std::exp(2 * (y - 0.25) / delta)) +
                                1.0 / (1.0 + std::exp(2 * (0.75 - y) / delta));
            d = d_in + ramp * (d_out - d_in);
            u = vin + ramp * (vout - vin);
          }
          else
          {
            const bool inner = y >= 0.25 && y <= 0.75;
            d = inner ? d_in : d_out;
            u = inner ? vin : vout;
          }
          v = w0 * std::sin(n * kPi * x);
          U[c + ID * sv] = d;
          U[c + IU * sv] = d * u;
          U[c + IV * sv] = d * v;
          U[c + IA * sv] = bx;
          U[c + IB * sv] = by;
          U[c + IC * sv] = bz;
          U[c + IP * sv] = pressure / g1 + 0.5 * d * (u * u + v * v) + 0.5 * (bx * bx + by * by + bz * bz);
        }
        else
        {
          const double z = m.z(k);
          if (p.problem_int[1])
          {
            const double ramp = 1.0 / (1.0 + std::exp(2 * (z - 0.25) / delta)) +
                                1.0 / (1.0 + std::exp(2 * (0.75 - z) / delta));
            d = d_in + ramp * (d_out - d_in);
            u = vin + ramp * (vout - vin);
            v = vin / 2 + ramp * (vout / 2 - vin / 2);
            w = w0 * std::sin(n * kPi * x) * std::sin(n * kPi * y);
          }
          else
          {
            const bool inner = z >= 0.25 && z <= 0.75;
            d = inner ? d_in : d_out;
            u = inner ? vin : vout;
            v = 0;
            w = w0 * std::sin(n * kPi * x);
          }
          U[c + ID * sv] = d;
          U[c + IU * sv] = d * u;
          U[c + IV * sv] = d * v;
          U[c + IW * sv] = d * w;
          U[c + IA * sv] = bx;
          U[c + IB * sv] = by;
          U[c + IC * sv] = bz;
          U[c + IP * sv] =
            pressure / g1 + 0.5 * d * (u * u + v * v + w * w) + 0.5 * (bx * bx + by * by + bz * bz);
        }
      }
}

// problem_real: r0, r1, u0, p0, b0
void
rotor(const mhd_params & p, const Mesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   r0 = r[0], r1 = r[1], u0 = r[2], p0 = r[3], b0 = r[4];
  const double   xc = (m.xmax + m.xmin) / 2, yc = (m.ymax + m.ymin) / 2;
  const int64_t  sv = m.sv;
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double  x = m.x(i), y = m.y(j);
        const double  rr = std::sqrt((x - xc) * (x - xc) + (y - yc) * (y - yc));
        const double  f_r = (r1 - rr) / (r1 - r0);
        const int64_t c = m.at(i, j, k);
        double        d, mu, mv;
        if (p.dim == 2) // momenta
        {
          if (rr <= r0)
          {
            d = 10.0;
            mu = -d * f_r * u0 * (y - yc) / r0;
            mv = d * f_r * u0 * (x - xc) / r0;
          }
          else if (rr <= r1)
          {
            d = 1 + 9 * f_r;
            mu = -d * f_r * u0 * (y - yc) / rr;
            mv = d * f_r * u0 * (x - xc) / rr;
          }
          else
          {
            d = 1.0;
            mu = 0.0;
            mv = 0.0;
          }
        }
        else // the reference's 3D functor stores velocities in IU, IV
        {
          if (rr <= r0)
          {
            d = 10.0;
            mu = -u0 * (y - yc) / r0;
            mv = u0 * (x - xc) / r0;
          }
          else if (rr <= r1)
          {
            d = 1 + 9 * f_r;
            mu = -f_r * u0 * (y - yc) / rr;
            mv = f_r * u0 * (x - xc) / rr;
          }
          else
          {
            d = 1.0;
            mu = 0.0;
            mv = 0.0;
          }
        }
        U[c + ID * sv] = d;
        U[c + IU * sv] = mu;
        U[c + IV * sv] = mv;
        U[c + IW * sv] = 0.0;
        U[c + IA * sv] = b0;
        U[c + IB * sv] = 0.0;
        U[c + IC * sv] = 0.0;
        if (p.dim == 2)
          U[c + IP * sv] = p0 / (p.gamma0 - 1.0) + 0.5 * (mu * mu + mv * mv + 0.0 * 0.0) / d +
                           0.5 * (b0 * b0);
        else
          U[c + IP * sv] = p0 / (p.gamma0 - 1.0) + (mu * mu + mv * mv + 0.0 * 0.0) / 2 / d + (b0 * b0) / 2;
      }
}

// problem_real: radius, density_in, amplitude, vflow
void
field_loop(const mhd_params & p, const Mesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   radius = r[0], density_in = r[1], amplitude = r[2], vflow = r[3];
  const int64_t  sv = m.sv;
  // edge vector potential Az (2D) / A (3D, only the z component is non-zero)
  std::vector<double> Az((size_t)m.sv, 0.0);
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double x = m.x(i), y = m.y(j);
        const double rr = std::sqrt(x * x + y * y);
        if (rr < radius)
          Az[m.at(i, j, k)] = amplitude * (radius - rr);
      }
  const double cos_theta = 2.0 / std::sqrt(5.0);
  const double sin_theta = std::sqrt(1 - cos_theta * cos_theta);
  const double diag = std::sqrt(1.0 * (p.nx * p.nx + p.ny * p.ny + p.nz * p.nz));
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        if (!m.interior(i, j, k))
          continue;
        const double  x = m.x(i), y = m.y(j);
        const double  rr = std::sqrt(x * x + y * y);
        const int64_t c = m.at(i, j, k);
        const double  d = rr < radius ? density_in : 1.0;
        U[c + ID * sv] = d;
        U[c + IU * sv] = d * vflow * cos_theta;
        U[c + IV * sv] = d * vflow * sin_theta;
        if (p.dim == 2)
        {
          U[c + IW * sv] = d * vflow * p.nz / diag;
          U[c + IA * sv] = (Az[c + m.sj] - Az[c]) / m.dy;
          U[c + IB * sv] = -(Az[c + 1] - Az[c]) / m.dx;
          U[c + IC * sv] = 0.0;
        }
        else
        {
          // A_x = A_y = 0
          U[c + IW * sv] = d * vflow;
          U[c + IA * sv] = (Az[c + m.sj] - Az[c]) / m.dy - (0.0 - 0.0) / m.dz;
          U[c + IB * sv] = (0.0 - 0.0) / m.dz - (Az[c + 1] - Az[c]) / m.dx;
          U[c + IC * sv] = (0.0 - 0.0) / m.dx - (0.0 - 0.0) / m.dy;
        }
      }
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        if (!m.interior(i, j, k))
          continue;
        const int64_t c = m.at(i, j, k);
        const double  kin = 0.5 *
                           (U[c + IU * sv] * U[c + IU * sv] + U[c + IV * sv] * U[c + IV * sv] +
                            (p.dim == 3 ? U[c + IW * sv] * U[c + IW * sv] : 0.0)) /
                           U[c + ID * sv];
        double mag = 0.25 * sqr(U[c + IA * sv] + U[c + 1 + IA * sv]) +
                     0.25 * sqr(U[c + IB * sv] + U[c + m.sj + IB * sv]);
        if (p.dim == 3)
          mag += 0.25 * sqr(U[c + IC * sv] + U[c + m.sk + IC * sv]);
        U[c + IP * sv] = 1.0 / (p.gamma0 - 1.0) + 0.5 * mag + kin;
      }
}

// problem_real: amplitude, V0, rev[7], d0, p0, sin_a2, cos_a2, sin_a3,
// cos_a3, dby, dbz, bx0, by0, bz0, k_par (the fields of WaveParams)
void
wave(const mhd_params & p, const Mesh & m, double * U)
{
  if (p.dim != 3)
    return; // the reference's 2D wave initialiser does nothing
  const double * r = p.problem_real;
  const double   amp = r[0], V0 = r[1];
  const double * rev = r + 2;
  const double   d0 = r[9], p0 = r[10], sin_a2 = r[11], cos_a2 = r[12], sin_a3 = r[13],
               cos_a3 = r[14], dby = r[15], dbz = r[16], bx0 = r[17], by0 = r[18], bz0 = r[19],
               k_par = r[20];
  const int64_t sv = m.sv;
  std::vector<double> A((size_t)m.sv * 3, 0.0);
  auto potential = [&](double x1, double x2, double x3, double & Ay, double & Az) {
    const double tmpx = x1 * cos_a2 * cos_a3 + x2 * cos_a2 * sin_a3 + x3 * sin_a2;
    const double tmpy = -x1 * sin_a3 + x2 * cos_a3;
    Ay = bz0 * tmpx - (dbz / k_par) * std::cos(k_par * tmpx);
    Az = -by0 * tmpx + (dby / k_par) * std::cos(k_par * tmpx) + bx0 * tmpy;
  };
  for (int k = 0; k < m.ksize; ++k)
    for (int j = 0; j < m.jsize; ++j)
      for (int i = 0; i < m.isize; ++i)
      {
        const double  x = m.x(i), y = m.y(j), z = m.z(k);
        const int64_t c = m.at(i, j, k);
        double        Ay, Az;
        potential(x, y - m.dy / 2, z - m.dz / 2, Ay, Az);
        A[c] = -Ay * sin_a3 - Az * sin_a2 * cos_a3;
        potential(x - m.dx / 2, y, z - m.dz / 2, Ay, Az);
        A[c + sv] = Ay * cos_a3 - Az * sin_a2 * sin_a3;
        potential(x - m.dx / 2, y - m.dy / 2, z, Ay, Az);
        A[c + 2 * sv] = Az * cos_a2;
      }
  const int g = m.g;
  for (int k = g - 1; k < m.ksize - g + 1; ++k)
    for (int j = g - 1; j < m.jsize - g + 1; ++j)
      for (int i = g - 1; i < m.isize - g + 1; ++i)
      {
        const int64_t c = m.at(i, j, k);
        const double *Ax = A.data(), *Ay = A.data() + sv, *Az = A.data() + 2 * sv;
        U[c + IA * sv] = (Az[c + m.sj] - Az[c]) / m.dy - (Ay[c + m.sk] - Ay[c]) / m.dz;
        U[c + IB * sv] = (Ax[c + m.sk] - Ax[c]) / m.dz - (Az[c + 1] - Az[c]) / m.dx;
        U[c + IC * sv] = (Ay[c + 1] - Ay[c]) / m.dx - (Ax[c + m.sj] - Ax[c]) / m.dy;
      }
  for (int k = g; k < m.ksize - g; ++k)
    for (int j = g; j < m.jsize - g; ++j)
      for (int i = g; i < m.isize - g; ++i)
      {
        const double  x = m.x(i), y = m.y(j), z = m.z(k);
        const int64_t c = m.at(i, j, k);
        const double  X = cos_a2 * (x * cos_a3 + y * sin_a3) + z * sin_a2;
        const double  sn = std::sin(k_par * X);
        const double  Mx = d0 * V0 + amp * sn * rev[1];
        const double  My = amp * sn * rev[2];
        const double  Mz = amp * sn * rev[3];
        U[c + ID * sv] = d0 + amp * sn * rev[0];
        U[c + IU * sv] = Mx * cos_a2 * cos_a3 - My * sin_a3 - Mz * sin_a2 * cos_a3;
        U[c + IV * sv] = Mx * cos_a2 * sin_a3 + My * cos_a3 - Mz * sin_a2 * sin_a3;
        U[c + IW * sv] = Mx * sin_a2 + Mz * cos_a2;
        U[c + IP * sv] = p0 / (p.gamma0 - 1.0) + 0.5 * d0 * V0 * V0 +
                         0.5 * (bx0 * bx0 + by0 * by0 + bz0 * bz0) + amp * sn * rev[4];
      }
}

} // namespace

void
init_problem_host(const mhd_params & p, double * U)
{
  if (p.solver == MHD_SOLVER_HYDRO_MUSCL)
    return init_hydro_problem_host(p, U);
  const Mesh m(p);
  switch (p.problem)
  {
  case MHD_PROBLEM_BLAST:
    return blast(p, m, U);
  case MHD_PROBLEM_IMPLODE:
    return implode(p, m, U);
  case MHD_PROBLEM_KELVIN_HELMHOLTZ:
    return kelvin_helmholtz(p, m, U);
  case MHD_PROBLEM_ROTOR:
    return rotor(p, m, U);
  case MHD_PROBLEM_FIELD_LOOP:
    return field_loop(p, m, U);
  case MHD_PROBLEM_WAVE:
    return wave(p, m, U);
  default:
    return orszag_tang(p, m, U);
  }
}

void
init_orszag_tang_host(const mhd_params & p, double * U)
{
  orszag_tang(p, Mesh(p), U);
}

} // namespace mhd
