// Initial conditions of the hydro-only MUSCL solver's problems, in FP64 on
// the host, LayoutLeft with ghost cells (U[i + isize*(j + jsize*(k +
// ksize*v))], dim + 2 variables).  Each follows the reference's init functor
// for [hydro] problem (dispatch of SolverHydroMuscl<dim>::init,
// SolverHydroMuscl.cpp:110-250; unknown names fall back to implode),
// operation for operation, so that the initial state is bitwise the
// reference's (host libm for exp, sin, cos, atan2, log, pow):
//   implode            HydroInitFunctors2D.h:35-124, 3D:76-160 (the momentum
//                      slots hold the velocities, as the reference writes)
//   blast              HydroInitFunctors2D.h:129-212, 3D:165-250
//   kelvin_helmholtz   HydroInitFunctors2D.h:216-348, 3D:255-420 (the
//                      Robertson seed; the random seed is rejected)
//   gresho_vortex      HydroInitFunctors2D.h:352-448, 3D:425-510
//   four_quadrant      HydroInitFunctors2D.h:453-565 with
//                      SolverHydroMuscl.cpp:60-82 and the Lax-Liu states of
//                      initRiemannConfig2d.h (2D)
//   isentropic_vortex  HydroInitFunctors2D.h:570-663 (2D)
//   rayleigh_taylor    HydroInitFunctors2D.h:668-787, 3D:520-640
//   rising_bubble      HydroInitFunctors2D.h:795-902, 3D:645-760
//   disk               HydroInitFunctors2D.h:907-1060, 3D (with the
//                      point-source gravity field, init_hydro_gravity_host)
// The problem parameters arrive in mhd_params::problem_real/problem_int in
// the layout documented in ppkmhd_gb300.h.
#include <cmath>
#include <cstdint>

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
  IW = 4
};

constexpr double kPi = 3.141592653589793238462643383279502884;

struct HMesh
{
  int     g, nx, ny, nz, isize, jsize, ksize, dim;
  int64_t sj, sk, sv;
  double  xmin, xmax, ymin, ymax, zmin, zmax, dx, dy, dz, gamma0;
  explicit HMesh(const mhd_params & p)
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
    gamma0 = p.gamma0;
  }
  // cell centres: xmin + dx / 2 + (i - ghostWidth) * dx
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
  template <class F>
  void
  each(F && f) const
  {
    for (int k = 0; k < ksize; ++k)
      for (int j = 0; j < jsize; ++j)
        for (int i = 0; i < isize; ++i)
          f(i, j, k, i + j * sj + k * sk);
  }
};

void
implode(const mhd_params & p, const HMesh & m, double * U)
{
  const double * r = p.problem_real; // outer rho, p, vx, vy, vz, (B), inner ...
  const double   g0 = m.gamma0;
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    bool         out;
    if (m.dim == 2)
    {
      if (p.problem_int[0] == 1)
        out = x + y * y > 0.5 && x + y * y < 1.5;
      else
        out = x + y > (m.xmin + m.xmax) / 2. + m.ymin;
    }
    else
    {
      const double z = m.z(k);
      if (p.problem_int[0] == 1)
        out = x + y + z > 0.5 && x + y + z < 2.5;
      else
        out = x + y + z > (m.xmin + m.xmax) / 2. + m.ymin + m.zmin;
    }
    const double * s = out ? r : r + 8;
    const double   rho = s[0], pr = s[1], u = s[2], v = s[3], w = s[4];
    U[c + ID * m.sv] = rho;
    if (m.dim == 2)
      U[c + IP * m.sv] = pr / (g0 - 1.0) + 0.5 * rho * (u * u + v * v);
    else
      U[c + IP * m.sv] = pr / (g0 - 1.0) + 0.5 * rho * (u * u + v * v + w * w);
    U[c + IU * m.sv] = u;
    U[c + IV * m.sv] = v;
    if (m.dim == 3)
      U[c + IW * m.sv] = w;
  });
}

void
blast(const mhd_params & p, const HMesh & m, double * U)
{
  const double * r = p.problem_real; // radius, center x, y, z, d_in, d_out, p_in, p_out
  const double   radius2 = r[0] * r[0];
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    double       d2 = (x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]);
    if (m.dim == 3)
    {
      const double z = m.z(k);
      d2 = (x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]) + (z - r[3]) * (z - r[3]);
    }
    const bool in = d2 < radius2;
    U[c + ID * m.sv] = in ? r[4] : r[5];
    U[c + IP * m.sv] = (in ? r[6] : r[7]) / (m.gamma0 - 1.0);
    U[c + IU * m.sv] = 0.0;
    U[c + IV * m.sv] = 0.0;
    if (m.dim == 3)
      U[c + IW * m.sv] = 0.0;
  });
}

void
kelvin_helmholtz(const mhd_params & p, const HMesh & m, double * U)
{
  // d_in, d_out, pressure, vflow_in, vflow_out, amplitude, w0, delta; int mode
  const double * r = p.problem_real;
  const double   rho1 = r[0], rho2 = r[1], pressure = r[2];
  const double   w0 = r[6], delta = r[7];
  const int      n = p.problem_int[2];
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    double       d, u, v, w = 0.0;
    if (m.dim == 2)
    {
      const double y1 = 0.25, y2 = 0.75;
      const double ramp =
        1.0 / (1.0 + std::exp(2 * (y - y1) / delta)) + 1.0 / (1.0 + std::exp(2 * (y2 - y) / delta));
      d = rho1 + ramp * (rho2 - rho1);
      u = r[3] + ramp * (r[4] - r[3]);
      v = w0 * std::sin(n * kPi * x);
    }
    else
    {
      const double z = m.z(k);
      const double z1 = 0.25, z2 = 0.75;
      const double v1y = r[3] / 2, v2y = r[4] / 2;
      const double ramp =
        1.0 / (1.0 + std::exp(2 * (z - z1) / delta)) + 1.0 / (1.0 + std::exp(2 * (z2 - z) / delta));
      d = rho1 + ramp * (rho2 - rho1);
      u = r[3] + ramp * (r[4] - r[3]);
      v = v1y + ramp * (v2y - v1y);
      w = w0 * std::sin(n * kPi * x) * std::sin(n * kPi * y);
    }
    U[c + ID * m.sv] = d;
    U[c + IU * m.sv] = d * u;
    U[c + IV * m.sv] = d * v;
    if (m.dim == 2)
      U[c + IP * m.sv] = pressure / (m.gamma0 - 1.0) + 0.5 * d * (u * u + v * v);
    else
    {
      U[c + IW * m.sv] = d * w;
      U[c + IP * m.sv] = pressure / (m.gamma0 - 1.0) + 0.5 * d * (u * u + v * v + w * w);
    }
  });
}

void
gresho_vortex(const mhd_params & p, const HMesh & m, double * U)
{
  const double rho0 = p.problem_real[0], Ma = p.problem_real[1];
  const double g0 = m.gamma0;
  const double p0 = rho0 / (g0 * Ma * Ma);
  m.each([&](int i, int j, int, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    const double r = std::sqrt(x * x + y * y);
    const double theta = std::atan2(y, x);
    const double cosT = std::cos(theta);
    const double sinT = std::sin(theta);
    double       uphi, pr;
    if (r < 0.2)
    {
      uphi = 5 * r;
      pr = p0 + 25 / 2.0 * r * r;
    }
    else if (r < 0.4)
    {
      uphi = 2 - 5 * r;
      pr = p0 + 25 / 2.0 * r * r + 4 * (1 - 5 * r - std::log(0.2) + std::log(r));
    }
    else
    {
      uphi = 0;
      pr = p0 - 2 + 4 * std::log(2.0);
    }
    const double mu = rho0 * (-sinT * uphi), mv = rho0 * (cosT * uphi);
    U[c + ID * m.sv] = rho0;
    U[c + IU * m.sv] = mu;
    U[c + IV * m.sv] = mv;
    if (m.dim == 2)
      U[c + IP * m.sv] = pr / (g0 - 1.0) + 0.5 * (mu * mu + mv * mv) / rho0;
    else
    {
      // the 3D functor writes rho0 (cos T uphi) into rho w as well
      const double mw = rho0 * (cosT * uphi);
      U[c + IW * m.sv] = mw;
      U[c + IP * m.sv] = pr / (g0 - 1.0) + 0.5 * (mu * mu + mv * mv + mw * mw) / rho0;
    }
  });
}

// The four constant states of the Lax-Liu two-dimensional Riemann problems
// (P. D. Lax, X.-D. Liu, SIAM J. Sci. Comput. 19, 319-340, 1998), as the
// reference tabulates them (rho, u, v, p of the quadrants 0..3):
// getRiemannConfig2d, initRiemannConfig2d.h.  Its case 18 falls through
// into the default, so 18 and every number outside 0..17 give row 0.
const double kLaxLiu[18][4][4] = {
  { { 1.0, 0.0, 0.0, 1.0 }, { 0.5197, -0.7259, 0.0, 0.4 }, { 0.1072, -0.7259, -1.4045, 0.0439 },
    { 0.2579, 0.0, -1.4045, 0.15 } },
  { { 1.0, 0.0, 0.0, 1.0 }, { 0.5197, -0.7259, 0.0, 0.4 }, { 1.0, -0.7259, -0.7259, 1.0 },
    { 0.5197, 0.0, -0.7259, 0.4 } },
  { { 1.5, 0.0, 0.0, 1.5 }, { 0.5323, 1.206, 0.0, 0.3 }, { 0.138, 1.206, 1.206, 0.029 },
    { 0.5323, 0.0, 1.206, 0.3 } },
  { { 1.1, 0.0, 0.0, 1.1 }, { 0.5065, 0.8939, 0.0, 0.35 }, { 1.1, 0.8939, 0.8939, 1.1 },
    { 0.5065, 0.0, 0.8939, 0.35 } },
  { { 1.0, -0.75, -0.5, 1.0 }, { 2.0, -0.75, 0.5, 1.0 }, { 1.0, 0.75, 0.5, 1.0 },
    { 3.0, 0.75, -0.5, 1.0 } },
  { { 1.0, 0.75, -0.5, 1.0 }, { 2.0, 0.75, 0.5, 0.5 }, { 1.0, -0.75, 0.5, 1.0 },
    { 3.0, -0.75, -0.5, 1.0 } },
  { { 1.0, 0.1, 0.1, 1.0 }, { 0.5197, -0.6259, 0.1, 0.4 }, { 0.8, 0.1, 0.1, 0.4 },
    { 0.5197, 0.1, -0.6259, 0.4 } },
  { { 0.5197, 0.1, 0.1, 0.4 }, { 1.0, -0.6259, 0.1, 1.0 }, { 0.8, 0.1, 0.1, 1.0 },
    { 1.0, 0.1, -0.6259, 1.0 } },
  { { 1.0, 0.0, 0.3, 1.0 }, { 2.0, 0.0, -0.3, 1.0 }, { 1.039, 0.0, -0.8133, 0.4 },
    { 0.5197, 0.0, -0.4259, 0.4 } },
  { { 1.0, 0.0, 0.4297, 1.0 }, { 0.5, 0.0, 0.6076, 1.0 }, { 0.2281, 0.0, -0.6076, 0.3333 },
    { 0.4562, 0.0, -0.4259, 0.3333 } },
  { { 1.0, 0.1, 0.0, 1.0 }, { 0.5313, 0.8276, 0.0, 0.4 }, { 0.8, 0.1, 0.0, 0.4 },
    { 0.5313, 0.1, 0.7276, 0.4 } },
  { { 0.5313, 0.0, 0.0, 0.4 }, { 1.0, 0.7276, 0.0, 1.0 }, { 0.8, 0.0, 0.0, 1.0 },
    { 1.0, 0.0, 0.7276, 1.0 } },
  { { 1.0, 0.0, -0.3, 1.0 }, { 2.0, 0.0, 0.3, 1.0 }, { 1.0625, 0.0, 0.8145, 0.4 },
    { 0.5313, 0.0, 0.4276, 0.4 } },
  { { 2.0, 0.0, -0.5606, 8.0 }, { 1.0, 0.0, -1.2172, 8.0 }, { 0.4736, 0.0, 1.2172, 2.6667 },
    { 0.9474, 0.0, 1.1606, 2.6667 } },
  { { 1.0, 0.1, -0.3, 1.0 }, { 0.5197, -0.6259, -0.3, 0.4 }, { 0.8, 0.1, -0.3, 0.4 },
    { 0.5313, 0.1, 0.4276, 0.4 } },
  { { 0.5313, 0.1, 0.1, 0.4 }, { 1.0222, -0.6179, 0.1, 1.0 }, { 0.8, 0.1, 0.1, 1.0 },
    { 1.0, 0.1, 0.8276, 1.0 } },
  { { 1.0, 0.0, -0.4, 1.0 }, { 2.0, 0.0, -0.3, 1.0 }, { 1.0625, 0.0, 0.2145, 0.4 },
    { 0.5197, 0.0, -1.1259, 0.4 } },
  { { 1.0, 0.0, 1.0, 1.0 }, { 2.0, 0.0, -0.3, 1.0 }, { 1.0625, 0.0, 0.2145, 0.4 },
    { 0.5197, 0.0, 0.2741, 0.4 } },
};

void
four_quadrant(const mhd_params & p, const HMesh & m, double * U)
{
  const int    cfg = p.problem_int[0];
  const auto & row = kLaxLiu[(cfg >= 0 && cfg < 18) ? cfg : 0];
  const double xt = p.problem_real[0], yt = p.problem_real[1];
  // primToCons_2D (initRiemannConfig2d.h:22-36)
  double cons[4][4];
  for (int q = 0; q < 4; ++q)
  {
    const double rho = row[q][0], u = row[q][1], v = row[q][2], pr = row[q][3];
    cons[q][ID] = rho;
    cons[q][IU] = u * rho;
    cons[q][IV] = v * rho;
    cons[q][IP] = pr / (m.gamma0 - 1.0) + rho * (u * u + v * v) * 0.5;
  }
  m.each([&](int i, int j, int, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    const int    q = x < xt ? (y < yt ? 2 : 1) : (y < yt ? 3 : 0);
    for (int v = 0; v < 4; ++v)
      U[c + v * m.sv] = cons[q][v];
  });
}

void
isentropic_vortex(const mhd_params & p, const HMesh & m, double * U)
{
  // rho_a, T_a, u_a, v_a, center_x, center_y, strength
  const double * r = p.problem_real;
  const double   rho_a = r[0], T_a = r[1], u_a = r[2], v_a = r[3], beta = r[6];
  const double   g0 = m.gamma0;
  m.each([&](int i, int j, int, int64_t c) {
    const double xp = m.x(i) - r[4], yp = m.y(j) - r[5];
    const double rr = std::sqrt(xp * xp + yp * yp);
    const double du = -yp * beta / (2 * kPi) * std::exp(0.5 * (1.0 - rr * rr));
    const double dv = xp * beta / (2 * kPi) * std::exp(0.5 * (1.0 - rr * rr));
    const double T =
      T_a - (g0 - 1) * beta * beta / (8 * g0 * kPi * kPi) * std::exp(1.0 - rr * rr);
    const double rho = rho_a * std::pow(T / T_a, 1.0 / (g0 - 1));
    U[c + ID * m.sv] = rho;
    U[c + IU * m.sv] = rho * (u_a + du);
    U[c + IV * m.sv] = rho * (v_a + dv);
    U[c + IP * m.sv] = rho * T / (g0 - 1.0) + 0.5 * rho * (u_a + du) * (u_a + du) +
                       0.5 * rho * (v_a + dv) * (v_a + dv);
  });
}

void
rayleigh_taylor(const mhd_params & p, const HMesh & m, double * U)
{
  // amplitude, d0, d1, gx, gy, gz
  const double * r = p.problem_real;
  const double   Lx = m.xmax - m.xmin, Ly = m.ymax - m.ymin;
  const double   P0 = 1.0;
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    const double pert = r[0] * (1 + std::cos(2 * kPi * x / Lx)) * (1 + std::cos(2 * kPi * y / Ly)) / 4;
    if (m.dim == 2)
    {
      const double d = y > (m.ymin + m.ymax) / 2 ? r[2] : r[1];
      U[c + ID * m.sv] = d;
      U[c + IU * m.sv] = 0.0;
      U[c + IV * m.sv] = pert;
      U[c + IP * m.sv] = (P0 + d * (r[3] * x + r[4] * y)) / (m.gamma0 - 1.0);
    }
    else
    {
      const double z = m.z(k);
      const double d = z > (m.zmin + m.zmax) / 2 ? r[2] : r[1];
      U[c + ID * m.sv] = d;
      U[c + IU * m.sv] = 0.0;
      U[c + IV * m.sv] = 0.0;
      U[c + IW * m.sv] = pert;
      U[c + IP * m.sv] = (P0 + d * (r[3] * x + r[4] * y + r[5] * z)) / (m.gamma0 - 1);
    }
  });
}

void
rising_bubble(const mhd_params & p, const HMesh & m, double * U)
{
  // R, x0, y0, z0, din, dout, gx, gy, gz
  const double * r = p.problem_real;
  const double   P0 = 1.0;
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i), y = m.y(j);
    double       d, e;
    if (m.dim == 2)
    {
      const double rr = std::sqrt((x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]));
      d = rr < r[0] ? r[4] : r[5];
      e = (P0 + d * (r[6] * x + r[7] * y)) / (m.gamma0 - 1.0);
    }
    else
    {
      const double z = m.z(k);
      const double rr =
        std::sqrt((x - r[1]) * (x - r[1]) + (y - r[2]) * (y - r[2]) + (z - r[3]) * (z - r[3]));
      d = rr < r[0] ? r[4] : r[5];
      e = (P0 + d * (r[6] * x + r[7] * y + r[8] * z)) / (m.gamma0 - 1.0);
      U[c + IW * m.sv] = 0.0;
    }
    U[c + ID * m.sv] = d;
    U[c + IU * m.sv] = 0.0;
    U[c + IV * m.sv] = 0.0;
    U[c + IP * m.sv] = e;
  });
}

// PointSourceGravity::eval (PointSourceGravity.h): the softened
// point-source field at (x, y, z)
void
point_source(const double * r, double x, double y, double z, double & gx, double & gy, double & gz)
{
  const double xs = r[9], ys = r[10], zs = r[11], GM = r[12], eps = r[13];
  const double rr = std::sqrt((x - xs) * (x - xs) + (y - ys) * (y - ys) + (z - zs) * (z - zs) +
                              eps * eps);
  const double GM2 = GM / (rr * rr * rr);
  gx = GM2 * (xs - x);
  gy = GM2 * (ys - y);
  gz = GM2 * (zs - z);
}

// InitDiskFunctor2D / 3D (HydroInitFunctors2D.h:907-1060, 3D): a rotating
// disk around the point source, coordinates relative to the disk centre
void
disk(const mhd_params & p, const HMesh & m, double * U)
{
  const double * r = p.problem_real;
  const double   radius = r[0], radius_inner = r[1], xc = r[2], yc = r[3], zc = r[4];
  const double   rho0 = r[5], rho_contrast = r[6], contrast_width = r[7], ref_cs = r[8];
  const double   GM = r[12], eps = r[13];
  m.each([&](int i, int j, int k, int64_t c) {
    const double x = m.x(i) - xc, y = m.y(j) - yc;
    const double z = m.dim == 3 ? m.z(k) - zc : 0;
    const double r2 = x * x + y * y;
    const double rc = std::sqrt(r2);
    const double r_soft = std::sqrt(r2 + eps * eps);
    const double r_sph = std::sqrt(r2 + eps * eps + z * z);
    const double x_soft = x * (r_soft / rc);
    const double y_soft = y * (r_soft / rc);
    // DiskParams::radial_speed_of_sound
    const double csound =
      rc < radius_inner ? ref_cs / std::sqrt(radius_inner / radius) : ref_cs / std::sqrt(rc / radius);
    double omega2 = 0;
    if (rc >= radius_inner)
      omega2 = GM / (r_soft * r_soft * r_sph) - 3.5 * (csound / r_soft) * (csound / r_soft);
    else
      omega2 = GM / (r_soft * r_soft * r_soft) - 2.5 * (csound / r_soft) * (csound / r_soft);
    const double omega = std::sqrt(std::fmax(omega2, 0.0));
    double       rho = rho0 * std::pow(r_soft / radius, -2.5) *
                 std::exp(GM / (csound * csound) * (1. / r_sph - 1. / r_soft));
    if (rc > radius || std::fabs(z) > 0.5 * radius)
    {
      if (rc > radius + contrast_width || std::fabs(z) > 0.5 * radius + contrast_width)
        rho /= rho_contrast;
      else
      {
        const double cutdown = std::fmax((rc - radius) / contrast_width,
                                         (std::fabs(z) - 0.5 * radius) / contrast_width);
        rho *= std::pow(rho_contrast, -cutdown);
      }
    }
    rho = std::fmax(rho, 1e-6);
    U[c + ID * m.sv] = rho;
    U[c + IU * m.sv] = -y_soft * omega * rho;
    U[c + IV * m.sv] = x_soft * omega * rho;
    if (m.dim == 3)
      U[c + IW * m.sv] = 0.0;
    const double pressure = csound * csound * rho;
    U[c + IP * m.sv] = pressure / (m.gamma0 - 1.0) + 0.5 * rho * omega2 * (r2 + eps * eps);
  });
}

} // namespace

void
init_hydro_gravity_host(const mhd_params & p, double * g)
{
  // RayleighTaylorInstabilityFunctor / RisingBubbleFunctor write the uniform
  // (gx, gy[, gz]); InitDiskFunctor the point-source field at the cell
  // centre relative to the disk centre (z = 0 in 2D); other problems write
  // none (the reference's field stays zero)
  const HMesh m(p);
  m.each([&](int i, int j, int k, int64_t c) {
    double gx = p.gravity_field[0], gy = p.gravity_field[1], gz = p.gravity_field[2];
    if (p.problem == MHD_PROBLEM_DISK)
    {
      const double * r = p.problem_real;
      const double   x = m.x(i) - r[2], y = m.y(j) - r[3];
      const double   z = m.dim == 3 ? m.z(k) - r[4] : 0;
      point_source(r, x, y, z, gx, gy, gz);
    }
    else if (p.problem != MHD_PROBLEM_RAYLEIGH_TAYLOR && p.problem != MHD_PROBLEM_RISING_BUBBLE)
      gx = gy = gz = 0.0;
    g[c] = gx;
    g[c + m.sv] = gy;
    if (m.dim == 3)
      g[c + 2 * m.sv] = gz;
  });
}

void
init_hydro_problem_host(const mhd_params & p, double * U)
{
  const HMesh m(p);
  switch (p.problem)
  {
  case MHD_PROBLEM_BLAST:
    return blast(p, m, U);
  case MHD_PROBLEM_KELVIN_HELMHOLTZ:
    return kelvin_helmholtz(p, m, U);
  case MHD_PROBLEM_GRESHO_VORTEX:
    return gresho_vortex(p, m, U);
  case MHD_PROBLEM_FOUR_QUADRANT:
    return four_quadrant(p, m, U);
  case MHD_PROBLEM_ISENTROPIC_VORTEX:
    return isentropic_vortex(p, m, U);
  case MHD_PROBLEM_RAYLEIGH_TAYLOR:
    return rayleigh_taylor(p, m, U);
  case MHD_PROBLEM_RISING_BUBBLE:
    return rising_bubble(p, m, U);
  case MHD_PROBLEM_DISK:
    return disk(p, m, U);
  default:
    return implode(p, m, U);
  }
}

} // namespace mhd
