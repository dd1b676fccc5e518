/*
 * CPU oracle of the HLLD flux surrogate (test infrastructure only).
 *
 * Restates, in double precision, what ppkmhd_gb300/csrc/mhd_mlp.cuh and
 * mhd_mlp.cu compute on the GPU: the dimensionless face encoding, the
 * central flux, the 27-64-64-19 GELU perceptron (tanh form of Hendrycks and
 * Gimpel, 2016) whose odd transverse flux components are its coefficients
 * times the odd bases, with optional emulation of the deployed BF16
 * rounding of weights, inputs and hidden activations, and the
 * mean-squared-error loss with its gradient by back-propagation.  The physical flux follows the flux
 * vector of riemann_hlld (RiemannSolvers_MHD.h:358-366).  The gradient is
 * checked against central finite differences in the tests, so this file is
 * pinned independently of the GPU code.
 *
 * Parameter vector: W1[32][64] b1[64] W2[64][64] b2[64] W3[64][24] b3[24].
 * Features of a face: 32 network inputs, then the 8 odd bases u1[4], u2[4].
 */
#include <math.h>
#include <stdint.h>
#include <string.h>

#define NIN 32
#define NH 64
#define NOUT 24
#define NUSED 7
#define NFEAT 40
#define OFF_W1 0
#define OFF_B1 (OFF_W1 + NIN * NH)
#define OFF_W2 (OFF_B1 + NH)
#define OFF_B2 (OFF_W2 + NH * NH)
#define OFF_W3 (OFF_B2 + NH)
#define OFF_B3 (OFF_W3 + NH * NOUT)
#define NPARAM (OFF_B3 + NOUT)

static const double J_FLOOR = 1e-4;
static const double TAU_REF = 0.1;
static const double GC0 = 0.7978845608028654; /* sqrt(2/pi) */
static const double GC1 = 0.044715;

int
mlp_nparams(void)
{
  return NPARAM;
}

/* float -> bfloat16 (round to nearest even) -> float */
static double
bf16(double x)
{
  float    f = (float)x;
  uint32_t u;
  memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u)
    return x;
  u += 0x7fffu + ((u >> 16) & 1u);
  u &= 0xffff0000u;
  memcpy(&f, &u, 4);
  return (double)f;
}

double
mlp_bf16(double x)
{
  return bf16(x);
}

/* q = rho, vn, vt1, vt2, p, Bt1, Bt2; f[NFEAT] = inputs, then odd bases;
 * returns J */
double
mlp_encode(const double * qL, const double * qR, double a, double * f, double * scale)
{
  const double rs = 0.5 * (qL[0] + qR[0]);
  const double b2L = a * a + qL[5] * qL[5] + qL[6] * qL[6];
  const double b2R = a * a + qR[5] * qR[5] + qR[6] * qR[6];
  const double Ps = 0.5 * (qL[4] + qR[4]) + 0.25 * (b2L + b2R);
  const double vs = sqrt(Ps / rs), bs = sqrt(Ps);
  const double div[7] = { rs, vs, vs, vs, Ps, bs, bs };
  double       h[7], J = 0.0;
  for (int q = 0; q < 7; ++q)
  {
    h[q] = 0.5 * (qR[q] - qL[q]) / div[q];
    if (fabs(h[q]) > J)
      J = fabs(h[q]);
  }
  const double sJ = J > J_FLOOR ? J : J_FLOOR;
  f[0] = 0.5 * (qL[1] + qR[1]) / vs;
  f[1] = 0.5 * (qL[4] + qR[4]) / Ps;
  f[2] = a / bs;
  f[3] = h[0] / sJ;
  f[4] = h[1] / sJ;
  f[5] = h[4] / sJ;
  f[6] = sJ / TAU_REF;
  double * u1 = f + NIN;
  double * u2 = f + NIN + 4;
  u1[0] = 0.5 * (qL[2] + qR[2]) / vs;
  u1[1] = 0.5 * (qL[5] + qR[5]) / bs;
  u1[2] = h[2] / sJ;
  u1[3] = h[5] / sJ;
  u2[0] = 0.5 * (qL[3] + qR[3]) / vs;
  u2[1] = 0.5 * (qL[6] + qR[6]) / bs;
  u2[2] = h[3] / sJ;
  u2[3] = h[6] / sJ;
  int o = 7;
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      f[o++] = u1[i] * u1[j];
  for (int i = 0; i < 4; ++i)
    for (int j = i; j < 4; ++j)
      f[o++] = u2[i] * u2[j];
  for (; o < NIN; ++o)
    f[o] = 0.0;
  scale[0] = rs * vs * sJ;
  scale[1] = Ps * vs * sJ;
  scale[2] = scale[3] = scale[4] = Ps * sJ;
  scale[5] = scale[6] = bs * vs * sJ;
  return J;
}

/* raw outputs y[NOUT] and bases u[8] -> dissipation D[7] */
static void
combine(const double * y, const double * u, double * D)
{
  const double *u1 = u, *u2 = u + 4;
  D[0] = y[0];
  D[1] = y[1];
  D[2] = y[2];
  D[3] = y[3] * u1[0] + y[4] * u1[1] + y[5] * u1[2] + y[6] * u1[3];
  D[5] = y[7] * u1[0] + y[8] * u1[1] + y[9] * u1[2] + y[10] * u1[3];
  D[4] = y[11] * u2[0] + y[12] * u2[1] + y[13] * u2[2] + y[14] * u2[3];
  D[6] = y[15] * u2[0] + y[16] * u2[1] + y[17] * u2[2] + y[18] * u2[3];
}

static void
physical_flux(const double * q, double a, double g, double * F)
{
  const double r = q[0], u = q[1], v = q[2], w = q[3], p = q[4], b = q[5], c = q[6];
  const double B2 = a * a + b * b + c * c, Pt = p + 0.5 * B2;
  const double E = p / (g - 1.0) + 0.5 * r * (u * u + v * v + w * w) + 0.5 * B2;
  const double vB = u * a + v * b + w * c;
  F[0] = r * u;
  F[1] = (E + Pt) * u - a * vB;
  F[2] = r * u * u + Pt - a * a;
  F[3] = r * u * v - a * b;
  F[4] = r * u * w - a * c;
  F[5] = b * u - a * v;
  F[6] = c * u - a * w;
}

void
mlp_central_flux(const double * qL, const double * qR, double a, double g, double * Fc)
{
  double FL[7], FR[7];
  physical_flux(qL, a, g, FL);
  physical_flux(qR, a, g, FR);
  for (int q = 0; q < 7; ++q)
    Fc[q] = 0.5 * (FL[q] + FR[q]);
}

static double
gelu(double x)
{
  return 0.5 * x * (1.0 + tanh(GC0 * (x + GC1 * x * x * x)));
}

/* The deployed BF16 evaluation of the same formula: BF16 input, each
 * multiply / fused multiply-add rounded to BF16, BF16 constants. */
static double
gelu_bf16(double z)
{
  const double x = bf16(z);
  const double c0 = bf16(GC0), c01 = bf16(GC0 * GC1), h = bf16(0.5);
  const double u = bf16(x * bf16(bf16(x * x) * c01 + c0));
  const double t = bf16(tanh(u));
  const double hx = bf16(x * h);
  return bf16(hx * t + hx);
}

static double
gelu_grad(double x)
{
  const double t = tanh(GC0 * (x + GC1 * x * x * x));
  return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GC0 * (1.0 + 3.0 * GC1 * x * x);
}

/* y[8] = net(x[16]); with rounding != 0 the weights and inputs are rounded
 * to BF16 (biases stay exact) and the activation is the BF16 evaluation of
 * GELU, as deployed. */
void
mlp_forward(const double * P, const double * x_in, double * D, int rounding)
{
  double x[NIN], h1[NH], h2[NH], y[NOUT];
#define W(off, idx) (rounding ? bf16(P[(off) + (idx)]) : P[(off) + (idx)])
  for (int i = 0; i < NIN; ++i)
    x[i] = rounding ? bf16(x_in[i]) : x_in[i];
  for (int k = 0; k < NH; ++k)
  {
    double z = P[OFF_B1 + k];
    for (int i = 0; i < NIN; ++i)
      z += x[i] * W(OFF_W1, i * NH + k);
    h1[k] = rounding ? gelu_bf16(z) : gelu(z);
  }
  for (int k = 0; k < NH; ++k)
  {
    double z = P[OFF_B2 + k];
    for (int j = 0; j < NH; ++j)
      z += h1[j] * W(OFF_W2, j * NH + k);
    h2[k] = rounding ? gelu_bf16(z) : gelu(z);
  }
  for (int o = 0; o < NOUT; ++o)
  {
    double z = P[OFF_B3 + o];
    for (int j = 0; j < NH; ++j)
      z += h2[j] * W(OFF_W3, j * NOUT + o);
    y[o] = z;
  }
#undef W
  combine(y, x_in + NIN, D);
  D[7] = 0.0;
}

void
mlp_forward_batch(const double * P, const double * X, long n, double * Y, int rounding)
{
#pragma omp parallel for schedule(static)
  for (long s = 0; s < n; ++s)
    mlp_forward(P, X + s * NFEAT, Y + s * 8, rounding);
}

/* Mean squared error over n samples and the 7 used outputs (no rounding),
 * and its gradient with respect to P (grad[NPARAM], overwritten). */
double
mlp_loss_grad(const double * P, const double * X, const double * T, long n, double * grad)
{
  memset(grad, 0, sizeof(double) * NPARAM);
  const double norm = 1.0 / ((double)n * NUSED);
  double       loss = 0.0;
  for (long s = 0; s < n; ++s)
  {
    const double * x = X + s * NFEAT;
    const double * t = T + s * 8;
    const double * u1 = x + NIN;
    const double * u2 = x + NIN + 4;
    double         z1[NH], h1[NH], z2[NH], h2[NH], y[NOUT], D[NUSED], dD[NUSED], dy[NOUT];
    double         dz2[NH], dz1[NH];
    for (int k = 0; k < NH; ++k)
    {
      double z = P[OFF_B1 + k];
      for (int i = 0; i < NIN; ++i)
        z += x[i] * P[OFF_W1 + i * NH + k];
      z1[k] = z;
      h1[k] = gelu(z);
    }
    for (int k = 0; k < NH; ++k)
    {
      double z = P[OFF_B2 + k];
      for (int j = 0; j < NH; ++j)
        z += h1[j] * P[OFF_W2 + j * NH + k];
      z2[k] = z;
      h2[k] = gelu(z);
    }
    for (int o = 0; o < NOUT; ++o)
    {
      double z = P[OFF_B3 + o];
      for (int j = 0; j < NH; ++j)
        z += h2[j] * P[OFF_W3 + j * NOUT + o];
      y[o] = z;
    }
    combine(y, x + NIN, D);
    for (int c = 0; c < NUSED; ++c)
    {
      const double e = D[c] - t[c];
      loss += e * e;
      dD[c] = 2.0 * e * norm;
    }
    for (int o = 0; o < NOUT; ++o)
      dy[o] = 0.0;
    dy[0] = dD[0];
    dy[1] = dD[1];
    dy[2] = dD[2];
    for (int k = 0; k < 4; ++k)
    {
      dy[3 + k] = dD[3] * u1[k];
      dy[7 + k] = dD[5] * u1[k];
      dy[11 + k] = dD[4] * u2[k];
      dy[15 + k] = dD[6] * u2[k];
    }
    for (int j = 0; j < NH; ++j)
    {
      double d = 0.0;
      for (int o = 0; o < NOUT; ++o)
        d += dy[o] * P[OFF_W3 + j * NOUT + o];
      dz2[j] = d * gelu_grad(z2[j]);
    }
    for (int j = 0; j < NH; ++j)
    {
      double d = 0.0;
      for (int k = 0; k < NH; ++k)
        d += dz2[k] * P[OFF_W2 + j * NH + k];
      dz1[j] = d * gelu_grad(z1[j]);
    }
    for (int i = 0; i < NIN; ++i)
      for (int k = 0; k < NH; ++k)
        grad[OFF_W1 + i * NH + k] += x[i] * dz1[k];
    for (int k = 0; k < NH; ++k)
      grad[OFF_B1 + k] += dz1[k];
    for (int j = 0; j < NH; ++j)
      for (int k = 0; k < NH; ++k)
        grad[OFF_W2 + j * NH + k] += h1[j] * dz2[k];
    for (int k = 0; k < NH; ++k)
      grad[OFF_B2 + k] += dz2[k];
    for (int j = 0; j < NH; ++j)
      for (int o = 0; o < NOUT; ++o)
        grad[OFF_W3 + j * NOUT + o] += h2[j] * dy[o];
    for (int o = 0; o < NOUT; ++o)
      grad[OFF_B3 + o] += dy[o];
  }
  return loss * norm;
}
