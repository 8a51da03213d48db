// Deterministic log / exp / pow for the step-size controllers: the same sequence of IEEE
// operations (+, -, *, /, fma, frexp, ldexp, rint, all exact or correctly rounded) on the host
// and on the device, so a controller evaluated inside a kernel produces the same bits as the
// host integrator and the CPU oracle. Accuracy is a few units in the last place, which is far
// below what a step-size controller needs.
//
//   log x: x = m 2^k with m in [sqrt(1/2), sqrt(2)), log m = 2 atanh(f), f = (m-1)/(m+1),
//          atanh series f + f^3/3 + ... + f^25/25 (|f| <= 0.1716: truncation < 1e-20);
//   exp y: k = rint(y / ln 2), r = y - k ln 2 (two-part ln 2), |r| <= 0.347,
//          Taylor series of e^r to r^17/17! (truncation < 1e-19), times 2^k.
#pragma once
#include <cmath>

#if defined(__CUDACC__)
#define STS_HD __host__ __device__ __forceinline__
#else
#define STS_HD static inline
#endif

namespace stsm {
// ln 2 = LN2_HI + LN2_LO: LN2_HI is ln 2 rounded to a double, LN2_LO the remainder
constexpr double LN2_HI  = 0.6931471805599453094;
constexpr double LN2_LO  = 2.3190468138462996e-17;
constexpr double INV_LN2 = 1.4426950408889634074;

STS_HD double log(double x)
{
  if (!(x > 0.0)) return x == 0.0 ? -HUGE_VAL : NAN;
  if (x == HUGE_VAL) return x;
  int k    = 0;
  double m = frexp(x, &k); // m in [0.5, 1)
  if (m < 0.70710678118654752440)
  {
    m = m * 2.0;
    k = k - 1;
  }
  const double f  = (m - 1.0) / (m + 1.0);
  const double f2 = f * f;
  double s        = 1.0 / 25.0;
  for (int i = 11; i >= 0; --i) s = fma(s, f2, 1.0 / (double)(2 * i + 1));
  const double lm = 2.0 * f * s;
  const double kd = (double)k;
  return fma(kd, LN2_HI, fma(kd, LN2_LO, lm));
}

STS_HD double exp(double y)
{
  if (y != y) return y;
  if (y > 709.78) return HUGE_VAL;
  if (y < -745.2) return 0.0;
  const double k = rint(y * INV_LN2);
  double r       = fma(-k, LN2_HI, y);
  r              = fma(-k, LN2_LO, r);
  // 1/i! for i = 17 .. 0 by the recurrence c_i = c_{i+1} * (i+1), evaluated by Horner
  double c[18];
  c[0] = 1.0;
  for (int i = 1; i < 18; ++i) c[i] = c[i - 1] / (double)i;
  double s = c[17];
  for (int i = 16; i >= 0; --i) s = fma(s, r, c[i]);
  return ldexp(s, (int)k);
}

// x^y for x > 0 (the controllers' error ratios are at least 1e-10)
STS_HD double pow(double x, double y) { return stsm::exp(y * stsm::log(x)); }
} // namespace stsm
