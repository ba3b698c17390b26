// eexp.cuh -- eexp (utilities.cpp:1507-1540): x as a mantissa m in [1, 10)
// and a decimal exponent z with e^x = m 10^z, by the reference's method (the
// power of two split off, a ten-term Taylor polynomial for the rest), so
// that sums of such terms rescaled to their largest exponent follow the
// reference's (jointp, calc_pop_expomig).
#pragma once

namespace {

constexpr double EEXP_LOG2 = 0.69314718055994530941723212146;

__device__ __forceinline__ void eexp_dev(double x, double *m, int *z)
{
  const double inv_fact[10] = {1.0, 0.5, 0.16666666666666666666666666667,
                               0.04166666666666666666666666667, 0.00833333333333333333333333333,
                               0.001388888888888888888888888889, 0.000198412698412698412698412698,
                               0.000024801587301587301587301587301,
                               2.75573192239858906525573192239859e-6,
                               2.75573192239858906525573192239e-7};
  const double log10_2 = 0.30102999566398119521;
  int n = (int)floor(x / EEXP_LOG2);
  double zr = log10_2 * (double)n;
  *z = (int)zr;
  zr -= (double)*z;
  double u = x - ((double)n) * EEXP_LOG2;
  double t = inv_fact[9];
  for (int k = 8; k >= 0; k--) t = inv_fact[k] + u * t;
  t = 1 + u * t;
  *m = t * pow(10.0, zr);
  if (fabs(*m) > 10) { *m = *m / 10.0; *z = *z + 1; }
  if (fabs(*m) < 1) { *m = *m * 10.0; *z = *z - 1; }
}

}  // namespace
