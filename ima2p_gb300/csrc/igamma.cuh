// igamma.cuh -- the reference's incomplete gamma functions on the device
// (uppergamma, lowergamma, gser/gserlog, gcf/gcflog, expint(1, x) and
// LogDiff; utilities.cpp:808-1130, imamp.hpp:257-262), shared by the p(G)
// integrals (k_treeweight.cu) and the 2NM densities (k_popmig.cu).  Both
// files are compiled with -fmad=false so that these add and multiply in the
// reference's order; log and exp are the device's.
#pragma once

#include "internal.h"

namespace {

enum { IG_E_TERM = 4, IG_E_LF = 5 };  // a series or fraction that did not converge; a count past logfact

// The reference's incomplete gamma functions, restated from the published
// Numerical Recipes methods it uses (series, Lentz continued fraction, E1
// series / continued fraction) with its constants: EPS 3e-7, ITMAX 1000,
// FPMIN 1e-30, expint's MAXIT 100 and Euler constant 0.5772156649.
constexpr double IG_EPS = 3.0e-7, IG_FPMIN = 1.0e-30, EI_EULER = 0.5772156649;
constexpr int IG_ITMAX = 1000, EI_MAXIT = 100;
constexpr double LD_CUT = 7.0978271289338397e+02, MPRIORMIN = 0.000001;
constexpr double LOG2 = 0.69314718055994530941723212146;

struct IgBase {
  const double *lft;
  int st;
  __device__ double lf(int i)
  {
    if (i < 0 || i >= TW_LF_N) {
      st = IG_E_LF;
      return 0.0;
    }
    return lft[i];
  }
  __device__ double gser(int a, double x, double *gln, bool lg)
  {
    *gln = lf(a - 1);
    if (x <= 0.0) {
      if (x < 0.0) st = IG_E_TERM;
      return 0.0;
    }
    double ap = a, del = 1.0 / a, sum = del;
    for (int n = 1; n <= IG_ITMAX; n++) {
      ++ap;
      del *= x / ap;
      sum += del;
      if (fabs(del) < fabs(sum) * IG_EPS)
        return lg ? log(sum) + (-x + a * log(x) - (*gln)) : sum * exp(-x + a * log(x) - (*gln));
    }
    st = IG_E_TERM;
    return 0.0;
  }
  __device__ double gcf(double a, double x, double *gln, bool lg)
  {
    *gln = lf((int)a - 1);
    double b = x + 1.0 - a, c = 1.0 / IG_FPMIN, d = 1.0 / b, h = d;
    int i;
    for (i = 1; i <= IG_ITMAX; i++) {
      const double an = -i * (i - a);
      b += 2.0;
      d = an * d + b;
      if (fabs(d) < IG_FPMIN) d = IG_FPMIN;
      c = b + an / c;
      if (fabs(c) < IG_FPMIN) c = IG_FPMIN;
      d = 1.0 / d;
      const double del = d * c;
      h *= del;
      if (fabs(del - 1.0) < IG_EPS) break;
    }
    if (i > IG_ITMAX) st = IG_E_TERM;
    return lg ? (-x + a * log(x) - (*gln)) + log(h) : exp(-x + a * log(x) - (*gln)) * h;
  }
  __device__ double expint1(double x, bool *islog)
  {
    *islog = false;
    if (x <= 0.0) {
      st = IG_E_TERM;
      return 0.0;
    }
    if (x > 1.0) {
      double b = x + 1, c = 1.0 / IG_FPMIN, d = 1.0 / b, h = d;
      for (int i = 1; i <= EI_MAXIT; i++) {
        const double an = -i * i;
        b += 2.0;
        d = 1.0 / (an * d + b);
        c = b + an / c;
        const double del = c * d;
        h *= del;
        if (fabs(del - 1.0) < IG_EPS) {
          *islog = true;
          return log(h) - x;
        }
      }
      st = IG_E_TERM;
      return 0.0;
    }
    double ans = -log(x) - EI_EULER, fact = 1.0;
    for (int i = 1; i <= EI_MAXIT; i++) {
      fact *= -x / i;
      const double del = -fact / i;
      ans += del;
      if (fabs(del) < fabs(ans) * IG_EPS) return ans;
    }
    st = IG_E_TERM;
    return ans;
  }
  __device__ double upper(int a, double x)  // uppergamma: log Gamma(a, x)
  {
    double p, gln;
    if (x < 0.0 || a < 0) {
      st = IG_E_TERM;
      return 0.0;
    }
    if (a == 0) {
      bool islog;
      const double t = expint1(x, &islog);
      p = islog ? t : log(t);
    } else if (x < (a + 1.0)) {
      const double gs = gser(a, x, &gln, false);
      p = gln + log(1.0 - gs);
    } else {
      p = gln_plus_gcf(a, x, true);
    }
    return p < -1e200 ? -1e200 : p;
  }
  __device__ double gln_plus_gcf(int a, double x, bool lg)
  {
    double gln;
    const double v = gcf((double)a, x, &gln, lg);
    return lg ? gln + v : gln + log(1 - v);
  }
  __device__ double lower(int a, double x)  // lowergamma: log gamma(a, x)
  {
    double p, gln;
    if (x < 0.0 || a <= 0) {
      st = IG_E_TERM;
      return 0.0;
    }
    if (x < (a + 1.0)) {
      const double gs = gser(a, x, &gln, true);
      p = gln + gs;
    } else {
      p = gln_plus_gcf(a, x, false);
    }
    return p < -1e200 ? -1e200 : p;
  }
  __device__ double logdiff(double a, double b)  // LogDiff, imamp.hpp:257-262
  {
    if (a <= b) {
      st = IG_E_TERM;
      return 0.0;
    }
    return (a - b < LD_CUT) ? b + log(exp(a - b) - 1.0) : a;
  }
};

// The integral terms of initialize_integrate_tree_prob
// (update_gtree_common.cpp:108-304, MORESTABLE) on the functions above.
struct Ig : IgBase {
  __device__ double coal(int cc, double fc, double hcc, double max, double min)
  {
    double p;
    if (cc > 0) {
      if (!(fc > 0)) {
        st = IG_E_TERM;
        return 0.0;
      }
      if (min == 0) {
        double ug = upper(cc - 1, 2 * fc / max);
        if (cc > 1) {
          const double fullg = lf(cc - 2);
          if (fullg - ug < 1e-15 || fullg - ug > LD_CUT) {
            const double lg = lower(cc - 1, 2 * fc / max);
            if (fullg > lg) {
              const double ugalt = logdiff(fullg, lg);
              if (fabs(ugalt - ug) > 1e-10) ug = ugalt;
            }
          }
        }
        p = ug + LOG2 - hcc + (1 - cc) * log(fc);
      } else {
        const double aa = upper(cc - 1, 2 * fc / max), bb = upper(cc - 1, 2 * fc / min);
        p = logdiff(aa, bb);
        p += (LOG2 - hcc + (1 - cc) * log(fc));
      }
    } else if (2 * fc / max > 0) {
      if (min == 0) {
        const double aa = log(max) - 2.0 * fc / max;
        const double bb = LOG2 + log(fc) + upper(0, 2.0 * fc / max);
        p = logdiff(aa, bb);
      } else {
        double aa = upper(0, 2 * fc / max), bb = upper(0, 2 * fc / min);
        double c = logdiff(aa, bb);
        c += LOG2 + log(fc);
        aa = log(max) - 2.0 * fc / max;
        bb = log(min) - 2.0 * fc / min;
        const double d = logdiff(aa, bb);
        p = logdiff(d, c);
      }
    } else {
      p = log(max - min);
    }
    return p;
  }
  __device__ double mig(int cm, double fm, double max, double min)
  {
    double p;
    if (cm > 0) {
      if (!(fm > 0)) {
        st = IG_E_TERM;
        return 0.0;
      }
      if (min == 0) {
        double lg = lower(cm + 1, fm * max);
        const double fullg = lf(cm);
        if (fullg - lg < 1e-15 || fullg - lg > LD_CUT) {
          const double ug = upper(cm + 1, fm * max);
          if (fullg > ug) {
            const double lgalt = logdiff(fullg, ug);
            if (fabs(lgalt - lg) > 1e-12) lg = lgalt;
          }
        }
        p = (-1 - cm) * log(fm) + lg;
      } else {
        const double aa = upper(cm + 1, fm * min), bb = upper(cm + 1, fm * max);
        p = (-1 - cm) * log(fm) + logdiff(aa, bb);
      }
    } else if (fm > MPRIORMIN) {
      if (min == 0) {
        p = (max == MPRIORMIN) ? 0 : logdiff(0.0, -fm * max) - log(fm);
      } else {
        p = logdiff(-fm * min, -fm * max) - log(fm);
      }
    } else {
      p = log(max - min);
    }
    return p;
  }
  __device__ double mig_expo(int cm, double fm, double mean)
  {
    return -log(mean) + (-(cm + 1) * log(fm + 1.0 / mean)) + lf(cm);
  }
};

}  // namespace
