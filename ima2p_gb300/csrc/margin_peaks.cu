// margin_peaks.cu -- the numeric core of findmarginpeaks
// (surface_call_functions.cpp:316-734): the peaks of every parameter's 1-D
// marginal density over the two halves of the saved genealogies and over all
// of them (marginalopt, :178-266: two bracketing searches, mnbrakmod, then a
// golden-section search, goldenmod; surface_search_functions.cpp:42-200),
// the likelihood-ratio test of each migration rate against zero, the 95%
// limits by bisection (margin95 / marginbis, :86-113, :268-292), and the
// same peaks and tests for the 2NM terms (marginalopt_popmig, popmig.cpp:
// 361-428: a 100-point scan, then goldenmod).
//
// Host code.  Each search is sequential -- the next point depends on the
// last value -- but the searches of all parameters, terms and genealogy
// ranges are independent, so they advance together: every search is a
// function of its function values, run by replay.  Each round re-runs every
// unfinished search from its start against the values found so far (held
// per search, keyed by x); a search that needs a value it does not have
// stops and leaves its x.  All the x's of a round go to the device in a few
// batched launches (one per kind of density and genealogy range), and the
// next round continues.  A search thus follows exactly the reference's
// sequence of points, given the values; the values agree with the
// reference's to rounding (the device sums in another order).
#include <cfloat>
#include <cmath>
#include <cstring>
#include <functional>
#include <unordered_map>
#include <vector>

#include "internal.h"

namespace {

constexpr double MINPARAMVAL = 0.0000001;  // imamp.hpp:130
constexpr double OFFSCALEVAL = 1.0;        // marginp / marginpopmig outside the prior
constexpr double DOWN95 = 1.92;
constexpr int BIS_JMAX = 40;
constexpr double BISTOL = 1e-4;
constexpr double GOLD = 1.618034, GLIMIT = 100.0, TINY = 1.0e-20, GR = 0.61803399;
constexpr int POPMIG_MARGINBINS = 100;
constexpr int NUMTREEINT = 2;
constexpr int MAXSAVED = 300000;  // MAXGENEALOGIESTOSAVE

struct Need {};  // a search asked for values it does not have yet

// The function values of one search, by x; the x's it still needs.
struct Feed {
  std::unordered_map<uint64_t, double> known;
  std::vector<double> want;
  static uint64_t key(double x)
  {
    uint64_t k;
    memcpy(&k, &x, 8);
    return k;
  }
  double get(double x)
  {
    auto it = known.find(key(x));
    if (it != known.end()) return it->second;
    want.push_back(x);
    throw Need{};
  }
  // the values of xs before any of them is used (one round for a scan)
  void prefetch(const std::vector<double> &xs)
  {
    for (double x : xs)
      if (!known.count(key(x))) want.push_back(x);
    if (!want.empty()) throw Need{};
  }
};

// marginp; margincalc's log (95% limits); the 2NM peak search's density
// (marginpop_expomig under the exponential prior); marginpopmig, which the
// 2NM test calls whatever the prior (:463-466)
enum Kind { K_MARGINP = 0, K_LOG95 = 1, K_POPMIG = 2, K_POPMIG_UNIFORM = 3 };

struct Search {
  Kind kind;
  int idx;         // parameter (marginp, 95%) or term (2NM)
  int range;       // genealogy range 0..NUMTREEINT
  int ul = 0;      // K_LOG95: 0 lower limit, 1 upper
  double yadjust;  // K_LOG95
  double lo, hi;   // the density's prior range (off-scale outside), K_MARGINP / K_POPMIG
  Feed feed;
  bool done = false;
  // the reference's function at x: off-scale values without the device
  double f(double x)
  {
    if (kind != K_LOG95 && (x < lo || x > hi)) return OFFSCALEVAL;
    if (x != x) return NAN;  // a search that ran off to NaN: every term is NaN
    return feed.get(x);
  }
};

// sign (surface_search_functions.cpp:21-28)
double nr_sign(double a, double b) { return b > 0.0 ? fabs(a) : -fabs(a); }

// mnbrakmod (surface_search_functions.cpp:42-121).  Its FMAX keeps both
// arguments in float variables, so the parabolic step's denominator is
// rounded to float as there.
void mnbrakmod(Search &s, double *ax, double *bx, double *cx, double *fa, double *fb, double *fc)
{
  double ulim, u, rr, q, fu, dum;
  *fa = s.f(*ax);
  *fb = s.f(*bx);
  if (*fb > *fa) {
    dum = *ax;
    *ax = *bx;
    *bx = dum;
    dum = *fb;
    *fb = *fa;
    *fa = dum;
  }
  *cx = fabs(*bx + GOLD * (*bx - *ax));
  *fc = s.f(*cx);
  while (*fb >= *fc && *fb > -DBL_MAX && !(*fb == 0 && *fc == 0)) {
    rr = (*bx - *ax) * (*fb - *fc);
    q = (*bx - *cx) * (*fb - *fa);
    const float m1 = (float)fabs(q - rr), m2 = (float)TINY;
    const float mx = m1 > m2 ? m1 : m2;
    u = (double)*bx - ((*bx - *cx) * q - (*bx - *ax) * rr) / (2.0 * nr_sign(mx, q - rr));
    ulim = *bx + GLIMIT * (*cx - *bx);
    if ((*bx - u) * (u - *cx) > 0.0) {
      fu = s.f(u);
      if (fu < *fc) {
        *ax = *bx;
        *fa = *fb;
        *bx = u;
        *fb = fu;
        continue;
      }
      if (fu > *fb) {
        *cx = u;
        *fc = fu;
        continue;
      }
      u = *cx + GOLD * (*cx - *bx);
      fu = s.f(u);
    } else if ((*cx - u) * (u - ulim) > 0.0) {
      fu = s.f(u);
      if (fu < *fc) {
        *bx = *cx;
        *cx = u;
        u = *cx + GOLD * (*cx - *bx);
        *fb = *fc;
        *fc = fu;
        fu = s.f(u);
      }
    } else if ((u - ulim) * (ulim - *cx) >= 0.0) {
      u = ulim;
      fu = s.f(u);
    } else {
      u = *cx + GOLD * (*cx - *bx);
      fu = s.f(u);
    }
    *ax = *bx;
    *bx = *cx;
    *cx = u;
    *fa = *fb;
    *fb = *fc;
    *fc = fu;
  }
}

// goldenmod (surface_search_functions.cpp:129-200)
double goldenmod(Search &s, double ax, double bx, double cx, double tol, double *xmin)
{
  double f1, f2, x0, x1, x2, x3;
  const double c = 1.0 - GR;
  x0 = ax;
  x3 = cx;
  if (fabs(cx - bx) > fabs(bx - ax)) {
    x1 = bx;
    x2 = bx + c * (cx - bx);
  } else {
    x2 = bx;
    x1 = bx - c * (bx - ax);
  }
  f1 = s.f(x1);
  f2 = s.f(x2);
  while (fabs(x3 - x0) > tol * (fabs(x1) + fabs(x2)) && (x3 > -DBL_MAX)) {
    if (f2 < f1) {
      x0 = x1;
      x1 = x2;
      x2 = GR * x1 + c * x3;
      f1 = f2;
      f2 = s.f(x2);
      continue;
    }
    x3 = x2;
    x2 = x1;
    x1 = GR * x2 + c * x0;
    f2 = f1;
    f1 = s.f(x1);
  }
  if (f1 < f2) {
    *xmin = x1;
    return f1;
  }
  *xmin = x2;
  return f2;
}

// marginbis (surface_call_functions.cpp:86-108) on margincalc(logi = 1)
double marginbis(Search &s, double x1, double x2)
{
  double dx, f, fmid, xmid, rtb;
  f = s.f(x1);
  fmid = s.f(x2);
  if (f * fmid >= 0.0) return DBL_MIN;
  rtb = f < 0.0 ? (dx = x2 - x1, x1) : (dx = x1 - x2, x2);
  for (int j = 1; j <= BIS_JMAX; j++) {
    fmid = s.f(xmid = rtb + (dx *= 0.5));
    if (fmid <= 0.0) rtb = xmid;
    if (fabs(dx) < BISTOL || fmid == 0.0) return rtb;
  }
  return DBL_MAX;
}

// the two brackets of marginalopt for one parameter (:198-207)
struct Bracket {
  double axt, bxt, cxt, ax, bx, cx;
};

}  // namespace

int findmarginpeaks_run(const MarginPeaksIn &in, const MarginPeaksEval &eval, MarginPeaksOut &out)
{
  const int np = in.np, nm = in.nm, npar = np + nm, nt = in.nterms;
  const int Gs = in.G < MAXSAVED - 1 ? in.G : MAXSAVED - 1;  // IMIN(MAXGENEALOGIESTOSAVE - 1, .)
  out.too_few = Gs <= 10;
  if (out.too_few) {
    for (int i = 0; i < npar; i++) out.holdpeakloc[i] = -1;
    return 0;
  }
  // the genealogy ranges: the NUMTREEINT intervals as the reference steps
  // them (each starting one past the last one's end), then all
  int rlo[NUMTREEINT + 1], rhi[NUMTREEINT + 1];
  {
    int first = 0, last = Gs / NUMTREEINT;
    for (int j = 0; j < NUMTREEINT; j++) {
      rlo[j] = first;
      rhi[j] = last;
      first = last + 1;
      last += Gs / NUMTREEINT;
      if (last > Gs) last = Gs;
    }
    rlo[NUMTREEINT] = 0;
    rhi[NUMTREEINT] = Gs;
  }
  auto prior_lo = [&](int i) { return i < np ? in.theta_min[i] : in.mig_min[i - np]; };
  auto prior_hi = [&](int i) { return i < np ? in.theta_max[i] : in.mig_max[i - np]; };
  auto popmig_upper = [&](int t) {
    return in.mig_mean ? 20.0 * in.mig_mean[in.mterm[t]] : in.theta_max[in.mpop[t]] * in.mig_max[in.mterm[t]] / 2.0;
  };

  // run a set of searches to completion, round by round
  auto drive = [&](std::vector<Search *> &ss, const std::function<void(Search &, int)> &body) -> int {
    for (;;) {
      std::vector<MarginPeaksReq> reqs;
      std::vector<std::pair<Search *, double>> who;
      for (size_t k = 0; k < ss.size(); k++) {
        Search &s = *ss[k];
        if (s.done) continue;
        s.feed.want.clear();
        try {
          body(s, (int)k);
          s.done = true;
        } catch (Need &) {
          for (double x : s.feed.want) {
            MarginPeaksReq q;
            q.kind = s.kind;
            q.idx = s.idx;
            q.lo = rlo[s.range];
            q.hi = rhi[s.range];
            q.x = x;
            reqs.push_back(q);
            who.push_back({&s, x});
          }
        }
      }
      if (reqs.empty()) return 0;
      if (out.rounds >= 20000) return -1;  // a search that does not end
      std::vector<double> v(reqs.size());
      if (int r = eval(reqs, v)) return r;
      for (size_t k = 0; k < reqs.size(); k++) {
        Search &s = *who[k].first;
        // marginp / marginpopmig return the negated density; margincalc
        // log(density) - yadjust
        const double f = s.kind == K_LOG95 ? v[k] - s.yadjust : -v[k];
        s.feed.known[Feed::key(who[k].second)] = f;
      }
      out.rounds++;
    }
  };

  // 1. the brackets of every parameter over every range, and the 2NM
  //    terms' scan and golden section, together
  const int nR = NUMTREEINT + 1;
  std::vector<Search> sp((size_t)nR * npar), st((size_t)nR * nt);
  std::vector<Bracket> br((size_t)nR * npar);
  std::vector<Search *> all;
  for (int r = 0; r < nR; r++) {
    for (int i = 0; i < npar; i++) {
      Search &s = sp[(size_t)r * npar + i];
      s.kind = K_MARGINP;
      s.idx = i;
      s.range = r;
      s.lo = prior_lo(i);
      s.hi = prior_hi(i);
      all.push_back(&s);
    }
    for (int t = 0; t < nt; t++) {
      Search &s = st[(size_t)r * nt + t];
      s.kind = K_POPMIG;
      s.idx = t;
      s.range = r;
      s.lo = 0;
      s.hi = popmig_upper(t);
      all.push_back(&s);
    }
  }
  std::vector<double> pm_ml((size_t)nR * nt), pm_pk((size_t)nR * nt);
  int rc = drive(all, [&](Search &s, int) {
    if (s.kind == K_MARGINP) {
      const double prior = prior_hi(s.idx);
      Bracket b;
      double fa, fb, fc;
      b.ax = prior;
      b.bx = prior / 2;
      mnbrakmod(s, &b.ax, &b.bx, &b.cx, &fa, &fb, &fc);
      b.axt = b.ax;
      b.bxt = b.bx;
      b.cxt = b.cx;
      b.bx = prior / 2;
      b.ax = MINPARAMVAL;
      mnbrakmod(s, &b.ax, &b.bx, &b.cx, &fa, &fb, &fc);
      br[(size_t)s.range * npar + s.idx] = b;
      return;
    }
    // marginalopt_popmig for one term
    const double ub = popmig_upper(s.idx);
    std::vector<double> grid(POPMIG_MARGINBINS);
    for (int j = 0; j < POPMIG_MARGINBINS; j++) grid[j] = MINPARAMVAL + j * (ub / (double)POPMIG_MARGINBINS);
    s.feed.prefetch(grid);
    double maxf = 1e100, ax, bx, cx;
    int maxj = -1;
    for (int j = 0; j < POPMIG_MARGINBINS; j++) {
      const double fa = s.f(grid[j]);
      if (fa < maxf) {
        maxf = fa;
        maxj = j;
      }
    }
    if (maxj == 0) {
      ax = MINPARAMVAL;
      cx = MINPARAMVAL + ub / (double)POPMIG_MARGINBINS;
      bx = (ax + cx) / 2.0;
    } else if (maxj == POPMIG_MARGINBINS - 1) {
      ax = MINPARAMVAL + ((double)POPMIG_MARGINBINS - 1) * (ub / (double)POPMIG_MARGINBINS);
      bx = MINPARAMVAL + ((double)POPMIG_MARGINBINS - 2) * (ub / (double)POPMIG_MARGINBINS);
      cx = ub;
    } else {
      bx = MINPARAMVAL + ((double)maxj - 1) * (ub / (double)POPMIG_MARGINBINS);
      cx = MINPARAMVAL + ((double)maxj + 1) * (ub / (double)POPMIG_MARGINBINS);
      ax = MINPARAMVAL + ((double)maxj) * (ub / (double)POPMIG_MARGINBINS);
    }
    double xmax;
    const double ml = -goldenmod(s, ax, bx, cx, 1e-7, &xmax);
    pm_ml[(size_t)s.range * nt + s.idx] = ml;
    pm_pk[(size_t)s.range * nt + s.idx] = xmax;
  });
  if (rc) return rc;

  // 2. marginalopt's bracket comparison (:208-258), parameter by parameter
  //    as the reference runs them: its min0/max0/min1/max1 keep the previous
  //    parameter's values where ties leave them unset (they start at 0 here),
  //    and the clamps to the prior move the second bracket's ends
  std::vector<char> run_golden((size_t)nR * npar, 0);
  for (int r = 0; r < nR; r++) {
    double max0 = 0, min0 = 0, max1 = 0, min1 = 0;
    for (int i = 0; i < npar; i++) {
      Bracket &b = br[(size_t)r * npar + i];
      const double prior = prior_hi(i);
      double &axt = b.axt, &bxt = b.bxt, &cxt = b.cxt, &ax = b.ax, &bx = b.bx, &cx = b.cx;
      if (axt < bxt && axt < cxt) min0 = axt;
      if (bxt < axt && bxt < cxt) min0 = bxt;
      if (cxt < axt && cxt < bxt) min0 = cxt;
      if (axt > bxt && axt > cxt) {
        if (axt > prior) axt = prior;
        max0 = axt;
      }
      if (bxt > axt && bxt > cxt) {
        if (bxt > prior) bxt = prior;
        max0 = bxt;
      }
      if (cxt > axt && cxt > bxt) {
        if (cxt > prior) cxt = prior;
        max0 = cxt;
      }
      if (ax < bx && ax < cx) min1 = ax;
      if (bx < ax && bx < cx) min1 = bx;
      if (cx < ax && cx < bx) min1 = cx;
      if (ax > bx && ax > cx) max1 = ax;
      {  // unconditional in the reference: a brace block after the if
        if (ax > prior) ax = prior;
        max1 = ax;
      }
      if (bx > ax && bx > cx) {
        if (bx > prior) bx = prior;
        max1 = bx;
      }
      if (cx > ax && cx > bx) {
        if (cx > prior) cx = prior;
        max1 = cx;
      }
      if (max0 <= min1 || max1 <= min0) {
        out.peakloc[(size_t)r * npar + i] = -1;
        out.mlval[(size_t)r * npar + i] = NAN;
      } else {
        run_golden[(size_t)r * npar + i] = 1;
      }
    }
  }

  // 3. goldenmod where the brackets overlap
  std::vector<Search *> gold;
  for (size_t k = 0; k < sp.size(); k++)
    if (run_golden[k]) {
      sp[k].done = false;
      gold.push_back(&sp[k]);
    }
  rc = drive(gold, [&](Search &s, int) {
    const Bracket &b = br[(size_t)s.range * npar + s.idx];
    double xmax;
    const double ml = -goldenmod(s, b.ax, b.bx, b.cx, 1e-7, &xmax);
    out.mlval[(size_t)s.range * npar + s.idx] = ml;
    out.peakloc[(size_t)s.range * npar + s.idx] = xmax;
  });
  if (rc) return rc;

  // 4. the likelihood-ratio tests (:450-469) and the 95% limits (:596-652)
  const double *pk = out.peakloc + (size_t)NUMTREEINT * npar, *ml = out.mlval + (size_t)NUMTREEINT * npar;
  std::vector<Search> tests((size_t)nm + nt), lim(2 * (size_t)npar);
  std::vector<Search *> last;
  for (int i = 0; i < nm; i++) {
    Search &s = tests[i];
    s.kind = K_MARGINP;
    s.idx = np + i;
    s.range = NUMTREEINT;
    s.lo = prior_lo(np + i);
    s.hi = prior_hi(np + i);
    last.push_back(&s);
  }
  for (int t = 0; t < nt; t++) {
    Search &s = tests[nm + t];
    s.kind = K_POPMIG_UNIFORM;
    s.idx = t;
    s.range = NUMTREEINT;
    s.lo = 0;
    s.hi = in.theta_max[in.mpop[t]] * in.mig_max[in.mterm[t]] / 2.0;
    last.push_back(&s);
  }
  for (int i = 0; i < npar; i++) {
    out.lo95[i] = out.hi95[i] = NAN;
    if (!(pk[i] >= 0)) continue;
    for (int ul = 0; ul < 2; ul++) {
      Search &s = lim[2 * (size_t)i + ul];
      s.kind = K_LOG95;
      s.idx = i;
      s.range = NUMTREEINT;
      s.ul = ul;
      s.yadjust = log(ml[i]) - DOWN95;
      last.push_back(&s);
    }
  }
  rc = drive(last, [&](Search &s, int) {
    if (s.kind == K_LOG95) {
      const int i = s.idx, ul = s.ul;
      const double x1 = ul == 0 ? MINPARAMVAL : pk[i], x2 = ul == 0 ? pk[i] : prior_hi(i);
      (ul == 0 ? out.lo95 : out.hi95)[i] = marginbis(s, x1, x2);
      return;
    }
    if (s.kind == K_MARGINP) {
      const int i = s.idx - np;
      const double maxp = -s.f(pk[np + i]), max0p = -s.f(MINPARAMVAL);
      out.migtest[i] = 2 * log(maxp / max0p);
      return;
    }
    const double maxp = -s.f(pm_pk[(size_t)NUMTREEINT * nt + s.idx]), max0p = -s.f(MINPARAMVAL);
    out.pm_test[s.idx] = 2 * log(maxp / max0p);
  });
  if (rc) return rc;
  for (int k = 0; k < nR * nt; k++) {
    out.pm_mlval[k] = pm_ml[k];
    out.pm_peakloc[k] = pm_pk[k];
  }
  for (int i = 0; i < npar; i++) out.holdpeakloc[i] = (float)(pk[i] < 0 ? MINPARAMVAL : pk[i]);
  return 0;
}
