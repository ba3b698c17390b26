// jointpeaks.cu -- the L-mode peak search: differential evolution over the
// jointp surface (jointfind.cpp:594-812), with every generation's trial
// vectors evaluated in one batched surface call on the GPU.
//
// The reference evaluates jointp once per trial vector, in sequence, but the
// population is only updated after the whole generation, so evaluating all
// trial vectors together is the same algorithm.  The uniforms are drawn from
// the caller's MT19937 state in the reference's order -- per member A, B, C
// (randposint), then per active parameter u and, when the trial leaves the
// bounds, one more -- so with the reference's own jointp (IMA_SURF_COMPAT)
// the search follows the reference's trajectory.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "ima_gpu.h"

namespace {

// jointfind.cpp:136-147 and imamp.hpp:130
constexpr double MINPARAMVAL = 0.0000001;
constexpr double STARTHI = 1E200, STARTLOW = -1E200;
constexpr double SPREADTOL = 1.0e-7;  // stop a search when the population's values agree
constexpr double PLOOPTOL = 1.0e-6;   // two searches found the same peak
constexpr int LOOPMATCHCRITERIA = 2;  // times the best peak must be found
constexpr int MAXRESTART = 10;
constexpr double RECRATE = 0.9;       // crossover rate
constexpr double FWEIGHT = 0.8;       // difference weight
constexpr int MAXGENERATIONS = 1000000;  // guard against a surface that never converges

// MT19937 (Matsumoto & Nishimura 1998), the generator of utilities.cpp.
uint32_t mt_next(ima_mt19937 *g)
{
  constexpr int N = 624, M = 397;
  if (g->mti >= N) {
    for (int k = 0; k < N; k++) {
      const uint32_t y = (g->mt[k] & 0x80000000u) | (g->mt[(k + 1) % N] & 0x7fffffffu);
      g->mt[k] = g->mt[(k + M) % N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    g->mti = 0;
  }
  uint32_t y = g->mt[g->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double uniform(ima_mt19937 *g) { return ((double)mt_next(g) + 0.5) * (1.0 / 4294967296.0); }
int randposint(ima_mt19937 *g, int n) { return (int)std::floor(uniform(g) * n); }

struct Search {
  ima_ctx *c;
  int n, modeltype, method, dep, r0, jmax;
  const double *xmap;
  std::vector<double> lo, hi, pop, trial, full, q;
  double &P(int i, int j) { return pop[(size_t)i * (n + 1) + j]; }
  double &T(int i, int j) { return trial[(size_t)i * (n + 1) + j]; }

  // the full parameter vector jointp sees (mapvals, jointfind.cpp:555-566).
  // Parameters outside the model (population sizes under modeltype 2,
  // migration rates under 1) hold -1 or 0 here; jointp ignores them, and
  // they get a positive placeholder because the surface checks every value.
  void to_full(const double *v, double *out) const
  {
    for (int i = 0; i < n; i++) {
      out[i] = xmap ? (xmap[i] < 0 ? -xmap[i] : v[(int)xmap[i]]) : v[i];
      if (!(out[i] > 0.0)) out[i] = 1.0;
    }
  }

  // evaluates rows [0, dep) of vals (pop or trial) into their last column
  int evaluate(std::vector<double> &vals)
  {
    for (int i = 0; i < dep; i++) to_full(&vals[(size_t)i * (n + 1)], &full[(size_t)i * n]);
    int r = ima_gpu_surface_eval(c, dep, full.data(), modeltype, method, q.data(), nullptr);
    if (r) return r;
    for (int i = 0; i < dep; i++) vals[(size_t)i * (n + 1) + n] = q[i];
    return IMA_OK;
  }

  // startpop (jointfind.cpp:658-702)
  int startpop(ima_mt19937 *g)
  {
    for (int i = 0; i < dep; i++)
      for (int j = 0; j < n; j++) P(i, j) = (j >= r0 && j < jmax) ? lo[j] + uniform(g) * (hi[j] - lo[j]) : -1.0;
    return evaluate(pop);
  }

  // nextgen (jointfind.cpp:594-656)
  int nextgen(ima_mt19937 *g, double *lowpd, double *hipd)
  {
    *lowpd = STARTHI;
    *hipd = STARTLOW;
    for (int i = 0; i < dep; i++) {
      const int A = randposint(g, dep), B = randposint(g, dep), Cv = randposint(g, dep);
      for (int j = r0; j < jmax; j++) {
        if (uniform(g) < RECRATE) {
          double t = P(Cv, j) + FWEIGHT * (P(A, j) - P(B, j));
          if (t < lo[j]) t = P(Cv, j) - uniform(g) * (P(Cv, j) - lo[j]);  // part of the way to the bound
          if (t > hi[j]) t = P(Cv, j) + uniform(g) * (hi[j] - P(Cv, j));
          T(i, j) = t;
        } else {
          T(i, j) = P(i, j);
        }
      }
    }
    int r = evaluate(trial);
    if (r) return r;
    for (int i = 0; i < dep; i++) {
      if (T(i, n) < P(i, n))
        for (int j = 0; j <= n; j++) P(i, j) = T(i, j);
      if (P(i, n) < *lowpd) *lowpd = P(i, n);
      if (P(i, n) > *hipd) *hipd = P(i, n);
    }
    return IMA_OK;
  }
};

}  // namespace

extern "C" void ima_mt19937_seed(ima_mt19937 *g, uint32_t seed)
{
  if (!g) return;
  g->mt[0] = seed;
  for (int i = 1; i < 624; i++) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
  g->mti = 624;
}

extern "C" double ima_mt19937_uniform(ima_mt19937 *g) { return g ? uniform(g) : 0.0; }

extern "C" int ima_gpu_modelloop(ima_ctx *c, int modeltype, const double *upper, int popsizemultiplier,
                                 const double *xmap, int nested, int method, ima_mt19937 *rng, double *best,
                                 double *ess, int *generations, int *restarts)
{
  int G = 0, np = 0, nm = 0, npops = 0;
  int r = ima_gpu_surface_info(c, &G, &np, &nm, &npops);
  if (r) return r;
  if (!upper || !rng || !best || popsizemultiplier < 1 || modeltype < 0 || modeltype > 2 ||
      (xmap && (nested < 1 || modeltype == 2)))
    return IMA_ERR_ARG;
  Search s;
  s.c = c;
  s.n = np + nm;
  s.modeltype = modeltype;
  s.method = method;
  s.xmap = xmap;
  s.r0 = modeltype == 2 ? np : 0;
  int modelparams = modeltype == 0 ? s.n : (modeltype == 1 ? np : nm);
  if (xmap) {
    for (int i = 0; i < s.n; i++)
      if (xmap[i] >= nested || (xmap[i] < 0 && !(-xmap[i] > 0.0))) return IMA_ERR_ARG;
    modelparams = nested;
  }
  s.jmax = s.r0 + modelparams;
  s.dep = modelparams * popsizemultiplier;
  s.lo.assign(s.n, 0.0);
  s.hi.assign(s.n, 0.0);
  if (!xmap) {
    for (int j = 0; j < s.n; j++) {
      s.lo[j] = MINPARAMVAL;
      s.hi[j] = upper[j];
    }
  } else {
    // reversemapvals (jointfind.cpp:540-552): the first full parameter that
    // maps to each nested index gives its bounds
    for (int i = 0, k = 0; i < s.n; i++)
      if (k == (int)xmap[i]) {
        s.lo[k] = MINPARAMVAL;
        s.hi[k] = upper[i];
        k++;
      }
  }
  s.pop.assign((size_t)s.dep * (s.n + 1), 0.0);
  s.trial.assign((size_t)s.dep * (s.n + 1), 0.0);
  s.full.assign((size_t)s.dep * s.n, 1.0);
  s.q.assign(s.dep, 0.0);
  std::vector<double> bestv(s.n + 1, 0.0);

  // modelloop (jointfind.cpp:746-812)
  int gens = 0, nrun = 0;
  double global_pd = STARTHI;
  if ((r = s.startpop(rng))) return r;
  for (int i = 0; i < s.dep; i++)
    if (s.P(i, s.n) < global_pd) global_pd = s.P(i, s.n);
  int newstart = 0, countloop = 0;
  do {
    if (newstart > 0 && (r = s.startpop(rng))) return r;
    double lowpd, hipd;
    do {  // difeloop (jointfind.cpp:705-720)
      if ((r = s.nextgen(rng, &lowpd, &hipd))) return r;
      if (++gens > MAXGENERATIONS) return IMA_ERR_DATA;
    } while (hipd - lowpd > SPREADTOL);
    nrun++;
    if (std::fabs(lowpd - global_pd) < PLOOPTOL) countloop++;
    else if (lowpd < global_pd) countloop = 0;
    if (lowpd < global_pd) {  // copybest (jointfind.cpp:723-738)
      double t = STARTHI;
      int k = 0;
      for (int i = 0; i < s.dep; i++)
        if (s.P(i, s.n) < t) {
          t = s.P(i, s.n);
          k = i;
        }
      for (int j = 0; j <= s.n; j++) bestv[j] = s.P(k, j);
      bestv[s.n] = t;
      global_pd = lowpd;
    }
    newstart++;
  } while (countloop < LOOPMATCHCRITERIA && newstart < MAXRESTART);

  // the peak in the full model's parameters, and its effective sample size
  std::vector<double> fb(s.n);
  for (int i = 0; i < s.n; i++) fb[i] = xmap ? (xmap[i] < 0 ? -xmap[i] : bestv[(int)xmap[i]]) : bestv[i];
  for (int i = 0; i < s.n; i++) best[i] = fb[i];
  best[s.n] = bestv[s.n];
  if (ess) {
    std::vector<double> x(fb);
    for (int i = 0; i < s.n; i++)
      if (!(x[i] > 0.0)) x[i] = 1.0;
    double qv = 0.0;
    if ((r = ima_gpu_surface_eval(c, 1, x.data(), modeltype, method, &qv, ess))) return r;
  }
  if (generations) *generations = gens;
  if (restarts) *restarts = nrun;
  return IMA_OK;
}
