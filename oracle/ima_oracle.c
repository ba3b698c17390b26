/*
 * ima_oracle.c -- CPU restatement of IMa2p's hot-path arithmetic (FP64).
 *
 * TEST INFRASTRUCTURE ONLY: the parity checker for the GB300 kernels.  Only
 * tests/, __graft_entry__.smoke() and bench.py's CPU legs load it; the
 * product library never links or calls it.
 *
 * Each block names the reference function it restates (paths relative to
 * the IMa2p tree).  The restatement is pinned against the compiled
 * reference (oracle/_ref/imaref) by tests/test_oracle_vs_ref.py and against
 * the committed fixtures in tests/golden/.
 */
#include "ima_oracle.h"
#include <float.h>
#include <ctype.h>
#include <stdio.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#define ORA_REJECT_IS (-1000000000.0) /* imamp.hpp:157 */
#define ORA_BESSI_MIN (-1e+100)       /* imamp.hpp:173 */
#define ORA_LOG2 0.69314718055994530941723212146
#define ORA_LOG10 2.3025850929940456840

/* ======================================================================
 * Infinite sites.  labelgtree (calc_prob_data.cpp:537-581): starting at a
 * tip, walk towards the root, merging the tip's 0/1 label into each parent
 * according to the sister's label (-1 unset, 2 mixed); stop as soon as a
 * parent's label is left unchanged.
 * ==================================================================== */
static void is_walk(int8_t *mut, const int *up0, const int *up1,
                    const int *down, int e)
{
  for (;;) {
    int p = down[e];
    if (p < 0) return;
    int sis = (up0[p] == e) ? up1[p] : up0[p];
    int8_t me = mut[e], mp = mut[p], ms = mut[sis];
    if (mp != me) {
      if (me == 2)
        mut[p] = (ms != -1) ? ms : 2;
      else if (ms != -1 && ms != 2 && ms != me)
        mut[p] = 2;
      else
        mut[p] = me;
    } else if (mp == 2 && ms != -1 && ms != 2) {
      mut[p] = ms;
    } else {
      return;
    }
    e = p;
  }
}

static void is_label_site(int n, int S, int site, const int8_t *seq,
                          const int *up0, const int *up1, const int *down,
                          int8_t *mut)
{
  int nl = 2 * n - 1;
  for (int j = 0; j < n; j++) mut[j] = seq[(size_t)j * S + site];
  for (int j = n; j < nl; j++) mut[j] = -1;
  for (int j = 0; j < n; j++) is_walk(mut, up0, up1, down, j);
}

static inline int is_split(const int8_t *mut, int a, int b)
{
  return (mut[a] == 0 && mut[b] == 1) || (mut[a] == 1 && mut[b] == 0);
}

static inline double branch_len(const int *up0, const double *time, int c)
{
  int u = up0[c];
  return (u == -1) ? time[c] : time[c] - time[u];
}

int ora_is_sumlogk(int n, int S, const int8_t *seq, const int *up0,
                   const int *up1, const int *down, double *sumlogk,
                   int *counts)
{
  int nl = 2 * n - 1;
  int8_t *mut = (int8_t *)malloc((size_t)nl);
  memset(counts, 0, sizeof(int) * (size_t)(n - 1));
  *sumlogk = 0.0;
  for (int site = 0; site < S; site++) {
    is_label_site(n, S, site, seq, up0, up1, down, mut);
    int hit = -1;
    for (int node = n; node < nl; node++) {
      if (is_split(mut, up0[node], up1[node])) {
        if (hit != -1) { free(mut); return 1; }
        hit = node;
        counts[node - n]++;
      }
    }
    if (hit == -1) { free(mut); return 2; }
  }
  double sum = 0.0;
  for (int i = 0; i < n - 1; i++) {
    double f = 1.0;
    for (int j = 1; j <= counts[i]; j++) f *= (double)j;
    sum += log(f);
  }
  *sumlogk = sum;
  free(mut);
  return 0;
}

double ora_is_likelihood(int n, int S, const int8_t *seq, const int *up0,
                         const int *up1, const int *down, const double *time,
                         double length, double u, double sumlogk,
                         int *site_node, int *status)
{
  int nl = 2 * n - 1;
  int8_t *mut = (int8_t *)malloc((size_t)nl);
  double p = -length * u;
  *status = 0;
  for (int site = 0; site < S; site++) {
    is_label_site(n, S, site, seq, up0, up1, down, mut);
    int hit = -1;
    double t = 0.0;
    for (int node = n; node < nl; node++) {
      int a = up0[node], b = up1[node];
      if (!is_split(mut, a, b)) continue;
      if (hit != -1) {
        free(mut);
        *status = 1;
        if (site_node) site_node[site] = -2;
        return ORA_REJECT_IS;
      }
      if (down[node] == -1)
        t = branch_len(up0, time, a) + branch_len(up0, time, b);
      else if (mut[down[node]] == mut[a])
        t = branch_len(up0, time, b);
      else
        t = branch_len(up0, time, a);
      hit = node;
    }
    if (site_node) site_node[site] = hit;
    if (hit == -1) { free(mut); *status = 2; return 0.0; }
    p = p + log(t * u);
  }
  free(mut);
  return p - sumlogk;
}

/* ======================================================================
 * HKY85 pruning (makefrac, calc_prob_data.cpp:118-471; getstandfactor
 * :473-493; likelihoodHKY :583-607).  P_jk(b) with Pi_k / A_k taken from
 * the purine/pyrimidine class of the target state k.
 * ==================================================================== */
double ora_hky_standfactor(const double *pi, double kappa)
{
  double p = 0.0;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      if (i == j) continue;
      if (i + j == 2 || i + j == 4) p += pi[i] * pi[j] * kappa;
      else p += pi[i] * pi[j];
    }
  return p;
}

static void hky_pmatrix(const double *pi, double kappa, double b, double P[4][4])
{
  double e1 = exp(-b);
  for (int k = 0; k < 4; k++) {
    double Pk = (k == 0 || k == 2) ? pi[0] + pi[2] : pi[1] + pi[3];
    double A = 1.0 + Pk * (kappa - 1.0);
    double e2 = exp(-b * A);
    for (int j = 0; j < 4; j++) {
      if (j == k)
        P[j][k] = pi[k] + pi[k] * e1 * (1.0 / Pk - 1.0) + e2 * ((Pk - pi[k]) / Pk);
      else if (j + k == 2 || j + k == 4)
        P[j][k] = pi[k] + pi[k] * e1 * (1.0 / Pk - 1.0) - (pi[k] / Pk) * e2;
      else
        P[j][k] = pi[k] * (1.0 - e1);
    }
  }
}

typedef struct {
  int n, S;
  const int8_t *seq;
  const double *pi;
  const int *up0, *up1;
  const double *time;
  double mu, kappa;
  const int *e;
  double *frac, *newfrac, *sf;
} hky_job;

/* returns 1 when `node` was recomputed or is itself on the dirty list */
static int hky_visit(hky_job *J, int node)
{
  const int *e = J->e;
  int ret = (node == e[0] || node == e[1] || node == e[2] || node == e[3] || e[0] == -1);
  int c[2] = {J->up0[node], J->up1[node]};
  if (c[0] == -1) return ret;
  int fresh[2];
  for (int k = 0; k < 2; k++) {
    fresh[k] = hky_visit(J, c[k]);
    if (fresh[k]) ret = 1;
  }
  if (!ret) return 0;
  int S = J->S;
  double P[2][4][4];
  for (int k = 0; k < 2; k++)
    hky_pmatrix(J->pi, J->kappa, J->mu * branch_len(J->up0, J->time, c[k]), P[k]);
  for (int i = 0; i < S; i++) {
    double v[2][4];
    double scale = 0.0;
    for (int k = 0; k < 2; k++) {
      int ch = c[k];
      if (J->up0[ch] == -1) {
        int s = J->seq[(size_t)ch * S + i];
        for (int j = 0; j < 4; j++) v[k][j] = P[k][j][s];
      } else {
        const double *L = (fresh[k] ? J->newfrac : J->frac) + ((size_t)ch * S + i) * 4;
        for (int j = 0; j < 4; j++)
          v[k][j] = P[k][j][0] * L[0] + P[k][j][1] * L[1] + P[k][j][2] * L[2] + P[k][j][3] * L[3];
        scale += J->sf[(size_t)ch * S + i];
      }
    }
    double *out = J->newfrac + ((size_t)node * S + i) * 4;
    double mx = 0.0;
    for (int j = 0; j < 4; j++) {
      out[j] = v[0][j] * v[1][j];
      if (out[j] > mx) mx = out[j];
    }
    for (int j = 0; j < 4; j++) out[j] /= mx;
    J->sf[(size_t)node * S + i] = scale + log(mx);
  }
  return 1;
}

double ora_hky_likelihood(int n, int S, int totsites, const int8_t *seq,
                          const int *mult, const double *pi, const int *up0,
                          const int *up1, const int *down, int root,
                          const double *time, double u, double kappa,
                          const int *e, double *frac, double *newfrac,
                          double *sf, double *oldsf)
{
  (void)down; (void)oldsf;
  hky_job J;
  J.n = n; J.S = S; J.seq = seq; J.pi = pi; J.up0 = up0; J.up1 = up1;
  J.time = time; J.kappa = kappa; J.e = e;
  J.frac = frac; J.newfrac = newfrac; J.sf = sf;
  J.mu = u / ((double)totsites * ora_hky_standfactor(pi, kappa));
  for (int i = n; i < 2 * n - 1; i++) newfrac[(size_t)i * S * 4] = -1.0;
  hky_visit(&J, root);
  double p = 0.0;
  for (int i = 0; i < S; i++) {
    const double *L = newfrac + ((size_t)root * S + i) * 4;
    double f = 0.0;
    for (int j = 0; j < 4; j++) f += pi[j] * L[j];
    p += mult[i] * (log(f) + sf[(size_t)root * S + i]);
  }
  return p;
}

void ora_hky_copyfraclike(int n, int S, const double *newfrac, double *frac)
{
  for (int i = n; i < 2 * n - 1; i++) {
    const double *src = newfrac + (size_t)i * S * 4;
    if (src[0] != -1.0) memcpy(frac + (size_t)i * S * 4, src, sizeof(double) * 4 * (size_t)S);
  }
}

void ora_hky_storescalefactors(int n, int S, const double *sf, double *oldsf)
{
  memcpy(oldsf + (size_t)n * S, sf + (size_t)n * S, sizeof(double) * (size_t)(n - 1) * S);
}

void ora_hky_restorescalefactors(int n, int S, double *sf, const double *oldsf)
{
  memcpy(sf + (size_t)n * S, oldsf + (size_t)n * S, sizeof(double) * (size_t)(n - 1) * S);
}

/* ======================================================================
 * Bessel I_n as the reference evaluates it: Abramowitz & Stegun 9.8.1-9.8.4
 * polynomials for n = 0, 1 (utilities.cpp:54-124) and Miller's downward
 * recurrence from j = 2(n + floor(sqrt(40 n))) with 1e10 rescaling for
 * n >= 2 (utilities.cpp:1449-1496).
 * ==================================================================== */
static const double AS_I0_SMALL[7] = {1.0, 3.5156229, 3.0899424, 1.2067492,
                                      0.2659732, 0.360768e-1, 0.45813e-2};
static const double AS_I0_LARGE[9] = {0.39894228, 0.1328592e-1, 0.225319e-2,
                                      -0.157565e-2, 0.916281e-2, -0.2057706e-1,
                                      0.2635537e-1, -0.1647633e-1, 0.392377e-2};
static const double AS_I1_SMALL[7] = {0.5, 0.87890594, 0.51498869, 0.15084934,
                                      0.2658733e-1, 0.301532e-2, 0.32411e-3};
static const double AS_I1_LARGE[9] = {0.39894228, -0.3988024e-1, -0.362018e-2,
                                      0.163801e-2, -0.1031555e-1, 0.2282967e-1,
                                      -0.2895312e-1, 0.1787654e-1, -0.420059e-2};

static double horner(const double *c, int m, double y)
{
  double r = c[m - 1];
  for (int k = m - 2; k >= 0; k--) r = c[k] + y * r;
  return r;
}

double ora_bessi0(double x)
{
  double ax = fabs(x);
  if (ax < 3.75) {
    double y = x / 3.75;
    y *= y;
    return horner(AS_I0_SMALL, 7, y);
  }
  double y = 3.75 / ax;
  return (exp(ax) / sqrt(ax)) * horner(AS_I0_LARGE, 9, y);
}

double ora_bessi1(double x)
{
  double ax = fabs(x), ans;
  if (ax < 3.75) {
    double y = x / 3.75;
    y *= y;
    ans = ax * horner(AS_I1_SMALL, 7, y);
  } else {
    double y = 3.75 / ax;
    /* the reference evaluates the tail (coefficients 5..8) first */
    double tail = AS_I1_LARGE[5] + y * (AS_I1_LARGE[6] + y * (AS_I1_LARGE[7] + y * AS_I1_LARGE[8]));
    ans = AS_I1_LARGE[0] + y * (AS_I1_LARGE[1] + y * (AS_I1_LARGE[2] + y * (AS_I1_LARGE[3] + y * (AS_I1_LARGE[4] + y * tail))));
    ans *= (exp(ax) / sqrt(ax));
  }
  return x < 0.0 ? -ans : ans;
}

double ora_bessi(int n, double x)
{
  n = abs(n);
  if (x > 700) return DBL_MAX / 1e10;
  if (n == 0) return ora_bessi0(x);
  if (n == 1) return ora_bessi1(x);
  if (x == 0.0) return 0.0;
  double tox = 2.0 / fabs(x);
  double bip = 0.0, ans = 0.0, bi = 1.0;
  for (int j = 2 * (n + (int)sqrt(40.0 * n)); j > 0; j--) {
    double bim = bip + j * tox * bi;
    bip = bi;
    bi = bim;
    if (fabs(bi) > 1.0e10) {
      ans *= 1.0e-10;
      bi *= 1.0e-10;
      bip *= 1.0e-10;
    }
    if (j == n) ans = bip;
  }
  ans *= ora_bessi0(x) / bi;
  return (x < 0.0 && (n & 1)) ? -ans : ans;
}

double ora_sw_branch_term(int d, double t, double u)
{
  double b = ora_bessi(d, t * u);
  if (!(b > 0.0)) return ORA_BESSI_MIN;
  return -(t * u) + log(b);
}

double ora_sw_likelihood(int n, const int *A, const int *down, const int *up0,
                         const double *time, double u, double tr,
                         double *dlikeA)
{
  int nl = 2 * n - 1, zero = 0;
  double like = 0.0;
  for (int i = 0; i < nl; i++) {
    if (down[i] == -1) { if (dlikeA) dlikeA[i] = 0.0; continue; }
    int d = A[i] - A[down[i]];
    double t = (up0[i] == -1) ? time[i] * tr : tr * (time[i] - time[up0[i]]);
    double b = ora_bessi(d, t * u);
    double v;
    if (!(b > 0.0)) { zero = 1; v = ORA_BESSI_MIN; }
    else v = -(t * u) + log(b);
    if (dlikeA) dlikeA[i] = v;
    like += v;
  }
  return zero ? -DBL_MAX : like;
}

/* ======================================================================
 * MT19937 (Matsumoto & Nishimura 1998), as vendored at utilities.cpp:323-427
 * ==================================================================== */
void ora_mt_seed(ora_mt *s, uint32_t seed)
{
  s->mt[0] = seed;
  for (int i = 1; i < 624; i++)
    s->mt[i] = 1812433253u * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (uint32_t)i;
  s->mti = 624;
}

uint32_t ora_mt_u32(ora_mt *s)
{
  if (s->mti >= 624) {
    for (int k = 0; k < 624; k++) {
      uint32_t y = (s->mt[k] & 0x80000000u) | (s->mt[(k + 1) % 624] & 0x7fffffffu);
      s->mt[k] = s->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    s->mti = 0;
  }
  uint32_t y = s->mt[s->mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

double ora_mt_uniform(ora_mt *s)
{
  return ((double)ora_mt_u32(s) + 0.5) * 2.32830643653869628906e-10;
}

void ora_mt_fill_u32(uint32_t seed, int count, uint32_t *out)
{
  ora_mt s;
  ora_mt_seed(&s, seed);
  for (int i = 0; i < count; i++) out[i] = ora_mt_u32(&s);
}

/* ======================================================================
 * MC3 (setheat swapchains.cpp:71-178; swapchains :526-653; swapweight :12-34)
 * ==================================================================== */
int ora_setheat(int nchains, double h1, double h2, int heatmode, double *beta,
                double *allbetas)
{
  int N = nchains;
  if (N == 1) { beta[0] = allbetas[0] = 1.0; return 0; }
  for (int i = 0; i < N; i++) {
    if (heatmode == 0) allbetas[i] = 1.0 / (1.0 + h1 * i);
    else if (heatmode == 1) allbetas[i] = 1 - (1 - h2) * (i) * pow(h1, (double)(N - 1 - i)) / (double)(N - 1);
    else allbetas[i] = 1.0 - i * (1.0 / (N - 1));
  }
  double hl = (heatmode == 0 && h1 < 0.05) ? 0.05 : h1;
  for (int i = 0; i < N; i++) {
    if (heatmode == 0) beta[i] = 1.0 / (1.0 + hl * i);
    else if (heatmode == 1) beta[i] = 1 - (1 - h2) * (i) * pow(h1, (double)(N - 1 - i)) / (double)(N - 1);
    else beta[i] = 1.0 - i * (1.0 / (N - 1));
    if (beta[i] <= 0.0 || beta[i] > 1.0) return 1;
  }
  return 0;
}

void ora_chain_sums(int nchains, int nloci, const double *pdg,
                    const double *probg, int include_probg, double *S)
{
  for (int c = 0; c < nchains; c++) {
    double s = 0.0;
    for (int l = 0; l < nloci; l++) s += pdg[(size_t)c * nloci + l];
    if (include_probg) s += probg[c];
    S[c] = s;
  }
}

static int beta_index(int N, const double *allbetas, double b)
{
  for (int p = 0; p < N; p++)
    if (allbetas[p] == b) return p;
  return -1;
}

int ora_swapchains(int nchains, int swaptries, const double *S, double *beta,
                   const double *allbetas, const double *u, int *used,
                   int *swapcount, int *tempcount, int *accepted_pairs)
{
  int n = nchains, k = 0, swap0ok = 0;
  for (int t = 0; t < swaptries; t++) {
    int ci, cj, cjmin, cjrange;
    do { ci = (int)(u[k++] * n); } while (ci < 0 || ci >= n);
    if (n < 2 * 7 + 3) { cjmin = 0; cjrange = n; }
    else {
      cjmin = ci - 7 > 0 ? ci - 7 : 0;
      cjrange = (n < ci + 7 ? n : ci + 7) - cjmin;
    }
    do { cj = cjmin + (int)(u[k++] * cjrange); } while (cj == ci || cj < 0 || cj >= n);
    int p = beta_index(n, allbetas, beta[ci]);
    int q = beta_index(n, allbetas, beta[cj]);
    int hi = ci > cj ? ci : cj, lo = ci > cj ? cj : ci;
    int phi = p > q ? p : q, plo = p > q ? q : p;
    if (p >= 0 && q >= 0) tempcount[phi * n + plo]++;
    swapcount[hi * n + lo]++;
    double w = exp((beta[ci] - beta[cj]) * (S[cj] - S[ci]));
    int acc = 0;
    if (w >= 1.0) acc = 1;
    else if (w > u[k++]) acc = 1;
    if (accepted_pairs) {
      accepted_pairs[3 * t] = ci;
      accepted_pairs[3 * t + 1] = cj;
      accepted_pairs[3 * t + 2] = acc;
    }
    if (acc) {
      double bt = beta[ci];
      beta[ci] = beta[cj];
      beta[cj] = bt;
      swapcount[lo * n + hi]++;
      if (p >= 0 && q >= 0) tempcount[plo * n + phi]++;
      if (ci == 0 || cj == 0) swap0ok = 1;
    }
  }
  *used = k;
  return swap0ok;
}

/* ======================================================================
 * L-mode surface (jointp, jointfind.cpp:885-1047; eexp utilities.cpp:1507-1540)
 * ==================================================================== */
void ora_gsamp_offsets(int np, int nm, int *ccp, int *fcp, int *hccp, int *mcp,
                       int *fmp, int *qip, int *mip, int *pdgp, int *probgp)
{
  *ccp = 0;
  *fcp = np;
  *hccp = 2 * np;
  *mcp = 3 * np;
  *fmp = 3 * np + nm;
  *qip = 3 * np + 2 * nm;
  *mip = 4 * np + 2 * nm;
  *pdgp = 4 * np + 3 * nm;
  *probgp = *pdgp + 1;
}

void ora_surface_p(int G, int rowlen, const float *g, int np, int nm,
                   int npops, int modeltype, const double *lognorm,
                   const double *x, double *pout)
{
  int ccp, fcp, hccp, mcp, fmp, qip, mip, pdgp, probgp;
  ora_gsamp_offsets(np, nm, &ccp, &fcp, &hccp, &mcp, &fmp, &qip, &mip, &pdgp, &probgp);
  int lo = 0, hi = np + nm;
  if (modeltype == 1) hi = np;
  if (modeltype == 2) lo = np;
  double logx[64], divx[64], l2d[64];
  for (int i = 0; i < np; i++) l2d[i] = ORA_LOG2 - log(x[i]);
  for (int i = lo; i < hi; i++) { logx[i] = log(x[i]); divx[i] = 1.0 / x[i]; }
  for (int gi = 0; gi < G; gi++) {
    const float *r = g + (size_t)gi * rowlen;
    double p;
    if (lognorm) p = lognorm[gi];
    else if (npops == 2) p = -r[probgp];
    else {
      double s = 0.0;
      if (modeltype == 1) for (int i = 0; i < np; i++) s += r[qip + i];
      else for (int i = 0; i < nm; i++) s += r[mip + i];
      p = -s;
    }
    for (int i = lo; i < hi; i++) {
      if (i < np) {
        double dg = 2.0 * r[fcp + i];
        p += r[ccp + i] * l2d[i] - r[hccp + i] - dg * divx[i];
      } else {
        int i1 = i - np;
        p += r[mcp + i1] * logx[i] - r[fmp + i1] * x[i];
      }
    }
    pout[gi] = p;
  }
}

double ora_jointp_exact(int G, int rowlen, const float *g, int np, int nm,
                        int npops, int modeltype, const double *lognorm,
                        const double *x, double *ess)
{
  double *p = (double *)malloc(sizeof(double) * (size_t)G);
  ora_surface_p(G, rowlen, g, np, nm, npops, modeltype, lognorm, x, p);
  double M = -INFINITY;
  for (int i = 0; i < G; i++) if (p[i] > M) M = p[i];
  long double s = 0.0L, s2 = 0.0L;
  for (int i = 0; i < G; i++) {
    long double w = expl((long double)(p[i] - M));
    s += w;
    s2 += w * w;
  }
  free(p);
  if (ess) *ess = (double)(s * s / s2);
  return log((double)G) - (M + (double)logl(s));
}

void ora_eexp(double x, double *m, int *z)
{
  static const double inv_fact[10] = {
      1.0, 0.5, 0.16666666666666666666666666667, 0.04166666666666666666666666667,
      0.00833333333333333333333333333, 0.001388888888888888888888888889,
      0.000198412698412698412698412698, 0.000024801587301587301587301587301,
      2.75573192239858906525573192239859e-6, 2.75573192239858906525573192239e-7};
  const double log10_2 = 0.30102999566398119521;
  int n = (int)floor(x / ORA_LOG2);
  double zr = log10_2 * (double)n;
  *z = (int)zr;
  zr -= (double)*z;
  double u = x - ((double)n) * ORA_LOG2;
  double t = inv_fact[9];
  for (int k = 8; k >= 0; k--) t = inv_fact[k] + u * t;
  t = 1 + u * t;
  *m = t * pow(10.0, zr);
  if (fabs(*m) > 10) { *m = *m / 10.0; *z = *z + 1; }
  if (fabs(*m) < 1) { *m = *m * 10.0; *z = *z - 1; }
}

static int cmp_desc(const void *a, const void *b)
{
  double x = *(const double *)a, y = *(const double *)b;
  return (x < y) - (x > y);
}

double ora_jointp_compat(int G, int rowlen, const float *g, int np, int nm,
                         int npops, int modeltype, const double *lognorm,
                         const double *x, double *ess)
{
  double *p = (double *)malloc(sizeof(double) * (size_t)G);
  double *list = (double *)malloc(sizeof(double) * (size_t)G);
  ora_surface_p(G, rowlen, g, np, nm, npops, modeltype, lognorm, x, p);
  /* list membership: the first value, then every value within 10 of the
   * running maximum at the time it is seen */
  int m = 0;
  double runmax = p[0];
  list[m++] = p[0];
  for (int i = 1; i < G; i++) {
    if (runmax - p[i] < 10) {
      list[m++] = p[i];
      if (p[i] > runmax) runmax = p[i];
    }
  }
  qsort(list, (size_t)m, sizeof(double), cmp_desc);
  int iin = m - 1;
  int cnt = 0;
  do { cnt++; } while (cnt < iin && list[0] - list[cnt] < 10);
  double *mm = (double *)malloc(sizeof(double) * (size_t)cnt);
  int *zz = (int *)malloc(sizeof(int) * (size_t)cnt);
  int maxz = -10000000;
  for (int i = 0; i < cnt; i++) {
    ora_eexp(list[i], &mm[i], &zz[i]);
    if (zz[i] > maxz) maxz = zz[i];
  }
  maxz -= 10;
  double acc = 0.0, acc2 = 0.0;
  for (int i = 0; i < cnt; i++) {
    int zadj = zz[i] - maxz;
    if (zadj > -308 && zadj < 308) mm[i] *= pow(10.0, (double)zadj);
    else if (zadj <= -308) mm[i] = 0.0;
    else mm[i] = DBL_MAX;
    acc += mm[i];
    acc2 += mm[i] * mm[i];
  }
  if (ess) *ess = acc * acc / acc2;
  double q = log((double)G) - (log(acc) + maxz * ORA_LOG10);
  free(mm); free(zz); free(p); free(list);
  return q;
}

/* ======================================================================
 * L-mode peak search by differential evolution (jointfind.cpp:594-812)
 * ==================================================================== */
typedef struct {
  int G, rowlen, np, nm, npops, modeltype, compat;
  const float *g;
  const double *lognorm;
} de_obj;

static double de_eval(const de_obj *o, const double *x, double *ess)
{
  double e = 0.0;
  double q = o->compat ? ora_jointp_compat(o->G, o->rowlen, o->g, o->np, o->nm, o->npops,
                                           o->modeltype, o->lognorm, x, &e)
                       : ora_jointp_exact(o->G, o->rowlen, o->g, o->np, o->nm, o->npops,
                                          o->modeltype, o->lognorm, x, &e);
  if (ess) *ess = e;
  return q;
}

#define DE_MINPARAMVAL 0.0000001 /* imamp.hpp:130 */
#define DE_STARTHI 1E200         /* jointfind.cpp:136-142 */
#define DE_STARTLOW -1E200
#define DE_SPREADTOL 1.0e-7
#define DE_PLOOPTOL 1.0e-6
#define DE_LOOPMATCH 2
#define DE_MAXRESTART 10
#define DE_RECRATE 0.9 /* :145-146 */
#define DE_FWEIGHT 0.8

static int de_randposint(ora_mt *r, int n) { return (int)floor(ora_mt_uniform(r) * n); }

/* the full parameter vector jointp sees for population member v */
static void de_full(const double *v, const double *xmap, int n, double *full)
{
  if (!xmap) {
    for (int i = 0; i < n; i++) full[i] = v[i];
    return;
  }
  for (int i = 0; i < n; i++) full[i] = xmap[i] < 0 ? -xmap[i] : v[(int)xmap[i]];
}

int ora_modelloop(int G, int rowlen, const float *g, int np, int nm, int npops,
                  const double *lognorm, int compat, int modeltype,
                  const double *upper, int multiplier, const double *xmap,
                  int nested, ora_mt *rng, double *best, double *ess,
                  int *restarts)
{
  const int n = np + nm;
  if (xmap && (nested < 1 || modeltype == 2)) return -1; /* see the header */
  de_obj o = {G, rowlen, np, nm, npops, modeltype, compat, g, lognorm};
  const int r0 = (modeltype == 2) ? np : 0;
  int modelparams = modeltype == 0 ? n : (modeltype == 1 ? np : nm);
  if (xmap) modelparams = nested;
  const int jmax = r0 + modelparams;
  const int dep = modelparams * multiplier;
  double *lo = (double *)calloc(n, sizeof(double)), *hi = (double *)calloc(n, sizeof(double));
  if (!xmap) {
    for (int j = 0; j < n; j++) {
      lo[j] = DE_MINPARAMVAL;
      hi[j] = upper[j];
    }
  } else {
    /* reversemapvals: the first full parameter mapped to each nested index */
    for (int i = 0, k = 0; i < n; i++)
      if (k == (int)xmap[i]) {
        lo[k] = DE_MINPARAMVAL;
        hi[k] = upper[i];
        k++;
      }
  }
  double *pop = (double *)calloc((size_t)dep * (n + 1), sizeof(double));
  double *trial = (double *)calloc((size_t)dep * (n + 1), sizeof(double));
  double *full = (double *)calloc(n, sizeof(double));
  double *bestv = (double *)calloc(n + 1, sizeof(double));
#define POP(i, j) pop[(size_t)(i) * (n + 1) + (j)]
#define TRI(i, j) trial[(size_t)(i) * (n + 1) + (j)]
  int gens = 0, nrun = 0;
  double global_pd = DE_STARTHI;
  /* startpop */
  {
    for (int i = 0; i < dep; i++) {
      for (int j = 0; j < n; j++)
        POP(i, j) = (j >= r0 && j < jmax) ? lo[j] + ora_mt_uniform(rng) * (hi[j] - lo[j]) : -1.0;
      de_full(&POP(i, 0), xmap, n, full);
      POP(i, n) = de_eval(&o, full, NULL);
    }
  }
  for (int i = 0; i < dep; i++)
    if (POP(i, n) < global_pd) global_pd = POP(i, n);
  int newstart = 0, countloop = 0;
  do {
    if (newstart > 0) {
      for (int i = 0; i < dep; i++) {
        for (int j = 0; j < n; j++)
          POP(i, j) = (j >= r0 && j < jmax) ? lo[j] + ora_mt_uniform(rng) * (hi[j] - lo[j]) : -1.0;
        de_full(&POP(i, 0), xmap, n, full);
        POP(i, n) = de_eval(&o, full, NULL);
      }
    }
    /* difeloop: nextgen until the spread of the population's values is small */
    double lowpd, hipd;
    do {
      lowpd = DE_STARTHI;
      hipd = DE_STARTLOW;
      for (int i = 0; i < dep; i++) {
        int A = de_randposint(rng, dep), B = de_randposint(rng, dep), Cv = de_randposint(rng, dep);
        for (int j = r0; j < jmax; j++) {
          double u = ora_mt_uniform(rng);
          if (u < DE_RECRATE) {
            double t = POP(Cv, j) + DE_FWEIGHT * (POP(A, j) - POP(B, j));
            if (t < lo[j]) t = POP(Cv, j) - ora_mt_uniform(rng) * (POP(Cv, j) - lo[j]);
            if (t > hi[j]) t = POP(Cv, j) + ora_mt_uniform(rng) * (hi[j] - POP(Cv, j));
            TRI(i, j) = t;
          } else {
            TRI(i, j) = POP(i, j);
          }
        }
        de_full(&TRI(i, 0), xmap, n, full);
        TRI(i, n) = de_eval(&o, full, NULL);
      }
      for (int i = 0; i < dep; i++) {
        if (TRI(i, n) < POP(i, n))
          for (int j = 0; j <= n; j++) POP(i, j) = TRI(i, j);
        if (POP(i, n) < lowpd) lowpd = POP(i, n);
        if (POP(i, n) > hipd) hipd = POP(i, n);
      }
      gens++;
    } while (hipd - lowpd > DE_SPREADTOL);
    double local_pd = lowpd;
    nrun++;
    if (fabs(local_pd - global_pd) < DE_PLOOPTOL) countloop++;
    else if (local_pd < global_pd) countloop = 0;
    if (local_pd < global_pd) {
      /* copybest */
      double t = DE_STARTHI;
      int k = 0;
      for (int i = 0; i < dep; i++)
        if (POP(i, n) < t) {
          t = POP(i, n);
          k = i;
        }
      for (int j = 0; j <= n; j++) bestv[j] = POP(k, j);
      bestv[n] = t;
      global_pd = local_pd;
    }
    newstart++;
  } while (countloop < DE_LOOPMATCH && newstart < DE_MAXRESTART);
  de_full(bestv, xmap, n, full);
  for (int j = 0; j < n; j++) best[j] = full[j];
  best[n] = bestv[n];
  de_eval(&o, full, ess);
  if (restarts) *restarts = nrun;
#undef POP
#undef TRI
  free(lo); free(hi); free(pop); free(trial); free(full); free(bestv);
  return gens;
}

/* ======================================================================
 * 1-D marginal densities (surface_call_functions.cpp:119-175)
 * ==================================================================== */
static long ora_intround(double v) { return v >= 0 ? (long)(v + 0.5) : (long)(v - 0.5); } /* INTEGERROUND */

double ora_margincalc(int G, int rowlen, const float *g, int np, int nm, int pi,
                      double x, double yadjust, int logi, const double *expo_mean)
{
  int ccp, fcp, hccp, mcp, fmp, qip, mip, pdgp, probgp;
  ora_gsamp_offsets(np, nm, &ccp, &fcp, &hccp, &mcp, &fmp, &qip, &mip, &pdgp, &probgp);
  double meani = 0.0;
  if (expo_mean && pi >= np && pi < np + nm) meani = 1.0 / expo_mean[pi - np];
  double sum = 0.0;
  for (int e = 0; e < G; e++) {
    const float *r = g + (size_t)e * rowlen;
    if (pi < np) {
      int p = pi;
      double hval = r[hccp + p];
      double temp = -r[qip + p] + ora_intround(r[ccp + p]) * (ORA_LOG2 - log(x)) - hval - 2 * r[fcp + p] / x;
      sum += exp(temp);
    } else {
      int p = pi - np;
      if (expo_mean)
        sum += exp(-r[mip + p] + log(meani) - x * meani + ora_intround(r[mcp + p]) * log(x) - r[fmp + p] * x);
      else
        sum += exp(-r[mip + p] + ora_intround(r[mcp + p]) * log(x) - r[fmp + p] * x);
    }
  }
  sum /= G;
  if (logi) sum = (sum <= 0) ? -1e200 : log(sum);
  return sum - yadjust;
}

/* ======================================================================
 * Genealogy weights.  treeweight (update_gtree_common.cpp:1680-1937): every
 * coalescence (internal node, at the time of its daughters' tops), every
 * migration (with the population it leaves, found by following the edge's
 * population through the splits, :1770-1790) and every split younger than
 * the root becomes an event; the events are visited in time order and, over
 * each interval, each population of the current period accumulates
 * n(n-1)*dt/(2h) (fc) and n*dt (fm, the same for every partner); counts
 * (cc, mc) and the lineage numbers change at each event.
 * ==================================================================== */
int ora_tw_sizes(int npops, int *T, int *M)
{
  int m = 0;
  for (int k = 0; k < npops - 1; k++) m += (npops - k) * (npops - k);
  *T = npops * (npops + 1) / 2;
  *M = m;
  return 0;
}

static int tw_toff(int npops, int k) { return k * npops - k * (k - 1) / 2; }
static int tw_moff(int npops, int k)
{
  int m = 0;
  for (int j = 0; j < k; j++) m += (npops - j) * (npops - j);
  return m;
}

typedef struct { double t; int cmt, pop, topop, ord; } tw_event;

static int tw_cmp(const void *a, const void *b)
{
  const tw_event *x = (const tw_event *)a, *y = (const tw_event *)b;
  if (x->t < y->t) return -1;
  if (x->t > y->t) return 1;
  return x->ord - y->ord;
}

static int tw_period(const double *tvals, int nsplit, double t) /* findperiod, :1626 */
{
  int k = 0;
  while (k < nsplit && tvals[k] <= t) k++;
  return k;
}

int ora_treeweight(int npops, const int *plist, const int *droppops, const int *addpop,
                   const int *pop_e, const int *pop_down, const double *tvals, int nomig,
                   int ng, const int *samppop, double hval, const int *up0,
                   const double *time, const int *pop, const int *mig_off,
                   const double *mig_t, const int *mig_p, int *cc, double *hcc,
                   double *fc, int *mc, double *fm, double *out3, int *mignum)
{
  int T, M, nl = 2 * ng - 1, nsplit = npops - 1, ntp = 2 * npops - 1;
  ora_tw_sizes(npops, &T, &M);
  memset(cc, 0, sizeof(int) * (size_t)T);
  memset(hcc, 0, sizeof(double) * (size_t)T);
  memset(fc, 0, sizeof(double) * (size_t)T);
  memset(mc, 0, sizeof(int) * (size_t)M);
  memset(fm, 0, sizeof(double) * (size_t)M);
  if (npops < 2) return 1;
  int nmig = mig_off[nl];
  /* roottime: the root's coalescence, the latest of all */
  double roottime = 0.0;
  for (int i = ng; i < nl; i++)
    if (time[up0[i]] > roottime) roottime = time[up0[i]];
  int kroot = tw_period(tvals, nsplit, roottime);
  int ne = (ng - 1) + nmig + kroot;
  tw_event *ev = (tw_event *)malloc(sizeof(tw_event) * (size_t)(ne > 0 ? ne : 1));
  int e = 0;
  for (int i = 0; i < nl; i++) {
    int nowpop = pop[i];
    if (nowpop < 0 || nowpop >= ntp) { free(ev); return 1; }
    if (i >= ng) {
      ev[e].t = time[up0[i]];
      ev[e].cmt = 0;
      ev[e].pop = nowpop;
      ev[e].topop = -1;
      ev[e].ord = e;
      e++;
    }
    for (int j = mig_off[i]; j < mig_off[i + 1]; j++) {
      int per = tw_period(tvals, nsplit, mig_t[j]);
      while (pop_e[nowpop] <= per && pop_e[nowpop] != -1) nowpop = pop_down[nowpop];
      ev[e].t = mig_t[j];
      ev[e].cmt = 1;
      ev[e].pop = nowpop;
      ev[e].topop = mig_p[j];
      ev[e].ord = e;
      if (mig_p[j] == nowpop || mig_p[j] < 0 || mig_p[j] >= ntp) { free(ev); return 1; }
      nowpop = mig_p[j];
      e++;
    }
  }
  for (int i = 0; i < kroot; i++) {
    ev[e].t = tvals[i];
    ev[e].cmt = -1;
    ev[e].pop = ev[e].topop = -1;
    ev[e].ord = e;
    e++;
  }
  qsort(ev, (size_t)ne, sizeof(tw_event), tw_cmp);

  int n[2 * 10 - 1];
  for (int i = 0; i < ntp; i++) n[i] = 0;
  for (int i = 0; i < npops; i++) n[i] = samppop[i];
  int nsum = ng, k = 0, bad = 0;
  double lasttime = 0.0, length = 0.0, tlength = 0.0;
  double h2term = 1 / (2 * hval);
  double lastsplitt = tvals[nsplit - 1];
  for (int j = 0; j < ne && !bad; j++) {
    const tw_event *s = &ev[j];
    double dt = s->t - lasttime;
    double tadd = nsum * dt;
    length += tadd;
    if (s->t < lastsplitt) tlength += tadd;
    else if (lasttime < lastsplitt) tlength += nsum * (lastsplitt - lasttime);
    lasttime = s->t;
    for (int ii = 0; ii < npops - k; ii++) {
      int ip = plist[k * npops + ii];
      double nn1 = (double)n[ip] * ((double)n[ip] - 1);
      fc[tw_toff(npops, k) + ii] += nn1 * dt * h2term;
      if (!nomig && k < nsplit) {
        double fmtemp = n[ip] * dt;
        for (int jj = 0; jj < npops - k; jj++)
          if (jj != ii) fm[tw_moff(npops, k) + ii * (npops - k) + jj] += fmtemp;
      }
    }
    if (s->cmt == 0) {
      int ii = 0;
      while (ii < npops - k && plist[k * npops + ii] != s->pop) ii++;
      if (ii == npops - k || n[s->pop] < 2) { bad = 1; break; }
      cc[tw_toff(npops, k) + ii]++;
      n[s->pop]--;
      nsum--;
    } else if (s->cmt == 1) {
      int ii = 0, jj = 0;
      while (ii < npops - k && plist[k * npops + ii] != s->pop) ii++;
      while (jj < npops - k && plist[k * npops + jj] != s->topop) jj++;
      if (ii == npops - k || jj == npops - k || n[s->pop] < 1 || k >= nsplit) { bad = 1; break; }
      mc[tw_moff(npops, k) + ii * (npops - k) + jj]++;
      n[s->pop]--;
      n[s->topop]++;
    } else {
      k++;
      n[addpop[k]] = n[droppops[2 * k]] + n[droppops[2 * k + 1]];
      n[droppops[2 * k]] = n[droppops[2 * k + 1]] = 0;
    }
  }
  free(ev);
  if (bad || nsum != 1) return 1;
  double hlog = log(hval);
  if (hlog != 0.0)
    for (int i = 0; i < T; i++) hcc[i] += hlog * cc[i];
  out3[0] = length;
  out3[1] = tlength;
  *mignum = nmig;
  return 0;
}

/* ======================================================================
 * p(G) integrals.  The reference's incomplete gamma functions
 * (utilities.cpp:808-1130; Numerical Recipes series and Lentz continued
 * fraction, EPS 3e-7, ITMAX 1000; expint with MAXIT 100 and its own
 * truncated Euler constant) return logs; logfact[i] is the running sum
 * log(1)+...+log(i) (setlogfact, utilities.cpp:1406-1415).  A stop the
 * reference would take through IM_err sets *st.
 * ==================================================================== */
#define IG_EPS 3.0e-7
#define IG_ITMAX 1000
#define IG_FPMIN 1.0e-30
#define EI_MAXIT 100
#define EI_EULER 0.5772156649
#define LD_CUT 7.0978271289338397e+02
#define ORA_MPRIORMIN 0.000001 /* imamp.hpp:137 */

static double *lf_tab;
static int lf_n;
static double lf(int i, int *st)
{
  if (i < 0) { *st = 3; return 0.0; }
  if (i >= lf_n) {
    int nn = lf_n ? lf_n : 1024;
    while (nn <= i) nn *= 2;
    double *t = (double *)realloc(lf_tab, sizeof(double) * (size_t)nn);
    if (!t) { *st = 3; return 0.0; }
    if (lf_n == 0) t[0] = 0.0;
    for (int k = lf_n ? lf_n : 1; k < nn; k++) t[k] = t[k - 1] + log((double)k);
    lf_tab = t;
    lf_n = nn;
  }
  return lf_tab[i];
}

static double ig_gser(int a, double x, double *gln, int lg, int *st) /* gser / gserlog */
{
  *gln = lf(a - 1, st);
  if (x <= 0.0) {
    if (x < 0.0) *st = 3;
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
  *st = 2;
  return 0.0;
}

static double ig_gcf(double a, double x, double *gln, int lg, int *st) /* gcf / gcflog */
{
  *gln = lf((int)a - 1, st);
  double b = x + 1.0 - a, c = 1.0 / IG_FPMIN, d = 1.0 / b, h = d, an, del;
  int i;
  for (i = 1; i <= IG_ITMAX; i++) {
    an = -i * (i - a);
    b += 2.0;
    d = an * d + b;
    if (fabs(d) < IG_FPMIN) d = IG_FPMIN;
    c = b + an / c;
    if (fabs(c) < IG_FPMIN) c = IG_FPMIN;
    d = 1.0 / d;
    del = d * c;
    h *= del;
    if (fabs(del - 1.0) < IG_EPS) break;
  }
  if (i > IG_ITMAX) *st = 2;
  return lg ? (-x + a * log(x) - (*gln)) + log(h) : exp(-x + a * log(x) - (*gln)) * h;
}

static double ig_expint1(double x, int *islog, int *st) /* expint(1, x) */
{
  *islog = 0;
  if (x <= 0.0) { *st = 3; return 0.0; }
  if (x > 1.0) {
    double b = x + 1, c = 1.0 / IG_FPMIN, d = 1.0 / b, h = d, a, del;
    for (int i = 1; i <= EI_MAXIT; i++) {
      a = -i * i;
      b += 2.0;
      d = 1.0 / (a * d + b);
      c = b + a / c;
      del = c * d;
      h *= del;
      if (fabs(del - 1.0) < IG_EPS) {
        *islog = 1;
        return log(h) - x;
      }
    }
    *st = 2;
    return 0.0;
  }
  double ans = -log(x) - EI_EULER, fact = 1.0, del;
  for (int i = 1; i <= EI_MAXIT; i++) {
    fact *= -x / i;
    del = -fact / i;
    ans += del;
    if (fabs(del) < fabs(ans) * IG_EPS) return ans;
  }
  *st = 2;
  return ans;
}

static double ig_upper(int a, double x, int *st) /* uppergamma, :1068 */
{
  double p, gln;
  if (x < 0.0 || a < 0) { *st = 3; return 0.0; }
  if (a == 0) {
    int islog;
    double t = ig_expint1(x, &islog, st);
    p = islog ? t : log(t);
  } else if (x < (a + 1.0)) {
    double g = ig_gser(a, x, &gln, 0, st);
    p = gln + log(1.0 - g);
  } else {
    double g = ig_gcf((double)a, x, &gln, 1, st);
    p = gln + g;
  }
  if (p < -1e200) p = -1e200;
  return p;
}

static double ig_lower(int a, double x, int *st) /* lowergamma, :1104 */
{
  double p, gln;
  if (x < 0.0 || a <= 0) { *st = 3; return 0.0; }
  if (x < (a + 1.0)) {
    double g = ig_gser(a, x, &gln, 1, st);
    p = gln + g;
  } else {
    double g = ig_gcf((double)a, x, &gln, 0, st);
    p = gln + log(1 - g);
  }
  if (p < -1e200) p = -1e200;
  return p;
}

/* LogDiff (imamp.hpp:257-262): log(exp(a) - exp(b)), a > b required */
static double ld(double a, double b, int *st)
{
  if (a <= b) { *st = 1; return 0.0; }
  return (a - b < LD_CUT) ? b + log(exp(a - b) - 1.0) : a;
}

static double it_coal(int cc, double fc, double hcc, double max, double min, int *st)
{
  double p;
  if (cc > 0) {
    if (!(fc > 0)) { *st = 3; return 0.0; }
    if (min == 0) {
      double ug = ig_upper(cc - 1, 2 * fc / max, st);
      if (cc > 1) {
        double fullg = lf(cc - 2, st);
        if (fullg - ug < 1e-15 || fullg - ug > LD_CUT) {
          double lg = ig_lower(cc - 1, 2 * fc / max, st);
          if (fullg > lg) {
            double ugalt = ld(fullg, lg, st);
            if (fabs(ugalt - ug) > 1e-10) ug = ugalt;
          }
        }
      }
      p = ug + ORA_LOG2 - hcc + (1 - cc) * log(fc);
    } else {
      double a = ig_upper(cc - 1, 2 * fc / max, st), b = ig_upper(cc - 1, 2 * fc / min, st);
      p = ld(a, b, st);
      p += (ORA_LOG2 - hcc + (1 - cc) * log(fc));
    }
  } else if (2 * fc / max > 0) {
    if (min == 0) {
      double a = log(max) - 2.0 * fc / max;
      double b = ORA_LOG2 + log(fc) + ig_upper(0, 2.0 * fc / max, st);
      p = ld(a, b, st);
    } else {
      double a = ig_upper(0, 2 * fc / max, st), b = ig_upper(0, 2 * fc / min, st);
      double c = ld(a, b, st);
      c += ORA_LOG2 + log(fc);
      a = log(max) - 2.0 * fc / max;
      b = log(min) - 2.0 * fc / min;
      double d = ld(a, b, st);
      p = ld(d, c, st);
    }
  } else {
    p = log(max - min);
  }
  return p;
}

static double it_mig(int cm, double fm, double max, double min, int *st)
{
  double p;
  if (cm > 0) {
    if (!(fm > 0)) { *st = 3; return 0.0; }
    if (min == 0) {
      double lg = ig_lower(cm + 1, fm * max, st);
      double fullg = lf(cm, st);
      if (fullg - lg < 1e-15 || fullg - lg > LD_CUT) {
        double ug = ig_upper(cm + 1, fm * max, st);
        if (fullg > ug) {
          double lgalt = ld(fullg, ug, st);
          if (fabs(lgalt - lg) > 1e-12) lg = lgalt;
        }
      }
      p = (-1 - cm) * log(fm) + lg;
    } else {
      double a = ig_upper(cm + 1, fm * min, st), b = ig_upper(cm + 1, fm * max, st);
      double c = ld(a, b, st);
      p = (-1 - cm) * log(fm) + c;
    }
  } else if (fm > ORA_MPRIORMIN) {
    if (min == 0) {
      if (max == ORA_MPRIORMIN) {
        p = 0;
      } else {
        double c = ld(0.0, -fm * max, st);
        p = c - log(fm);
      }
    } else {
      double c = ld(-fm * min, -fm * max, st);
      p = c - log(fm);
    }
  } else {
    p = log(max - min);
  }
  return p;
}

static double it_mig_expo(int cm, double fm, double mean, int *st)
{
  return -log(mean) + (-(cm + 1) * log(fm + 1.0 / mean)) + lf(cm, st);
}

double ora_iterm(int kind, int c, double f, double h, double max, double min, int *status)
{
  int st = 0;
  double v = kind == 0 ? it_coal(c, f, h, max, min, &st)
           : kind == 1 ? it_mig(c, f, max, min, &st) : it_mig_expo(c, f, max, &st);
  *status = st;
  return v;
}

int ora_tree_prob(int nomig, int expo, const int *cc, const double *hcc, const double *fc,
                  const int *mc, const double *fm, int nth, const int *th_off,
                  const int *th_idx, const double *th_max, const double *th_min, int nmg,
                  const int *mg_off, const int *mg_idx, const double *mg_max,
                  const double *mg_min, const double *mg_mean, int nchk, const int *chk_idx,
                  double *probg, double *q, double *m)
{
  int st = 0;
  if (!nomig)
    for (int i = 0; i < nchk; i++)
      if (mc[chk_idx[i]] != 0) {
        *probg = -DBL_MAX; /* MYDBL_MAX, imamp.hpp */
        return 0;
      }
  double psum = 0;
  for (int i = 0; i < nth; i++) {
    int c = 0;
    double f = 0.0, hc = 0.0;
    for (int j = th_off[i]; j < th_off[i + 1]; j++) {
      c += cc[th_idx[j]];
      f += fc[th_idx[j]];
      hc += hcc[th_idx[j]];
    }
    q[i] = it_coal(c, f, hc, th_max[i], th_min[i], &st);
    psum += q[i];
  }
  if (!nomig)
    for (int i = 0; i < nmg; i++) {
      int c = 0;
      double f = 0.0;
      for (int j = mg_off[i]; j < mg_off[i + 1]; j++) {
        c += mc[mg_idx[j]];
        f += fm[mg_idx[j]];
      }
      m[i] = expo ? it_mig_expo(c, f, mg_mean[i], &st) : it_mig(c, f, mg_max[i], mg_min[i], &st);
      psum += m[i];
    }
  *probg = psum;
  return st;
}

void ora_gsamp_row(int nomig, const int *cc, const double *hcc, const double *fc,
                   const int *mc, const double *fm, int nth, const int *th_off,
                   const int *th_idx, int nmg, const int *mg_off, const int *mg_idx,
                   const double *q, const double *m, double pdg, double probg,
                   int nsplit, const double *tvals, float *row)
{
  int nmg_eff = nomig ? 0 : nmg;
  int ccp = 0, fcp = nth, hccp = 2 * nth, mcp = 3 * nth, fmp = mcp + nmg_eff;
  int qip = fmp + nmg_eff, mip = qip + nth, pdgp = mip + nmg_eff, probgp = pdgp + 1,
      tp = probgp + 1;
  for (int i = 0; i < nth; i++) {
    int c = 0;
    float f = 0.0f, hc = 0.0f;
    for (int j = th_off[i]; j < th_off[i + 1]; j++) {
      c += cc[th_idx[j]];
      f += (float)fc[th_idx[j]];
      hc += (float)hcc[th_idx[j]];
    }
    row[ccp + i] = (float)c;
    row[fcp + i] = f;
    row[hccp + i] = hc;
  }
  for (int i = 0; i < nmg_eff; i++) {
    int c = 0;
    float f = 0.0f;
    for (int j = mg_off[i]; j < mg_off[i + 1]; j++) {
      c += mc[mg_idx[j]];
      f += (float)fm[mg_idx[j]];
    }
    row[mcp + i] = (float)c;
    row[fmp + i] = f;
  }
  for (int i = 0; i < nth; i++) row[qip + i] = (float)q[i];
  for (int i = 0; i < nmg_eff; i++) row[mip + i] = (float)m[i];
  row[pdgp] = (float)pdg;
  row[probgp] = (float)probg;
  for (int i = 0; i < nsplit; i++) row[tp + i] = (float)tvals[i];
}

int ora_treeweight_batch(int npops, const int *plist, const int *droppops, const int *addpop,
                         const int *pop_e, const int *pop_down, int nomig, int ngen, const int *node_off,
                         const int *up0, const double *time, const int *pop, const int *mig_off,
                         const double *mig_t, const int *mig_p, const int *gen_locus, const int *gen_tv,
                         const double *hval, const int *samppop, const double *tvals, int *cc, double *hcc,
                         double *fc, int *mc, double *fm, double *lens, int *mignum)
{
  int T, M, bad = 0;
  ora_tw_sizes(npops, &T, &M);
  int *moff = (int *)malloc(sizeof(int) * (size_t)(node_off[ngen] + 1));
  for (int g = 0; g < ngen; g++) {
    const int a0 = node_off[g], nl = node_off[g + 1] - a0, li = gen_locus[g];
    for (int i = 0; i <= nl; i++) moff[i] = mig_off[a0 + i] - mig_off[a0];
    const int mb = mig_off[a0];
    if (ora_treeweight(npops, plist, droppops, addpop, pop_e, pop_down, tvals + (size_t)gen_tv[g] * (npops - 1),
                       nomig, (nl + 1) / 2, samppop + (size_t)li * npops, hval[li], up0 + a0, time + a0, pop + a0,
                       moff, mig_t + mb, mig_p + mb, cc + (size_t)g * T, hcc + (size_t)g * T, fc + (size_t)g * T,
                       mc + (size_t)g * M, fm + (size_t)g * M, lens + 2 * (size_t)g, mignum + g))
      bad++;
  }
  free(moff);
  return bad;
}

/* ======================================================================
 * 2NM densities.  calc_popmig (popmig.cpp:9-91): the posterior density of
 * the population migration rate 2N_i m_j at x, a sum over the saved
 * genealogies of exp(temp1 + temp2) with one or two incomplete gamma terms
 * per genealogy (terms outside +-700 skipped); calc_pop_expomig (:96-172)
 * the same under an exponential migration prior, its terms summed as eexp
 * mantissa / decimal-exponent pairs rescaled to the largest exponent.
 * prob_or_like = 1 divides by the prior density of 2NM.  Counts are
 * truncated as the reference's (int) casts truncate them.
 * ==================================================================== */
static void popmig_cols(int np, int nm, int thetai, int mi, int *c)
{
  int ccp, fcp, hccp, mcp, fmp, qip, mip, pdgp, probgp;
  ora_gsamp_offsets(np, nm, &ccp, &fcp, &hccp, &mcp, &fmp, &qip, &mip, &pdgp, &probgp);
  c[0] = ccp + thetai; c[1] = fcp + thetai; c[2] = hccp + thetai; c[3] = mcp + mi;
  c[4] = fmp + mi; c[5] = qip + thetai; c[6] = mip + mi;
}

/* calc_popmig's term of one genealogy (popmig.cpp:33-84): temp1 + temp2 */
static double pm_term(const float *r, const int *c, double x, double qmax, double mmax, int *st)
{
  int cc = (int)r[c[0]], mc = (int)r[c[3]];
  double fc = r[c[1]], hc = r[c[2]], fm = r[c[4]], qintg = r[c[5]], mintg = r[c[6]];
  double temp1, temp2;
  if (fc == 0 && cc == 0 && fm > 0) {
    temp1 = ORA_LOG2 - (mc * log(fm)) - hc - qintg - mintg;
    temp2 = log(exp(ig_upper(mc, 2 * fm * x / qmax, st)) - exp(ig_upper(mc, mmax * fm, st)));
  } else if (fm == 0 && mc == 0 && fc > 0) {
    temp1 = ORA_LOG2 - (cc * log(fc)) - hc - qintg - mintg;
    temp2 = log(exp(ig_upper(cc, 2 * fc / qmax, st)) - exp(ig_upper(cc, fc * mmax / x, st)));
  } else if (fc == 0 && cc == 0 && mc == 0 && fm == 0) {
    temp1 = log(2 * log(mmax * qmax / (2 * x))) - hc - qintg - mintg;
    temp2 = 0;
  } else {
    temp1 = ORA_LOG2 + (mc * log(x)) - ((cc + mc) * log(fc + fm * x)) - hc - qintg - mintg;
    double a = ig_upper(cc + mc, 2 * (fc + fm * x) / qmax, st);
    double b = ig_upper(cc + mc, mmax * (fm + fc / x), st);
    if (a == b) {
      b = ig_lower(cc + mc, 2 * (fc + fm * x) / qmax, st);
      a = ig_lower(cc + mc, mmax * (fm + fc / x), st);
    }
    if (a > b) {
      temp2 = ld(a, b, st);
    } else {
      temp1 = temp2 = 0.0;
    }
  }
  return temp1 + temp2;
}

/* calc_pop_expomig's log term of one genealogy (popmig.cpp:114-147) */
static double pe_term(const float *r, const int *c, double x, double qmax, double mmean, int *st)
{
  int cc = (int)r[c[0]], mc = (int)r[c[3]];
  double fc = r[c[1]], hc = r[c[2]], fm = r[c[4]], qintg = r[c[5]], mintg = r[c[6]];
  double temp1 = x + fc * mmean + fm * mmean * x;
  double temp2 = ORA_LOG2 - hc - log(mmean) - qintg - mintg;
  double temp3 = 2 * temp1 / (mmean * qmax);
  if (mc == 0 && cc == 0) {
    temp3 = ig_upper(0, temp3, st);
    temp2 += temp3;
  } else if (cc == 0) {
    temp3 = ig_upper(mc, temp3, st);
    temp2 += temp3 - mc * log(fm + 1 / mmean);
  } else if (mc == 0) {
    temp3 = ig_upper(cc, temp3, st);
    temp2 += temp3 + -cc * log(fc + x * (fm + 1 / mmean));
  } else {
    temp3 = ig_upper(mc + cc, temp3, st);
    temp2 += temp3 - cc * log(x) + (cc + mc) * log(mmean * x / temp1);
  }
  return temp2;
}

/* sum over genealogies [ft, lt) of exp(term) (terms outside +-700 skipped) */
static double pm_sum(const float *g, int rowlen, const int *c, int ft, int lt, double x, double qmax, double mmax,
                     int *st)
{
  double sum = 0.0;
  for (int e = ft; e < lt; e++) {
    double t = pm_term(g + (size_t)e * rowlen, c, x, qmax, mmax, st);
    if ((t < 700) && (t > -700)) sum += exp(t);
  }
  return sum;
}

/* log of the eexp-rescaled sum over genealogies [ft, lt) (popmig.cpp:148-160) */
static double pe_logsum(const float *g, int rowlen, const int *c, int ft, int lt, double x, double qmax,
                        double mmean, int *st)
{
  int n = lt - ft;
  double *mm = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
  int *zz = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (!mm || !zz) { free(mm); free(zz); *st = 3; return 0.0; }
  int maxz = -1000000000;
  for (int e = 0; e < n; e++) {
    ora_eexp(pe_term(g + (size_t)(ft + e) * rowlen, c, x, qmax, mmean, st), &mm[e], &zz[e]);
    if (zz[e] > maxz) maxz = zz[e];
  }
  double acumm = 0.0;
  for (int e = 0; e < n; e++) {
    int zadj = zz[e] - (maxz - 10);
    mm[e] *= pow(10.0, (double)zadj);
    acumm += mm[e];
  }
  free(mm);
  free(zz);
  return log(acumm) + (maxz - 10) * ORA_LOG10;
}

double ora_popmig(int G, int rowlen, const float *g, int np, int nm, int thetai, int mi, double x,
                  double qmax, double mmax, int prob_or_like, int *st)
{
  int c[7];
  popmig_cols(np, nm, thetai, mi, c);
  double sum = pm_sum(g, rowlen, c, 0, G, x, qmax, mmax, st);
  sum /= G;
  if (prob_or_like) {
    double temp = 2 * (log(qmax) + log(mmax) - log(2 * x)) / (qmax * mmax);
    sum /= temp;
  }
  return sum;
}

double ora_pop_expomig(int G, int rowlen, const float *g, int np, int nm, int thetai, int mi, double x,
                       double qmax, double mmean, int prob_or_like, int *st)
{
  int c[7];
  popmig_cols(np, nm, thetai, mi, c);
  double sum = pe_logsum(g, rowlen, c, 0, G, x, qmax, mmean, st);
  sum -= log((double)G);
  sum = exp(sum);
  if (prob_or_like) {
    double temp = 2 * exp(ig_upper(0, 2 * x / (mmean * qmax), st)) / (qmax * mmean);
    sum /= temp;
  }
  return sum;
}

/* ======================================================================
 * findmarginpeaks' numbers (surface_call_functions.cpp:316-734).  marginp
 * (:25-80) is margincalc's density over genealogies [ft, lt) with cc as
 * stored, divided by lt - ft + (ft == 0), negated, and OFFSCALEVAL (1)
 * outside the prior; marginpopmig / marginpop_expomig (popmig.cpp:181-351)
 * the same for 2NM.  The searches: mnbrakmod and goldenmod
 * (surface_search_functions.cpp:42-200), marginalopt (:178-266),
 * marginbis / margin95 (:86-113, :268-292), marginalopt_popmig
 * (popmig.cpp:361-428).
 * ==================================================================== */
#define PK_MINPARAMVAL 0.0000001
typedef struct {
  int G, rowlen, np, nm, expo, uniform2nm, kind, idx, ft, lt;
  const float *g;
  const double *thmin, *thmax, *mgmin, *mgmax, *mgmean;
  const int *mpop, *mterm;
  double yadjust;
  int st;
} PkCtx;

static double pk_marginp(PkCtx *k, double x)
{
  int p = k->idx, np = k->np, ccp, fcp, hccp, mcp, fmp, qip, mip, pdgp, probgp;
  double max = p < np ? k->thmax[p] : k->mgmax[p - np], min = p < np ? k->thmin[p] : k->mgmin[p - np];
  if (x < min || x > max) return 1;
  ora_gsamp_offsets(np, k->nm, &ccp, &fcp, &hccp, &mcp, &fmp, &qip, &mip, &pdgp, &probgp);
  double meani = (k->expo && p >= np) ? 1.0 / k->mgmean[p - np] : 0.0, sumtemp = 0.0;
  for (int e = k->ft; e < k->lt; e++) {
    const float *r = k->g + (size_t)e * k->rowlen;
    double temp;
    if (p < np) {
      temp = -r[qip + p] + r[ccp + p] * (ORA_LOG2 - log(x)) - r[hccp + p] - 2 * r[fcp + p] / x;
    } else {
      int q = p - np;
      if (k->expo)
        temp = -r[mip + q] + log(meani) - x * meani + ora_intround(r[mcp + q]) * log(x) - r[fmp + q] * x;
      else
        temp = -r[mip + q] + ora_intround(r[mcp + q]) * log(x) - r[fmp + q] * x;
    }
    sumtemp += exp(temp);
  }
  sumtemp /= (k->lt - k->ft + (k->ft == 0));
  return -sumtemp;
}

static double pk_marginpopmig(PkCtx *k, double x)
{
  int t = k->idx, th = k->mpop[t], mi = k->mterm[t], c[7];
  int expo = k->expo && !k->uniform2nm;
  double qmax = k->thmax[th], max = expo ? 20.0 * k->mgmean[mi] : qmax * k->mgmax[mi] / 2.0;
  if (x < 0 || x > max) return 1.0;
  popmig_cols(k->np, k->nm, th, mi, c);
  if (!expo) {
    double sum = pm_sum(k->g, k->rowlen, c, k->ft, k->lt, x, qmax, k->mgmax[mi], &k->st);
    sum /= (k->lt - k->ft + (k->ft == 0));
    return -sum;
  }
  double sum = pe_logsum(k->g, k->rowlen, c, k->ft, k->lt, x, qmax, k->mgmean[mi], &k->st);
  sum -= log((double)k->lt - k->ft + (k->ft == 0));
  return -exp(sum);
}

static double pk_f(PkCtx *k, double x)
{
  if (k->kind == 0) return pk_marginp(k, x);
  if (k->kind == 1) return ora_margincalc(k->lt, k->rowlen, k->g, k->np, k->nm, k->idx, x, k->yadjust, 1,
                                          k->expo ? k->mgmean : NULL);
  return pk_marginpopmig(k, x);
}

static double pk_sign(double a, double b) { return b > 0.0 ? fabs(a) : -fabs(a); }

static void pk_mnbrak(PkCtx *k, double *ax, double *bx, double *cx, double *fa, double *fb, double *fc)
{
  const double gold = 1.618034, glimit = 100.0, tiny = 1.0e-20;
  double ulim, u, rr, q, fu, dum;
  *fa = pk_f(k, *ax);
  *fb = pk_f(k, *bx);
  if (*fb > *fa) {
    dum = *ax; *ax = *bx; *bx = dum;
    dum = *fb; *fb = *fa; *fa = dum;
  }
  *cx = fabs(*bx + gold * (*bx - *ax));
  *fc = pk_f(k, *cx);
  while (*fb >= *fc && *fb > -DBL_MAX && !(*fb == 0 && *fc == 0)) {
    rr = (*bx - *ax) * (*fb - *fc);
    q = (*bx - *cx) * (*fb - *fa);
    float m1 = (float)fabs(q - rr), m2 = (float)tiny; /* FMAX's float variables */
    u = (double)*bx - ((*bx - *cx) * q - (*bx - *ax) * rr) / (2.0 * pk_sign(m1 > m2 ? m1 : m2, q - rr));
    ulim = *bx + glimit * (*cx - *bx);
    if ((*bx - u) * (u - *cx) > 0.0) {
      fu = pk_f(k, u);
      if (fu < *fc) { *ax = *bx; *fa = *fb; *bx = u; *fb = fu; continue; }
      if (fu > *fb) { *cx = u; *fc = fu; continue; }
      u = *cx + gold * (*cx - *bx);
      fu = pk_f(k, u);
    } else if ((*cx - u) * (u - ulim) > 0.0) {
      fu = pk_f(k, u);
      if (fu < *fc) {
        *bx = *cx; *cx = u; u = *cx + gold * (*cx - *bx);
        *fb = *fc; *fc = fu; fu = pk_f(k, u);
      }
    } else if ((u - ulim) * (ulim - *cx) >= 0.0) {
      u = ulim;
      fu = pk_f(k, u);
    } else {
      u = *cx + gold * (*cx - *bx);
      fu = pk_f(k, u);
    }
    *ax = *bx; *bx = *cx; *cx = u;
    *fa = *fb; *fb = *fc; *fc = fu;
  }
}

static double pk_golden(PkCtx *k, double ax, double bx, double cx, double tol, double *xmin)
{
  const double r = 0.61803399, c = 1.0 - r;
  double f1, f2, x0 = ax, x1, x2, x3 = cx;
  if (fabs(cx - bx) > fabs(bx - ax)) { x1 = bx; x2 = bx + c * (cx - bx); }
  else { x2 = bx; x1 = bx - c * (bx - ax); }
  f1 = pk_f(k, x1);
  f2 = pk_f(k, x2);
  while (fabs(x3 - x0) > tol * (fabs(x1) + fabs(x2)) && (x3 > -DBL_MAX)) {
    if (f2 < f1) {
      x0 = x1; x1 = x2; x2 = r * x1 + c * x3; f1 = f2; f2 = pk_f(k, x2);
      continue;
    }
    x3 = x2; x2 = x1; x1 = r * x2 + c * x0; f2 = f1; f1 = pk_f(k, x1);
  }
  if (f1 < f2) { *xmin = x1; return f1; }
  *xmin = x2;
  return f2;
}

static double pk_bis(PkCtx *k, double x1, double x2)
{
  double dx, f, fmid, xmid, rtb;
  f = pk_f(k, x1);
  fmid = pk_f(k, x2);
  if (f * fmid >= 0.0) return DBL_MIN;
  rtb = f < 0.0 ? (dx = x2 - x1, x1) : (dx = x1 - x2, x2);
  for (int j = 1; j <= 40; j++) {
    fmid = pk_f(k, xmid = rtb + (dx *= 0.5));
    if (fmid <= 0.0) rtb = xmid;
    if (fabs(dx) < 1e-4 || fmid == 0.0) return rtb;
  }
  return DBL_MAX;
}

static void pk_marginalopt(PkCtx *k, double *mlval, double *peakloc)
{
  int npar = k->np + k->nm;
  double ax, bx, cx, fa, fb, fc, axt, bxt, cxt, prior, xmax;
  double max0 = 0, min0 = 0, max1 = 0, min1 = 0; /* the reference leaves them unset */
  k->kind = 0;
  for (int i = 0; i < npar; i++) {
    k->idx = i;
    prior = i < k->np ? k->thmax[i] : k->mgmax[i - k->np];
    ax = prior; bx = prior / 2;
    pk_mnbrak(k, &ax, &bx, &cx, &fa, &fb, &fc);
    axt = ax; bxt = bx; cxt = cx;
    bx = prior / 2; ax = PK_MINPARAMVAL;
    pk_mnbrak(k, &ax, &bx, &cx, &fa, &fb, &fc);
    if (axt < bxt && axt < cxt) min0 = axt;
    if (bxt < axt && bxt < cxt) min0 = bxt;
    if (cxt < axt && cxt < bxt) min0 = cxt;
    if (axt > bxt && axt > cxt) { if (axt > prior) axt = prior; max0 = axt; }
    if (bxt > axt && bxt > cxt) { if (bxt > prior) bxt = prior; max0 = bxt; }
    if (cxt > axt && cxt > bxt) { if (cxt > prior) cxt = prior; max0 = cxt; }
    if (ax < bx && ax < cx) min1 = ax;
    if (bx < ax && bx < cx) min1 = bx;
    if (cx < ax && cx < bx) min1 = cx;
    if (ax > bx && ax > cx) max1 = ax;
    { if (ax > prior) ax = prior; max1 = ax; } /* unconditional, as in the reference */
    if (bx > ax && bx > cx) { if (bx > prior) bx = prior; max1 = bx; }
    if (cx > ax && cx > bx) { if (cx > prior) cx = prior; max1 = cx; }
    if (max0 <= min1 || max1 <= min0) {
      peakloc[i] = -1;
      mlval[i] = NAN;
    } else {
      mlval[i] = -pk_golden(k, ax, bx, cx, 1e-7, &xmax);
      peakloc[i] = xmax;
    }
  }
}

static void pk_marginalopt_popmig(PkCtx *k, int nt, double *mlval, double *peakloc)
{
  double ax, bx, cx, fa, xmax, ub, maxf;
  int maxj;
  k->kind = 2;
  k->uniform2nm = 0;
  for (int i = 0; i < nt; i++) {
    k->idx = i;
    ub = k->expo ? 20.0 * k->mgmean[k->mterm[i]] : k->thmax[k->mpop[i]] * k->mgmax[k->mterm[i]] / 2.0;
    maxf = 1e100;
    maxj = -1;
    for (int j = 0; j < 100; j++) {
      ax = PK_MINPARAMVAL + j * (ub / (double)100);
      fa = pk_f(k, ax);
      if (fa < maxf) { maxf = fa; maxj = j; }
    }
    if (maxj == 0) {
      ax = PK_MINPARAMVAL; cx = PK_MINPARAMVAL + ub / (double)100; bx = (ax + cx) / 2.0;
    } else if (maxj == 100 - 1) {
      ax = PK_MINPARAMVAL + ((double)100 - 1) * (ub / (double)100);
      bx = PK_MINPARAMVAL + ((double)100 - 2) * (ub / (double)100);
      cx = ub;
    } else {
      bx = PK_MINPARAMVAL + ((double)maxj - 1) * (ub / (double)100);
      cx = PK_MINPARAMVAL + ((double)maxj + 1) * (ub / (double)100);
      ax = PK_MINPARAMVAL + ((double)maxj) * (ub / (double)100);
    }
    mlval[i] = -pk_golden(k, ax, bx, cx, 1e-7, &xmax);
    peakloc[i] = xmax;
  }
}

int ora_findmarginpeaks(int G, int rowlen, const float *g, int np, int nm, const double *thmin,
                        const double *thmax, const double *mgmin, const double *mgmax, const double *mgmean,
                        int nt, const int *mpop, const int *mterm, double *mlval, double *peakloc,
                        double *migtest, double *lo95, double *hi95, double *pm_mlval, double *pm_peakloc,
                        double *pm_test)
{
  PkCtx k;
  memset(&k, 0, sizeof(k));
  k.G = G; k.rowlen = rowlen; k.g = g; k.np = np; k.nm = nm; k.expo = mgmean != NULL;
  k.thmin = thmin; k.thmax = thmax; k.mgmin = mgmin; k.mgmax = mgmax; k.mgmean = mgmean;
  k.mpop = mpop; k.mterm = mterm;
  int Gs = G < 300000 - 1 ? G : 300000 - 1, npar = np + nm, ft, lt, j;
  if (Gs <= 10) return -1;
  for (ft = 0, lt = Gs / 2, j = 0; j < 2; j++) {
    k.ft = ft; k.lt = lt;
    pk_marginalopt(&k, mlval + (size_t)j * npar, peakloc + (size_t)j * npar);
    if (nt) pk_marginalopt_popmig(&k, nt, pm_mlval + (size_t)j * nt, pm_peakloc + (size_t)j * nt);
    ft = lt + 1;
    lt += Gs / 2;
    if (lt > Gs) lt = Gs;
  }
  k.ft = 0; k.lt = Gs;
  double *pk = peakloc + 2 * (size_t)npar, *ml = mlval + 2 * (size_t)npar;
  pk_marginalopt(&k, ml, pk);
  k.kind = 0;
  for (int i = 0; i < nm; i++) {
    k.idx = np + i;
    double maxp = -pk_f(&k, pk[np + i]), max0p = -pk_f(&k, PK_MINPARAMVAL);
    migtest[i] = 2 * log(maxp / max0p);
  }
  k.kind = 1;
  for (int i = 0; i < npar; i++) {
    lo95[i] = hi95[i] = NAN;
    if (!(pk[i] >= 0)) continue;
    k.idx = i;
    k.yadjust = log(ml[i]) - 1.92;
    lo95[i] = pk_bis(&k, PK_MINPARAMVAL, pk[i]);
    hi95[i] = pk_bis(&k, pk[i], i < np ? thmax[i] : mgmax[i - np]);
  }
  if (nt) {
    pk_marginalopt_popmig(&k, nt, pm_mlval + 2 * (size_t)nt, pm_peakloc + 2 * (size_t)nt);
    k.kind = 2;
    k.uniform2nm = 1; /* the test calls marginpopmig whatever the prior */
    for (int t = 0; t < nt; t++) {
      k.idx = t;
      double maxp = -pk_f(&k, pm_peakloc[2 * (size_t)nt + t]), max0p = -pk_f(&k, PK_MINPARAMVAL);
      pm_test[t] = 2 * log(maxp / max0p);
    }
  }
  return k.st;
}

/* ======================================================================
 * .ti loading, the reference's way (loadgenealogyvalues,
 * ima_main_mpi.cpp:3370-3400): lines up to VALUESSTART skipped, then one
 * fgets per genealogy (a buffer of rowlen * 20 characters) and one
 * sscanf("%f") per value, stepping to the next whitespace; every genealogy
 * kept.  Returns the number of rows read (at most cap), or -1 when the file
 * cannot be opened.  Used as the one-core baseline of the library's parser.
 * ==================================================================== */
int ora_ti_load(const char *path, int rowlen, float *rows, int cap)
{
  FILE *f = fopen(path, "r");
  if (!f) return -1;
  char head[300];
  while (fgets(head, sizeof(head), f) && strstr(head, "VALUESSTART") == NULL && !feof(f)) {
  }
  size_t blen = (size_t)rowlen * 20;
  char *line = (char *)malloc(blen);
  int loaded = 0;
  while (line && loaded < cap && fgets(line, (int)blen, f) && !feof(f)) {
    char *c = line;
    for (int i = 0; i < rowlen; i++) {
      sscanf(c, "%f", &rows[(size_t)loaded * rowlen + i]);
      while (*c && isspace((unsigned char)*c)) c++; /* nextwhite: past this value */
      while (*c && !isspace((unsigned char)*c)) c++;
    }
    loaded++;
  }
  free(line);
  fclose(f);
  return loaded;
}
