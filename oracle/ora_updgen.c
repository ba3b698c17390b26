/* ora_updgen.c -- TEST INFRASTRUCTURE (the CPU checker and the timed CPU
 * baseline), never part of the product.
 *
 * The genealogy update updategenealogy (update_gtree.cpp:723-966) of the
 * no-migration model restated in C: the edge draw, normdev's slide distance
 * (utilities.cpp:476-503), joinsisdown (update_gtree.cpp:375-455), the slide
 * slider_nomigration (:79-254) with findjointime (:34-77) and bitran
 * (utilities.cpp:438-455), splitsisdown (update_gtree.cpp:457-534), the
 * slide's Hastings term, the locus's new weights (ora_treeweight), the
 * chain's sums plus new minus old (sum_subtract_treeinfo, ginfo.cpp:249-285),
 * p(G) with the unchanged theta integrals kept (integrate_tree_prob,
 * update_gtree_common.cpp:1945-2055), the likelihood (ora_is_likelihood in
 * full, ora_hky_likelihood from the four edited edges) and the
 * Metropolis-Hastings decision with one uniform (none when the IS
 * likelihood rejects).  A rejection restores the genealogy, its weights and
 * the HKY scale factors.  Stepwise loci (one marker) take finishSWupdateA
 * (update_gtree_common.cpp:2219-2362) for the likelihood change: a new allele
 * for the freed node drawn around its neighbours' (geometric, bitran), the
 * moved branches' terms, and the allele proposal's Hastings term; a
 * rejection restores them as restoreedges does (:706-825), which leaves the
 * new sister's term in place when it was 0 before (the root edge's).  Each
 * chain draws from its own generators (ora_ug_rng), as the device form does;
 * chains run on host threads. */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ima_oracle.h"

#define UG_TIMEMAX 1000000.0          /* imamp.hpp:129 */
#define UG_SLIDESTDVMAX 20.0          /* update_gtree.cpp:686 */
#define UG_ONEOVERSQRT2PI 0.3989422803 /* utilities.cpp:461 */
#define UG_REJECT_IS -1000000000.0    /* imamp.hpp:157 */

void ora_ug_rng_seed(ora_ug_rng *g, int seed)
{
  ora_mt_seed(&g->mt, (uint32_t)seed);
  g->iset = 0;
  g->gset = 0.0;
  g->iseed = 0x7fffffffffffffffull + (uint64_t)(int64_t)seed;
}

static double ug_uniform(ora_ug_rng *g) { return ora_mt_uniform(&g->mt); }

static int ug_bitran(ora_ug_rng *g)
{
  if (g->iseed & 131072ull) {
    g->iseed = ((g->iseed ^ 19ull) << 1) | 1ull;
    return 1;
  }
  g->iseed <<= 1;
  return 0;
}

static double ug_normdev(ora_ug_rng *g, double mean, double stdev)
{
  if (g->iset == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * ug_uniform(g) - 1.0;
      v2 = 2.0 * ug_uniform(g) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = sqrt(-2.0 * log(rsq) / rsq);
    g->gset = v1 * fac;
    g->iset = 1;
    return v2 * fac * stdev + mean;
  }
  g->iset = 0;
  return g->gset * stdev + mean;
}

static double ug_normprob(double mean, double stdev, double val)
{
  const double z = (val - mean) / stdev;
  const double sq = (z == 0.0) ? 0.0 : z * z;
  return UG_ONEOVERSQRT2PI * exp(-sq / 2) / stdev;
}

static double ug_dmin(double a, double b) { return a < b ? a : b; }

static int ug_period(const double *tv, int nsplit, double t)
{
  int k = 0;
  while (k < nsplit && tv[k] <= t) k++;
  return k;
}

typedef struct {
  int npops;
  const int *plist, *droppops, *addpop, *pop_e, *pop_down;
  int nth;
  const int *th_off, *th_idx;
  const double *th_max, *th_min;
  int nloci;
  const int *model, *n, *S, *totsites;
  const long long *seq_off, *mult_off;
  const int8_t *seq;
  const int *mult;
  const double *hval;
  const int *samppop;
  const double *sumlogk;
  const int *arange;   /* SW: [nloci][2] minA, maxA */
  int *alleles;        /* SW: per node, in place */
  int nchains;
  const long long *node_off;
  int *up0, *up1, *down, *pop;
  double *time;
  const double *tvals, *beta, *u, *kappa, *pi;
  double gbeta;
  int nsweeps;
  ora_ug_rng *rng;
  int *res;
  double *resd, *pdg_out, *probg_out;
  int next, err;
} ug_job;

static double ug_jointime(const ug_job *J, const double *tv, int slidepop, int sispop, double eut, double sut)
{
  const int nsplit = J->npops - 1;
  int ep = ug_period(tv, nsplit, eut), sp = ug_period(tv, nsplit, sut);
  const int *dp = J->droppops;
  while (ep < sp) {
    ep++;
    if (slidepop == dp[2 * ep] || slidepop == dp[2 * ep + 1]) slidepop = J->pop_down[slidepop];
  }
  while (sp < ep) {
    sp++;
    if (sispop == dp[2 * sp] || sispop == dp[2 * sp + 1]) sispop = J->pop_down[sispop];
  }
  while (slidepop != sispop && ep < nsplit) {
    ep++;
    if (slidepop == dp[2 * ep] || slidepop == dp[2 * ep + 1]) slidepop = J->pop_down[slidepop];
    if (sispop == dp[2 * ep] || sispop == dp[2 * ep + 1]) sispop = J->pop_down[sispop];
  }
  return ep == 0 ? 0.0 : tv[ep - 1];
}

/* the proposal on one genealogy (edge arrays of one chain-locus, in place);
 * out: e[4] = edge, freed, oldsis, newsis; *topol, *tmrca, *sw; returns 0 or
 * 1 for a slide that did not end / a root beyond TIMEMAX */
static int ug_propose(const ug_job *J, const double *tv, ora_ug_rng *g, int n, int *up0, int *up1, int *down,
                      double *t, int *pop, double *dl, int *e, int *topol, int *tmrca, double *sw)
{
  const int nl = 2 * n - 1, nsplit = J->npops - 1;
  int root = -1;
  for (int k = 0; k < nl; k++)
    if (down[k] == -1) root = k;
  double roottime = t[up0[root]];
  int edge;
  do {
    edge = (int)floor(ug_uniform(g) * nl);
  } while (down[edge] == -1);
  const int freed = down[edge];
  const int oldsis = (up0[freed] == edge) ? up1[freed] : up0[freed];
  double slidestdv = ug_dmin(UG_SLIDESTDVMAX, roottime / 3);
  const double hold = ug_normdev(g, 0.0, slidestdv);
  double dist = hold;
  int rootmove, bad = 0;
  *tmrca = 0;
  {
    const int dn = down[oldsis];
    t[oldsis] = t[dn];
    const int dd = down[dn];
    down[oldsis] = dd;
    if (dd != -1) {
      rootmove = 0;
      if (up0[dd] == dn) up0[dd] = oldsis;
      else up1[dd] = oldsis;
    } else {
      rootmove = 1;
      (*tmrca)++;
      const double uptime = (oldsis < n) ? 0.0 : t[up0[oldsis]];
      root = oldsis;
      down[oldsis] = -1;
      t[oldsis] = UG_TIMEMAX;
      if (dl) dl[oldsis] = 0;
      roottime = uptime;
    }
  }
  int sis = oldsis;
  double tp = t[edge];
  long steps = 0;
  for (;;) {
    if (++steps > (1L << 20)) {
      bad = 1;
      break;
    }
    if (dist < 0) {
      dist = -dist;
      const double eut = (edge < n) ? 0.0 : t[up0[edge]];
      const double sut = (sis < n) ? 0.0 : t[up0[sis]];
      const double pjt = (pop[edge] != pop[sis]) ? ug_jointime(J, tv, pop[edge], pop[sis], eut, sut) : 0.0;
      if (pjt > eut && pjt > sut) {
        if (dist < tp - pjt) {
          tp -= dist;
          dist = 0;
          break;
        }
        dist -= tp - pjt;
        tp = pjt;
      } else if (sut == 0 || eut >= sut) {
        if (dist < tp - eut) {
          tp -= dist;
          dist = 0;
          break;
        }
        dist -= tp - eut;
        tp = eut;
      } else {
        if (dist < tp - sut) {
          tp -= dist;
          dist = 0;
          break;
        }
        dist -= tp - sut;
        tp = sut;
        sis = ug_bitran(g) ? up0[sis] : up1[sis];
        dist = -dist;
      }
    } else {
      if (down[sis] == -1 || tp + dist < t[sis]) {
        tp += dist;
        if (tp >= UG_TIMEMAX) tp = UG_TIMEMAX;
        dist = 0;
        break;
      }
      dist -= t[sis] - tp;
      tp = t[sis];
      if (ug_bitran(g)) {
        sis = down[sis];
      } else {
        const int d = down[sis];
        sis = (up0[d] == sis) ? up1[d] : up0[d];
        dist = -dist;
      }
    }
  }
  t[edge] = tp;
  const int newsis = sis;
  {
    const double curt = t[edge];
    t[freed] = t[newsis];
    t[newsis] = curt;
    const int dd = down[newsis];
    if (dd != -1) {
      if (up0[dd] == newsis) up0[dd] = freed;
      else up1[dd] = freed;
    } else {
      root = freed;
      roottime = curt;
      rootmove = 1;
      if (roottime > UG_TIMEMAX) bad = 1;
      if (dl) dl[freed] = 0;
    }
    down[freed] = dd;
    int nowpop = pop[newsis];
    const int j = ug_period(tv, nsplit, curt);
    while (J->pop_e[nowpop] <= j && J->pop_e[nowpop] != -1) nowpop = J->pop_down[nowpop];
    pop[freed] = nowpop;
    down[newsis] = freed;
    down[edge] = freed;
    up0[freed] = newsis;
    up1[freed] = edge;
  }
  *sw = 0.0;
  if (rootmove) {
    *sw = -log(ug_normprob(0.0, slidestdv, hold));
    slidestdv = ug_dmin(UG_SLIDESTDVMAX, roottime / 3);
    *sw += log(ug_normprob(0.0, slidestdv, hold));
  }
  e[0] = edge;
  e[1] = freed;
  e[2] = oldsis;
  e[3] = newsis;
  *topol = (oldsis != newsis);
  return bad;
}

/* finishSWupdateA (update_gtree_common.cpp:2219-2362) for one marker on the
 * proposed genealogy; bkA/bkdl/bkdown: the alleles, terms and parents
 * before the proposal (storeoldedges' copies).  Returns likeadj - oldlikeadj;
 * *aterm the allele proposal's Hastings term, *holdsis the new sister's
 * term before the update (restoreedges puts it back only when nonzero). */
static double ug_sw_update(ora_ug_rng *g, int n, const int *up0, const int *down, const double *t, int *A, double *dl,
                           int edge, int freed, int oldsis, int newsis, double u, int minA, int maxA,
                           const int *bkA, const double *bkdl, const int *bkdown, double *aterm, double *holdsis)
{
  const int oldA = A[freed];
  *holdsis = (newsis != oldsis) ? dl[newsis] : 0.0;
  const double cp2 = bkdown[freed] != -1 ? bkdl[freed] : 0.0;
  const int holddownA = bkdown[freed] != -1 ? bkA[bkdown[freed]] : -1;
  const double oldlikeadj = bkdl[edge] + bkdl[oldsis] + cp2 + *holdsis;
  const int e[3] = {edge, newsis, down[edge]};
  double tt[3] = {0.0, 0.0, 0.0};
  for (int i = 0; i < 3; i++) {
    const double upt = e[i] >= n ? t[up0[e[i]]] : 0.0;
    if (down[e[i]] != -1) tt[i] = t[e[i]] - upt;
  }
  int wsumdiff = 0, j = 0;
  for (int i = 0; i < 3; i++)
    if (down[e[i]] != -1) {
      const int d = (i < 2 ? A[e[i]] : A[down[e[i]]]) - oldA;
      wsumdiff += abs(d);
      j++;
    }
  double geotermnew = j / ((double)(wsumdiff + j));
  if (geotermnew > 0.95) geotermnew = 0.95;
  int dA = (int)ceil(log(ug_uniform(g)) / log(1.0 - geotermnew)) - 1;
  if (ug_bitran(g)) dA = -dA;
  int newA;
  if (dA >= 0) newA = (maxA < oldA + dA) ? maxA : oldA + dA;
  else newA = (minA > oldA + dA) ? minA : oldA + dA;
  A[freed] = newA;
  dA = newA - oldA;
  if (down[oldsis] != -1 && oldsis != newsis) {
    const double upt = oldsis >= n ? t[up0[oldsis]] : 0.0;
    const int d = A[oldsis] - A[down[oldsis]];
    dl[oldsis] = -(t[oldsis] - upt) * u + log(ora_bessi(d, (t[oldsis] - upt) * u));
  } else {
    dl[oldsis] = 0;
  }
  double likeadj = dl[oldsis];
  for (int i = 0; i < 3; i++)
    if (down[e[i]] != -1) {
      const int d = (i < 2 ? A[e[i]] : A[down[e[i]]]) - newA;
      dl[e[i]] = -(tt[i] * u) + log(ora_bessi(d, tt[i] * u));
      likeadj += dl[e[i]];
    }
  wsumdiff = abs(bkA[edge] - newA) + abs(bkA[oldsis] - newA);
  j = 2;
  if (bkdown[freed] != -1) {
    wsumdiff += abs(holddownA - newA);
    j++;
  }
  double geotermold = j / ((double)(wsumdiff + j));
  if (geotermold > 0.95) geotermold = 0.95;
  *aterm = (abs(dA) * log(1 - geotermold) + log(geotermold)) - (abs(dA) * log(1 - geotermnew) + log(geotermnew));
  return likeadj - oldlikeadj;
}

static int ug_root(int nl, const int *down)
{
  for (int i = 0; i < nl; i++)
    if (down[i] == -1) return i;
  return nl - 1;
}

static int ug_chain(ug_job *J, int c)
{
  const int nl_ = J->nloci, npops = J->npops, nsplit = npops - 1;
  int T, M;
  ora_tw_sizes(npops, &T, &M);
  const double *tv = J->tvals + (size_t)c * nsplit;
  ora_ug_rng *g = J->rng + c;
  int maxn = 0, maxS = 0;
  for (int l = 0; l < nl_; l++) {
    if (J->n[l] > maxn) maxn = J->n[l];
    if (J->S[l] > maxS) maxS = J->S[l];
  }
  const int mnl = 2 * maxn - 1;
  int *wcc = (int *)calloc((size_t)nl_ * T, sizeof(int)), *ncc = (int *)calloc(T, sizeof(int));
  double *wfc = (double *)calloc((size_t)nl_ * T, sizeof(double)), *whc = (double *)calloc((size_t)nl_ * T, sizeof(double));
  double *nfc = (double *)calloc(T, sizeof(double)), *nhc = (double *)calloc(T, sizeof(double));
  int *mc = (int *)calloc(M > 0 ? M : 1, sizeof(int));
  double *fm = (double *)calloc(M > 0 ? M : 1, sizeof(double));
  int *agc = (int *)calloc(T, sizeof(int)), *sgc = (int *)calloc(T, sizeof(int));
  double *agf = (double *)calloc(T, sizeof(double)), *agh = (double *)calloc(T, sizeof(double));
  double *sgf = (double *)calloc(T, sizeof(double)), *sgh = (double *)calloc(T, sizeof(double));
  double *qint = (double *)calloc(J->nth, sizeof(double)), *nq = (double *)calloc(J->nth, sizeof(double));
  double *len = (double *)calloc(nl_, sizeof(double)), *pdg = (double *)calloc(nl_, sizeof(double));
  int *moff = (int *)calloc((size_t)mnl + 1, sizeof(int));
  int *bk = (int *)malloc(sizeof(int) * 4 * (size_t)mnl);
  double *bkt = (double *)malloc(sizeof(double) * (size_t)mnl);
  double **frac = (double **)calloc(nl_, sizeof(double *));
  double **dls = (double **)calloc(nl_, sizeof(double *));  /* SW: the branch terms (dlikeA) */
  int *bkA = (int *)malloc(sizeof(int) * (size_t)mnl);
  double *bkdl = (double *)malloc(sizeof(double) * (size_t)mnl);
  int err = 0;
  if (!wcc || !ncc || !wfc || !whc || !nfc || !nhc || !mc || !fm || !agc || !sgc || !agf || !agh || !sgf || !sgh ||
      !qint || !nq || !len || !pdg || !moff || !bk || !bkt || !frac || !dls || !bkA || !bkdl) {
    err = 5;
    goto out;
  }
  /* the chain as finish_setup_C leaves it */
  for (int l = 0; l < nl_ && !err; l++) {
    const int n = J->n[l], nl = 2 * n - 1, S = J->S[l];
    const long long o = J->node_off[(size_t)c * nl_ + l];
    int *u0 = J->up0 + o, *u1 = J->up1 + o, *dn = J->down + o, *pp = J->pop + o;
    double *t = J->time + o, out3[3];
    int mig;
    if (ora_treeweight(npops, J->plist, J->droppops, J->addpop, J->pop_e, J->pop_down, tv, 1, n,
                       J->samppop + (size_t)l * npops, J->hval[l], u0, t, pp, moff, NULL, NULL,
                       wcc + (size_t)l * T, whc + (size_t)l * T, wfc + (size_t)l * T, mc, fm, out3, &mig)) {
      err = 2;
      break;
    }
    len[l] = out3[0];
    for (int q = 0; q < T; q++) {
      agc[q] += wcc[(size_t)l * T + q];
      agf[q] += wfc[(size_t)l * T + q];
      agh[q] += whc[(size_t)l * T + q];
    }
    const int8_t *sq = J->seq + J->seq_off[l];
    const double uu = J->u[(size_t)c * nl_ + l];
    int st = 0;
    if (J->model[l] == 2) {
      dls[l] = (double *)calloc((size_t)nl, sizeof(double));
      if (!dls[l]) { err = 5; break; }
      pdg[l] = ora_sw_likelihood(n, J->alleles + o, dn, u0, t, uu, 1.0, dls[l]);
    } else if (J->model[l] == 1) {
      frac[l] = (double *)calloc((size_t)nl * S * 10, sizeof(double));
      if (!frac[l]) { err = 5; break; }
      double *f = frac[l], *nf = f + (size_t)nl * S * 4, *sf = nf + (size_t)nl * S * 4, *osf = sf + (size_t)nl * S;
      const int efull[4] = {-1, -1, -1, -1};
      pdg[l] = ora_hky_likelihood(n, S, J->totsites[l], sq, J->mult + J->mult_off[l],
                                  J->pi + 4 * ((size_t)c * nl_ + l), u0, u1, dn, ug_root(nl, dn), t, uu,
                                  J->kappa[(size_t)c * nl_ + l], efull, f, nf, sf, osf);
      ora_hky_copyfraclike(n, S, nf, f);
      ora_hky_storescalefactors(n, S, sf, osf);
    } else {
      pdg[l] = ora_is_likelihood(n, S, sq, u0, u1, dn, t, len[l], uu, J->sumlogk[l], NULL, &st);
      if (st) err = 3;
    }
  }
  double probg = 0.0;
  if (!err) {
    double mq[1];
    int z = 0;
    if (ora_tree_prob(1, 0, agc, agh, agf, &z, mq, J->nth, J->th_off, J->th_idx, J->th_max, J->th_min, 0, &z, &z,
                      mq, mq, mq, 0, &z, &probg, qint, mq))
      err = 4;
  }
  for (int s = 0; s < J->nsweeps && !err; s++)
    for (int l = 0; l < nl_ && !err; l++) {
      const int n = J->n[l], nl = 2 * n - 1, S = J->S[l];
      const long long o = J->node_off[(size_t)c * nl_ + l];
      int *u0 = J->up0 + o, *u1 = J->up1 + o, *dn = J->down + o, *pp = J->pop + o;
      double *t = J->time + o;
      memcpy(bk, u0, sizeof(int) * nl);
      memcpy(bk + mnl, u1, sizeof(int) * nl);
      memcpy(bk + 2 * mnl, dn, sizeof(int) * nl);
      memcpy(bk + 3 * mnl, pp, sizeof(int) * nl);
      memcpy(bkt, t, sizeof(double) * nl);
      int *A = J->model[l] == 2 ? J->alleles + o : NULL;
      double *dl = dls[l];
      if (A) {
        memcpy(bkA, A, sizeof(int) * nl);
        memcpy(bkdl, dl, sizeof(double) * nl);
      }
      int e[4], topol, tmrca, acc = 0;
      double sw;
      if (ug_propose(J, tv, g, n, u0, u1, dn, t, pp, dl, e, &topol, &tmrca, &sw)) {
        err = 1;
        break;
      }
      double out3[3];
      int mig;
      if (ora_treeweight(npops, J->plist, J->droppops, J->addpop, J->pop_e, J->pop_down, tv, 1, n,
                         J->samppop + (size_t)l * npops, J->hval[l], u0, t, pp, moff, NULL, NULL, ncc, nhc, nfc, mc,
                         fm, out3, &mig)) {
        err = 2;
        break;
      }
      const int8_t *sq = J->seq + J->seq_off[l];
      const double uu = J->u[(size_t)c * nl_ + l];
      double newpdg, aterm = 0.0, holdsis = 0.0;
      int rejectIS = 0, st = 0;
      double *f = NULL, *nf = NULL, *sf = NULL, *osf = NULL;
      if (A) {
        const double dlt = ug_sw_update(g, n, u0, dn, t, A, dl, e[0], e[1], e[2], e[3], uu, J->arange[2 * l],
                                        J->arange[2 * l + 1], bkA, bkdl, bk + 2 * mnl, &aterm, &holdsis);
        newpdg = 0.0 + (pdg[l] + dlt);
      } else if (J->model[l] == 1) {
        f = frac[l];
        nf = f + (size_t)nl * S * 4;
        sf = nf + (size_t)nl * S * 4;
        osf = sf + (size_t)nl * S;
        newpdg = ora_hky_likelihood(n, S, J->totsites[l], sq, J->mult + J->mult_off[l],
                                    J->pi + 4 * ((size_t)c * nl_ + l), u0, u1, dn, ug_root(nl, dn), t, uu,
                                    J->kappa[(size_t)c * nl_ + l], e, f, nf, sf, osf);
      } else {
        newpdg = ora_is_likelihood(n, S, sq, u0, u1, dn, t, out3[0], uu, J->sumlogk[l], NULL, &st);
        if (st == 2) {
          err = 3;
          break;
        }
        rejectIS = (newpdg == UG_REJECT_IS);
      }
      double psum = probg;
      if (!rejectIS) {
        const int *oc = wcc + (size_t)l * T;
        const double *of = wfc + (size_t)l * T, *oh = whc + (size_t)l * T;
        for (int q = 0; q < T; q++) {
          sgc[q] = agc[q] + (ncc[q] - oc[q]);
          double x = agf[q];
          x -= of[q];
          x += nfc[q];
          sgf[q] = (0 > x) ? 0.0 : x;
          double h = agh[q];
          h -= oh[q];
          h += nhc[q];
          sgh[q] = h;
        }
        psum = 0;
        for (int i = 0; i < J->nth && !err; i++) {
          int cc = 0, holdc = 0;
          double ff = 0.0, holdf = 0.0, hc = 0.0;
          for (int j = J->th_off[i]; j < J->th_off[i + 1]; j++) {
            const int cell = J->th_idx[j];
            cc += sgc[cell];
            holdc += agc[cell];
            ff += sgf[cell];
            holdf += agf[cell];
            hc += sgh[cell];
          }
          int ist = 0;
          nq[i] = (cc == holdc && ff == holdf) ? qint[i] : ora_iterm(0, cc, ff, hc, J->th_max[i], J->th_min[i], &ist);
          if (ist) err = 4;
          psum += nq[i];
        }
        if (err) break;
        double tpw = -probg;
        tpw += psum;
        double mh = tpw + J->gbeta * (newpdg - pdg[l]);
        mh = exp(J->beta[c] * mh + sw + aterm);
        const double U = ug_uniform(g);
        acc = U < ug_dmin(1.0, mh);
      }
      if (acc) {
        probg = psum;
        pdg[l] = newpdg;
        len[l] = out3[0];
        memcpy(agc, sgc, sizeof(int) * T);
        memcpy(agf, sgf, sizeof(double) * T);
        memcpy(agh, sgh, sizeof(double) * T);
        memcpy(qint, nq, sizeof(double) * J->nth);
        memcpy(wcc + (size_t)l * T, ncc, sizeof(int) * T);
        memcpy(wfc + (size_t)l * T, nfc, sizeof(double) * T);
        memcpy(whc + (size_t)l * T, nhc, sizeof(double) * T);
        if (f) {
          ora_hky_copyfraclike(n, S, nf, f);
          ora_hky_storescalefactors(n, S, sf, osf);
        }
      } else {
        memcpy(u0, bk, sizeof(int) * nl);
        memcpy(u1, bk + mnl, sizeof(int) * nl);
        memcpy(dn, bk + 2 * mnl, sizeof(int) * nl);
        memcpy(pp, bk + 3 * mnl, sizeof(int) * nl);
        memcpy(t, bkt, sizeof(double) * nl);
        if (f) ora_hky_restorescalefactors(n, S, sf, osf);
        if (A) {  /* restoreedges: the three moved edges from their copies, the new sister only if nonzero */
          const int freed = e[1], oldsis = e[2], newsis = e[3];
          A[freed] = bkA[freed];
          dl[e[0]] = bkdl[e[0]];
          dl[oldsis] = bkdl[oldsis];
          dl[freed] = bk[2 * mnl + freed] != -1 ? bkdl[freed] : 0.0;
          if (holdsis != 0) dl[newsis] = holdsis;
        }
        topol = tmrca = 0;
      }
      const size_t r = ((size_t)c * J->nsweeps + s) * nl_ + l;
      if (J->res) {
        J->res[3 * r] = acc;
        J->res[3 * r + 1] = topol;
        J->res[3 * r + 2] = tmrca;
      }
      if (J->resd) {
        J->resd[2 * r] = pdg[l];
        J->resd[2 * r + 1] = probg;
      }
    }
  if (!err) {
    for (int l = 0; l < nl_; l++)
      if (J->pdg_out) J->pdg_out[(size_t)c * nl_ + l] = pdg[l];
    if (J->probg_out) J->probg_out[c] = probg;
  }
out:
  if (frac)
    for (int l = 0; l < nl_; l++) free(frac[l]);
  free(frac);
  if (dls)
    for (int l = 0; l < nl_; l++) free(dls[l]);
  free(dls);
  free(bkA);
  free(bkdl);
  free(wcc); free(ncc); free(wfc); free(whc); free(nfc); free(nhc); free(mc); free(fm);
  free(agc); free(sgc); free(agf); free(agh); free(sgf); free(sgh); free(qint); free(nq);
  free(len); free(pdg); free(moff); free(bk); free(bkt);
  return err;
}

static void *ug_worker(void *arg)
{
  ug_job *J = (ug_job *)arg;
  for (;;) {
    const int c = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (c >= J->nchains) break;
    const int e = ug_chain(J, c);
    if (e) __atomic_store_n(&J->err, e, __ATOMIC_RELAXED);
  }
  return NULL;
}

int ora_ug_run(int npops, const int *plist, const int *droppops, const int *addpop, const int *pop_e,
               const int *pop_down, int nth, const int *th_off, const int *th_idx, const double *th_max,
               const double *th_min, int nloci, const int *model, const int *n, const int *S, const int *totsites,
               const long long *seq_off, const long long *mult_off, const int8_t *seq, const int *mult,
               const double *hval, const int *samppop, const double *sumlogk, const int *arange, int nchains,
               const long long *node_off, int *up0, int *up1, int *down, double *time, int *pop, int *alleles,
               const double *tvals, const double *beta, double gbeta, const double *u, const double *kappa,
               const double *pi, int nsweeps, ora_ug_rng *rng, int nthreads, int *res, double *resd,
               double *pdg_out, double *probg_out)
{
  ug_job J = {npops, plist, droppops, addpop, pop_e, pop_down, nth, th_off, th_idx, th_max, th_min, nloci, model,
              n, S, totsites, seq_off, mult_off, seq, mult, hval, samppop, sumlogk, arange, alleles, nchains,
              node_off, up0, up1, down, pop, time, tvals, beta, u, kappa, pi, gbeta, nsweeps, rng, res, resd,
              pdg_out, probg_out, 0, 0};
  if (nthreads < 1) nthreads = 1;
  if (nthreads > nchains) nthreads = nchains;
  if (nthreads == 1) {
    ug_worker(&J);
    return J.err;
  }
  pthread_t *th = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
  if (!th) return 5;
  int started = 0;
  for (int i = 0; i < nthreads; i++)
    if (pthread_create(&th[i], NULL, ug_worker, &J) == 0) started++;
    else break;
  if (started == 0) ug_worker(&J);
  for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
  free(th);
  return J.err;
}
