/* ora_batch.c -- TEST INFRASTRUCTURE (the CPU checker and the timed CPU
 * baseline), never part of the product.
 *
 * Batched forms of the oracle's likelihood functions: many chain-loci over
 * packed arrays in one call, spread over host threads.  Each chain-locus is
 * evaluated by the single-item restatement (ora_is_likelihood,
 * ora_hky_likelihood, ora_sw_likelihood in ima_oracle.c, which follow
 * calc_prob_data.cpp:731-836, :118-607 and :841-909), so the results are the
 * same numbers; the batch only removes per-call marshalling from the
 * caller and lets every host core work, as the reference's own CPU path
 * runs one chain-locus at a time per process.
 *
 * Packed layout (item k):
 *   n[k] tips; nodes node_off[k] .. node_off[k] + 2n[k] - 2 of up0 / up1 /
 *   down / time (the reference's gtree[] fields, -1 for none);
 *   HKY: S[k] patterns, totsites[k], seq[seq_off[k] ..] int8 [n][S],
 *        mult[mult_off[k] ..] int32 [S], pi[4k .. 4k+3];
 *   SW:  alleles A[al_off[k] ..] int32 [2n-1];
 *   IS:  S[k] sites, seq as for HKY, length[k] (G->length), sumlogk[k].
 * Work is handed out 8 items at a time from a shared counter. */
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "ima_oracle.h"

typedef struct {
  int kind; /* 0 IS, 1 HKY, 2 SW */
  int nitems;
  const int *n;
  const long long *node_off;
  const int *up0, *up1, *down;
  const double *time;
  const int *S, *totsites;
  const long long *seq_off, *mult_off, *al_off;
  const int8_t *seq;
  const int *mult, *A;
  const double *pi, *u, *par, *length, *sumlogk;
  double *out;
  int *status;
  int next; /* shared work counter */
} batch_job;

static int root_of(int nl, const int *down)
{
  for (int i = 0; i < nl; i++)
    if (down[i] == -1) return i;
  return nl - 1;
}

static void *batch_worker(void *arg)
{
  batch_job *J = (batch_job *)arg;
  double *scr = NULL;
  size_t scr_cap = 0;
  int *site = NULL;
  size_t site_cap = 0;
  const int e_full[4] = {-1, -1, -1, -1};
  for (;;) {
    const int k0 = __atomic_fetch_add(&J->next, 8, __ATOMIC_RELAXED);
    if (k0 >= J->nitems) break;
    const int k1 = k0 + 8 < J->nitems ? k0 + 8 : J->nitems;
    for (int k = k0; k < k1; k++) {
      const int n = J->n[k], nl = 2 * n - 1;
      const long long o = J->node_off[k];
      const int *up0 = J->up0 + o, *up1 = J->up1 ? J->up1 + o : NULL, *down = J->down + o;
      const double *t = J->time + o;
      int st = 0;
      if (J->kind == 2) {
        J->out[k] = ora_sw_likelihood(n, J->A + J->al_off[k], down, up0, t, J->u[k], J->par[k], NULL);
      } else if (J->kind == 1) {
        const int S = J->S[k];
        const size_t need = (size_t)nl * S * 10; /* frac, newfrac (4 each), sf, oldsf */
        if (need > scr_cap) {
          free(scr);
          scr = (double *)malloc(need * sizeof(double));
          scr_cap = scr ? need : 0;
          if (!scr) { st = -1; J->out[k] = 0.0; goto done; }
        }
        double *frac = scr, *newfrac = scr + (size_t)nl * S * 4, *sf = newfrac + (size_t)nl * S * 4,
               *oldsf = sf + (size_t)nl * S;
        J->out[k] = ora_hky_likelihood(n, S, J->totsites[k], J->seq + J->seq_off[k], J->mult + J->mult_off[k],
                                       J->pi + 4 * (size_t)k, up0, up1, down, root_of(nl, down), t, J->u[k],
                                       J->par[k], e_full, frac, newfrac, sf, oldsf);
      } else {
        const int S = J->S[k];
        if ((size_t)(S > 0 ? S : 1) > site_cap) {
          free(site);
          site_cap = (size_t)(S > 0 ? S : 1);
          site = (int *)malloc(site_cap * sizeof(int));
          if (!site) { site_cap = 0; st = -1; J->out[k] = 0.0; goto done; }
        }
        J->out[k] = ora_is_likelihood(n, S, J->seq + J->seq_off[k], up0, up1, down, t, J->length[k], J->u[k],
                                      J->sumlogk[k], site, &st);
      }
    done:
      if (J->status) J->status[k] = st;
    }
  }
  free(scr);
  free(site);
  return NULL;
}

static int run_batch(batch_job *J, int nthreads)
{
  if (J->nitems <= 0) return 0;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 1024) nthreads = 1024;
  J->next = 0;
  pthread_t th[1024];
  int started = 0;
  for (int i = 1; i < nthreads; i++) {
    if (pthread_create(&th[started], NULL, batch_worker, J) != 0) break;
    started++;
  }
  batch_worker(J); /* the caller's thread works too */
  for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
  return started + 1;
}

int ora_sw_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *down,
                 const double *time, const long long *al_off, const int *A, const double *u, const double *tr,
                 int nthreads, double *out)
{
  batch_job J;
  memset(&J, 0, sizeof(J));
  J.kind = 2; J.nitems = nitems; J.n = n; J.node_off = node_off; J.up0 = up0; J.down = down; J.time = time;
  J.al_off = al_off; J.A = A; J.u = u; J.par = tr; J.out = out;
  return run_batch(&J, nthreads);
}

int ora_hky_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *up1,
                  const int *down, const double *time, const int *S, const int *totsites,
                  const long long *seq_off, const int8_t *seq, const long long *mult_off, const int *mult,
                  const double *pi, const double *u, const double *kappa, int nthreads, double *out)
{
  batch_job J;
  memset(&J, 0, sizeof(J));
  J.kind = 1; J.nitems = nitems; J.n = n; J.node_off = node_off; J.up0 = up0; J.up1 = up1; J.down = down;
  J.time = time; J.S = S; J.totsites = totsites; J.seq_off = seq_off; J.seq = seq; J.mult_off = mult_off;
  J.mult = mult; J.pi = pi; J.u = u; J.par = kappa; J.out = out;
  return run_batch(&J, nthreads);
}

int ora_is_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *up1,
                 const int *down, const double *time, const int *S, const long long *seq_off, const int8_t *seq,
                 const double *length, const double *u, const double *sumlogk, int nthreads, double *out,
                 int *status)
{
  batch_job J;
  memset(&J, 0, sizeof(J));
  J.kind = 0; J.nitems = nitems; J.n = n; J.node_off = node_off; J.up0 = up0; J.up1 = up1; J.down = down;
  J.time = time; J.S = S; J.seq_off = seq_off; J.seq = seq; J.length = length; J.u = u; J.sumlogk = sumlogk;
  J.out = out; J.status = status;
  return run_batch(&J, nthreads);
}

/* jointp's log density (the exact FP64 log-sum-exp of ora_jointp_exact,
 * jointfind.cpp:885-1047 without the reference's truncation) at many points,
 * spread over host threads. */
typedef struct {
  int G, rowlen, np, nm, npops, modeltype, npoints;
  const float *g;
  const double *lognorm, *x;
  double *q, *ess;
  int next;
} jointp_job;

static void *jointp_worker(void *arg)
{
  jointp_job *J = (jointp_job *)arg;
  const int npar = J->np + J->nm;
  for (;;) {
    const int k = __atomic_fetch_add(&J->next, 1, __ATOMIC_RELAXED);
    if (k >= J->npoints) break;
    double e = 0.0;
    J->q[k] = ora_jointp_exact(J->G, J->rowlen, J->g, J->np, J->nm, J->npops, J->modeltype, J->lognorm,
                               J->x + (size_t)k * npar, &e);
    if (J->ess) J->ess[k] = e;
  }
  return NULL;
}

int ora_jointp_batch(int G, int rowlen, const float *g, int np, int nm, int npops, int modeltype,
                     const double *lognorm, int npoints, const double *x, int nthreads, double *q, double *ess)
{
  jointp_job J;
  memset(&J, 0, sizeof(J));
  J.G = G; J.rowlen = rowlen; J.g = g; J.np = np; J.nm = nm; J.npops = npops; J.modeltype = modeltype;
  J.npoints = npoints; J.lognorm = lognorm; J.x = x; J.q = q; J.ess = ess;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > 1024) nthreads = 1024;
  pthread_t th[1024];
  int started = 0;
  for (int i = 1; i < nthreads; i++) {
    if (pthread_create(&th[started], NULL, jointp_worker, &J) != 0) break;
    started++;
  }
  jointp_worker(&J);
  for (int i = 0; i < started; i++) pthread_join(th[i], NULL);
  return started + 1;
}
