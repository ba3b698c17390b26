/*
 * ima_oracle.h -- CPU restatement of IMa2p's hot-path arithmetic.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the
 * GB300 kernels: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference legs may load it.  The product path
 * (ima2p_gb300/, libima2p_gb300.so) never calls it.
 *
 * Every function restates the reference algorithm cited beside it
 * (paths relative to the IMa2p source tree).  The restatement is pinned
 * against the compiled reference itself (oracle/_ref/imaref, built by
 * oracle/Makefile from the untouched sources) by tests/test_oracle_vs_ref.py
 * and by the committed fixtures under tests/golden/.
 *
 * Genealogy layout used throughout: numlines = 2n-1 nodes, tips 0..n-1,
 * internal nodes n..2n-2; up0/up1 = daughter ids (-1 at tips), down =
 * parent id (-1 at the root), time[c] = time at the lower end of edge c,
 * so the branch length of c is time[c] (tip) or time[c]-time[up0[c]].
 */
#ifndef IMA_ORACLE_H
#define IMA_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* ---- infinite sites (calc_prob_data.cpp:537-836) ---------------------- */
/* calc_sumlogk restated (calc_prob_data.cpp:609-719).  Returns 0 on success,
 * 1 when a site maps to two mutation nodes (the reference returns early and
 * leaves the constant at 0), 2 when a site maps to none (IM_err in the
 * reference).  counts[n-1] receives the per-internal-node mutation counts. */
int ora_is_sumlogk(int n, int S, const int8_t *seq, const int *up0,
                   const int *up1, const int *down, double *sumlogk,
                   int *counts);
/* likelihoodIS restated (calc_prob_data.cpp:731-836).  site_node[S] gets the
 * node whose daughters carry {0,1}.  *status: 0 ok, 1 = two mutation nodes
 * (return value REJECTINFINITESITESCONSTANT), 2 = incompatible site. */
double ora_is_likelihood(int n, int S, const int8_t *seq, const int *up0,
                         const int *up1, const int *down, const double *time,
                         double length, double u, double sumlogk,
                         int *site_node, int *status);

/* ---- HKY pruning (calc_prob_data.cpp:118-607, update_gtree_common.cpp:2140-2181) */
/* Buffers: frac/newfrac [numlines][S][4], sf/oldsf [numlines][S] (only
 * internal rows are used).  e[4] = dirty node ids, e[0] == -1 => full. */
double ora_hky_likelihood(int n, int S, int totsites, const int8_t *seq,
                          const int *mult, const double *pi, const int *up0,
                          const int *up1, const int *down, int root,
                          const double *time, double u, double kappa,
                          const int *e, double *frac, double *newfrac,
                          double *sf, double *oldsf);
void ora_hky_copyfraclike(int n, int S, const double *newfrac, double *frac);
void ora_hky_storescalefactors(int n, int S, const double *sf, double *oldsf);
void ora_hky_restorescalefactors(int n, int S, double *sf, const double *oldsf);
double ora_hky_standfactor(const double *pi, double kappa);

/* ---- stepwise microsatellites (calc_prob_data.cpp:841-909, utilities.cpp:54-124, 1449-1496) */
double ora_bessi0(double x);
double ora_bessi1(double x);
double ora_bessi(int n, double x);
/* Returns the locus log-likelihood; dlikeA[numlines] receives the per-branch
 * terms.  A[numlines] = allele states at the top of every edge. */
double ora_sw_likelihood(int n, const int *A, const int *down, const int *up0,
                         const double *time, double u, double tr,
                         double *dlikeA);
/* Rescore a list of branches with the per-branch term of likelihoodSW, as
 * finishSWupdateA does for its 3-4 changed edges
 * (update_gtree_common.cpp:2219-2362). */
double ora_sw_branch_term(int d, double t, double u);

/* ---- MT19937 (utilities.cpp:323-427) ----------------------------------- */
typedef struct { uint32_t mt[624]; int mti; } ora_mt;
void ora_mt_seed(ora_mt *s, uint32_t seed);
uint32_t ora_mt_u32(ora_mt *s);
double ora_mt_uniform(ora_mt *s);          /* genrand_real3: (k+0.5)/2^32 */
void ora_mt_fill_u32(uint32_t seed, int count, uint32_t *out);

/* ---- genealogy update, no-migration model (update_gtree.cpp:723-966) ---- */
/* a chain's generators: uniform()'s MT19937, normdev's cached deviate,
 * bitran's register (the layout of the library's ima_ug_rng) */
typedef struct { ora_mt mt; int32_t iset; double gset; uint64_t iseed; } ora_ug_rng;
void ora_ug_rng_seed(ora_ug_rng *g, int seed); /* setseeds (utilities.cpp:399-408) */
/* nsweeps updategenealogy sweeps (every locus in order) of each of nchains
 * chains, each from its own generator, chains spread over nthreads host
 * threads.  Genealogies of chain c, locus l at node_off[c*nloci+l] in up0 /
 * up1 / down / time / pop (updated in place); loci: model 0 IS (seq, S
 * sites, sumlogk), 1 HKY (seq patterns, mult, totsites; pi per
 * chain-locus) or 2 SW (one marker: arange[2l], arange[2l+1] its allele
 * range; the alleles of every node in `alleles`, updated in place).  The chain's state starts as finish_setup_C leaves it.  res
 * [nchains][nsweeps][nloci][3] (accepted, topology changed, tmrca changed)
 * and resd [...][2] (G.pdg, p(G) after the proposal) may be NULL; pdg_out
 * [nchains*nloci], probg_out [nchains].  Returns 0, or 1 a slide that did not
 * end, 2 a genealogy the model cannot hold, 3 an IS site no edge carries, 4
 * an integral term the reference rejects, 5 no memory. */
int ora_ug_run(int npops, const int *plist, const int *droppops, const int *addpop, const int *pop_e,
               const int *pop_down, int nth, const int *th_off, const int *th_idx, const double *th_max,
               const double *th_min, int nloci, const int *model, const int *n, const int *S, const int *totsites,
               const long long *seq_off, const long long *mult_off, const int8_t *seq, const int *mult,
               const double *hval, const int *samppop, const double *sumlogk, const int *arange, int nchains,
               const long long *node_off, int *up0, int *up1, int *down, double *time, int *pop, int *alleles,
               const double *tvals, const double *beta, double gbeta, const double *u, const double *kappa,
               const double *pi, int nsweeps, ora_ug_rng *rng, int nthreads, int *res, double *resd,
               double *pdg_out, double *probg_out);

/* ---- MC3 (swapchains.cpp:12-178, 526-662) ------------------------------ */
/* setheat for one process (numprocesses=1): heatmode 0 linear, 1 geometric,
 * 2 even (imamp.hpp heating enum order HLINEAR, HGEOMETRIC, HEVEN). */
int ora_setheat(int nchains, double h1, double h2, int heatmode, double *beta,
                double *allbetas);
/* Serial swapchains with swapbetasonly=1.  S[c] = sum_loci pdg + probg
 * (already reduced).  Uniforms come from u[] in order; *used returns how
 * many were consumed.  swapcount/tempcount are nchains x nchains row-major
 * and are incremented in place.  Returns swap0ok. */
int ora_swapchains(int nchains, int swaptries, const double *S, double *beta,
                   const double *allbetas, const double *u, int *used,
                   int *swapcount, int *tempcount, int *accepted_pairs);
/* S[c] = sum_li pdg[c*nloci+li] (in locus order) + probg[c] */
void ora_chain_sums(int nchains, int nloci, const double *pdg,
                    const double *probg, int include_probg, double *S);

/* ---- L-mode surface (jointfind.cpp:885-1047) ---------------------------- */
/* Column offsets of a gsampinf row (ginfo.cpp:288-316 / jointfind.cpp:914-926)
 * for numpopsizeparams = np, nummigrateparams = nm. */
void ora_gsamp_offsets(int np, int nm, int *ccp, int *fcp, int *hccp, int *mcp,
                       int *fmp, int *qip, int *mip, int *pdgp, int *probgp);
/* p_g for every genealogy at x.  modeltype 0 full (bias -probg), 1 theta
 * only (bias -sum qi), 2 migration only (bias -sum mi); lognorm (optional,
 * may be NULL) replaces the bias term with an FP64 per-genealogy value. */
void ora_surface_p(int G, int rowlen, const float *g, int np, int nm,
                   int npops, int modeltype, const double *lognorm,
                   const double *x, double *p);
/* Exact FP64 log-sum-exp form: q = log G - log sum_g exp(p_g) (+ESS). */
double ora_jointp_exact(int G, int rowlen, const float *g, int np, int nm,
                        int npops, int modeltype, const double *lognorm,
                        const double *x, double *ess);
/* The reference's truncated sum: linked list within PRANGELOG=10 of the
 * running max, descending traversal with its off-by-one, eexp mantissa /
 * decimal exponent accumulation. */
double ora_jointp_compat(int G, int rowlen, const float *g, int np, int nm,
                         int npops, int modeltype, const double *lognorm,
                         const double *x, double *ess);
void ora_eexp(double x, double *m, int *z);

/* margincalc (surface_call_functions.cpp:119-175): the marginal posterior
 * density of parameter pi (population sizes first, then migration rates) at
 * x, (1/G) sum_g exp(term_g), summed in genealogy order without a shift, then
 * log'd when logi (LOWLOG -1e200 for a sum <= 0), less yadjust.  expo_mean:
 * NULL, or the prior means of the migration parameters when their prior is
 * exponential (EXPOMIGRATIONPRIOR). */
double ora_margincalc(int G, int rowlen, const float *g, int np, int nm, int pi,
                      double x, double yadjust, int logi, const double *expo_mean);

/* L-mode peak search: modelloop (jointfind.cpp:746-812) with startpop
 * (:658-702), nextgen (:594-656), difeloop (:705-720) and copybest
 * (:723-738), for one model type, or a nested model given by xmap (nested > 0
 * parameters; mapvals :555-566, reversemapvals :540-552).  Lower bounds are
 * MINPARAMVAL, upper bounds the priors' maxima (setbounds :578-590).  The
 * objective is jointp on the given rows, compat (the reference's truncated
 * sum) or exact.  Uniforms come from *rng.  best[nparams+1] holds the peak's
 * parameters (mapped to the full model) and -log density; returns the number
 * of generations over all restarts, *restarts the number of DE runs; -1 for
 * a nested model of modeltype 2, whose bounds the reference indexes past the
 * mapped ones. */
int ora_modelloop(int G, int rowlen, const float *g, int np, int nm, int npops,
                  const double *lognorm, int compat, int modeltype,
                  const double *upper, int multiplier, const double *xmap,
                  int nested, ora_mt *rng, double *best, double *ess,
                  int *restarts);

/* ---- genealogy weights and p(G) (update_gtree_common.cpp:108-304,
 *      :1680-2134; ginfo.cpp:209-244, :318-377) ---------------------------
 * Weight layout for npops sampled populations (numsplittimes = npops-1):
 *   T = npops(npops+1)/2 entries for cc/hcc/fc: period k, position ii in the
 *       period's population list at  k*npops - k(k-1)/2 + ii;
 *   M = sum_{k<npops-1} (npops-k)^2 entries for mc/fm: period k, positions
 *       (ii, jj) at  moff(k) + ii*(npops-k) + jj.
 * Population model tables, as fillplist (build_poptree.cpp:391-450) leaves
 * them: plist[k*npops+ii], droppops[k*2+{0,1}], addpop[k] (k = 1..npops-1),
 * pop_e[p] / pop_down[p] for the 2npops-1 tree populations.  */
int ora_tw_sizes(int npops, int *T, int *M);
/* treeweight restated (update_gtree_common.cpp:1680-1937) for one genealogy
 * whose weights start at zero.  up0/time/pop per node (2ng-1), migration
 * events per node in CSR form (mig_off[2ng], times, destination pops).
 * out3 = {length, tlength}; *mignum.  Returns 0, or 1 for a genealogy the
 * model cannot hold (a coalescence or migration in a population that does
 * not exist in that period, or a count going negative). */
int ora_treeweight(int npops, const int *plist, const int *droppops, const int *addpop,
                   const int *pop_e, const int *pop_down, const double *tvals, int nomig,
                   int ng, const int *samppop, double hval, const int *up0,
                   const double *time, const int *pop, const int *mig_off,
                   const double *mig_t, const int *mig_p, int *cc, double *hcc,
                   double *fc, int *mc, double *fm, double *out3, int *mignum);
/* ora_treeweight over ngen genealogies in the CSR layout of
 * ima_gpu_treeweight (the CPU baseline of that call); returns the number
 * of genealogies the model could not hold. */
int ora_treeweight_batch(int npops, const int *plist, const int *droppops, const int *addpop,
                         const int *pop_e, const int *pop_down, int nomig, int ngen, const int *node_off,
                         const int *up0, const double *time, const int *pop, const int *mig_off,
                         const double *mig_t, const int *mig_p, const int *gen_locus, const int *gen_tv,
                         const double *hval, const int *samppop, const double *tvals, int *cc, double *hcc,
                         double *fc, int *mc, double *fm, double *lens, int *mignum);
/* The integral terms (update_gtree_common.cpp:108-304, MORESTABLE form) on
 * the reference's incomplete gamma functions (utilities.cpp:808-1130).
 * kind 0: integrate_coalescent_term(c, f, h, max, min); 1:
 * integrate_migration_term(c, f, max, min); 2:
 * integrate_migration_term_expo_prior(c, f, mean = max).  *status 0 ok,
 * else the reference would stop with IM_err (LogDiff order, iteration
 * limit, bad argument). */
double ora_iterm(int kind, int c, double f, double h, double max, double min, int *status);
/* initialize_integrate_tree_prob restated (:2089-2134) on weights already
 * summed over loci.  Theta parameter i sums the T entries th_idx[th_off[i] ..
 * th_off[i+1]) in order, migration parameter i the M entries mg_idx[...];
 * chk_idx: M entries that must hold no migration (nomigrationchecklist).
 * Returns 0, or the term's status. */
int ora_tree_prob(int nomig, int expo, const int *cc, const double *hcc, const double *fc,
                  const int *mc, const double *fm, int nth, const int *th_off,
                  const int *th_idx, const double *th_max, const double *th_min, int nmg,
                  const int *mg_off, const int *mg_idx, const double *mg_max,
                  const double *mg_min, const double *mg_mean, int nchk, const int *chk_idx,
                  double *probg, double *q, double *m);
/* savegsampinf restated (ginfo.cpp:318-377): one gsampinf row (float) from
 * summed weights, integrals, pdg and split times. */
void ora_gsamp_row(int nomig, const int *cc, const double *hcc, const double *fc,
                   const int *mc, const double *fm, int nth, const int *th_off,
                   const int *th_idx, int nmg, const int *mg_off, const int *mg_idx,
                   const double *q, const double *m, double pdg, double probg,
                   int nsplit, const double *tvals, float *row);
/* calc_popmig (popmig.cpp:9-91) and calc_pop_expomig (:96-172): the
 * posterior density (prob_or_like = 0) or likelihood (1) of 2N_i m_j at x
 * for theta parameter thetai and migration parameter mi over G gsampinf
 * rows; qmax / mmax the priors' maxima, mmean the exponential prior's mean.
 * *st is set where the reference would stop in an incomplete gamma term. */
double ora_popmig(int G, int rowlen, const float *g, int np, int nm, int thetai, int mi, double x,
                  double qmax, double mmax, int prob_or_like, int *st);
double ora_pop_expomig(int G, int rowlen, const float *g, int np, int nm, int thetai, int mi, double x,
                       double qmax, double mmean, int prob_or_like, int *st);
/* findmarginpeaks' numbers (surface_call_functions.cpp:316-734): mlval,
 * peakloc [3][np+nm] over the first half, the second half and all of the
 * genealogies (G clamped to 299,999), migtest [nm], lo95 / hi95 [np+nm]
 * (NaN where no peak), and for the nt 2NM terms (mpop, mterm) pm_mlval,
 * pm_peakloc [3][nt], pm_test [nt].  mgmean NULL: uniform migration
 * priors.  Returns -1 for 10 or fewer genealogies, else an incomplete-gamma
 * status (0 = fine). */
int ora_findmarginpeaks(int G, int rowlen, const float *g, int np, int nm, const double *thmin,
                        const double *thmax, const double *mgmin, const double *mgmax, const double *mgmean,
                        int nt, const int *mpop, const int *mterm, double *mlval, double *peakloc,
                        double *migtest, double *lo95, double *hi95, double *pm_mlval, double *pm_peakloc,
                        double *pm_test);
/* .ti loading the reference's way (fgets per genealogy, sscanf("%f") per
 * value; ima_main_mpi.cpp:3370-3400), every genealogy kept, at most cap. */
int ora_ti_load(const char *path, int rowlen, float *rows, int cap);

/* Batched likelihoods over packed arrays on nthreads host threads
 * (ora_batch.c); return the threads used. */
int ora_sw_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *down,
                 const double *time, const long long *al_off, const int *A, const double *u, const double *tr,
                 int nthreads, double *out);
int ora_hky_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *up1,
                  const int *down, const double *time, const int *S, const int *totsites,
                  const long long *seq_off, const int8_t *seq, const long long *mult_off, const int *mult,
                  const double *pi, const double *u, const double *kappa, int nthreads, double *out);
int ora_is_batch(int nitems, const int *n, const long long *node_off, const int *up0, const int *up1,
                 const int *down, const double *time, const int *S, const long long *seq_off, const int8_t *seq,
                 const double *length, const double *u, const double *sumlogk, int nthreads, double *out,
                 int *status);
int ora_jointp_batch(int G, int rowlen, const float *g, int np, int nm, int npops, int modeltype,
                     const double *lognorm, int npoints, const double *x, int nthreads, double *q, double *ess);

#ifdef __cplusplus
}
#endif
#endif
