/*
 * ima_gpu.h -- C ABI of the GB300 implementation of IMa2p's data-parallel
 * hot paths: the per-locus data likelihoods (infinite sites, HKY pruning,
 * stepwise microsatellites), the MC3 temperature swaps and the L-mode
 * joint-posterior surface.
 *
 * Conventions
 *  - Plain C types only; every function returns an IMA_* status (never exits).
 *    ima_gpu_error() returns the text of the last failure on a context.
 *  - Host buffers are caller-owned; genealogies, partial likelihoods and chain
 *    state are device-resident and owned by the context.
 *  - One context = one CUDA stream on one device; call it from one host
 *    thread at a time.
 *  - Chains are numbered 0..nruns*chains_per_run-1 (run r owns chains
 *    r*chains_per_run ..); loci 0..nloci-1 in the order they were added.
 *    A (chain, locus) pair is a "chain-locus".
 *  - Genealogy layout is the reference's struct edge (imamp.hpp:651-679):
 *    numlines = 2n-1 nodes, tips 0..n-1, up0/up1 daughters (-1 at tips),
 *    down parent (-1 at the root), time[c] = time at the lower end of edge c.
 *
 * Each entry point names the reference interface it replaces
 * (paths relative to the IMa2p source tree, src/).
 */
#ifndef IMA_GPU_H
#define IMA_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ima_ctx ima_ctx;

/* status codes */
#define IMA_OK 0
#define IMA_ERR_ARG (-1)           /* bad argument (index, size, pointer)          */
#define IMA_ERR_CUDA (-2)          /* a CUDA call failed                          */
#define IMA_ERR_STATE (-3)         /* call out of order (e.g. no chains yet)       */
#define IMA_ERR_NOMEM (-4)         /* device or host allocation failed            */
#define IMA_ERR_DATA (-5)          /* data incompatible with a genealogy: the
                                      reference's IM_err(IMERR_INFINITESITESFAIL) */
#define IMA_ERR_TIMEOUT (-6)       /* a bounded device wait ran out               */

/* mutation models, in the reference's enum order (imamp.hpp mutation models) */
#define IMA_MODEL_IS 0
#define IMA_MODEL_HKY 1
#define IMA_MODEL_SW 2

/* arithmetic of an evaluation */
#define IMA_PREC_FAST 0            /* float-float pruning and Bessel, FP64 sums   */
#define IMA_PREC_FP64 1            /* plain FP64 per chain-locus                  */
#define IMA_PREC_FP32 2            /* HKY: plain FP32 pruning (log L off by ~1e-4
                                      on a 1000-bp locus); IS, SW as IMA_PREC_FAST */

/* per chain-locus evaluation status */
#define IMA_EVAL_OK 0
#define IMA_EVAL_IS_REJECT 1       /* two mutation nodes: REJECTINFINITESITESCONSTANT */
#define IMA_EVAL_IS_FAIL 2         /* no mutation node: data incompatible         */
#define IMA_EVAL_SW_ZERO 3         /* a Bessel term was 0: result is -DBL_MAX     */

/* ------------------------------------------------------------------ context */
int ima_gpu_create(int device, ima_ctx **out);
void ima_gpu_destroy(ima_ctx *ctx);
const char *ima_gpu_error(const ima_ctx *ctx);
int ima_gpu_synchronize(ima_ctx *ctx);

/* ------------------------------------------------------------------- loci
 * Locus tables shared by every chain; replace the L[li] arrays built by
 * readseqIS / readseqHKY / readseqSW (readata.cpp:347-495, :247-345, :499-588).
 * seq is [numgenes][numsites] row-major: 0/1 for IS (coded against the first
 * sequence), 0..3 = A,C,G,T site patterns for HKY with their multiplicities. */
int ima_gpu_add_locus_is(ima_ctx *ctx, int numgenes, int numsites, const int8_t *seq, int *li);
int ima_gpu_add_locus_hky(ima_ctx *ctx, int numgenes, int numsites, int totsites,
                          const int8_t *seq, const int32_t *mult, int *li);
/* nlinked = number of linked stepwise markers (allele arrays per node). */
int ima_gpu_add_locus_sw(ima_ctx *ctx, int numgenes, int nlinked, int *li);

/* Allocate the resident state of nruns * chains_per_run chains over every
 * locus added so far (replaces the per-chain allocations of setup,
 * initialize.cpp:2074).  Loci cannot be added afterwards. */
int ima_gpu_set_chains(ima_ctx *ctx, int nruns, int chains_per_run);

/* -------------------------------------------------------------- genealogy
 * Upload one genealogy (replaces writes to C[ci]->G[li].gtree).  length is the
 * genealogy length from treeweight (update_gtree_common.cpp:1822-1840), used
 * by the infinite-sites likelihood; pass a negative value to use the sum of
 * branch lengths.  Edits are staged on the host and shipped to the device,
 * as one copy per changed range, before the next evaluation. */
int ima_gpu_set_genealogy(ima_ctx *ctx, int ci, int li, const int32_t *up0, const int32_t *up1,
                          const int32_t *down, const double *time, double length);
/* Many genealogies in one call: arrays of pair k start at offset
 * sum_{j<k} numlines_j of the packed up0/up1/down/time arrays; length may be
 * NULL (sum of branch lengths). */
int ima_gpu_set_genealogies(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li,
                            const int32_t *up0, const int32_t *up1, const int32_t *down,
                            const double *time, const double *length);
/* New node times for genealogies whose topology is unchanged (the moves of
 * changet_RY1, update_t_RY.cpp:279-335, and other re-timings): time is
 * packed per pair as in ima_gpu_set_genealogies, length (may be NULL: the
 * sum of branch lengths) per pair.  Each pair must already hold a genealogy
 * (IMA_ERR_STATE).  Only the FP64 times travel: the device makes the
 * float-float copy.  Pairs that are consecutive chain-loci in order (chain
 * major, locus minor, as a batch of whole chains lists them) go to the
 * device in one copy straight from the caller's buffers, with the lengths
 * summed there; other lists are staged and copied with the next
 * evaluation.  The buffers may be reused when the call returns. */
int ima_gpu_set_times(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li, const double *time,
                      const double *length);
/* ima_gpu_set_times for every pair, then ima_gpu_eval of the same pairs
 * (full evaluations): a re-timing move of many chains (changet_RY1,
 * update_t_RY.cpp:223-389, whose loop over loci calls the likelihood of each
 * re-timed genealogy) in one call.  Where the device can read the caller's
 * memory (cudaDevAttrPageableMemoryAccess), a contiguous run of pairs is
 * read in place by the first kernel of the evaluation's stream.  The
 * buffers may be reused when the call returns. */
int ima_gpu_eval_times(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li, const double *time,
                       const double *length, const double *u, const double *kappa, const int32_t *ai,
                       int precision, double *result, int32_t *status);
/* Base frequencies of an HKY chain-locus (C[ci]->G[li].pi). */
int ima_gpu_set_pi(ima_ctx *ctx, int ci, int li, const double *pi4);
/* Allele states of linked marker ai on every node (gtree[i].A[ai]). */
int ima_gpu_set_alleles(ima_ctx *ctx, int ci, int li, int ai, const int32_t *A);
/* The resident allele states of marker ai on every node (after device
 * updates, e.g. ima_gpu_updategenealogy_sweep's allele proposals). */
int ima_gpu_get_alleles(ima_ctx *ctx, int ci, int li, int ai, int32_t *A);
/* Edit list of single allele states: gtree[node[k]].A[ai[k]] = A[k] on chain
 * ci[k], locus li[k], for k < n -- the state finishSWupdateA
 * (update_gtree_common.cpp:2219-2362) proposes for the moved node.  The
 * proposal itself (geometric step, bitran sign, Hastings term Aterm) stays on
 * the host; the likelihood change likeadj - oldlikeadj is the difference of
 * the batched SW evaluations after and before the edits.  The whole list is
 * validated first; nothing is applied when any entry is invalid. */
int ima_gpu_set_allele_edits(ima_ctx *ctx, int n, const int *ci, const int *li, const int *ai,
                             const int *node, const int32_t *A);

/* --------------------------------------------- per-call reference mirrors
 * Same names, argument meaning, return values and side effects as the
 * reference functions, evaluated on the GPU from the resident state. */
/* likelihoodIS (calc_prob_data.cpp:731-836): the per-locus constant sum log k!
 * is taken from the first genealogy evaluated for the locus, as the reference's
 * static sumlogk cache does (:760-765). */
int ima_gpu_likelihoodIS(ima_ctx *ctx, int ci, int li, double mutrate, double *result);
/* likelihoodHKY (calc_prob_data.cpp:583-607): e1..e4 are the dirty nodes
 * (e1 == -1 recomputes every node). */
int ima_gpu_likelihoodHKY(ima_ctx *ctx, int ci, int li, double mutrate, double kappa,
                          int e1, int e2, int e3, int e4, double *result);
/* copyfraclike / storescalefactors / restorescalefactors
 * (update_gtree_common.cpp:2140-2181): accept or reject the partial
 * likelihoods of the last HKY evaluation of (ci, li). */
int ima_gpu_copyfraclike(ima_ctx *ctx, int ci, int li);
int ima_gpu_storescalefactors(ima_ctx *ctx, int ci, int li);
int ima_gpu_restorescalefactors(ima_ctx *ctx, int ci, int li);
/* likelihoodSW (calc_prob_data.cpp:841-909): also refreshes the resident
 * per-branch terms dlikeA of marker ai. */
int ima_gpu_likelihoodSW(ima_ctx *ctx, int ci, int li, int ai, double u, double tr, double *result);
/* Per-branch dlikeA terms of marker ai (gtree[i].dlikeA[ai]) after the last
 * SW evaluation; dlikeA has numlines entries. */
int ima_gpu_get_dlikeA(ima_ctx *ctx, int ci, int li, int ai, double *dlikeA);

/* ------------------------------------------------------ batched likelihoods
 * One launch over many chain-locus pairs of mixed models (the batched form
 * of the calls above, as changet_RY1 / updategenealogy make them,
 * update_t_RY.cpp:343-389, update_gtree.cpp:838-888).
 *   ci, li     : chain-locus pairs (may repeat loci and mix models)
 *   u          : mutation rate scalar per pair
 *   kappa      : HKY kappa per pair; for SW pairs the branch-time scale tr
 *                of likelihoodSW (ignored for IS; NULL = 1.0)
 *   edits      : 4 dirty node ids per pair for HKY (NULL = full recompute)
 *   ai         : SW marker per pair (NULL = 0)
 *   precision  : IMA_PREC_FAST, IMA_PREC_FP64 or IMA_PREC_FP32.  HKY partials
 *                of IMA_PREC_FAST and IMA_PREC_FP32 share their slots: a
 *                node last computed in FP32 enters a later float-float
 *                evaluation of its ancestors with FP32 accuracy (e1 = -1
 *                recomputes every node)
 *   result     : log P(D|G) per pair (host)
 *   status     : IMA_EVAL_* per pair (host, may be NULL)
 * Staged requests can be replayed without host copies through the batch
 * handle functions below. */
int ima_gpu_eval(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li, const double *u,
                 const double *kappa, const int32_t *edits, const int32_t *ai, int precision,
                 double *result, int32_t *status);
/* accept[k] != 0 commits pair k (copyfraclike + storescalefactors and
 * G.pdg = result), else reverts it (restorescalefactors). */
int ima_gpu_commit(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li,
                   const uint8_t *accept);

/* Batches: stage requests once, run them from device memory (optionally as a
 * CUDA graph replay), read the results when needed. */
int ima_gpu_batch_create(ima_ctx *ctx, int npairs, const int32_t *ci, const int32_t *li,
                         const double *u, const double *kappa, const int32_t *edits,
                         const int32_t *ai, int precision, int *batch);
int ima_gpu_batch_run(ima_ctx *ctx, int batch, int use_graph);
/* Launch-shape autotuner for a batch's FP32 kernels: times each variant on
 * the batch's own requests (reps timed runs after one untimed) and keeps the
 * fastest -- HKY: 128 threads per chain-locus (0, the default), 64 (1), 256
 * (2), 128 without the shared-memory partial cache (3), 128 with registers
 * for 8 resident CTAs per SM instead of 12 (4); SW: 8 chain-loci per CTA
 * (0), 4 (1), 16 (2).  The default stays unless another variant is more
 * than 2% faster.  Every variant gives the same likelihoods up to the order
 * of the final FP64 reduction.  Out (may be NULL): the chosen variants. */
int ima_gpu_batch_autotune(ima_ctx *ctx, int batch, int reps, int *hky_variant, int *sw_variant);
/* Pins a batch's launch variants (numbering as above). */
int ima_gpu_batch_set_variants(ima_ctx *ctx, int batch, int hky_variant, int sw_variant);
int ima_gpu_batch_results(ima_ctx *ctx, int batch, double *result, int32_t *status);
/* One MC3 sweep of a batch (the loop body of ima_main_mpi.cpp:1821-1981 for
 * the batch's chain-loci): every request evaluated, the accepted ones
 * committed as copyfraclike does (accept [npairs] in the batch's caller
 * order, or NULL: all), then swapchains (swapchains.cpp:526) of every run
 * with swaptries attempts on the committed sums, drawing the device's
 * per-run Philox stream keyed by seed.  With use_graph every kernel of the
 * sweep is one CUDA graph launch, captured on the first call and replayed
 * while swaptries, include_probg and seed stay the same. */
int ima_gpu_batch_sweep(ima_ctx *ctx, int batch, const uint8_t *accept, int swaptries, int include_probg,
                        uint64_t seed, int use_graph);
int ima_gpu_batch_destroy(ima_ctx *ctx, int batch);
/* Copy every staged genealogy edit to the device now (normally implicit). */
int ima_gpu_flush_genealogies(ima_ctx *ctx);

/* -------------------------------------------------------------- MC3 swaps */
/* setheat (swapchains.cpp:71-178) for every run (numprocesses = 1 within a
 * run); heatmode 0 linear, 1 geometric, 2 even. */
int ima_gpu_setheat(ima_ctx *ctx, double hval1, double hval2, int heatmode);
int ima_gpu_get_betas(ima_ctx *ctx, double *beta);        /* nchains values */
int ima_gpu_set_betas(ima_ctx *ctx, const double *beta);
/* The heat ladder the swap counts index (allbetas, imamp.hpp:1081), nchains
 * values, for a caller that ran setheat itself. */
int ima_gpu_set_allbetas(ima_ctx *ctx, const double *allbetas);
/* G.pdg of every chain-locus ([nchains][nloci]) and allpcalc.probg per chain. */
int ima_gpu_set_pdg(ima_ctx *ctx, const double *pdg);
int ima_gpu_get_pdg(ima_ctx *ctx, double *pdg);
int ima_gpu_set_probg(ima_ctx *ctx, const double *probg);
int ima_gpu_get_probg(ima_ctx *ctx, double *probg);
/* swapchains (swapchains.cpp:526-653) with swapbetasonly = 1 in every run.
 * Uniform source: if uniforms != NULL, run r consumes uniforms[r*stride ...]
 * in the reference's order (ci, cj rejection loop, then U only when w < 1)
 * and used[r] returns how many it consumed; else a per-run Philox stream
 * keyed by seed is used.  include_probg = 0 reproduces -c4.
 * swap0ok[r] (may be NULL) as the reference returns it. */
int ima_gpu_swapchains(ima_ctx *ctx, int swaptries, int include_probg, const double *uniforms,
                       int stride, uint64_t seed, int32_t *used, int32_t *swap0ok);
/* The same attempts for a caller whose generator must be drawn one value at
 * a time, as the reference's uniform() is (utilities.cpp:323-427): the
 * per-chain sums come from the device, the attempts call uniform(arg)
 * exactly where swapchains (swapchains.cpp:549-605) calls uniform() -- ci,
 * the cj rejection loop, then U only when w < 1 -- and update the resident
 * betas and both count matrices.  used[r] (may be NULL): the draws run r
 * made.  Replaces swapchains() in the reference-side binding. */
int ima_gpu_swapchains_cb(ima_ctx *ctx, int swaptries, int include_probg, double (*uniform)(void *arg),
                          void *arg, int32_t *used, int32_t *swap0ok);
/* How many points the last IMA_SURF_TC evaluation took a second time: its
 * sums are fixed-point numbers relative to a first bound on each point's
 * maximum, and points with a term more than 55 nats above that bound are
 * evaluated again relative to their exact maximum (same results, more
 * time). */
int ima_gpu_surface_retaken(ima_ctx *ctx, int *n);
/* swapcount and tempbasedswapcount (imamp.hpp:1123-1129) of run r,
 * chains_per_run^2 each, row-major. */
int ima_gpu_get_swapcounts(ima_ctx *ctx, int run, int32_t *swapcount, int32_t *tempcount);

/* --------------------------------------------------------- L-mode surface
 * Load G saved genealogies (gsampinf rows, ginfo.cpp:288-316) for jointp.
 * lognorm (may be NULL) replaces the per-genealogy bias -probg (or -sum qi,
 * -sum mi) with an FP64 value. */
int ima_gpu_surface_load(ima_ctx *ctx, int G, int rowlen, const float *gsampinf,
                         int numpopsizeparams, int nummigrateparams, int npops,
                         const double *lognorm);
/* methods */
#define IMA_SURF_FAST 0     /* split-precision contraction + online log-sum-exp */
#define IMA_SURF_FP64 1     /* FP64 CUDA-core form, exact log-sum-exp           */
#define IMA_SURF_COMPAT 2   /* the reference's truncated sum (PRANGELOG, eexp)   */
#define IMA_SURF_TC 3       /* IMA_SURF_FAST with its screen on the tensor cores  */
/* q = log G - log sum_g exp(p_g(x)) at npoints points x[npoints][nparams];
 * modeltype 0 full, 1 population sizes only, 2 migration only (jointp's
 * nowmodeltype).  ess (may be NULL) = effective number of genealogies.
 * IMA_SURF_TC is the fastest exact method (G < 2^24); IMA_SURF_FAST gives
 * the same sum with its screen on CUDA cores.  Both keep the operands derived
 * from the rows between calls while the rows and modeltype are unchanged. */
int ima_gpu_surface_eval(ima_ctx *ctx, int npoints, const double *x, int modeltype, int method,
                         double *q, double *ess);
/* Checks the tensor-core path on this device: one 128 x 256 x 32 bf16 tile of
 * small integers through TMA, tcgen05.mma and tcgen05.ld, compared element by
 * element with CUDA cores.  *mismatches = 0 when every element matches. */
int ima_gpu_tc_selftest(ima_ctx *ctx, int *mismatches, float *max_abs_err);

/* jointp (jointfind.cpp:885-1047) at one point, reference semantics. */
int ima_gpu_jointp(ima_ctx *ctx, const double *x, int calc_ess, double *effective_n, double *q);
/* margincalc (surface_call_functions.cpp:119-175) at n points over the
 * loaded genealogies: out[k] = (logi ? log s (LOWLOG -1e200 when s <= 0) : s)
 * - yadjust, where s = (1/G) sum_g exp(term_g) is the marginal posterior
 * density of parameter param[k] (population sizes first, then migration
 * rates) at x[k] > 0, summed in FP64 without a shift as the reference sums
 * it.  expo_mean: NULL, or the prior mean of every migration parameter when
 * the migration prior is exponential (EXPOMIGRATIONPRIOR).  The peak and 95%
 * searches (marginalopt, margin95) call it from the host. */
int ima_gpu_margincalc(ima_ctx *ctx, int n, const int32_t *param, const double *x, double yadjust, int logi,
                       const double *expo_mean, double *out);
/* fillvec (histograms.cpp:82-99): every parameter's marginal density on its
 * grid x_j = pmin + (j + 0.5)(pmax - pmin) / gridsize (initialize.cpp:189-194,
 * :236-241; GRIDSIZE is 1000).  x_out (may be NULL) and y_out are
 * [np+nm][gridsize]; migration rates whose prior maximum is at most
 * MPRIORMIN (1e-6) are skipped, as fillvec skips them, with y = 0. */
int ima_gpu_fillvec(ima_ctx *ctx, int gridsize, const double *pmin, const double *pmax,
                    const double *expo_mean, double *x_out, double *y_out);
/* calc_popmig (popmig.cpp:9-91), or calc_pop_expomig (:96-172) when
 * mig_mean != NULL (EXPOMIGRATIONPRIOR): the posterior density of the
 * population migration rate 2N_i m_j of the term (thetai[k], mi[k]) at
 * x[k] > 0, over the loaded genealogies; prob_or_like = 1 divides it by the
 * prior density of 2NM (the likelihood curve).  theta_max [np] and mig_max
 * [nm] are the priors' maxima (itheta[].pr.max, imig[].pr.max), mig_mean
 * [nm] the exponential priors' means.  The terms follow the reference's
 * branches and operation order, including its quirks (counts truncated, a
 * genealogy whose two gamma terms do not separate adds exp(0)); the sum over
 * genealogies is in FP64, chunked, so it agrees with the reference's to
 * rounding.  IMA_ERR_DATA where the reference's series or fraction would
 * not converge. */
int ima_gpu_popmig(ima_ctx *ctx, int n, const int32_t *thetai, const int32_t *mi, const double *x,
                   const double *theta_max, const double *mig_max, const double *mig_mean, int prob_or_like,
                   double *y);
/* The 2NM curves print_populationmigrationrate_histograms computes for the
 * default parameterisation (histograms.cpp:755-805): for each term t, the
 * grid (j + 0.5) pmmax / gridsize (pmmax = theta_max * mig_max / 2, or
 * EXPOMIGPLOTSCALE (20) * mig_mean under the exponential prior) is scanned
 * from the top for the first density above 1e-9, which sets maxx[t] (pmmax
 * when there is none); then x_out[t][j] = (j + 0.5) maxx[t] / gridsize and
 * y_out[t][j] the density there (GRIDSIZE is 1000).  Each pass is one launch
 * over every term.  maxx may be NULL.  The caller picks the terms (thetai
 * below numtreepops - 1, each migration parameter whose first population is
 * thetai), as the reference does from the parameter names. */
int ima_gpu_popmig_curves(ima_ctx *ctx, int nterms, const int32_t *thetai, const int32_t *mi, int gridsize,
                          const double *theta_max, const double *mig_max, const double *mig_mean,
                          int prob_or_like, double *x_out, double *y_out, double *maxx);
/* The numbers of findmarginpeaks (surface_call_functions.cpp:316-734) over
 * the loaded genealogies, G clamped to MAXGENEALOGIESTOSAVE - 1 as there:
 *   mlval, peakloc [3][np+nm]: marginalopt (:178-266) of every parameter
 *     over the first half of the genealogies, the second (starting one past
 *     the first's end, as the reference steps), and all of them; the peak
 *     of marginp's density (:25-80: cc as stored, the genealogy range's
 *     length + 1 when it starts at 0) by two mnbrakmod brackets and
 *     goldenmod (surface_search_functions.cpp:42-200); peakloc -1 (mlval
 *     NaN) where the brackets do not overlap;
 *   migtest [nm]: 2 log(density at the peak / density at MINPARAMVAL);
 *   lo95, hi95 [np+nm]: margin95 (:268-292), bisection (marginbis, 40
 *     steps, tolerance 1e-4) of margincalc's log density 1.92 below the
 *     peak; DBL_MIN where no crossing, DBL_MAX where the bisection did not
 *     end; NaN for parameters without a peak;
 *   pm_mlval, pm_peakloc [3][nterms], pm_test [nterms]: the same for the
 *     2NM terms (mpop[t], mterm[t]) -- marginalopt_popmig (popmig.cpp:361-428,
 *     a 100-point scan then goldenmod on marginpopmig / marginpop_expomig)
 *     and its test; nterms = 0 skips them (POPMIGPARAMHIST off);
 *   holdpeakloc [np+nm]: the all-genealogy peaks (MINPARAMVAL where none),
 *     -1 everywhere when 10 or fewer genealogies are loaded.
 * theta_min/max, mig_min/max: the priors (itheta[].pr, imig[].pr);
 * mig_mean: NULL, or the exponential priors' means (EXPOMIGRATIONPRIOR).
 * Every search follows the reference's sequence of points given its values;
 * the searches of all parameters, terms and genealogy ranges advance
 * together, each round's points evaluated in one batched launch per kind
 * of density and range.  *rounds (may be NULL): the number of rounds. */
int ima_gpu_findmarginpeaks(ima_ctx *ctx, const double *theta_min, const double *theta_max,
                            const double *mig_min, const double *mig_max, const double *mig_mean,
                            int nterms, const int32_t *mpop, const int32_t *mterm, double *mlval,
                            double *peakloc, double *migtest, double *lo95, double *hi95, double *pm_mlval,
                            double *pm_peakloc, double *pm_test, float *holdpeakloc, int *rounds);
/* The loaded surface's shape (any pointer may be NULL). */
int ima_gpu_surface_info(ima_ctx *ctx, int *G, int *numpopsizeparams, int *nummigrateparams, int *npops);

/* ------------------------------- genealogy weights and p(G) integrals
 * The population model: the tables fillplist leaves in the reference's
 * chain (build_poptree.cpp:391-450) and the parameter maps of setup_iparams
 * (initialize.cpp:202-727).  npops in 2..10 sampled populations;
 * numtreepops = 2npops-1; numsplittimes = npops-1.
 *   plist[k*npops + ii]   population ii of period k (ids ascending; npops-k used)
 *   droppops[2k + {0,1}], addpop[k]   the k-th split (k = 1..npops-1; row 0 unused)
 *   pop_e[p], pop_down[p]   the period at which population p ends (-1 root), its ancestor
 * Weight cells, for every genealogy and chain: T = npops(npops+1)/2
 * coalescent cells (cc/hcc/fc of period k, position ii at
 * k*npops - k(k-1)/2 + ii) and M = sum_{k<npops-1} (npops-k)^2 migration
 * cells (mc/fm of period k, positions (ii, jj) at moff(k) + ii(npops-k) + jj,
 * moff(k) = sum_{j<k} (npops-j)^2).  Theta parameter i sums the T cells
 * th_idx[th_off[i] .. th_off[i+1]) in that order (itheta[i].wp); migration
 * parameter i the M cells mg_idx[...] (imig[i].wp); their priors are
 * th_max/th_min (itheta[i].pr) and mg_max/mg_min/mg_mean (imig[i].pr).
 * chk_idx: M cells that must hold no migration (nomigrationchecklist).
 * nomig, expo: modeloptions[NOMIGRATION], modeloptions[EXPOMIGRATIONPRIOR]. */
int ima_gpu_set_popmodel(ima_ctx *ctx, int npops, int nomig, int expo, const int32_t *plist,
                         const int32_t *droppops, const int32_t *addpop, const int32_t *pop_e,
                         const int32_t *pop_down, int nth, const int32_t *th_off, const int32_t *th_idx,
                         const double *th_max, const double *th_min, int nmg, const int32_t *mg_off,
                         const int32_t *mg_idx, const double *mg_max, const double *mg_min,
                         const double *mg_mean, int nchk, const int32_t *chk_idx);
/* treeweight (update_gtree_common.cpp:1680-1937) for ngen genealogies at
 * once, each from zero weights (the reference zeroes G->gweight first).
 * Genealogy g holds nodes node_off[g] .. node_off[g+1] (2n-1 of them, local
 * ids as in struct edge); per node: up0, time (as everywhere in this ABI) and
 * pop = gtree[i].pop; its migration events, oldest last, are mig_t/mig_p
 * [mig_off[node] .. mig_off[node+1]) over the global node index
 * (gtree[i].mig[].mt/.mp).  gen_locus[g] picks the locus row of hval
 * (L[li].hval) and samppop[npops] (L[li].samppop); gen_tv[g] the row of
 * tvals[ntv][npops-1] (C[ci]->tvals).  Outputs (each may be NULL):
 * cc/hcc/fc [ngen][T], mc/fm [ngen][M], lens [ngen][2] = {G->length,
 * G->tlength}, mignum [ngen] = G->mignum.  The weights stay on the device
 * for ima_gpu_tree_prob.  IMA_ERR_DATA: a genealogy the model cannot hold
 * (the reference asserts): a population outside its period, a count below
 * zero.  Weights equal the reference's bit for bit. */
int ima_gpu_treeweight(ima_ctx *ctx, int ngen, const int32_t *node_off, const int32_t *up0,
                       const double *time, const int32_t *pop, const int32_t *mig_off,
                       const double *mig_t, const int32_t *mig_p, const int32_t *gen_locus,
                       const int32_t *gen_tv, int nloci, const double *hval, const int32_t *samppop,
                       int ntv, const double *tvals, int32_t *cc, double *hcc, double *fc, int32_t *mc,
                       double *fm, double *lens, int32_t *mignum);
/* sum_treeinfo (ginfo.cpp:209-244) of each chain's genealogies from the
 * last ima_gpu_treeweight (group i = genealogies group_off[i] ..
 * group_off[i+1], summed in that order, i.e. locus order) followed by
 * initialize_integrate_tree_prob (update_gtree_common.cpp:2089-2134):
 * probg[ngroups] (C[ci]->allpcalc.probg), q [ngroups][nth] (qintegrate),
 * m [ngroups][nmg] (mintegrate).  rows (may be NULL): the gsampinf row
 * savegsampinf (ginfo.cpp:318-377) writes, [ngroups][4nth + 3nmg + 2 +
 * npops-1] floats, with pdg[i] (may be NULL: 0) and the split times of
 * tvals row group_tv[i] (may be NULL: row 0).  IMA_ERR_DATA where the
 * reference stops in an integral term (LogDiff order, iteration limit). */
int ima_gpu_tree_prob(ima_ctx *ctx, int ngroups, const int32_t *group_off, const double *pdg,
                      const int32_t *group_tv, double *probg, double *q, double *m, float *rows);
/* The M-mode sampling step on the device: append the gsampinf rows of the
 * chains groups[0..n) from the last ima_gpu_tree_prob (its rows are kept on
 * the device whether or not they were copied out) to the resident surface,
 * as savegsampinf appends the cold chain's row to gsampinf
 * (savegenealogyinfo, ima_main_mpi.cpp:3096-3117).  The first append on a context without
 * surface rows starts one with this model's shape (numpopsizeparams = nth,
 * nummigrateparams = nmg); later appends must match it.  The surface
 * functions (ima_gpu_surface_eval, ima_gpu_modelloop, ima_gpu_fillvec, ...)
 * then see every appended row.  IMA_ERR_STATE: the resident surface has
 * another shape or per-genealogy normalisers. */
int ima_gpu_surface_append_tree_rows(ima_ctx *ctx, int n, const int32_t *groups);
/* ------------------------- resident labels and the split-time update
 * For device-resident chains: the population labels and migration events of
 * every chain-locus stay on the device with its genealogy, and the
 * split-time update changet_RY1 (update_t_RY.cpp:223-518) moves their times
 * there.  The host keeps the generator draws and the Metropolis-Hastings
 * decision.  Host genealogy uploads (ima_gpu_set_genealogy(ies), set_pi,
 * set_alleles) after device moves first copy the device's times back, so
 * the two never overwrite each other.
 *
 * L[li].hval and L[li].samppop[npops] of every locus (after
 * ima_gpu_set_popmodel and ima_gpu_set_chains). */
int ima_gpu_set_locus_pops(ima_ctx *ctx, const double *hval, const int32_t *samppop);
/* gtree[].pop and gtree[].mig[] of the chain-loci (ci[k], li[k]); packed per
 * pair: pop[2n-1], mig_off[2n] (the pair's events, node by node, from 0),
 * mig_t/mig_p (times, destination populations). */
int ima_gpu_set_labels(ima_ctx *ctx, int n, const int32_t *ci, const int32_t *li, const int32_t *pop,
                       const int32_t *mig_off, const double *mig_t, const int32_t *mig_p);
/* The device's node times [2n-1] and (mig_t may be NULL) migration times of
 * a chain-locus; *nmig = its number of events. */
int ima_gpu_get_times(ima_ctx *ctx, int ci, int li, double *time, int32_t *nmig, double *mig_t);
/* changet_RY1's moves (update_t_RY.cpp:279-335; beforesplit/aftersplit
 * :59-86) on every locus of the nch chains: node times of non-root edges and
 * migration times in (t_u, oldt] and (oldt, t_d) of chain k's period
 * period[k] go to their image under oldt -> newt.  counts (may be NULL)
 * [nch][4] = ecd, ecu, emd, emu as the reference counts them (node times
 * once per daughter edge).  inverse = 1 moves them back (:444-491) and
 * restores the genealogies' lengths. */
int ima_gpu_rubber_band(ima_ctx *ctx, int nch, const int32_t *chains, const int32_t *period,
                        const double *oldt, const double *newt, const double *t_u, const double *t_d,
                        int inverse, int32_t *counts);
/* treeweight of every locus of the nch chains from the resident genealogies
 * and labels, with split times tvals [nch][npops-1] (C[ci]->tvals); the
 * genealogies' lengths (G->length) are updated on the device for the
 * likelihoods; then sum_treeinfo and initialize_integrate_tree_prob per chain:
 * probg [nch], q [nch][nth], m [nch][nmg] (q, m may be NULL).  The weights
 * of these chains stay available to ima_gpu_tree_prob (genealogy index =
 * chain * nloci + locus); a group there that takes in a genealogy of a chain
 * not in this call gives IMA_ERR_STATE. */
int ima_gpu_chain_weights(ima_ctx *ctx, int nch, const int32_t *chains, const double *tvals,
                          double *probg, double *q, double *m);

/* One changet_RY1 of each of the nch chains, decided on the device: the
 * band forward, the chains' weights and p(G), their likelihoods (u, kappa
 * [nch][nloci]; kappa may be NULL), then per chain the reference's
 * Metropolis-Hastings term (update_t_RY.cpp:394-410) from the likelihood
 * sums in locus order, p(G) against the resident p(G) (ima_gpu_set_probg),
 * the resident heat (ima_gpu_set_betas), gbeta, the counts and the host's
 * log_hu = log((newt - t_u)/(oldt - t_u)), log_hd = log((t_d - newt)/
 * (t_d - oldt)) (0 for the last period), against logU = log(U).  Accepted
 * chains are committed (likelihoods, p(G)); the others moved back.  tvals
 * [nch][npops-1]: the proposed split times.  accept [nch]; pdgsum and probg
 * (may be NULL) [nch]: each chain's likelihood sum and p(G) after the
 * decision.  The caller draws newt and U in the reference's order (getnewt's
 * uniform, then the acceptance uniform, chain by chain). */
int ima_gpu_changet_ry1_sweep(ima_ctx *ctx, int nch, const int32_t *chains, const int32_t *period,
                              const double *oldt, const double *newt, const double *t_u, const double *t_d,
                              const double *log_hu, const double *log_hd, const double *logU, double gbeta,
                              const double *tvals, const double *u, const double *kappa, int precision,
                              uint8_t *accept, double *pdgsum, double *probg);

/* Copy surface rows start .. start+count to the host ([count][rowlen]), e.g.
 * to write them with ima_ti_write_binary.  rowlen must be the surface's
 * (IMA_ERR_ARG otherwise). */
int ima_gpu_surface_get_rows(ima_ctx *ctx, int start, int count, int rowlen, float *rows);
/* The split times the resident labels follow, [nchains][npops-1]: the last
 * tvals given to ima_gpu_chain_weights, moved by ima_gpu_rubber_band (to
 * newt, and back to oldt with inverse = 1) and by the rejections of
 * ima_gpu_changet_ry1_sweep.  After ima_gpu_set_locus_pops. */
int ima_gpu_get_split_times(ima_ctx *ctx, double *tvals);

/* ------------------------------------------ saved genealogies (.ti files)
 * Host functions, no context.  ima_ti_read parses the reference's text
 * format (loadgenealogyvalues, ima_main_mpi.cpp:3216-3440): header lines up
 * to one containing VALUESSTART, then one line of `rowlen` (gsampinflength)
 * values per genealogy.  Files are taken in the order given (the reference
 * takes them in directory order).  When more genealogies are present than
 * min(maxload (0 = no limit), MAXGENEALOGIESTOSAVE = 300000), lines are kept
 * by the reference's running-fraction rule.  rows == NULL: counts only (*loaded
 * and *total).  Otherwise rows [rows_cap][rowlen] receives the kept rows, to
 * be passed to ima_gpu_surface_load.  IMA_ERR_DATA: no VALUESSTART line, or a
 * line with too few or too many values. */
int ima_ti_read(int nfiles, const char *const *paths, int rowlen, int maxload, float *rows, int rows_cap,
                int *loaded, int *total);
/* Binary side-car of loaded rows, reloaded without parsing. */
int ima_ti_write_binary(const char *path, int G, int rowlen, const float *rows);
/* rows == NULL: header only (*G, *rowlen).  Otherwise *rowlen on input is
 * the row length rows [rows_cap][*rowlen] was sized for: a file with another
 * row length gives IMA_ERR_DATA, more than rows_cap rows IMA_ERR_TOO_LARGE,
 * before anything is read.  *G and *rowlen return the file's header. */
int ima_ti_read_binary(const char *path, int *G, int *rowlen, float *rows, int rows_cap);

/* ---------------------------------------------------- L-mode peak search
 * MT19937 generator state (utilities.cpp:323-427, Matsumoto & Nishimura):
 * the reference's global generator, carried by the caller so that a peak
 * search continues the caller's stream. */
typedef struct {
  uint32_t mt[624];
  int mti;
} ima_mt19937;
/* init_genrand, as setseeds (utilities.cpp:399-408) seeds the generator */
void ima_mt19937_seed(ima_mt19937 *rng, uint32_t seed);
/* genrand_real3, the reference's uniform() in (0,1) */
double ima_mt19937_uniform(ima_mt19937 *rng);
/* modelloop (jointfind.cpp:746-812): differential-evolution search for the
 * peak of the loaded surface, for modeltype 0 (full), 1 (population sizes)
 * or 2 (migration rates) -- findjointpeaks (:1089-1183) runs 0 for two
 * populations, 1 and 2 otherwise.  Bounds are (MINPARAMVAL, upper[k]], the
 * priors' maxima (setbounds :578-590).  xmap (NULL for the model itself)
 * gives a nested model of `nested` parameters as setup_mapping does: entry k
 * is the nested index of full parameter k, or -value for a constant;
 * nested models of modeltype 2 are not accepted (the reference's bounds for
 * them index past the mapped ones).  Each generation's popsizemultiplier *
 * (model parameters) trial vectors are evaluated in one surface call with
 * `method`; IMA_SURF_COMPAT (the reference's jointp) follows the reference's
 * search exactly, draw for draw from *rng.  Out: best[np+nm] the peak in the
 * full model's parameters and best[np+nm] its -log density; *ess the
 * effective number of genealogies there; generations over all restarts; the
 * number of searches run.  Any of ess, generations, restarts may be NULL. */
int ima_gpu_modelloop(ima_ctx *ctx, int modeltype, const double *upper, int popsizemultiplier,
                      const double *xmap, int nested, int method, ima_mt19937 *rng, double *best,
                      double *ess, int *generations, int *restarts);

/* ------------------------------------------------ checkpoint and restart
 * The resident chain state to a file and back, for the restart the
 * reference makes from its .mcf file (writemcf / readmcf, mcmcfile.cpp:
 * 204-292 / 310-442, called at ima_main_mpi.cpp:1778, 2146, 4176): every
 * chain-locus's genealogy (nodes, times, level schedule, length, base
 * frequencies, alleles), its likelihood G.pdg, population labels and
 * migration events (after ima_gpu_set_labels), the chains' p(G), heats and
 * split times (after ima_gpu_set_locus_pops), each locus's hval and samppop,
 * and (rng may be NULL) the caller's generator.  ima_gpu_checkpoint_read
 * restores it into a context with the same loci and number of chains (the
 * reference also fills more chains than the file holds by rereading it;
 * here the counts must agree) and, when the
 * file holds labels, the same population model already set -- IMA_ERR_STATE
 * otherwise, IMA_ERR_DATA for a file that is not one or is truncated.  HKY
 * partial likelihoods are not saved: the first evaluation after a restore
 * is a full one (edits NULL), which gives the same G.pdg.  The reference's
 * .mcf also carries its burn-in and sampling counters and the running
 * tables of the host program; those stay with the caller. */
int ima_gpu_checkpoint_write(ima_ctx *ctx, const char *path, const ima_mt19937 *rng);
int ima_gpu_checkpoint_read(ima_ctx *ctx, const char *path, ima_mt19937 *rng);

/* ima_gpu_changet_ry1_sweep with the draws made here: for each chain k in
 * order, getnewt (update_gtree_common.cpp:2501-2519) on period[k] with the
 * prior range [tprior_lo[p], tprior_hi[p]] inside the neighbouring split
 * times (the context's, ima_gpu_get_split_times; TIMEMAX above the last
 * one), then the acceptance uniform, both from *rng, as the reference draws
 * them; then the sweep.  newt_out [nch] (may be NULL): the proposed times. */
int ima_gpu_changet_ry1_sweep_mt(ima_ctx *ctx, int nch, const int32_t *chains, const int32_t *period,
                                 const double *tprior_lo, const double *tprior_hi, ima_mt19937 *rng, double gbeta,
                                 const double *u, const double *kappa, int precision, uint8_t *accept,
                                 double *pdgsum, double *probg, double *newt_out);

/* ------------------------------------------------- genealogy update
 * A chain's generators for the genealogy update, as the reference keeps
 * them in globals: the MT19937 of uniform() (utilities.cpp:419-426), the
 * second deviate normdev caches between calls (iset, gset; :476-503) and
 * bitran's shift register (iseed; :438-455). */
typedef struct {
  ima_mt19937 mt;
  int32_t iset;
  double gset;
  uint64_t iseed;
} ima_ug_rng;
/* setseeds (utilities.cpp:399-408): init_genrand(seed), iseed =
 * ULONG_MAX / 2 + seed, no cached deviate */
void ima_ug_rng_seed(ima_ug_rng *rng, int32_t seed);
/* updategenealogy (update_gtree.cpp:723-966) of the no-migration model
 * (slider_nomigration, :79-254) on the resident genealogies of the listed
 * chains: nsweeps sweeps, each proposing a new genealogy for every locus in
 * order on every listed chain (chains in parallel, each drawing from its own
 * rng[k], updated in place), as qupdate calls it (ima_main_mpi.cpp:1821-1841).
 * A proposal picks an edge (randposint until it is not the root's), slides
 * its bottom by a normal deviate of sd min(20, roottime / 3) through the
 * genealogy (bitran at every node), reattaches it, recomputes the locus's
 * weights, the chain's p(G) from its summed weights (+ new - old) and the
 * locus's likelihood (IS in full; HKY from the four edited edges, in
 * `precision`; SW by finishSWupdateA, update_gtree_common.cpp:2219-2362: a
 * new allele for the freed node and the moved branches' terms, in FP64), and
 * accepts with the reference's Metropolis-Hastings term (heat from
 * ima_gpu_set_betas, gbeta; the allele proposal's Hastings term for SW) and
 * one more uniform -- none when the IS likelihood rejects the genealogy.  A
 * rejection restores the genealogy (and for SW the alleles and terms, as
 * restoreedges does).  Needs the population model with nomig = 1, labels and
 * locus populations (ima_gpu_set_labels, ima_gpu_set_locus_pops), and IS,
 * HKY or one-marker SW loci (IMA_ERR_ARG for more markers).  tvals
 * [nch][npops-1]: the chains' split times; u [nch * nloci], kappa [nch *
 * nloci] (may be NULL: 1); allele_range [nloci][2]: each SW locus's minA and
 * maxA (L[li].minA/maxA; NULL when there is no SW locus).  The call starts from a full
 * evaluation of the chains' loci and their weights summed afresh (what the
 * reference holds after its set-up or an accepted split-time update), then
 * carries the sums from proposal to proposal as the reference does.  Out
 * (each may be NULL): accepted [nch * nloci] and topology [nch * nloci]
 * accepted proposals and accepted topology changes per chain-locus; probg
 * [nch] the chains' p(G) at the end.  Resident G.pdg and p(G) are updated. */
int ima_gpu_updategenealogy_sweep(ima_ctx *ctx, int nch, const int32_t *chains, const double *tvals, int nsweeps,
                                  const double *u, const double *kappa, const int32_t *allele_range, double gbeta,
                                  int precision, ima_ug_rng *rng, int32_t *accepted, int32_t *topology,
                                  double *probg);
/* The resident genealogy of chain ci, locus li: up0, up1, down, time and
 * the population labels [2n-1] (any may be NULL). */
int ima_gpu_get_genealogy(ima_ctx *ctx, int ci, int li, int32_t *up0, int32_t *up1, int32_t *down, double *time,
                          int32_t *pop);

/* No counterpart in the reference.  The FP64 surface of ima_gpu_surface_eval
 * (IMA_SURF_FP64) for callers that may not allocate device memory: a plugin
 * inside a host application that owns every device allocation through its
 * own pool (a cudaMalloc there would bypass the pool's accounting and
 * synchronise the device).  No context and no allocation: every pointer is
 * caller-owned DEVICE memory (rows [G][rowlen] float, lognorm [G] or NULL,
 * x [npoints][np+nm], q and ess [npoints], ess may be NULL); work is queued
 * on `stream` (a cudaStream_t, NULL = legacy default stream) and results are
 * ready when that stream is.  The kernel's scratch is a fixed 4 MiB device
 * array inside this library, held on every GPU that loads it until the
 * process exits; it bounds npoints at 174762 -- larger requests return
 * IMA_ERR_TOO_LARGE without launching anything.  The first call on a device
 * looks up the array's device address (make it before any stream capture).
 * All calls share the array: calls that overlap on the GPU (different
 * streams, or other threads) race, so serialise them.  An error already
 * pending on the calling thread (cudaPeekAtLastError) is returned as
 * IMA_ERR_CUDA before anything is launched and left pending.  The looked-up
 * address does not survive a cudaDeviceReset of the device: do not call this
 * after a reset in the same process. */
#define IMA_ERR_TOO_LARGE (-7)
int ima_gpu_surface_fp64_noalloc(const float *rows, int G, int rowlen, int numpopsizeparams,
                                 int nummigrateparams, int npops, const double *lognorm,
                                 const double *x, int npoints, int modeltype, double *q,
                                 double *ess, void *stream);

/* ------------------------------------------------------------ measurement */
/* CUDA-event timer on the context stream. */
int ima_gpu_timer_begin(ima_ctx *ctx);
int ima_gpu_timer_end(ima_ctx *ctx, float *ms);
/* Per-kernel accounting: when enabled, every launch of kernel `kind` is
 * bracketed by events on its stream; totals are read with kernel_stats. */
int ima_gpu_set_profiling(ima_ctx *ctx, int on);
int ima_gpu_kernel_stats(ima_ctx *ctx, int kind, long long *launches, double *ms_total,
                         double *bytes_total);
/* kernel kinds for kernel_stats */
#define IMA_K_IS 0
#define IMA_K_IS_SUMLOGK 1
#define IMA_K_HKY_FAST 2
#define IMA_K_HKY_FP64 3
#define IMA_K_SW_FAST 4
#define IMA_K_SW_FP64 5
#define IMA_K_SWAP 6
#define IMA_K_SURF_FAST 7
#define IMA_K_SURF_FP64 8
#define IMA_K_SURF_COMPAT 9
#define IMA_K_SURF_TC 10
#define IMA_K_MARGIN 11
#define IMA_K_TREEWEIGHT 12
#define IMA_K_TREE_PROB 13
#define IMA_K_POPMIG 14
#define IMA_K_HKY_FP32 15
#define IMA_K_TIMES 16             /* re-timing uploads: float-float copies, lengths, in-place reads */
#define IMA_K_UG 17                /* genealogy update: proposals and decisions */
#define IMA_K_COUNT 18
/* Total kernel launches issued by this library on the context. */
int ima_gpu_launch_count(ima_ctx *ctx, long long *n);
/* Write a device buffer larger than L2 (evicts resident data). */
int ima_gpu_flush_l2(ima_ctx *ctx);
/* Device bytes held by the context. */
int ima_gpu_memory(ima_ctx *ctx, size_t *bytes);

#ifdef __cplusplus
}
#endif
#endif /* IMA_GPU_H */
