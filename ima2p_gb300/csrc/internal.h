// internal.h -- device data layout and launch interfaces shared by the
// context (ima_ctx.cu) and the kernels (k_*.cu).
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <functional>
#include <vector>

#include "../../include/ima_gpu.h"

// One genealogy node: the reference's struct edge (imamp.hpp:651-679) reduced
// to its topology, packed into 8 bytes so a node is one load.
struct NodeRec {
  int16_t up0, up1, down, pad;
};

// Locus table entry (shared by every chain).
struct LocusDev {
  int model;      // IMA_MODEL_*
  int n;          // gene copies (tips)
  int nsites;     // IS segregating sites / HKY patterns
  int totsites;   // HKY: columns before pattern compression
  int nlinked;    // SW: linked markers
  int seq_off;    // int8 [n][nsites] in the seq pool
  int mult_off;   // int32 [nsites] in the mult pool
  int pad;
};

// Static placement of one chain-locus in the resident pools.
struct ItemDev {
  int locus;
  int n;
  int node_off;            // nodes / times / slot / fresh pools
  int sched_off;           // int16 [2n] level schedule
  long long part_off;      // HKY: float4 index of slot 0 (slot 1 at + (n-1)*S)
  long long part64_off;    // HKY FP64: double index (x4 per pattern) of slot 0
  int al_off;              // SW: int32 [nlinked][2n-1] alleles
  int dl_off;              // SW: double [nlinked][2n-1] dlikeA
  long long is_off;        // IS: int32 [S] per-site mutation branch cache
};

// One evaluation request (a chain-locus with its parameters).
struct ReqDev {
  int item;
  int ai;
  int e[4];
  double u;
  double par;  // HKY: kappa; SW: branch-time scale tr
  // the item's and locus's fixed offsets and sizes, copied in when the
  // request is built, so a kernel's first load brings them (the HKY kernel
  // otherwise chains request -> item -> locus before its tree loads)
  long long part_off;
  int node_off, sched_off, n, nsites, totsites, seq_off, mult_off, pad;
};

// Everything a kernel may read; passed by value.
struct Pools {
  const LocusDev *loci;
  const ItemDev *items;
  const int8_t *seq;
  const int32_t *mult;
  const NodeRec *nodes;
  const double *t64;        // FP64 node times
  const float2 *tff;        // float-float node times (hi, lo)
  const int16_t *sched;     // per item: order[n-1] then level starts[nlev+1]
  const int32_t *nlev;      // levels per item
  const double *length;     // genealogy length per item (from treeweight)
  const double *pi;         // [item][4]
  const int32_t *alleles;
  double *dlike;            // SW per-branch terms
  double *sumlogk;          // IS per-locus constant
  int32_t *is_site;         // IS: per item and site, (mutation node << 8) | branch (0 first daughter,
                            // 1 second, 2 both at the root); node -1 none, -2 two
  uint8_t *is_valid;        // IS: the item's site cache matches its topology
  double *pdg_new;          // last evaluated log P(D|G) per item
  // HKY state
  float4 *part;             // FP32 partials (float-float form: the hi parts)
  float4 *partlo;           // float-float form: the lo parts (null until first used)
  int32_t *pexp;            // FP32 partial power-of-two exponents
  double *part64;           // FP64 partials (4 per pattern)
  double *psf64;            // FP64 log scale factors
  uint8_t *slot32, *fresh32, *slot64, *fresh64;
};

// Launch wrappers (k_*.cu).  All launch on `st`.
void launch_is_sumlogk(const Pools &P, int item, int locus, int maxn, int maxS, int *d_flag,
                       cudaStream_t st);
void launch_is(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, double *result,
               int32_t *status, int32_t *site_node, cudaStream_t st);
// variant: launch shape chosen by the batch autotuner (0 is the default)
constexpr int HKY_FAST_VARIANTS = 6;  // float-float: 128 threads with registers for 8 CTAs per SM, 64 threads
                                      // (16 CTAs), 256 (4), 128 at 10 CTAs, 128 at 6, 96 at 11;
                                      // FP32: 128 threads (12 CTAs per SM), 64, 256, 128 uncached, 128 at 8,
                                      // 96 at 16
constexpr int SW_FAST_VARIANTS = 3;   // one wave (5 or 6 CTAs per SM), 8 chain-loci per CTA
void launch_hky_fast(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, int variant,
                     double *result, int32_t *status, cudaStream_t st);
void launch_hky_fp32(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, int variant,
                     double *result, int32_t *status, cudaStream_t st);
void launch_hky_fp64(const Pools &P, const ReqDev *reqs, int nreq, int maxn, double *result,
                     int32_t *status, cudaStream_t st);
int hky_init_tables();
void launch_hky_commit(const Pools &P, const int32_t *items, const uint8_t *accept, int n,
                       cudaStream_t st);
void launch_sw_fast(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int variant, double *result,
                    int32_t *status, cudaStream_t st);
void launch_sw_fp64(const Pools &P, const ReqDev *reqs, int nreq, double *result,
                    int32_t *status, cudaStream_t st);

// MC3
struct SwapArgs {
  int nruns, cpr, nloci, swaptries, include_probg, stride;
  const double *pdg;        // [nchains][nloci]
  const double *probg;      // [nchains]
  double *beta;             // [nchains]
  const double *allbetas;   // [nchains]
  const double *uniforms;   // [nruns][stride] or null
  unsigned long long seed;
  unsigned long long *counter;  // per-run Philox counters
  int32_t *used, *swap0ok;
  int32_t *swapcount, *tempcount;  // [nruns][cpr][cpr]
  double *S;                       // scratch [nchains]
};
void launch_swap(const SwapArgs &a, cudaStream_t st);
void launch_pdg_commit(const int32_t *items, const uint8_t *accept, const double *pdg_new,
                       double *pdg, int n, cudaStream_t st);

// Surface
struct SurfArgs {
  int G, rowlen, np, nm, npops, modeltype, npoints;
  const float *rows;        // [G][rowlen]
  const double *lognorm;    // [G] or null
  const double *x;          // [npoints][np+nm]
  double *q, *ess;
};
void launch_surface_fp64(const SurfArgs &a, double *scratch, cudaStream_t st);
void launch_surface_compat(const SurfArgs &a, double *scratch, cudaStream_t st);
constexpr int SURF_COMPAT_CONCURRENT = 64;  // points per launch of the compat surface
// the surface launchers report how many kernels they enqueued in *nkernels
int launch_surface_fast(const SurfArgs &a, void *scratch, size_t scratch_bytes, bool rows_ready, int *nkernels,
                        cudaStream_t st);
size_t surface_fast_scratch_bytes(int G, int npoints);
// *nretaken: points whose terms left the fixed-point sums and were taken again
int launch_surface_tc(const SurfArgs &a, void *scratch, size_t scratch_bytes, int *d_err, bool rows_ready,
                      int *nkernels, int *nretaken, cudaStream_t st);
size_t surface_tc_scratch_bytes(int G, int npoints);
int tc_selftest(cudaStream_t st, void *scratch, size_t bytes, int *h_bad, float *h_maxerr);
size_t surface_fp64_scratch_bytes(int G, int npoints);

// 1-D marginal densities (margincalc)
struct MarginArgs {
  int G, rowlen, np, nm, n, logi;
  int g_lo, g_hi;           // genealogies [g_lo, g_hi) are summed
  int raw_cc;               // marginp: the theta term takes cc as stored, not rounded
  double div;               // the sum is divided by this (G for margincalc)
  int ccp, fcp, hccp, mcp, fmp, qip, mip;  // gsampinf column offsets
  const float *rows;        // [G][rowlen]
  const int32_t *param;     // [n] parameter index (population sizes first)
  const double *x;          // [n]
  const double *expo_mean;  // [nm] or null
  double yadjust;
};
int margin_chunks(int G, int n);
int launch_margin(const MarginArgs &a, double *part, int nchunks, double *out, cudaStream_t st);

// 2NM densities (calc_popmig / calc_pop_expomig) at n requested points
struct PopmigArgs {
  int G, rowlen, n, expo, prob_or_like;
  int g_lo, g_hi;                          // genealogies [g_lo, g_hi) are summed
  double div;                              // the sum is divided by this (G for calc_popmig)
  int ccp, fcp, hccp, mcp, fmp, qip, mip;  // gsampinf column offsets
  const float *rows;                       // [G][rowlen]
  const int32_t *thetai, *mi;              // [n] parameter indices of each point's term
  const double *x, *qmax, *mmax, *mmean;   // [n]; mmean only under the exponential prior
  const double *logfact;                   // [TW_LF_N]
  int32_t *err;                            // first failing series / fraction (0 = none)
};
int popmig_chunks(int G, int n);
int launch_popmig(const PopmigArgs &a, double *part, int nchunks, double *out, cudaStream_t st);

// findmarginpeaks' numeric core (margin_peaks.cu, host): the searches run
// together, their function values evaluated in batches by `eval`
struct MarginPeaksIn {
  int G, np, nm, nterms;
  const double *theta_min, *theta_max, *mig_min, *mig_max;
  const double *mig_mean;      // null: uniform migration priors
  const int32_t *mpop, *mterm; // [nterms] the 2NM terms
};
struct MarginPeaksOut {
  int too_few = 0, rounds = 0;
  double *mlval, *peakloc;       // [NUMTREEINT + 1 = 3][np+nm]
  double *migtest;               // [nm]
  double *lo95, *hi95;           // [np+nm]
  double *pm_mlval, *pm_peakloc; // [3][nterms]
  double *pm_test;               // [nterms]
  float *holdpeakloc;            // [np+nm]
};
// kind 0: marginp's density (cc as stored) of parameter idx; 1: margincalc's
// log density (cc rounded); 2: the 2NM density of term idx under the run's
// migration prior; 3: the same under the uniform prior (marginpopmig);
// summed over genealogies [lo, hi), divided by hi - lo + (lo == 0)
// (margincalc: by hi - lo)
struct MarginPeaksReq {
  int kind, idx, lo, hi;
  double x;
};
using MarginPeaksEval = std::function<int(const std::vector<MarginPeaksReq> &, std::vector<double> &)>;
// returns 0, eval's error, or -1 when a search runs past 20000 rounds
int findmarginpeaks_run(const MarginPeaksIn &in, const MarginPeaksEval &eval, MarginPeaksOut &out);

// genealogy weights (treeweight) and p(G) integrals (initialize_integrate_tree_prob)
#define TW_MAXPOPS 10                      // MAXPOPS, imamp.hpp:122
#define TW_MAXTP (2 * TW_MAXPOPS - 1)
#define TW_MAXT (TW_MAXPOPS * (TW_MAXPOPS + 1) / 2)
#define TW_MAXM 384                        // sum_{k<9} (10-k)^2
#define TW_MAXTH TW_MAXTP
#define TW_MAXMG (2 * (TW_MAXPOPS - 1) * (TW_MAXPOPS - 1))
#define TW_LF_N (1 << 17)                  // logfact entries on the device
struct TwModel {                           // tables of fillplist and setup_iparams
  int npops, nomig, expo, T, M, nth, nmg, nchk;
  int8_t plist[TW_MAXPOPS][TW_MAXPOPS];    // period k: populations in id order
  int8_t pos[TW_MAXPOPS][TW_MAXTP];        // position of population p in period k, -1 absent
  int8_t droppops[TW_MAXPOPS][2], addpop[TW_MAXPOPS];
  int8_t pop_e[TW_MAXTP], pop_down[TW_MAXTP];
  int16_t toff[TW_MAXPOPS + 1], moff[TW_MAXPOPS + 1];
  int16_t th_off[TW_MAXTH + 1], th_idx[TW_MAXT];
  int16_t mg_off[TW_MAXMG + 1], mg_idx[TW_MAXM], chk_idx[TW_MAXM];
  double th_max[TW_MAXTH], th_min[TW_MAXTH];
  double mg_max[TW_MAXMG], mg_min[TW_MAXMG], mg_mean[TW_MAXMG];
};
struct TwArgs {
  int ngen, P;                             // genealogies; sort size (power of 2 >= events)
  const TwModel *model;
  const int32_t *perm;                     // genealogies in processing order
  const int32_t *node_off, *up0, *pop, *mig_off, *mig_p, *gen_locus, *gen_tv;
  const double *time, *mig_t, *tvals;      // tvals [rows][npops-1]
  const double *hlog, *h2term;             // per locus, from the host's log
  const int32_t *samppop;                  // [loci][npops]
  int32_t *cc, *mc, *mignum;               // [ngen][T], [ngen][M], [ngen]
  double *hcc, *fc, *fm, *lens;            // [ngen][T], [ngen][T], [ngen][M], [ngen][2]
  int32_t *err;                            // {code, genealogy}: first failure
  const long long *ev_off;                 // [ngen+1] event-list offsets (an upper bound each)
  double *ev_t;                            // sorted event times (pass 1 -> pass 2)
  uint32_t *ev_c;                          // sorted event codes
  int32_t *ev_n;                           // [ngen] events, -1 when rejected
  // resident genealogies (null for host-packed inputs): up0 from the node
  // records, migration offsets of genealogy g at mig_off + moff_start[g]
  // (relative to its events, which start at mig_t/mig_p + mbase[g])
  const NodeRec *nodes;
  const int32_t *moff_start;
  const long long *mbase;
  double *len_out;                         // [ngen] G->length also written here, or null
};
struct TwProbArgs {
  int ngroups;
  const TwModel *model;
  const int32_t *group_off, *group_tv;     // genealogy ranges summed in order
  const int32_t *cc, *mc;
  const double *hcc, *fc, *fm, *tvals, *pdg, *logfact;
  double *probg, *q, *m;                   // [ngroups], [ngroups][nth], [ngroups][nmg]
  float *rows;                             // [ngroups][rowlen] or null
  int rowlen;
  int32_t *err;
  int32_t *sc;                             // [ngroups][T+M] summed counts (cc, mc)
  double *sd;                              // [ngroups][2T+M] summed fc, hcc, fm
  const int32_t *group_end;                // group i ends at group_end[i] (null: group_off[i+1])
};
// the split-time update's rubber band (changet_RY1) on resident genealogies
struct BandArgs {
  const ItemDev *items;
  const NodeRec *nodes;
  double *t64;
  float2 *tff;
  const int32_t *moff;                     // per item: nl+1 relative offsets at node_off + item
  const long long *mbase;                  // per item: first migration event
  double *mig_t;
  const int32_t *chains;                   // [nch]
  const double *prm;                       // [nch][5]: period, o, n, t_u, t_d
  int nch, nloci, last, inverse;
  int32_t *counts;                         // [nch][4]: ecd, ecu, emd, emu (forward)
  int32_t *item_counts;                    // [nch * nloci][4] per chain-locus counts (forward)
  double *len, *len_hold;                  // per item: saved going forward, restored on the way back
};
int launch_band(const BandArgs &a, cudaStream_t st);  // returns the kernels launched
// changet_RY1's Metropolis-Hastings decision (update_t_RY.cpp:394-410), a
// thread per chain, on the device's weights and likelihoods
struct RyArgs {
  int nch, nloci;
  const int32_t *chains, *counts;          // counts [nch][4] from the band
  const double *lhu, *lhd, *logU;          // [nch] host logs of the Hastings ratios, log U
  const double *probg_new;                 // [nch]
  double gbeta;
  const double *beta;                      // per chain (resident)
  double *probg;                           // per chain (resident): updated on acceptance
  const double *pdg, *pdg_new;             // per item: committed, last evaluation
  uint8_t *accept;                         // [nch]
  double *pdgsum;                          // [nch] the chain's likelihood sum after the decision
};
int launch_ry_decide(const RyArgs &a, cudaStream_t st);
// The genealogy update updategenealogy (update_gtree.cpp:723-966) of the
// no-migration model on resident genealogies, one locus of every listed
// chain per step (k_updgen.cu): a warp per chain proposes (edge, slide,
// reattachment), the weights and the likelihood of the proposed genealogies
// run as batches, and a warp per chain decides, then commits or restores.
struct UgArgs {
  int nch, nloci, locus, maxn, nsplit, hky;
  const int32_t *chains;                   // [nch]
  const ItemDev *items;
  NodeRec *nodes;
  double *t64;
  float2 *tff;
  int32_t *pop;
  int16_t *sched;
  int32_t *nlev;
  double *len;
  uint8_t *is_valid;
  const TwModel *model;
  const double *tvals;                     // [nchains][nsplit]
  ima_ug_rng *rng;                         // [nch] the listed chains' generators
  ReqDev *req;                             // the locus's evaluation requests
  const int32_t *req_of;                   // [nch] request of each listed chain
  // per listed chain: the genealogy before the proposal, for a rejection
  NodeRec *bk_nodes;                       // [nch][2 maxn]
  double *bk_t;                            // [nch][2 maxn]
  int32_t *bk_pop;                         // [nch][2 maxn]
  int16_t *bk_sched;                       // [nch][2 maxn]
  double *bk_len;                          // [nch]
  int32_t *bk_nlev;                        // [nch]
  int32_t *prop;                           // [nch][2]: topology changed, tmrca changed
  double *slidew;                          // [nch] the slide's Hastings term
  // predraw: the proposal draws the acceptance uniform itself, right after
  // its own draws, into ustore [nch] (an HKY locus always draws it, so the
  // stream's order is the reference's); otherwise the decision draws it
  int predraw;
  double *ustore;
  int32_t *edges;                          // [nch][4]: edge, freed, old sister, new sister
  // stepwise loci (one marker): finishSWupdateA on the proposal (k_ug_sw)
  int sw;
  int32_t *alleles;                        // the allele pool (per item at al_off)
  double *dlike;                           // FP64 branch terms (per item at dl_off)
  const int32_t *arange;                   // [nloci][2] allele range
  const double *u_cl;                      // [nch][nloci] mutation rates
  int32_t *bk_A;                           // [nch][2 maxn] alleles before the proposal
  double *bk_dl;                           // [nch][2 maxn] branch terms before the proposal
  double *swnew;                           // [nch] proposed G.pdg
  double *aterm;                           // [nch] the allele proposal's Hastings term
  double *holdsis;                         // [nch] the new sister's term before the update
  int32_t *err;                            // {code, listed chain} of the first failure
  // the decision
  const double *res;                       // the batch's results
  const int32_t *st;                       // and status words
  const int32_t *ncc;                      // proposed genealogies' weights [items][T]
  const double *nfc, *nhcc;
  int32_t *cc;                             // committed weights [items][T]
  double *fc, *hcc;
  int32_t *ag_cc;                          // the chains' summed weights [nch][T]
  double *ag_fc, *ag_hcc;
  double *qint;                            // [nch][nth] the chains' integrals
  double *probg;                           // [nchains] resident p(G)
  double *pdg;                             // [items] resident log P(D|G)
  const double *beta;                      // [nchains]
  double gbeta;
  const double *logfact;
  uint8_t *slot32, *fresh32, *slot64, *fresh64;
  int32_t *nacc, *ntopo;                   // [nch][nloci] accepted proposals, accepted topology changes
};
enum { UG_E_SLIDE = 1, UG_E_ROOTTIME = 2, UG_E_ISFAIL = 3, UG_E_TERM = 4, UG_E_TREE = 5 };
void launch_ug_propose(const UgArgs &a, cudaStream_t st);
void launch_ug_sw(const UgArgs &a, cudaStream_t st);  // k_sw.cu
void launch_ug_decide(const UgArgs &a, cudaStream_t st);
bool tw_fits(int P);                       // P events fit one warp's shared memory
int launch_treeweight(const TwArgs &a, const TwModel &h, cudaStream_t st);
int launch_tree_prob(const TwProbArgs &a, const TwModel &h, cudaStream_t st);
int launch_gather_rows(const float *rows, int rowlen, const int32_t *groups, int n, float *dst, cudaStream_t st);
