// ima2p_shims.cpp -- the IMa2p-side binding of the hot paths to
// libima2p_gb300: the same functions the IMa2p host program calls
// (prototypes in imamp.hpp:1165-1174 and :1268-1280), with bodies that hand
// the work to the GPU library.  Compiled against IMa2p's own headers and
// linked with the untouched IMa2p objects; the objects that define these
// functions are compiled with them renamed (cpu_likelihoodHKY, ...), so
// every call site of the host program reaches the bodies below.
//
// The host keeps its genealogies, proposals and decisions.  Before each
// evaluation the chain-locus's genealogy is copied to the device (topology,
// times and the tree length treeweight left in C[ci]->G[li].length; HKY base
// frequencies; SW allele states), the library evaluates it on the GPU, and
// the reference's side effects (gtree[].dlikeA, the committed partial
// likelihoods, the swapped betas and swap counts) are kept.
//
// Loci of the joint models (one infinite-sites or HKY part plus linked
// stepwise markers) are refused: the library holds one model per locus.
#include <cstring>
#include <vector>

#include "imamp.hpp"
#include "ima_gpu.h"

namespace {

ima_ctx *g_ima = nullptr;
std::vector<int32_t> g_sc, g_tc;  // the device's swap counts after the last call

void check(int r, const char *what)
{
  if (r != IMA_OK) IM_err(IMERR_MEM, "GB300 library, %s: %s", what, g_ima ? ima_gpu_error(g_ima) : "no context");
}

// The locus tables as readata.cpp built them, once per process: created on
// the first call, after setup() has read the data and sized the chains.
void setup()
{
  if (g_ima) return;
  if (ima_gpu_create(0, &g_ima) != IMA_OK) IM_err(IMERR_MEM, "GB300 library: no usable GPU");
  for (int li = 0; li < nloci; li++) {
    const int n = L[li].numgenes, S = L[li].numsites;
    std::vector<int8_t> seq((size_t)n * (S > 0 ? S : 1));
    int id = -1;
    switch (L[li].model) {
      case INFINITESITES:
      case HKY:
        for (int i = 0; i < n; i++)
          for (int s = 0; s < S; s++) seq[(size_t)i * S + s] = (int8_t)L[li].seq[i][s];
        if (L[li].model == INFINITESITES) check(ima_gpu_add_locus_is(g_ima, n, S, seq.data(), &id), "IS locus");
        else check(ima_gpu_add_locus_hky(g_ima, n, S, L[li].totsites, seq.data(), L[li].mult, &id), "HKY locus");
        break;
      case STEPWISE:
        check(ima_gpu_add_locus_sw(g_ima, n, L[li].nlinked, &id), "SW locus");
        break;
      default:
        IM_err(IMERR_MEM, "GB300 library: locus %d mixes mutation models, which it does not hold", li);
    }
  }
  check(ima_gpu_set_chains(g_ima, 1, numchains), "chains");
}

// C[ci]->G[li] to the device
void push_tree(int ci, int li)
{
  setup();
  const struct edge *t = C[ci]->G[li].gtree;
  const int nl = L[li].numlines;
  std::vector<int32_t> up0(nl), up1(nl), down(nl);
  std::vector<double> time(nl);
  for (int k = 0; k < nl; k++) {
    up0[k] = t[k].up[0];
    up1[k] = t[k].up[1];
    down[k] = t[k].down;
    time[k] = t[k].time;
  }
  check(ima_gpu_set_genealogy(g_ima, ci, li, up0.data(), up1.data(), down.data(), time.data(),
                              C[ci]->G[li].length), "genealogy");
  if (L[li].model == HKY) check(ima_gpu_set_pi(g_ima, ci, li, C[ci]->G[li].pi), "base frequencies");
  if (L[li].model == STEPWISE)
    for (int ai = 0; ai < L[li].nlinked; ai++) {
      std::vector<int32_t> A(nl);
      for (int k = 0; k < nl; k++) A[k] = t[k].A[ai];
      check(ima_gpu_set_alleles(g_ima, ci, li, ai, A.data()), "alleles");
    }
}

double ref_uniform(void *) { return uniform(); }

}  // namespace

// calc_prob_data.cpp:731
double likelihoodIS(int ci, int li, double mutrate)
{
  push_tree(ci, li);
  double r = 0.0;
  const int st = ima_gpu_likelihoodIS(g_ima, ci, li, mutrate, &r);
  if (st == IMA_ERR_DATA)
    IM_err(IMERR_INFINITESITESFAIL, "Data incompatible with current genealogy, likelihood calculation failed, "
                                    "chain %d, locus %d", ci, li);
  check(st, "likelihoodIS");
  return r;  // REJECTINFINITESITESCONSTANT when a site needs two mutations
}

// calc_prob_data.cpp:583
double likelihoodHKY(int ci, int li, double mutrate, double kappa, int e1, int e2, int e3, int e4)
{
  push_tree(ci, li);
  double r = 0.0;
  check(ima_gpu_likelihoodHKY(g_ima, ci, li, mutrate, kappa, e1, e2, e3, e4, &r), "likelihoodHKY");
  return r;
}

// calc_prob_data.cpp:841
double likelihoodSW(int ci, int li, int ai, double u, double tr)
{
  push_tree(ci, li);
  double r = 0.0;
  check(ima_gpu_likelihoodSW(g_ima, ci, li, ai, u, tr, &r), "likelihoodSW");
  const int nl = L[li].numlines;
  std::vector<double> dl(nl);
  check(ima_gpu_get_dlikeA(g_ima, ci, li, ai, dl.data()), "dlikeA");
  for (int i = 0; i < nl; i++) C[ci]->G[li].gtree[i].dlikeA[ai] = dl[i];
  return r;
}

// update_gtree_common.cpp:2140, :2158, :2170 -- the partial likelihoods
// stay on the device; accept keeps the new ones, reject the old
void copyfraclike(int ci, int li)
{
  setup();
  check(ima_gpu_copyfraclike(g_ima, ci, li), "copyfraclike");
}
void storescalefactors(int ci, int li)
{
  setup();
  check(ima_gpu_storescalefactors(g_ima, ci, li), "storescalefactors");
}
void restorescalefactors(int ci, int li)
{
  setup();
  check(ima_gpu_restorescalefactors(g_ima, ci, li), "restorescalefactors");
}

// swapchains.cpp:526 -- the host's likelihoods and heats go to the device,
// which sums them per chain; the attempts draw uniform() exactly where the
// reference draws it; betas and both count matrices come back.
int swapchains(int swaptries, int swapbetasonly, int currentid, int heatmode)
{
  (void)currentid;
  (void)heatmode;
  if (!swapbetasonly) IM_err(IMERR_MEM, "GB300 library: swaps exchange heats only (swapbetasonly)");
  setup();
  if (numchains < 2) return 0;
  std::vector<double> pdg((size_t)numchains * nloci), probg(numchains), b(beta, beta + numchains),
      ab(allbetas, allbetas + numchains);
  for (int c = 0; c < numchains; c++) {
    for (int l = 0; l < nloci; l++) pdg[(size_t)c * nloci + l] = C[c]->G[l].pdg;
    probg[c] = C[c]->allpcalc.probg;
  }
  check(ima_gpu_set_pdg(g_ima, pdg.data()), "pdg");
  check(ima_gpu_set_probg(g_ima, probg.data()), "probg");
  check(ima_gpu_set_betas(g_ima, b.data()), "betas");
  check(ima_gpu_set_allbetas(g_ima, ab.data()), "heat ladder");
  const size_t nn = (size_t)numchains * numchains;
  if (g_sc.size() != nn) {
    g_sc.assign(nn, 0);
    g_tc.assign(nn, 0);
    check(ima_gpu_get_swapcounts(g_ima, 0, g_sc.data(), g_tc.data()), "swap counts");
  }
  int32_t used = 0, ok = 0;
  check(ima_gpu_swapchains_cb(g_ima, swaptries, !calcoptions[CALCMARGINALLIKELIHOOD], ref_uniform, nullptr, &used,
                              &ok), "swapchains");
  check(ima_gpu_get_betas(g_ima, b.data()), "betas");
  for (int c = 0; c < numchains; c++) beta[c] = b[c];
  std::vector<int32_t> sc(nn), tc(nn);
  check(ima_gpu_get_swapcounts(g_ima, 0, sc.data(), tc.data()), "swap counts");
  for (int i = 0; i < numchains; i++)
    for (int j = 0; j < numchains; j++) {
      swapcount[i][j] += sc[(size_t)i * numchains + j] - g_sc[(size_t)i * numchains + j];
      tempbasedswapcount[i][j] += tc[(size_t)i * numchains + j] - g_tc[(size_t)i * numchains + j];
    }
  g_sc = sc;
  g_tc = tc;
  return ok;
}
