/*
 * ref_harness.cpp -- drives the UNMODIFIED IMa2p reference functions on
 * dumped inputs, to pin the oracle restatement (oracle/ima_oracle.c) and to
 * produce the golden fixtures under tests/golden/.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the reference sources where they lie (nothing is copied into this repo);
 * the result, oracle/_ref/imaref, is git-ignored.
 *
 * The reference keeps some hot-path state in file statics (the sumlogk cache
 * in calc_prob_data.cpp, jointp's list and model range in jointfind.cpp);
 * ref_access_cpd.cpp and ref_access_jf.cpp include those two reference
 * sources to reach them.  The other reference objects are linked unchanged.
 *
 * Usage:  imaref is|hky|sw|swap|jointp|de|margin|tw|iterm|ry|popmig|peaks|iparams|ug <input.txt>
 *         (results on stdout)
 */
#undef GLOBVARS
#include "imamp.hpp"
#include "ref_access.h"
#include <string>

#include <array>
#include <cstdio>
#include <cstdlib>
#include <vector>

static FILE *g_in;
static int rd_i() { int v; if (fscanf(g_in, "%d", &v) != 1) { fprintf(stderr, "short input\n"); exit(3); } return v; }
static double rd_d() { double v; if (fscanf(g_in, "%lf", &v) != 1) { fprintf(stderr, "short input\n"); exit(3); } return v; }

static void alloc_chains(int nchains, int nl)
{
  numchains = nchains;
  numprocesses = 1;
  nloci = nl;
  C = (struct chain **)calloc((size_t)nchains, sizeof(struct chain *));
  for (int c = 0; c < nchains; c++) {
    C[c] = (struct chain *)calloc(1, sizeof(struct chain));
    C[c]->G = (struct genealogy *)calloc((size_t)nl, sizeof(struct genealogy));
  }
  L = (struct locus *)calloc((size_t)nl, sizeof(struct locus));
}

static struct edge *alloc_tree(int nlines)
{
  return (struct edge *)calloc((size_t)nlines, sizeof(struct edge));
}

/* reads up0[nl] up1[nl] down[nl] time[nl] into gtree */
static void read_tree(struct edge *t, int nlines)
{
  for (int i = 0; i < nlines; i++) t[i].up[0] = rd_i();
  for (int i = 0; i < nlines; i++) t[i].up[1] = rd_i();
  for (int i = 0; i < nlines; i++) t[i].down = rd_i();
  for (int i = 0; i < nlines; i++) t[i].time = rd_d();
}

static int find_root(struct edge *t, int nlines)
{
  for (int i = 0; i < nlines; i++) if (t[i].down == -1) return i;
  return -1;
}

/* IS: n S seq[n*S] nitems {tree length u}*   ->  pdg sumlogk_cache own_sumlogk */
static void run_is()
{
  int n = rd_i(), S = rd_i();
  int nl = 2 * n - 1;
  std::vector<int> seq((size_t)n * S);
  for (auto &v : seq) v = rd_i();
  int nitems = rd_i();
  alloc_chains(nitems, 1);
  L[0].numgenes = n;
  L[0].numlines = nl;
  L[0].numsites = S;
  L[0].seq = (int **)malloc(sizeof(int *) * n);
  for (int i = 0; i < n; i++) L[0].seq[i] = &seq[(size_t)i * S];
  std::vector<double> us(nitems);
  for (int c = 0; c < nitems; c++) {
    C[c]->G[0].gtree = alloc_tree(nl);
    read_tree(C[c]->G[0].gtree, nl);
    C[c]->G[0].root = find_root(C[c]->G[0].gtree, nl);
    C[c]->G[0].length = rd_d();
    us[c] = rd_d();
  }
  for (int c = 0; c < nitems; c++) {
    double pdg = likelihoodIS(c, 0, us[c]);
    double own = 0.0;
    calc_sumlogk(c, 0, &own);
    printf("%.17g %.17g %.17g\n", pdg, refacc_sumlogk(0), own);
  }
}

/* HKY: n S totsites seq mult pi[4] nitems
 *   per item: tree u kappa nedits { tree e1 e2 e3 e4 accept }*
 *   -> one line per evaluation */
static void alloc_hky(struct edge *t, int n, int S)
{
  for (int i = n; i < 2 * n - 1; i++) {
    t[i].hkyi.frac = (double **)malloc(sizeof(double *) * S);
    t[i].hkyi.newfrac = (double **)malloc(sizeof(double *) * S);
    for (int k = 0; k < S; k++) {
      t[i].hkyi.frac[k] = (double *)calloc(4, sizeof(double));
      t[i].hkyi.newfrac[k] = (double *)calloc(4, sizeof(double));
    }
    t[i].hkyi.scalefactor = (double *)calloc((size_t)S, sizeof(double));
    t[i].hkyi.oldscalefactor = (double *)calloc((size_t)S, sizeof(double));
  }
}

static void run_hky()
{
  int n = rd_i(), S = rd_i(), tots = rd_i();
  int nl = 2 * n - 1;
  std::vector<int> seq((size_t)n * S);
  for (auto &v : seq) v = rd_i();
  std::vector<int> mult(S);
  for (auto &v : mult) v = rd_i();
  double pi[4];
  for (int j = 0; j < 4; j++) pi[j] = rd_d();
  int nitems = rd_i();
  alloc_chains(1, 1);
  L[0].numgenes = n;
  L[0].numlines = nl;
  L[0].numsites = S;
  L[0].totsites = tots;
  L[0].mult = mult.data();
  L[0].seq = (int **)malloc(sizeof(int *) * n);
  for (int i = 0; i < n; i++) L[0].seq[i] = &seq[(size_t)i * S];
  for (int j = 0; j < 4; j++) C[0]->G[0].pi[j] = pi[j];
  struct edge *t = alloc_tree(nl);
  alloc_hky(t, n, S);
  C[0]->G[0].gtree = t;
  for (int it = 0; it < nitems; it++) {
    read_tree(t, nl);
    C[0]->G[0].root = find_root(t, nl);
    double u = rd_d(), kappa = rd_d();
    double p = likelihoodHKY(0, 0, u, kappa, -1, -1, -1, -1);
    printf("%.17g\n", p);
    copyfraclike(0, 0);
    storescalefactors(0, 0);
    int nedits = rd_i();
    for (int k = 0; k < nedits; k++) {
      read_tree(t, nl);
      C[0]->G[0].root = find_root(t, nl);
      int e1 = rd_i(), e2 = rd_i(), e3 = rd_i(), e4 = rd_i(), acc = rd_i();
      double pe = likelihoodHKY(0, 0, u, kappa, e1, e2, e3, e4);
      printf("%.17g\n", pe);
      if (acc) { copyfraclike(0, 0); storescalefactors(0, 0); }
      else restorescalefactors(0, 0);
    }
  }
}

/* SW: n nitems {tree A[nl] u tr}*  ->  like dlikeA[nl] */
static void run_sw()
{
  int n = rd_i();
  int nl = 2 * n - 1;
  int nitems = rd_i();
  alloc_chains(1, 1);
  L[0].numgenes = n;
  L[0].numlines = nl;
  L[0].minA[0] = -1000000;
  L[0].maxA[0] = 1000000;
  struct edge *t = alloc_tree(nl);
  for (int i = 0; i < nl; i++) {
    t[i].A = (int *)calloc(1, sizeof(int));
    t[i].dlikeA = (double *)calloc(1, sizeof(double));
  }
  C[0]->G[0].gtree = t;
  for (int it = 0; it < nitems; it++) {
    read_tree(t, nl);
    for (int i = 0; i < nl; i++) t[i].A[0] = rd_i();
    double u = rd_d(), tr = rd_d();
    double like = likelihoodSW(0, 0, 0, u, tr);
    printf("%.17g", like);
    for (int i = 0; i < nl; i++) printf(" %.17g", t[i].dlikeA[0]);
    printf("\n");
  }
}

/* SWAP: nchains nloci swaptries nsteps heatmode h1 h2 seed pdg[nchains*nloci] probg[nchains]
 *   -> per step: beta[]; then swapcount and tempbasedswapcount rows */
static void run_swap()
{
  int nch = rd_i(), nl = rd_i(), tries = rd_i(), nsteps = rd_i(), mode = rd_i();
  double h1 = rd_d(), h2 = rd_d();
  int seed = rd_i();
  alloc_chains(nch, nl);
  for (int c = 0; c < nch; c++)
    for (int l = 0; l < nl; l++) C[c]->G[l].pdg = rd_d();
  for (int c = 0; c < nch; c++) C[c]->allpcalc.probg = rd_d();
  setseeds(seed);
  setheat(h1, h2, mode, 0);
  for (int s = 0; s < nsteps; s++) {
    int ok = swapchains(tries, 1, 0, mode);
    printf("%d", ok);
    for (int c = 0; c < nch; c++) printf(" %.17g", beta[c]);
    printf("\n");
  }
  for (int i = 0; i < nch; i++) {
    for (int j = 0; j < nch; j++) printf("%d ", swapcount[i][j]);
    printf("\n");
  }
  for (int i = 0; i < nch; i++) {
    for (int j = 0; j < nch; j++) printf("%d ", tempbasedswapcount[i][j]);
    printf("\n");
  }
}

static void load_gsampinf(int G, int rowlen, int np, int nm, int npp)
{
  genealogiessaved = G;
  numpopsizeparams = np;
  nummigrateparams = nm;
  npops = npp;
  gsampinf = (float **)malloc(sizeof(float *) * G);
  for (int g = 0; g < G; g++) {
    gsampinf[g] = (float *)malloc(sizeof(float) * rowlen);
    for (int k = 0; k < rowlen; k++) gsampinf[g][k] = (float)rd_d();
  }
  eexpsum = (struct extendnum *)malloc(sizeof(struct extendnum) * G);
}

/* JOINTP: G rowlen np nm npops modeltype rows[G*rowlen] npoints points[npoints*(np+nm)]
 *   -> q ess per point */
static void run_jointp()
{
  int G = rd_i(), rowlen = rd_i(), np = rd_i(), nm = rd_i(), npp = rd_i(), mt = rd_i();
  load_gsampinf(G, rowlen, np, nm, npp);
  refacc_jointp_setup(np + nm, mt);
  int npts = rd_i();
  std::vector<double> x(np + nm);
  for (int p = 0; p < npts; p++) {
    for (int k = 0; k < np + nm; k++) x[k] = rd_d();
    double ess = 0.0;
    double q = refacc_jointp(x.data(), &ess);
    printf("%.17g %.17g\n", q, ess);
  }
}

/* DE: G rowlen np nm npops modeltype multiplier seed nested rows[G*rowlen]
 *     upper[np+nm] [xmap[np+nm] when nested > 0]
 *   -> "BEST" best[np+nm] objective; "ESS" ess  (modelloop's own progress
 *      lines also go to stdout) */
static void run_de()
{
  int G = rd_i(), rowlen = rd_i(), np = rd_i(), nm = rd_i(), npp = rd_i(), mt = rd_i();
  int mult = rd_i(), seed = rd_i(), nested = rd_i();
  load_gsampinf(G, rowlen, np, nm, npp);
  int n = np + nm;
  std::vector<double> upper(n), xmap(n), best(n + 1);
  for (int k = 0; k < n; k++) upper[k] = rd_d();
  if (nested > 0)
    for (int k = 0; k < n; k++) xmap[k] = rd_d();
  refacc_jointp_setup(n, mt);
  setseeds(seed);
  double ess = 0.0;
  refacc_modelloop(n, mt, upper.data(), mult, nested > 0 ? xmap.data() : nullptr, nested, best.data(), &ess);
  printf("BEST");
  for (int k = 0; k <= n; k++) printf(" %.17g", best[k]);
  printf("\nESS %.17g\n", ess);
}

/* MARGIN: G rowlen np nm expo rows[G*rowlen] [mean[nm] when expo] npts
 *         then per point: pi x logi yadjust   -> margincalc value per point */
static void run_margin()
{
  int G = rd_i(), rowlen = rd_i(), np = rd_i(), nm = rd_i(), expo = rd_i();
  load_gsampinf(G, rowlen, np, nm, 2);
  gsamp_ccp = 0;  // as setup_iparams (initialize.cpp:709-718) sets them
  gsamp_fcp = gsamp_ccp + np;
  gsamp_hccp = gsamp_fcp + np;
  gsamp_mcp = gsamp_hccp + np;
  gsamp_fmp = gsamp_mcp + nm;
  gsamp_qip = gsamp_fmp + nm;
  gsamp_mip = gsamp_qip + np;
  gsamp_pdgp = gsamp_mip + nm;
  gsamp_probgp = gsamp_pdgp + 1;
  gsamp_tp = gsamp_probgp + 1;
  modeloptions[EXPOMIGRATIONPRIOR] = expo;
  imig = static_cast<struct i_param *>(calloc(nm > 0 ? nm : 1, sizeof(struct i_param)));
  if (expo)
    for (int i = 0; i < nm; i++) imig[i].pr.mean = rd_d();
  int npts = rd_i();
  for (int k = 0; k < npts; k++) {
    int pi = rd_i();
    double x = rd_d();
    int logi = rd_i();
    double ya = rd_d();
    printf("%.17g\n", margincalc(x, ya, pi, logi));
  }
}

/* POPMIG: G rowlen np nm expo rows[G*rowlen] qmax[np] mmax[nm] mmean[nm] npts
 *         then per point: thetai mi x prob_or_like -> calc_popmig (calc_pop_expomig
 *         when expo) per point */
static void run_popmig()
{
  int G = rd_i(), rowlen = rd_i(), np = rd_i(), nm = rd_i(), expo = rd_i();
  load_gsampinf(G, rowlen, np, nm, 2);
  setlogfact();
  gsamp_ccp = 0;  // as setup_iparams (initialize.cpp:709-718) sets them
  gsamp_fcp = gsamp_ccp + np;
  gsamp_hccp = gsamp_fcp + np;
  gsamp_mcp = gsamp_hccp + np;
  gsamp_fmp = gsamp_mcp + nm;
  gsamp_qip = gsamp_fmp + nm;
  gsamp_mip = gsamp_qip + np;
  modeloptions[EXPOMIGRATIONPRIOR] = expo;
  itheta = static_cast<struct i_param *>(calloc(np, sizeof(struct i_param)));
  imig = static_cast<struct i_param *>(calloc(nm, sizeof(struct i_param)));
  for (int i = 0; i < np; i++) itheta[i].pr.max = rd_d();
  for (int i = 0; i < nm; i++) imig[i].pr.max = rd_d();
  for (int i = 0; i < nm; i++) imig[i].pr.mean = rd_d();
  int npts = rd_i();
  for (int k = 0; k < npts; k++) {
    int ti = rd_i(), mi = rd_i();
    double x = rd_d();
    int pl = rd_i();
    printf("%.17g\n", expo ? calc_pop_expomig(ti, mi, x, pl) : calc_popmig(ti, mi, x, pl));
  }
}

/* PEAKS: G rowlen np nm expo rows[G*rowlen] thmin[np] thmax[np] mgmin[nm] mgmax[nm]
 *        mgmean[nm] nterms mpop[nterms] mterm[nterms]
 *   -> findmarginpeaks' numbers (surface_call_functions.cpp:433-470, :596-652):
 *      "ML j" / "PK j" per range j = 0..2, "MT" migtest, "LO" / "HI" (margin95 where
 *      the peak exists, else nan), and with terms "PML j" / "PPK j", "PT" */
static void run_peaks()
{
  int G = rd_i(), rowlen = rd_i(), np = rd_i(), nm = rd_i(), expo = rd_i();
  load_gsampinf(G, rowlen, np, nm, 2);
  setlogfact();
  gsamp_ccp = 0;
  gsamp_fcp = gsamp_ccp + np;
  gsamp_hccp = gsamp_fcp + np;
  gsamp_mcp = gsamp_hccp + np;
  gsamp_fmp = gsamp_mcp + nm;
  gsamp_qip = gsamp_fmp + nm;
  gsamp_mip = gsamp_qip + np;
  modeloptions[EXPOMIGRATIONPRIOR] = expo;
  itheta = static_cast<struct i_param *>(calloc(np, sizeof(struct i_param)));
  imig = static_cast<struct i_param *>(calloc(nm > 0 ? nm : 1, sizeof(struct i_param)));
  for (int i = 0; i < np; i++) itheta[i].pr.min = rd_d();
  for (int i = 0; i < np; i++) itheta[i].pr.max = rd_d();
  for (int i = 0; i < nm; i++) imig[i].pr.min = rd_d();
  for (int i = 0; i < nm; i++) imig[i].pr.max = rd_d();
  for (int i = 0; i < nm; i++) imig[i].pr.mean = rd_d();
  int nt = rd_i();
  std::vector<int> mpop(nt > 0 ? nt : 1), mterm(nt > 0 ? nt : 1);
  for (int t = 0; t < nt; t++) mpop[t] = rd_i();
  for (int t = 0; t < nt; t++) mterm[t] = rd_i();
  const int p = np + nm, NT = 2;
  genealogiessaved = IMIN(MAXGENEALOGIESTOSAVE - 1, genealogiessaved);
  if (genealogiessaved <= 10) {
    printf("TOOFEW\n");
    return;
  }
  std::vector<std::vector<double>> ml(NT + 1, std::vector<double>(p, NAN)), pk(NT + 1, std::vector<double>(p, NAN));
  std::vector<std::vector<double>> pml(NT + 1, std::vector<double>(nm > 0 ? nm : 1, NAN)),
      ppk(NT + 1, std::vector<double>(nm > 0 ? nm : 1, NAN));
  int firsttree, lasttree, j;
  for (firsttree = 0, lasttree = (int)genealogiessaved / NT, j = 0; j < NT; j++) {
    marginalopt(firsttree, lasttree, ml[j].data(), pk[j].data());
    if (nt) marginalopt_popmig(firsttree, lasttree, pml[j].data(), ppk[j].data(), mpop.data(), mterm.data());
    firsttree = lasttree + 1;
    lasttree += (int)genealogiessaved / NT;
    if (lasttree > genealogiessaved) lasttree = genealogiessaved;
  }
  marginalopt(0, genealogiessaved, ml[NT].data(), pk[NT].data());
  for (j = 0; j <= NT; j++) {
    printf("ML %d", j);
    for (int i = 0; i < p; i++) printf(" %.17g", pk[j][i] < 0 ? NAN : ml[j][i]);
    printf("\nPK %d", j);
    for (int i = 0; i < p; i++) printf(" %.17g", pk[j][i]);
    printf("\n");
  }
  printf("MT");
  for (int i = 0; i < nm; i++) {
    double maxp = -refacc_marginp(i + np, 0, genealogiessaved, pk[NT][i + np]);
    double max0p = -refacc_marginp(i + np, 0, genealogiessaved, MINPARAMVAL);
    printf(" %.17g", 2 * log(maxp / max0p));
  }
  printf("\nLO");
  for (int i = 0; i < p; i++) printf(" %.17g", pk[NT][i] >= 0 ? margin95(ml[NT].data(), pk[NT].data(), i, 0) : NAN);
  printf("\nHI");
  for (int i = 0; i < p; i++) printf(" %.17g", pk[NT][i] >= 0 ? margin95(ml[NT].data(), pk[NT].data(), i, 1) : NAN);
  printf("\n");
  if (nt) {
    marginalopt_popmig(0, genealogiessaved, pml[NT].data(), ppk[NT].data(), mpop.data(), mterm.data());
    for (j = 0; j <= NT; j++) {
      printf("PML %d", j);
      for (int t = 0; t < nt; t++) printf(" %.17g", pml[j][t]);
      printf("\nPPK %d", j);
      for (int t = 0; t < nt; t++) printf(" %.17g", ppk[j][t]);
      printf("\n");
    }
    printf("PT");
    for (int t = 0; t < nt; t++) {
      double maxp = -marginpopmig(mterm[t], 0, genealogiessaved, ppk[NT][t], mpop[t]);
      double max0p = -marginpopmig(mterm[t], 0, genealogiessaved, MINPARAMVAL, mpop[t]);
      printf(" %.17g", 2 * log(maxp / max0p));
    }
    printf("\n");
  }
}

/* TW: npops nchains nloci expo nomig treestring thetaprior mprior
 *     per locus: numgenes hval samppop[npops]
 *     per chain: tvals[npops-1]
 *     per chain, per locus: nlines up0[] up1[] down[] time[] pop[], then per
 *       node: nm {mt mp}*nm
 *   -> "PARAMS np nm", "TH i n {p r}*n max min", "MG i n {p r c}*n max min mean",
 *      per chain·locus "GW ci li mignum length tlength cc.. hcc.. fc.. mc.. fm..",
 *      per chain "PG ci probg q.. m.."
 * treeweight (update_gtree_common.cpp:1680-1937) per chain·locus, summed per
 * chain by sum_treeinfo (ginfo.cpp:209) in locus order, then
 * initialize_integrate_tree_prob (:2089-2134), as finish_setup_C does. */
extern "C" void init_gtreecommon(void);  /* C linkage, as update_gtree_common.hpp declares it */
/* IP: npops treestring flags[8] thetaprior mprior varrank[npops]
 *   flags: PARAMETERSBYPERIOD ANCESTRALPOPSIZESSETTOLARGESTSAMPLED
 *          ONEMIGRATIONPARAMETER MIGRATIONBETWEENSAMPLED NOMIGBETWEENNONSISTERS
 *          SINGLEMIGRATIONBOTHDIRECTIONS NOMIGRATION EXPOMIGRATIONPRIOR
 *   -> "PARAMS np nm", "TH i str b e n {p r}*n max min",
 *      "MG i str b e n {p r c}*n max min mean", "CHK n {p r c}*n"
 * setup_iparams (initialize.cpp:202-727) and set_nomigrationchecklist
 * (:761-809) on the population tree of chain 0, without a prior file. */
static void run_iparams()
{
  int npp = rd_i();
  char treestr[POPTREESTRINGLENGTHMAX];
  if (fscanf(g_in, "%255s", treestr) != 1) { fprintf(stderr, "short input\n"); exit(3); }
  const int opt[8] = {PARAMETERSBYPERIOD, ANCESTRALPOPSIZESSETTOLARGESTSAMPLED, ONEMIGRATIONPARAMETER,
                      MIGRATIONBETWEENSAMPLED, NOMIGBETWEENNONSISTERS, SINGLEMIGRATIONBOTHDIRECTIONS, NOMIGRATION,
                      EXPOMIGRATIONPRIOR};
  for (int k = 0; k < 8; k++) modeloptions[opt[k]] = rd_i();
  thetaprior = rd_d();
  mprior = rd_d();
  npops = npp;
  numtreepops = 2 * npops - 1;
  lastperiodnumber = numsplittimes = npops - 1;
  double vr[MAXPOPS];
  for (int p = 0; p < npops; p++) vr[p] = rd_d();
  refacc_set_varrank(vr, npops);
  alloc_chains(1, 1);
  setup_poptree(0, treestr);
  refacc_setup_iparams();
  refacc_set_nomigrationchecklist();
  printf("PARAMS %d %d\n", numpopsizeparams, nummigrateparams);
  for (int i = 0; i < numpopsizeparams; i++) {
    printf("TH %d %s %d %d %d", i, itheta[i].str, itheta[i].b, itheta[i].e, itheta[i].wp.n);
    for (int j = 0; j < itheta[i].wp.n; j++) printf(" %d %d", itheta[i].wp.p[j], itheta[i].wp.r[j]);
    printf(" %.17g %.17g\n", itheta[i].pr.max, itheta[i].pr.min);
  }
  for (int i = 0; i < nummigrateparams; i++) {
    printf("MG %d %s %d %d %d", i, imig[i].str, imig[i].b, imig[i].e, imig[i].wp.n);
    for (int j = 0; j < imig[i].wp.n; j++) printf(" %d %d %d", imig[i].wp.p[j], imig[i].wp.r[j], imig[i].wp.c[j]);
    printf(" %.17g %.17g %.17g\n", imig[i].pr.max, imig[i].pr.min, imig[i].pr.mean);
  }
  printf("CHK %d", nomigrationchecklist.n);
  for (int j = 0; j < nomigrationchecklist.n; j++)
    printf(" %d %d %d", nomigrationchecklist.p[j], nomigrationchecklist.r[j], nomigrationchecklist.c[j]);
  printf("\n");
}

static void run_tw()
{
  int npp = rd_i(), nch = rd_i(), nl = rd_i(), expo = rd_i(), nomig = rd_i();
  char treestr[POPTREESTRINGLENGTHMAX];
  if (fscanf(g_in, "%255s", treestr) != 1) { fprintf(stderr, "short input\n"); exit(3); }
  thetaprior = rd_d();
  mprior = rd_d();
  npops = npp;
  numtreepops = 2 * npops - 1;
  lastperiodnumber = numsplittimes = npops - 1;
  modeloptions[EXPOMIGRATIONPRIOR] = expo;
  modeloptions[NOMIGRATION] = nomig;
  alloc_chains(nch, nl);
  for (int li = 0; li < nl; li++) {
    L[li].numgenes = rd_i();
    L[li].hval = rd_d();
    for (int p = 0; p < npops; p++) L[li].samppop[p] = rd_i();
  }
  setlogfact();
  init_gtreecommon();
  init_treeweight();
  for (int ci = 0; ci < nch; ci++) {
    setup_poptree(ci, treestr);
    C[ci]->tvals = (double *)calloc((size_t)npops, sizeof(double));
    for (int k = 0; k < npops - 1; k++) C[ci]->tvals[k] = rd_d();
  }
  refacc_setup_iparams();
  printf("PARAMS %d %d\n", numpopsizeparams, nummigrateparams);
  for (int i = 0; i < numpopsizeparams; i++) {
    printf("TH %d %d", i, itheta[i].wp.n);
    for (int j = 0; j < itheta[i].wp.n; j++) printf(" %d %d", itheta[i].wp.p[j], itheta[i].wp.r[j]);
    printf(" %.17g %.17g\n", itheta[i].pr.max, itheta[i].pr.min);
  }
  for (int i = 0; i < nummigrateparams; i++) {
    printf("MG %d %d", i, imig[i].wp.n);
    for (int j = 0; j < imig[i].wp.n; j++) printf(" %d %d %d", imig[i].wp.p[j], imig[i].wp.r[j], imig[i].wp.c[j]);
    printf(" %.17g %.17g %.17g\n", imig[i].pr.max, imig[i].pr.min, imig[i].pr.mean);
  }
  for (int ci = 0; ci < nch; ci++) {
    init_genealogy_weights(&C[ci]->allgweight);
    init_probcalc(&C[ci]->allpcalc);
    for (int li = 0; li < nl; li++) {
      int nlines = rd_i();
      struct genealogy *G = &C[ci]->G[li];
      G->gtree = alloc_tree(nlines);
      read_tree(G->gtree, nlines);
      for (int i = 0; i < nlines; i++) G->gtree[i].pop = rd_i();
      for (int i = 0; i < nlines; i++) {
        int nm = rd_i();
        G->gtree[i].mig = (struct migstruct *)calloc((size_t)nm + 1, sizeof(struct migstruct));
        for (int j = 0; j < nm; j++) {
          G->gtree[i].mig[j].mt = rd_d();
          G->gtree[i].mig[j].mp = rd_i();
        }
        G->gtree[i].mig[nm].mt = -1.0;
      }
      G->root = find_root(G->gtree, nlines);
      G->roottime = G->gtree[G->gtree[G->root].up[0]].time;
      init_genealogy_weights(&G->gweight);
      treeweight(ci, li);
      sum_treeinfo(&C[ci]->allgweight, &G->gweight);
      struct genealogy_weights *w = &G->gweight;
      printf("GW %d %d %d %.17g %.17g", ci, li, G->mignum, G->length, G->tlength);
      for (int k = 0; k < npops; k++) for (int i = 0; i < npops - k; i++) printf(" %d", w->cc[k][i]);
      for (int k = 0; k < npops; k++) for (int i = 0; i < npops - k; i++) printf(" %.17g", w->hcc[k][i]);
      for (int k = 0; k < npops; k++) for (int i = 0; i < npops - k; i++) printf(" %.17g", w->fc[k][i]);
      if (!nomig) {
        for (int k = 0; k < lastperiodnumber; k++)
          for (int i = 0; i < npops - k; i++) for (int j = 0; j < npops - k; j++) printf(" %d", w->mc[k][i][j]);
        for (int k = 0; k < lastperiodnumber; k++)
          for (int i = 0; i < npops - k; i++) for (int j = 0; j < npops - k; j++) printf(" %.17g", w->fm[k][i][j]);
      }
      printf("\n");
    }
    total_numgenes = 0;
    for (int li = 0; li < nl; li++) total_numgenes += L[li].numgenes;
    initialize_integrate_tree_prob(ci, &C[ci]->allgweight, &C[ci]->allpcalc);
    printf("PG %d %.17g", ci, C[ci]->allpcalc.probg);
    for (int i = 0; i < numpopsizeparams; i++) printf(" %.17g", C[ci]->allpcalc.qintegrate[i]);
    if (!nomig)
      for (int i = 0; i < nummigrateparams; i++) printf(" %.17g", C[ci]->allpcalc.mintegrate[i]);
    printf("\n");
  }
}

/* RY: npops nchains nloci seed nsteps expo treestring thetaprior mprior
 *     per period k: tmin tmax                         (T[k].pr)
 *     per locus: numgenes hval samppop[npops] u numsites seq[numgenes*numsites]
 *     per chain: tvals[npops-1] beta
 *     per chain, per locus: nlines up0[] up1[] down[] time[] pop[], then per
 *       node: nm {mt mp}*nm
 *     per step: ci period
 *   -> per step "STEP accepted tval probg pdg", then per chain-locus
 *      "TIMES ci li time[nlines]" and "MIGT ci li mt..." (all events in
 *      node order)
 * The split-time update changet_RY1 (update_t_RY.cpp:223-518) on infinite-
 * sites loci, after the chain state is set up as finish_setup_C does it
 * (treeweight, likelihoodIS, sum_treeinfo, initialize_integrate_tree_prob). */
static void run_ry()
{
  int npp = rd_i(), nch = rd_i(), nl = rd_i(), seed = rd_i(), nsteps = rd_i(), expo = rd_i();
  char treestr[POPTREESTRINGLENGTHMAX];
  if (fscanf(g_in, "%255s", treestr) != 1) { fprintf(stderr, "short input\n"); exit(3); }
  thetaprior = rd_d();
  mprior = rd_d();
  npops = npp;
  numtreepops = 2 * npops - 1;
  lastperiodnumber = numsplittimes = npops - 1;
  modeloptions[EXPOMIGRATIONPRIOR] = expo;
  gbeta = 1.0;
  T = (struct chainstate_record_updates_and_values *)calloc((size_t)lastperiodnumber, sizeof(*T));
  for (int k = 0; k < lastperiodnumber; k++) {
    T[k].pr.min = rd_d();
    T[k].pr.max = rd_d();
  }
  alloc_chains(nch, nl);
  nurates = nl;
  std::vector<double> us(nl);
  std::vector<std::vector<int>> seqs(nl);
  for (int li = 0; li < nl; li++) {
    L[li].numgenes = rd_i();
    L[li].numlines = 2 * L[li].numgenes - 1;
    L[li].hval = rd_d();
    for (int p = 0; p < npops; p++) L[li].samppop[p] = rd_i();
    us[li] = rd_d();
    L[li].numsites = rd_i();
    L[li].model = INFINITESITES;
    L[li].nlinked = 1;
    L[li].uii[0] = li;
    seqs[li].resize((size_t)L[li].numgenes * L[li].numsites);
    for (auto &v : seqs[li]) v = rd_i();
    L[li].seq = (int **)malloc(sizeof(int *) * L[li].numgenes);
    for (int i = 0; i < L[li].numgenes; i++) L[li].seq[i] = &seqs[li][(size_t)i * L[li].numsites];
  }
  total_numgenes = 0;
  for (int li = 0; li < nl; li++) total_numgenes += L[li].numgenes;
  setlogfact();
  init_gtreecommon();
  init_treeweight();
  for (int ci = 0; ci < nch; ci++) {
    setup_poptree(ci, treestr);
    C[ci]->tvals = (double *)calloc((size_t)npops, sizeof(double));
    for (int k = 0; k < npops - 1; k++) C[ci]->tvals[k] = rd_d();
    C[ci]->tvals[lastperiodnumber] = TIMEMAX;
    beta[ci] = rd_d();
  }
  refacc_setup_iparams();
  for (int ci = 0; ci < nch; ci++) {
    init_genealogy_weights(&C[ci]->allgweight);
    init_probcalc(&C[ci]->allpcalc);
    C[ci]->allpcalc.pdg = 0;
    for (int li = 0; li < nl; li++) {
      int nlines = rd_i();
      struct genealogy *G = &C[ci]->G[li];
      G->gtree = alloc_tree(nlines);
      read_tree(G->gtree, nlines);
      for (int i = 0; i < nlines; i++) G->gtree[i].pop = rd_i();
      for (int i = 0; i < nlines; i++) {
        int nm = rd_i();
        G->gtree[i].mig = (struct migstruct *)calloc((size_t)ABSMIGMAX, sizeof(struct migstruct));
        for (int j = 0; j < nm; j++) {
          G->gtree[i].mig[j].mt = rd_d();
          G->gtree[i].mig[j].mp = rd_i();
        }
        G->gtree[i].mig[nm].mt = -1.0;
      }
      G->root = find_root(G->gtree, nlines);
      G->roottime = G->gtree[G->gtree[G->root].up[0]].time;
      G->uvals = (double *)malloc(sizeof(double));
      G->uvals[0] = us[li];
      G->pdg_a = (double *)malloc(sizeof(double));
      init_genealogy_weights(&G->gweight);
      treeweight(ci, li);
      sum_treeinfo(&C[ci]->allgweight, &G->gweight);
      G->pdg = G->pdg_a[0] = likelihoodIS(ci, li, us[li]);
      C[ci]->allpcalc.pdg += G->pdg;
    }
    initialize_integrate_tree_prob(ci, &C[ci]->allgweight, &C[ci]->allpcalc);
  }
  init_t_RY();
  setseeds(seed);
  for (int s = 0; s < nsteps; s++) {
    int ci = rd_i(), k = rd_i();
    int acc = changet_RY1(ci, k);
    printf("STEP %d %.17g %.17g %.17g\n", acc, C[ci]->tvals[k], C[ci]->allpcalc.probg, C[ci]->allpcalc.pdg);
  }
  for (int ci = 0; ci < nch; ci++)
    for (int li = 0; li < nl; li++) {
      struct genealogy *G = &C[ci]->G[li];
      printf("TIMES %d %d", ci, li);
      for (int i = 0; i < L[li].numlines; i++) printf(" %.17g", G->gtree[i].time);
      printf("\nMIGT %d %d", ci, li);
      for (int i = 0; i < L[li].numlines; i++)
        for (int j = 0; G->gtree[i].mig[j].mt > -0.5; j++) printf(" %.17g", G->gtree[i].mig[j].mt);
      printf("\n");
    }
}

/* UG: npops nchains nloci nsweeps treestring thetaprior
 *     per locus: model(0 IS, 1 HKY, 2 SW) numgenes hval samppop[npops] u, then
 *       IS/HKY: numsites seq[numgenes*numsites]; HKY adds totsites
 *       mult[numsites] pi[4] kappa; SW (one marker): minA maxA
 *     per chain: tvals[npops-1] beta seed
 *     per chain, per locus: nlines up0[] up1[] down[] time[] pop[], SW adds
 *       the alleles A[nlines]
 *   -> per proposal "UG ci li accepted topolchange tmrcachange pdg probg",
 *      then per chain-locus "TREE ci li" with up0[] up1[] down[] time[] pop[]
 * The genealogy update updategenealogy (update_gtree.cpp:723-966) of the
 * no-migration model (slider_nomigration, :79-254), after the chain state is
 * set up as finish_setup_C does it.  Each chain runs all its sweeps (every
 * locus in order per sweep) before the next chain, from setseeds(seed) of
 * its own: with an even number of proposals per chain, normdev's cached
 * second deviate (utilities.cpp:476-503) is spent before the next chain
 * starts, so every chain sees a generator of its own. */
static void run_ug()
{
  int npp = rd_i(), nch = rd_i(), nl = rd_i(), nsweeps = rd_i();
  char treestr[POPTREESTRINGLENGTHMAX];
  if (fscanf(g_in, "%255s", treestr) != 1) { fprintf(stderr, "short input\n"); exit(3); }
  thetaprior = rd_d();
  mprior = 0.0;
  npops = npp;
  numtreepops = 2 * npops - 1;
  lastperiodnumber = numsplittimes = npops - 1;
  modeloptions[NOMIGRATION] = 1;
  gbeta = 1.0;
  alloc_chains(nch, nl);
  nurates = nl;
  std::vector<double> us(nl), kappas(nl, 1.0);
  std::vector<std::vector<int>> seqs(nl), mults(nl);
  std::vector<std::array<double, 4>> pis(nl);
  for (int li = 0; li < nl; li++) {
    const int model = rd_i();
    L[li].numgenes = rd_i();
    L[li].numlines = 2 * L[li].numgenes - 1;
    L[li].hval = rd_d();
    for (int p = 0; p < npops; p++) L[li].samppop[p] = rd_i();
    us[li] = rd_d();
    L[li].nlinked = 1;
    L[li].uii[0] = li;
    if (model == 2) {
      L[li].model = STEPWISE;
      L[li].minA[0] = rd_i();
      L[li].maxA[0] = rd_i();
      somestepwise = 1;
      continue;
    }
    L[li].numsites = rd_i();
    L[li].model = model == 1 ? HKY : INFINITESITES;
    seqs[li].resize((size_t)L[li].numgenes * L[li].numsites);
    for (auto &v : seqs[li]) v = rd_i();
    L[li].seq = (int **)malloc(sizeof(int *) * L[li].numgenes);
    for (int i = 0; i < L[li].numgenes; i++) L[li].seq[i] = &seqs[li][(size_t)i * L[li].numsites];
    if (model == 1) {
      L[li].totsites = rd_i();
      mults[li].resize(L[li].numsites);
      for (auto &v : mults[li]) v = rd_i();
      L[li].mult = mults[li].data();
      for (int j = 0; j < 4; j++) pis[li][j] = rd_d();
      kappas[li] = rd_d();
    }
  }
  total_numgenes = 0;
  for (int li = 0; li < nl; li++) total_numgenes += L[li].numgenes;
  setlogfact();
  init_gtreecommon();
  init_treeweight();
  std::vector<int> seeds(nch);
  for (int ci = 0; ci < nch; ci++) {
    setup_poptree(ci, treestr);
    C[ci]->tvals = (double *)calloc((size_t)npops, sizeof(double));
    for (int k = 0; k < npops - 1; k++) C[ci]->tvals[k] = rd_d();
    C[ci]->tvals[lastperiodnumber] = TIMEMAX;
    beta[ci] = rd_d();
    seeds[ci] = rd_i();
  }
  refacc_setup_iparams();
  init_updategenealogy();  // its held probcalc is sized by setup_iparams' parameter counts
  for (int ci = 0; ci < nch; ci++) {
    init_genealogy_weights(&C[ci]->allgweight);
    init_probcalc(&C[ci]->allpcalc);
    C[ci]->allpcalc.pdg = 0;
    for (int li = 0; li < nl; li++) {
      int nlines = rd_i();
      struct genealogy *G = &C[ci]->G[li];
      G->gtree = alloc_tree(nlines);
      read_tree(G->gtree, nlines);
      for (int i = 0; i < nlines; i++) G->gtree[i].pop = rd_i();
      for (int i = 0; i < nlines; i++) {
        G->gtree[i].mig = (struct migstruct *)calloc((size_t)ABSMIGMAX, sizeof(struct migstruct));
        G->gtree[i].cmm = ABSMIGMAX;
        G->gtree[i].mig[0].mt = -1.0;
      }
      if (L[li].model == STEPWISE)
        for (int i = 0; i < nlines; i++) {
          G->gtree[i].A = (int *)calloc(MAXLINKED, sizeof(int));
          G->gtree[i].dlikeA = (double *)calloc(MAXLINKED, sizeof(double));
          G->gtree[i].A[0] = rd_i();
        }
      G->root = find_root(G->gtree, nlines);
      G->gtree[G->root].time = TIMEMAX;
      G->roottime = G->gtree[G->gtree[G->root].up[0]].time;
      G->uvals = (double *)malloc(sizeof(double));
      G->uvals[0] = us[li];
      G->pdg_a = (double *)malloc(sizeof(double));
      init_genealogy_weights(&G->gweight);
      treeweight(ci, li);
      sum_treeinfo(&C[ci]->allgweight, &G->gweight);
      if (L[li].model == STEPWISE) {
        G->pdg = G->pdg_a[0] = likelihoodSW(ci, li, 0, us[li], 1.0);
      } else if (L[li].model == HKY) {
        alloc_hky(G->gtree, L[li].numgenes, L[li].numsites);
        for (int j = 0; j < 4; j++) G->pi[j] = pis[li][j];
        G->kappaval = kappas[li];
        G->pdg = G->pdg_a[0] = likelihoodHKY(ci, li, us[li], kappas[li], -1, -1, -1, -1);
        copyfraclike(ci, li);
        storescalefactors(ci, li);
      } else {
        G->pdg = G->pdg_a[0] = likelihoodIS(ci, li, us[li]);
      }
      C[ci]->allpcalc.pdg += G->pdg;
    }
    initialize_integrate_tree_prob(ci, &C[ci]->allgweight, &C[ci]->allpcalc);
  }
  for (int ci = 0; ci < nch; ci++) {
    setseeds(seeds[ci]);
    for (int s = 0; s < nsweeps; s++)
      for (int li = 0; li < nl; li++) {
        int topol = 0, tmrca = 0;
        int acc = updategenealogy(ci, li, &topol, &tmrca);
        printf("UG %d %d %d %d %d %.17g %.17g\n", ci, li, acc, topol, tmrca, C[ci]->G[li].pdg,
               C[ci]->allpcalc.probg);
      }
  }
  for (int ci = 0; ci < nch; ci++)
    for (int li = 0; li < nl; li++) {
      const struct edge *t = C[ci]->G[li].gtree;
      printf("TREE %d %d", ci, li);
      for (int i = 0; i < L[li].numlines; i++) printf(" %d", t[i].up[0]);
      for (int i = 0; i < L[li].numlines; i++) printf(" %d", t[i].up[1]);
      for (int i = 0; i < L[li].numlines; i++) printf(" %d", t[i].down);
      for (int i = 0; i < L[li].numlines; i++) printf(" %.17g", t[i].time);
      for (int i = 0; i < L[li].numlines; i++) printf(" %d", t[i].pop);
      if (L[li].model == STEPWISE)
        for (int i = 0; i < L[li].numlines; i++) printf(" %d", t[i].A[0]);
      printf("\n");
    }
}

/* ITERM: n, then per line: kind(0 coal, 1 mig, 2 mig expo) c f h max min
 *   -> the reference integral term per line (update_gtree_common.cpp:108-304) */
static void run_iterm()
{
  setlogfact();
  int n = rd_i();
  for (int k = 0; k < n; k++) {
    int kind = rd_i(), c = rd_i();
    double f = rd_d(), h = rd_d(), mx = rd_d(), mn = rd_d();
    double v = kind == 0 ? refacc_icoal(c, f, h, mx, mn)
             : kind == 1 ? refacc_imig(c, f, mx, mn) : refacc_imig_expo(c, f, mx);
    printf("%.17g\n", v);
  }
}

int main(int argc, char **argv)
{
  if (argc != 3) { fprintf(stderr, "usage: imaref is|hky|sw|swap|jointp|de|margin|tw|iterm|ry|popmig|peaks|iparams|ug <input>\n"); return 2; }
  g_in = fopen(argv[2], "r");
  if (!g_in) { perror(argv[2]); return 2; }
  std::string mode = argv[1];
  if (mode == "is") run_is();
  else if (mode == "hky") run_hky();
  else if (mode == "sw") run_sw();
  else if (mode == "swap") run_swap();
  else if (mode == "jointp") run_jointp();
  else if (mode == "de") run_de();
  else if (mode == "margin") run_margin();
  else if (mode == "tw") run_tw();
  else if (mode == "iterm") run_iterm();
  else if (mode == "ry") run_ry();
  else if (mode == "popmig") run_popmig();
  else if (mode == "peaks") run_peaks();
  else if (mode == "iparams") run_iparams();
  else if (mode == "ug") run_ug();
  else { fprintf(stderr, "unknown mode\n"); return 2; }
  fclose(g_in);
  return 0;
}
