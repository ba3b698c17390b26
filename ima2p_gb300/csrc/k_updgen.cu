// k_updgen.cu -- the genealogy update of the no-migration model on the
// device: updategenealogy (update_gtree.cpp:723-966) with
// slider_nomigration (:79-254), findjointime (:34-77), joinsisdown
// (:375-455) and splitsisdown (:457-534).
//
// A step proposes a new genealogy for one locus of every listed chain.  The
// chains are independent (each draws from generators of its own), so they
// run in parallel, a warp each; the loci of a chain follow one another, as
// in qupdate.  The proposal stages the chain-locus's nodes, times and
// population labels in shared memory, and lane 0 runs the reference's
// sequential steps on them -- the edge and slide draws, the join, the slide
// (the reference's tail recursion as a loop), the split -- then the warp
// writes the proposed genealogy back with its level schedule and keeps the
// old one for a rejection.  The weights and the likelihood of the proposed
// genealogies run next as batches (k_treeweight, k_is / k_hky).  The
// decision adds the locus's new weights into the chain's sums
// (sum_subtract_treeinfo, ginfo.cpp:249-285), keeps the theta integrals
// whose count and length did not change (integrate_tree_prob,
// update_gtree_common.cpp:1945-2055), draws one uniform and commits or
// restores.  The file is compiled with -fmad=false: the reference's adds and
// multiplies round as written; log, exp and sqrt are the device's.
#include "internal.h"

#include <cfloat>

#include "igamma.cuh"
#include "ug_rng.cuh"

namespace {

constexpr double TIMEMAX = 1000000.0;        // imamp.hpp:129
constexpr double SLIDESTDVMAX = 20.0;        // update_gtree.cpp:686
constexpr double ONEOVERSQRT2PI = 0.3989422803;  // utilities.cpp:461, as the reference writes it
constexpr int SLIDE_MAX_STEPS = 1 << 20;     // a slide that long is an error, not a loop

// normdev (utilities.cpp:476-503): the polar method, keeping the second
// deviate for the next call
__device__ double normdev(LocalRng &r, double mean, double stdev)
{
  if (r.iset == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * uniform(r) - 1.0;
      v2 = 2.0 * uniform(r) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = sqrt(-2.0 * log(rsq) / rsq);
    r.gset = v1 * fac;
    r.iset = 1;
    return v2 * fac * stdev + mean;
  }
  r.iset = 0;
  return r.gset * stdev + mean;
}

__device__ double normprob(double mean, double stdev, double val)
{
  const double z = (val - mean) / stdev;
  const double sq = (z == 0.0) ? 0.0 : z * z;
  return ONEOVERSQRT2PI * exp(-sq / 2) / stdev;
}

__device__ double dmin(double a, double b) { return a < b ? a : b; }

// findperiod (update_gtree_common.cpp:1626-1636)
__device__ int findperiod(const double *tv, int nsplit, double t)
{
  int k = 0;
  while (k < nsplit && tv[k] <= t) k++;
  return k;
}

// findjointime (update_gtree.cpp:34-77): when the populations of the sliding
// edge and its sister come together
__device__ double findjointime(const TwModel &M, const double *tv, int nsplit, int slidepop, int sispop,
                               double edgeuptime, double sisuptime)
{
  int ep = findperiod(tv, nsplit, edgeuptime), sp = findperiod(tv, nsplit, sisuptime);
  while (ep < sp) {
    ep++;
    if (slidepop == M.droppops[ep][0] || slidepop == M.droppops[ep][1]) slidepop = M.pop_down[slidepop];
  }
  while (sp < ep) {
    sp++;
    if (sispop == M.droppops[sp][0] || sispop == M.droppops[sp][1]) sispop = M.pop_down[sispop];
  }
  while (slidepop != sispop && ep < nsplit) {
    ep++;
    if (slidepop == M.droppops[ep][0] || slidepop == M.droppops[ep][1]) slidepop = M.pop_down[slidepop];
    if (sispop == M.droppops[ep][0] || sispop == M.droppops[ep][1]) sispop = M.pop_down[sispop];
  }
  return ep == 0 ? 0.0 : tv[ep - 1];
}

struct UgSmem {
  uint32_t *mt;    // the chain's MT19937 words
  NodeRec *nd;
  double *t;
  int32_t *pop;
  int32_t *h;      // heights, then the level counts
  int16_t *sch;
};

__device__ UgSmem ug_carve(char *base, int maxn)
{
  const int maxnl = 2 * maxn - 1;
  UgSmem s;
  s.mt = reinterpret_cast<uint32_t *>(base);
  s.t = reinterpret_cast<double *>(base + 624 * 4);
  s.nd = reinterpret_cast<NodeRec *>(s.t + maxnl);
  s.pop = reinterpret_cast<int32_t *>(s.nd + maxnl);
  s.h = s.pop + maxnl;
  s.sch = reinterpret_cast<int16_t *>(s.h + maxnl + maxn + 2);
  return s;
}

// the generator's words [624]; times, nodes and labels [2n-1]; heights
// [2n-1] then level counts [n+2]; the schedule [2n]
size_t ug_smem(int maxn)
{
  const size_t maxnl = 2 * (size_t)maxn - 1;
  return 624 * 4 + maxnl * (8 + 8 + 4) + (maxnl + maxn + 2) * 4 + 2 * (size_t)maxn * 2 + 16;
}

__device__ void ug_fail(int32_t *err, int code, int who)
{
  if (atomicCAS(&err[0], 0, code) == 0) atomicExch(&err[1], who);
}

// One warp per listed chain: propose the locus's new genealogy.
__global__ void __launch_bounds__(32) k_ug_propose(UgArgs a)
{
  extern __shared__ __align__(16) char smem[];
  __shared__ int s_root;
  const int w = blockIdx.x, lane = threadIdx.x;
  const int ci = a.chains[w], item = ci * a.nloci + a.locus;
  const ItemDev it = a.items[item];
  const int n = it.n, nl = 2 * n - 1, maxnl = 2 * a.maxn;
  const size_t base = it.node_off;
  UgSmem s = ug_carve(smem, a.maxn);
  NodeRec *bkn = a.bk_nodes + (size_t)w * maxnl;
  double *bkt = a.bk_t + (size_t)w * maxnl;
  int32_t *bkp = a.bk_pop + (size_t)w * maxnl;
  int16_t *bks = a.bk_sched + (size_t)w * maxnl;
  for (int k = lane; k < nl; k += 32) {
    const NodeRec r = a.nodes[base + k];
    const double t = a.t64[base + k];
    const int32_t p = a.pop[base + k];
    s.nd[k] = r;
    s.t[k] = t;
    s.pop[k] = p;
    bkn[k] = r;
    bkt[k] = t;
    bkp[k] = p;
  }
  if (a.hky)
    for (int k = lane; k < 2 * n; k += 32) bks[k] = a.sched[it.sched_off + k];
  double *dl = nullptr;  // stepwise: the branch terms (joinsisdown and splitsisdown zero the new root's)
  if (a.sw) {
    const int32_t *A = a.alleles + it.al_off;
    dl = a.dlike + it.dl_off;
    int32_t *bka = a.bk_A + (size_t)w * maxnl;
    double *bkd = a.bk_dl + (size_t)w * maxnl;
    for (int k = lane; k < nl; k += 32) {
      bka[k] = A[k];
      bkd[k] = dl[k];
    }
  }
  if (lane == 0) {
    a.bk_len[w] = a.len[item];
    a.bk_nlev[w] = a.nlev[item];
  }
  LocalRng g;
  rng_load(g, a.rng + w, s.mt, lane);
  if (lane == 0) {
    const TwModel &M = *a.model;
    const double *tv = a.tvals + (size_t)ci * a.nsplit;
    NodeRec *nd = s.nd;
    double *t = s.t;
    int root = -1;
    for (int k = 0; k < nl; k++)
      if (nd[k].down == -1) root = k;
    if (root < n) {  // uploads are checked for one internal root; stop rather than read past the genealogy
      ug_fail(a.err, UG_E_TREE, w);
      root = nl - 1;
    }
    double roottime = t[nd[root].up0];
    // pick an edge that is not the root's
    int edge;
    do {
      edge = (int)floor(uniform(g) * nl);
    } while (nd[edge].down == -1);
    const int freed = nd[edge].down;
    const int oldsis = (nd[freed].up0 == edge) ? nd[freed].up1 : nd[freed].up0;
    double slidestdv = dmin(SLIDESTDVMAX, roottime / 3);
    const double hold = normdev(g, 0.0, slidestdv);
    double dist = hold;
    // joinsisdown: extend the sister over the freed edge
    int rootmove, tmrca = 0;
    {
      const int down = nd[oldsis].down;
      t[oldsis] = t[down];
      const int dd = nd[down].down;
      nd[oldsis].down = (int16_t)dd;
      if (dd != -1) {
        rootmove = 0;
        if (nd[dd].up0 == down) nd[dd].up0 = (int16_t)oldsis;
        else nd[dd].up1 = (int16_t)oldsis;
      } else {
        rootmove = 1;
        tmrca++;
        const double uptime = (oldsis < n) ? 0.0 : t[nd[oldsis].up0];
        root = oldsis;
        nd[oldsis].down = -1;
        t[oldsis] = TIMEMAX;
        if (dl) dl[oldsis] = 0.0;
        roottime = uptime;
      }
    }
    // slider_nomigration: move the edge's bottom `dist` through the genealogy
    int sis = oldsis, steps = 0;
    double tp = t[edge];
    bool ok = true;
    for (;;) {
      if (++steps > SLIDE_MAX_STEPS) {
        ok = false;
        break;
      }
      if (dist < 0) {  // up
        dist = -dist;
        const double edgeuptime = (edge < n) ? 0.0 : t[nd[edge].up0];
        const double sisuptime = (sis < n) ? 0.0 : t[nd[sis].up0];
        const int slidepop = s.pop[edge], sispop = s.pop[sis];
        const double popjointime =
            (slidepop != sispop) ? findjointime(M, tv, a.nsplit, slidepop, sispop, edgeuptime, sisuptime) : 0.0;
        if (popjointime > edgeuptime && popjointime > sisuptime) {
          if (dist < tp - popjointime) {
            tp -= dist;
            dist = 0;
            break;
          }
          dist -= tp - popjointime;
          tp = popjointime;
        } else if (sisuptime == 0 || edgeuptime >= sisuptime) {
          if (dist < tp - edgeuptime) {
            tp -= dist;
            dist = 0;
            break;
          }
          dist -= tp - edgeuptime;
          tp = edgeuptime;
        } else {
          if (dist < tp - sisuptime) {
            tp -= dist;
            dist = 0;
            break;
          }
          dist -= tp - sisuptime;
          tp = sisuptime;
          sis = bitran(g) ? nd[sis].up0 : nd[sis].up1;
          dist = -dist;
        }
      } else {  // down
        if (nd[sis].down == -1 || tp + dist < t[sis]) {
          tp += dist;
          if (tp >= TIMEMAX) tp = TIMEMAX;
          dist = 0;
          break;
        }
        dist -= t[sis] - tp;
        tp = t[sis];
        if (bitran(g)) {
          sis = nd[sis].down;
        } else {
          const int d = nd[sis].down;
          sis = (nd[d].up0 == sis) ? nd[d].up1 : nd[d].up0;
          dist = -dist;
        }
      }
    }
    t[edge] = tp;
    const int newsis = sis;
    // splitsisdown: the freed edge becomes the new sister's lower part
    {
      const double curt = t[edge];
      t[freed] = t[newsis];
      t[newsis] = curt;
      const int dd = nd[newsis].down;
      if (dd != -1) {
        if (nd[dd].up0 == newsis) nd[dd].up0 = (int16_t)freed;
        else nd[dd].up1 = (int16_t)freed;
      } else {
        root = freed;
        roottime = curt;
        rootmove = 1;
        if (roottime > TIMEMAX) ok = false;
        if (dl) dl[freed] = 0.0;
      }
      nd[freed].down = (int16_t)dd;
      int nowpop = s.pop[newsis];
      const int j = findperiod(tv, a.nsplit, curt);
      while (M.pop_e[nowpop] <= j && M.pop_e[nowpop] != -1) nowpop = M.pop_down[nowpop];
      s.pop[freed] = nowpop;
      nd[newsis].down = (int16_t)freed;
      nd[edge].down = (int16_t)freed;
      nd[freed].up0 = (int16_t)newsis;
      nd[freed].up1 = (int16_t)edge;
    }
    double sw = 0.0;
    if (rootmove) {
      sw = -log(normprob(0.0, slidestdv, hold));
      slidestdv = dmin(SLIDESTDVMAX, roottime / 3);
      sw += log(normprob(0.0, slidestdv, hold));
    }
    if (!ok) ug_fail(a.err, steps > SLIDE_MAX_STEPS ? UG_E_SLIDE : UG_E_ROOTTIME, w);
    a.slidew[w] = sw;
    a.prop[2 * w] = (oldsis != newsis);
    a.prop[2 * w + 1] = tmrca;
    if (a.hky) {  // the edited edges, as likelihoodHKY takes them
      ReqDev &R = a.req[a.req_of[w]];
      R.e[0] = edge;
      R.e[1] = freed;
      R.e[2] = oldsis;
      R.e[3] = newsis;
    }
    int32_t *eo = a.edges + 4 * (size_t)w;
    eo[0] = edge;
    eo[1] = freed;
    eo[2] = oldsis;
    eo[3] = newsis;
    if (a.sw) {
      // finishSWupdateA's allele draw (update_gtree_common.cpp:2219-2362):
      // a geometric step whose parameter comes from the freed node's
      // neighbours' distances, signed by bitran, clamped to the locus's
      // range.  k_ug_sw forms the branch terms from the result.
      int32_t *A = a.alleles + it.al_off;
      const int oldA = A[freed];
      const int e3[3] = {edge, newsis, nd[edge].down};
      int wsumdiff = 0, j = 0;
      for (int i = 0; i < 3; i++)
        if (nd[e3[i]].down != -1) {
          wsumdiff += abs((i < 2 ? A[e3[i]] : A[nd[e3[i]].down]) - oldA);
          j++;
        }
      double geo = j / ((double)(wsumdiff + j));
      if (geo > 0.95) geo = 0.95;
      int dA = (int)ceil(log(uniform(g)) / log(1.0 - geo)) - 1;  // geometric(), utilities.cpp:609-617
      if (bitran(g)) dA = -dA;
      const int minA = a.arange[2 * a.locus], maxA = a.arange[2 * a.locus + 1];
      if (dA >= 0) A[freed] = (maxA < oldA + dA) ? maxA : oldA + dA;
      else A[freed] = (minA > oldA + dA) ? minA : oldA + dA;
    }
    // the acceptance uniform, next in the stream (after a stepwise locus's
    // allele draw)
    if (a.predraw) a.ustore[w] = uniform(g);
    s_root = root;
  }
  __syncwarp();
  rng_store(g, a.rng + w, lane);
  if (a.hky) {
    // heights (tips 0, a node one above its higher daughter) by rounds of
    // relaxation over the internal nodes: heights only grow, towards the
    // true ones, and a round that changes nothing ends it (at most n)
    int32_t *h = s.h;
    for (int k = lane; k < nl; k += 32) h[k] = 0;
    __syncwarp();
    bool done = false;
    for (int round = 0; round <= n && !done; round++) {
      bool changed = false;
      for (int k = n + lane; k < nl; k += 32) {
        const int ha = h[s.nd[k].up0], hb = h[s.nd[k].up1];
        const int v = 1 + (ha > hb ? ha : hb);
        if (v != h[k]) {
          h[k] = v;
          changed = true;
        }
      }
      done = !__any_sync(~0u, changed);
    }
    __syncwarp();
    int H = h[s_root];
    if (!done || H < 1 || H > n - 1) {
      if (lane == 0) ug_fail(a.err, UG_E_TREE, w);
      H = 1;
      __syncwarp();
      for (int k = n + lane; k < nl; k += 32) h[k] = 1;
    }
    // the level schedule as the genealogy upload builds it: internal nodes
    // by height, in index order within a level
    int16_t *order = s.sch, *lstart = s.sch + (n - 1);
    int32_t *cnt = h + nl;  // H + 2 <= n + 1 entries past the heights
    for (int k = lane; k <= H + 1; k += 32) cnt[k] = 0;
    __syncwarp();
    for (int k = n + lane; k < nl; k += 32) atomicAdd(&cnt[h[k] + 1], 1);
    __syncwarp();
    if (lane == 0) {
      for (int k = 1; k <= H + 1; k++) {
        cnt[k] += cnt[k - 1];
        lstart[k - 1] = (int16_t)cnt[k];
      }
      a.nlev[item] = H;
    }
    __syncwarp();
    for (int b0 = n; b0 < nl; b0 += 32) {
      const int k = b0 + lane;
      const int hk = k < nl ? h[k] : -1;
      const unsigned peers = __match_any_sync(~0u, hk);
      const int rank = __popc(peers & ((1u << lane) - 1u));
      if (k < nl) order[cnt[hk] + rank] = (int16_t)k;
      __syncwarp();
      if (k < nl && rank == 0) cnt[hk] += __popc(peers);
      __syncwarp();
    }
    __syncwarp();
    for (int k = lane; k < n + H; k += 32) a.sched[it.sched_off + k] = s.sch[k];  // order, then level starts
  }
  for (int k = lane; k < nl; k += 32) {
    a.nodes[base + k] = s.nd[k];
    const double t = s.t[k];
    a.t64[base + k] = t;
    const float hi = (float)t;
    a.tff[base + k] = make_float2(hi, (float)(t - (double)hi));
    a.pop[base + k] = s.pop[k];
  }
  if (lane == 0) a.is_valid[item] = 0;  // the IS site labels follow daughter order, which moved
}

// One warp per listed chain: the Metropolis-Hastings decision, then commit
// or restore.
__global__ void __launch_bounds__(32) k_ug_decide(UgArgs a)
{
  __shared__ int32_t s_cn[TW_MAXT], s_c0[TW_MAXT];
  __shared__ double s_fn[TW_MAXT], s_f0[TW_MAXT], s_hn[TW_MAXT];
  __shared__ double s_q[TW_MAXTH];
  __shared__ int s_acc;
  const int w = blockIdx.x, lane = threadIdx.x;
  const int ci = a.chains[w], item = ci * a.nloci + a.locus;
  const ItemDev it = a.items[item];
  const int n = it.n, nl = 2 * n - 1, maxnl = 2 * a.maxn;
  const TwModel &M = *a.model;
  const int T = M.T, nth = M.nth;
  const int k = a.sw ? 0 : a.req_of[w];
  const int code = a.sw ? IMA_EVAL_OK : a.st[k];
  const double pdgnew = a.sw ? a.swnew[w] : a.res[k];
  const double aterm = a.sw ? a.aterm[w] : 0.0;
  const bool rejectIS = !a.hky && code == IMA_EVAL_IS_REJECT;
  const bool failed = (!a.hky && code == IMA_EVAL_IS_FAIL) || a.err[0] != 0;
  if (!rejectIS && !failed) {
    // sum_subtract_treeinfo: the chain's sums plus the new weights minus the old
    for (int q = lane; q < T; q += 32) {
      const size_t ic = (size_t)item * T + q, gc = (size_t)w * T + q;
      const int c0 = a.ag_cc[gc];
      double f = a.ag_fc[gc], hh = a.ag_hcc[gc];
      s_c0[q] = c0;
      s_f0[q] = f;
      s_cn[q] = c0 + (a.ncc[ic] - a.cc[ic]);
      f -= a.fc[ic];
      f += a.nfc[ic];
      s_fn[q] = (0 > f) ? 0.0 : f;
      hh -= a.hcc[ic];
      hh += a.nhcc[ic];
      s_hn[q] = hh;
    }
  }
  __syncwarp();
  // the theta integrals, a lane each: count and length summed over the
  // parameter's cells in order, the last accepted value kept when neither
  // changed (integrate_tree_prob)
  const bool decide = !rejectIS && !failed;
  if (decide)
    for (int i = lane; i < nth; i += 32) {
      int c = 0, holdc = 0;
      double f = 0.0, holdf = 0.0, hc = 0.0;
      for (int j = M.th_off[i]; j < M.th_off[i + 1]; j++) {
        const int cell = M.th_idx[j];
        c += s_cn[cell];
        holdc += s_c0[cell];
        f += s_fn[cell];
        holdf += s_f0[cell];
        hc += s_hn[cell];
      }
      Ig ig{{a.logfact, 0}};
      s_q[i] = (c == holdc && f == holdf) ? a.qint[(size_t)w * nth + i]
                                          : ig.coal(c, f, hc, M.th_max[i], M.th_min[i]);
      if (ig.st) ug_fail(a.err, UG_E_TERM, w);
    }
  // the acceptance uniform: one word of the chain's MT19937, or the whole
  // state staged for a twist
  int mti = 0;
  if (decide && !a.predraw) mti = a.rng[w].mt.mti;
  const bool stage = decide && !a.predraw && mti >= 624;
  __shared__ __align__(16) uint32_t s_mt[624];  // read as 8-byte words
  LocalRng g{};
  if (stage) rng_load(g, a.rng + w, s_mt, lane);
  __syncwarp();
  if (lane == 0) {
    int acc = 0;
    if (failed) {
      if (!a.hky && code == IMA_EVAL_IS_FAIL) ug_fail(a.err, UG_E_ISFAIL, w);
    } else if (!rejectIS) {
      double psum = 0;
      for (int i = 0; i < nth; i++) psum += s_q[i];
      double tpw = -a.probg[ci];
      tpw += psum;
      double mh = tpw + a.gbeta * (pdgnew - a.pdg[item]);
      mh = exp(a.beta[ci] * mh + a.slidew[w] + aterm);
      double U;
      if (a.predraw) {
        U = a.ustore[w];
      } else if (stage) {
        U = uniform(g);
      } else {
        uint32_t y = a.rng[w].mt.mt[mti];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        U = ((double)y + 0.5) * (1.0 / 4294967296.0);
        a.rng[w].mt.mti = mti + 1;
      }
      acc = U < dmin(1.0, mh);
      if (acc) {
        a.probg[ci] = psum;
        a.pdg[item] = pdgnew;
      }
    }
    if (acc && a.nacc) {
      a.nacc[(size_t)w * a.nloci + a.locus]++;
      if (a.prop[2 * w]) a.ntopo[(size_t)w * a.nloci + a.locus]++;
    }
    s_acc = acc;
  }
  __syncwarp();
  if (stage) rng_store(g, a.rng + w, lane);
  const bool acc = s_acc != 0;
  const size_t base = it.node_off;
  if (acc) {
    for (int i = lane; i < nth; i += 32) a.qint[(size_t)w * nth + i] = s_q[i];
    for (int q = lane; q < T; q += 32) {
      const size_t ic = (size_t)item * T + q, gc = (size_t)w * T + q;
      a.ag_cc[gc] = s_cn[q];
      a.ag_fc[gc] = s_fn[q];
      a.ag_hcc[gc] = s_hn[q];
      a.cc[ic] = a.ncc[ic];
      a.fc[ic] = a.nfc[ic];
      a.hcc[ic] = a.nhcc[ic];
    }
  } else {  // restoreedges, storegenealogystats(..., 1)
    const NodeRec *bkn = a.bk_nodes + (size_t)w * maxnl;
    const double *bkt = a.bk_t + (size_t)w * maxnl;
    const int32_t *bkp = a.bk_pop + (size_t)w * maxnl;
    const int16_t *bks = a.bk_sched + (size_t)w * maxnl;
    for (int j = lane; j < nl; j += 32) {
      a.nodes[base + j] = bkn[j];
      const double t = bkt[j];
      a.t64[base + j] = t;
      const float hi = (float)t;
      a.tff[base + j] = make_float2(hi, (float)(t - (double)hi));
      a.pop[base + j] = bkp[j];
    }
    if (a.hky)
      for (int j = lane; j < 2 * n; j += 32) a.sched[it.sched_off + j] = bks[j];
    if (lane == 0) {
      a.len[item] = a.bk_len[w];
      a.nlev[item] = a.bk_nlev[w];
      a.is_valid[item] = 0;  // the site labels cached by the evaluation are the proposal's
      if (a.sw) {  // restoreedges: the three moved edges from their copies, the new sister only if nonzero
        const int32_t *eo = a.edges + 4 * (size_t)w;
        const int edge = eo[0], freed = eo[1], oldsis = eo[2], newsis = eo[3];
        const int32_t *bka = a.bk_A + (size_t)w * maxnl;
        const double *bkd = a.bk_dl + (size_t)w * maxnl;
        double *dl = a.dlike + it.dl_off;
        a.alleles[it.al_off + freed] = bka[freed];
        dl[edge] = bkd[edge];
        dl[oldsis] = bkd[oldsis];
        dl[freed] = bkn[freed].down != -1 ? bkd[freed] : 0.0;
        const double hs = a.holdsis[w];
        if (hs != 0) dl[newsis] = hs;
      }
    }
  }
  if (a.hky)  // copyfraclike / restorescalefactors: the recomputed nodes' slots
    for (int j = lane; j < nl; j += 32) {
      const size_t g = base + j;
      if (a.fresh32[g]) {
        if (acc) a.slot32[g] ^= 1;
        a.fresh32[g] = 0;
      }
      if (a.slot64 && a.fresh64[g]) {
        if (acc) a.slot64[g] ^= 1;
        a.fresh64[g] = 0;
      }
    }
}

}  // namespace

void launch_ug_propose(const UgArgs &a, cudaStream_t st)
{
  k_ug_propose<<<a.nch, 32, ug_smem(a.maxn), st>>>(a);
}

void launch_ug_decide(const UgArgs &a, cudaStream_t st) { k_ug_decide<<<a.nch, 32, 0, st>>>(a); }

extern "C" void ima_ug_rng_seed(ima_ug_rng *g, int32_t seed)
{
  if (!g) return;
  ima_mt19937_seed(&g->mt, (uint32_t)seed);
  g->iset = 0;
  g->gset = 0.0;
  g->iseed = 0x7fffffffffffffffull + (uint64_t)(int64_t)seed;
}
