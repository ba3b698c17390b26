// k_treeweight.cu -- genealogy weights and p(G) integrals on the device.
//
// k_treeweight restates treeweight (update_gtree_common.cpp:1680-1937) with
// a group of lanes per genealogy (as many as the populations, rounded up to
// a power of two: 4 lanes for 3 populations, 8 genealogies per warp).  The
// group lays the genealogy's events out in shared memory -- a coalescence
// per internal node at its daughters' time, every migration with the
// population it leaves (the edge's population carried through the splits,
// :1770-1790) and every split younger than the root -- sorts them by (time,
// position) with a bitonic network and sweeps them in time order.  Lane l of
// the group owns population l of the current period: its lineage count, its
// fc accumulator (n(n-1) dt / 2h) and its fm accumulator (n dt; the
// reference adds the same n dt to every partner cell, :1861-1867).  At a
// split the lanes flush their period and take the counts of their new
// population from the daughters' lanes by shuffle.  Every accumulator
// receives the reference's terms in the reference's order, so with FMA
// contraction off (this file is compiled with -fmad=false) the weights are
// the reference's bit for bit.  The sweep is FP64-issue bound (GB300 runs
// FP64 at 1/64 of the FP32 rate), which is why genealogies share warps
// rather than each taking a warp of mostly idle lanes.
//
// k_tp_params / k_tp_final restate sum_treeinfo (ginfo.cpp:209-244) over a
// chain's loci in locus order, initialize_integrate_tree_prob
// (update_gtree_common.cpp:2089-2134) with the integral terms (:108-304,
// MORESTABLE) on the reference's incomplete gamma functions
// (utilities.cpp:808-1130), and optionally savegsampinf (ginfo.cpp:318-377):
// a thread per (chain, weight cell) sums the cell over the chain's loci, a
// thread per (parameter, chain) evaluates the integral, then a thread per
// chain adds the integrals in parameter order.
// The integrals use the device's log/exp, so they agree with the host's to
// rounding, not bit for bit.
#include "internal.h"

#include <cfloat>

#include "igamma.cuh"

namespace {

constexpr int TW_WPB = 4;  // genealogies (warps) per block
enum { EV_COAL = 0, EV_MIG = 1, EV_SPLIT = 2, EV_PAD = 3 };
enum { TW_E_POP = 1, TW_E_COUNT = 2, TW_E_SIZE = 3, TW_E_TERM = 4, TW_E_LF = 5, TW_E_MIGOFF = 6 };
constexpr uint32_t POS_MASK = 0xFFFFFu;  // event position: 20 bits

__device__ __forceinline__ uint32_t ev_pack(int type, int pop, int topop, int pos)
{
  return ((uint32_t)type << 30) | ((uint32_t)(topop & 31) << 25) | ((uint32_t)(pop & 31) << 20) |
         ((uint32_t)pos & POS_MASK);
}

// findperiod (update_gtree_common.cpp:1626)
__device__ __forceinline__ int tw_period(const double *tv, int nsplit, double t)
{
  int k = 0;
  while (k < nsplit && tv[k] <= t) k++;
  return k;
}

__device__ void tw_fail(int32_t *err, int code, int who)
{
  if (atomicCAS(&err[0], 0, code) == 0) atomicExch(&err[1], who);
}

// Pass 1, one warp per genealogy: lay out the events in shared memory, sort
// them and write the sorted list to ev_t/ev_c at the genealogy's offset;
// ev_n[g] = the number of events, or -1 for a genealogy the model cannot hold.
__global__ void __launch_bounds__(32 * TW_WPB) k_tw_events(TwArgs a, int wpb)
{
  extern __shared__ __align__(16) unsigned char sm[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int slot = blockIdx.x * wpb + warp;
  if (slot >= a.ngen) return;  // whole warps only
  const int g = a.perm[slot];  // the selected genealogies, most events first
  const TwModel &M = *a.model;
  const int npops = M.npops, nsplit = npops - 1, ntp = 2 * npops - 1;
  unsigned char *base = sm + (size_t)warp * a.P * 12;
  double *ev_t = reinterpret_cast<double *>(base);
  uint32_t *ev_c = reinterpret_cast<uint32_t *>(base + (size_t)a.P * 8);

  const int a0 = a.node_off[g], nl = a.node_off[g + 1] - a0, ng = (nl + 1) >> 1;
  const double *tv = a.tvals + (size_t)a.gen_tv[g] * nsplit;
  const int32_t *up0 = a.nodes ? nullptr : a.up0 + a0, *pp = a.pop + a0;
  const int32_t *mo = a.mig_off + (a.moff_start ? a.moff_start[g] : a0);
  const long long mb = a.mbase ? a.mbase[g] : 0;
  const double *tm = a.time + a0;
  const int nmig = mo[nl] - mo[0];
  auto daughter = [&](int i) { return a.nodes ? (int)a.nodes[a0 + i].up0 : up0[i]; };

  // roottime: the root's coalescence, the latest one (times are >= 0, so
  // their bit patterns order as the values do)
  int bad = 0;
  long long rtb = 0;
  for (int i = ng + lane; i < nl; i += 32) {
    const int u = daughter(i);
    if ((unsigned)u >= (unsigned)nl) bad = TW_E_POP;
    else rtb = max(rtb, __double_as_longlong(tm[u]));
  }
  for (int d = 16; d; d >>= 1) rtb = max(rtb, __shfl_xor_sync(~0u, rtb, d));
  const int kroot = tw_period(tv, nsplit, __longlong_as_double(rtb));
  const int E = (ng - 1) + nmig + kroot;
  if (__any_sync(~0u, bad) || E > a.P || a.ev_off[g] + E > a.ev_off[g + 1]) {
    if (lane == 0) {
      a.ev_n[g] = -1;
      tw_fail(a.err, bad ? TW_E_POP : TW_E_SIZE, g);
    }
    return;
  }

  // events: node i's coalescence first, then its migrations in edge order
  int run = 0;
  for (int b0 = 0; b0 < nl; b0 += 32) {
    const int i = b0 + lane;
    int cnt = 0, m0 = 0, m1 = 0;
    if (i < nl) {
      m0 = mo[i];
      m1 = mo[i + 1];
      cnt = (i >= ng) + (m1 - m0);
    }
    int inc = cnt;
    for (int d = 1; d < 32; d <<= 1) {
      const int v = __shfl_up_sync(~0u, inc, d);
      if (lane >= d) inc += v;
    }
    int e = run + inc - cnt;
    run += __shfl_sync(~0u, inc, 31);
    if (i < nl) {
      int nowpop = pp[i];
      if (m1 < m0 || m0 < mo[0] || m1 > mo[nl]) {
        bad = TW_E_MIGOFF;  // checked before any migration is read
      } else if ((unsigned)nowpop >= (unsigned)ntp || e < 0 || e + cnt > E) {
        bad = TW_E_POP;
      } else {
        if (i >= ng) {
          ev_t[e] = tm[daughter(i)];
          ev_c[e] = ev_pack(EV_COAL, nowpop, 0, e);
          e++;
        }
        for (int j = m0; j < m1; j++) {
          const double t = a.mig_t[mb + j];
          const int per = tw_period(tv, nsplit, t);
          while (M.pop_e[nowpop] <= per && M.pop_e[nowpop] != -1) nowpop = M.pop_down[nowpop];
          const int to = a.mig_p[mb + j];
          if ((unsigned)to >= (unsigned)ntp || to == nowpop) {
            bad = TW_E_POP;
            break;
          }
          ev_t[e] = t;
          ev_c[e] = ev_pack(EV_MIG, nowpop, to, e);
          e++;
          nowpop = to;
        }
      }
    }
  }
  if (lane < kroot) {
    ev_t[run + lane] = tv[lane];
    ev_c[run + lane] = ev_pack(EV_SPLIT, 0, 0, run + lane);
  }
  int Pg = 1;
  while (Pg < E) Pg <<= 1;
  for (int i = E + lane; i < Pg; i += 32) {
    ev_t[i] = __longlong_as_double(0x7ff0000000000000LL);  // +inf: after every event
    ev_c[i] = ev_pack(EV_PAD, 0, 0, i);
  }
  if (__any_sync(~0u, bad)) {
    const int code = __reduce_max_sync(~0u, bad);
    if (lane == 0) {
      a.ev_n[g] = -1;
      tw_fail(a.err, code, g);
    }
    return;
  }
  __syncwarp();

  // bitonic sort on (time, position), compared as integers: the positions
  // are distinct, so the order is total and ties in time keep list order
  for (int size = 2; size <= Pg; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < (Pg >> 1); i += 32) {
        const int lo = ((i & ~(stride - 1)) << 1) | (i & (stride - 1));
        const int hi = lo + stride;
        const long long tl = __double_as_longlong(ev_t[lo]), th = __double_as_longlong(ev_t[hi]);
        const uint32_t cl = ev_c[lo], ch = ev_c[hi];
        const bool gt = tl > th || (tl == th && (cl & POS_MASK) > (ch & POS_MASK));
        if (gt == ((lo & size) == 0)) {
          ev_t[lo] = __longlong_as_double(th);
          ev_t[hi] = __longlong_as_double(tl);
          ev_c[lo] = ch;
          ev_c[hi] = cl;
        }
      }
      __syncwarp();
    }
  }
  const long long off = a.ev_off[g];
  for (int j = lane; j < E; j += 32) {
    a.ev_t[off + j] = ev_t[j];
    a.ev_c[off + j] = ev_c[j];
  }
  if (lane == 0) a.ev_n[g] = E;
}

// Pass 2, the sweep (update_gtree_common.cpp:1827-1927): one group of GW
// lanes per genealogy (GW = the smallest power of two >= npops), 32/GW
// genealogies per warp, taken in the order perm gives (most events first) so
// that a warp's groups sweep about as many events each.  Lane l of a group
// owns population l of the current period.
//
// With MERGE (npops < GW: a group lane without a population), lane npops
// carries G->length and G->tlength through the same two multiply-adds the
// population lanes use for fc and fm -- length += (nsum * dt) * 1.0 and
// tlength += nsum * d with d = dt before the last split, lastsplitt - lasttime
// across it and 0 after it, each factor exact -- so the FP64 pipe does 8
// operations per event instead of 12, with the reference's values.
template <int GW, bool MERGE>
__global__ void __launch_bounds__(32 * TW_WPB) k_tw_sweep(TwArgs a, int wpb, int gbytes)
{
  extern __shared__ __align__(16) unsigned char sm[];
  constexpr int GPW = 32 / GW;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int grp = lane / GW, gl = lane % GW;
  const unsigned gmask = GW == 32 ? 0xffffffffu : ((1u << GW) - 1) << (grp * GW);
  const int slot = (blockIdx.x * wpb + warp) * GPW + grp;
  if (slot >= a.ngen) return;  // whole groups only
  const int g = a.perm[slot];
  const int E = a.ev_n[g];
  if (E < 0) return;  // pass 1 rejected it
  const TwModel &M = *a.model;
  const int npops = M.npops, nsplit = npops - 1, T = M.T, MM = M.M;
  double *fc_s = reinterpret_cast<double *>(sm + (size_t)(warp * GPW + grp) * gbytes);
  double *fm_s = fc_s + T;
  int *cc_s = reinterpret_cast<int *>(fm_s + MM);
  int *mc_s = cc_s + T;
  for (int i = gl; i < T; i += GW) {
    fc_s[i] = 0.0;
    cc_s[i] = 0;
  }
  for (int i = gl; i < MM; i += GW) {
    fm_s[i] = 0.0;
    mc_s[i] = 0;
  }
  const int a0 = a.node_off[g], nl = a.node_off[g + 1] - a0, ng = (nl + 1) >> 1;
  const double *tv = a.tvals + (size_t)a.gen_tv[g] * nsplit;
  const int loc = a.gen_locus[g];
  const double *et = a.ev_t + a.ev_off[g];
  const uint32_t *ec = a.ev_c + a.ev_off[g];
  const double h2 = a.h2term[loc], hl = a.hlog[loc];
  const double lastsplitt = tv[nsplit - 1];
  const long long lsb = __double_as_longlong(lastsplitt);  // times >= 0: compare bit patterns
  int k = 0, nsum = ng, nmine = gl < npops ? a.samppop[(size_t)loc * npops + gl] : 0, ccm = 0, bad = 0;
  double accfc = 0.0, accfm = 0.0, last = 0.0, len = 0.0, tlen = 0.0;
  __syncwarp(gmask);
  auto flush = [&](int kk) {
    const int w = npops - kk;
    if (gl < w && !(MERGE && gl == npops)) {
      fc_s[M.toff[kk] + gl] = accfc;
      cc_s[M.toff[kk] + gl] = ccm;
      if (!M.nomig && kk < nsplit)
        for (int jj = 0; jj < w; jj++)
          if (jj != gl) fm_s[M.moff[kk] + gl * w + jj] = accfm;
    }
  };
  const bool lenlane = MERGE && gl == npops;
  // one event: returns true when the genealogy is found bad
  auto event = [&](const double t, const uint32_t c) -> bool {
    const double dt = t - last;
    const bool before = __double_as_longlong(t) < lsb, lbefore = __double_as_longlong(last) < lsb;
    const int w = npops - k;
    if constexpr (MERGE) {
      // n(n-1) is exact in an int and in a double, so converting the
      // product equals the reference's (double)n * ((double)n - 1)
      if (gl < w || lenlane) {
        double d2;
        if (lenlane) {
          d2 = before ? dt : 0.0;
          if (!before && lbefore) d2 = lastsplitt - last;
        } else {
          d2 = (!M.nomig && k < nsplit) ? dt : 0.0;
        }
        const int x1 = lenlane ? nsum : nmine * (nmine - 1), x2 = lenlane ? nsum : nmine;
        accfc += (double)x1 * dt * (lenlane ? 1.0 : h2);  // lenlane: length
        accfm += (double)x2 * d2;                         // lenlane: tlength
      }
    } else {
      const double tadd = nsum * dt;
      len += tadd;
      if (before)
        tlen += tadd;
      else if (lbefore)
        tlen += nsum * (lastsplitt - last);
      if (gl < w) {
        accfc += (double)(nmine * (nmine - 1)) * dt * h2;
        if (!M.nomig && k < nsplit) accfm += nmine * dt;
      }
    }
    last = t;
    const int type = (int)(c >> 30);
    int lbad = 0;
    if (type == EV_COAL) {
      const int o = M.pos[k][(c >> 20) & 31];
      if (o < 0) {
        bad = TW_E_POP;
      } else if (gl == o) {
        lbad = nmine < 2;
        nmine--;
        ccm++;
      }
      nsum--;
    } else if (type == EV_MIG) {
      const int op = M.pos[k][(c >> 20) & 31], oq = M.pos[k][(c >> 25) & 31];
      if (op < 0 || oq < 0 || k >= nsplit) {
        bad = TW_E_POP;
      } else {
        if (gl == op) {
          lbad = nmine < 1;
          nmine--;
          mc_s[M.moff[k] + op * w + oq]++;
        }
        if (gl == oq) nmine++;
      }
    } else {  // a split: the period ends
      if (k >= nsplit || nsum < 2) {
        bad = TW_E_COUNT;
      } else {
        flush(k);
        const int k1 = k + 1;
        int s0 = 0, s1 = -1;
        if (gl < npops - k1) {
          const int np1 = M.plist[k1][gl];
          if (np1 == M.addpop[k1]) {
            s0 = M.pos[k][M.droppops[k1][0]];
            s1 = M.pos[k][M.droppops[k1][1]];
          } else {
            s0 = M.pos[k][np1];
          }
        }
        const int v0 = __shfl_sync(gmask, nmine, s0 < 0 ? 0 : s0, GW);
        const int v1 = __shfl_sync(gmask, nmine, s1 < 0 ? 0 : s1, GW);
        nmine = gl < npops - k1 ? v0 + (s1 >= 0 ? v1 : 0) : 0;
        k = k1;
        if (!lenlane) {
          accfc = accfm = 0.0;
          ccm = 0;
        }
      }
    }
    if (__any_sync(gmask, lbad)) bad = TW_E_COUNT;
    return bad != 0;
  };
  // events four at a time, the next four loaded while these are swept: the
  // sweep is a dependent chain, and one L2 round trip per event would set
  // its pace
  double q0 = 0.0, q1 = 0.0, q2 = 0.0, q3 = 0.0;
  uint32_t r0 = 0, r1 = 0, r2 = 0, r3 = 0;
  if (0 < E) { q0 = et[0]; r0 = ec[0]; }
  if (1 < E) { q1 = et[1]; r1 = ec[1]; }
  if (2 < E) { q2 = et[2]; r2 = ec[2]; }
  if (3 < E) { q3 = et[3]; r3 = ec[3]; }
  for (int j = 0; j < E; j += 4) {
    const double t0 = q0, t1 = q1, t2 = q2, t3 = q3;
    const uint32_t c0 = r0, c1 = r1, c2 = r2, c3 = r3;
    if (j + 4 < E) { q0 = et[j + 4]; r0 = ec[j + 4]; }
    if (j + 5 < E) { q1 = et[j + 5]; r1 = ec[j + 5]; }
    if (j + 6 < E) { q2 = et[j + 6]; r2 = ec[j + 6]; }
    if (j + 7 < E) { q3 = et[j + 7]; r3 = ec[j + 7]; }
    if (event(t0, c0)) break;
    if (j + 1 < E && event(t1, c1)) break;
    if (j + 2 < E && event(t2, c2)) break;
    if (j + 3 < E && event(t3, c3)) break;
  }
  if (!bad && nsum != 1) bad = TW_E_COUNT;
  if (bad) {
    if (gl == 0) tw_fail(a.err, bad, g);
    return;
  }
  flush(k);
  __syncwarp(gmask);
  if (lenlane) {
    len = accfc;
    tlen = accfm;
  }
  const size_t oT = (size_t)g * T, oM = (size_t)g * MM;
  for (int i = gl; i < T; i += GW) {
    a.cc[oT + i] = cc_s[i];
    a.fc[oT + i] = fc_s[i];
    a.hcc[oT + i] = hl != 0.0 ? 0.0 + hl * cc_s[i] : 0.0;
  }
  for (int i = gl; i < MM; i += GW) {
    a.mc[oM + i] = mc_s[i];
    a.fm[oM + i] = fm_s[i];
  }
  if (gl == (MERGE ? npops : 0)) {
    const int32_t *mo = a.mig_off + (a.moff_start ? a.moff_start[g] : a0);
    a.lens[2 * (size_t)g] = len;
    a.lens[2 * (size_t)g + 1] = tlen;
    a.mignum[g] = mo[nl] - mo[0];
    if (a.len_out) a.len_out[g] = len;
  }
}

// ---------------------------------------------------------------- p(G)
// The integral terms (Ig) are in igamma.cuh.

constexpr int TP_BS = 128;

// p(G) runs on the FP64 pipe, which GB300 issues at 1/64 of the FP32 rate:
// the work is packed densely into lanes so that every FP64 instruction
// carries 32 useful operations.
//
// Pass 1: a thread per (chain, summed quantity): the chain's weights added
// over its genealogies in order -- sum_treeinfo's order for that cell.
// Doubles (fc, hcc, fm cells) first, then the counts (cc, mc).
__global__ void __launch_bounds__(TP_BS) k_tp_cells(TwProbArgs a)
{
  const TwModel &M = *a.model;
  const int T = M.T, MM = M.nomig ? 0 : M.M;
  const int Qd = 2 * T + MM, Qi = T + MM;
  const long long tid = (long long)blockIdx.x * TP_BS + threadIdx.x;
  const long long nd = (long long)a.ngroups * Qd, ni = (long long)a.ngroups * Qi;
  if (tid < nd) {
    const int grp = (int)(tid / Qd), q = (int)(tid % Qd);
    const double *src;
    int stride;
    if (q < T) {
      src = a.fc + q;
      stride = T;
    } else if (q < 2 * T) {
      src = a.hcc + (q - T);
      stride = T;
    } else {
      src = a.fm + (q - 2 * T);
      stride = M.M;
    }
    double sum = 0.0;
    const int g1 = a.group_end ? a.group_end[grp] : a.group_off[grp + 1];
#pragma unroll 8
    for (int g = a.group_off[grp]; g < g1; g++) sum += src[(size_t)g * stride];
    a.sd[(size_t)grp * Qd + q] = sum;
  } else if (tid < nd + ni) {
    const long long t2 = tid - nd;
    const int grp = (int)(t2 / Qi), q = (int)(t2 % Qi);
    const int32_t *src = q < T ? a.cc + q : a.mc + (q - T);
    const int stride = q < T ? T : M.M;
    int sum = 0;
    const int g1 = a.group_end ? a.group_end[grp] : a.group_off[grp + 1];
#pragma unroll 8
    for (int g = a.group_off[grp]; g < g1; g++) sum += src[(size_t)g * stride];
    a.sc[(size_t)grp * Qi + q] = sum;
  }
}

// Pass 2: a thread per (parameter, chain), parameter-major so that a warp's
// lanes evaluate one parameter for 32 chains (similar arguments, similar
// series lengths): the cells added in the parameter's order, the integral,
// and the parameter's entries of the gsampinf row (float sums, as
// savegsampinf makes them).
__global__ void __launch_bounds__(TP_BS) k_tp_params(TwProbArgs a)
{
  const TwModel &M = *a.model;
  const int nth = M.nth, nmg = M.nomig ? 0 : M.nmg, G = a.ngroups;
  const int T = M.T, MM = M.nomig ? 0 : M.M, Qd = 2 * T + MM, Qi = T + MM;
  const long long tid = (long long)blockIdx.x * TP_BS + threadIdx.x;
  if (tid >= (long long)G * (nth + nmg)) return;
  const bool th = tid < (long long)G * nth;
  const long long t2 = th ? tid : tid - (long long)G * nth;
  const int i = (int)(t2 / G), grp = (int)(t2 % G);
  const double *sd = a.sd + (size_t)grp * Qd;
  const int32_t *sc = a.sc + (size_t)grp * Qi;
  int c = 0;
  double f = 0.0, hc = 0.0;
  float ff = 0.0f, hf = 0.0f;
  Ig ig{{a.logfact, 0}};
  double v;
  if (th) {
    for (int j = M.th_off[i]; j < M.th_off[i + 1]; j++) {
      const int cell = M.th_idx[j];
      c += sc[cell];
      f += sd[cell];
      hc += sd[T + cell];
      ff += (float)sd[cell];
      hf += (float)sd[T + cell];
    }
    v = ig.coal(c, f, hc, M.th_max[i], M.th_min[i]);
    a.q[(size_t)grp * nth + i] = v;
  } else {
    for (int j = M.mg_off[i]; j < M.mg_off[i + 1]; j++) {
      const int cell = M.mg_idx[j];
      c += sc[T + cell];
      f += sd[2 * T + cell];
      ff += (float)sd[2 * T + cell];
    }
    v = M.expo ? ig.mig_expo(c, f, M.mg_mean[i]) : ig.mig(c, f, M.mg_max[i], M.mg_min[i]);
    a.m[(size_t)grp * nmg + i] = v;
  }
  if (ig.st) tw_fail(a.err, ig.st, grp);
  if (a.rows) {  // ccp 0, fcp nth, hccp 2nth, mcp 3nth, fmp mcp+nmg, qip fmp+nmg, mip qip+nth
    float *row = a.rows + (size_t)grp * a.rowlen;
    if (th) {
      row[i] = (float)c;
      row[nth + i] = ff;
      row[2 * nth + i] = hf;
      row[3 * nth + 2 * nmg + i] = (float)v;
    } else {
      row[3 * nth + i] = (float)c;
      row[3 * nth + nmg + i] = ff;
      row[4 * nth + 2 * nmg + i] = (float)v;
    }
  }
}

// Pass 2 of p(G): one lane per chain.  probg = the integrals added in
// parameter order (initialize_integrate_tree_prob), or -DBL_MAX when a
// cell of nomigrationchecklist holds a migration; the rest of the row.
__global__ void __launch_bounds__(128) k_tp_final(TwProbArgs a)
{
  const int grp = blockIdx.x * blockDim.x + threadIdx.x;
  if (grp >= a.ngroups) return;
  const TwModel &M = *a.model;
  const int nth = M.nth, nmg = M.nomig ? 0 : M.nmg;
  bool checkm = true;
  if (!M.nomig)
    for (int i = 0; i < M.nchk && checkm; i++) {
      int cnt = 0;
      const int g1 = a.group_end ? a.group_end[grp] : a.group_off[grp + 1];
      for (int g = a.group_off[grp]; g < g1; g++) cnt += a.mc[(size_t)g * M.M + M.chk_idx[i]];
      checkm = cnt == 0;
    }
  double psum = 0;
  if (!checkm) {
    psum = -DBL_MAX;  // the reference's rejection value (MYDBL_MAX)
  } else {
    for (int i = 0; i < nth; i++) psum += a.q[(size_t)grp * nth + i];
    for (int i = 0; i < nmg; i++) psum += a.m[(size_t)grp * nmg + i];
  }
  a.probg[grp] = psum;
  if (a.rows) {
    float *row = a.rows + (size_t)grp * a.rowlen;
    const int pdgp = 4 * nth + 3 * nmg, probgp = pdgp + 1, tp = probgp + 1;
    row[pdgp] = a.pdg ? (float)a.pdg[grp] : 0.0f;
    row[probgp] = (float)psum;
    const double *tv = a.tvals + (size_t)a.group_tv[grp] * (M.npops - 1);
    for (int i = 0; i < M.npops - 1; i++) row[tp + i] = (float)tv[i];
  }
}

// The rubber band of changet_RY1 (update_t_RY.cpp:59-86, 279-335 going
// forward, 444-491 back) on every locus of the listed chains, a warp per
// chain-locus: node times of non-root edges in (t_u, o] go through
// beforesplit, those in (o, t_d) through aftersplit, with o -> n; migration
// times alike.  The float-float copy of each moved time follows it.  Going
// forward the chain's counts are added up (each node time twice, once per
// daughter edge, as the reference counts them) and the item's length is
// saved; going back (o and n exchanged by the caller) the length is restored.
constexpr int BAND_WPB = 8;  // chain-loci (warps) per block
constexpr int RY_STAGE_MAX = 3000;  // loci staged in shared memory (48 KB of rows)

__global__ void __launch_bounds__(32 * BAND_WPB) k_band(BandArgs a)
{
  const int lane = threadIdx.x & 31;
  const int slot = blockIdx.x * BAND_WPB + (threadIdx.x >> 5);
  if (slot >= a.nch * a.nloci) return;  // whole warps only
  const int c = slot / a.nloci, li = slot % a.nloci;
  const int item = a.chains[c] * a.nloci + li;
  const ItemDev it = a.items[item];
  const int nl = 2 * it.n - 1, off = it.node_off;
  const double *P = a.prm + 5 * (size_t)c;
  const int period = (int)P[0];
  const double o = P[1], n = P[2], tu = P[3], td = P[4];
  auto band = [&](double t, int *lo, int *hi) -> double {
    if (t <= o && t > tu) {
      (*lo)++;
      return period == 0 ? t * n / o : tu + (t - tu) * (n - tu) / (o - tu);
    }
    if (t > o && t < td) {
      (*hi)++;
      return period == a.last - 1 ? t + n - o : td - (td - n) * (td - t) / (td - o);
    }
    return t;
  };
  int lo = 0, hi = 0, mlo = 0, mhi = 0;
  const int32_t *mo = a.moff + off + item;
  const long long mb = a.mbase[item];
  for (int k = lane; k < nl; k += 32) {
    if (a.nodes[off + k].down == -1) continue;
    const double t = a.t64[off + k];
    const int moved = lo + hi;
    const double tn = band(t, &lo, &hi);
    if (lo + hi != moved) {
      a.t64[off + k] = tn;
      const float h = (float)tn;
      a.tff[off + k] = make_float2(h, (float)(tn - (double)h));
    }
    for (int j = mo[k]; j < mo[k + 1]; j++) a.mig_t[mb + j] = band(a.mig_t[mb + j], &mlo, &mhi);
  }
  if (!a.inverse) {  // the chain-locus's counts in its own slot (no atomics)
    for (int d = 16; d; d >>= 1) {
      lo += __shfl_xor_sync(~0u, lo, d);
      hi += __shfl_xor_sync(~0u, hi, d);
      mlo += __shfl_xor_sync(~0u, mlo, d);
      mhi += __shfl_xor_sync(~0u, mhi, d);
    }
    if (lane == 0) {
      int32_t *ic = a.item_counts + 4 * (size_t)slot;
      ic[0] = hi;
      ic[1] = lo;
      ic[2] = mhi;
      ic[3] = mlo;
    }
  }
  if (lane == 0) {
    if (a.inverse)
      a.len[item] = a.len_hold[item];
    else
      a.len_hold[item] = a.len[item];
  }
}

// per-chain counts: the chain-loci's slots summed (a thread per chain and count)
__global__ void k_band_sum(const int32_t *item_counts, int nch, int nloci, int32_t *counts)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 4 * nch) return;
  const int c = t >> 2, q = t & 3;
  int v = 0;
  for (int li = 0; li < nloci; li++) v += item_counts[4 * ((size_t)c * nloci + li) + q];
  counts[t] = v;
}

// changet_RY1's decision: likelihood sums in locus order (allpcalc.pdg is
// that sum), tpw = gbeta (new - old) + probg_new - probg_old, the MH term
// beta tpw + (ecd + emd) log(t_d ratio) + (ecu + emu) log(t_u ratio) with
// the node counts halved, and log U < DMIN(1, term) -- NaN rejects, as the
// reference's comparison does.
// One block per chain: the chain's old and new likelihood rows are staged in
// shared memory with coalesced loads, then one thread adds them in locus
// order (the reference's association) and decides.
__global__ void k_ry_decide(RyArgs a)
{
  extern __shared__ double rowbuf[];  // [2][nloci] when staged
  const int c = blockIdx.x;
  if (c >= a.nch) return;
  const int ci = a.chains[c];
  const double *pn = a.pdg_new + (size_t)ci * a.nloci, *po = a.pdg + (size_t)ci * a.nloci;
  const bool staged = a.nloci <= RY_STAGE_MAX;
  if (staged) {
    for (int li = threadIdx.x; li < a.nloci; li += blockDim.x) {
      rowbuf[li] = pn[li];
      rowbuf[a.nloci + li] = po[li];
    }
    __syncthreads();
    pn = rowbuf;
    po = rowbuf + a.nloci;
  }
  if (threadIdx.x != 0) return;
  double snew = 0.0, sold = 0.0;
  for (int li = 0; li < a.nloci; li++) {
    snew += pn[li];
    sold += po[li];
  }
  const int ecd = a.counts[4 * c] / 2, ecu = a.counts[4 * c + 1] / 2, emd = a.counts[4 * c + 2],
            emu = a.counts[4 * c + 3];
  double tpw = a.gbeta * (snew - sold);
  tpw += a.probg_new[c] - a.probg[ci];
  const double mh = a.beta[ci] * tpw + (ecd + emd) * a.lhd[c] + (ecu + emu) * a.lhu[c];
  const double lim = (1.0 < mh) ? 1.0 : mh;
  const bool acc = a.logU[c] < lim;
  a.accept[c] = acc;
  a.pdgsum[c] = acc ? snew : sold;
  if (acc) a.probg[ci] = a.probg_new[c];
}

// rows[groups[i]] -> dst + i * rowlen (a warp per row)
__global__ void __launch_bounds__(128) k_gather_rows(const float *rows, int rowlen, const int32_t *groups, int n,
                                                     float *dst)
{
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= n) return;
  const float *src = rows + (size_t)groups[w] * rowlen;
  for (int k = lane; k < rowlen; k += 32) dst[(size_t)w * rowlen + k] = src[k];
}

}  // namespace

int launch_band(const BandArgs &a, cudaStream_t st)
{
  if (a.nch < 1) return 0;
  const int slots = a.nch * a.nloci;
  k_band<<<(slots + BAND_WPB - 1) / BAND_WPB, 32 * BAND_WPB, 0, st>>>(a);
  if (!a.inverse) k_band_sum<<<(4 * a.nch + 127) / 128, 128, 0, st>>>(a.item_counts, a.nch, a.nloci, a.counts);
  return a.inverse ? 1 : 2;
}

int launch_ry_decide(const RyArgs &a, cudaStream_t st)
{
  if (a.nch < 1) return 0;
  const size_t sm = a.nloci <= RY_STAGE_MAX ? 2 * sizeof(double) * (size_t)a.nloci : 0;
  k_ry_decide<<<a.nch, 128, sm, st>>>(a);
  return 0;
}

int launch_gather_rows(const float *rows, int rowlen, const int32_t *groups, int n, float *dst, cudaStream_t st)
{
  if (n < 1) return 0;
  k_gather_rows<<<(n + 3) / 4, 128, 0, st>>>(rows, rowlen, groups, n, dst);
  return 0;
}

size_t tw_stage_bytes(const TwModel &h) { return ((size_t)(h.T + h.M) * 12 + 15) / 16 * 16; }

bool tw_fits(int P) { return (size_t)P * 12 <= 200 * 1024; }

template <int GW, bool MERGE>
static void launch_sweep(const TwArgs &a, const TwModel &h, cudaStream_t st)
{
  const size_t per = tw_stage_bytes(h);
  const int wpb = TW_WPB;
  const size_t smem = per * (32 / GW) * wpb;
  const int per_block = wpb * (32 / GW);
  k_tw_sweep<GW, MERGE><<<(a.ngen + per_block - 1) / per_block, 32 * wpb, smem, st>>>(a, wpb, (int)per);
}

int launch_treeweight(const TwArgs &a, const TwModel &h, cudaStream_t st)
{
  if (a.ngen < 1) return 0;
  if (!tw_fits(a.P)) return 1;
  // pass 1: a warp per genealogy, P events of shared memory per warp
  const size_t wbytes = (size_t)a.P * 12;
  int wpb = (int)((200 * 1024) / wbytes);
  wpb = wpb < 1 ? 1 : (wpb > TW_WPB ? TW_WPB : wpb);
  const size_t smem = wbytes * wpb;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_tw_events, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return 2;
  }
  k_tw_events<<<(a.ngen + wpb - 1) / wpb, 32 * wpb, smem, st>>>(a, wpb);
  // pass 2: lane groups
  int gw = 2;
  while (gw < h.npops) gw <<= 1;
  // a spare lane (npops < gw) takes the length sums: fewer FP64 operations
  // per event; with none, every lane computes them alongside
  const bool merge = h.npops < gw;
  switch (gw) {
    case 2: launch_sweep<2, false>(a, h, st); break;
    case 4: merge ? launch_sweep<4, true>(a, h, st) : launch_sweep<4, false>(a, h, st); break;
    case 8: merge ? launch_sweep<8, true>(a, h, st) : launch_sweep<8, false>(a, h, st); break;
    default: merge ? launch_sweep<16, true>(a, h, st) : launch_sweep<16, false>(a, h, st); break;
  }
  return 0;
}

int launch_tree_prob(const TwProbArgs &a, const TwModel &h, cudaStream_t st)
{
  if (a.ngroups < 1) return 0;
  const int MM = h.nomig ? 0 : h.M;
  const long long cells = (long long)a.ngroups * ((2 * h.T + MM) + (h.T + MM));
  const long long params = (long long)a.ngroups * (h.nth + (h.nomig ? 0 : h.nmg));
  k_tp_cells<<<(unsigned)((cells + TP_BS - 1) / TP_BS), TP_BS, 0, st>>>(a);
  k_tp_params<<<(unsigned)((params + TP_BS - 1) / TP_BS), TP_BS, 0, st>>>(a);
  k_tp_final<<<(a.ngroups + 127) / 128, 128, 0, st>>>(a);
  return 0;
}
