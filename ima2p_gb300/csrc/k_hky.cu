// k_hky.cu -- HKY85 Felsenstein pruning over site patterns (makefrac,
// calc_prob_data.cpp:118-471; likelihoodHKY :583-607) and the accept/reject of
// its partial likelihoods (copyfraclike / storescalefactors /
// restorescalefactors, update_gtree_common.cpp:2140-2181).
//
// One CTA per chain-locus.  Internal nodes are visited level by level (the
// host supplies, with each genealogy, its internal nodes sorted by height);
// inside a level every (node, pattern) pair is independent, so the CTA's
// threads sweep them with one barrier per level.  A node is recomputed when
// it is on the dirty list, when the list is -1 (full), or when a daughter is
// dirty or recomputed -- the reference's propagation rule (:137-163).
//
// Partial likelihoods are resident state in two slots per node: slot[node]
// names the committed one ("frac"), the other receives new values
// ("newfrac").  Accept flips the slot of every recomputed node, reject keeps
// it; this replaces the reference's buffer copies with a one-byte flip.
//
// FP32 form: partials are float4, rescaled after every node by an exact
// power of two whose exponent is kept as an integer, so the log scale factor
// carries no rounding; the root sum log(sum_j pi_j L_j) is formed from an
// FP32 mantissa log and the integer exponent, accumulated in FP64.
// Float-float form (the default fast precision): the same kernel with every
// partial, coefficient and product as a float-float pair (about 46 bits):
// the hi parts in the FP32 partial array, the lo parts in a second one, the
// exponents shared.  An FP32 partial's rounding (6e-8) repeats in every
// site of a pattern, so a 1000-bp locus of FP32 pruning is off by ~1e-4 in
// log L; the pairs bring that below 1e-8.
// FP64 form: the reference's arithmetic -- partials divided by their maximum,
// log(max) accumulated into an FP64 scale factor.
#include <cmath>

#include "ff.cuh"
#include "internal.h"

namespace {

__constant__ FFConsts c_ffh;  // ln 2 and the log table (filled by hky_init_tables)

constexpr int HKY_BS = 128;
constexpr double LN2 = 0.69314718055994530941723212146;

__device__ __forceinline__ float branch_ff(const NodeRec *nd, const float2 *t, int c)
{
  int u = nd[c].up0;
  if (u < 0) return t[c].x + t[c].y;
  return (t[c].x - t[u].x) + (t[c].y - t[u].y);
}

__device__ __forceinline__ double branch_64(const NodeRec *nd, const double *t, int c)
{
  int u = nd[c].up0;
  return (u < 0) ? t[c] : t[c] - t[u];
}

// HKY85 transition matrix P[j][k] = P(j -> k | b), Pi and A from the class
// (purine / pyrimidine) of the target state k.
template <typename T>
__device__ __forceinline__ void hky_p(const T *pi, T kpa, T b, T *P)
{
  T e1 = exp(-b);
  T PR = pi[0] + pi[2], PY = pi[1] + pi[3];
  T eR = exp(-b * (T(1) + PR * kpa)), eY = exp(-b * (T(1) + PY * kpa));
#pragma unroll
  for (int k = 0; k < 4; k++) {
    T Pk = (k == 0 || k == 2) ? PR : PY;
    T e2 = (k == 0 || k == 2) ? eR : eY;
    T base = pi[k] + pi[k] * e1 * (T(1) / Pk - T(1));
#pragma unroll
    for (int j = 0; j < 4; j++) {
      T v;
      if (j == k) v = base + e2 * ((Pk - pi[k]) / Pk);
      else if (j + k == 2 || j + k == 4) v = base - (pi[k] / Pk) * e2;
      else v = pi[k] * (T(1) - e1);
      P[j * 4 + k] = v;
    }
  }
}

// The same matrix for FP32 as five coefficients per branch.  With
// E1 = 1 - exp(-b) and E2_c = 1 - exp(-b A_c), A_c = 1 + Pi_c (kappa - 1),
// both taken from expm1 so that short branches do not cancel, the entries are
//   transversion  pi_k E1
//   transition    (pi_k / Pi_c) (E2_c - E1 (1 - Pi_c))
//   identity      the transition value plus 1 - E2_c
// and with the states ordered A, C, G, T (purines R = {A, G}, pyrimidines
// Y = {C, T}) the product of P(b) with a partial L is, for j in class c and
// the other class o,
//   v_j = E1 S_o + b_c S_c + d_c L_j,   S_c = sum_{k in c} pi_k L_k,
//   b_c = (E2_c - E1 (1 - Pi_c)) / Pi_c,   d_c = 1 - E2_c.
// K = {E1, b_R, b_Y, d_R, d_Y}.
__device__ __forceinline__ void hky_coef_fast(const float *pi, float kpa, float b, float *K)
{
  const float E1 = -expm1f(-b);
  const float PR = pi[0] + pi[2], PY = pi[1] + pi[3];
  const float ER = -expm1f(-b * (1.0f + PR * kpa)), EY = -expm1f(-b * (1.0f + PY * kpa));
  K[0] = E1;
  K[1] = (ER - E1 * (1.0f - PR)) / PR;
  K[2] = (EY - E1 * (1.0f - PY)) / PY;
  K[3] = 1.0f - ER;
  K[4] = 1.0f - EY;
}

// P(b) L for one child at one pattern: a tip observed in state st, or an
// internal node's partial Lc
struct HkyCoef {
  float a, bR, bY, dR, dY;
};
__device__ __forceinline__ void hky_apply_tip(const HkyCoef &K, const float *pi, int st, float *v)
{
  const float p = pi[st];
  const bool isR = (st & 1) == 0;
  const float tR = (isR ? K.bR : K.a) * p, tY = (isR ? K.a : K.bY) * p;
  v[0] = tR + (st == 0 ? K.dR : 0.0f);
  v[2] = tR + (st == 2 ? K.dR : 0.0f);
  v[1] = tY + (st == 1 ? K.dY : 0.0f);
  v[3] = tY + (st == 3 ? K.dY : 0.0f);
}
__device__ __forceinline__ void hky_apply(const HkyCoef &K, const float *pi, float4 L, float *v)
{
  const float SR = fmaf(pi[2], L.z, pi[0] * L.x), SY = fmaf(pi[3], L.w, pi[1] * L.y);
  const float tR = fmaf(K.bR, SR, K.a * SY), tY = fmaf(K.bY, SY, K.a * SR);
  v[0] = fmaf(K.dR, L.x, tR);
  v[2] = fmaf(K.dR, L.z, tR);
  v[1] = fmaf(K.dY, L.y, tY);
  v[3] = fmaf(K.dY, L.w, tY);
}

// Float-float coefficients of one branch, K = {E1, b_R, b_Y, d_R, d_Y} as
// (hi, lo) pairs: E1 = 1 - e^-b, E2_c = 1 - e^(-b A_c), d_c = e^(-b A_c)
// taken directly (1 - E2_c would cancel on long branches).
__device__ __forceinline__ void hky_coef_ff(const ff *pi, ff kpa, ff b, float *K)
{
  const ff PR = ff_add(pi[0], pi[2]), PY = ff_add(pi[1], pi[3]);
  ff e1, m1, eR, mR, eY, mY;
  ff_exp_expm1(ff_neg(b), &e1, &m1);
  ff_exp_expm1(ff_neg(ff_mul(b, ff_add_f(ff_mul(PR, kpa), 1.0f))), &eR, &mR);
  ff_exp_expm1(ff_neg(ff_mul(b, ff_add_f(ff_mul(PY, kpa), 1.0f))), &eY, &mY);
  const ff E1 = ff_neg(m1), ER = ff_neg(mR), EY = ff_neg(mY);
  const ff bR = ff_div(ff_sub(ER, ff_mul(E1, ff_add_f(ff_neg(PR), 1.0f))), PR);
  const ff bY = ff_div(ff_sub(EY, ff_mul(E1, ff_add_f(ff_neg(PY), 1.0f))), PY);
  K[0] = E1.hi; K[1] = E1.lo;
  K[2] = bR.hi; K[3] = bR.lo;
  K[4] = bY.hi; K[5] = bY.lo;
  K[6] = eR.hi; K[7] = eR.lo;
  K[8] = eY.hi; K[9] = eY.lo;
}

// Every operand of the pruning products is >= 0, so these sums never cancel.
// a*b + c:
__device__ __forceinline__ ff ff_fma_pos(ff a, ff b, ff c)
{
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  const ff s = two_sum(p, c.hi);
  return fast_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(pe, c.lo)));
}

struct HkyCoefFF {
  ff a, bR, bY, dR, dY;
};
__device__ __forceinline__ HkyCoefFF load_coef_ff(const float *Kp)
{
  HkyCoefFF K;
  K.a = ff_make(Kp[0], Kp[1]);
  K.bR = ff_make(Kp[2], Kp[3]);
  K.bY = ff_make(Kp[4], Kp[5]);
  K.dR = ff_make(Kp[6], Kp[7]);
  K.dY = ff_make(Kp[8], Kp[9]);
  return K;
}
// P(b) applied to a tip observed in state st: column st of P(b)
__device__ __forceinline__ void hky_apply_tip_ff(const HkyCoefFF &K, const ff *pi, int st, ff *v)
{
  const ff p = st == 0 ? pi[0] : st == 1 ? pi[1] : st == 2 ? pi[2] : pi[3];
  const bool isR = (st & 1) == 0;
  const ff tR = ff_mul(isR ? K.bR : K.a, p), tY = ff_mul(isR ? K.a : K.bY, p);
  const ff own = ff_add(isR ? tR : tY, isR ? K.dR : K.dY);  // the observed state's entry
  v[0] = st == 0 ? own : tR;
  v[2] = st == 2 ? own : tR;
  v[1] = st == 1 ? own : tY;
  v[3] = st == 3 ? own : tY;
}
// The same steps leaving the pair unnormalised (|lo| may reach a few
// ulp(hi)), for intermediate values: the next step's TwoSum is exact
// whatever lo is, so only the values that leave the apply are renormalised.
__device__ __forceinline__ ff ff_mul_u(ff a, ff b)
{
  const float p = __fmul_rn(a.hi, b.hi);
  return ff_make(p, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p))));
}
__device__ __forceinline__ ff ff_fma_pos_u(ff a, ff b, ff c)
{
  const float p = __fmul_rn(a.hi, b.hi);
  const float pe = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, __fmaf_rn(a.hi, b.hi, -p)));
  const ff s = two_sum(p, c.hi);
  return ff_make(s.hi, __fadd_rn(s.lo, __fadd_rn(pe, c.lo)));
}

// v_j = E1 S_o + b_c S_c + d_c L_j, left unnormalised too: its only use is
// the product of the two daughters, whose ff_mul renormalises
__device__ __forceinline__ void hky_apply_ff(const HkyCoefFF &K, const ff *pi, const ff *L, ff *v)
{
  const ff SR = ff_fma_pos_u(pi[2], L[2], ff_mul_u(pi[0], L[0]));
  const ff SY = ff_fma_pos_u(pi[3], L[3], ff_mul_u(pi[1], L[1]));
  const ff tR = ff_fma_pos_u(K.bR, SR, ff_mul_u(K.a, SY));
  const ff tY = ff_fma_pos_u(K.bY, SY, ff_mul_u(K.a, SR));
  v[0] = ff_fma_pos_u(K.dR, L[0], tR);
  v[2] = ff_fma_pos_u(K.dR, L[2], tR);
  v[1] = ff_fma_pos_u(K.dY, L[1], tY);
  v[3] = ff_fma_pos_u(K.dY, L[3], tY);
}

__device__ __forceinline__ ff ff_of(float2 v) { return ff_make(v.x, v.y); }

// Shared-memory carve-up, identical on host (sizing) and device.
struct HkyLayout {
  size_t nd, fresh, order, total;
};
__host__ __device__ inline HkyLayout hky_layout(int maxnl, size_t elem)
{
  HkyLayout l;
  l.nd = elem * 16 * (size_t)maxnl;
  l.fresh = l.nd + sizeof(NodeRec) * (size_t)maxnl;
  l.order = (l.fresh + 3 * (size_t)maxnl + 15) & ~size_t(15);
  l.total = (l.order + sizeof(int16_t) * (size_t)(maxnl + 3) + 15) & ~size_t(15);
  return l;
}

// Per-CTA shared state common to both precisions.
struct Tree {
  NodeRec *nd;
  uint8_t *fresh;
  uint8_t *dirty;
  uint8_t *slot;
  int16_t *order;
  int16_t *lstart;
};

__device__ double standfactor(const double *pi, double kappa)
{
  double p = 0.0;
  for (int i = 0; i < 4; i++)
    for (int j = 0; j < 4; j++) {
      if (i == j) continue;
      p += (i + j == 2 || i + j == 4) ? pi[i] * pi[j] * kappa : pi[i] * pi[j];
    }
  return p;
}

// Loads topology and schedule, marks dirty nodes and decides which internal
// nodes are recomputed.  Returns after a barrier.
__device__ void load_tree(const Pools &P, const ItemDev &it, const ReqDev &R, int nlev, Tree &T,
                          const uint8_t *gslot)
{
  const int n = it.n, nl = 2 * n - 1;
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    T.nd[k] = P.nodes[it.node_off + k];
    T.dirty[k] = 0;
    T.slot[k] = gslot[it.node_off + k];
  }
  for (int k = threadIdx.x; k < n - 1 + nlev + 1; k += blockDim.x)
    T.order[k] = P.sched[it.sched_off + k];
  __syncthreads();
  if (threadIdx.x == 0) {
    bool full = (R.e[0] == -1);
    for (int q = 0; q < 4; q++)
      if (R.e[q] >= 0 && R.e[q] < nl) T.dirty[R.e[q]] = 1;
    for (int k = 0; k < n - 1; k++) {
      int node = T.order[k];
      int a = T.nd[node].up0, b = T.nd[node].up1;
      bool f = full || T.dirty[node] || T.dirty[a] || T.dirty[b] ||
               (a >= n && T.fresh[a]) || (b >= n && T.fresh[b]);
      T.fresh[node] = f ? 1 : 0;
    }
  }
  __syncthreads();
}

__device__ __forceinline__ float pow2f(int k)  // 2^k for -126 <= k <= 127
{
  return __int_as_float((127 + k) << 23);
}

__device__ __forceinline__ int expo_of(float m)  // floor(log2(m)) for normal m > 0
{
  return ((__float_as_int(m) >> 23) & 0xff) - 127;
}

// ------------------------------------------------------------------ FP32
// One CTA per chain-locus, internal nodes level by level.  Each branch gets
// the five coefficients of hky_coef_fast (in place of a 4 x 4 matrix), and a
// warp works on one node and 32 of its patterns at a time, so the children's
// coefficients are warp-uniform and no warp mixes tip and internal children.
// With CACHE, the partials this launch computes are also kept in shared
// memory ([internal node][pattern]) and daughters are read from there instead
// of making an L2 round trip per level.  BS threads per CTA, registers for
// MINB resident CTAs per SM.  FF: every value a float-float pair (the lo
// parts of the partials in P.partlo); otherwise FP32 (which clears the lo
// parts of what it writes when they exist, so a later FF evaluation reads
// its partials as exact pairs).
template <bool FF, bool CACHE, int BS, int MINB>
__global__ void __launch_bounds__(BS, MINB) k_hky_fast(Pools P, const ReqDev *reqs,
                                                     double *result, int32_t *status, int maxnl,
                                                     int cache_S, int tip_cap)
{
  extern __shared__ __align__(16) char smem[];
  // the request carries the item's offsets and sizes, so the tree loads
  // below wait on this one load only
  const ReqDev R = reqs[blockIdx.x];
  const int n = R.n, nl = 2 * n - 1, S = R.nsites, nint = n - 1;
  // [maxnl][PMS]: 5 coefficients per branch (FF: pairs); FF tip branches
  // hold instead the columns of P(b) for the four observed states, [4][4]
  // pairs, so a tip daughter costs four loads
  constexpr int PMS = FF ? 32 : 16;
  const HkyLayout lay = hky_layout(maxnl, FF ? 2 * sizeof(float) : sizeof(float));
  float *Pm = reinterpret_cast<float *>(smem);
  Tree T;
  T.nd = reinterpret_cast<NodeRec *>(smem + lay.nd);
  T.fresh = reinterpret_cast<uint8_t *>(smem + lay.fresh);
  T.dirty = T.fresh + maxnl;
  T.slot = T.dirty + maxnl;
  T.order = reinterpret_cast<int16_t *>(smem + lay.order);
  // the tips' states [n][S] when they fit in tip_cap bytes: the level loop
  // then reads no global memory when the partials are cached too
  int8_t *stip = reinterpret_cast<int8_t *>(smem + lay.total);
  const size_t tipb = ((size_t)tip_cap + 15) & ~size_t(15);
  const bool tips = n * S <= tip_cap;
  float4 *cpart = reinterpret_cast<float4 *>(smem + lay.total + tipb);  // [nint][cache_S]
  float4 *cpartlo = cpart + (FF ? (size_t)(maxnl / 2) * cache_S : 0);   // FF: lo parts
  int32_t *cexp = reinterpret_cast<int32_t *>(cpartlo + (size_t)(maxnl / 2) * cache_S);
  __shared__ double red_d[BS / 32];
  __shared__ long long red_e[BS / 32];
  __shared__ float2 spi[4];   // pi (FP32: .x only)
  __shared__ float2 smu, skpa;

  const int tid = threadIdx.x;
  const bool full = (R.e[0] == -1);
  for (int k = tid; k < nl; k += BS) {
    T.nd[k] = P.nodes[R.node_off + k];
    T.slot[k] = P.slot32[R.node_off + k];
    T.dirty[k] = 0;
    T.fresh[k] = full ? 1 : 0;
  }
  // the schedule (n-1 + nlev+1 entries, nlev <= n-1) in its 2n-entry slot,
  // without waiting for the level count
  for (int k = tid; k < 2 * n; k += BS) T.order[k] = P.sched[R.sched_off + k];
  const int nlev = P.nlev[R.item];
  T.lstart = T.order + nint;
  if (tips) {
    const int8_t *sq = P.seq + R.seq_off;
    for (int k = tid; k < n * S; k += BS) stip[k] = sq[k];
  }
  if (tid == 0) {
    const double *pid = P.pi + 4 * (size_t)R.item;
    const double mu = R.u / ((double)R.totsites * standfactor(pid, R.par));
    const double kp = R.par - 1.0;
    smu = make_float2((float)mu, (float)(mu - (double)(float)mu));
    skpa = make_float2((float)kp, (float)(kp - (double)(float)kp));
    for (int j = 0; j < 4; j++) spi[j] = make_float2((float)pid[j], (float)(pid[j] - (double)(float)pid[j]));
  }
  __syncthreads();
  if (!full && tid == 0) {  // the reference's propagation rule, bottom-up
    for (int q = 0; q < 4; q++)
      if (R.e[q] >= 0 && R.e[q] < nl) T.dirty[R.e[q]] = 1;
    for (int k = 0; k < nint; k++) {
      int node = T.order[k];
      int a = T.nd[node].up0, b = T.nd[node].up1;
      T.fresh[node] = (T.dirty[node] || T.dirty[a] || T.dirty[b] || (a >= n && T.fresh[a]) ||
                       (b >= n && T.fresh[b])) ? 1 : 0;
    }
  }
  if (!full) __syncthreads();
  const float2 *tff = P.tff + R.node_off;
  for (int c = tid; c < nl; c += BS) {
    int d = T.nd[c].down;
    if (d < 0 || !T.fresh[d]) continue;
    if constexpr (FF) {
      const ff pif[4] = {ff_of(spi[0]), ff_of(spi[1]), ff_of(spi[2]), ff_of(spi[3])};
      const int u = T.nd[c].up0;
      const ff tc = ff_of(tff[c]);
      const ff br = (u < 0) ? tc : ff_sub(tc, ff_of(tff[u]));
      float Kc[10];
      hky_coef_ff(pif, ff_of(skpa), ff_mul(ff_of(smu), br), Kc);
      float *dst = Pm + PMS * c;
      if (c < n) {
        const HkyCoefFF K = load_coef_ff(Kc);
#pragma unroll
        for (int st = 0; st < 4; st++) {
          ff v[4];
          hky_apply_tip_ff(K, pif, st, v);
#pragma unroll
          for (int j = 0; j < 4; j++) reinterpret_cast<float2 *>(dst)[4 * st + j] = make_float2(v[j].hi, v[j].lo);
        }
      } else {
#pragma unroll
        for (int j = 0; j < 10; j++) dst[j] = Kc[j];
      }
    } else {
      float pil[4] = {spi[0].x, spi[1].x, spi[2].x, spi[3].x};
      hky_coef_fast(pil, skpa.x, smu.x * branch_ff(T.nd, tff, c), Pm + PMS * c);
    }
  }
  __syncthreads();

  const size_t slot_stride = (size_t)nint * S;
  float4 *part = P.part + R.part_off;
  float4 *partlo = P.partlo ? P.partlo + R.part_off : nullptr;
  int32_t *pexp = P.pexp + R.part_off;
  const int8_t *seq = P.seq + R.seq_off;
  const float pi4[4] = {spi[0].x, spi[1].x, spi[2].x, spi[3].x};
  // warps take (node, 32-pattern chunk) pairs of a level in turn, so a warp
  // works on one node at a time and its children's coefficients stay in
  // registers; lanes are patterns
  constexpr int NW = BS / 32;
  const int warp = tid >> 5, lane = tid & 31;
  const int nch = (S + 31) >> 5;
  // a warp's task q = jj * nch + chunk advances by NW: by NW / nch nodes and
  // NW % nch chunks (no division in the loop)
  const int jstep = NW / nch, cstep = NW - jstep * nch;
  const int j0 = warp / nch, c0 = warp - j0 * nch;
  for (int lv = 0; lv < nlev; lv++) {
    const int beg = T.lstart[lv], total = (T.lstart[lv + 1] - beg) * nch;
    int jj = j0, ch = c0;
    for (int q = warp; q < total; q += NW, jj += jstep, ch += cstep) {
      if (ch >= nch) {
        ch -= nch;
        jj++;
      }
      const int i = ch * 32 + lane;
      const int node = T.order[beg + jj];
      if (!T.fresh[node] || i >= S) continue;
      const int cc[2] = {T.nd[node].up0, T.nd[node].up1};
      int e = 0;
      float4 ov, ol = make_float4(0.f, 0.f, 0.f, 0.f);
      if constexpr (FF) {
        const ff pif[4] = {ff_of(spi[0]), ff_of(spi[1]), ff_of(spi[2]), ff_of(spi[3])};
        ff v[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = cc[h];
          if (c < n) {
            const int st = tips ? stip[c * S + i] : seq[(size_t)c * S + i];
            const float4 *col = reinterpret_cast<const float4 *>(Pm + PMS * c) + 2 * st;
            const float4 a = col[0], b = col[1];
            v[h][0] = ff_make(a.x, a.y);
            v[h][1] = ff_make(a.z, a.w);
            v[h][2] = ff_make(b.x, b.y);
            v[h][3] = ff_make(b.z, b.w);
          } else {
            const HkyCoefFF K = load_coef_ff(Pm + PMS * c);
            float4 hi, lo;
            if (CACHE && T.fresh[c]) {
              const size_t ci = (size_t)(c - n) * cache_S + i;
              hi = cpart[ci];
              lo = cpartlo[ci];
              e += cexp[ci];
            } else {
              const int rs = T.fresh[c] ? 1 - T.slot[c] : T.slot[c];
              const size_t idx = rs * slot_stride + (size_t)(c - n) * S + i;
              hi = part[idx];
              lo = partlo[idx];
              e += pexp[idx];
            }
            const ff Lc[4] = {ff_make(hi.x, lo.x), ff_make(hi.y, lo.y), ff_make(hi.z, lo.z), ff_make(hi.w, lo.w)};
            hky_apply_ff(K, pif, Lc, v[h]);
          }
        }
        ff o[4];
#pragma unroll
        for (int j = 0; j < 4; j++) o[j] = ff_mul(v[0][j], v[1][j]);
        // normalise by an exact power of two when the largest entry drops
        // below 2^-20: the lo parts (2^-24 below) stay far from subnormal
        const float m = fmaxf(fmaxf(o[0].hi, o[1].hi), fmaxf(o[2].hi, o[3].hi));
        if (m < 9.5367432e-07f && m > 0.f) {
          const int k = expo_of(m);
          const float sc = pow2f(-k);
#pragma unroll
          for (int j = 0; j < 4; j++) o[j] = ff_make(o[j].hi * sc, o[j].lo * sc);
          e += k;
        }
        ov = make_float4(o[0].hi, o[1].hi, o[2].hi, o[3].hi);
        ol = make_float4(o[0].lo, o[1].lo, o[2].lo, o[3].lo);
      } else {
        float v[2][4];
#pragma unroll
        for (int h = 0; h < 2; h++) {
          const int c = cc[h];
          const float *Kp = Pm + PMS * c;
          const HkyCoef K = {Kp[0], Kp[1], Kp[2], Kp[3], Kp[4]};
          if (c < n) {
            hky_apply_tip(K, pi4, tips ? stip[c * S + i] : seq[(size_t)c * S + i], v[h]);
          } else {
            float4 Lc;
            if (CACHE && T.fresh[c]) {
              const size_t ci = (size_t)(c - n) * cache_S + i;
              Lc = cpart[ci];
              e += cexp[ci];
            } else {
              const int rs = T.fresh[c] ? 1 - T.slot[c] : T.slot[c];
              const size_t idx = rs * slot_stride + (size_t)(c - n) * S + i;
              Lc = part[idx];
              e += pexp[idx];
            }
            hky_apply(K, pi4, Lc, v[h]);
          }
        }
        ov = make_float4(v[0][0] * v[1][0], v[0][1] * v[1][1], v[0][2] * v[1][2], v[0][3] * v[1][3]);
        // rescale by an exact 2^40 only when the largest entry drops below
        // 2^-40: products of two daughters then stay above 2^-80 (normal)
        const float m = fmaxf(fmaxf(ov.x, ov.y), fmaxf(ov.z, ov.w));
        if (m < 9.094947e-13f) {
          const float up = 1.0995116e12f;  // 2^40
          ov.x *= up; ov.y *= up; ov.z *= up; ov.w *= up;
          e -= 40;
          if (m * up < 9.094947e-13f) {  // very small value: normalise exactly
            const float mm = m * up;
            const int k = (mm > 0.f) ? expo_of(mm) : 0;
            const float sc = pow2f(-k);
            ov.x *= sc; ov.y *= sc; ov.z *= sc; ov.w *= sc;
            e += k;
          }
        }
      }
      const size_t widx = (1 - T.slot[node]) * slot_stride + (size_t)(node - n) * S + i;
      part[widx] = ov;
      if (partlo) partlo[widx] = ol;
      pexp[widx] = e;
      if (CACHE) {
        const size_t ci = (size_t)(node - n) * cache_S + i;
        cpart[ci] = ov;
        if (FF) cpartlo[ci] = ol;
        cexp[ci] = e;
      }
    }
    __syncthreads();
  }

  // root: sum_i mult_i * (log(sum_j pi_j L_j) + scale_i)
  const int root = T.order[nint - 1];
  const int rs = T.fresh[root] ? 1 - T.slot[root] : T.slot[root];
  const int32_t *mult = P.mult + R.mult_off;
  double acc = 0.0;
  long long acce = 0;
  for (int i = tid; i < S; i += BS) {
    float4 Lr, Ll = make_float4(0.f, 0.f, 0.f, 0.f);
    int er;
    if (CACHE && T.fresh[root]) {
      size_t ci = (size_t)(root - n) * cache_S + i;
      Lr = cpart[ci];
      if (FF) Ll = cpartlo[ci];
      er = cexp[ci];
    } else {
      size_t idx = rs * slot_stride + (size_t)(root - n) * S + i;
      Lr = part[idx];
      if (FF) Ll = partlo[idx];
      er = pexp[idx];
    }
    const int mlt = mult[i];
    if constexpr (FF) {
      ff f = ff_mul(ff_of(spi[0]), ff_make(Lr.x, Ll.x));
      f = ff_fma_pos(ff_of(spi[1]), ff_make(Lr.y, Ll.y), f);
      f = ff_fma_pos(ff_of(spi[2]), ff_make(Lr.z, Ll.z), f);
      f = ff_fma_pos(ff_of(spi[3]), ff_make(Lr.w, Ll.w), f);
      const int k = expo_of(f.hi);
      const float sc = pow2f(-k);
      const ff lg = ff_log(ff_make(f.hi * sc, f.lo * sc), c_ffh);
      acc += (double)mlt * ((double)lg.hi + (double)lg.lo);
      acce += (long long)mlt * (long long)(er + k);
    } else {
      float f = spi[0].x * Lr.x + spi[1].x * Lr.y + spi[2].x * Lr.z + spi[3].x * Lr.w;
      int k = expo_of(f);
      float mant = f * pow2f(-k);
      acc += (double)mlt * (double)logf(mant);
      acce += (long long)mlt * (long long)(er + k);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    acc += __shfl_xor_sync(0xffffffffu, acc, o);
    acce += __shfl_xor_sync(0xffffffffu, acce, o);
  }
  if ((tid & 31) == 0) {
    red_d[tid >> 5] = acc;
    red_e[tid >> 5] = acce;
  }
  // recomputed marks for the commit step
  for (int k = tid; k < nl; k += BS) P.fresh32[R.node_off + k] = (k >= n) ? T.fresh[k] : 0;
  __syncthreads();
  if (tid == 0) {
    double s = 0.0;
    long long se = 0;
    for (int w = 0; w < BS / 32; w++) { s += red_d[w]; se += red_e[w]; }
    result[blockIdx.x] = s + (double)se * LN2;
    P.pdg_new[R.item] = result[blockIdx.x];
    status[blockIdx.x] = IMA_EVAL_OK;
  }
}

// ------------------------------------------------------------------ FP64
__global__ void __launch_bounds__(HKY_BS) k_hky_fp64(Pools P, const ReqDev *reqs,
                                                     double *result, int32_t *status, int maxnl)
{
  extern __shared__ __align__(16) char smem[];
  const ReqDev R = reqs[blockIdx.x];
  const ItemDev it = P.items[R.item];
  const LocusDev L = P.loci[it.locus];
  const int n = it.n, nl = 2 * n - 1, S = L.nsites, nint = n - 1;
  const int nlev = P.nlev[R.item];
  const HkyLayout lay = hky_layout(maxnl, sizeof(double));
  double *Pm = reinterpret_cast<double *>(smem);  // [maxnl][16]
  Tree T;
  T.nd = reinterpret_cast<NodeRec *>(smem + lay.nd);
  T.fresh = reinterpret_cast<uint8_t *>(smem + lay.fresh);
  T.dirty = T.fresh + maxnl;
  T.slot = T.dirty + maxnl;
  T.order = reinterpret_cast<int16_t *>(smem + lay.order);
  __shared__ double red_d[HKY_BS / 32];
  __shared__ double spi[4];
  __shared__ double smu;

  load_tree(P, it, R, nlev, T, P.slot64);
  T.lstart = T.order + nint;
  if (threadIdx.x == 0) {
    const double *pid = P.pi + 4 * (size_t)R.item;
    smu = R.u / ((double)L.totsites * standfactor(pid, R.par));
    for (int j = 0; j < 4; j++) spi[j] = pid[j];
  }
  __syncthreads();
  const double *t64 = P.t64 + it.node_off;
  double kpa = R.par - 1.0;
  for (int c = threadIdx.x; c < nl; c += blockDim.x) {
    int d = T.nd[c].down;
    if (d < 0 || !T.fresh[d]) continue;
    double pil[4] = {spi[0], spi[1], spi[2], spi[3]};
    hky_p<double>(pil, kpa, smu * branch_64(T.nd, t64, c), Pm + 16 * c);
  }
  __syncthreads();

  const size_t slot_stride = (size_t)nint * S;
  double *part = P.part64 + it.part64_off * 4;
  double *psf = P.psf64 + it.part64_off;
  const int8_t *seq = P.seq + L.seq_off;
  for (int lv = 0; lv < nlev; lv++) {
    int beg = T.lstart[lv], cnt = T.lstart[lv + 1] - beg;
    for (int w = threadIdx.x; w < cnt * S; w += blockDim.x) {
      int node = T.order[beg + w / S];
      int i = w - (w / S) * S;
      if (!T.fresh[node]) continue;
      double v[2][4];
      double sf = 0.0;
#pragma unroll
      for (int h = 0; h < 2; h++) {
        int c = h ? T.nd[node].up1 : T.nd[node].up0;
        const double *Pc = Pm + 16 * c;
        if (c < n) {
          int s = seq[(size_t)c * S + i];
#pragma unroll
          for (int j = 0; j < 4; j++) v[h][j] = Pc[j * 4 + s];
        } else {
          int rs = T.fresh[c] ? 1 - T.slot[c] : T.slot[c];
          size_t idx = rs * slot_stride + (size_t)(c - n) * S + i;
          const double2 *Lp = reinterpret_cast<const double2 *>(part + 4 * idx);
          double2 a = Lp[0], b = Lp[1];
          sf += psf[idx];
#pragma unroll
          for (int j = 0; j < 4; j++)
            v[h][j] = Pc[j * 4 + 0] * a.x + Pc[j * 4 + 1] * a.y + Pc[j * 4 + 2] * b.x +
                      Pc[j * 4 + 3] * b.y;
        }
      }
      double o[4];
      double m = 0.0;
#pragma unroll
      for (int j = 0; j < 4; j++) {
        o[j] = v[0][j] * v[1][j];
        if (o[j] > m) m = o[j];
      }
      size_t widx = (1 - T.slot[node]) * slot_stride + (size_t)(node - n) * S + i;
      double2 *W = reinterpret_cast<double2 *>(part + 4 * widx);
      W[0] = make_double2(o[0] / m, o[1] / m);
      W[1] = make_double2(o[2] / m, o[3] / m);
      psf[widx] = sf + log(m);
    }
    __syncthreads();
  }

  int root = T.order[nint - 1];
  int rs = T.fresh[root] ? 1 - T.slot[root] : T.slot[root];
  const int32_t *mult = P.mult + L.mult_off;
  double acc = 0.0;
  for (int i = threadIdx.x; i < S; i += blockDim.x) {
    size_t idx = rs * slot_stride + (size_t)(root - n) * S + i;
    const double2 *Lp = reinterpret_cast<const double2 *>(part + 4 * idx);
    double2 a = Lp[0], b = Lp[1];
    double f = spi[0] * a.x + spi[1] * a.y + spi[2] * b.x + spi[3] * b.y;
    acc += mult[i] * (log(f) + psf[idx]);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red_d[threadIdx.x >> 5] = acc;
  for (int k = threadIdx.x; k < nl; k += blockDim.x)
    P.fresh64[it.node_off + k] = (k >= n) ? T.fresh[k] : 0;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < HKY_BS / 32; w++) s += red_d[w];
    result[blockIdx.x] = s;
    P.pdg_new[R.item] = s;
    status[blockIdx.x] = IMA_EVAL_OK;
  }
}

// accept: recomputed nodes' new slot becomes the committed one; reject: the
// committed slot stays.  Either way the recomputed marks are cleared, so a
// repeated accept is a no-op as the reference's repeated copy is.
__global__ void k_hky_commit(Pools P, const int32_t *items, const uint8_t *accept)
{
  const ItemDev it = P.items[items[blockIdx.x]];
  const bool acc = accept[blockIdx.x] != 0;
  const int nl = 2 * it.n - 1;
  for (int k = threadIdx.x; k < nl; k += blockDim.x) {
    size_t g = (size_t)it.node_off + k;
    if (P.fresh32[g]) {
      if (acc) P.slot32[g] ^= 1;
      P.fresh32[g] = 0;
    }
    if (P.slot64 && P.fresh64[g]) {
      if (acc) P.slot64[g] ^= 1;
      P.fresh64[g] = 0;
    }
  }
}

size_t hky_smem(int maxn, size_t elem) { return hky_layout(2 * maxn - 1, elem).total; }

}  // namespace

// Partials stay in shared memory when the largest chain-locus of the batch
// fits in this budget (keeps >= 3 CTAs per SM).
constexpr size_t HKY_CACHE_BUDGET = 64 * 1024;
constexpr size_t HKY_TIP_BUDGET = 8 * 1024;

template <bool FF, int BS, int MINB>
static void hky_fast_bs(const Pools &P, const ReqDev *reqs, int nreq, int maxnl, int maxS, bool cache_ok,
                        double *result, int32_t *status, cudaStream_t st)
{
  // tip states staged in shared memory when the largest locus's fit in
  // HKY_TIP_BUDGET bytes (a few KB: occupancy is unchanged)
  const size_t maxn = (size_t)(maxnl + 1) / 2;
  const int tip_cap = (maxn * maxS <= HKY_TIP_BUDGET) ? (int)(maxn * maxS) : 0;
  size_t base = hky_smem((int)maxn, FF ? 2 * sizeof(float) : sizeof(float)) + (((size_t)tip_cap + 15) & ~size_t(15));
  size_t cache = (size_t)(maxnl / 2) * maxS * ((FF ? 2 : 1) * sizeof(float4) + sizeof(int32_t));
  if (cache_ok && cache <= HKY_CACHE_BUDGET) {
    size_t sm = base + cache;
    if (sm > 48 * 1024)
      cudaFuncSetAttribute(k_hky_fast<FF, true, BS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    k_hky_fast<FF, true, BS, MINB><<<nreq, BS, sm, st>>>(P, reqs, result, status, maxnl, maxS, tip_cap);
  } else {
    if (base > 48 * 1024)
      cudaFuncSetAttribute(k_hky_fast<FF, false, BS, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)base);
    k_hky_fast<FF, false, BS, MINB><<<nreq, BS, base, st>>>(P, reqs, result, status, maxnl, 0, tip_cap);
  }
}

void launch_hky_fast(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, int variant,
                     double *result, int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  const int maxnl = 2 * maxn - 1;
  switch (variant) {
    case 1: hky_fast_bs<true, 64, 16>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 2: hky_fast_bs<true, 256, 4>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 3: hky_fast_bs<true, 128, 10>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 4: hky_fast_bs<true, 128, 6>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 5: hky_fast_bs<true, 96, 11>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    default: hky_fast_bs<true, 128, 8>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
  }
}

void launch_hky_fp32(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, int variant,
                     double *result, int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  const int maxnl = 2 * maxn - 1;
  switch (variant) {
    case 1: hky_fast_bs<false, 64, 24>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 2: hky_fast_bs<false, 256, 6>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 3: hky_fast_bs<false, 128, 12>(P, reqs, nreq, maxnl, maxS, false, result, status, st); break;
    case 4: hky_fast_bs<false, 128, 8>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    case 5: hky_fast_bs<false, 96, 16>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
    default: hky_fast_bs<false, 128, 12>(P, reqs, nreq, maxnl, maxS, true, result, status, st); break;
  }
}

// ln 2 and the log table of the float-float root sum (once per device)
int hky_init_tables()
{
  FFConsts K{};
  for (int i = 0; i < 64; i++) {
    const double v = std::log(1.0 + (2.0 * i + 1.0) / 128.0);
    K.logtab[i] = make_float2((float)v, (float)(v - (double)(float)v));
  }
  const double ln2 = 0.69314718055994530941723212146;
  const double a = 355.0 / 512.0;
  K.ln2a = make_float2((float)a, (float)(ln2 - a));
  K.ln2b = (float)(ln2 - a - (double)(float)(ln2 - a));
  return cudaMemcpyToSymbol(c_ffh, &K, sizeof(K)) == cudaSuccess ? 0 : -1;
}

void launch_hky_fp64(const Pools &P, const ReqDev *reqs, int nreq, int maxn, double *result,
                     int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  size_t sm = hky_smem(maxn, sizeof(double));
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_hky_fp64, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_hky_fp64<<<nreq, HKY_BS, sm, st>>>(P, reqs, result, status, 2 * maxn - 1);
}

void launch_hky_commit(const Pools &P, const int32_t *items, const uint8_t *accept, int n,
                       cudaStream_t st)
{
  if (n <= 0) return;
  k_hky_commit<<<n, 128, 0, st>>>(P, items, accept);
}
