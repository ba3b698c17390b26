// k_sw.cu -- stepwise-mutation likelihood (likelihoodSW, calc_prob_data.cpp:841-909).
//
// Per non-root branch i with allele difference d = A[i] - A[down[i]] and
// x = t*u:  dlikeA = -x + log(bessi(|d|, x)), where bessi is the reference's
// modified Bessel function (utilities.cpp:54-124 and 1449-1496):
// Abramowitz & Stegun 9.8.1-9.8.4 polynomials for |d| <= 1 and Miller's
// downward recurrence from j = 2(|d| + floor(sqrt(40|d|))) with rescaling for
// |d| >= 2.  A zero Bessel value makes the branch term -1e100 and the locus
// total -DBL_MAX.  There is no pruning: internal alleles are chain state.
//
// Fast form: every branch term is evaluated in the log domain, so the
// exp(x) of the large-x polynomials cancels against -x analytically and no
// FP64 instruction is issued per branch; the terms are summed per
// chain-locus in float-float and converted to FP64 once.  Short branches
// (x <= 0.375, y = (x / 3.75)^2 <= 0.01: 81% of them in the 100-locus
// benchmark) take a cheaper form: bessi0 = 1 + u0(y), bessi1 = x (1 + u1(y))
// / 2 with u(y) <= 0.036 and log(1 + u) from its series, the leading terms
// in float-float and the rest in FP32.  Longer branches use the float-float
// core (A&S polynomial and table log).  Both keep about 1e-11 per branch.
// Branches outside the float-float range (x below 1e-15 with |d| >= 2, or a
// Miller value the reference would take below 1e-300) take the FP64 path.
// FP64 form: the reference algorithm in FP64, one thread per branch.
#include <algorithm>
#include <mutex>
#include <cfloat>

#include "ff.cuh"
#include "internal.h"

namespace {

constexpr int SW_BS = 128;
constexpr double BESSI_MIN = -1e+100;  // imamp.hpp:173

__constant__ FFConsts c_ff;
__constant__ double c_i0s[7], c_i0l[9], c_i1s[7], c_i1l[9];
__constant__ float c_cheap[2][7];  // A&S 9.8.1 / 9.8.3 coefficients over their constant term
__constant__ float2 c_cheap1[2];   // the first of them as float-float
constexpr float SW_CHEAP_Y = 0.01f;

// ---------------------------------------------------------------- FP64
__device__ __forceinline__ double horner64(const double *c, int m, double y)
{
  double r = c[m - 1];
  for (int k = m - 2; k >= 0; k--) r = c[k] + y * r;
  return r;
}

__device__ double bessi0_64(double x)
{
  double ax = fabs(x);
  if (ax < 3.75) {
    double y = x / 3.75;
    y *= y;
    return horner64(c_i0s, 7, y);
  }
  double y = 3.75 / ax;
  return (exp(ax) / sqrt(ax)) * horner64(c_i0l, 9, y);
}

__device__ double bessi1_64(double x)
{
  double ax = fabs(x), ans;
  if (ax < 3.75) {
    double y = x / 3.75;
    y *= y;
    ans = ax * horner64(c_i1s, 7, y);
  } else {
    double y = 3.75 / ax;
    ans = horner64(c_i1l, 9, y) * (exp(ax) / sqrt(ax));
  }
  return x < 0.0 ? -ans : ans;
}

__device__ double bessi_64(int n, double x)
{
  n = abs(n);
  if (x > 700) return DBL_MAX / 1e10;
  if (n == 0) return bessi0_64(x);
  if (n == 1) return bessi1_64(x);
  if (x == 0.0) return 0.0;
  double tox = 2.0 / fabs(x);
  double bip = 0.0, ans = 0.0, bi = 1.0;
  for (int j = 2 * (n + (int)sqrt(40.0 * n)); j > 0; j--) {
    double bim = bip + j * tox * bi;
    bip = bi;
    bi = bim;
    if (fabs(bi) > 1.0e10) {
      ans *= 1.0e-10;
      bi *= 1.0e-10;
      bip *= 1.0e-10;
    }
    if (j == n) ans = bip;
  }
  ans *= bessi0_64(x) / bi;
  return (x < 0.0 && (n & 1)) ? -ans : ans;
}

// branch term; *zero set when the Bessel value is not positive
__device__ __forceinline__ double term_64(int d, double x, bool *zero)
{
  double b = bessi_64(d, x);
  if (!(b > 0.0)) {
    *zero = true;
    return BESSI_MIN;
  }
  return -x + log(b);
}

// --------------------------------------------------------- float-float
// Coefficient tables of the four |d| <= 1 regimes, zero-padded to 9 terms:
// [d01 * 2 + small]: d=0 large, d=0 small, d=1 large, d=1 small.
struct SwTables {
  float2 c[4][9];
};

__device__ __forceinline__ ff ff_add_fast(ff a, ff b)  // no cancellation expected
{
  ff s = two_sum(a.hi, b.hi);
  float e = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, e);
}

// log(bessi(n, x)) - x for n <= 1 (and the log(bessi0) - x part for n >= 2),
// one code path for every lane: the regime only selects the argument and
// the coefficient table.
//   x < 3.75:  bessi0 = P0(y), bessi1 = x P1(y), y = (x / 3.75)^2
//   x >= 3.75: bessi_n = exp(x) / sqrt(x) Q_n(z), z = 3.75 / x
__device__ __forceinline__ ff sw_core(ff x, int d01, const SwTables &T)
{
  const bool small = x.hi < 3.75f;
  const ff xs = (x.hi > 0.f) ? x : ff_from(1.0f);
  ff y = ff_mul(x, ffc(c_ff.inv375));
  y = ff_mul(y, y);
  // the division (x >= 3.75: 1% of branches) and log x (x >= 3.75 or
  // |d| = 1) only where a lane needs them
  ff arg = y;
  if (!small) arg = ff_div(ff_from(3.75f), xs);
  const float2 *c = T.c[d01 * 2 + (small ? 1 : 0)];
  ff acc = ffc(c[8]);
#pragma unroll
  for (int k = 7; k >= 0; k--) acc = ff_add_fast(ff_mul(acc, arg), ffc(c[k]));
  ff lp = ff_log(acc, c_ff);
  ff lx = ff_from(0.0f);
  if (!small || d01) lx = ff_log(xs, c_ff);
  ff tail = small ? (d01 ? ff_sub(lx, x) : ff_neg(x)) : ff_make(-0.5f * lx.hi, -0.5f * lx.lo);
  return ff_add(lp, tail);
}

// log(bessi_d01(x)) - x for a short branch (y = (x / 3.75)^2 <= SW_CHEAP_Y):
// with the polynomial written as c0 (1 + u), u = c1' y + y^2 (c2' + c3' y +
// ...), c_k' = c_k / c0, log(1 + u) (|u| <= 0.036) from its series: u and
// u - u^2/2 in float-float, u^3 (1/3 - u/4 + ... - u^5/8) in FP32 (its
// weight is below 1.6e-5, the first term left out below 1.2e-14).  About
// 1e-11 per branch, like the float-float core, at a quarter of its work.
__device__ __forceinline__ ff sw_cheap(ff x, ff y, int d01)
{
  const float *c = c_cheap[d01];
  float t = c[6];
#pragma unroll
  for (int k = 5; k >= 2; k--) t = __fmaf_rn(t, y.hi, c[k]);
  const ff u = ff_add_f(ff_mul(ffc(c_cheap1[d01]), y), y.hi * y.hi * t);
  const ff u2 = ff_mul(u, u);
  const float h = u.hi;
  const float s3 = h * h * h *
                   (0.33333334f + h * (-0.25f + h * (0.2f + h * (-0.16666667f + h * (0.14285715f + h * -0.125f)))));
  const ff l = ff_add_f(ff_sub(u, ff_make(0.5f * u2.hi, 0.5f * u2.lo)), s3);
  ff v = ff_sub(l, x);
  if (d01) v = ff_add(v, ff_sub(ff_log(x, c_ff), ff_make(LN2_HI, LN2_LO)));  // + log(x / 2)
  return v;
}

// log(ans / bi) of the reference's Miller recurrence and its 1e10 rescaling
// count; false when the value must come from the FP64 path.
__device__ bool sw_miller(int n, ff x, ff *out)
{
  if (x.hi < 1e-15f) return false;
  ff tox = ff_div(ff_from(2.0f), x);
  ff bip = ff_from(0.0f), bi = ff_from(1.0f), ans = ff_from(0.0f);
  const ff tiny = ffc(c_ff.e10m);  // 1e-10
  int scaled = 0;
  bool got = false;
  for (int j = 2 * (n + (int)sqrtf(40.0f * n)); j > 0; j--) {
    ff bim = ff_add_fast(bip, ff_mul_f(ff_mul(tox, bi), (float)j));
    bip = bi;
    bi = bim;
    if (bi.hi > 1.0e10f) {
      if (got) scaled++;
      bi = ff_mul(bi, tiny);
      bip = ff_mul(bip, tiny);
    }
    if (j == n) {
      ans = bip;
      got = true;
    }
  }
  // the reference's FP64 `ans` is ans * 1e-10^scaled: leave the range where
  // that value is not a normal double to the FP64 path
  if (!(ans.hi > 0.0f) || __log10f(ans.hi) - 10.0f * scaled < -300.0f) return false;
  ff r = ff_sub(ff_log(ans, c_ff), ff_log(bi, c_ff));
  *out = ff_sub(r, ff_mul_f(ffc(c_ff.ln1e10), (float)scaled));
  return true;
}

__device__ __forceinline__ ff branch_len_ff(const NodeRec &nd, const float2 *t, int c, ff tr)
{
  ff a = ff_make(t[c].x, t[c].y);
  if (nd.up0 < 0) return ff_mul(a, tr);
  float2 b = t[nd.up0];
  return ff_mul(tr, ff_sub(a, ff_make(b.x, b.y)));
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ ff warp_sum_ff(ff v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ff w = ff_make(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
    v = ff_add(v, w);
  }
  return v;
}

// Per CTA of 256 threads, `per` chain-loci (the host picks it so that the
// batch is one wave of resident CTAs), in three phases:
//  (A) classify: every branch's x = t tr u (float-float) goes to shared
//      memory and the branch to one of four task lists, the longest work
//      first: Miller recurrences (|d| >= 2), the float-float core (y > 0.01),
//      short branches with |d| = 1 (series plus log x), short branches with
//      d = 0 (series only);
//  (T) tasks: warps take 32 consecutive tasks at a time from a shared
//      counter, so lanes of a warp run the same form and warps that drew
//      long recurrences take fewer tasks; each task writes its branch's term;
//  (C) one warp per chain-locus sums its branch terms in float-float.
// Lists 0 and 1 share one int32 array, filled from its two ends, and lists
// 2 and 3 another; an entry is the branch (low 16 bits) and min(|d|, 65535).
constexpr int SW_NT = 256;  // threads per CTA
template <int MAXI, int MINB>
__global__ void __launch_bounds__(SW_NT, MINB) k_sw_fast(Pools P, const ReqDev *reqs, int nreq, int per,
                                                           double *result, int32_t *status, int maxb)
{
  __shared__ SwTables T;
  extern __shared__ __align__(16) char sw_smem[];
  float2 *vals = reinterpret_cast<float2 *>(sw_smem);          // x, then the branch term
  int32_t *q01 = reinterpret_cast<int32_t *>(vals + maxb);      // Miller from the front, core from the back
  int32_t *q23 = q01 + maxb;                                   // |d| = 1 short from the front, d = 0 from the back
  __shared__ int qn[4], next;
  __shared__ int bstart[MAXI + 1];
  __shared__ int zero[MAXI];
  __shared__ float2 uff[MAXI], trff[MAXI];
  // each chain-locus's node base and marker allele base, staged once so a
  // branch's loads start from shared memory (request -> item -> node would
  // be two more dependent global loads per branch)
  __shared__ int s_noff[MAXI], s_alb[MAXI], s_nl[MAXI];
  const int r0 = blockIdx.x * per;
  const int nit = min(per, nreq - r0);
  const int tid = threadIdx.x;
  if (tid < 36) {
    int t = tid / 9, k = tid % 9;
    int d01 = t >> 1, small = t & 1;
    int m = small ? 7 : 9;
    float2 v = make_float2(0.f, 0.f);
    if (k < m) v = d01 ? (small ? c_ff.i1s[k] : c_ff.i1l[k]) : (small ? c_ff.i0s[k] : c_ff.i0l[k]);
    T.c[t][k] = v;
  }
  if (tid < 4) qn[tid] = 0;
  if (tid == 0) next = 0;
  if (tid < nit) {
    const ReqDev R = reqs[r0 + tid];
    const ItemDev it = P.items[R.item];
    const int nl = 2 * it.n - 1;
    s_noff[tid] = it.node_off;
    s_alb[tid] = it.al_off + R.ai * nl;
    s_nl[tid] = nl;
    float uh = (float)R.u, th = (float)R.par;
    uff[tid] = make_float2(uh, (float)(R.u - (double)uh));
    trff[tid] = make_float2(th, (float)(R.par - (double)th));
    zero[tid] = 0;
  }
  __syncthreads();
  if (tid == 0) {
    int b = 0;
    for (int i = 0; i < nit; i++) {
      bstart[i] = b;
      b += s_nl[i];
    }
    bstart[nit] = b;
  }
  __syncthreads();
  const int total = bstart[nit];
  // ---- phase A: classify (a thread's branches only move forward: its
  // chain-locus index carries over)
  {
    int i = 0;
    for (int b = tid; b < total; b += SW_NT) {
      while (b >= bstart[i + 1]) i++;
      const int c = b - bstart[i];
      const NodeRec nd = P.nodes[s_noff[i] + c];
      float2 out = make_float2(0.f, 0.f);
      if (nd.down >= 0) {
        const int32_t *A = P.alleles + s_alb[i];
        const int n = abs(A[c] - A[nd.down]);
        const ff x = ff_mul(branch_len_ff(nd, P.tff + s_noff[i], c, ffc(trff[i])), ffc(uff[i]));
        if (x.hi > 700.0f || (x.hi == 700.0f && x.lo > 0.0f)) {
          const ff v = ff_sub(ffc(c_ff.logmydblmax), x);
          out = make_float2(v.hi, v.lo);
        } else if (n >= 1 && x.hi == 0.0f) {
          zero[i] = 1;
          out = make_float2(-INFINITY, 0.f);
        } else {
          out = make_float2(x.hi, x.lo);
          const ff xq = ff_mul(x, ffc(c_ff.inv375));  // x / 3.75
          const float yh = ff_mul(xq, xq).hi;
          const int e = b | (min(n, 65535) << 16);
          if (n >= 2) q01[atomicAdd(&qn[0], 1)] = e;
          else if (yh > SW_CHEAP_Y) q01[maxb - 1 - atomicAdd(&qn[1], 1)] = e;
          else if (n == 1) q23[atomicAdd(&qn[2], 1)] = e;
          else q23[maxb - 1 - atomicAdd(&qn[3], 1)] = e;
        }
      }
      vals[b] = out;
    }
  }
  __syncthreads();
  // ---- phase T: the four lists as one sequence of tasks
  const int n0 = qn[0], n1 = n0 + qn[1], n2 = n1 + qn[2], ntask = n2 + qn[3];
  const int lane = tid & 31;
  for (;;) {
    int t0 = 0;
    if (lane == 0) t0 = atomicAdd(&next, 32);
    t0 = __shfl_sync(0xffffffffu, t0, 0);
    if (t0 >= ntask) break;
    const int t = t0 + lane;
    if (t >= ntask) continue;
    const int e = t < n0 ? q01[t] : t < n1 ? q01[maxb - 1 - (t - n0)] : t < n2 ? q23[t - n1] : q23[maxb - 1 - (t - n2)];
    const int b = e & 0xffff;
    int n = (int)((unsigned)e >> 16);
    const float2 xv = vals[b];
    const ff x = ff_make(xv.x, xv.y);
    const ff xq = ff_mul(x, ffc(c_ff.inv375));
    const ff y = ff_mul(xq, xq);
    ff v;
    if (t >= n1) {  // short branches
      v = sw_cheap(x, y, t < n2 ? 1 : 0);
    } else if (t >= n0) {  // the float-float core, |d| <= 1
      v = sw_core(x, n, T);
    } else {  // |d| >= 2: the d = 0 term and the Miller ratio
      int i = 0;
      while (b >= bstart[i + 1]) i++;
      const int c = b - bstart[i];
      if (n == 65535) {  // the exact difference from the alleles
        const NodeRec nd = P.nodes[s_noff[i] + c];
        const int32_t *A = P.alleles + s_alb[i];
        n = abs(A[c] - A[nd.down]);
      }
      const ff base = (y.hi <= SW_CHEAP_Y) ? sw_cheap(x, y, 0) : sw_core(x, 0, T);
      ff r;
      if (sw_miller(n, x, &r)) {
        v = ff_add(base, r);
      } else {  // rare: the reference's FP64 arithmetic
        const NodeRec nd = P.nodes[s_noff[i] + c];
        const ReqDev &R = reqs[r0 + i];
        const double *t64 = P.t64 + s_noff[i];
        double tt = (nd.up0 < 0) ? t64[c] * R.par : R.par * (t64[c] - t64[nd.up0]);
        bool z = false;
        double w = term_64(n, tt * R.u, &z);
        if (z) {
          zero[i] = 1;
          v = ff_make(-INFINITY, 0.f);
        } else {
          float wh = (float)w;
          v = ff_make(wh, (float)(w - (double)wh));
        }
      }
    }
    vals[b] = make_float2(v.hi, v.lo);
  }
  __syncthreads();
  // ---- phase C: per chain-locus sums, dlikeA write-back
  for (int w = tid >> 5; w < nit; w += SW_NT / 32) {
    const ReqDev &R = reqs[r0 + w];
    const ItemDev it = P.items[R.item];
    const int nl = 2 * it.n - 1;
    float2 *dl = reinterpret_cast<float2 *>(P.dlike) + it.dl_off + (size_t)R.ai * nl;
    ff acc = ff_from(0.f);
    for (int c = lane; c < nl; c += 32) {
      float2 v = vals[bstart[w] + c];
      dl[c] = v;
      if (v.x != -INFINITY) acc = ff_add(acc, ffc(v));
    }
    acc = warp_sum_ff(acc);
    if (lane == 0) {
      double res = zero[w] ? -DBL_MAX : ff_to_double(acc);
      result[r0 + w] = res;
      status[r0 + w] = zero[w] ? IMA_EVAL_SW_ZERO : IMA_EVAL_OK;
      P.pdg_new[R.item] = res;
    }
  }
}

__global__ void __launch_bounds__(SW_BS) k_sw_fp64(Pools P, const ReqDev *reqs, double *result,
                                                   int32_t *status)
{
  const ReqDev R = reqs[blockIdx.x];
  const double tr = R.par;
  const ItemDev it = P.items[R.item];
  const int nl = 2 * it.n - 1;
  const NodeRec *nd = P.nodes + it.node_off;
  const double *t64 = P.t64 + it.node_off;
  const int32_t *A = P.alleles + it.al_off + (size_t)R.ai * nl;
  double *dl = P.dlike + it.dl_off + (size_t)R.ai * nl;
  double acc = 0.0;
  bool zero = false;
  for (int c = threadIdx.x; c < nl; c += SW_BS) {
    NodeRec r = nd[c];
    if (r.down < 0) {
      dl[c] = 0.0;
      continue;
    }
    int d = A[c] - A[r.down];
    double t = (r.up0 < 0) ? t64[c] * tr : tr * (t64[c] - t64[r.up0]);
    double v = term_64(d, t * R.u, &zero);
    dl[c] = v;
    acc += v;
  }
  __shared__ double red[SW_BS / 32];
  __shared__ int anyzero;
  if (threadIdx.x == 0) anyzero = 0;
  __syncthreads();
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  if (zero) anyzero = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < SW_BS / 32; w++) s += red[w];
    result[blockIdx.x] = anyzero ? -DBL_MAX : s;
    P.pdg_new[R.item] = result[blockIdx.x];
    status[blockIdx.x] = anyzero ? IMA_EVAL_SW_ZERO : IMA_EVAL_OK;
  }
}

// Abramowitz & Stegun 9.8.1-9.8.4 coefficients, lowest order first, as the
// reference writes them (utilities.cpp:54-124).
const double AS_I0S[7] = {1.0, 3.5156229, 3.0899424, 1.2067492, 0.2659732, 0.360768e-1, 0.45813e-2};
const double AS_I0L[9] = {0.39894228, 0.1328592e-1, 0.225319e-2, -0.157565e-2, 0.916281e-2,
                          -0.2057706e-1, 0.2635537e-1, -0.1647633e-1, 0.392377e-2};
const double AS_I1S[7] = {0.5, 0.87890594, 0.51498869, 0.15084934, 0.2658733e-1, 0.301532e-2,
                          0.32411e-3};
const double AS_I1L[9] = {0.39894228, -0.3988024e-1, -0.362018e-2, 0.163801e-2, -0.1031555e-1,
                          0.2282967e-1, -0.2895312e-1, 0.1787654e-1, -0.420059e-2};

float2 split(double v)
{
  float h = (float)v;
  return make_float2(h, (float)(v - (double)h));
}


// finishSWupdateA (update_gtree_common.cpp:2219-2362) for a genealogy
// update's proposal on a stepwise locus (one marker), a warp per chain, lane
// 0 in the reference's order: the freed node's new allele (geometric around
// its neighbours' alleles, sign by bitran, clamped to the locus's range), the
// terms of the old sister and the three moved branches in FP64 with the
// reference's Bessel functions, the allele proposal's Hastings term, then the
// acceptance uniform, next in the generator's stream.  Products and sums are
// rounded one at a time (no contraction), as the reference writes them.
__global__ void __launch_bounds__(32) k_ug_sw(UgArgs a)
{
  const int w = blockIdx.x, lane = threadIdx.x;
  const int ci = a.chains[w], item = ci * a.nloci + a.locus;
  const ItemDev it = a.items[item];
  const int n = it.n, maxnl = 2 * a.maxn;
  const NodeRec *nd = a.nodes + it.node_off;
  const double *t = a.t64 + it.node_off;
  const int32_t *A = a.alleles + it.al_off;
  double *dl = a.dlike + it.dl_off;
  const int32_t *bka = a.bk_A + (size_t)w * maxnl;
  const double *bkd = a.bk_dl + (size_t)w * maxnl;
  const NodeRec *bkn = a.bk_nodes + (size_t)w * maxnl;
  const int32_t *eo = a.edges + 4 * (size_t)w;
  const int edge = eo[0], freed = eo[1], oldsis = eo[2], newsis = eo[3];
  const double u = a.u_cl[(size_t)w * a.nloci + a.locus];
  const int e[3] = {edge, newsis, nd[edge].down};
  // the proposal drew the freed node's allele (bka holds the alleles before)
  const int oldA = bka[freed], newA = A[freed], dA = newA - oldA;
  double holdsis = 0.0, oldlikeadj = 0.0, geotermnew = 0.0;
  bool fdown = false;
  if (lane == 0) {
    holdsis = (newsis != oldsis) ? dl[newsis] : 0.0;
    fdown = bkn[freed].down != -1;
    const double cp2 = fdown ? bkd[freed] : 0.0;
    oldlikeadj = bkd[edge] + bkd[oldsis] + cp2 + holdsis;
    int wsumdiff = 0, j = 0;
    for (int i = 0; i < 3; i++)
      if (nd[e[i]].down != -1) {
        wsumdiff += abs((i < 2 ? bka[e[i]] : bka[nd[e[i]].down]) - oldA);
        j++;
      }
    geotermnew = j / ((double)(wsumdiff + j));
    if (geotermnew > 0.95) geotermnew = 0.95;
  }
  // The four branch terms, one lane each through one code path: lane 0 the
  // old sister's branch, lane 1 + i the branch above e[i], from the alleles
  // after the draw.  -(len * u) is the reference's (-len) * u exactly:
  // rounding to nearest is symmetric in sign.
  auto allele = [&](int v) { return A[v]; };
  bool has = false;
  int d = 0;
  double len = 0.0;
  if (lane == 0) {
    if (nd[oldsis].down != -1 && oldsis != newsis) {
      len = t[oldsis] - (oldsis >= n ? t[nd[oldsis].up0] : 0.0);
      d = allele(oldsis) - allele(nd[oldsis].down);
      has = true;
    }
  } else if (lane < 4) {
    const int v = lane == 1 ? e[0] : (lane == 2 ? e[1] : e[2]);
    if (nd[v].down != -1) {
      len = t[v] - (v >= n ? t[nd[v].up0] : 0.0);
      d = (lane < 3 ? allele(v) : allele(nd[v].down)) - newA;
      has = true;
    }
  }
  double term = 0.0;
  if (has) {
    const double x = len * u;
    term = __dadd_rn(-x, log(bessi_64(d, x)));
  }
  const unsigned hasm = __ballot_sync(0xffffffffu, has);
  const double tm0 = __shfl_sync(0xffffffffu, term, 0), tm1 = __shfl_sync(0xffffffffu, term, 1);
  const double tm2 = __shfl_sync(0xffffffffu, term, 2), tm3 = __shfl_sync(0xffffffffu, term, 3);
  if (lane == 0) {
    // written and summed in the reference's order (finishSWupdateA)
    dl[oldsis] = tm0;
    double likeadj = tm0;
    const double tmi[3] = {tm1, tm2, tm3};
    for (int i = 0; i < 3; i++)
      if ((hasm >> (i + 1)) & 1) {
        dl[e[i]] = tmi[i];
        likeadj += tmi[i];
      }
    const int holddownA = fdown ? bka[bkn[freed].down] : -1;
    int wsumdiff = abs(bka[edge] - newA) + abs(bka[oldsis] - newA);
    int j = 2;
    if (fdown) {
      wsumdiff += abs(holddownA - newA);
      j++;
    }
    double geotermold = j / ((double)(wsumdiff + j));
    if (geotermold > 0.95) geotermold = 0.95;
    const double adA = (double)abs(dA);
    const double at = __dadd_rn(__dmul_rn(adA, log(1 - geotermold)), log(geotermold)) -
                      __dadd_rn(__dmul_rn(adA, log(1 - geotermnew)), log(geotermnew));
    a.aterm[w] = at;
    a.holdsis[w] = holdsis;
    a.swnew[w] = 0.0 + (a.pdg[item] + __dadd_rn(likeadj, -oldlikeadj));
  }
}

}  // namespace

// Uploads the coefficient and table constants (once per device).
int sw_init_tables()
{
  FFConsts K;
  for (int i = 0; i < 64; i++) K.logtab[i] = split(std::log(1.0 + (2.0 * i + 1.0) / 128.0));
  for (int i = 0; i < 7; i++) { K.i0s[i] = split(AS_I0S[i]); K.i1s[i] = split(AS_I1S[i]); }
  for (int i = 0; i < 9; i++) { K.i0l[i] = split(AS_I0L[i]); K.i1l[i] = split(AS_I1L[i]); }
  const double ln2 = 0.69314718055994530941723212146;
  const double a = 355.0 / 512.0;
  K.ln2a = make_float2((float)a, (float)(ln2 - a));
  K.ln2b = (float)(ln2 - a - (double)(float)(ln2 - a));
  K.ln1e10 = split(std::log(1e10));
  K.logmydblmax = split(std::log(DBL_MAX / 1e10));
  K.inv375 = split(1.0 / 3.75);
  K.e10m = split(1e-10);
  if (cudaMemcpyToSymbol(c_ff, &K, sizeof(K)) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_i0s, AS_I0S, sizeof(AS_I0S)) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_i0l, AS_I0L, sizeof(AS_I0L)) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_i1s, AS_I1S, sizeof(AS_I1S)) != cudaSuccess) return -1;
  if (cudaMemcpyToSymbol(c_i1l, AS_I1L, sizeof(AS_I1L)) != cudaSuccess) return -1;
  float cheap[2][7];
  for (int k = 0; k < 7; k++) {
    cheap[0][k] = (float)(AS_I0S[k] / AS_I0S[0]);
    cheap[1][k] = (float)(AS_I1S[k] / AS_I1S[0]);
  }
  if (cudaMemcpyToSymbol(c_cheap, cheap, sizeof(cheap)) != cudaSuccess) return -1;
  const float2 c1[2] = {split(AS_I0S[1] / AS_I0S[0]), split(AS_I1S[1] / AS_I1S[0])};
  if (cudaMemcpyToSymbol(c_cheap1, c1, sizeof(c1)) != cudaSuccess) return -1;
  return 0;
}

// Chain-loci per CTA that make the batch one wave of resident CTAs (at most
// MAXI, and few enough that a task entry's 16 bits index every branch).
// The answer is remembered for the last few (device, batch size, branch
// count): a batch replayed step after step asks the occupancy calculator
// once.
template <int MAXI, int MINB>
static int sw_balanced_per(int nreq, int nlb)
{
  struct Memo {
    int dev = -1, nreq = 0, nlb = 0, per = 0;
  };
  static std::mutex mu;
  static Memo memo[8];  // the last few shapes, replaced in turn
  static int turn = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  {
    std::lock_guard<std::mutex> lk(mu);
    for (const Memo &m : memo)
      if (m.dev == dev && m.nreq == nreq && m.nlb == nlb) return m.per;
  }
  int nsm = 152;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int cap = std::min(MAXI, 32767 / nlb);
  int per = std::max(1, std::min(cap, (nreq + 4 * nsm - 1) / (4 * nsm)));
  for (int round = 0; round < 3; round++) {
    const size_t sm = (size_t)per * nlb * (sizeof(float2) + 2 * sizeof(int32_t));
    if (sm > 48 * 1024)
      cudaFuncSetAttribute(k_sw_fast<MAXI, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_sw_fast<MAXI, MINB>, SW_NT, sm) != cudaSuccess) nb = 1;
    nb = std::max(1, nb);
    const long long slots = (long long)nsm * nb;
    const int want = std::max(1, std::min(cap, (int)((nreq + slots - 1) / slots)));
    if (want == per) break;
    per = want;
  }
  std::lock_guard<std::mutex> lk(mu);
  memo[turn] = Memo{dev, nreq, nlb, per};
  turn = (turn + 1) % 8;
  return per;
}

template <int MAXI, int MINB>
static void sw_fast_launch(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int per, double *result,
                           int32_t *status, cudaStream_t st)
{
  const int nlb = 2 * maxn - 1;
  if (per <= 0) per = sw_balanced_per<MAXI, MINB>(nreq, nlb);
  per = std::max(1, std::min(per, std::min(MAXI, 32767 / nlb)));
  const int maxb = per * nlb;
  const size_t sm = (size_t)maxb * (sizeof(float2) + 2 * sizeof(int32_t));
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_sw_fast<MAXI, MINB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_sw_fast<MAXI, MINB><<<(nreq + per - 1) / per, SW_NT, sm, st>>>(P, reqs, nreq, per, result, status, maxb);
}

void launch_sw_fast(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int variant, double *result,
                    int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  // 0: one wave, registers for 5 CTAs of 256 threads per SM; 1: one wave,
  // registers for 6; 2: 8 chain-loci per CTA whatever the wave count
  if (variant == 1) sw_fast_launch<16, 6>(P, reqs, nreq, maxn, 0, result, status, st);
  else if (variant == 2) sw_fast_launch<8, 5>(P, reqs, nreq, maxn, 8, result, status, st);
  else sw_fast_launch<16, 5>(P, reqs, nreq, maxn, 0, result, status, st);
}

void launch_ug_sw(const UgArgs &a, cudaStream_t st) { k_ug_sw<<<a.nch, 32, 0, st>>>(a); }

void launch_sw_fp64(const Pools &P, const ReqDev *reqs, int nreq, double *result,
                    int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  k_sw_fp64<<<nreq, SW_BS, 0, st>>>(P, reqs, result, status);
}
