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
// Fast form: every branch term is evaluated in the log domain in float-float
// arithmetic (ff.cuh), so the exp(x) of the large-x polynomials cancels
// against -x analytically and no FP64 instruction is issued per branch; the
// float-float terms are summed per chain-locus and converted to FP64 once.
// Branches outside the float-float range (x below 1e-15 with |d| >= 2, or a
// Miller value the reference would take below 1e-300) take the FP64 path.
// FP64 form: the reference algorithm in FP64, one thread per branch.
#include <cfloat>

#include "ff.cuh"
#include "internal.h"

namespace {

constexpr int SW_BS = 128;
constexpr double BESSI_MIN = -1e+100;  // imamp.hpp:173

__constant__ FFConsts c_ff;
__constant__ double c_i0s[7], c_i0l[9], c_i1s[7], c_i1l[9];

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
// log(bessi0(x)) - x
__device__ ff l0_ff(ff x)
{
  if (x.hi < 3.75f) {
    ff y = ff_mul(x, ffc(c_ff.inv375));
    y = ff_mul(y, y);
    return ff_sub(ff_log(ff_horner(c_ff.i0s, 7, y), c_ff), x);
  }
  ff z = ff_div(ff_from(3.75f), x);
  ff lx = ff_log(x, c_ff);
  return ff_sub(ff_log(ff_horner(c_ff.i0l, 9, z), c_ff), ff_make(0.5f * lx.hi, 0.5f * lx.lo));
}

// log(bessi1(x)) - x, x > 0
__device__ ff l1_ff(ff x)
{
  if (x.hi < 3.75f) {
    ff y = ff_mul(x, ffc(c_ff.inv375));
    y = ff_mul(y, y);
    return ff_sub(ff_add(ff_log(x, c_ff), ff_log(ff_horner(c_ff.i1s, 7, y), c_ff)), x);
  }
  ff z = ff_div(ff_from(3.75f), x);
  ff lx = ff_log(x, c_ff);
  return ff_sub(ff_log(ff_horner(c_ff.i1l, 9, z), c_ff), ff_make(0.5f * lx.hi, 0.5f * lx.lo));
}

// Returns false when the branch must be evaluated in FP64.
__device__ bool term_ff(int d, ff x, ff *out, bool *zero)
{
  int n = abs(d);
  if (x.hi > 700.0f || (x.hi == 700.0f && x.lo > 0.0f)) {
    *out = ff_sub(ffc(c_ff.logmydblmax), x);
    return true;
  }
  if (n == 0) {
    *out = l0_ff(x);
    return true;
  }
  if (x.hi == 0.0f) {
    *zero = true;
    *out = ff_from(0.0f);
    return true;
  }
  if (n == 1) {
    *out = l1_ff(x);
    return true;
  }
  if (x.hi < 1e-15f) return false;
  // Miller recurrence; the reference's 1e10 rescaling of `ans` after it is
  // captured is counted instead of applied, keeping it in float range
  ff tox = ff_div(ff_from(2.0f), x);
  ff bip = ff_from(0.0f), bi = ff_from(1.0f), ans = ff_from(0.0f);
  const ff big = ffc(c_ff.e10m);  // 1e-10
  int scaled = 0;
  bool got = false;
  for (int j = 2 * (n + (int)sqrtf(40.0f * n)); j > 0; j--) {
    ff bim = ff_add(bip, ff_mul(ff_mul_f(tox, (float)j), bi));
    bip = bi;
    bi = bim;
    if (bi.hi > 1.0e10f) {
      if (got) scaled++;
      bi = ff_mul(bi, big);
      bip = ff_mul(bip, big);
    }
    if (j == n) {
      ans = bip;
      got = true;
    }
  }
  // the reference's FP64 `ans` is ans * 1e-10^scaled: leave the range where
  // that value is normal to the FP64 path
  if (!(ans.hi > 0.0f) || __log10f(ans.hi) - 10.0f * scaled < -300.0f) return false;
  // log(ans) - log(bi): the ratio itself may leave float range
  ff r = ff_sub(ff_log(ans, c_ff), ff_log(bi, c_ff));
  ff s = ff_mul_f(ffc(c_ff.ln1e10), (float)scaled);
  *out = ff_add(ff_sub(r, s), l0_ff(x));
  return true;
}

__device__ __forceinline__ ff branch_ff(const NodeRec &nd, const float2 *t, int c, ff tr)
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

__global__ void __launch_bounds__(SW_BS) k_sw_fast(Pools P, const ReqDev *reqs, double *result,
                                                   int32_t *status)
{
  const ReqDev R = reqs[blockIdx.x];
  const double tr = R.par;
  const ItemDev it = P.items[R.item];
  const int nl = 2 * it.n - 1;
  const NodeRec *nd = P.nodes + it.node_off;
  const float2 *tff = P.tff + it.node_off;
  const double *t64 = P.t64 + it.node_off;
  const int32_t *A = P.alleles + it.al_off + (size_t)R.ai * nl;
  float2 *dl = reinterpret_cast<float2 *>(P.dlike) + it.dl_off + (size_t)R.ai * nl;
  const float uh = (float)R.u;
  const ff u = ff_make(uh, (float)(R.u - (double)uh));
  const float trh = (float)tr;
  const ff trf = ff_make(trh, (float)(tr - (double)trh));
  ff acc = ff_from(0.0f);
  bool zero = false;
  for (int c = threadIdx.x; c < nl; c += SW_BS) {
    NodeRec r = nd[c];
    if (r.down < 0) {
      dl[c] = make_float2(0.f, 0.f);
      continue;
    }
    int d = A[c] - A[r.down];
    ff x = ff_mul(branch_ff(r, tff, c, trf), u);
    ff v;
    bool z = false;
    if (!term_ff(d, x, &v, &z)) {  // rare: exact FP64 evaluation
      double t = (r.up0 < 0) ? t64[c] * tr : tr * (t64[c] - t64[r.up0]);
      double w = term_64(d, t * R.u, &z);
      float wh = (float)w;
      v = ff_make(wh, (float)(w - (double)wh));
    }
    if (z) {
      zero = true;
      v = ff_make(-1e30f, 0.f);  // placeholder: the total is -DBL_MAX anyway
      dl[c] = make_float2(-INFINITY, 0.f);
    } else {
      dl[c] = make_float2(v.hi, v.lo);
    }
    acc = ff_add(acc, v);
  }
  __shared__ float2 red[SW_BS / 32];
  __shared__ int anyzero;
  if (threadIdx.x == 0) anyzero = 0;
  __syncthreads();
  acc = warp_sum_ff(acc);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = make_float2(acc.hi, acc.lo);
  if (zero) anyzero = 1;
  __syncthreads();
  if (threadIdx.x == 0) {
    ff s = ff_from(0.0f);
    for (int w = 0; w < SW_BS / 32; w++) s = ff_add(s, ff_make(red[w].x, red[w].y));
    result[blockIdx.x] = anyzero ? -DBL_MAX : ff_to_double(s);
    P.pdg_new[R.item] = result[blockIdx.x];
    status[blockIdx.x] = anyzero ? IMA_EVAL_SW_ZERO : IMA_EVAL_OK;
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
  return 0;
}

void launch_sw_fast(const Pools &P, const ReqDev *reqs, int nreq, double *result,
                    int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  k_sw_fast<<<nreq, SW_BS, 0, st>>>(P, reqs, result, status);
}

void launch_sw_fp64(const Pools &P, const ReqDev *reqs, int nreq, double *result,
                    int32_t *status, cudaStream_t st)
{
  if (nreq <= 0) return;
  k_sw_fp64<<<nreq, SW_BS, 0, st>>>(P, reqs, result, status);
}
