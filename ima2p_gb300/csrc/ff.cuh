// ff.cuh -- float-float ("double-FP32") arithmetic for sm_103a, whose FP64
// pipe runs at 1/64 of the FP32 rate.  A value is hi + lo with |lo| <= ulp(hi)/2,
// about 46 significant bits.  Error-free transformations after Knuth (TwoSum),
// Dekker (Fast2Sum) and the FMA form of TwoProd; the logarithm is a
// table-driven reduction (Tang 1990) with a short log1p series.
#pragma once
#include <cuda_runtime.h>

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float h, float l) { ff r; r.hi = h; r.lo = l; return r; }
__device__ __forceinline__ ff ff_from(float a) { return ff_make(a, 0.0f); }

__device__ __forceinline__ ff fast_two_sum(float a, float b)  // |a| >= |b|
{
  float s = __fadd_rn(a, b);
  float e = __fsub_rn(b, __fsub_rn(s, a));
  return ff_make(s, e);
}

__device__ __forceinline__ ff two_sum(float a, float b)
{
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff_make(s, e);
}

__device__ __forceinline__ ff two_prod(float a, float b)
{
  float p = __fmul_rn(a, b);
  float e = __fmaf_rn(a, b, -p);
  return ff_make(p, e);
}

// accurate sum (both halves through TwoSum), safe under cancellation
__device__ __forceinline__ ff ff_add(ff a, ff b)
{
  ff s = two_sum(a.hi, b.hi);
  ff t = two_sum(a.lo, b.lo);
  float e = __fadd_rn(s.lo, t.hi);
  ff u = fast_two_sum(s.hi, e);
  e = __fadd_rn(t.lo, u.lo);
  return fast_two_sum(u.hi, e);
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff_make(-a.hi, -a.lo); }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

__device__ __forceinline__ ff ff_add_f(ff a, float b)
{
  ff s = two_sum(a.hi, b);
  float e = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, e);
}

__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
  ff p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, e);
}

__device__ __forceinline__ ff ff_mul_f(ff a, float b)
{
  ff p = two_prod(a.hi, b);
  float e = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, e);
}

// a / b: quotient estimate, exact remainder by FMA, one correction
__device__ __forceinline__ ff ff_div(ff a, ff b)
{
  float q1 = __fdiv_rn(a.hi, b.hi);
  ff p = ff_mul_f(b, q1);
  ff r = ff_sub(a, p);
  float q2 = __fdiv_rn(r.hi, b.hi);
  return fast_two_sum(q1, q2);
}

// float-float constants: (hi, lo) of an FP64 value, filled by the host
struct FFConsts {
  float2 logtab[64];   // log(1 + (2i+1)/128)
  float2 i0s[7], i0l[9], i1s[7], i1l[9];  // Abramowitz & Stegun 9.8.1-9.8.4
  float2 ln2a;         // ln 2 = ln2a.x + ln2a.y + ln2b
  float ln2b;
  float2 ln1e10;       // ln(1e10)
  float2 logmydblmax;  // ln(DBL_MAX / 1e10)
  float2 inv375;       // 1 / 3.75
  float2 e10m;         // 1e-10
};

__device__ __forceinline__ ff ffc(float2 v) { return ff_make(v.x, v.y); }

// natural log of a positive, normal float-float value
__device__ __forceinline__ ff ff_log(ff v, const FFConsts &K)
{
  int k = ((__float_as_int(v.hi) >> 23) & 0xff) - 127;
  float sc = __int_as_float((127 - k) << 23);
  float m = v.hi * sc;           // [1, 2), exact
  float ml = v.lo * sc;
  int idx = (int)((m - 1.0f) * 64.0f);
  idx = idx > 63 ? 63 : idx;
  float c = 1.0f + (float)(2 * idx + 1) * (1.0f / 128.0f);
  ff d = two_sum(__fsub_rn(m, c), ml);  // m - c is exact
  // r = d / c
  float q = __fdiv_rn(d.hi, c);
  float rem = __fmaf_rn(-q, c, d.hi);
  float ql = __fdiv_rn(__fadd_rn(rem, d.lo), c);
  ff r = fast_two_sum(q, ql);
  // log1p(r) = r - r^2/2 + r^3 (1/3 - r/4 + r^2/5 - r^3/6), |r| <= 1/129
  ff r2 = two_prod(r.hi, r.hi);
  r2.lo = __fmaf_rn(2.0f * r.hi, r.lo, r2.lo);
  ff half_r2 = ff_make(0.5f * r2.hi, 0.5f * r2.lo);
  float rh = r.hi;
  float tail = rh * rh * rh *
               (0.33333334f + rh * (-0.25f + rh * (0.2f + rh * (-0.16666667f))));
  ff l1p = ff_add_f(ff_sub(r, half_r2), tail);
  // k ln2 exactly enough: k * ln2a.x is exact (ln2a.x has 16 significant bits)
  ff kl = ff_add(ff_from((float)k * K.ln2a.x), two_prod((float)k, K.ln2a.y));
  kl = ff_add_f(kl, (float)k * K.ln2b);
  return ff_add(ff_add(kl, ffc(K.logtab[idx])), l1p);
}

__device__ __forceinline__ ff ff_horner(const float2 *c, int m, ff y)
{
  ff acc = ffc(c[m - 1]);
  for (int k = m - 2; k >= 0; k--) acc = ff_add(ff_mul(acc, y), ffc(c[k]));
  return acc;
}

__device__ __forceinline__ double ff_to_double(ff a) { return (double)a.hi + (double)a.lo; }

// ln 2 = LN2_A + LN2_B + LN2_C: LN2_A = 355/512 (9 significant bits, so k
// LN2_A is exact for |k| < 2^15), LN2_B and LN2_C the next two float parts
constexpr float LN2_A = 0.693359375f;
constexpr float LN2_B = -2.121944417e-04f;
constexpr float LN2_C = 1.646571768e-12f;
// ln 2 as a normalised float-float pair
constexpr float LN2_HI = 6.931471825e-01f;
constexpr float LN2_LO = -1.904654212e-09f;

// e^x and e^x - 1 for -86 < x < 88 in float-float.  x = k ln2 + r with
// |r| <= ln2 / 2, y = expm1(r / 16) from its Taylor series (degree 7,
// |r / 16| <= 0.022), four doublings expm1(2z) = expm1(z) (expm1(z) + 2),
// then e^x = 2^k (1 + y) and e^x - 1 = y (k = 0) or 2^k (1 + y) - 1.  No
// step cancels: e^x - 1 of a short branch keeps its relative accuracy
// (about 1e-14).
__device__ __forceinline__ void ff_exp_expm1(ff x, ff *ex, ff *em1)
{
  if (x.hi < -86.0f) {
    *ex = ff_from(0.0f);
    *em1 = ff_from(-1.0f);
    return;
  }
  const float kf = rintf(x.hi * 1.44269504f);
  ff r = ff_sub(x, ff_from(kf * LN2_A));
  r = ff_sub(r, two_prod(kf, LN2_B));
  r = ff_add_f(r, -kf * LN2_C);
  const ff s = ff_make(r.hi * 0.0625f, r.lo * 0.0625f);
  // the coefficients from 1/120 on in float (their terms weigh < 2e-9 of
  // the sum), the rest in float-float
  const float tail = __fmaf_rn(s.hi, __fmaf_rn(s.hi, 1.0f / 5040.0f, 1.0f / 720.0f), 1.0f / 120.0f);
  ff u = ff_add(ff_make(0.041666668f, -1.2417635e-09f), ff_mul_f(s, tail));  // 1/24 + s tail
  u = ff_add(ff_make(0.16666667f, -4.967054e-09f), ff_mul(s, u));          // 1/6 + s u
  u = ff_add_f(ff_mul(s, u), 0.5f);
  u = ff_add_f(ff_mul(s, u), 1.0f);
  ff y = ff_mul(s, u);
#pragma unroll
  for (int i = 0; i < 4; i++) y = ff_mul(y, ff_add_f(y, 2.0f));
  const int k = (int)kf;
  const float p2 = __int_as_float((127 + k) << 23);  // 2^k, -125 <= k <= 127
  const ff one_y = ff_add_f(y, 1.0f);
  *ex = ff_make(one_y.hi * p2, one_y.lo * p2);
  *em1 = (k == 0) ? y : ff_add_f(*ex, -1.0f);
}
