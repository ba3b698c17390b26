// surf_common.cuh -- shared pieces of the split-precision surface: the
// prepared operands, the exact recomputation of one term, the online
// log-sum-exp state, shared per-point thresholds and the FP64 merge of
// per-chunk partials.
#pragma once
#include <cstdint>

#include "ff.cuh"
#include "internal.h"

constexpr int SURF_K = 30;          // exact terms: 2 (theta + migration parameters)
constexpr int SURF_KP = 32;         // screened columns: the terms, the bias, zero padding
constexpr int SURF_MAX_CHUNKS = 64;
constexpr float SURF_MARGIN = 32.0f;  // nats below the running max that still count
constexpr int SURF_SEED = 256;      // genealogies sampled per point for the seed maximum (FP32 screen)
constexpr int SURF_TC_M = 128;      // tensor-core screen: points per A tile
constexpr int SURF_TC_N = 256;      // tensor-core screen: genealogies per B tile

// Operands prepared once per evaluation (model type and points fixed).
struct SurfPrep {
  int G, Gpad, K, np, nm;
  float *sT;        // [SURF_KP][Gpad] statistics (exact floats), column K = bias (rounded)
  float2 *biasff;   // [Gpad] bias as float-float
  float2 *phiff;    // [npoints][SURF_K] phi as float-float
  float *phi32;     // [npoints][SURF_KP] phi rounded, 1 in the bias column
  float *mag;       // [npoints] sum_k colmax_k |phi_k|: scale of screening errors
  float *seed;      // [npoints] exact max over a sample of genealogies
  unsigned *best;   // [npoints] best exact maximum found so far (ordered bits), shared by chunks
  unsigned *xmax;   // [npoints] largest exact value the refinement met (ordered bits; tensor-core screen)
  unsigned *colmax; // [SURF_KP] max |column| as float bits
  uint16_t *sbf;    // bf16 statistics, hi and lo planes of 256-row MMA tiles (tensor-core screen)
  uint16_t *pbf;    // bf16 phi, hi and lo planes of 128-row MMA tiles (tensor-core screen)
};

// Per (point, chunk) partial of the online log-sum-exp.
struct SurfPart {
  float mh, ml;  // running maximum (float-float)
  float sh, sl;  // sum of exp(p - max) (float-float)
  float s2;      // sum of exp(2 (p - max)) for the effective sample size
  float pad;
};

// exact p_g(x) = bias + sum_k s_k phi_k, s_k exact floats, phi_k float-float:
// compensated dot product (Ogita, Rump & Oishi 2005, Dot2) on the high parts,
// the low parts and all error terms gathered in one float
__device__ __forceinline__ ff surf_exact(const SurfPrep &S, int g, const float *col, int stride,
                                         const float2 *phi)
{
  float2 b = S.biasff[g];
  float sum = b.x, comp = b.y;
  // fully unrolled with a bound check: phi stays in registers and the
  // column loads issue together
#pragma unroll
  for (int k = 0; k < SURF_K; k++) {
    if (k >= S.K) break;
    float s = col[k * stride];
    float2 f = phi[k];
    float p = __fmul_rn(s, f.x);
    float pe = __fmaf_rn(s, f.x, -p);
    float t = __fadd_rn(sum, p);
    float bb = __fsub_rn(t, sum);
    float te = __fadd_rn(__fsub_rn(sum, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    sum = t;
    comp = __fadd_rn(comp, __fadd_rn(te, __fmaf_rn(s, f.y, pe)));
  }
  return fast_two_sum(sum, comp);
}

struct LseState {
  ff m, s;
  float s2;
  __device__ __forceinline__ void init()
  {
    m = ff_make(-INFINITY, 0.f);
    s = ff_from(0.f);
    s2 = 0.f;
  }
  __device__ __forceinline__ void add(ff y)
  {
    if (m.hi == -INFINITY) {
      m = y;
      s = ff_from(1.f);
      s2 = 1.f;
      return;
    }
    ff d = ff_sub(y, m);
    float dd = d.hi + d.lo;
    if (dd > 0.f) {
      float e = expf(-dd);
      s = ff_add_f(ff_mul_f(s, e), 1.0f);
      s2 = s2 * e * e + 1.0f;
      m = y;
    } else {
      float e = expf(dd);
      s = ff_add_f(s, e);
      s2 += e * e;
    }
  }
  __device__ __forceinline__ SurfPart pack() const
  {
    SurfPart p;
    p.mh = m.hi;
    p.ml = m.lo;
    p.sh = s.hi;
    p.sl = s.lo;
    p.s2 = s2;
    p.pad = 0.f;
    return p;
  }
  __device__ __forceinline__ void unpack(const SurfPart &o)
  {
    m = ff_make(o.mh, o.ml);
    s = ff_make(o.sh, o.sl);
    s2 = o.s2;
  }
  // fold another partial (same point) into this one
  __device__ __forceinline__ void merge(const SurfPart &o)
  {
    if (o.mh == -INFINITY) return;
    if (m.hi == -INFINITY) {
      m = ff_make(o.mh, o.ml);
      s = ff_make(o.sh, o.sl);
      s2 = o.s2;
      return;
    }
    ff om = ff_make(o.mh, o.ml);
    ff d = ff_sub(om, m);
    float dd = d.hi + d.lo;
    ff os = ff_make(o.sh, o.sl);
    if (dd > 0.f) {
      float e = expf(-dd);
      s = ff_add(ff_mul_f(s, e), os);
      s2 = s2 * e * e + o.s2;
      m = om;
    } else {
      float e = expf(dd);
      s = ff_add(s, ff_mul_f(os, e));
      s2 += o.s2 * e * e;
    }
  }
};

// order-preserving float <-> uint for atomicMax on shared thresholds
__device__ __forceinline__ unsigned f2ord(float f)
{
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u)
{
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7fffffffu) : ~u);
}

size_t surf_prep_bytes(int G, int npoints);
SurfPart *surf_prep_carve(SurfPrep *S, char *base, int G, int npoints);
// rows_ready: the row-derived operands (sT, biasff, colmax, sbf) are already
// in place from an earlier evaluation of the same rows and model type
void surf_prep(const SurfArgs &a, SurfPrep &S, bool bf16, bool rows_ready, cudaStream_t st);
void surf_merge(const SurfArgs &a, const SurfPart *part, int nchunks, cudaStream_t st);
void surf_seed(const SurfPrep &S, int npoints, int samples, cudaStream_t st);
