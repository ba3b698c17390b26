// surf_common.cu -- operand preparation and the FP64 merge of the
// split-precision surface (see k_surf_fast.cu).
#include <cuda_bf16.h>

#include "surf_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr double LOG2 = 0.69314718055994530941723212146;

__host__ __device__ inline size_t align256(size_t v) { return (v + 255) & ~size_t(255); }

// Statistics of one genealogy in exact floats and its bias in float-float.
// Columns: cc_i, 2 fc_i (theta terms), mc_j, fm_j (migration terms); the
// bias is the reference's -probg (2 populations), -sum qi / -sum mi (model
// types 1 / 2) or the supplied FP64 normaliser, minus sum hcc_i.
__global__ void k_prep_rows(SurfArgs a, SurfPrep S)
{
  int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= S.Gpad) return;
  const int np = a.np, nm = a.nm, K = S.K;
  float col[SURF_KP];
  for (int k = 0; k < SURF_KP; k++) col[k] = 0.f;
  double bias = 0.0;
  if (g < a.G) {
    const float *r = a.rows + (size_t)g * a.rowlen;
    const int cc = 0, fc = np, hcc = 2 * np, mc = 3 * np, fm = 3 * np + nm, qi = 3 * np + 2 * nm,
              mi = 4 * np + 2 * nm, probg = 4 * np + 3 * nm + 1;
    if (a.lognorm) bias = a.lognorm[g];
    else if (a.npops == 2) bias = -(double)r[probg];
    else {
      double s = 0.0;
      if (a.modeltype == 1) for (int i = 0; i < np; i++) s += r[qi + i];
      else for (int i = 0; i < nm; i++) s += r[mi + i];
      bias = -s;
    }
    if (a.modeltype != 2)
      for (int i = 0; i < np; i++) bias -= r[hcc + i];
    for (int i = 0; i < np; i++) {
      col[i] = r[cc + i];
      col[np + i] = 2.0f * r[fc + i];
    }
    for (int j = 0; j < nm; j++) {
      col[2 * np + j] = r[mc + j];
      col[2 * np + nm + j] = r[fm + j];
    }
    col[K] = (float)bias;
  }
  // the grid covers Gpad (a multiple of 256) exactly, so every warp is full
  const unsigned lane = threadIdx.x & 31;
  for (int k = 0; k < SURF_KP; k++) {
    S.sT[(size_t)k * S.Gpad + g] = col[k];
    const unsigned m = __reduce_max_sync(0xffffffffu, g < a.G ? __float_as_uint(fabsf(col[k])) : 0u);
    if (lane == 0 && m) atomicMax(&S.colmax[k], m);
  }
  float bh = (float)bias;
  S.biasff[g] = make_float2(bh, (float)(bias - (double)bh));
  if (S.sbf) {  // the MMA's tile layout, SURF_TC_N genealogies per tile: hi plane, then lo plane
    const size_t plane = (size_t)SURF_TC_N * SURF_KP * 2;
    char *tile = reinterpret_cast<char *>(S.sbf) + (size_t)(g / SURF_TC_N) * 2 * plane;
    for (int k = 0; k < SURF_KP; k++) {
      __nv_bfloat16 hi = __float2bfloat16_rn(col[k]);
      __nv_bfloat16 lo = __float2bfloat16_rn(col[k] - __bfloat162float(hi));
      *reinterpret_cast<__nv_bfloat16 *>(tile + tc::tile_off(g % SURF_TC_N, k)) = hi;
      *reinterpret_cast<__nv_bfloat16 *>(tile + plane + tc::tile_off(g % SURF_TC_N, k)) = lo;
    }
  }
}

// phi(x) of every point; terms outside the model type get coefficient 0.
__global__ void k_prep_points(SurfArgs a, SurfPrep S, int npad)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npad) return;
  const int np = a.np, nm = a.nm, K = S.K;
  const int lo = (a.modeltype == 2) ? np : 0, hi = (a.modeltype == 1) ? np : np + nm;
  double phi[SURF_KP];
  for (int k = 0; k < SURF_KP; k++) phi[k] = 0.0;
  if (p < a.npoints) {
    const double *x = a.x + (size_t)p * (np + nm);
    for (int i = 0; i < np; i++) {
      if (i < lo || i >= hi) continue;
      phi[i] = LOG2 - log(x[i]);
      phi[np + i] = -1.0 / x[i];
    }
    for (int j = 0; j < nm; j++) {
      if (np + j < lo || np + j >= hi) continue;
      phi[2 * np + j] = log(x[np + j]);
      phi[2 * np + nm + j] = -x[np + j];
    }
    phi[K] = 1.0;
  }
  float mag = 0.f;
  for (int k = 0; k < SURF_KP; k++) {
    float v = (float)phi[k];
    if (p < a.npoints) {
      S.phi32[(size_t)p * SURF_KP + k] = v;
      if (k < SURF_K) S.phiff[(size_t)p * SURF_K + k] = make_float2(v, (float)(phi[k] - (double)v));
    }
    mag += __uint_as_float(S.colmax[k]) * fabsf(v);
    if (S.pbf) {  // the MMA's tile layout, 128 points per tile: hi plane, then lo plane
      const size_t plane = (size_t)SURF_TC_M * SURF_KP * 2;
      char *tile = reinterpret_cast<char *>(S.pbf) + (size_t)(p / SURF_TC_M) * 2 * plane;
      __nv_bfloat16 hi = __float2bfloat16_rn(v);
      __nv_bfloat16 lo = __float2bfloat16_rn((float)(phi[k] - (double)__bfloat162float(hi)));
      *reinterpret_cast<__nv_bfloat16 *>(tile + tc::tile_off(p % SURF_TC_M, k)) = hi;
      *reinterpret_cast<__nv_bfloat16 *>(tile + plane + tc::tile_off(p % SURF_TC_M, k)) = lo;
    }
  }
  if (p < a.npoints) S.mag[p] = mag;
}

__global__ void k_surf_merge_ff(SurfArgs a, const SurfPart *part, int nchunks)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npoints) return;
  const SurfPart *w = part + (size_t)p * nchunks;
  double M = -INFINITY;
  for (int c = 0; c < nchunks; c++)
    if (w[c].mh != -INFINITY) M = fmax(M, (double)w[c].mh + (double)w[c].ml);
  double s = 0.0, s2 = 0.0;
  for (int c = 0; c < nchunks; c++) {
    if (w[c].mh == -INFINITY) continue;
    double f = exp((double)w[c].mh + (double)w[c].ml - M);
    s += ((double)w[c].sh + (double)w[c].sl) * f;
    s2 += (double)w[c].s2 * f * f;
  }
  a.q[p] = log((double)a.G) - (M + log(s));
  if (a.ess) a.ess[p] = s * s / s2;
}

}  // namespace

size_t surf_prep_bytes(int G, int npoints)
{
  size_t Gpad = ((size_t)G + 255) / 256 * 256;
  size_t npad = ((size_t)npoints + 255) / 256 * 256;
  size_t b = 0;
  b += align256(sizeof(float) * SURF_KP * Gpad);
  b += align256(sizeof(float2) * Gpad);
  b += align256(sizeof(float2) * SURF_K * npad);
  b += align256(sizeof(float) * SURF_KP * npad);
  b += align256(sizeof(float) * npad);
  b += align256(sizeof(float) * npad);
  b += align256(sizeof(unsigned) * npad);
  b += align256(sizeof(unsigned) * npad);
  b += align256(sizeof(unsigned) * SURF_KP);
  b += align256(2 * sizeof(uint16_t) * SURF_KP * Gpad);
  b += align256(2 * sizeof(uint16_t) * SURF_KP * npad);
  return b;
}

SurfPart *surf_prep_carve(SurfPrep *S, char *base, int G, int npoints)
{
  size_t Gpad = ((size_t)G + 255) / 256 * 256;
  size_t npad = ((size_t)npoints + 255) / 256 * 256;
  size_t o = 0;
  auto take = [&](size_t bytes) {
    char *p = base + o;
    o += align256(bytes);
    return p;
  };
  S->G = G;
  S->Gpad = (int)Gpad;
  // operands derived from the rows alone come first, at offsets that do not
  // depend on the number of points, so they survive between evaluations
  S->sT = reinterpret_cast<float *>(take(sizeof(float) * SURF_KP * Gpad));
  S->biasff = reinterpret_cast<float2 *>(take(sizeof(float2) * Gpad));
  S->colmax = reinterpret_cast<unsigned *>(take(sizeof(unsigned) * SURF_KP));
  S->sbf = reinterpret_cast<uint16_t *>(take(2 * sizeof(uint16_t) * SURF_KP * Gpad));
  S->phiff = reinterpret_cast<float2 *>(take(sizeof(float2) * SURF_K * npad));
  S->phi32 = reinterpret_cast<float *>(take(sizeof(float) * SURF_KP * npad));
  S->mag = reinterpret_cast<float *>(take(sizeof(float) * npad));
  S->seed = reinterpret_cast<float *>(take(sizeof(float) * npad));
  S->best = reinterpret_cast<unsigned *>(take(sizeof(unsigned) * npad));
  S->xmax = reinterpret_cast<unsigned *>(take(sizeof(unsigned) * npad));
  S->pbf = reinterpret_cast<uint16_t *>(take(2 * sizeof(uint16_t) * SURF_KP * npad));
  return reinterpret_cast<SurfPart *>(base + o);
}

void surf_prep(const SurfArgs &a, SurfPrep &S, bool bf16, bool rows_ready, cudaStream_t st)
{
  S.np = a.np;
  S.nm = a.nm;
  S.K = 2 * (a.np + a.nm);
  if (!bf16) {
    S.sbf = nullptr;
    S.pbf = nullptr;
  }
  if (!rows_ready) {
    cudaMemsetAsync(S.colmax, 0, sizeof(unsigned) * SURF_KP, st);
    k_prep_rows<<<S.Gpad / 256, 256, 0, st>>>(a, S);
  }
  int npad = (a.npoints + 255) / 256 * 256;
  k_prep_points<<<npad / 256, 256, 0, st>>>(a, S, npad);
}

// exact maximum over an even sample of `samples` genealogies, one warp per
// point; also the starting value of the maximum shared by genealogy chunks
__global__ void k_surf_seed(SurfPrep S, int npoints, int samples)
{
  const int p = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (p >= npoints) return;  // warp-uniform
  float2 phi[SURF_K];
#pragma unroll
  for (int k = 0; k < SURF_K; k++) phi[k] = S.phiff[(size_t)p * SURF_K + k];
  float best = -INFINITY;
  const int n = min(samples, S.G);
  for (int i = lane; i < n; i += 32) {
    int g = (int)(((long long)i * S.G) / n);
    ff y = surf_exact(S, g, S.sT + g, S.Gpad, phi);
    best = fmaxf(best, y.hi);
  }
#pragma unroll
  for (int o = 16; o >= 1; o >>= 1) best = fmaxf(best, __shfl_xor_sync(0xffffffffu, best, o));
  if (lane == 0) {
    S.seed[p] = best;
    S.best[p] = f2ord(best);
    S.xmax[p] = f2ord(best);
  }
}

void surf_seed(const SurfPrep &S, int npoints, int samples, cudaStream_t st)
{
  k_surf_seed<<<(npoints * 32 + 255) / 256, 256, 0, st>>>(S, npoints, samples);
}

void surf_merge(const SurfArgs &a, const SurfPart *part, int nchunks, cudaStream_t st)
{
  k_surf_merge_ff<<<(a.npoints + 127) / 128, 128, 0, st>>>(a, part, nchunks);
}
