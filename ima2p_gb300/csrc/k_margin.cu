// k_margin.cu -- 1-D marginal posterior densities (margincalc,
// surface_call_functions.cpp:119-175; fillvec, histograms.cpp:82-99).
//
// For parameter p at x the density is (1/G) sum_g exp(term_g):
//   population size p:  -qi_p + round(cc_p) (ln 2 - ln x) - hcc_p - 2 fc_p / x
//   migration rate p:   -mi_p + round(mc_p) ln x - fm_p x
//                       (+ ln(1/mean) - x / mean under an exponential prior)
// summed in FP64 without a shift, as the reference sums it (the values span
// hundreds of orders of magnitude and the reference returns them as they are).
// marginp (surface_call_functions.cpp:25-80), the peak searches' form, sums a
// range of genealogies, takes the theta term's cc as stored and divides by
// the range's length (+1 when it starts at genealogy 0).
//
// One thread per requested (parameter, x) and genealogy chunk; tiles of whole
// gsampinf rows are staged in shared memory with coalesced loads, and every
// thread reads its parameter's three or four columns from there.  Partial sums
// per chunk are added in chunk order by the merge kernel.
#include <cfloat>
#include <cmath>

#include "internal.h"

namespace {

constexpr int MG_BS = 128;   // requests per CTA
constexpr int MG_TG = 64;    // genealogies per shared-memory tile
constexpr int MG_MAXROW = 64;
constexpr double LOG2 = 0.69314718055994530942;

__device__ __forceinline__ double intround(float v)  // INTEGERROUND (imamp.hpp:180)
{
  return v >= 0.f ? (double)(long long)((double)v + 0.5) : (double)(long long)((double)v - 0.5);
}

__global__ void __launch_bounds__(MG_BS) k_margin(MarginArgs a, int chunk, double *part)
{
  __shared__ float tile[MG_TG * MG_MAXROW];
  const int k = blockIdx.x * MG_BS + threadIdx.x;
  const bool live = k < a.n;
  const int pi = live ? a.param[k] : 0;
  const double x = live ? a.x[k] : 1.0;
  const bool theta = pi < a.np;
  // per-request constants
  const double lx = theta ? LOG2 - log(x) : log(x);
  const double ix = 1.0 / x;
  double cst = 0.0, slope = 0.0;
  if (!theta && a.expo_mean) {
    const double meani = 1.0 / a.expo_mean[pi - a.np];
    cst = log(meani);
    slope = meani;
  }
  int c0, c1, c2, c3;  // columns: (qi, cc, hcc, fc) or (mi, mc, fm, -)
  if (theta) {
    c0 = a.qip + pi; c1 = a.ccp + pi; c2 = a.hccp + pi; c3 = a.fcp + pi;
  } else {
    const int p = pi - a.np;
    c0 = a.mip + p; c1 = a.mcp + p; c2 = a.fmp + p; c3 = c2;
  }
  const int g0 = a.g_lo + blockIdx.y * chunk, g1 = min(a.g_hi, g0 + chunk);
  double sum = 0.0;
  for (int t0 = g0; t0 < g1; t0 += MG_TG) {
    const int nt = min(MG_TG, g1 - t0);
    __syncthreads();
    const float *src = a.rows + (size_t)t0 * a.rowlen;  // nt whole rows are contiguous
    for (int i = threadIdx.x; i < nt * a.rowlen; i += MG_BS) tile[i] = src[i];
    __syncthreads();
    if (!live) continue;
    for (int j = 0; j < nt; j++) {
      const float *r = tile + j * a.rowlen;
      double temp;
      if (theta)
        temp = -(double)r[c0] + (a.raw_cc ? (double)r[c1] : intround(r[c1])) * lx - (double)r[c2] -
               2.0 * (double)r[c3] * ix;
      else
        temp = -(double)r[c0] + cst - x * slope + intround(r[c1]) * lx - (double)r[c2] * x;
      sum += exp(temp);
    }
  }
  if (live) part[(size_t)k * gridDim.y + blockIdx.y] = sum;
}

__global__ void k_margin_merge(MarginArgs a, int nchunks, const double *part, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  double s = 0.0;
  for (int c = 0; c < nchunks; c++) s += part[(size_t)k * nchunks + c];
  s /= a.div;
  if (a.logi) s = (s <= 0.0) ? -1e200 : log(s);  // LOWLOG
  out[k] = s - a.yadjust;
}

}  // namespace

int margin_chunks(int G, int n)
{
  const int rblocks = (n + MG_BS - 1) / MG_BS;
  int nchunks = (4 * 152 + rblocks - 1) / rblocks;  // about four waves of CTAs
  const int maxc = (G + 4 * MG_TG - 1) / (4 * MG_TG);  // at least four tiles per chunk
  if (nchunks > maxc) nchunks = maxc;
  return nchunks < 1 ? 1 : nchunks;
}

int launch_margin(const MarginArgs &a, double *part, int nchunks, double *out, cudaStream_t st)
{
  if (a.rowlen > MG_MAXROW || a.n < 1) return 2;
  const int ng = a.g_hi - a.g_lo;
  if (ng < 1) return 2;
  const int chunk = ((ng + nchunks - 1) / nchunks + MG_TG - 1) / MG_TG * MG_TG;
  nchunks = (ng + chunk - 1) / chunk;
  k_margin<<<dim3((a.n + MG_BS - 1) / MG_BS, nchunks), MG_BS, 0, st>>>(a, chunk, part);
  k_margin_merge<<<(a.n + 127) / 128, 128, 0, st>>>(a, nchunks, part, out);
  return 0;
}
