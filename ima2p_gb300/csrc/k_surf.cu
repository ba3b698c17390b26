// k_surf.cu -- L-mode joint posterior surface, FP64 CUDA-core form and the
// reference-compatible truncated form (jointp, jointfind.cpp:885-1047).
//
// For a parameter point x the reference forms, per saved genealogy g,
//   p_g = bias_g + sum_i [cc_i (ln2 - ln theta_i) - hcc_i - 2 fc_i / theta_i]
//                + sum_j [mc_j ln m_j - fm_j m_j]
// with bias_g = -probg (2 populations) or -sum qi / -sum mi (model types 1/2),
// and returns q = ln G - ln sum_g exp(p_g).  p_g is a dot product of the
// genealogy's statistics with a per-point coefficient vector phi(x); the
// hcc terms fold into the bias.
//
// FP64 form: each CTA takes 128 points and a chunk of genealogies staged
// through shared memory; every thread keeps an online (max, sum, sum of
// squares) of exp(p_g - max) for its point; a second kernel merges the
// chunks.  Compat form: one CTA per point reproduces the reference's
// truncation -- the linked list keeps values within PRANGELOG = 10 of the
// running maximum, the final traversal drops values 10 or more below the
// overall maximum and, when every listed value is in range, also the
// smallest one -- and its eexp decimal-exponent accumulation.
#include <cfloat>
#include <mutex>

#include "internal.h"
#include "eexp.cuh"

namespace {

constexpr double LOG2 = 0.69314718055994530941723212146;
constexpr double LOG10 = 2.3025850929940456840;
constexpr int KMAX = 64;

struct Offs {
  int cc, fc, hcc, mc, fm, qi, mi, probg;
};

__device__ __forceinline__ Offs offsets(int np, int nm)
{
  Offs o;
  o.cc = 0;
  o.fc = np;
  o.hcc = 2 * np;
  o.mc = 3 * np;
  o.fm = 3 * np + nm;
  o.qi = 3 * np + 2 * nm;
  o.mi = 4 * np + 2 * nm;
  o.probg = 4 * np + 3 * nm + 1;
  return o;
}

__device__ __forceinline__ void param_range(int np, int nm, int mt, int *lo, int *hi)
{
  *lo = (mt == 2) ? np : 0;
  *hi = (mt == 1) ? np : np + nm;
}

// p_g at one point; phi holds the per-point coefficients
//   phi[i] = ln2 - ln theta_i, phi[np+i] = 1/theta_i, phi[2np+j] = ln m_j,
//   phi[2np+nm+j] = m_j
__device__ __forceinline__ double p_of(const SurfArgs &a, const float *r, double bias,
                                       const double *phi, const Offs &o, int lo, int hi)
{
  double p = bias;
  for (int i = lo; i < hi; i++) {
    if (i < a.np) {
      double dg = 2.0 * r[o.fc + i];
      p += r[o.cc + i] * phi[i] - r[o.hcc + i] - dg * phi[a.np + i];
    } else {
      int j = i - a.np;
      p += r[o.mc + j] * phi[2 * a.np + j] - r[o.fm + j] * phi[2 * a.np + a.nm + j];
    }
  }
  return p;
}

__device__ __forceinline__ double bias_of(const SurfArgs &a, const float *r, int g, const Offs &o)
{
  if (a.lognorm) return a.lognorm[g];
  if (a.npops == 2) return -(double)r[o.probg];
  double s = 0.0;
  if (a.modeltype == 1)
    for (int i = 0; i < a.np; i++) s += r[o.qi + i];
  else
    for (int i = 0; i < a.nm; i++) s += r[o.mi + i];
  return -s;
}

__device__ void make_phi(const SurfArgs &a, const double *x, double *phi)
{
  for (int i = 0; i < a.np; i++) {
    phi[i] = LOG2 - log(x[i]);
    phi[a.np + i] = 1.0 / x[i];
  }
  for (int j = 0; j < a.nm; j++) {
    double m = x[a.np + j];
    phi[2 * a.np + j] = log(m);
    phi[2 * a.np + a.nm + j] = m;
  }
}

// ---------------------------------------------------------------- FP64
constexpr int F64_PTS = 128;
constexpr int F64_TILE = 32;

__global__ void __launch_bounds__(F64_PTS) k_surf_fp64(SurfArgs a, int chunk, double *part)
{
  __shared__ float rows[F64_TILE * KMAX];
  __shared__ double bias[F64_TILE];
  const int pt = blockIdx.x * F64_PTS + threadIdx.x;
  const int g0 = blockIdx.y * chunk, g1 = min(a.G, g0 + chunk);
  const Offs o = offsets(a.np, a.nm);
  int lo, hi;
  param_range(a.np, a.nm, a.modeltype, &lo, &hi);
  const int npar = a.np + a.nm;
  double phi[KMAX];
  if (pt < a.npoints) make_phi(a, a.x + (size_t)pt * npar, phi);
  double m = -INFINITY, s = 0.0, s2 = 0.0;
  for (int t0 = g0; t0 < g1; t0 += F64_TILE) {
    int nt = min(F64_TILE, g1 - t0);
    __syncthreads();
    for (int k = threadIdx.x; k < nt * a.rowlen; k += F64_PTS)
      rows[k] = a.rows[(size_t)t0 * a.rowlen + k];
    __syncthreads();
    for (int k = threadIdx.x; k < nt; k += F64_PTS) bias[k] = bias_of(a, rows + k * a.rowlen, t0 + k, o);
    __syncthreads();
    if (pt < a.npoints) {
      for (int k = 0; k < nt; k++) {
        double p = p_of(a, rows + k * a.rowlen, bias[k], phi, o, lo, hi);
        if (p > m) {
          double f = exp(m - p);
          s = s * f + 1.0;
          s2 = s2 * f * f + 1.0;
          m = p;
        } else {
          double e = exp(p - m);
          s += e;
          s2 += e * e;
        }
      }
    }
  }
  if (pt < a.npoints) {
    double *w = part + ((size_t)pt * gridDim.y + blockIdx.y) * 3;
    w[0] = m;
    w[1] = s;
    w[2] = s2;
  }
}

__global__ void k_surf_merge(SurfArgs a, int nchunks, const double *part)
{
  int pt = blockIdx.x * blockDim.x + threadIdx.x;
  if (pt >= a.npoints) return;
  const double *w = part + (size_t)pt * nchunks * 3;
  double M = -INFINITY;
  for (int c = 0; c < nchunks; c++) M = fmax(M, w[3 * c]);
  double s = 0.0, s2 = 0.0;
  for (int c = 0; c < nchunks; c++) {
    if (w[3 * c + 1] == 0.0) continue;
    double f = exp(w[3 * c] - M);
    s += w[3 * c + 1] * f;
    s2 += w[3 * c + 2] * f * f;
  }
  a.q[pt] = log((double)a.G) - (M + log(s));
  if (a.ess) a.ess[pt] = s * s / s2;
}

// -------------------------------------------------------------- compat
constexpr int CP_BS = 256;

template <typename T, typename Op>
__device__ T block_reduce(T v, Op op, T *sh)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = op(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
  __syncthreads();
  T r = sh[0];
  for (int w = 1; w < CP_BS / 32; w++) r = op(r, sh[w]);
  return r;
}

struct MaxOp { __device__ double operator()(double a, double b) const { return fmax(a, b); } };
struct MinOp { __device__ double operator()(double a, double b) const { return fmin(a, b); } };
struct AddOp { __device__ double operator()(double a, double b) const { return a + b; } };
struct IMaxOp { __device__ int operator()(int a, int b) const { return max(a, b); } };
struct IOrOp { __device__ int operator()(int a, int b) const { return a | b; } };
struct IAddOp { __device__ int operator()(int a, int b) const { return a + b; } };
struct IMinOp { __device__ int operator()(int a, int b) const { return min(a, b); } };

__global__ void __launch_bounds__(CP_BS) k_surf_compat(SurfArgs a, int pt0, double *pbuf,
                                                       uint8_t *listed)
{
  __shared__ double shd[CP_BS / 32];
  __shared__ int shi[CP_BS / 32];
  __shared__ double scan[CP_BS];
  const int pt = pt0 + blockIdx.x;
  const Offs o = offsets(a.np, a.nm);
  int lo, hi;
  param_range(a.np, a.nm, a.modeltype, &lo, &hi);
  const int npar = a.np + a.nm;
  double phi[KMAX];
  make_phi(a, a.x + (size_t)pt * npar, phi);
  double *p = pbuf + (size_t)blockIdx.x * a.G;
  uint8_t *lst = listed + (size_t)blockIdx.x * a.G;
  // pass 1: values, list membership against the running maximum
  double carry = -INFINITY;
  for (int c0 = 0; c0 < a.G; c0 += CP_BS) {
    int g = c0 + threadIdx.x;
    double v = -INFINITY;
    if (g < a.G) {
      const float *r = a.rows + (size_t)g * a.rowlen;
      v = p_of(a, r, bias_of(a, r, g, o), phi, o, lo, hi);
      p[g] = v;
    }
    // inclusive prefix max over the chunk (Hillis-Steele in shared memory)
    __syncthreads();
    scan[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < CP_BS; off <<= 1) {
      double t = (threadIdx.x >= off) ? scan[threadIdx.x - off] : -INFINITY;
      __syncthreads();
      scan[threadIdx.x] = fmax(scan[threadIdx.x], t);
      __syncthreads();
    }
    double excl = fmax(carry, threadIdx.x ? scan[threadIdx.x - 1] : -INFINITY);
    if (g < a.G) lst[g] = (g == 0 || excl - v < 10.0) ? 1 : 0;
    carry = fmax(carry, scan[CP_BS - 1]);
    __syncthreads();
  }
  const double M = carry;
  // pass 2: in-range set, whether any listed value fell out of range, its minimum
  double vmin = INFINITY;
  int anyout = 0, nlist = 0;
  for (int g = threadIdx.x; g < a.G; g += CP_BS) {
    bool inr = M - p[g] < 10.0;
    if (lst[g]) nlist++;
    if (lst[g] && !inr) anyout = 1;
    if (inr) vmin = fmin(vmin, p[g]);
  }
  vmin = block_reduce(vmin, MinOp(), shd);
  anyout = block_reduce(anyout, IOrOp(), shi);
  nlist = block_reduce(nlist, IAddOp(), shi);
  const bool skip = !anyout && nlist >= 2;
  // the skipped element: the first index holding the minimum
  int skipidx = a.G;
  if (skip)
    for (int g = threadIdx.x; g < a.G; g += CP_BS)
      if (p[g] == vmin && M - p[g] < 10.0) skipidx = min(skipidx, g);
  skipidx = block_reduce(skipidx, IMinOp(), shi);
  // pass 3: eexp terms, decimal exponent normalisation as the reference
  int maxz = -10000000;
  for (int g = threadIdx.x; g < a.G; g += CP_BS) {
    if (!(M - p[g] < 10.0) || g == skipidx) continue;
    double mm;
    int z;
    eexp_dev(p[g], &mm, &z);
    maxz = max(maxz, z);
  }
  maxz = block_reduce(maxz, IMaxOp(), shi) - 10;
  double acc = 0.0, acc2 = 0.0;
  for (int g = threadIdx.x; g < a.G; g += CP_BS) {
    if (!(M - p[g] < 10.0) || g == skipidx) continue;
    double mm;
    int z;
    eexp_dev(p[g], &mm, &z);
    int zadj = z - maxz;
    if (zadj > -308 && zadj < 308) mm *= pow(10.0, (double)zadj);
    else if (zadj <= -308) mm = 0.0;
    else mm = DBL_MAX;
    acc += mm;
    acc2 += mm * mm;
  }
  acc = block_reduce(acc, AddOp(), shd);
  acc2 = block_reduce(acc2, AddOp(), shd);
  if (threadIdx.x == 0) {
    a.q[pt] = log((double)a.G) - (log(acc) + maxz * LOG10);
    if (a.ess) a.ess[pt] = acc * acc / acc2;
  }
}


}  // namespace

size_t surface_fp64_scratch_bytes(int G, int npoints)
{
  int nchunks = (G + 65535) / 65536;
  if (nchunks > 64) nchunks = 64;
  size_t f64 = (size_t)npoints * nchunks * 3 * sizeof(double);
  size_t cp = (size_t)(npoints < SURF_COMPAT_CONCURRENT ? npoints : SURF_COMPAT_CONCURRENT) * G *
              (sizeof(double) + 1);
  return f64 > cp ? f64 : cp;
}

void launch_surface_fp64(const SurfArgs &a, double *scratch, cudaStream_t st)
{
  if (a.npoints <= 0) return;
  int nchunks = (a.G + 65535) / 65536;
  if (nchunks > 64) nchunks = 64;
  int chunk = (a.G + nchunks - 1) / nchunks;
  dim3 grid((a.npoints + F64_PTS - 1) / F64_PTS, nchunks);
  k_surf_fp64<<<grid, F64_PTS, 0, st>>>(a, chunk, scratch);
  k_surf_merge<<<(a.npoints + 127) / 128, 128, 0, st>>>(a, nchunks, scratch);
}

void launch_surface_compat(const SurfArgs &a, double *scratch, cudaStream_t st)
{
  for (int p0 = 0; p0 < a.npoints; p0 += SURF_COMPAT_CONCURRENT) {
    int np = a.npoints - p0 < SURF_COMPAT_CONCURRENT ? a.npoints - p0 : SURF_COMPAT_CONCURRENT;
    int conc = a.npoints < SURF_COMPAT_CONCURRENT ? a.npoints : SURF_COMPAT_CONCURRENT;
    uint8_t *listed = reinterpret_cast<uint8_t *>(scratch + (size_t)conc * a.G);
    k_surf_compat<<<np, CP_BS, 0, st>>>(a, p0, scratch, listed);
  }
}

// ======================================================================
// Allocation-free variant of the FP64 surface, for callers that may not call
// cudaMalloc: a plugin whose host application owns every device allocation
// through its own pool.  Its only scratch -- one (max, sum, sum of squares)
// triple per point and genealogy chunk -- lives in the fixed device array
// below, which every GPU that loads this library holds until the process
// exits.  The array's device address is looked up once per device and kept;
// after a cudaDeviceReset of that device the kept address is stale, so the
// entry point is not for use after a reset in the same process.
namespace {

constexpr size_t NOALLOC_SCRATCH_DOUBLES = (size_t)1 << 19;  // 4 MiB
constexpr int NOALLOC_MAX_DEVICES = 64;

__device__ __align__(256) double g_surf_scratch[NOALLOC_SCRATCH_DOUBLES];

std::mutex g_noalloc_mu;
double *g_noalloc_addr[NOALLOC_MAX_DEVICES];

// Device address of g_surf_scratch on the current device, looked up once per
// device (host code cannot use the symbol itself as a device pointer).
int noalloc_scratch(double **out)
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return IMA_ERR_CUDA;
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) return IMA_ERR_ARG;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    double *p = nullptr;
    if (cudaGetSymbolAddress(reinterpret_cast<void **>(&p), g_surf_scratch) != cudaSuccess)
      return IMA_ERR_CUDA;
    g_noalloc_addr[dev] = p;
  }
  *out = g_noalloc_addr[dev];
  return IMA_OK;
}

}  // namespace

extern "C" int ima_gpu_surface_fp64_noalloc(const float *rows, int G, int rowlen, int np, int nm,
                                            int npops, const double *lognorm, const double *x,
                                            int npoints, int modeltype, double *q, double *ess,
                                            void *stream)
{
  if (!rows || !x || !q || G < 1 || npoints < 1 || np < 0 || nm < 0 || np + nm < 1 ||
      np + nm > 32 || rowlen < 4 * np + 3 * nm + 2 || rowlen > 64 || modeltype < 0 || modeltype > 2)
    return IMA_ERR_ARG;
  // one triple per point and chunk: use as many chunks as the array allows
  size_t per_point = 3;
  if ((size_t)npoints * per_point > NOALLOC_SCRATCH_DOUBLES) return IMA_ERR_TOO_LARGE;
  int nchunks = (G + 65535) / 65536;
  if (nchunks > 64) nchunks = 64;
  size_t fit = NOALLOC_SCRATCH_DOUBLES / ((size_t)npoints * per_point);
  if ((size_t)nchunks > fit) nchunks = (int)fit;
  // an error already pending on this thread is the caller's: report it
  // without launching (and leave it pending) rather than take it for ours
  if (cudaPeekAtLastError() != cudaSuccess) return IMA_ERR_CUDA;
  double *scratch = nullptr;
  int r = noalloc_scratch(&scratch);
  if (r) return r;
  SurfArgs a;
  a.G = G;
  a.rowlen = rowlen;
  a.np = np;
  a.nm = nm;
  a.npops = npops;
  a.modeltype = modeltype;
  a.npoints = npoints;
  a.rows = rows;
  a.lognorm = lognorm;
  a.x = x;
  a.q = q;
  a.ess = ess;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // every (point, chunk) triple is written before the merge reads it, so the
  // contents left by an earlier call never leak into this one
  int chunk = (G + nchunks - 1) / nchunks;
  dim3 grid((npoints + F64_PTS - 1) / F64_PTS, nchunks);
  k_surf_fp64<<<grid, F64_PTS, 0, st>>>(a, chunk, scratch);
  k_surf_merge<<<(npoints + 127) / 128, 128, 0, st>>>(a, nchunks, scratch);
  return cudaGetLastError() == cudaSuccess ? IMA_OK : IMA_ERR_CUDA;
}
