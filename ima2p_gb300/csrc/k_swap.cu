// k_swap.cu -- MC3 temperature swaps (swapchains, swapchains.cpp:526-653, with
// swapbetasonly = 1; swapweight :12-34; swapbetas :655-662).
//
// One CTA per independent run.  The CTA first forms every chain's
// S = sum_li pdg[li] (+ probg unless -c4), one thread per chain, adding the
// loci in the reference's order so S is bit-identical; then warp 0 makes the
// run's swap attempts in sequence, because each attempt sees the betas the
// previous one left.  Uniforms are consumed exactly as the reference consumes
// them: ci, then cj until it differs from ci, then U only when w < 1 (C's
// short-circuit in `w >= 1.0 || w > uniform()`).  The uniform source is either
// a caller-supplied stream per run (the reference's MT19937 output, for
// decision-level parity) or a per-run Philox4x32-10 counter stream.
#include "internal.h"

namespace {

constexpr int SWAPDIST = 7;  // swapchains.cpp:537

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): 64-bit key, 128-bit counter.
__device__ __forceinline__ uint4 philox(uint4 c, uint2 k)
{
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; r++) {
    uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += W0;
    k.y += W1;
  }
  return c;
}

struct Uni {
  const double *buf;
  int stride, k;
  bool over;
  uint2 key;
  unsigned long long ctr;
  uint4 blk;
  int have;
  __device__ double next()
  {
    if (buf) {
      if (k >= stride) { over = true; return 0.5; }
      return buf[k++];
    }
    if (have == 0) {
      blk = philox(make_uint4((uint32_t)ctr, (uint32_t)(ctr >> 32), 0u, 0u), key);
      ctr++;
      have = 4;
    }
    uint32_t w = (have == 4) ? blk.x : (have == 3) ? blk.y : (have == 2) ? blk.z : blk.w;
    have--;
    k++;
    return ((double)w + 0.5) * 2.32830643653869628906e-10;  // (0,1) as genrand_real3
  }
};

// first p with allb[p] == b, searched by the whole warp (-1 if absent)
__device__ __forceinline__ int beta_index_warp(const double *allb, int n, double b)
{
  const int lane = threadIdx.x & 31;
  for (int base = 0; base < n; base += 32) {
    unsigned hit = __ballot_sync(0xffffffffu, base + lane < n && allb[base + lane] == b);
    if (hit) return base + __ffs(hit) - 1;
  }
  return -1;
}

// Run state (betas, ladder, sums) is staged in shared memory; warp 0 makes
// the attempts, lane 0 drawing the uniforms and deciding, the warp searching
// the ladder for the two temperatures.
__global__ void k_swap(SwapArgs a)
{
  extern __shared__ double sw_sm[];
  const int run = blockIdx.x, n = a.cpr;
  const int c0 = run * n;
  double *beta = sw_sm, *allb = sw_sm + n, *S = sw_sm + 2 * n;
  for (int c = threadIdx.x; c < n; c += blockDim.x) {
    const double *row = a.pdg + (size_t)(c0 + c) * a.nloci;
    double s = 0.0;
    for (int l = 0; l < a.nloci; l++) s += row[l];
    if (a.include_probg) s += a.probg[c0 + c];
    S[c] = s;
    a.S[c0 + c] = s;
    beta[c] = a.beta[c0 + c];
    allb[c] = a.allbetas[c0 + c];
  }
  __syncthreads();
  if (threadIdx.x >= 32) return;
  const int lane = threadIdx.x;
  int32_t *sc = a.swapcount + (size_t)run * n * n;
  int32_t *tc = a.tempcount + (size_t)run * n * n;
  Uni U;
  U.buf = a.uniforms ? a.uniforms + (size_t)run * a.stride : nullptr;
  U.stride = a.stride;
  U.k = 0;
  U.over = false;
  U.key = make_uint2((uint32_t)a.seed, (uint32_t)(a.seed >> 32) ^ (uint32_t)run);
  U.ctr = a.counter ? a.counter[run] : 0ull;
  U.have = 0;
  int swap0ok = 0;
  for (int t = 0; t < a.swaptries; t++) {
    int ci = 0, cj = 0, over = 0;
    if (lane == 0) {
      int cjmin, cjrange;
      do { ci = (int)(U.next() * n); } while ((ci < 0 || ci >= n) && !U.over);
      if (n < 2 * SWAPDIST + 3) {
        cjmin = 0;
        cjrange = n;
      } else {
        cjmin = max(0, ci - SWAPDIST);
        cjrange = min(n, ci + SWAPDIST) - cjmin;
      }
      do { cj = cjmin + (int)(U.next() * cjrange); } while ((cj == ci || cj < 0 || cj >= n) && !U.over);
      over = U.over;
    }
    ci = __shfl_sync(0xffffffffu, ci, 0);
    cj = __shfl_sync(0xffffffffu, cj, 0);
    if (__shfl_sync(0xffffffffu, over, 0)) break;
    const int p = beta_index_warp(allb, n, beta[ci]);
    const int q = beta_index_warp(allb, n, beta[cj]);
    if (lane == 0) {
      int hi = max(ci, cj), lo = min(ci, cj);
      int phi = max(p, q), plo = min(p, q);
      if (p >= 0 && q >= 0) tc[phi * n + plo]++;
      sc[hi * n + lo]++;
      double w = exp((beta[ci] - beta[cj]) * (S[cj] - S[ci]));
      bool acc = (w >= 1.0) || (w > U.next());
      over = U.over;
      if (acc && !over) {
        double bt = beta[ci];
        beta[ci] = beta[cj];
        beta[cj] = bt;
        sc[lo * n + hi]++;
        if (p >= 0 && q >= 0) tc[plo * n + phi]++;
        if (ci == 0 || cj == 0) swap0ok = 1;
      }
    }
    __syncwarp();
    if (__shfl_sync(0xffffffffu, over, 0)) break;
  }
  for (int c = lane; c < n; c += 32) a.beta[c0 + c] = beta[c];
  if (lane == 0) {
    if (a.used) a.used[run] = U.over ? -1 : U.k;
    if (a.swap0ok) a.swap0ok[run] = swap0ok;
    if (a.counter) a.counter[run] = U.ctr;
  }
}

__global__ void k_pdg_commit(const int32_t *items, const uint8_t *accept, const double *pdg_new,
                             double *pdg, int n)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && accept[i]) pdg[items[i]] = pdg_new[items[i]];
}

}  // namespace

void launch_swap(const SwapArgs &a, cudaStream_t st)
{
  if (a.nruns <= 0) return;
  const size_t sm = 3 * sizeof(double) * (size_t)a.cpr;
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_swap, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_swap<<<a.nruns, 128, sm, st>>>(a);
}

void launch_pdg_commit(const int32_t *items, const uint8_t *accept, const double *pdg_new,
                       double *pdg, int n, cudaStream_t st)
{
  if (n <= 0) return;
  k_pdg_commit<<<(n + 255) / 256, 256, 0, st>>>(items, accept, pdg_new, pdg, n);
}
