// k_surf_fast.cu -- L-mode surface, split precision (jointp's log density,
// jointfind.cpp:885-1047, summed exactly over every genealogy).
//
// p_g(x) = bias_g + s_g . phi(x) with s_g = [cc_i, 2 fc_i, mc_j, fm_j] and
// phi(x) = [ln2 - ln theta_i, -1/theta_i, ln m_j, -m_j]; q = ln G - LSE_g p_g.
//
// Two precisions do two jobs.  A cheap SCREEN forms every p_g(x) approximately
// together with a bound on its error; only terms that can lie within MARGIN
// nats of the best maximum known for the point are RECOMPUTED exactly (a
// compensated float dot product on the exact float statistics and a
// float-float phi) and enter an online log-sum-exp whose sum is kept in
// float-float.  A skipped term weighs < e^-MARGIN of the maximum.
//
// The per-point threshold is shared by every thread of the CTA and seeded
// with the exact maximum over a sample of genealogies, so it is tight from
// the first tile; candidates of a warp are drained with a ballot loop, one per
// lane per pass.  Maxima found during a tile go to a second array that is
// folded into the thresholds between tiles, so a tile's thresholds depend
// only on the earlier tiles: the candidate set, each thread's fold order and
// so the result are the same on every run.
//
// Screens: FP32 FMA on CUDA cores (this file) and a bf16 tcgen05 GEMM
// (k_surf_tc.cu).  Partial (max, sum) per point and genealogy chunk are
// merged in FP64.
#include <cfloat>
#include <cstdint>

#include "ff.cuh"
#include "internal.h"
#include "surf_common.cuh"

namespace {

constexpr int TP = 64;   // points per CTA
constexpr int TG = 128;  // genealogies per tile
constexpr int BS = 256;

// FP32 screen error: the statistics are exact floats, phi and the bias are
// rounded to FP32 and 32 FMAs accumulate -- bounded by 3.3e-6 of
// sum_k |s_k phi_k|; use 1e-5 of the per-point magnitude bound.
constexpr float FP32_SCREEN_ERR = 1e-5f;

__global__ void __launch_bounds__(BS) k_surf_screen_fp32(SurfPrep S, int npoints, int chunk,
                                                         SurfPart *part)
{
  __shared__ __align__(16) float sP[SURF_KP][TP];      // phi, point-contiguous
  __shared__ __align__(16) float sS[SURF_KP][TG];      // statistics, genealogy-contiguous
  __shared__ __align__(16) float2 sPff[TP][SURF_K + 1];
  __shared__ float sOff[TP];                           // margin + screening error bound
  __shared__ unsigned sBest[TP];                       // best known maximum per point (this tile's thresholds)
  __shared__ unsigned sBestNext[TP];                   // maxima found during the current tile
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int p0 = blockIdx.x * TP;
  const int g0 = blockIdx.y * chunk, g1 = min(S.G, g0 + chunk);
  for (int k = tid; k < SURF_KP * TP; k += BS) {
    int kk = k / TP, p = k % TP;
    sP[kk][p] = (p0 + p < npoints) ? S.phi32[(size_t)(p0 + p) * SURF_KP + kk] : 0.0f;
  }
  for (int k = tid; k < TP * SURF_K; k += BS) {
    int p = k / SURF_K, kk = k % SURF_K;
    sPff[p][kk] = (p0 + p < npoints) ? S.phiff[(size_t)(p0 + p) * SURF_K + kk] : make_float2(0.f, 0.f);
  }
  for (int p = tid; p < TP; p += BS) {
    bool ok = p0 + p < npoints;
    sOff[p] = ok ? FP32_SCREEN_ERR * S.mag[p0 + p] + SURF_MARGIN : 0.f;
    sBest[p] = f2ord(ok ? S.seed[p0 + p] : -INFINITY);
    sBestNext[p] = sBest[p];
  }
  __syncthreads();
  LseState st[4];
#pragma unroll
  for (int j = 0; j < 4; j++) st[j].init();
  for (int t0 = g0; t0 < g1; t0 += TG) {
    const int nt = min(TG, g1 - t0);
    __syncthreads();
    // every drain of the previous tile is done: its maxima become thresholds
    for (int p = tid; p < TP; p += BS) sBest[p] = sBestNext[p];
    for (int k = tid; k < SURF_KP * TG; k += BS) {
      int kk = k / TG, g = k % TG;
      sS[kk][g] = (g < nt) ? S.sT[(size_t)kk * S.Gpad + t0 + g] : 0.0f;
    }
    __syncthreads();
    float acc[8][4];
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int j = 0; j < 4; j++) acc[i][j] = 0.f;
#pragma unroll
    for (int k = 0; k < SURF_KP; k++) {
      float4 pv = *reinterpret_cast<const float4 *>(&sP[k][4 * tx]);
      float4 g0v = *reinterpret_cast<const float4 *>(&sS[k][8 * ty]);
      float4 g1v = *reinterpret_cast<const float4 *>(&sS[k][8 * ty + 4]);
      float gv[8] = {g0v.x, g0v.y, g0v.z, g0v.w, g1v.x, g1v.y, g1v.z, g1v.w};
      float pw[4] = {pv.x, pv.y, pv.z, pv.w};
#pragma unroll
      for (int i = 0; i < 8; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) acc[i][j] = fmaf(gv[i], pw[j], acc[i][j]);
    }
    float thr[4];
#pragma unroll
    for (int j = 0; j < 4; j++) thr[j] = ord2f(sBest[4 * tx + j]) - sOff[4 * tx + j];
    unsigned mask = 0;
#pragma unroll
    for (int i = 0; i < 8; i++)
#pragma unroll
      for (int j = 0; j < 4; j++)
        if (8 * ty + i < nt && acc[i][j] > thr[j]) mask |= 1u << (i * 4 + j);
    // drain candidates: every lane refines one per pass
    while (__any_sync(0xffffffffu, mask != 0)) {
      if (mask) {
        int b = __ffs(mask) - 1;
        mask &= mask - 1;
        int i = b >> 2, j = b & 3;
        int gl = 8 * ty + i, pl = 4 * tx + j;
        ff y = surf_exact(S, t0 + gl, &sS[0][gl], TG, sPff[pl]);
#pragma unroll
        for (int jj = 0; jj < 4; jj++)
          if (jj == j) {
            float before = st[jj].m.hi;
            st[jj].add(y);
            if (st[jj].m.hi > before) atomicMax(&sBestNext[pl], f2ord(st[jj].m.hi));
          }
      }
    }
  }
  // merge the 16 genealogy lanes of every point: the two halves of each warp
  // by shuffle, then the 8 warps through shared memory
#pragma unroll
  for (int j = 0; j < 4; j++) {
    SurfPart o = st[j].pack();
    o.mh = __shfl_xor_sync(0xffffffffu, o.mh, 16);
    o.ml = __shfl_xor_sync(0xffffffffu, o.ml, 16);
    o.sh = __shfl_xor_sync(0xffffffffu, o.sh, 16);
    o.sl = __shfl_xor_sync(0xffffffffu, o.sl, 16);
    o.s2 = __shfl_xor_sync(0xffffffffu, o.s2, 16);
    st[j].merge(o);
  }
  __syncthreads();
  SurfPart *red = reinterpret_cast<SurfPart *>(&sS[0][0]);  // reuse: 8 x 64 x 24 B = 12 KB
  if ((tid & 31) < 16)
    for (int j = 0; j < 4; j++) red[(tid >> 5) * TP + 4 * tx + j] = st[j].pack();
  __syncthreads();
  if (tid < TP) {
    LseState m;
    m.init();
    for (int r = 0; r < BS / 32; r++) m.merge(red[r * TP + tid]);
    if (p0 + tid < npoints) part[(size_t)(p0 + tid) * gridDim.y + blockIdx.y] = m.pack();
  }
}

}  // namespace

size_t surface_fast_scratch_bytes(int G, int npoints)
{
  return surf_prep_bytes(G, npoints) + (size_t)npoints * SURF_MAX_CHUNKS * sizeof(SurfPart) + 256;
}

int launch_surface_fast(const SurfArgs &a, void *scratch, size_t scratch_bytes, bool rows_ready, int *nkernels,
                        cudaStream_t st)
{
  if (a.np + a.nm > SURF_K / 2) return 2;
  if (scratch_bytes < surface_fast_scratch_bytes(a.G, a.npoints)) return 3;
  SurfPrep S;
  char *base = static_cast<char *>(scratch);
  SurfPart *part = surf_prep_carve(&S, base, a.G, a.npoints);
  surf_prep(a, S, false, rows_ready, st);
  surf_seed(S, a.npoints, SURF_SEED, st);
  int nchunks = (a.G + 65535) / 65536;
  if (nchunks > SURF_MAX_CHUNKS) nchunks = SURF_MAX_CHUNKS;
  int chunk = (a.G + nchunks - 1) / nchunks;
  chunk = (chunk + TG - 1) / TG * TG;
  nchunks = (a.G + chunk - 1) / chunk;
  dim3 grid((a.npoints + TP - 1) / TP, nchunks);
  k_surf_screen_fp32<<<grid, BS, 0, st>>>(S, a.npoints, chunk, part);
  surf_merge(a, part, nchunks, st);
  *nkernels = (rows_ready ? 0 : 1) + 4;  // rows, points, seed, screen, merge
  return 0;
}
