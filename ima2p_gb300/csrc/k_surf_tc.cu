// k_surf_tc.cu -- tensor-core screen of the L-mode surface (tcgen05, sm_103a).
//
// The screen of the split-precision surface (see k_surf_fast.cu) as a
// split-bf16 GEMM on the 5th-generation tensor cores: D[point][genealogy] =
// phi(x_point) . s_genealogy over 32 columns (26 statistics, the bias, zero
// padding), with both operands split into bf16 hi + lo planes and
// D = phi_hi s_hi + phi_lo s_hi + phi_hi s_lo accumulated in FP32 in tensor
// memory (three K = 32 products, six tcgen05.mma per tile): about 16
// significant bits per product, so few terms reach the exact recomputation.
//
// One CTA owns 128 points (the A operand, loaded once) and streams tiles of
// 256 genealogies (the B operand) through a 4-stage shared-memory ring filled
// by 1-D bulk copies (the TMA engine; the prepared operand is already in the
// tile layout, so one copy per tile).  One thread issues six K=16 MMAs per
// tile into one of two 256-column TMEM accumulators; eight epilogue warps
// drain the other accumulator with tcgen05.ld -- warps 4-7 take genealogy
// columns 0-127, warps 8-11 columns 128-255, each thread one point (its TMEM
// lane) -- and send every term within MARGIN + screen error of the point's
// best maximum to the exact float-float recomputation.
//
// Every wait is bounded: a wait that runs out sets the error word, the CTA
// stops issuing work, waits (bounded) for the copies and MMAs it started,
// frees its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cstring>

#include "surf_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TC_M = SURF_TC_M;  // points per CTA (TMEM lanes)
constexpr int TC_N = SURF_TC_N;  // genealogies per tile (accumulator columns)
constexpr int TC_STAGES = 4;
constexpr uint32_t A_PLANE = TC_M * SURF_KP * 2;   // 8 KB
constexpr uint32_t B_PLANE = TC_N * SURF_KP * 2;   // 16 KB
constexpr uint32_t A_BYTES = 2 * A_PLANE;          // hi + lo
constexpr uint32_t B_BYTES = 2 * B_PLANE;
// shared memory requested per CTA: more than half an SM's, so one CTA holds
// an SM and its 512 TMEM columns at a time
constexpr size_t TC_SMEM = 152 * 1024;
constexpr uint32_t WAIT_LIMIT = 1u << 24;          // polls before a wait gives up
constexpr int TC_THREADS = 384;                    // warp 0 loads, warp 1 MMAs, 4-11 epilogue

// split-bf16 screen error, relative to sum_k colmax_k |phi_k| (u = 2^-8, the
// bf16 unit roundoff): the dropped lo*lo product and the residuals of both
// splits, <= 3 u^2 = 4.6e-5 per product, plus the FP32 accumulation of 96
// products even if every addition truncates, <= 96 * 2^-23 = 1.1e-5;
// bounded with margin by 1e-4.
constexpr float BF16_SCREEN_ERR = 1e-4f;

struct TcSmem {
  uint64_t full[TC_STAGES], empty[TC_STAGES], accfull[2], accempty[2], abar;
  uint32_t tmem;
  int err;
};

__device__ __forceinline__ void set_err(int *err_shared, int *err_global, int code)
{
  atomicCAS(err_shared, 0, code);
  atomicCAS(err_global, 0, code);
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_surf_tc(SurfPrep S, int npoints, int tiles_per_chunk, SurfPart *part, int *gerr)
{
  extern __shared__ __align__(1024) char smem[];
  char *bufA = smem;
  char *bufB = smem + A_BYTES;
  TcSmem &sh = *reinterpret_cast<TcSmem *>(smem + A_BYTES + TC_STAGES * B_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ptile = blockIdx.x;
  const int ntiles_all = S.Gpad / TC_N;
  const int t0 = blockIdx.y * tiles_per_chunk, t1 = min(ntiles_all, t0 + tiles_per_chunk);
  const int ntiles = max(0, t1 - t0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      tc::mbar_init(&sh.full[s], 1);
      tc::mbar_init(&sh.empty[s], 1);
    }
    for (int a = 0; a < 2; a++) {
      tc::mbar_init(&sh.accfull[a], 1);
      tc::mbar_init(&sh.accempty[a], 8);  // one arrival per epilogue warp
    }
    tc::mbar_init(&sh.abar, 1);
    sh.err = 0;
    tc::fence_barrier_init();
  }
  if (warp == 1) {
    tc::tmem_alloc(&sh.tmem, 512);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sh.tmem;

  if (warp == 0 && lane == 0) {
    // ------------------------------------------------------------ loader
    tc::mbar_expect_tx(&sh.abar, A_BYTES);
    tc::bulk_g2s(bufA, S.pbf + (size_t)ptile * (A_BYTES / 2), A_BYTES, &sh.abar);
    int issued = 0;
    for (int i = 0; i < ntiles; i++) {
      const int s = i % TC_STAGES;
      if (i >= TC_STAGES && !tc::mbar_wait(&sh.empty[s], ((i / TC_STAGES) - 1) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 1);
        break;
      }
      if (*(volatile int *)&sh.err) break;
      tc::mbar_expect_tx(&sh.full[s], B_BYTES);
      tc::bulk_g2s(bufB + s * B_BYTES, S.sbf + (size_t)(t0 + i) * (B_BYTES / 2), B_BYTES, &sh.full[s]);
      issued = i + 1;
    }
    // copies this thread started must land before the CTA can leave
    for (int i = max(0, issued - TC_STAGES); i < issued; i++)
      tc::mbar_wait(&sh.full[i % TC_STAGES], (i / TC_STAGES) & 1, WAIT_LIMIT);
    tc::mbar_wait(&sh.abar, 0, WAIT_LIMIT);
  } else if (warp == 1 && lane == 0) {
    // --------------------------------------------------------------- MMA
    const uint32_t idesc = tc::idesc_bf16_f32(TC_M, TC_N);
    const uint32_t aaddr = tc::smem_u32(bufA);
    bool ok = tc::mbar_wait(&sh.abar, 0, WAIT_LIMIT);
    if (!ok) set_err(&sh.err, gerr, 2);
    int done = 0;
    for (int i = 0; ok && i < ntiles; i++) {
      const int s = i % TC_STAGES, a = i & 1;
      if (!tc::mbar_wait(&sh.full[s], (i / TC_STAGES) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 3);
        break;
      }
      if (i >= 2 && !tc::mbar_wait(&sh.accempty[a], ((i >> 1) - 1) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 4);
        break;
      }
      if (*(volatile int *)&sh.err) break;
      tc::fence_after_sync();
      const uint32_t baddr = tc::smem_u32(bufB + s * B_BYTES);
      const uint32_t d = tmem + (uint32_t)(a * TC_N);
      // phi_hi s_hi + phi_lo s_hi + phi_hi s_lo, each K = 32 as two K = 16
      const uint32_t ap[3] = {aaddr, aaddr + A_PLANE, aaddr};
      const uint32_t bp[3] = {baddr, baddr, baddr + B_PLANE};
#pragma unroll
      for (int t = 0; t < 3; t++)
#pragma unroll
        for (int kh = 0; kh < 2; kh++)
          tc::mma_bf16(d, tc::sdesc(ap[t] + kh * 256, 128, 512), tc::sdesc(bp[t] + kh * 256, 128, 512),
                       idesc, (t | kh) ? 1u : 0u);
      tc::mma_commit(&sh.empty[s]);   // stage s free once these MMAs have read it
      tc::mma_commit(&sh.accfull[a]); // accumulator a ready for the epilogue
      done = i + 1;
    }
    if (done > 0) tc::mbar_wait(&sh.accfull[(done - 1) & 1], ((done - 1) >> 1) & 1, WAIT_LIMIT);
  } else if (warp >= 4) {
    // ---------------------------------------------------------- epilogue
    const int q = warp & 3;             // TMEM lane quarter of this warp
    const int half = (warp - 4) >> 2;   // genealogy columns [128 half, +128)
    const int pl = q * 32 + lane;       // point within the tile = TMEM lane
    const int p = ptile * TC_M + pl;
    const bool live = p < npoints;
    float2 phi[SURF_K];
    float off = 0.f, best = -INFINITY;
    if (live) {
      for (int k = 0; k < S.K; k++) phi[k] = S.phiff[(size_t)p * SURF_K + k];
      off = BF16_SCREEN_ERR * S.mag[p] + SURF_MARGIN;
      best = S.seed[p];
    }
    LseState st;
    st.init();
    for (int i = 0; i < ntiles; i++) {
      const int a = i & 1;
      if (!tc::mbar_wait(&sh.accfull[a], (i >> 1) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 5);
        break;
      }
      tc::fence_after_sync();
      const int gbase = (t0 + i) * TC_N + half * 128;
      const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * TC_N + half * 128);
#pragma unroll 1
      for (int c = 0; c < 4; c++) {
        float v[32];
        tc::tmem_ld32(tl + c * 32, v);
        const float thr = best - off;
        unsigned mask = 0;
#pragma unroll
        for (int j = 0; j < 32; j++)
          if (v[j] > thr) mask |= 1u << j;
        if (!live) mask = 0;
        while (mask) {
          const int j = __ffs(mask) - 1;
          mask &= mask - 1;
          const int g = gbase + c * 32 + j;
          if (g >= S.G) continue;
          ff y = surf_exact(S, g, S.sT + g, S.Gpad, phi);
          st.add(y);
          best = fmaxf(best, y.hi);
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&sh.accempty[a]);
    }
    if (live) part[((size_t)p * 2 + half) * gridDim.y + blockIdx.y] = st.pack();
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
}

__global__ void k_tc_merge(SurfArgs a, const SurfPart *part, int nchunks)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npoints) return;
  LseState m;
  m.init();
  for (int h = 0; h < 2; h++)
    for (int c = 0; c < nchunks; c++) m.merge(part[((size_t)p * 2 + h) * nchunks + c]);
  // the FP64 merge kernel reads one partial per (point, chunk)
  SurfPart *out = const_cast<SurfPart *>(part) + (size_t)a.npoints * 2 * nchunks;
  out[p] = m.pack();
}

// ------------------------------------------------------------ self-test
// One 128 x 256 x 32 tile of small integers (exact in bf16 and FP32),
// checked element by element against CUDA cores.
__global__ void __launch_bounds__(128, 1) k_tc_selftest(const uint16_t *A, const uint16_t *B, float *D,
                                                         int *err)
{
  constexpr uint32_t A_BYTES = A_PLANE, B_BYTES = B_PLANE;
  extern __shared__ __align__(1024) char smem[];
  char *bufA = smem, *bufB = smem + A_BYTES;
  __shared__ uint64_t bar, mbar;
  __shared__ uint32_t tslot;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    tc::mbar_init(&bar, 1);
    tc::mbar_init(&mbar, 1);
    tc::fence_barrier_init();
  }
  if (warp == 0) {
    tc::tmem_alloc(&tslot, 256);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = tslot;
  __shared__ int ok;
  if (threadIdx.x == 0) {
    ok = 1;
    tc::mbar_expect_tx(&bar, A_BYTES + B_BYTES);
    tc::bulk_g2s(bufA, A, A_BYTES, &bar);
    tc::bulk_g2s(bufB, B, B_BYTES, &bar);
    if (!tc::mbar_wait(&bar, 0, WAIT_LIMIT)) {
      ok = 0;
      atomicCAS(err, 0, 1);
    } else {
      tc::fence_after_sync();
      const uint32_t idesc = tc::idesc_bf16_f32(TC_M, TC_N);
      const uint32_t aa = tc::smem_u32(bufA), bb = tc::smem_u32(bufB);
      for (int kh = 0; kh < 2; kh++)
        tc::mma_bf16(tmem, tc::sdesc(aa + kh * 256, 128, 512), tc::sdesc(bb + kh * 256, 128, 512), idesc, kh);
      tc::mma_commit(&mbar);
    }
  }
  __syncthreads();
  if (ok) {
    if (!tc::mbar_wait(&mbar, 0, WAIT_LIMIT)) {
      atomicCAS(err, 0, 2);
    } else {
      tc::fence_after_sync();
      const int row = warp * 32 + lane;
      for (int c = 0; c < TC_N / 32; c++) {
        float v[32];
        tc::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 32), v);
        for (int j = 0; j < 32; j++) D[(size_t)row * TC_N + c * 32 + j] = v[j];
      }
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 0) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 256);
  }
}

__device__ __forceinline__ int st_a(int r, int k) { return ((r * 7 + k * 3) % 17) - 8; }
__device__ __forceinline__ int st_b(int n, int k) { return ((n * 5 + k * 11) % 13) - 6; }

__global__ void k_tc_selftest_fill(uint16_t *A, uint16_t *B)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < TC_M * SURF_KP) {
    int r = i / SURF_KP, k = i % SURF_KP;
    __nv_bfloat16 v = __float2bfloat16_rn((float)st_a(r, k));
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(A) + tc::tile_off(r, k)) = v;
  }
  if (i < TC_N * SURF_KP) {
    int n = i / SURF_KP, k = i % SURF_KP;
    __nv_bfloat16 v = __float2bfloat16_rn((float)st_b(n, k));
    *reinterpret_cast<__nv_bfloat16 *>(reinterpret_cast<char *>(B) + tc::tile_off(n, k)) = v;
  }
}

__global__ void k_tc_selftest_check(const float *D, int *bad, float *maxerr)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= TC_M * TC_N) return;
  int r = i / TC_N, n = i % TC_N;
  int want = 0;
  for (int k = 0; k < SURF_KP; k++) want += st_a(r, k) * st_b(n, k);
  float e = fabsf(D[i] - (float)want);
  if (e != 0.f) atomicAdd(bad, 1);
  atomicMax(reinterpret_cast<int *>(maxerr), __float_as_int(e));
}

}  // namespace

// ---------------------------------------------------------------- host
size_t surface_tc_scratch_bytes(int G, int npoints)
{
  const int nchunks = SURF_MAX_CHUNKS;
  return surf_prep_bytes(G, npoints) + ((size_t)npoints * 2 * nchunks + npoints) * sizeof(SurfPart) + 1024;
}

int launch_surface_tc(const SurfArgs &a, void *scratch, size_t scratch_bytes, int *d_err, cudaStream_t st)
{
  if (a.np + a.nm > SURF_K / 2) return 2;
  if (scratch_bytes < surface_tc_scratch_bytes(a.G, a.npoints)) return 3;
  SurfPrep S;
  SurfPart *part = surf_prep_carve(&S, static_cast<char *>(scratch), a.G, a.npoints);
  surf_prep(a, S, true, st);
  surf_seed(S, a.npoints, st);
  const int ntiles = S.Gpad / TC_N;
  const int ptiles = (a.npoints + TC_M - 1) / TC_M;
  // genealogy chunks: enough CTAs for every SM, at least 8 tiles per CTA
  int nchunks = (2 * 152 + ptiles - 1) / ptiles;
  nchunks = std::max(1, std::min(nchunks, std::min(SURF_MAX_CHUNKS, (ntiles + 7) / 8)));
  const int per = (ntiles + nchunks - 1) / nchunks;
  nchunks = (ntiles + per - 1) / per;
  static_assert(A_BYTES + TC_STAGES * B_BYTES + sizeof(TcSmem) + 1024 <= TC_SMEM, "smem");
  const size_t sm = TC_SMEM;
  cudaFuncSetAttribute(k_surf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  dim3 grid(ptiles, nchunks);
  k_surf_tc<<<grid, TC_THREADS, sm, st>>>(S, a.npoints, per, part, d_err);
  k_tc_merge<<<(a.npoints + 127) / 128, 128, 0, st>>>(a, part, nchunks);
  surf_merge(a, part + (size_t)a.npoints * 2 * nchunks, 1, st);
  return 0;
}

int tc_selftest(cudaStream_t st, void *scratch, size_t bytes, int *h_bad, float *h_maxerr)
{
  constexpr uint32_t A_BYTES = A_PLANE, B_BYTES = B_PLANE;
  // scratch: A (8 KB) | B (16 KB) | D (128 KB) | bad, maxerr, err
  const size_t need = A_BYTES + B_BYTES + (size_t)TC_M * TC_N * 4 + 16;
  if (bytes < need) return 3;
  char *p = static_cast<char *>(scratch);
  uint16_t *A = reinterpret_cast<uint16_t *>(p);
  uint16_t *B = reinterpret_cast<uint16_t *>(p + A_BYTES);
  float *D = reinterpret_cast<float *>(p + A_BYTES + B_BYTES);
  int *bad = reinterpret_cast<int *>(p + A_BYTES + B_BYTES + (size_t)TC_M * TC_N * 4);
  float *mx = reinterpret_cast<float *>(bad + 1);
  int *err = bad + 2;
  cudaMemsetAsync(p, 0, need, st);
  k_tc_selftest_fill<<<(TC_N * SURF_KP + 255) / 256, 256, 0, st>>>(A, B);
  const size_t sm = A_BYTES + B_BYTES + 1024;
  cudaFuncSetAttribute(k_tc_selftest, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_tc_selftest<<<1, 128, sm, st>>>(A, B, D, err);
  k_tc_selftest_check<<<(TC_M * TC_N + 255) / 256, 256, 0, st>>>(D, bad, mx);
  int out[3];
  cudaMemcpyAsync(out, bad, sizeof(out), cudaMemcpyDeviceToHost, st);
  if (cudaStreamSynchronize(st) != cudaSuccess) return 4;
  *h_bad = out[2] ? -out[2] : out[0];
  memcpy(h_maxerr, &out[1], sizeof(float));
  return 0;
}
