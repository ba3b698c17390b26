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
// 256 genealogies (the B operand) through a 4-stage shared-memory ring
// filled by 1-D bulk copies (the TMA engine; the prepared operand is already
// in the tile layout, so one copy per tile).  Warp roles:
//   warp 0     one thread issues the bulk copies;
//   warp 1     one thread issues six K=16 MMAs per tile into one of two
//              256-column TMEM accumulators;
//   warps 4-19 drain the accumulators with tcgen05.ld -- warp w reads TMEM
//              lane quarter w % 4 (32 points, one per thread) and 64
//              genealogy columns -- and a max tree over each thread's values
//              decides whether any lies within MARGIN + screen error of the
//              point's lower bound; such candidates go to a ring;
//   warps 2-3  take the rings' candidates 32 at a time, recompute them
//              exactly (phi of every point is staged in shared memory) and
//              add exp(p - ref) to the point's sums.
//
// Results are bit-for-bit reproducible.  Two things would otherwise follow
// timing: which terms pass the screen, and the order in which they are added.
//   * The set: a drain warp's threshold is the point's lower bound from the
//     max-only pre-pass (a maximum over a fixed set of values, so fixed) raised
//     only by the screened maxima of the warp's own earlier tiles.  Nothing
//     another warp or chunk found moves it, so every warp screens the same
//     terms on every run.
//   * The order: each term's weight w = exp(p - ref), with ref the pre-pass
//     bound, is added as a 256-bit fixed-point integer (w * 2^64) by 64-bit
//     shared-memory atomics with exact carries.  Integer addition is
//     associative, so the sum does not depend on arrival order; the chunk
//     sums are merged in chunk order.
// A term with w >= 2^80 (the pre-pass bound more than 55 nats below the
// term) would leave the fixed-point range: the point is flagged.  The pass
// also keeps each point's largest exact value, a maximum and so the same on
// every run; the flagged points are then taken again by a second pass over
// just them, with that value as the reference, where no term can exceed it.
//
// Every wait is bounded: a wait that runs out sets the error word, the CTA
// stops issuing work, waits (bounded) for the copies and MMAs it started,
// frees its TMEM and returns.
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "surf_common.cuh"
#include "tc_ptx.cuh"

namespace {

constexpr int TC_M = SURF_TC_M;  // points per CTA (TMEM lanes)
constexpr int TC_N = SURF_TC_N;  // genealogies per tile (accumulator columns)
constexpr int NACC = 512 / TC_N;     // TMEM accumulators of TC_N columns
constexpr uint32_t A_PLANE = TC_M * SURF_KP * 2;   // 8 KB
constexpr uint32_t B_PLANE = TC_N * SURF_KP * 2;
constexpr uint32_t A_BYTES = 2 * A_PLANE;          // hi + lo
constexpr uint32_t B_BYTES = 2 * B_PLANE;
constexpr int TC_STAGES = (128 * 1024) / B_BYTES;  // operand ring stages (128 KB of B tiles)
static_assert(TC_STAGES >= NACC, "a stage's done barrier also marks its accumulator ready");
// shared memory requested per CTA: more than half an SM's, so one CTA holds
// an SM and its 512 TMEM columns at a time (the operand ring, phi of the
// CTA's points, the candidate rings and the per-point log-sum-exp states)
constexpr size_t TC_SMEM = 212 * 1024;
constexpr uint32_t WAIT_LIMIT = 1u << 24;          // try_wait rounds before a wait gives up
constexpr int TC_THREADS = 640;                    // roles: see the file comment

// split-bf16 screen error, relative to sum_k colmax_k |phi_k| (u = 2^-8, the
// bf16 unit roundoff): the dropped lo*lo product and the residuals of both
// splits, <= 3 u^2 = 4.6e-5 per product, plus the FP32 accumulation of 96
// products even if every addition truncates, <= 96 * 2^-23 = 1.1e-5;
// bounded with margin by 1e-4.
constexpr float BF16_SCREEN_ERR = 1e-4f;

constexpr int PHI_STRIDE = SURF_K + 1;   // float2 per point row of staged phi (padded)
constexpr int EPI_WARPS = 16;            // warps 4-19 drain the accumulators
constexpr int COL_GROUPS = EPI_WARPS / 4;          // accumulator column groups (TMEM lane quarters x 4)
constexpr int GROUP_COLS = TC_N / COL_GROUPS;      // columns per epilogue warp and tile
constexpr int REF_WARPS = 2;             // warps 2-3 recompute candidates exactly
constexpr int RING = 1024;               // candidate slots per refine warp

constexpr int FIXW = 4;  // 64-bit words of the fixed-point sums

struct TcSmem {
  // full[s]: B tile of stage s landed; done[s]: the MMAs of the tile in stage
  // s completed (stage free, accumulator ready); accempty[a]: accumulator a
  // drained by every epilogue warp
  uint64_t full[TC_STAGES], done[TC_STAGES], accempty[NACC], abar;
  uint32_t tmem;
  int err;
  int epi_done;                       // epilogue warps that have finished
  unsigned head[REF_WARPS];           // slots reserved so far in each ring
  int ring[REF_WARPS][RING];          // candidates: genealogy << 7 | point; -1 = free
  unsigned long long sum[TC_M][FIXW];   // sum of w * 2^64, w = exp(p - ref), 256-bit fixed point
  unsigned long long sum2[TC_M][FIXW];  // sum of w^2 * 2^64
  float ref[TC_M];                    // the point's lower bound after the pre-pass
  unsigned xmax[TC_M];                // largest exact value refined (ordered bits)
  int ovf[TC_M];                      // a term left the fixed-point range
  float2 phi[TC_M * PHI_STRIDE];      // float-float phi of the CTA's points
};

// w >= 2^80 (55.45 nats above ref) leaves the range the sums are sized for:
// 2^24 genealogies of w^2 * 2^64 < 2^160 * 2^64 stay below 2^248
constexpr double OVF_NATS = 55.0;

// w * 2^64 as a 256-bit integer, truncated (0 <= w < 2^180)
__device__ __forceinline__ void fixw(double w, unsigned long long o[FIXW])
{
#pragma unroll
  for (int i = 0; i < FIXW; i++) o[i] = 0ull;
  const unsigned long long b = (unsigned long long)__double_as_longlong(w);
  const int e = (int)((b >> 52) & 0x7ff);
  if (!(w > 0.0) || e == 0) return;  // zero or subnormal: nothing at this scale
  const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
  const int s = e - 1023 - 52 + 64;  // w * 2^64 = m * 2^s
  if (s <= -53) return;
  if (s < 0) {
    o[0] = m >> (-s);
    return;
  }
  const int wd = s >> 6, bit = s & 63;
  if (wd < FIXW) o[wd] = m << bit;
  if (bit && wd + 1 < FIXW) o[wd + 1] = m >> (64 - bit);
}

// acc += x on a 256-bit integer in shared memory, word by word with 64-bit
// atomics; a word that wraps carries one into the next.  Every wrap is seen
// by exactly one atomic, so the sum is exact whatever the interleaving.
__device__ __forceinline__ void atomic_addw(unsigned long long *acc, const unsigned long long x[FIXW])
{
  unsigned long long carry = 0ull;
#pragma unroll
  for (int i = 0; i < FIXW; i++) {
    unsigned long long out = 0ull;
    if (x[i]) {
      const unsigned long long old = atomicAdd(&acc[i], x[i]);
      out += (old + x[i] < old) ? 1ull : 0ull;
    }
    if (carry) {
      const unsigned long long old = atomicAdd(&acc[i], carry);
      out += (old + carry < old) ? 1ull : 0ull;
    }
    carry = out;
  }
}

__device__ __forceinline__ double fixw_to_double(const unsigned long long w[FIXW])
{
  // powers of two are exact; the order of the additions is fixed
  double v = 0.0;
#pragma unroll
  for (int i = FIXW - 1; i >= 0; i--) v = v * 18446744073709551616.0 + (double)w[i];
  return v * 5.421010862427522e-20;  // 2^-64
}

__device__ __forceinline__ void set_err(int *err_shared, int *err_global, int code)
{
  atomicCAS(err_shared, 0, code);
  atomicCAS(err_global, 0, code);
}

// hand one candidate (point pl, genealogy g) to the refine warp owning pl
__device__ __forceinline__ void push_candidate(TcSmem &sh, int *gerr, int pl, int g)
{
  const int r = pl & 1;
  const unsigned slot = atomicAdd(&sh.head[r], 1u);
  volatile int *dst = &sh.ring[r][slot % RING];
  // the slot is free once the refine warp has taken its previous occupant
  for (uint32_t it = 0; *dst != -1; it++) {
    if (it > WAIT_LIMIT || *(volatile int *)&sh.err) {
      set_err(&sh.err, gerr, 6);
      return;
    }
    __nanosleep(32);
  }
  *dst = (g << 7) | pl;
}

// Refine warp r: takes its ring's candidates 32 at a time, recomputes each
// exactly (one per lane) and adds its weight to its point's sums.  It stops
// when every epilogue warp has finished and the ring is drained.
__device__ void refine_loop(const SurfPrep &S, TcSmem &sh, int *gerr, int r, int lane)
{
  for (unsigned next = 0;; next += 32) {
    const unsigned slot = next + lane;
    volatile int *src = &sh.ring[r][slot % RING];
    int e = -1;
    for (uint32_t it = 0;; it++) {
      e = *src;
      if (e != -1) break;
      if (*(volatile int *)&sh.epi_done == EPI_WARPS && slot >= *(volatile unsigned *)&sh.head[r]) break;
      if (*(volatile int *)&sh.err) break;
      if (it > WAIT_LIMIT) {
        set_err(&sh.err, gerr, 7);
        break;
      }
      __nanosleep(64);
    }
    const bool have = e != -1;
    if (have) {
      *src = -1;
      const int pl = e & (TC_M - 1), g = e >> 7;
      const ff y = surf_exact(S, g, S.sT + g, S.Gpad, &sh.phi[pl * PHI_STRIDE]);
      atomicMax(&sh.xmax[pl], f2ord(y.hi));
      const ff d = ff_sub(y, ff_from(sh.ref[pl]));
      if (d.hi > (float)OVF_NATS) {
        sh.ovf[pl] = 1;
      } else {
        // w = e^d in float-float (FP32 pipes: GB300 runs FP64 at 1/64 of
        // the FP32 rate); hi + lo is exact in a double, and w^2 (up to 2^160,
        // beyond FP32's range) is squared there
        ff e, em1;
        ff_exp_expm1(d, &e, &em1);
        const double w = (double)e.hi + (double)e.lo;
        unsigned long long x[FIXW];
        fixw(w, x);
        atomic_addw(sh.sum[pl], x);
        fixw(w * w, x);
        atomic_addw(sh.sum2[pl], x);
      }
    }
    if (!__any_sync(0xffffffffu, have)) break;
  }
}

// stride > 0: max-only pass over genealogy tiles 0, stride, 2 stride, ...
// that only raises the per-point lower bounds S.best (no candidates, no
// partials); stride == 0: the full pass over every tile, which reads S.best
// and leaves it unchanged.
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_surf_tc(SurfPrep S, int npoints, int tiles_per_chunk, int stride, double2 *part, int *gerr)
{
  extern __shared__ __align__(1024) char smem[];
  char *bufA = smem;
  char *bufB = smem + A_BYTES;
  TcSmem &sh = *reinterpret_cast<TcSmem *>(smem + A_BYTES + TC_STAGES * B_BYTES);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ptile = blockIdx.x;
  const bool maxonly = stride > 0;
  const int step = maxonly ? stride : 1;
  const int ntiles_all = (S.Gpad / TC_N + step - 1) / step;  // tiles of this pass
  const int t0 = blockIdx.y * tiles_per_chunk, t1 = min(ntiles_all, t0 + tiles_per_chunk);
  const int ntiles = max(0, t1 - t0);

  if (threadIdx.x == 0) {
    for (int s = 0; s < TC_STAGES; s++) {
      tc::mbar_init(&sh.full[s], 1);
      tc::mbar_init(&sh.done[s], 1);
    }
    for (int a = 0; a < NACC; a++) tc::mbar_init(&sh.accempty[a], EPI_WARPS);  // one arrival per epilogue warp
    tc::mbar_init(&sh.abar, 1);
    sh.err = 0;
    sh.epi_done = 0;
    for (int r = 0; r < REF_WARPS; r++) sh.head[r] = 0;
    tc::fence_barrier_init();
  }
  // every thread stages phi, the rings and the per-point states
  for (int i = threadIdx.x; i < TC_M * SURF_K; i += TC_THREADS) {
    const int pl = i / SURF_K, k = i % SURF_K, p = ptile * TC_M + pl;
    sh.phi[pl * PHI_STRIDE + k] = p < npoints ? S.phiff[(size_t)p * SURF_K + k] : make_float2(0.f, 0.f);
  }
  for (int i = threadIdx.x; i < REF_WARPS * RING; i += TC_THREADS) (&sh.ring[0][0])[i] = -1;
  for (int pl = threadIdx.x; pl < TC_M; pl += TC_THREADS) {
    for (int w = 0; w < FIXW; w++) sh.sum[pl][w] = sh.sum2[pl][w] = 0ull;
    const int p = ptile * TC_M + pl;
    sh.ref[pl] = p < npoints ? ord2f(S.best[p]) : -INFINITY;
    sh.xmax[pl] = f2ord(-INFINITY);
    sh.ovf[pl] = 0;
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
      if (i >= TC_STAGES && !tc::mbar_wait(&sh.done[s], ((i / TC_STAGES) - 1) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 1);
        break;
      }
      if (*(volatile int *)&sh.err) break;
      tc::mbar_expect_tx(&sh.full[s], B_BYTES);
      tc::bulk_g2s(bufB + s * B_BYTES, S.sbf + (size_t)(t0 + i) * step * (B_BYTES / 2), B_BYTES, &sh.full[s]);
      issued = i + 1;
    }
    // copies this thread started must land before the CTA can leave
    for (int i = max(0, issued - TC_STAGES); i < issued; i++)
      tc::mbar_wait(&sh.full[i % TC_STAGES], (i / TC_STAGES) & 1, WAIT_LIMIT);
    tc::mbar_wait(&sh.abar, 0, WAIT_LIMIT);
  } else if (warp == 1 && lane == 0) {
    // --------------------------------------------------------------- MMA
    const uint32_t idesc = tc::idesc_bf16_f32(TC_M, TC_N);
    // descriptors: the address field counts 16-byte units, so offsets add
    const uint64_t ad = tc::sdesc(tc::smem_u32(bufA), 128, 512);
    const uint64_t bd0 = tc::sdesc(tc::smem_u32(bufB), 128, 512);
    bool ok = tc::mbar_wait(&sh.abar, 0, WAIT_LIMIT);
    if (!ok) set_err(&sh.err, gerr, 2);
    int ndone = 0;
    for (int i = 0; ok && i < ntiles; i++) {
      const int s = i % TC_STAGES, a = i % NACC;
      if (!tc::mbar_wait(&sh.full[s], (i / TC_STAGES) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 3);
        break;
      }
      if (i >= NACC && !tc::mbar_wait(&sh.accempty[a], ((i / NACC) - 1) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 4);
        break;
      }
      if (*(volatile int *)&sh.err) break;
      tc::fence_after_sync();
      const uint32_t d = tmem + (uint32_t)(a * TC_N);
      const uint64_t bd = bd0 + (uint64_t)((s * B_BYTES) >> 4);
      // phi_hi s_hi + phi_lo s_hi + phi_hi s_lo, each K = 32 as two K = 16
      const uint64_t ap[3] = {ad, ad + (A_PLANE >> 4), ad};
      const uint64_t bp[3] = {bd, bd, bd + (B_PLANE >> 4)};
#pragma unroll
      for (int t = 0; t < 3; t++)
#pragma unroll
        for (int kh = 0; kh < 2; kh++)
          tc::mma_bf16(d, ap[t] + kh * 16, bp[t] + kh * 16, idesc, (t | kh) ? 1u : 0u);
      tc::mma_commit(&sh.done[s]);  // stage s free and accumulator a ready once these complete
      ndone = i + 1;
    }
    if (ndone > 0) tc::mbar_wait(&sh.done[(ndone - 1) % TC_STAGES], ((ndone - 1) / TC_STAGES) & 1, WAIT_LIMIT);
  } else if ((warp == 2 || warp == 3) && !maxonly) {
    // ------------------------------------------------------------ refine
    refine_loop(S, sh, gerr, warp - 2, lane);
  } else if (warp >= 4) {
    // ---------------------------------------------------------- epilogue
    const int ew = warp - 4;            // epilogue warp
    const int q = warp & 3;             // TMEM lane quarter of this warp
    const int cg = ew >> 2;             // genealogy columns [GROUP_COLS cg, +GROUP_COLS)
    const int pl = q * 32 + lane;       // point within the tile = TMEM lane
    const int p = ptile * TC_M + pl;
    const bool live = p < npoints;
    const float err = live ? BF16_SCREEN_ERR * S.mag[p] : 0.f;  // screen error bound
    const float off = err + SURF_MARGIN;
    // lb: a lower bound on the point's maximum -- the pre-pass bound raised
    // by this warp's own screened values less their error bound, in tile
    // order, so the threshold of every tile is the same on every run
    float lb = live ? sh.ref[pl] : -INFINITY;
    for (int i = 0; i < ntiles; i++) {
      const int a = i % NACC;
      if (!tc::mbar_wait(&sh.done[i % TC_STAGES], (i / TC_STAGES) & 1, WAIT_LIMIT)) {
        set_err(&sh.err, gerr, 5);
        break;
      }
      tc::fence_after_sync();
      const int gbase = (t0 + i) * step * TC_N + cg * GROUP_COLS;
      const uint32_t tl = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(a * TC_N + cg * GROUP_COLS);
      float mxv;
      float v[32];
      if constexpr (GROUP_COLS == 32) {
        // one load and a max tree; the candidate masks come from the same
        // registers
        uint32_t r[32];
        tc::tmem_ld32_nowait(tl, r);
        tc::tmem_wait_ld(r);
#pragma unroll
        for (int j = 0; j < 32; j++) v[j] = __uint_as_float(r[j]);
        float mx[16];
#pragma unroll
        for (int j = 0; j < 16; j++) mx[j] = fmaxf(v[j], v[j + 16]);
#pragma unroll
        for (int w = 8; w >= 1; w >>= 1)
#pragma unroll
          for (int j = 0; j < w; j++) mx[j] = fmaxf(mx[j], mx[j + w]);
        mxv = mx[0];
      } else {
        // both loads in flight, one wait, a max tree in place; a passing
        // value reloads the columns
        static_assert(GROUP_COLS == 64, "one or two 32-column loads per warp and tile");
        uint32_t r[64];
        tc::tmem_ld32_nowait(tl, r);
        tc::tmem_ld32_nowait(tl + 32, r + 32);
        tc::tmem_wait_ld(r);
        tc::reg_fence32(r + 32);
        float w64[64];
#pragma unroll
        for (int j = 0; j < 64; j++) w64[j] = __uint_as_float(r[j]);
#pragma unroll
        for (int w = 32; w >= 1; w >>= 1)
#pragma unroll
          for (int j = 0; j < w; j++) w64[j] = fmaxf(w64[j], w64[j + w]);
        mxv = w64[0];
      }
      // padded genealogies (g >= G) screen to 0 and must not raise lb
      if (gbase + GROUP_COLS <= S.G) lb = fmaxf(lb, mxv - err);
      const float thr = lb - off;
      const bool hit = live && !maxonly && mxv > thr;
      if (__any_sync(0xffffffffu, hit)) {
#pragma unroll 1
        for (int c = 0; c < GROUP_COLS / 32; c++) {
          if constexpr (GROUP_COLS != 32) tc::tmem_ld32(tl + c * 32, v);
          unsigned mask = 0;
#pragma unroll
          for (int j = 0; j < 32; j++)
            if (v[j] > thr) mask |= 1u << j;
          const int gc = gbase + c * 32, nv = S.G - gc;
          if (!hit) mask = 0;
          else if (nv < 32) mask &= nv > 0 ? (1u << nv) - 1u : 0u;
          for (; mask; mask &= mask - 1) push_candidate(sh, gerr, pl, gc + __ffs(mask) - 1);
        }
      }
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(&sh.accempty[a]);
    }
    // the pre-pass publishes its bound once: a maximum, whatever the order
    if (maxonly && live) atomicMax(&S.best[p], f2ord(lb));
    __syncwarp();
    if (lane == 0) {
      __threadfence_block();
      atomicAdd(&sh.epi_done, 1);
    }
  }
  tc::fence_before_sync();
  __syncthreads();
  if (warp == 1) {
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, 512);
  }
  if (threadIdx.x < TC_M && !maxonly) {
    const int p = ptile * TC_M + threadIdx.x;
    if (p < npoints) atomicMax(&S.xmax[p], sh.xmax[threadIdx.x]);
    if (p < npoints)
      part[(size_t)p * gridDim.y + blockIdx.y] =
          make_double2(sh.ovf[threadIdx.x] ? -1.0 : fixw_to_double(sh.sum[threadIdx.x]),
                       fixw_to_double(sh.sum2[threadIdx.x]));
  }
}

// Chunk sums added in chunk order: q = ln G - (ref + ln sum).  A point with
// a flagged chunk goes to the list of points to take again (flag[0] = list
// length, flag[1..] = points; the list's order does not matter, each point
// is taken on its own).
__global__ void k_surf_tc_merge(SurfArgs a, SurfPrep S, const double2 *part, int nchunks, int *flag)
{
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npoints) return;
  const double2 *w = part + (size_t)p * nchunks;
  double s = 0.0, s2 = 0.0;
  int ovf = 0;
  for (int c = 0; c < nchunks; c++) {
    if (w[c].x < 0.0) ovf = 1;
    s += w[c].x;
    s2 += w[c].y;
  }
  if (ovf) {
    flag[1 + atomicAdd(&flag[0], 1)] = p;
    return;
  }
  const double ref = (double)ord2f(S.best[p]);
  a.q[p] = log((double)a.G) - (ref + log(s));
  if (a.ess) a.ess[p] = s * s / s2;
}

// The flagged points as a problem of their own: their coordinates and, as
// the reference, the largest exact value the first pass met.
__global__ void k_surf_tc_gather(const double *x, int npar, const unsigned *xmax, const int *flag, double *xs,
                                 unsigned *refs)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= flag[0]) return;
  const int p = flag[1 + k];
  for (int j = 0; j < npar; j++) xs[(size_t)k * npar + j] = x[(size_t)p * npar + j];
  refs[k] = xmax[p];
}

__global__ void k_surf_tc_setref(unsigned *best, unsigned *xmax, const unsigned *refs, int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) best[k] = xmax[k] = refs[k];
}

__global__ void k_surf_tc_scatter(const int *flag, const double *qs, const double *es, double *q, double *ess)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= flag[0]) return;
  const int p = flag[1 + k];
  q[p] = qs[k];
  if (ess) ess[p] = es[k];
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
  // prepared operands | chunk sums (double2 per point and chunk) | the list
  // of points to retake (a count, then points) | their coordinates,
  // references, densities, sample sizes and the retake's own list
  const size_t np = (size_t)npoints;
  return surf_prep_bytes(G, npoints) + np * SURF_MAX_CHUNKS * sizeof(double2) + 2 * (np + 1) * sizeof(int) +
         np * (SURF_K / 2) * sizeof(double) + np * sizeof(unsigned) + 2 * np * sizeof(double) + 4096;
}

namespace {

// tile stride of the max-only pre-pass: every tile, so the bound is the
// screened maximum itself and the full pass refines the fewest candidates
// (config 5: 1,311 per point with every 8th tile, 812 with every 2nd; 67.0,
// 48.7 and 44.4 ms per evaluation with every 8th, 2nd and every tile)
constexpr int PRE_STRIDE = 1;
constexpr int SEED_TC = 32;    // exact samples per point before the pre-pass (one per lane)

// genealogy chunks for a pass over `ntiles` tiles: one CTA holds an SM, so
// pick the chunk count whose CTA total fills its last wave best (at least
// 8 tiles per CTA); returns the chunk count, tiles per chunk in *per
int surf_tc_chunks(int ptiles, int ntiles, int nsm, int *per)
{
  const int maxch = std::max(1, std::min(SURF_MAX_CHUNKS, ntiles / 8));
  int nchunks = 1;
  *per = ntiles;
  double best_eff = -1.0;
  for (int c = 1; c <= maxch; c++) {
    const int pc = (ntiles + c - 1) / c, cc = (ntiles + pc - 1) / pc;
    const double waves = (double)ptiles * cc / nsm;
    const double eff = waves / std::ceil(waves);
    if (eff > best_eff + 0.02) {  // fewer chunks unless clearly better filled
      best_eff = eff;
      nchunks = cc;
      *per = pc;
    }
  }
  return nchunks;
}

}  // namespace

// One evaluation of the points of `a` on prepared operands S: the optional
// max-only pre-pass, the full pass and the merge; returns the kernels queued.
static int tc_passes(const SurfArgs &a, const SurfPrep &S, double2 *part, int *flag, int *d_err, int nsm, bool pre,
                     cudaStream_t st)
{
  const int ntiles = S.Gpad / TC_N;
  const int ptiles = (a.npoints + TC_M - 1) / TC_M;
  int per = 0, nk = 0;
  if (pre) {
    const int nch = surf_tc_chunks(ptiles, (ntiles + PRE_STRIDE - 1) / PRE_STRIDE, nsm, &per);
    k_surf_tc<<<dim3(ptiles, nch), TC_THREADS, TC_SMEM, st>>>(S, a.npoints, per, PRE_STRIDE, part, d_err);
    nk++;
  }
  const int nchunks = surf_tc_chunks(ptiles, ntiles, nsm, &per);
  k_surf_tc<<<dim3(ptiles, nchunks), TC_THREADS, TC_SMEM, st>>>(S, a.npoints, per, 0, part, d_err);
  cudaMemsetAsync(flag, 0, sizeof(int), st);
  k_surf_tc_merge<<<(a.npoints + 127) / 128, 128, 0, st>>>(a, S, part, nchunks, flag);
  return nk + 2;
}

int launch_surface_tc(const SurfArgs &a, void *scratch, size_t scratch_bytes, int *d_err, bool rows_ready,
                      int *nkernels, int *nretaken, cudaStream_t st)
{
  if (a.np + a.nm > SURF_K / 2) return 2;
  if (scratch_bytes < surface_tc_scratch_bytes(a.G, a.npoints)) return 3;
  if (a.G >= (1 << 24)) return 4;  // candidate entries pack the genealogy index into 24 bits
  const size_t np = (size_t)a.npoints;
  const int npar = a.np + a.nm;
  char *base = static_cast<char *>(scratch);
  SurfPrep S;
  double2 *part = reinterpret_cast<double2 *>(surf_prep_carve(&S, base, a.G, a.npoints));
  // the retake's buffers sit past everything the first evaluation uses
  int *flag = reinterpret_cast<int *>(part + np * SURF_MAX_CHUNKS);
  double *xs = reinterpret_cast<double *>(
      (reinterpret_cast<uintptr_t>(flag + np + 1) + 255) & ~static_cast<uintptr_t>(255));
  unsigned *refs = reinterpret_cast<unsigned *>(xs + np * (SURF_K / 2));
  double *qs = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(refs + np) + 255) & ~static_cast<uintptr_t>(255));
  double *es = qs + np;
  int *flag2 = reinterpret_cast<int *>(es + np);  // the retake's own list (always empty)
  static_assert(A_BYTES + TC_STAGES * B_BYTES + sizeof(TcSmem) + 1024 <= TC_SMEM, "smem");
  cudaFuncSetAttribute(k_surf_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  int nsm = 152;
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  }
  surf_prep(a, S, true, rows_ready, st);
  surf_seed(S, a.npoints, SEED_TC, st);
  // a max-only pre-pass over every PRE_STRIDE-th tile gives every point a
  // lower bound at (or near) its screened maximum before the full pass
  const bool pre = S.Gpad / TC_N >= 4 * PRE_STRIDE;
  int nk = (rows_ready ? 0 : 1) + 2 + tc_passes(a, S, part, flag, d_err, nsm, pre, st);
  // points whose terms left the fixed-point range: a second evaluation of
  // just them, referenced to their exact maxima
  int nflag = 0;
  if (cudaMemcpyAsync(&nflag, flag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return 5;
  *nretaken = nflag;
  if (nflag > 0) {
    k_surf_tc_gather<<<(nflag + 127) / 128, 128, 0, st>>>(a.x, npar, S.xmax, flag, xs, refs);
    SurfArgs b = a;
    b.npoints = nflag;
    b.x = xs;
    b.q = qs;
    b.ess = a.ess ? es : nullptr;
    SurfPrep S2;
    double2 *part2 = reinterpret_cast<double2 *>(surf_prep_carve(&S2, base, a.G, nflag));
    surf_prep(b, S2, true, true, st);
    k_surf_tc_setref<<<(nflag + 127) / 128, 128, 0, st>>>(S2.best, S2.xmax, refs, nflag);
    nk += 3 + tc_passes(b, S2, part2, flag2, d_err, nsm, false, st);
    k_surf_tc_scatter<<<(nflag + 127) / 128, 128, 0, st>>>(flag, qs, es, a.q, a.ess);
    nk++;
  }
  *nkernels = nk;
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
