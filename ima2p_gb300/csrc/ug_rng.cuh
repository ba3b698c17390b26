// ug_rng.cuh -- a chain's generators for the genealogy-update kernels
// (k_updgen.cu): the reference's uniform() (MT19937, utilities.cpp:323-427)
// and bitran (:438-455), staged for one kernel.
#pragma once

#include "internal.h"

namespace {

// The chain's generators for one kernel: MT19937 (Matsumoto & Nishimura
// 1998) with its 624 words in shared memory (the warp loads them and writes
// them back only when a twist changed them) and the rest in lane 0's
// registers, so that a draw costs a shared-memory read, not a dependent
// round trip to global memory.
struct LocalRng {
  uint32_t *mt;
  int mti, iset;
  double gset;
  unsigned long long iseed;
  bool twisted;
};

__device__ void rng_load(LocalRng &r, const ima_ug_rng *g, uint32_t *smt, int lane)
{
  const uint2 *src = reinterpret_cast<const uint2 *>(g->mt.mt);  // the state is 8-byte aligned
  uint2 *dst = reinterpret_cast<uint2 *>(smt);
  for (int k = lane; k < 312; k += 32) dst[k] = src[k];
  r.mt = smt;
  r.mti = g->mt.mti;
  r.iset = g->iset;
  r.gset = g->gset;
  r.iseed = g->iseed;
  r.twisted = false;
  __syncwarp();
}

// the warp writes the generator back (lane 0's registers, and the words
// when lane 0 twisted them)
__device__ void rng_store(const LocalRng &r, ima_ug_rng *g, int lane)
{
  const bool tw = __shfl_sync(~0u, (int)r.twisted, 0) != 0;
  if (tw) {
    const uint2 *src = reinterpret_cast<const uint2 *>(r.mt);
    uint2 *dst = reinterpret_cast<uint2 *>(g->mt.mt);
    for (int k = lane; k < 312; k += 32) dst[k] = src[k];
  }
  if (lane == 0) {
    g->mt.mti = r.mti;
    g->iset = r.iset;
    g->gset = r.gset;
    g->iseed = r.iseed;
  }
}

__device__ uint32_t mt_next(LocalRng &r)
{
  constexpr int N = 624, M = 397;
  if (r.mti >= N) {
    uint32_t *mt = r.mt;
    for (int k = 0; k < N; k++) {
      const uint32_t y = (mt[k] & 0x80000000u) | (mt[(k + 1) % N] & 0x7fffffffu);
      mt[k] = mt[(k + M) % N] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
    }
    r.mti = 0;
    r.twisted = true;
  }
  uint32_t y = r.mt[r.mti++];
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return y;
}

// uniform() = genrand_real3, in (0, 1)
__device__ double uniform(LocalRng &r) { return ((double)mt_next(r) + 0.5) * (1.0 / 4294967296.0); }

// bitran (utilities.cpp:438-455): Press et al.'s irbit2 on its own register
__device__ int bitran(LocalRng &r)
{
  if (r.iseed & 131072ull) {
    r.iseed = ((r.iseed ^ 19ull) << 1) | 1ull;
    return 1;
  }
  r.iseed <<= 1;
  return 0;
}

}  // namespace
