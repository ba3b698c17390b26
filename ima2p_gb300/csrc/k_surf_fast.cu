// k_surf_fast.cu -- placeholder until the tensor-core surface lands.
#include "internal.h"

size_t surface_fast_scratch_bytes(int G, int npoints)
{
  (void)G;
  (void)npoints;
  return 16;
}

int launch_surface_fast(const SurfArgs &a, void *scratch, size_t scratch_bytes, cudaStream_t st)
{
  (void)a;
  (void)scratch;
  (void)scratch_bytes;
  (void)st;
  return 1;
}
