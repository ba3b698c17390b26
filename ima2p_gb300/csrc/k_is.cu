// k_is.cu -- infinite-sites likelihood (likelihoodIS, calc_prob_data.cpp:731-836)
// and its per-locus constant sum log k! (calc_sumlogk, :609-719).
//
// One CTA per chain-locus, one thread per segregating site.  Each thread
// labels the genealogy for its site exactly as labelgtree does
// (calc_prob_data.cpp:537-581: walk down from every tip, merge the tip's 0/1
// state into the parent according to the sister's label, stop when a label
// does not change), finds the node whose daughters carry {0,1}, and takes the
// branch that carries the mutation.  Labels live in shared memory, laid out
// [node][thread] so the walks of a warp hit distinct banks.  log(t*u) is
// formed per site in FP64; the site terms are then added in site order by one
// thread, so the FP64 sum has the reference's association.  Each site's
// mutation branch is cached per chain-locus and reused while its topology is
// unchanged (the context clears the cache of every item whose topology it
// uploads), so re-timing updates skip the labelling.
#include "internal.h"

namespace {

constexpr int IS_BS = 64;
constexpr double REJECT_IS = -1000000000.0;  // imamp.hpp:157

// Site status, ordered as the reference reacts to them.
enum : int8_t { SITE_OK = 0, SITE_REJECT = 1, SITE_FAIL = 2 };

__device__ __forceinline__ void label_walk(int8_t *mut, const NodeRec *nd, int e)
{
  // mut is this thread's column: label of node k at mut[k * IS_BS]
  for (;;) {
    int p = nd[e].down;
    if (p < 0) return;
    int sis = (nd[p].up0 == e) ? nd[p].up1 : nd[p].up0;
    int8_t me = mut[e * IS_BS], mp = mut[p * IS_BS], ms = mut[sis * IS_BS];
    int8_t nv;
    if (mp != me) {
      if (me == 2) nv = (ms != -1) ? ms : (int8_t)2;
      else if (ms != -1 && ms != 2 && ms != me) nv = 2;
      else nv = me;
    } else if (mp == 2 && ms != -1 && ms != 2) {
      nv = ms;
    } else {
      return;
    }
    mut[p * IS_BS] = nv;
    e = p;
  }
}

__device__ __forceinline__ bool is_split(const int8_t *mut, int a, int b)
{
  int8_t x = mut[a * IS_BS], y = mut[b * IS_BS];
  return (x == 0 && y == 1) || (x == 1 && y == 0);
}

__device__ __forceinline__ double branch64(const NodeRec *nd, const double *t, int c)
{
  int u = nd[c].up0;
  return (u < 0) ? t[c] : t[c] - t[u];
}

// Labels one site; returns the mutation node, -1 if none, -2 if two.
__device__ int label_site(const NodeRec *nd, const int8_t *seq, int n, int S, int site,
                          int8_t *mut)
{
  int nl = 2 * n - 1;
  for (int j = 0; j < n; j++) mut[j * IS_BS] = seq[(size_t)j * S + site];
  for (int j = n; j < nl; j++) mut[j * IS_BS] = -1;
  for (int j = 0; j < n; j++) label_walk(mut, nd, j);
  int hit = -1;
  for (int node = n; node < nl; node++) {
    if (is_split(mut, nd[node].up0, nd[node].up1)) {
      if (hit != -1) return -2;
      hit = node;
    }
  }
  return hit;
}

struct IsSmem {
  NodeRec *nd;
  double *t;
  int8_t *mut;
  double *sv;
  int8_t *sst;
};

__device__ IsSmem carve(char *base, int nl, int S)
{
  IsSmem s;
  s.t = reinterpret_cast<double *>(base);
  s.sv = s.t + nl;
  s.nd = reinterpret_cast<NodeRec *>(s.sv + S);
  s.mut = reinterpret_cast<int8_t *>(s.nd + nl);
  s.sst = s.mut + (size_t)nl * IS_BS;
  return s;
}

__global__ void __launch_bounds__(IS_BS) k_is(Pools P, const ReqDev *reqs, double *result,
                                              int32_t *status, int32_t *site_node)
{
  extern __shared__ __align__(16) char smem[];
  const ReqDev R = reqs[blockIdx.x];
  const ItemDev it = P.items[R.item];
  const LocusDev L = P.loci[it.locus];
  const int n = L.n, nl = 2 * n - 1, S = L.nsites;
  IsSmem s = carve(smem, nl, S);
  for (int k = threadIdx.x; k < nl; k += IS_BS) {
    s.nd[k] = P.nodes[it.node_off + k];
    s.t[k] = P.t64[it.node_off + k];
  }
  __syncthreads();
  const int8_t *seq = P.seq + L.seq_off;
  int8_t *mut = s.mut + threadIdx.x;
  // the labelling depends on the topology and the data only: while the
  // item's topology is unchanged each site's mutation branch is read back
  const bool cached = P.is_valid[R.item] != 0;
  int32_t *cache = P.is_site + it.is_off;
  for (int site = threadIdx.x; site < S; site += IS_BS) {
    int hit, br = 0;
    if (cached) {
      const int32_t code = cache[site];
      hit = code >> 8;
      br = code & 0xff;
    } else {
      hit = label_site(s.nd, seq, n, S, site, mut);
      if (hit >= 0) {
        const int a = s.nd[hit].up0, dn = s.nd[hit].down;
        br = (dn < 0) ? 2 : (mut[dn * IS_BS] == mut[a * IS_BS]) ? 1 : 0;
      }
      cache[site] = (int32_t)(hit * 256 + br);
    }
    int8_t st = SITE_OK;
    double v = 0.0;
    if (hit == -2) {
      st = SITE_REJECT;
    } else if (hit == -1) {
      st = SITE_FAIL;
    } else {
      const int a = s.nd[hit].up0, b = s.nd[hit].up1;
      double t;
      if (br == 2) t = branch64(s.nd, s.t, a) + branch64(s.nd, s.t, b);
      else if (br == 1) t = branch64(s.nd, s.t, b);
      else t = branch64(s.nd, s.t, a);
      v = log(t * R.u);
    }
    s.sv[site] = v;
    s.sst[site] = st;
    if (site_node) site_node[(size_t)blockIdx.x * S + site] = (hit == -2) ? -2 : hit;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (!cached) P.is_valid[R.item] = 1;  // every site's entry is written (barrier above)
    double p = -P.length[R.item] * R.u;
    int code = IMA_EVAL_OK;
    for (int site = 0; site < S; site++) {
      if (s.sst[site] == SITE_REJECT) { code = IMA_EVAL_IS_REJECT; break; }
      if (s.sst[site] == SITE_FAIL) { code = IMA_EVAL_IS_FAIL; break; }
      p = p + s.sv[site];
    }
    if (code == IMA_EVAL_IS_REJECT) p = REJECT_IS;
    else if (code == IMA_EVAL_IS_FAIL) p = __longlong_as_double(0x7ff8000000000000ULL);
    else p -= P.sumlogk[it.locus];
    result[blockIdx.x] = p;
    P.pdg_new[R.item] = p;
    status[blockIdx.x] = code;
  }
}

// calc_sumlogk: per-internal-node mutation counts over all sites, then
// sum_i log(k_i!).  A site with two mutation nodes leaves the constant at 0
// (the reference returns before summing); a site with none is an error.
__global__ void __launch_bounds__(IS_BS) k_is_sumlogk(Pools P, int item, int locus, int *flag)
{
  extern __shared__ __align__(16) char smem[];
  const ItemDev it = P.items[item];
  const LocusDev L = P.loci[locus];
  const int n = L.n, nl = 2 * n - 1, S = L.nsites;
  IsSmem s = carve(smem, nl, S);
  int *cnt = reinterpret_cast<int *>(s.t);  // reuse the time area: n-1 <= nl ints
  for (int k = threadIdx.x; k < nl; k += IS_BS) s.nd[k] = P.nodes[it.node_off + k];
  for (int k = threadIdx.x; k < n; k += IS_BS) cnt[k] = 0;
  __syncthreads();
  const int8_t *seq = P.seq + L.seq_off;
  int8_t *mut = s.mut + threadIdx.x;
  for (int site = threadIdx.x; site < S; site += IS_BS) {
    int hit = label_site(s.nd, seq, n, S, site, mut);
    s.sst[site] = (hit == -2) ? SITE_REJECT : (hit == -1) ? SITE_FAIL : SITE_OK;
    if (hit >= 0) atomicAdd(&cnt[hit - n], 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    int code = 0;
    for (int site = 0; site < S; site++) {
      if (s.sst[site] != SITE_OK) { code = s.sst[site]; break; }
    }
    double sum = 0.0;
    if (code == 0) {
      for (int i = 0; i < n - 1; i++) {
        double f = 1.0;
        for (int j = 1; j <= cnt[i]; j++) f *= (double)j;
        sum += log(f);
      }
    }
    P.sumlogk[locus] = sum;
    *flag = code;
  }
}

size_t is_smem(int n, int S)
{
  int nl = 2 * n - 1;
  size_t b = sizeof(double) * (size_t)(nl + S) + sizeof(NodeRec) * nl + (size_t)nl * IS_BS + S;
  return (b + 15) & ~size_t(15);
}

}  // namespace

// Requests may mix IS loci; shared memory is sized for the largest of them.
void launch_is(const Pools &P, const ReqDev *reqs, int nreq, int maxn, int maxS, double *result,
               int32_t *status, int32_t *site_node, cudaStream_t st)
{
  if (nreq <= 0) return;
  size_t sm = is_smem(maxn, maxS);
  if (sm > 48 * 1024) cudaFuncSetAttribute(k_is, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_is<<<nreq, IS_BS, sm, st>>>(P, reqs, result, status, site_node);
}

void launch_is_sumlogk(const Pools &P, int item, int locus, int maxn, int maxS, int *d_flag,
                       cudaStream_t st)
{
  size_t sm = is_smem(maxn, maxS);
  if (sm > 48 * 1024)
    cudaFuncSetAttribute(k_is_sumlogk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  k_is_sumlogk<<<1, IS_BS, sm, st>>>(P, item, locus, d_flag);
}
