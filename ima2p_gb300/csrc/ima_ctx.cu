// ima_ctx.cu -- the C ABI (include/ima_gpu.h): context, resident pools,
// genealogy staging, request batching, commit/revert, swaps, surface, timing.
//
// Host-side genealogy edits land in a pinned mirror of the device pools and
// are shipped, one contiguous copy per pool over the range of touched
// chain-loci, before the next launch.  Requests of a batch are grouped by
// mutation model (one kernel per model) and their results are returned in
// the caller's order.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>
#include <memory>
#include <functional>
#include <condition_variable>
#include <mutex>
#include <atomic>
#include <exception>
#include <chrono>
#include <thread>

#include "internal.h"

int sw_init_tables();

namespace {

struct LocusHost {
  LocusDev d;
  std::vector<int8_t> seq;
  std::vector<int32_t> mult;
  bool sumlogk_done = false;
};

struct Batch {
  bool live = false;
  int n = 0, nis = 0, nhky = 0, nsw = 0, prec = IMA_PREC_FAST;
  std::vector<int> order;  // grouped position -> caller index
  ReqDev *d_req = nullptr;
  double *d_res = nullptr;   // results, then the status words (one allocation, one copy back)
  int32_t *d_st = nullptr;
  double *h_res = nullptr;   // pinned, the same layout
  int32_t *h_st = nullptr;
  ReqDev *h_reqpin = nullptr;  // pinned staging of h_req for its upload
  cudaEvent_t req_ev = nullptr;  // the last upload from h_reqpin
  double hky_bytes = 0.0, sw_bytes = 0.0;  // algorithmic bytes of one run (launch statistics)
  std::vector<int> dl_idx;  // SW requests' entries of ima_ctx::dl_fast
  bool in_order = false;    // order is the identity: results copy straight back
  long long dl_stamp = -1;  // ima_ctx::dl_stamp when this batch last set those entries
  std::vector<ReqDev> h_req;
  cudaGraphExec_t graph = nullptr;
  int maxn_is = 0, maxs_is = 0, maxn_hky = 0, maxs_hky = 0, maxn_sw = 0;
  int cap = 0;  // capacity of the device buffers
  int hky_variant = 0, sw_variant = 0;  // launch shapes (ima_gpu_batch_autotune)
  // MC3 sweep of the batch (ima_gpu_batch_sweep): its items and accept mask
  // on the device, and the graph of evaluation, commit and swaps
  int32_t *d_items = nullptr;
  uint8_t *d_acc = nullptr;
  cudaGraphExec_t sgraph = nullptr;
  int s_tries = -1, s_probg = -1;
  uint64_t s_seed = 0;
};

// A small persistent pool of host threads for per-genealogy packing: run(n,
// f) calls f(0) .. f(n-1) on the pool and the calling thread and returns
// when every call has finished.  Jobs are claimed under the mutex; between
// calls the workers spin (yielding) for a short while before they block, and
// the caller spins on the completion count, so that a call does not pay a
// condition-variable wake-up on each side (tens of microseconds per call).
class HostPool {
 public:
  explicit HostPool(int nthreads)
  {
    for (int i = 0; i < nthreads; i++) th_.emplace_back([this] { loop(); });
  }
  ~HostPool()
  {
    {
      std::lock_guard<std::mutex> lk(m_);
      stop_.store(true);
      gen_.fetch_add(1);
    }
    cv_.notify_all();
    for (auto &t : th_) t.join();
  }
  int size() const { return (int)th_.size() + 1; }
  void run(int n, const std::function<void(int)> &f)
  {
    {
      std::lock_guard<std::mutex> lk(m_);
      job_ = &f;
      njobs_ = n;
      next_ = 0;
      finished_.store(0);
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    {
      std::unique_lock<std::mutex> lk(m_);
      work(lk);
    }
    while (finished_.load(std::memory_order_acquire) < n) std::this_thread::yield();
    std::lock_guard<std::mutex> lk(m_);
    job_ = nullptr;
  }

 private:
  static constexpr auto kSpin = std::chrono::microseconds(200);
  void work(std::unique_lock<std::mutex> &lk)
  {
    while (job_ && next_ < njobs_) {
      const int j = next_++;
      const std::function<void(int)> *f = job_;
      lk.unlock();
      (*f)(j);
      lk.lock();
      finished_.fetch_add(1, std::memory_order_release);
    }
  }
  void loop()
  {
    uint64_t seen = 0;
    for (;;) {
      const auto t0 = std::chrono::steady_clock::now();
      while (gen_.load(std::memory_order_acquire) == seen && std::chrono::steady_clock::now() - t0 < kSpin)
        std::this_thread::yield();
      std::unique_lock<std::mutex> lk(m_);
      cv_.wait(lk, [&] { return stop_.load() || gen_.load() != seen; });
      if (stop_.load()) return;
      seen = gen_.load();
      work(lk);
    }
  }
  std::vector<std::thread> th_;
  std::mutex m_;
  std::condition_variable cv_;
  const std::function<void(int)> *job_ = nullptr;
  int njobs_ = 0, next_ = 0;
  std::atomic<int> finished_{0};
  std::atomic<uint64_t> gen_{0};
  std::atomic<bool> stop_{false};
};

struct PendingTiming {
  int kind;
  cudaEvent_t a, b;
  double bytes;
};

// Zeroed device allocation.  The zeroing is queued on the context stream so
// that it is ordered before every later copy or kernel on that stream (a
// plain cudaMemset would run on the legacy stream, which a non-blocking
// stream does not wait for).
template <typename T>
T *dev_alloc(size_t count, size_t &total, cudaStream_t st)
{
  if (count == 0) count = 1;
  void *p = nullptr;
  if (cudaMalloc(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
  if (cudaMemsetAsync(p, 0, count * sizeof(T), st) != cudaSuccess) {
    cudaFree(p);
    return nullptr;
  }
  total += count * sizeof(T);
  return static_cast<T *>(p);
}

template <typename T>
T *host_alloc(size_t count)
{
  if (count == 0) count = 1;
  void *p = nullptr;
  if (cudaMallocHost(&p, count * sizeof(T)) != cudaSuccess) return nullptr;
  memset(p, 0, count * sizeof(T));
  return static_cast<T *>(p);
}

}  // namespace

struct ima_ctx {
  int device = 0;
  int nsm = 152;  // SMs of the device
  int pageable_access = 0;  // the device reads pageable host memory (cudaDevAttrPageableMemoryAccess)
  cudaStream_t st = nullptr;
  std::string err;
  size_t dev_bytes = 0;
  long long launches = 0;

  // loci
  std::vector<LocusHost> loci;
  LocusDev *d_loci = nullptr;
  int8_t *d_seq = nullptr;
  int32_t *d_mult = nullptr;
  double *d_sumlogk = nullptr;
  int *d_flag = nullptr;

  // chains x loci
  int nruns = 0, cpr = 0, nchains = 0, nloci = 0, nitems = 0;
  std::vector<ItemDev> items;
  ItemDev *d_items = nullptr;
  size_t nnodes = 0, nsched = 0, nal = 0, npart = 0, npart64 = 0;
  // host mirrors (pinned)
  NodeRec *h_nodes = nullptr;
  double *h_t64 = nullptr;
  int16_t *h_sched = nullptr;
  int32_t *h_nlev = nullptr;
  double *h_len = nullptr;
  double *h_pi = nullptr;
  int32_t *h_al = nullptr;
  int dirty_lo = INT32_MAX, dirty_hi = -1;    // topology, schedule, pi, alleles
  int tdirty_lo = INT32_MAX, tdirty_hi = -1;  // times and lengths only
  // device pools
  NodeRec *d_nodes = nullptr;
  double *d_t64 = nullptr;
  float2 *d_tff = nullptr;
  int16_t *d_sched = nullptr;
  int32_t *d_nlev = nullptr;
  double *d_len = nullptr;
  double *d_pi = nullptr;
  int32_t *d_al = nullptr;
  double *d_dlike = nullptr;
  std::vector<uint8_t> dl_fast;  // per item x marker: last SW evaluation was float-float
  long long dl_stamp = 0;        // counts the batches that set dl_fast entries
  // launch shapes the autotuner chose, by batch shape (counts per kind,
  // largest loci, precision): a later batch of the same shape, ima_gpu_eval's
  // own included, starts on them
  struct Tuned {
    int key[7];
    int hky, sw;
  };
  std::vector<Tuned> tuned;
  // the last list of pairs upload_times checked, and what it found: a list
  // given again is not walked again (pairs only gain genealogies, except
  // when a checkpoint is read, which bumps tree_gen)
  std::vector<int32_t> tk_ci, tk_li;
  int tk_lo = 0, tk_hi = -1, tk_gen = -1;
  bool tk_run = false;
  int tree_gen = 0;
  std::vector<uint8_t> has_tree; // per item: a genealogy was uploaded
  std::unique_ptr<HostPool> pool;  // host threads for set_genealogies (made on first use)
  std::vector<int> pair_stamp;     // set_genealogies: repeated-pair check
  std::vector<size_t> pair_off;    // set_genealogies: node offset of each pair
  int stamp_gen = 0;
  float4 *d_part = nullptr, *d_partlo = nullptr;
  int32_t *d_pexp = nullptr;
  double *d_part64 = nullptr, *d_psf64 = nullptr;
  uint8_t *d_slot32 = nullptr, *d_fresh32 = nullptr, *d_slot64 = nullptr, *d_fresh64 = nullptr;
  double *d_pdg = nullptr, *d_pdg_new = nullptr;

  // MC3
  double *d_beta = nullptr, *d_allbetas = nullptr, *d_probg = nullptr, *d_S = nullptr;
  int32_t *d_swapcount = nullptr, *d_tempcount = nullptr, *d_used = nullptr, *d_swap0ok = nullptr;
  unsigned long long *d_ctr = nullptr;
  int32_t *d_is_site = nullptr;  // IS per-site mutation branches, valid while the topology is
  uint8_t *d_is_valid = nullptr;
  double *d_uni = nullptr;
  size_t uni_cap = 0;

  // surface
  int sG = 0, srowlen = 0, snp = 0, snm = 0, snpops = 0;
  float *d_rows = nullptr;
  double *d_lognorm = nullptr;
  void *d_sscratch = nullptr;
  size_t sscratch_cap = 0;
  void *d_mscratch = nullptr;  // marginal densities: points, partial sums
  size_t mscratch_cap = 0;
  // row-derived surface operands held in the scratch: 0 none, 1 FP32 (split
  // precision screen), 2 FP32 + bf16 planes (tensor-core screen); for the
  // model type srows_model
  int srows_state = 0, srows_model = -1;
  double *d_sx = nullptr, *d_sq = nullptr, *d_sess = nullptr;
  size_t spts_cap = 0;

  // genealogy weights: the population model, the inputs and weights of the
  // last ima_gpu_treeweight (kept for ima_gpu_tree_prob), logfact
  TwModel h_tw{};
  TwModel *d_tw = nullptr;
  bool tw_ready = false;
  double *d_logfact = nullptr;
  int32_t *d_twerr = nullptr;
  void *d_twin = nullptr, *d_twout = nullptr, *d_tpbuf = nullptr;
  size_t twin_cap = 0, twout_cap = 0, tpbuf_cap = 0;
  int tw_ngen = 0, tw_ntv = 0;
  int surf_retaken = 0;  // points the last tensor-core surface took a second time
  long long graph_launches = 0;  // graph replays of MC3 sweeps
  // which of the tw_ngen genealogies hold weights from the last treeweight
  // (all) or chain_weights call (the selected chains' items only)
  std::vector<uint8_t> tw_valid;
  // resident population labels for the split-time update: per node pop,
  // per item nl+1 relative migration offsets (at node_off + item), events in
  // a pool (item events from mbase[item]), split-time rows per chain
  int32_t *d_pop = nullptr, *d_moff = nullptr, *d_inode_off = nullptr, *d_gl = nullptr, *d_gt = nullptr;
  int32_t *d_moff_start = nullptr, *d_bcnt = nullptr, *d_bicnt = nullptr, *d_mig_p = nullptr, *d_rsamp = nullptr;
  long long *d_mbase = nullptr;
  double *d_mig_t = nullptr, *d_tvr = nullptr, *d_len_hold = nullptr, *d_rhlog = nullptr, *d_rh2 = nullptr;
  size_t mig_cap = 0, mig_used = 0;
  std::vector<long long> h_mbase;
  std::vector<int32_t> h_mcnt, h_mcap;
  std::vector<uint8_t> has_labels;
  std::vector<double> h_tvr, h_hval;
  std::vector<int32_t> h_samp;
  bool locus_pops = false;
  void *d_rsel = nullptr;
  size_t rsel_cap = 0;
  int dev_lo = INT32_MAX, dev_hi = -1;  // items whose device times/lengths are newer than the mirror
  int topo_lo = INT32_MAX, topo_hi = -1;  // items whose device topology and schedule are newer too
  // the genealogy update's buffers and per-locus evaluation requests
  void *d_ug = nullptr;
  size_t ug_cap = 0;
  std::vector<Batch> ugb;
  // the genealogy update's streams: weights, likelihoods and decisions run
  // behind the proposals (on st), ordered by per-step events
  cudaStream_t ug_sw = nullptr, ug_sw2 = nullptr, ug_sw3 = nullptr, ug_sh = nullptr, ug_sh2 = nullptr, ug_sd = nullptr;
  std::vector<cudaEvent_t> ug_ev;  // [4][ring slots]: proposal, weights, likelihood, decision done
  // items whose tree lengths are still to be summed from their device times
  // (re-timings without lengths): done when a reader needs them
  int lpend_lo = INT32_MAX, lpend_hi = -1;

  double *d_lterm = nullptr;  // per node: its branch term, for those sums
  float *tp_rows = nullptr;  // gsampinf rows of the last ima_gpu_tree_prob
  int tp_ngroups = 0, tp_rowlen = 0;
  size_t s_cap = 0;          // surface row capacity (rows appended on the device)
  int32_t *tw_cc = nullptr, *tw_mc = nullptr;
  double *tw_hcc = nullptr, *tw_fc = nullptr, *tw_fm = nullptr, *tw_tvals = nullptr;

  // batches
  std::vector<Batch> batches;
  Batch evb;  // buffers of ima_gpu_eval
  // the request list evb holds: a call with byte-identical arrays reuses it
  struct EvalKey {
    bool valid = false;
    int n = 0, prec = 0;
    std::vector<int32_t> ci, li, edits, ai;
    std::vector<double> u, kappa;
  } evkey;
  int32_t *d_citems = nullptr;
  uint8_t *d_cacc = nullptr;
  size_t ccap = 0;

  // timing
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  bool profiling = false;
  std::vector<PendingTiming> pending;
  long long k_launches[IMA_K_COUNT] = {0};
  double k_ms[IMA_K_COUNT] = {0}, k_bytes[IMA_K_COUNT] = {0};
  std::vector<cudaEvent_t> event_pool;
  void *d_flush = nullptr;
  size_t flush_bytes = 0;

  int fail(int code, const char *fmt, ...)
  {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    err = buf;
    return code;
  }
  int cuda(cudaError_t e, const char *what)
  {
    if (e == cudaSuccess) return IMA_OK;
    return fail(IMA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
  Pools pools() const
  {
    Pools P;
    P.loci = d_loci;
    P.items = d_items;
    P.seq = d_seq;
    P.mult = d_mult;
    P.nodes = d_nodes;
    P.t64 = d_t64;
    P.tff = d_tff;
    P.sched = d_sched;
    P.nlev = d_nlev;
    P.length = d_len;
    P.pi = d_pi;
    P.alleles = d_al;
    P.dlike = d_dlike;
    P.sumlogk = d_sumlogk;
    P.is_site = d_is_site;
    P.is_valid = d_is_valid;
    P.pdg_new = d_pdg_new;
    P.part = d_part;
    P.partlo = d_partlo;
    P.pexp = d_pexp;
    P.part64 = d_part64;
    P.psf64 = d_psf64;
    P.slot32 = d_slot32;
    P.fresh32 = d_fresh32;
    P.slot64 = d_slot64;
    P.fresh64 = d_fresh64;
    return P;
  }
  cudaEvent_t ev()
  {
    if (!event_pool.empty()) {
      cudaEvent_t e = event_pool.back();
      event_pool.pop_back();
      return e;
    }
    cudaEvent_t e;
    cudaEventCreate(&e);
    return e;
  }
  // bracket one kernel launch for accounting
  // launches by f() on stream on (the context stream by default), counted
  // and, when profiling, timed by events on that stream
  template <typename F>
  void launch(int kind, double bytes, F &&f, cudaStream_t on = nullptr)
  {
    if (!on) on = st;
    cudaEvent_t a = nullptr, b = nullptr;
    if (profiling) {
      a = ev();
      b = ev();
      cudaEventRecord(a, on);
    }
    f();
    launches++;
    k_launches[kind]++;
    k_bytes[kind] += bytes;
    if (profiling) {
      cudaEventRecord(b, on);
      pending.push_back({kind, a, b, bytes});
    }
  }
  void resolve_timings()
  {
    if (pending.empty()) return;
    cudaStreamSynchronize(st);
    for (auto &p : pending) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, p.a, p.b);
      k_ms[p.kind] += ms;
      event_pool.push_back(p.a);
      event_pool.push_back(p.b);
    }
    pending.clear();
  }
  int item_of(int ci, int li) const { return ci * nloci + li; }
  bool valid(int ci, int li) const { return ci >= 0 && ci < nchains && li >= 0 && li < nloci; }
};

// ======================================================================
// context
extern "C" int ima_gpu_create(int device, ima_ctx **out)
{
  if (!out) return IMA_ERR_ARG;
  *out = nullptr;
  ima_ctx *c = new (std::nothrow) ima_ctx;
  if (!c) return IMA_ERR_NOMEM;
  c->device = device;
  cudaError_t e = cudaSetDevice(device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete c;
    return IMA_ERR_CUDA;
  }
  cudaEventCreate(&c->t0);
  cudaEventCreate(&c->t1);
  cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device);
  cudaDeviceGetAttribute(&c->pageable_access, cudaDevAttrPageableMemoryAccess, device);
  if (sw_init_tables() != 0 || hky_init_tables() != 0) {
    delete c;
    return IMA_ERR_CUDA;
  }
  c->d_flag = dev_alloc<int>(64, c->dev_bytes, c->st);
  *out = c;
  return IMA_OK;
}

extern "C" void ima_gpu_destroy(ima_ctx *c)
{
  if (!c) return;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->st);
  c->batches.push_back(c->evb);
  for (auto &b : c->ugb) c->batches.push_back(b);
  for (auto &b : c->batches) {
    if (b.graph) cudaGraphExecDestroy(b.graph);
    if (b.sgraph) cudaGraphExecDestroy(b.sgraph);
    cudaFree(b.d_req);
    cudaFree(b.d_res);
    cudaFree(b.d_items);
    cudaFree(b.d_acc);
    cudaFreeHost(b.h_res);
    cudaFreeHost(b.h_reqpin);
    if (b.req_ev) cudaEventDestroy(b.req_ev);
  }
  void *devs[] = {c->d_loci, c->d_seq, c->d_mult, c->d_sumlogk, c->d_flag, c->d_items,
                  c->d_nodes, c->d_t64, c->d_tff, c->d_sched, c->d_nlev, c->d_len, c->d_pi,
                  c->d_al, c->d_dlike, c->d_part, c->d_partlo, c->d_pexp, c->d_part64, c->d_psf64,
                  c->d_slot32, c->d_fresh32, c->d_slot64, c->d_fresh64, c->d_pdg, c->d_pdg_new,
                  c->d_beta, c->d_allbetas, c->d_probg, c->d_S, c->d_swapcount, c->d_tempcount,
                  c->d_used, c->d_swap0ok, c->d_ctr, c->d_uni, c->d_rows, c->d_lognorm,
                  c->d_sscratch, c->d_sx, c->d_sq, c->d_sess, c->d_citems, c->d_cacc, c->d_flush,
                  c->d_mscratch, c->d_tw, c->d_logfact, c->d_twerr, c->d_twin, c->d_twout, c->d_tpbuf,
                  c->d_pop, c->d_moff, c->d_inode_off, c->d_gl, c->d_gt, c->d_moff_start, c->d_bcnt, c->d_bicnt,
                  c->d_mig_p, c->d_rsamp, c->d_mbase, c->d_mig_t, c->d_tvr, c->d_len_hold, c->d_rhlog,
                  c->d_rh2, c->d_rsel, c->d_is_site, c->d_is_valid, c->d_lterm, c->d_ug};
  for (void *p : devs)
    if (p) cudaFree(p);
  void *hosts[] = {c->h_nodes, c->h_t64, c->h_sched, c->h_nlev, c->h_len, c->h_pi, c->h_al};
  for (void *p : hosts)
    if (p) cudaFreeHost(p);
  for (auto &p : c->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto e : c->event_pool) cudaEventDestroy(e);
  if (c->t0) cudaEventDestroy(c->t0);
  if (c->t1) cudaEventDestroy(c->t1);

  for (auto e : c->ug_ev) cudaEventDestroy(e);
  for (cudaStream_t q : {c->ug_sw, c->ug_sw2, c->ug_sw3, c->ug_sh, c->ug_sh2, c->ug_sd})
    if (q) cudaStreamDestroy(q);
  if (c->st) cudaStreamDestroy(c->st);
  delete c;
}

extern "C" const char *ima_gpu_error(const ima_ctx *c) { return c ? c->err.c_str() : "null context"; }

extern "C" int ima_gpu_synchronize(ima_ctx *c)
{
  if (!c) return IMA_ERR_ARG;
  return c->cuda(cudaStreamSynchronize(c->st), "synchronize");
}

// ======================================================================
// loci
static int add_locus(ima_ctx *c, int model, int n, int S, int tots, const int8_t *seq,
                     const int32_t *mult, int nlinked, int *li)
{
  c->evkey.valid = false;
  if (!c || !li) return IMA_ERR_ARG;
  if (c->nchains) return c->fail(IMA_ERR_STATE, "loci must be added before ima_gpu_set_chains");
  if (n < 2 || n > 16000) return c->fail(IMA_ERR_ARG, "numgenes %d out of range", n);
  if (S < 0 || (S > 0 && !seq && model != IMA_MODEL_SW)) return c->fail(IMA_ERR_ARG, "bad sites");
  LocusHost L;
  L.d.model = model;
  L.d.n = n;
  L.d.nsites = S;
  L.d.totsites = tots;
  L.d.nlinked = nlinked;
  if (seq && S > 0) {
    L.seq.assign(seq, seq + (size_t)n * S);
    for (int8_t v : L.seq) {
      if (model == IMA_MODEL_IS && (v < 0 || v > 1)) return c->fail(IMA_ERR_ARG, "IS states must be 0/1");
      if (model == IMA_MODEL_HKY && (v < 0 || v > 3)) return c->fail(IMA_ERR_ARG, "HKY states must be 0..3");
    }
  }
  if (mult) L.mult.assign(mult, mult + S);
  *li = (int)c->loci.size();
  c->loci.push_back(std::move(L));
  return IMA_OK;
}

extern "C" int ima_gpu_add_locus_is(ima_ctx *c, int numgenes, int numsites, const int8_t *seq, int *li)
{
  return add_locus(c, IMA_MODEL_IS, numgenes, numsites, numsites, seq, nullptr, 1, li);
}

extern "C" int ima_gpu_add_locus_hky(ima_ctx *c, int numgenes, int numsites, int totsites,
                                     const int8_t *seq, const int32_t *mult, int *li)
{
  if (!c || !mult || numsites < 1 || totsites < 1) return c ? c->fail(IMA_ERR_ARG, "bad HKY locus") : IMA_ERR_ARG;
  return add_locus(c, IMA_MODEL_HKY, numgenes, numsites, totsites, seq, mult, 1, li);
}

extern "C" int ima_gpu_add_locus_sw(ima_ctx *c, int numgenes, int nlinked, int *li)
{
  if (nlinked < 1) return c ? c->fail(IMA_ERR_ARG, "nlinked must be >= 1") : IMA_ERR_ARG;
  if (numgenes > 256) return c ? c->fail(IMA_ERR_ARG, "stepwise loci hold at most 256 gene copies") : IMA_ERR_ARG;
  return add_locus(c, IMA_MODEL_SW, numgenes, 0, 0, nullptr, nullptr, nlinked, li);
}

extern "C" int ima_gpu_set_chains(ima_ctx *c, int nruns, int chains_per_run)
{
  if (c) c->evkey.valid = false;
  if (!c) return IMA_ERR_ARG;
  if (c->nchains) return c->fail(IMA_ERR_STATE, "chains already set");
  if (nruns < 1 || chains_per_run < 1 || c->loci.empty())
    return c->fail(IMA_ERR_ARG, "need >= 1 run, >= 1 chain and >= 1 locus");
  cudaSetDevice(c->device);
  c->nruns = nruns;
  c->cpr = chains_per_run;
  c->nchains = nruns * chains_per_run;
  c->nloci = (int)c->loci.size();
  c->nitems = c->nchains * c->nloci;
  // locus tables
  std::vector<int8_t> seq;
  std::vector<int32_t> mult;
  std::vector<LocusDev> ld;
  for (auto &L : c->loci) {
    L.d.seq_off = (int)seq.size();
    L.d.mult_off = (int)mult.size();
    seq.insert(seq.end(), L.seq.begin(), L.seq.end());
    mult.insert(mult.end(), L.mult.begin(), L.mult.end());
    ld.push_back(L.d);
  }
  // placement of every chain-locus
  c->items.resize(c->nitems);
  size_t nodes = 0, sched = 0, al = 0, part = 0, part64 = 0, iss = 0;
  for (int ci = 0; ci < c->nchains; ci++)
    for (int li = 0; li < c->nloci; li++) {
      const LocusDev &L = ld[li];
      ItemDev &it = c->items[c->item_of(ci, li)];
      int nl = 2 * L.n - 1;
      it.locus = li;
      it.n = L.n;
      it.node_off = (int)nodes;
      it.sched_off = (int)sched;
      it.al_off = (int)al;
      it.dl_off = (int)al;
      it.part_off = (long long)part;
      it.part64_off = (long long)part64;
      it.is_off = (long long)iss;
      if (L.model == IMA_MODEL_IS) iss += (size_t)L.nsites;
      nodes += nl;
      sched += 2 * L.n + 2;
      if (L.model == IMA_MODEL_SW) al += (size_t)L.nlinked * nl;
      if (L.model == IMA_MODEL_HKY) {
        part += 2 * (size_t)(L.n - 1) * L.nsites;
        part64 += 2 * (size_t)(L.n - 1) * L.nsites;
      }
    }
  if (nodes > (size_t)INT32_MAX || sched > (size_t)INT32_MAX || al > (size_t)INT32_MAX)
    return c->fail(IMA_ERR_ARG, "too many nodes for 32-bit offsets");
  c->nnodes = nodes;
  c->nsched = sched;
  c->nal = al;
  c->npart = part;
  c->npart64 = part64;
  size_t &B = c->dev_bytes;
  c->d_loci = dev_alloc<LocusDev>(ld.size(), B, c->st);
  c->d_seq = dev_alloc<int8_t>(seq.size(), B, c->st);
  c->d_mult = dev_alloc<int32_t>(mult.size(), B, c->st);
  c->d_sumlogk = dev_alloc<double>(c->nloci, B, c->st);
  c->d_items = dev_alloc<ItemDev>(c->nitems, B, c->st);
  c->d_nodes = dev_alloc<NodeRec>(nodes, B, c->st);
  c->d_t64 = dev_alloc<double>(nodes, B, c->st);
  c->d_tff = dev_alloc<float2>(nodes, B, c->st);
  c->d_slot32 = dev_alloc<uint8_t>(nodes, B, c->st);
  c->d_fresh32 = dev_alloc<uint8_t>(nodes, B, c->st);
  c->d_sched = dev_alloc<int16_t>(sched, B, c->st);
  c->d_nlev = dev_alloc<int32_t>(c->nitems, B, c->st);
  c->d_len = dev_alloc<double>(c->nitems, B, c->st);
  c->d_pi = dev_alloc<double>(4 * (size_t)c->nitems, B, c->st);
  c->d_al = dev_alloc<int32_t>(al, B, c->st);
  c->d_dlike = dev_alloc<double>(al, B, c->st);
  c->d_part = dev_alloc<float4>(part, B, c->st);
  c->d_pexp = dev_alloc<int32_t>(part, B, c->st);
  c->d_pdg = dev_alloc<double>(c->nitems, B, c->st);
  c->d_pdg_new = dev_alloc<double>(c->nitems, B, c->st);
  c->d_beta = dev_alloc<double>(c->nchains, B, c->st);
  c->d_allbetas = dev_alloc<double>(c->nchains, B, c->st);
  c->d_probg = dev_alloc<double>(c->nchains, B, c->st);
  c->d_S = dev_alloc<double>(c->nchains, B, c->st);
  c->d_swapcount = dev_alloc<int32_t>((size_t)c->nruns * c->cpr * c->cpr, B, c->st);
  c->d_tempcount = dev_alloc<int32_t>((size_t)c->nruns * c->cpr * c->cpr, B, c->st);
  c->d_used = dev_alloc<int32_t>(c->nruns, B, c->st);
  c->d_swap0ok = dev_alloc<int32_t>(c->nruns, B, c->st);
  c->d_ctr = dev_alloc<unsigned long long>(c->nruns, B, c->st);
  c->d_is_site = dev_alloc<int32_t>(iss > 0 ? iss : 1, B, c->st);
  c->d_is_valid = dev_alloc<uint8_t>(c->nitems, B, c->st);
  void *chk[] = {c->d_loci, c->d_seq, c->d_mult, c->d_sumlogk, c->d_items, c->d_nodes, c->d_t64,
                 c->d_tff, c->d_slot32, c->d_fresh32, c->d_sched, c->d_nlev, c->d_len, c->d_pi,
                 c->d_al, c->d_dlike, c->d_part, c->d_pexp, c->d_pdg, c->d_pdg_new, c->d_beta,
                 c->d_allbetas, c->d_probg, c->d_S, c->d_swapcount, c->d_tempcount, c->d_used,
                 c->d_swap0ok, c->d_ctr, c->d_is_site, c->d_is_valid};
  for (void *p : chk)
    if (!p) return c->fail(IMA_ERR_NOMEM, "device allocation failed (%zu bytes so far)", B);
  if (int r0 = c->cuda(cudaMemsetAsync(c->d_is_valid, 0, c->nitems, c->st), "IS site cache")) return r0;
  c->h_nodes = host_alloc<NodeRec>(nodes);
  c->h_t64 = host_alloc<double>(nodes);
  c->h_sched = host_alloc<int16_t>(sched);
  c->h_nlev = host_alloc<int32_t>(c->nitems);
  c->h_len = host_alloc<double>(c->nitems);
  c->h_pi = host_alloc<double>(4 * (size_t)c->nitems);
  c->h_al = host_alloc<int32_t>(al);
  if (!c->h_nodes || !c->h_t64 || !c->h_sched || !c->h_nlev || !c->h_len || !c->h_pi || !c->h_al)
    return c->fail(IMA_ERR_NOMEM, "pinned host allocation failed");
  for (int i = 0; i < c->nitems; i++)
    for (int j = 0; j < 4; j++) c->h_pi[4 * (size_t)i + j] = 0.25;
  c->dl_fast.assign(al ? al : 1, 0);
  c->has_tree.assign(c->nitems, 0);
  int r = IMA_OK;
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_loci, ld.data(), ld.size() * sizeof(LocusDev), cudaMemcpyHostToDevice, c->st), "loci");
  if (!seq.empty()) r = r ? r : c->cuda(cudaMemcpyAsync(c->d_seq, seq.data(), seq.size(), cudaMemcpyHostToDevice, c->st), "seq");
  if (!mult.empty()) r = r ? r : c->cuda(cudaMemcpyAsync(c->d_mult, mult.data(), mult.size() * 4, cudaMemcpyHostToDevice, c->st), "mult");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_items, c->items.data(), c->items.size() * sizeof(ItemDev), cudaMemcpyHostToDevice, c->st), "items");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_pi, c->h_pi, 4 * sizeof(double) * c->nitems, cudaMemcpyHostToDevice, c->st), "pi");
  // the host vectors above are about to go out of scope
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "set_chains");
}

// ======================================================================
// genealogies

// Device-side updates (the split-time rubber band, resident weights) leave
// times and lengths newer on the device than in the pinned mirror; every
// host write into the mirror first copies them back, so that a later range
// upload never carries stale values.
// Before the host writes its mirror: values newer on the device (moved or
// uploaded there) come back into it.
static int ensure_lengths(ima_ctx *c);

static int sync_mirror(ima_ctx *c)
{
  int r = ensure_lengths(c);
  if (c->topo_hi >= 0) {
    c->dev_lo = std::min(c->dev_lo, c->topo_lo);
    c->dev_hi = std::max(c->dev_hi, c->topo_hi);
  }
  if (r || c->dev_hi < 0) return r;
  const ItemDev &a = c->items[c->dev_lo], &b = c->items[c->dev_hi];
  const size_t n0 = a.node_off, n1 = (size_t)b.node_off + 2 * b.n - 1;
  r = c->cuda(cudaMemcpyAsync(c->h_t64 + n0, c->d_t64 + n0, (n1 - n0) * sizeof(double), cudaMemcpyDeviceToHost, c->st), "mirror");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->h_len + c->dev_lo, c->d_len + c->dev_lo, (size_t)(c->dev_hi - c->dev_lo + 1) * sizeof(double),
                                      cudaMemcpyDeviceToHost, c->st), "mirror");
  if (c->topo_hi >= 0) {  // genealogies the device changed: topology and level schedules too
    const ItemDev &ta = c->items[c->topo_lo], &tb = c->items[c->topo_hi];
    const size_t m0 = ta.node_off, m1 = (size_t)tb.node_off + 2 * tb.n - 1;
    const size_t s0 = ta.sched_off, s1 = (size_t)tb.sched_off + 2 * tb.n + 2;
    const size_t l0 = c->topo_lo, l1 = (size_t)c->topo_hi + 1;
    r = r ? r : c->cuda(cudaMemcpyAsync(c->h_nodes + m0, c->d_nodes + m0, (m1 - m0) * sizeof(NodeRec), cudaMemcpyDeviceToHost, c->st), "mirror");
    r = r ? r : c->cuda(cudaMemcpyAsync(c->h_sched + s0, c->d_sched + s0, (s1 - s0) * sizeof(int16_t), cudaMemcpyDeviceToHost, c->st), "mirror");
    r = r ? r : c->cuda(cudaMemcpyAsync(c->h_nlev + l0, c->d_nlev + l0, (l1 - l0) * sizeof(int32_t), cudaMemcpyDeviceToHost, c->st), "mirror");
    // the stepwise alleles the genealogy update drew
    const LocusDev &Lb = c->loci[tb.locus].d;
    const size_t a0 = ta.al_off, a1 = (size_t)tb.al_off + (Lb.model == IMA_MODEL_SW ? (size_t)Lb.nlinked * (2 * tb.n - 1) : 0);
    if (a1 > a0)
      r = r ? r : c->cuda(cudaMemcpyAsync(c->h_al + a0, c->d_al + a0, (a1 - a0) * sizeof(int32_t), cudaMemcpyDeviceToHost, c->st), "mirror");
  }
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "mirror");
  c->dev_lo = INT32_MAX;
  c->dev_hi = -1;
  c->topo_lo = INT32_MAX;
  c->topo_hi = -1;
  return r;
}

static void mark(ima_ctx *c, int item)
{
  sync_mirror(c);
  c->dirty_lo = std::min(c->dirty_lo, item);
  c->dirty_hi = std::max(c->dirty_hi, item);
}

// What one genealogy upload changed: dirty item ranges (topology and times
// only) and the error, kept per worker so that uploads can run in parallel.
struct SetOut {
  int lo = INT32_MAX, hi = -1, tlo = INT32_MAX, thi = -1;
  int code = IMA_OK;
  char msg[256] = {0};
  int fail(int c, const char *fmt, ...)
  {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(msg, sizeof(msg), fmt, ap);
    va_end(ap);
    code = c;
    return c;
  }
  void merge_into(ima_ctx *c) const;  // the dirty ranges (the caller reports the error)
};

// writes genealogy data of one item into the pinned mirrors; touches only
// that item's entries (and thread_local scratch)
static int set_one(ima_ctx *c, int item, const int32_t *up0, const int32_t *up1, const int32_t *down,
                   const double *time, double length, SetOut &o)
{
  const ItemDev &it = c->items[item];
  const int n = it.n, nl = 2 * n - 1;
  NodeRec *rec = c->h_nodes + it.node_off;
  // same topology as the resident genealogy: only times and length change
  bool same = c->has_tree[item] != 0;
  for (int k = 0; same && k < nl; k++)
    same = rec[k].up0 == up0[k] && rec[k].up1 == up1[k] && rec[k].down == down[k];
  if (same) {
    double L = 0.0;
    for (int k = 0; k < nl; k++) {
      double t = time[k];
      c->h_t64[it.node_off + k] = t;
      if (down[k] >= 0) L += (up0[k] < 0) ? t : t - time[up0[k]];
    }
    c->h_len[item] = (length >= 0.0) ? length : L;
    o.tlo = std::min(o.tlo, item);
    o.thi = std::max(o.thi, item);
    return IMA_OK;
  }
  // validate the topology: tips have no daughters, internal nodes two, one root
  int root = -1;
  for (int k = 0; k < nl; k++) {
    bool tip = k < n;
    if (tip != (up0[k] < 0) || tip != (up1[k] < 0)) return o.fail(IMA_ERR_ARG, "node %d: daughters do not match tip/internal numbering", k);
    if (!tip) {
      if (up0[k] >= nl || up1[k] >= nl || up0[k] == up1[k]) return o.fail(IMA_ERR_ARG, "node %d: bad daughters", k);
      if (down[up0[k]] != k || down[up1[k]] != k) return o.fail(IMA_ERR_ARG, "node %d: parent links disagree", k);
    }
    if (down[k] < 0) {
      if (root >= 0) return o.fail(IMA_ERR_ARG, "two roots (%d, %d)", root, k);
      root = k;
    } else if (down[k] < n || down[k] >= nl) {
      return o.fail(IMA_ERR_ARG, "node %d: bad parent %d", k, down[k]);
    }
  }
  if (root < n) return o.fail(IMA_ERR_ARG, "no internal root");
  // heights by an explicit post-order from the root; levels = heights 1..H
  thread_local std::vector<int> height, stack, cnt, pos;
  thread_local std::vector<uint8_t> seen;
  height.assign(nl, 0);
  seen.assign(nl, 0);
  stack.clear();
  stack.push_back(root);
  int visited = 0;
  while (!stack.empty()) {
    int v = stack.back();
    if (v < n) {
      stack.pop_back();
      visited++;
      continue;
    }
    if (!seen[v]) {
      seen[v] = 1;
      stack.push_back(up0[v]);
      stack.push_back(up1[v]);
      if (stack.size() > (size_t)4 * nl) return o.fail(IMA_ERR_ARG, "genealogy has a cycle");
      continue;
    }
    stack.pop_back();
    height[v] = 1 + std::max(height[up0[v]], height[up1[v]]);
    visited++;
  }
  if (visited != nl) return o.fail(IMA_ERR_ARG, "genealogy is not connected");
  int H = height[root];
  cnt.assign(H + 2, 0);
  for (int k = n; k < nl; k++) cnt[height[k]]++;
  int16_t *sch = c->h_sched + it.sched_off;
  int16_t *order = sch, *lstart = sch + (n - 1);
  pos.assign(H + 2, 0);
  for (int h = 1; h <= H; h++) pos[h + 1] = pos[h] + cnt[h];
  for (int h = 1; h <= H + 1; h++) lstart[h - 1] = (int16_t)pos[h];
  for (int k = n; k < nl; k++) order[pos[height[k]]++] = (int16_t)k;
  c->h_nlev[item] = H;
  double L = 0.0;
  for (int k = 0; k < nl; k++) {
    NodeRec &r = c->h_nodes[it.node_off + k];
    r.up0 = (int16_t)up0[k];
    r.up1 = (int16_t)up1[k];
    r.down = (int16_t)down[k];
    r.pad = 0;
    double t = time[k];
    c->h_t64[it.node_off + k] = t;
    if (down[k] >= 0) L += (up0[k] < 0) ? t : t - time[up0[k]];
  }
  c->h_len[item] = (length >= 0.0) ? length : L;
  c->has_tree[item] = 1;
  o.lo = std::min(o.lo, item);
  o.hi = std::max(o.hi, item);
  return IMA_OK;
}

void SetOut::merge_into(ima_ctx *c) const
{
  c->dirty_lo = std::min(c->dirty_lo, lo);
  c->dirty_hi = std::max(c->dirty_hi, hi);
  c->tdirty_lo = std::min(c->tdirty_lo, tlo);
  c->tdirty_hi = std::max(c->tdirty_hi, thi);
}

extern "C" int ima_gpu_set_genealogy(ima_ctx *c, int ci, int li, const int32_t *up0, const int32_t *up1,
                                     const int32_t *down, const double *time, double length)
{
  if (!c || !up0 || !up1 || !down || !time) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  int r = sync_mirror(c);
  if (r) return r;
  SetOut o;
  r = set_one(c, c->item_of(ci, li), up0, up1, down, time, length, o);
  o.merge_into(c);
  if (r) c->err = o.msg;
  return r;
}

extern "C" int ima_gpu_set_genealogies(ima_ctx *c, int n, const int32_t *ci, const int32_t *li,
                                       const int32_t *up0, const int32_t *up1, const int32_t *down,
                                       const double *time, const double *length)
{
  if (!c || n < 0 || (n > 0 && (!ci || !li || !up0 || !up1 || !down || !time))) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (int rs = sync_mirror(c)) return rs;
  // offsets of each pair's nodes, and whether a pair repeats (then the list
  // is applied in order on one thread)
  // node offset of each pair (a context vector: the pool's threads read it)
  std::vector<size_t> &off = c->pair_off;
  off.resize((size_t)n + 1);
  off[0] = 0;
  bool repeat = false;
  if ((int)c->pair_stamp.size() != c->nitems) c->pair_stamp.assign(c->nitems, -1);
  const int gen = ++c->stamp_gen;
  for (int k = 0; k < n; k++) {
    if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "pair %d: chain %d locus %d out of range", k, ci[k], li[k]);
    const int item = c->item_of(ci[k], li[k]);
    if (c->pair_stamp[item] == gen) repeat = true;
    c->pair_stamp[item] = gen;
    off[k + 1] = off[k] + 2 * c->loci[li[k]].d.n - 1;
  }
  const size_t *offp = off.data();
  auto apply = [c, ci, li, up0, up1, down, time, length, offp](int k0, int k1, SetOut &o) {
    for (int k = k0; k < k1; k++) {
      const size_t f = offp[k];
      if (set_one(c, c->item_of(ci[k], li[k]), up0 + f, up1 + f, down + f, time + f, length ? length[k] : -1.0, o))
        return;
    }
  };
  if (repeat || n < 128) {  // below this, waking the pool costs more than it saves
    SetOut o;
    apply(0, n, o);
    o.merge_into(c);
    if (o.code) c->err = o.msg;
    return o.code;
  }
  if (!c->pool) {
    const unsigned hw = std::thread::hardware_concurrency();
    c->pool.reset(new HostPool((int)std::max(1u, std::min(hw, 16u)) - 1));
  }
  const int nchunk = std::min(std::max(2, n / 64), 4 * c->pool->size());
  std::vector<SetOut> outs(nchunk);
  c->pool->run(nchunk, [&](int j) {
    apply((int)((long long)n * j / nchunk), (int)((long long)n * (j + 1) / nchunk), outs[j]);
  });
  int r = IMA_OK;
  for (int j = 0; j < nchunk; j++) {  // the first failing chunk names the error
    outs[j].merge_into(c);
    if (!r && outs[j].code) {
      r = outs[j].code;
      c->err = outs[j].msg;
    }
  }
  return r;
}

// the float-float copy of uploaded FP64 node times, made on the device (hi
// the nearest float, lo the nearest float to the remainder), so a re-timing
// copies 8 bytes per node instead of 16
__global__ void k_split_times(const double *t64, float2 *tff, size_t n)
{
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double t = t64[i];
  const float hi = (float)t;
  tff[i] = make_float2(hi, (float)(t - (double)hi));
}

// Tree lengths of items lo .. lo + n - 1 in two passes.  (1) A warp per
// item forms every node's branch term (coalesced reads, the daughter's time
// from L1/L2) into term[]; (2) a thread per item adds its terms in node
// order -- the host's sum, bit for bit -- with independent loads and one
// FP64 add per node on one lane each (GB300 issues FP64 at 1/64 of the FP32
// rate: a warp-wide sequential sum would spend 32 lanes per add).
__global__ void k_branch_terms(const ItemDev *items, const NodeRec *nodes, const double *t64, double *term, int lo,
                               int n)
{
  const int w = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (w >= n) return;
  const ItemDev it = items[lo + w];
  const int nl = 2 * it.n - 1;
  const NodeRec *r = nodes + it.node_off;
  const double *t = t64 + it.node_off;
  double *out = term + it.node_off;
  for (int j = lane; j < nl; j += 32) {
    const NodeRec nd = r[j];
    out[j] = nd.down < 0 ? 0.0 : (nd.up0 < 0 ? t[j] : t[j] - t[nd.up0]);
  }
}

__global__ void k_sum_terms(const ItemDev *items, const NodeRec *nodes, const double *term, double *len, int lo,
                            int n)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const ItemDev it = items[lo + k];
  const NodeRec *r = nodes + it.node_off;
  const double *v = term + it.node_off;
  const int nl = 2 * it.n - 1;
  double L = 0.0;
#pragma unroll 8
  for (int j = 0; j < nl; j++)
    if (r[j].down >= 0) L += v[j];
  len[lo + k] = L;
}

// A short run in one kernel, a warp per item: the times read from src
// (indexed by node_off - src0: the caller's packed run where the device can
// read it, or the device times themselves when src == t64), copied into t64,
// their float-float form, and the tree length -- given (src_len) or its
// branch terms added in node order, broadcast lane by lane (the host's sum,
// bit for bit; every lane repeats the FP64 adds, which only a short run can
// afford on GB300's FP64 pipe).
constexpr long long SHORT_RUN_NODES = 1 << 16;
// Longer runs are copied by the copy engine: on GB300 a kernel read 9.2 MB
// of the caller's pageable memory at ~175 GB/s but 478 MB at ~70 GB/s,
// where one pageable copy ran at ~170 GB/s
constexpr long long PULL_RUN_NODES = 1 << 22;
__global__ void k_times_short(const ItemDev *items, const NodeRec *nodes, const double *src, size_t src0,
                              const double *src_len, double *t64, float2 *tff, double *len, int lo, int n)
{
  const int w = (int)(((size_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
  if (w >= n) return;  // whole warps
  const ItemDev it = items[lo + w];
  const int nl = 2 * it.n - 1;
  const NodeRec *r = nodes + it.node_off;
  const double *t = src + (it.node_off - src0);
  double *t_out = t64 + it.node_off;
  float2 *f = tff + it.node_off;
  const bool copy = (src != t64);
  double L = 0.0;
  for (int j0 = 0; j0 < nl; j0 += 32) {
    const int j = j0 + lane;
    double term = 0.0;
    bool has = false;
    if (j < nl) {
      const double tj = t[j];
      if (copy) t_out[j] = tj;
      const float hi = (float)tj;
      f[j] = make_float2(hi, (float)(tj - (double)hi));
      const NodeRec nd = r[j];
      if (!src_len && nd.down >= 0) {
        has = true;
        term = (nd.up0 < 0) ? tj : tj - t[nd.up0];
      }
    }
    if (src_len) continue;  // uniform across the warp
    const unsigned mask = __ballot_sync(0xffffffffu, has);
    const int cnt = min(32, nl - j0);
    for (int k = 0; k < cnt; k++) {
      const double v = __shfl_sync(0xffffffffu, term, k);
      if ((mask >> k) & 1u) L += v;
    }
  }
  if (lane == 0) len[lo + w] = src_len ? src_len[w] : L;
}

// The caller's packed times of a run, read where they lie (host memory the
// device can access), into the device times and their float-float copy:
// one coalesced pass, grid-stride.
__global__ void k_pull_times(const double *src, double *t64, float2 *tff, size_t n)
{
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double t = src[i];
    t64[i] = t;
    const float hi = (float)t;
    tff[i] = make_float2(hi, (float)(t - (double)hi));
  }
}

__global__ void k_pull_lengths(const double *src, double *len, int n)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) len[i] = src[i];
}

// The lengths still pending, summed now (before a reader: the infinite-sites
// likelihood, the band and the genealogy weights, the mirror).
static int ensure_lengths(ima_ctx *c)
{
  if (c->lpend_hi < 0) return IMA_OK;
  const int lo = c->lpend_lo, n = c->lpend_hi - lo + 1;
  c->lpend_lo = INT32_MAX;
  c->lpend_hi = -1;
  if (!c->d_lterm) {
    c->d_lterm = dev_alloc<double>(c->nnodes, c->dev_bytes, c->st);
    if (!c->d_lterm) return c->fail(IMA_ERR_NOMEM, "branch-length scratch");
  }
  c->launch(IMA_K_TIMES, 0.0, [&] {
    k_branch_terms<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, c->st>>>(c->d_items, c->d_nodes, c->d_t64,
                                                                               c->d_lterm, lo, n);
    k_sum_terms<<<(n + 127) / 128, 128, 0, c->st>>>(c->d_items, c->d_nodes, c->d_lterm, c->d_len, lo, n);
  });
  return c->cuda(cudaGetLastError(), "lengths");
}

// Items lo .. hi get lengths summed later; a range apart from the pending
// one is summed first (the pending range stays one interval, and items
// between the two may hold lengths a caller gave).
static int pend_lengths(ima_ctx *c, int lo, int hi)
{
  if (c->lpend_hi >= 0 && (lo > c->lpend_hi + 1 || hi < c->lpend_lo - 1))
    if (int r = ensure_lengths(c)) return r;
  c->lpend_lo = std::min(c->lpend_lo, lo);
  c->lpend_hi = std::max(c->lpend_hi, hi);
  return IMA_OK;
}

static void split_times(ima_ctx *c, size_t n0, size_t n1)
{
  if (n1 <= n0) return;
  const size_t n = n1 - n0;
  k_split_times<<<(unsigned)((n + 255) / 256), 256, 0, c->st>>>(c->d_t64 + n0, c->d_tff + n0, n);
}

static int flush(ima_ctx *c);

// Re-timings with the topology kept (the moves of changet_RY1 and of a
// rubber band): only the node times, and the length (given, or summed here
// in node order), go to the mirror.
static void set_times_one(ima_ctx *c, int item, const double *time, double length)
{
  const ItemDev &it = c->items[item];
  const int nl = 2 * it.n - 1;
  memcpy(c->h_t64 + it.node_off, time, nl * sizeof(double));
  if (length >= 0.0) {
    c->h_len[item] = length;
    return;
  }
  const NodeRec *rec = c->h_nodes + it.node_off;
  double L = 0.0;
  for (int k = 0; k < nl; k++)
    if (rec[k].down >= 0) L += (rec[k].up0 < 0) ? time[k] : time[k] - time[rec[k].up0];
  c->h_len[item] = L;
}

// The pairs of a re-timing: each a chain-locus holding a genealogy; their
// item range, and whether they are items first, first + 1, ... in order (a
// run).  A list given again is not walked again (pairs only gain
// genealogies, except when a checkpoint is read, which bumps tree_gen).
static int check_pairs(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, int *lo_, int *hi_, bool *run_)
{
  int lo = INT32_MAX, hi = -1;
  bool run = false;
  if (c->tk_gen == c->tree_gen && (int)c->tk_ci.size() == n && !memcmp(c->tk_ci.data(), ci, n * sizeof(int32_t)) &&
      !memcmp(c->tk_li.data(), li, n * sizeof(int32_t))) {
    lo = c->tk_lo;
    hi = c->tk_hi;
    run = c->tk_run;
  } else {
    run = c->valid(ci[0], li[0]);
    const int first = run ? c->item_of(ci[0], li[0]) : 0;
    const uint8_t *has = c->has_tree.data();
    for (int k = 0; k < n; k++) {
      if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "pair %d: chain %d locus %d out of range", k, ci[k], li[k]);
      const int item = c->item_of(ci[k], li[k]);
      if (!has[item]) return c->fail(IMA_ERR_STATE, "pair %d: chain %d locus %d has no genealogy", k, ci[k], li[k]);
      lo = std::min(lo, item);
      hi = std::max(hi, item);
      run = run && item == first + k;
    }
    c->tk_ci.assign(ci, ci + n);
    c->tk_li.assign(li, li + n);
    c->tk_lo = lo;
    c->tk_hi = hi;
    c->tk_run = run;
    c->tk_gen = c->tree_gen;
  }
  *lo_ = lo;
  *hi_ = hi;
  *run_ = run;
  return IMA_OK;
}

// New times of genealogies whose topology is kept.  in_place: a contiguous
// run may be read by the device from the caller's buffers while the stream
// runs (the caller synchronises the stream before returning); *read_in_place
// tells whether that happened.
static int upload_times(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *time,
                        const double *length, bool in_place, bool *read_in_place)
{
  if (read_in_place) *read_in_place = false;
  if (!c || n < 0 || (n > 0 && (!ci || !li || !time))) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (n == 0) return IMA_OK;
  int lo = INT32_MAX, hi = -1;
  bool run = false;  // the pairs are items first, first + 1, ... in order
  if (int r = check_pairs(c, n, ci, li, &lo, &hi, &run)) return r;
  if (run) {
    // a contiguous run of items in order: the caller's packed times are the
    // device layout of the run, so they go to the device in one copy (from
    // pageable memory: the call returns once the buffer has been read), the
    // device makes their float-float form and, when no lengths are given,
    // the lengths (in the host's order of additions).
    // The device then holds the newer values; the mirror is refreshed before
    // the host next writes it.  Uploads still pending from the mirror go
    // first.
    if (int r = flush(c)) return r;
    const size_t n0 = c->items[lo].node_off, n1 = (size_t)c->items[hi].node_off + 2 * c->items[hi].n - 1;
    if (in_place && c->pageable_access && (long long)(n1 - n0) <= SHORT_RUN_NODES) {
      // a short run: one kernel reads it in place (times, float-float form,
      // lengths), nothing left pending
      if (int r = ensure_lengths(c)) return r;
      c->launch(IMA_K_TIMES, (double)(n1 - n0) * 16.0, [&] {
        k_times_short<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, c->st>>>(
            c->d_items, c->d_nodes, time, n0, length, c->d_t64, c->d_tff, c->d_len, lo, n);
      });
      if (read_in_place) *read_in_place = true;
      c->dev_lo = std::min(c->dev_lo, lo);
      c->dev_hi = std::max(c->dev_hi, hi);
      return c->cuda(cudaGetLastError(), "times upload");
    }
    if (in_place && c->pageable_access && (long long)(n1 - n0) <= PULL_RUN_NODES) {
      // the device reads the run where it lies (times and their float-float
      // form in one coalesced pass), no staging copy; the lengths are read
      // too, or summed from the device times
      if (length) {
        if (int r = ensure_lengths(c)) return r;  // pending ones inside the run would overwrite these
      } else if (int r = pend_lengths(c, lo, hi)) {
        return r;
      }
      c->launch(IMA_K_TIMES, (double)(n1 - n0) * 16.0, [&] {
        const unsigned g = (unsigned)std::min<size_t>(4 * (size_t)c->nsm, (n1 - n0 + 255) / 256);
        k_pull_times<<<g, 256, 0, c->st>>>(time, c->d_t64 + n0, c->d_tff + n0, n1 - n0);
        if (length) k_pull_lengths<<<(n + 255) / 256, 256, 0, c->st>>>(length, c->d_len + lo, n);
      });
      if (read_in_place) *read_in_place = true;
      c->dev_lo = std::min(c->dev_lo, lo);
      c->dev_hi = std::max(c->dev_hi, hi);
      return c->cuda(cudaGetLastError(), "times upload");
    }
    int r = c->cuda(cudaMemcpyAsync(c->d_t64 + n0, time, (n1 - n0) * sizeof(double), cudaMemcpyHostToDevice, c->st),
                    "times upload");
    if (r) return r;
    if (length) {
      r = ensure_lengths(c);  // pending ones inside the run would overwrite these
      r = r ? r : c->cuda(cudaMemcpyAsync(c->d_len + lo, length, (size_t)n * sizeof(double), cudaMemcpyHostToDevice,
                                          c->st), "length");
    }
    if (r) return r;
    if ((long long)(n1 - n0) <= SHORT_RUN_NODES) {  // one kernel, nothing left pending
      r = ensure_lengths(c);
      if (!r)
        c->launch(IMA_K_TIMES, (double)(n1 - n0) * 16.0, [&] {
          k_times_short<<<(unsigned)(((size_t)n * 32 + 127) / 128), 128, 0, c->st>>>(
              c->d_items, c->d_nodes, c->d_t64, 0, length ? c->d_len + lo : nullptr, c->d_t64, c->d_tff, c->d_len,
              lo, n);
        });
    } else {
      c->launch(IMA_K_TIMES, (double)(n1 - n0) * 16.0, [&] { split_times(c, n0, n1); });
      if (!length) r = pend_lengths(c, lo, hi);
    }
    c->dev_lo = std::min(c->dev_lo, lo);
    c->dev_hi = std::max(c->dev_hi, hi);
    return r ? r : c->cuda(cudaGetLastError(), "times upload");
  }

  // any order: staged in the mirror on the host threads (a pair given twice
  // keeps its later times only when the list is applied in order on one
  // thread), copied with the next evaluation
  std::vector<size_t> &off = c->pair_off;
  off.resize((size_t)n + 1);
  off[0] = 0;
  for (int k = 0; k < n; k++) off[k + 1] = off[k] + 2 * c->loci[li[k]].d.n - 1;
  const size_t *offp = off.data();
  if (int rs = sync_mirror(c)) return rs;
  bool repeat = false;
  if ((int)c->pair_stamp.size() != c->nitems) c->pair_stamp.assign(c->nitems, -1);
  const int gen = ++c->stamp_gen;
  for (int k = 0; k < n; k++) {
    const int item = c->item_of(ci[k], li[k]);
    if (c->pair_stamp[item] == gen) repeat = true;
    c->pair_stamp[item] = gen;
  }
  auto apply = [c, ci, li, time, length, offp](int k0, int k1) {
    for (int k = k0; k < k1; k++)
      set_times_one(c, c->item_of(ci[k], li[k]), time + offp[k], length ? length[k] : -1.0);
  };
  if (repeat || n < 128) {
    apply(0, n);
  } else {
    if (!c->pool) {
      const unsigned hw = std::thread::hardware_concurrency();
      c->pool.reset(new HostPool((int)std::max(1u, std::min(hw, 16u)) - 1));
    }
    const int nchunk = std::min(std::max(2, n / 64), 4 * c->pool->size());
    c->pool->run(nchunk, [&](int j) { apply((int)((long long)n * j / nchunk), (int)((long long)n * (j + 1) / nchunk)); });
  }
  c->tdirty_lo = std::min(c->tdirty_lo, lo);
  c->tdirty_hi = std::max(c->tdirty_hi, hi);
  return IMA_OK;
}

extern "C" int ima_gpu_set_times(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *time,
                                 const double *length)
{
  return upload_times(c, n, ci, li, time, length, false, nullptr);
}

extern "C" int ima_gpu_set_pi(ima_ctx *c, int ci, int li, const double *pi4)
{
  if (!c || !pi4) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  int item = c->item_of(ci, li);
  for (int j = 0; j < 4; j++) c->h_pi[4 * (size_t)item + j] = pi4[j];
  mark(c, item);
  return IMA_OK;
}

extern "C" int ima_gpu_set_alleles(ima_ctx *c, int ci, int li, int ai, const int32_t *A)
{
  if (!c || !A) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  const LocusDev &L = c->loci[li].d;
  if (L.model != IMA_MODEL_SW || ai < 0 || ai >= L.nlinked) return c->fail(IMA_ERR_ARG, "locus %d marker %d is not stepwise", li, ai);
  int item = c->item_of(ci, li);
  const ItemDev &it = c->items[item];
  int nl = 2 * it.n - 1;
  memcpy(c->h_al + it.al_off + (size_t)ai * nl, A, sizeof(int32_t) * nl);
  mark(c, item);
  return IMA_OK;
}

extern "C" int ima_gpu_get_alleles(ima_ctx *c, int ci, int li, int ai, int32_t *A)
{
  if (!c || !A) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  const LocusDev &L = c->loci[li].d;
  if (L.model != IMA_MODEL_SW || ai < 0 || ai >= L.nlinked) return c->fail(IMA_ERR_ARG, "locus %d marker %d is not stepwise", li, ai);
  cudaSetDevice(c->device);
  if (int r = flush(c)) return r;  // host edits not yet on the device go first
  const ItemDev &it = c->items[c->item_of(ci, li)];
  const int nl = 2 * it.n - 1;
  int r = c->cuda(cudaMemcpyAsync(A, c->d_al + it.al_off + (size_t)ai * nl, nl * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  c->st), "alleles");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "alleles");
}

extern "C" int ima_gpu_set_allele_edits(ima_ctx *c, int n, const int *ci, const int *li, const int *ai,
                                        const int *node, const int32_t *A)
{
  if (!c || n < 0 || (n > 0 && (!ci || !li || !ai || !node || !A))) return IMA_ERR_ARG;
  // validate the whole list before applying any edit
  for (int k = 0; k < n; k++) {
    if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "edit %d: chain %d locus %d out of range", k, ci[k], li[k]);
    const LocusDev &L = c->loci[li[k]].d;
    if (L.model != IMA_MODEL_SW || ai[k] < 0 || ai[k] >= L.nlinked)
      return c->fail(IMA_ERR_ARG, "edit %d: locus %d marker %d is not stepwise", k, li[k], ai[k]);
    const ItemDev &it = c->items[c->item_of(ci[k], li[k])];
    if (node[k] < 0 || node[k] >= 2 * it.n - 1) return c->fail(IMA_ERR_ARG, "edit %d: node %d out of range", k, node[k]);
  }
  for (int k = 0; k < n; k++) {
    const int item = c->item_of(ci[k], li[k]);
    const ItemDev &it = c->items[item];
    c->h_al[it.al_off + (size_t)ai[k] * (2 * it.n - 1) + node[k]] = A[k];
    mark(c, item);
  }
  return IMA_OK;
}

static int flush_times(ima_ctx *c)
{
  if (c->tdirty_hi < 0) return IMA_OK;
  int lo = c->tdirty_lo, hi = c->tdirty_hi;
  const ItemDev &a = c->items[lo], &b = c->items[hi];
  size_t n0 = a.node_off, n1 = (size_t)b.node_off + 2 * b.n - 1;
  cudaStream_t st = c->st;
  int r = IMA_OK;
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_t64 + n0, c->h_t64 + n0, (n1 - n0) * sizeof(double), cudaMemcpyHostToDevice, st), "times");
  if (!r) split_times(c, n0, n1);
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_len + lo, c->h_len + lo, (hi - lo + 1) * sizeof(double), cudaMemcpyHostToDevice, st), "length");
  c->tdirty_lo = INT32_MAX;
  c->tdirty_hi = -1;
  return r;
}

static int flush(ima_ctx *c)
{
  if (c->dirty_hi < 0) return flush_times(c);
  // a topology range covers times too; widen it by the time-only range
  if (c->tdirty_hi >= 0) {
    c->dirty_lo = std::min(c->dirty_lo, c->tdirty_lo);
    c->dirty_hi = std::max(c->dirty_hi, c->tdirty_hi);
    c->tdirty_lo = INT32_MAX;
    c->tdirty_hi = -1;
  }
  int lo = c->dirty_lo, hi = c->dirty_hi;
  const ItemDev &a = c->items[lo], &b = c->items[hi];
  size_t n0 = a.node_off, n1 = (size_t)b.node_off + 2 * b.n - 1;
  size_t s0 = a.sched_off, s1 = (size_t)b.sched_off + 2 * b.n + 2;
  size_t a0 = a.al_off, a1 = (size_t)b.al_off;
  a1 += (c->loci[b.locus].d.model == IMA_MODEL_SW) ? (size_t)c->loci[b.locus].d.nlinked * (2 * b.n - 1) : 0;
  cudaStream_t st = c->st;
  int r = IMA_OK;
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_nodes + n0, c->h_nodes + n0, (n1 - n0) * sizeof(NodeRec), cudaMemcpyHostToDevice, st), "nodes");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_t64 + n0, c->h_t64 + n0, (n1 - n0) * sizeof(double), cudaMemcpyHostToDevice, st), "times");
  if (!r) split_times(c, n0, n1);
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_sched + s0, c->h_sched + s0, (s1 - s0) * sizeof(int16_t), cudaMemcpyHostToDevice, st), "sched");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_nlev + lo, c->h_nlev + lo, (hi - lo + 1) * sizeof(int32_t), cudaMemcpyHostToDevice, st), "levels");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_len + lo, c->h_len + lo, (hi - lo + 1) * sizeof(double), cudaMemcpyHostToDevice, st), "length");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_pi + 4 * (size_t)lo, c->h_pi + 4 * (size_t)lo, 4 * (hi - lo + 1) * sizeof(double), cudaMemcpyHostToDevice, st), "pi");
  if (a1 > a0) r = r ? r : c->cuda(cudaMemcpyAsync(c->d_al + a0, c->h_al + a0, (a1 - a0) * sizeof(int32_t), cudaMemcpyHostToDevice, st), "alleles");
  // topologies may have changed: the IS site caches of the range are stale
  r = r ? r : c->cuda(cudaMemsetAsync(c->d_is_valid + lo, 0, hi - lo + 1, st), "IS site cache");
  c->dirty_lo = INT32_MAX;
  c->dirty_hi = -1;
  return r;
}

extern "C" int ima_gpu_flush_genealogies(ima_ctx *c)
{
  if (!c) return IMA_ERR_ARG;
  return flush(c);
}

// ======================================================================
// batches
static int ensure_fp64_hky(ima_ctx *c)
{
  if (c->d_part64 || c->npart64 == 0) {
    if (!c->d_slot64) {
      c->d_slot64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
      c->d_fresh64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
    }
    return IMA_OK;
  }
  c->d_part64 = dev_alloc<double>(4 * c->npart64, c->dev_bytes, c->st);
  c->d_psf64 = dev_alloc<double>(c->npart64, c->dev_bytes, c->st);
  c->d_slot64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
  c->d_fresh64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
  if (!c->d_part64 || !c->d_psf64 || !c->d_slot64 || !c->d_fresh64)
    return c->fail(IMA_ERR_NOMEM, "FP64 partial likelihood pools (%zu doubles) do not fit", 5 * c->npart64);
  return IMA_OK;
}

// lo parts of the float-float HKY partials, allocated on first use
static int ensure_ff_hky(ima_ctx *c)
{
  if (c->d_partlo || c->npart == 0) return IMA_OK;
  c->d_partlo = dev_alloc<float4>(c->npart, c->dev_bytes, c->st);
  if (!c->d_partlo) return c->fail(IMA_ERR_NOMEM, "float-float partial likelihoods (%zu float4) do not fit", c->npart);
  // the hi parts already in place (FP32 evaluations) read as exact pairs
  return c->cuda(cudaMemsetAsync(c->d_partlo, 0, c->npart * sizeof(float4), c->st), "float-float partials");
}

static double hky_bytes(ima_ctx *c, const Batch &b);
static double sw_bytes(ima_ctx *c, const Batch &b);

static void batch_shape(const Batch &b, int *k)
{
  const int v[7] = {b.nis, b.nhky, b.nsw, b.maxn_hky, b.maxs_hky, b.maxn_sw, b.prec};
  memcpy(k, v, sizeof(v));
}

static int build_batch(ima_ctx *c, Batch &b, int n, const int32_t *ci, const int32_t *li, const double *u,
                       const double *kappa, const int32_t *edits, const int32_t *ai, int prec)
{
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (n < 1 || !ci || !li || !u) return c->fail(IMA_ERR_ARG, "empty or null request list");
  if (prec != IMA_PREC_FAST && prec != IMA_PREC_FP64 && prec != IMA_PREC_FP32)
    return c->fail(IMA_ERR_ARG, "bad precision");
  std::vector<int> g[3];
  for (int k = 0; k < n; k++) {
    if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "request %d: chain %d locus %d out of range", k, ci[k], li[k]);
    const LocusDev &L = c->loci[li[k]].d;
    if (L.model == IMA_MODEL_SW && ai && (ai[k] < 0 || ai[k] >= L.nlinked)) return c->fail(IMA_ERR_ARG, "request %d: bad marker", k);
    if (!(u[k] > 0.0)) return c->fail(IMA_ERR_ARG, "request %d: mutation rate must be > 0", k);
    if (!c->has_tree[c->item_of(ci[k], li[k])]) return c->fail(IMA_ERR_STATE, "request %d: chain %d locus %d has no genealogy", k, ci[k], li[k]);
    g[L.model].push_back(k);
  }
  // largest chain-loci first inside each model (longest-processing-time
  // order: the big ones start in the first wave, small ones fill the tail)
  auto cost = [&](int k) {
    const LocusDev &L = c->loci[li[k]].d;
    return L.model == IMA_MODEL_HKY ? (long long)(L.n - 1) * L.nsites : (long long)L.n;
  };
  for (int m = 1; m < 3; m++)
    std::stable_sort(g[m].begin(), g[m].end(), [&](int a, int b) { return cost(a) > cost(b); });
  b.n = n;
  b.prec = prec;
  b.nis = (int)g[0].size();
  b.nhky = (int)g[1].size();
  b.nsw = (int)g[2].size();
  // fewer HKY chain-loci than SMs: each runs alone on its SM, so the
  // widest CTA (256 threads) shortens the level chain
  b.hky_variant = (b.nhky > 0 && b.nhky < c->nsm) ? 2 : 0;
  b.order.clear();
  b.h_req.clear();
  b.maxn_is = b.maxs_is = b.maxn_hky = b.maxs_hky = b.maxn_sw = 0;
  for (int m = 0; m < 3; m++)
    for (int k : g[m]) {
      ReqDev r;
      r.item = c->item_of(ci[k], li[k]);
      r.ai = ai ? ai[k] : 0;
      for (int q = 0; q < 4; q++) r.e[q] = edits ? edits[4 * k + q] : -1;
      {
        const ItemDev &it = c->items[r.item];
        const LocusDev &Ld = c->loci[it.locus].d;
        r.part_off = it.part_off;
        r.node_off = it.node_off;
        r.sched_off = it.sched_off;
        r.n = it.n;
        r.nsites = Ld.nsites;
        r.totsites = Ld.totsites;
        r.seq_off = Ld.seq_off;
        r.mult_off = Ld.mult_off;
        r.pad = 0;
      }
      r.u = u[k];
      r.par = kappa ? kappa[k] : 1.0;
      const LocusDev &L = c->loci[li[k]].d;
      if (m == 0) { b.maxn_is = std::max(b.maxn_is, L.n); b.maxs_is = std::max(b.maxs_is, L.nsites); }
      if (m == 1) { b.maxn_hky = std::max(b.maxn_hky, L.n); b.maxs_hky = std::max(b.maxs_hky, L.nsites); }
      if (m == 2) b.maxn_sw = std::max(b.maxn_sw, L.n);
      b.h_req.push_back(r);
      b.order.push_back(k);
    }
  if (b.nhky && prec == IMA_PREC_FP64) {
    int r = ensure_fp64_hky(c);
    if (r) return r;
  }
  if (b.nhky && prec == IMA_PREC_FAST) {
    int r = ensure_ff_hky(c);
    if (r) return r;
  }
  if (!c->d_slot64 && b.nhky) {
    // the commit kernel touches both slot sets; keep the FP64 marks allocated
    c->d_slot64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
    c->d_fresh64 = dev_alloc<uint8_t>(c->nnodes, c->dev_bytes, c->st);
  }
  if (b.cap < n) {
    // the previous capacity may still be read by queued work
    cudaStreamSynchronize(c->st);
    cudaFree(b.d_req);
    cudaFree(b.d_res);
    cudaFreeHost(b.h_res);
    cudaFreeHost(b.h_reqpin);
    size_t &B = c->dev_bytes;
    const size_t rw = (size_t)n + ((size_t)n + 1) / 2;  // doubles holding n results and n status words
    b.d_req = dev_alloc<ReqDev>(n, B, c->st);
    b.d_res = dev_alloc<double>(rw, B, c->st);
    b.d_st = b.d_res ? reinterpret_cast<int32_t *>(b.d_res + n) : nullptr;
    b.h_res = host_alloc<double>(rw);
    b.h_st = b.h_res ? reinterpret_cast<int32_t *>(b.h_res + n) : nullptr;
    b.h_reqpin = host_alloc<ReqDev>(n);
    if (!b.req_ev) cudaEventCreateWithFlags(&b.req_ev, cudaEventDisableTiming);
    if (!b.d_req || !b.d_res || !b.h_res || !b.h_reqpin || !b.req_ev) {
      b.cap = 0;
      return c->fail(IMA_ERR_NOMEM, "batch buffers");
    }
    b.cap = n;
  }
  b.hky_bytes = hky_bytes(c, b);
  b.sw_bytes = sw_bytes(c, b);
  {
    int key[7];
    batch_shape(b, key);
    for (const auto &t : c->tuned)
      if (!memcmp(t.key, key, sizeof(key))) {
        b.hky_variant = t.hky;
        b.sw_variant = t.sw;
      }
  }
  b.dl_idx.clear();
  for (int k = b.nis + b.nhky; k < b.n; k++)
    b.dl_idx.push_back(c->items[b.h_req[k].item].al_off + b.h_req[k].ai);
  b.dl_stamp = -1;
  b.in_order = true;
  for (int k = 0; k < b.n && b.in_order; k++) b.in_order = (b.order[k] == k);
  // an earlier upload from the staging buffer may still be queued
  if (int r = c->cuda(cudaEventSynchronize(b.req_ev), "requests")) return r;
  memcpy(b.h_reqpin, b.h_req.data(), n * sizeof(ReqDev));
  int r = c->cuda(cudaMemcpyAsync(b.d_req, b.h_reqpin, n * sizeof(ReqDev), cudaMemcpyHostToDevice, c->st), "requests");
  return r ? r : c->cuda(cudaEventRecord(b.req_ev, c->st), "requests");
}

static double hky_bytes(ima_ctx *c, const Batch &b)
{
  double s = 0;
  for (int k = b.nis; k < b.nis + b.nhky; k++) {
    const ItemDev &it = c->items[b.h_req[k].item];
    const LocusDev &L = c->loci[it.locus].d;
    double nodes = (double)(2 * it.n - 1);
    // written partials (FP32: 16 B + 4 B exponent; float-float: + 16 B lo
    // parts), tip states, multiplicities, topology and times
    const double pw = b.prec == IMA_PREC_FP32 ? 20.0 : 36.0;
    s += (double)(it.n - 1) * L.nsites * pw + (double)it.n * L.nsites + L.nsites * 4.0 + nodes * 16.0;
  }
  return b.prec == IMA_PREC_FP64 ? s * 40.0 / 36.0 : s;
}

static double sw_bytes(ima_ctx *c, const Batch &b)
{
  double s = 0;
  for (int k = b.nis + b.nhky; k < b.n; k++) {
    const ItemDev &it = c->items[b.h_req[k].item];
    s += (double)(2 * it.n - 1) * 28.0;  // node + times + allele + dlikeA write
  }
  return s;
}

// kernels of a batch (no host work, graph-capturable once sumlogk is set)
// kernels of a batch (no host work, graph-capturable once sumlogk is set)
static void enqueue(ima_ctx *c, Batch &b, cudaStream_t on = nullptr)
{
  Pools P = c->pools();
  cudaStream_t st = on ? on : c->st;
  if (b.nis)
    c->launch(IMA_K_IS, 0.0, [&] { launch_is(P, b.d_req, b.nis, b.maxn_is, b.maxs_is, b.d_res, b.d_st, nullptr, st); }, st);
  if (b.nhky) {
    const ReqDev *r = b.d_req + b.nis;
    if (b.prec == IMA_PREC_FP64)
      c->launch(IMA_K_HKY_FP64, b.hky_bytes, [&] { launch_hky_fp64(P, r, b.nhky, b.maxn_hky, b.d_res + b.nis, b.d_st + b.nis, st); }, st);
    else if (b.prec == IMA_PREC_FP32)
      c->launch(IMA_K_HKY_FP32, b.hky_bytes, [&] { launch_hky_fp32(P, r, b.nhky, b.maxn_hky, b.maxs_hky, b.hky_variant, b.d_res + b.nis, b.d_st + b.nis, st); }, st);
    else
      c->launch(IMA_K_HKY_FAST, b.hky_bytes, [&] { launch_hky_fast(P, r, b.nhky, b.maxn_hky, b.maxs_hky, b.hky_variant, b.d_res + b.nis, b.d_st + b.nis, st); }, st);
  }
  if (b.nsw) {
    const ReqDev *r = b.d_req + b.nis + b.nhky;
    int off = b.nis + b.nhky;
    if (b.prec == IMA_PREC_FP64)
      c->launch(IMA_K_SW_FP64, b.sw_bytes, [&] { launch_sw_fp64(P, r, b.nsw, b.d_res + off, b.d_st + off, st); }, st);
    else
      c->launch(IMA_K_SW_FAST, b.sw_bytes, [&] { launch_sw_fast(P, r, b.nsw, b.maxn_sw, b.sw_variant, b.d_res + off, b.d_st + off, st); }, st);
  }
}

// the reference caches sum log k! from the first genealogy it evaluates per locus
static int init_sumlogk(ima_ctx *c, Batch &b)
{
  bool any = false;
  for (int k = 0; k < b.nis; k++) {
    int li = c->items[b.h_req[k].item].locus;
    if (!c->loci[li].sumlogk_done) any = true;
  }
  if (!any) return IMA_OK;
  // first request of each uninitialised locus in the caller's order
  std::vector<std::pair<int, int>> firsts;  // (caller index, grouped index)
  for (int k = 0; k < b.nis; k++) firsts.push_back({b.order[k], k});
  std::sort(firsts.begin(), firsts.end());
  Pools P = c->pools();
  std::vector<int> inited;
  for (auto &f : firsts) {
    int item = b.h_req[f.second].item;
    int li = c->items[item].locus;
    LocusHost &L = c->loci[li];
    if (L.sumlogk_done) continue;
    c->launch(IMA_K_IS_SUMLOGK, 0.0, [&] { launch_is_sumlogk(P, item, li, L.d.n, L.d.nsites, c->d_flag, c->st); });
    int flag = 0;
    int r = c->cuda(cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->st), "sumlogk flag");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "sumlogk");
    if (r) return r;
    if (flag == 2) return c->fail(IMA_ERR_DATA, "Data incompatible with current genealogy, likelihood calculation failed, chain %d, locus %d", item / c->nloci, li);
    L.sumlogk_done = true;
  }
  return IMA_OK;
}

static int fetch(ima_ctx *c, Batch &b, double *result, int32_t *status)
{
  // results and status words lie together in one buffer of capacity
  // b.cap: two copies when the batch fills less than its capacity
  int r;
  if (b.n == b.cap) {
    r = c->cuda(cudaMemcpyAsync(b.h_res, b.d_res, b.n * (sizeof(double) + sizeof(int32_t)), cudaMemcpyDeviceToHost, c->st),
                "results");
  } else {
    r = c->cuda(cudaMemcpyAsync(b.h_res, b.d_res, b.n * sizeof(double), cudaMemcpyDeviceToHost, c->st), "results");
    r = r ? r : c->cuda(cudaMemcpyAsync(b.h_st, b.d_st, b.n * sizeof(int32_t), cudaMemcpyDeviceToHost, c->st), "status");
  }
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "evaluation");
  if (r) return r;
  if (b.in_order) {
    if (result) memcpy(result, b.h_res, b.n * sizeof(double));
    if (status) memcpy(status, b.h_st, b.n * sizeof(int32_t));
  } else {
    for (int k = 0; k < b.n; k++) {
      if (result) result[b.order[k]] = b.h_res[k];
      if (status) status[b.order[k]] = b.h_st[k];
    }
  }
  // remember the format of the per-branch SW terms (nothing to do when this
  // batch was the last to set them: its precision is fixed)
  if (!b.dl_idx.empty() && b.dl_stamp != c->dl_stamp) {
    const uint8_t fmt = (b.prec != IMA_PREC_FP64);
    for (int k : b.dl_idx) c->dl_fast[k] = fmt;
    b.dl_stamp = ++c->dl_stamp;
  }
  return IMA_OK;
}

static void free_batch(Batch &b)
{
  if (b.graph) cudaGraphExecDestroy(b.graph);
  if (b.sgraph) cudaGraphExecDestroy(b.sgraph);
  cudaFree(b.d_req);
  cudaFree(b.d_res);
  cudaFree(b.d_items);
  cudaFree(b.d_acc);
  cudaFreeHost(b.h_res);
  cudaFreeHost(b.h_reqpin);
  if (b.req_ev) cudaEventDestroy(b.req_ev);
  b = Batch();
}

// The request list of ima_gpu_eval staged in c->evb (kept when a call
// repeats the previous arrays).
static int eval_prepare(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *u,
                        const double *kappa, const int32_t *edits, const int32_t *ai, int precision)
{
  Batch &b = c->evb;  // reused request buffers: no allocation per call
  // the same request list as the last call (the changet_RY1 pattern: new
  // genealogies, same chain-loci and rates) reuses the staged requests
  auto same = [&](const auto &v, const auto *p, size_t cnt) {
    return p ? (v.size() == cnt && memcmp(v.data(), p, cnt * sizeof(*p)) == 0) : v.empty();
  };
  ima_ctx::EvalKey &K = c->evkey;
  const bool hit = K.valid && K.n == n && K.prec == precision && n > 0 && same(K.ci, ci, n) &&
                   same(K.li, li, n) && same(K.u, u, n) && same(K.kappa, kappa, n) &&
                   same(K.edits, edits, 4 * (size_t)n) && same(K.ai, ai, n);
  int r = IMA_OK;
  if (!hit) {
    K.valid = false;
    r = build_batch(c, b, n, ci, li, u, kappa, edits, ai, precision);
    if (!r) {
      auto keep = [&](auto &v, const auto *p, size_t cnt) {
        if (p) v.assign(p, p + cnt);
        else v.clear();
      };
      keep(K.ci, ci, n);
      keep(K.li, li, n);
      keep(K.u, u, n);
      keep(K.kappa, kappa, n);
      keep(K.edits, edits, 4 * (size_t)n);
      keep(K.ai, ai, n);
      K.n = n;
      K.prec = precision;
      K.valid = true;
    }
  }
  return r;
}

extern "C" int ima_gpu_eval(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *u,
                            const double *kappa, const int32_t *edits, const int32_t *ai, int precision,
                            double *result, int32_t *status)
{
  if (!c) return IMA_ERR_ARG;
  Batch &b = c->evb;
  int r = eval_prepare(c, n, ci, li, u, kappa, edits, ai, precision);
  r = r ? r : flush(c);
  r = r ? r : (b.nis ? ensure_lengths(c) : IMA_OK);  // the infinite-sites likelihood reads them
  r = r ? r : init_sumlogk(c, b);
  if (!r) enqueue(c, b);
  r = r ? r : c->cuda(cudaGetLastError(), "launch");
  r = r ? r : fetch(c, b, result, status);
  return r;
}

// New times of every pair (topologies kept), then their full evaluation:
// the batched form of a re-timing move followed by the likelihoods of the
// moved genealogies.  Where the device reads the caller's memory in place,
// the times go straight from the caller's buffer into the evaluation's
// stream; the stream is synchronised before returning whatever happens.
extern "C" int ima_gpu_eval_times(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *time,
                                  const double *length, const double *u, const double *kappa, const int32_t *ai,
                                  int precision, double *result, int32_t *status)
{
  if (!c) return IMA_ERR_ARG;
  bool in_place = false;
  int r = upload_times(c, n, ci, li, time, length, true, &in_place);
  r = r ? r : ima_gpu_eval(c, n, ci, li, u, kappa, nullptr, ai, precision, result, status);
  // a successful evaluation has synchronised the stream already; a failed
  // one must not return while a kernel may still read the caller's buffers
  if (r && in_place) cudaStreamSynchronize(c->st);
  return r;
}

extern "C" int ima_gpu_batch_create(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const double *u,
                                    const double *kappa, const int32_t *edits, const int32_t *ai,
                                    int precision, int *batch)
{
  if (!c || !batch) return IMA_ERR_ARG;
  Batch b;
  int r = build_batch(c, b, n, ci, li, u, kappa, edits, ai, precision);
  if (r) {
    free_batch(b);
    return r;
  }
  b.live = true;
  for (size_t k = 0; k < c->batches.size(); k++)
    if (!c->batches[k].live) {
      c->batches[k] = b;
      *batch = (int)k;
      return IMA_OK;
    }
  c->batches.push_back(b);
  *batch = (int)c->batches.size() - 1;
  return IMA_OK;
}

extern "C" int ima_gpu_batch_run(ima_ctx *c, int batch, int use_graph)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  Batch &b = c->batches[batch];
  int r = flush(c);
  r = r ? r : (b.nis ? ensure_lengths(c) : IMA_OK);  // the infinite-sites likelihood reads them
  r = r ? r : init_sumlogk(c, b);
  if (r) return r;
  if (!use_graph || c->profiling) {
    enqueue(c, b);
    return c->cuda(cudaGetLastError(), "launch");
  }
  if (!b.graph) {
    cudaGraph_t g;
    r = c->cuda(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal), "capture");
    if (r) return r;
    long long before = c->launches;
    enqueue(c, b);
    long long nk = c->launches - before;
    r = c->cuda(cudaStreamEndCapture(c->st, &g), "capture end");
    if (r) return r;
    r = c->cuda(cudaGraphInstantiate(&b.graph, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    if (r) return r;
    c->launches -= nk;  // counted when replayed
  }
  r = c->cuda(cudaGraphLaunch(b.graph, c->st), "graph launch");
  c->launches += (b.nis ? 1 : 0) + (b.nhky ? 1 : 0) + (b.nsw ? 1 : 0);
  return r;
}

// Launch-shape autotuner: each variant of a kind's kernel runs `reps` times
// on the batch's own requests (after one untimed run); the fastest is kept
// unless the default is within 2% of it.  The kernels write only the fresh
// partial slots and the batch results, so the repeats leave no trace.
extern "C" int ima_gpu_batch_autotune(ima_ctx *c, int batch, int reps, int *hky_variant, int *sw_variant)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  Batch &b = c->batches[batch];
  int r = flush(c);
  r = r ? r : (b.nis ? ensure_lengths(c) : IMA_OK);  // the infinite-sites likelihood reads them
  r = r ? r : init_sumlogk(c, b);
  if (r) return r;
  if (reps < 1) reps = 1;
  if (b.prec != IMA_PREC_FP64 && (b.nhky || b.nsw)) {
    Pools P = c->pools();
    cudaStream_t st = c->st;
    cudaEvent_t e0 = c->ev(), e1 = c->ev();
    auto timed = [&](auto launch) -> float {
      launch();
      cudaEventRecord(e0, st);
      for (int k = 0; k < reps; k++) launch();
      cudaEventRecord(e1, st);
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) return -1.f;
      c->launches += reps + 1;
      return ms / reps;
    };
    auto pick = [&](int nvar, auto launch_v) -> int {
      std::vector<float> t(nvar);
      for (int v = 0; v < nvar; v++) t[v] = timed([&] { launch_v(v); });
      int best = 0;
      for (int v = 1; v < nvar; v++)
        if (t[v] >= 0.f && t[v] < t[best]) best = v;
      return (t[0] >= 0.f && t[0] <= 1.02f * t[best]) ? 0 : best;
    };
    if (b.nhky) {
      const ReqDev *rq = b.d_req + b.nis;
      b.hky_variant = pick(HKY_FAST_VARIANTS, [&](int v) {
        if (b.prec == IMA_PREC_FP32)
          launch_hky_fp32(P, rq, b.nhky, b.maxn_hky, b.maxs_hky, v, b.d_res + b.nis, b.d_st + b.nis, st);
        else
          launch_hky_fast(P, rq, b.nhky, b.maxn_hky, b.maxs_hky, v, b.d_res + b.nis, b.d_st + b.nis, st);
      });
    }
    if (b.nsw) {
      const ReqDev *rq = b.d_req + b.nis + b.nhky;
      const int off = b.nis + b.nhky;
      b.sw_variant = pick(SW_FAST_VARIANTS, [&](int v) {
        launch_sw_fast(P, rq, b.nsw, b.maxn_sw, v, b.d_res + off, b.d_st + off, st);
      });
    }
    c->event_pool.push_back(e0);
    c->event_pool.push_back(e1);
    r = c->cuda(cudaGetLastError(), "autotune");
    if (r) return r;
    if (b.sgraph) {
      cudaGraphExecDestroy(b.sgraph);
      b.sgraph = nullptr;
    }
    if (b.graph) {  // re-captured with the chosen shapes on the next run
      cudaStreamSynchronize(c->st);
      cudaGraphExecDestroy(b.graph);
      b.graph = nullptr;
    }
  }
  {
    ima_ctx::Tuned t;
    batch_shape(b, t.key);
    t.hky = b.hky_variant;
    t.sw = b.sw_variant;
    bool found = false;
    for (auto &u : c->tuned)
      if (!memcmp(u.key, t.key, sizeof(t.key))) {
        u = t;
        found = true;
      }
    if (!found) c->tuned.push_back(t);
    if (c->evb.live || c->evkey.valid) {  // the evaluation buffers take the choice if they hold this shape
      int k2[7];
      batch_shape(c->evb, k2);
      if (!memcmp(k2, t.key, sizeof(k2))) {
        c->evb.hky_variant = t.hky;
        c->evb.sw_variant = t.sw;
      }
    }
  }
  if (hky_variant) *hky_variant = b.hky_variant;
  if (sw_variant) *sw_variant = b.sw_variant;
  return IMA_OK;
}

extern "C" int ima_gpu_batch_set_variants(ima_ctx *c, int batch, int hky_variant, int sw_variant)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  if (hky_variant < 0 || hky_variant >= HKY_FAST_VARIANTS || sw_variant < 0 || sw_variant >= SW_FAST_VARIANTS)
    return c->fail(IMA_ERR_ARG, "launch variants out of range (%d, %d)", hky_variant, sw_variant);
  Batch &b = c->batches[batch];
  b.hky_variant = hky_variant;
  b.sw_variant = sw_variant;
  if (b.graph || b.sgraph) cudaStreamSynchronize(c->st);
  if (b.graph) {
    cudaGraphExecDestroy(b.graph);
    b.graph = nullptr;
  }
  if (b.sgraph) {
    cudaGraphExecDestroy(b.sgraph);
    b.sgraph = nullptr;
  }
  return IMA_OK;
}

// the swap sweep of every run on the committed sums, Philox stream
static void enqueue_swap(ima_ctx *c, int swaptries, int include_probg, uint64_t seed)
{
  SwapArgs a{};
  a.nruns = c->nruns;
  a.cpr = c->cpr;
  a.nloci = c->nloci;
  a.swaptries = swaptries;
  a.include_probg = include_probg;
  a.stride = 1;
  a.pdg = c->d_pdg;
  a.probg = c->d_probg;
  a.beta = c->d_beta;
  a.allbetas = c->d_allbetas;
  a.uniforms = nullptr;
  a.seed = seed;
  a.counter = c->d_ctr;
  a.used = c->d_used;
  a.swap0ok = c->d_swap0ok;
  a.swapcount = c->d_swapcount;
  a.tempcount = c->d_tempcount;
  a.S = c->d_S;
  c->launch(IMA_K_SWAP, (double)c->nitems * 8.0, [&] { launch_swap(a, c->st); });
}

// One MC3 sweep of a batch: every request evaluated, the accepted ones
// committed (partial likelihoods and pdg), then the swap attempts of every
// run on the committed sums -- every kernel of the sweep in one graph launch
// when use_graph is set (captured on the first call, kept while swaptries,
// include_probg and seed are unchanged; the Philox counters advance on the
// device, so each replay draws new uniforms).
extern "C" int ima_gpu_batch_sweep(ima_ctx *c, int batch, const uint8_t *accept, int swaptries, int include_probg,
                                   uint64_t seed, int use_graph)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  if (swaptries < 0) return c->fail(IMA_ERR_ARG, "swaptries must be >= 0");
  Batch &b = c->batches[batch];
  int r = flush(c);
  r = r ? r : (b.nis ? ensure_lengths(c) : IMA_OK);  // the infinite-sites likelihood reads them
  r = r ? r : init_sumlogk(c, b);
  if (r) return r;
  if (!b.d_items) {
    std::vector<int32_t> items(b.n);
    for (int k = 0; k < b.n; k++) items[k] = b.h_req[k].item;
    b.d_items = dev_alloc<int32_t>(b.n, c->dev_bytes, c->st);
    b.d_acc = dev_alloc<uint8_t>(b.n, c->dev_bytes, c->st);
    if (!b.d_items || !b.d_acc) return c->fail(IMA_ERR_NOMEM, "sweep buffers");
    r = c->cuda(cudaMemcpyAsync(b.d_items, items.data(), b.n * 4, cudaMemcpyHostToDevice, c->st), "sweep items");
    r = r ? r : c->cuda(cudaMemsetAsync(b.d_acc, 1, b.n, c->st), "sweep mask");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "sweep items");
    if (r) return r;
  }
  if (accept) {  // caller order -> the batch's grouped order
    std::vector<uint8_t> acc(b.n);
    for (int k = 0; k < b.n; k++) acc[k] = accept[b.order[k]];
    r = c->cuda(cudaMemcpyAsync(b.d_acc, acc.data(), b.n, cudaMemcpyHostToDevice, c->st), "sweep mask");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "sweep mask");
    if (r) return r;
  }
  const bool swap = c->cpr >= 2;
  auto body = [&] {
    enqueue(c, b);
    Pools P = c->pools();
    launch_hky_commit(P, b.d_items, b.d_acc, b.n, c->st);
    launch_pdg_commit(b.d_items, b.d_acc, c->d_pdg_new, c->d_pdg, b.n, c->st);
    c->launches += 2;
    if (swap) enqueue_swap(c, swaptries, include_probg, seed);
  };
  const int nk = (b.nis ? 1 : 0) + (b.nhky ? 1 : 0) + (b.nsw ? 1 : 0) + 2 + (swap ? 1 : 0);
  if (!use_graph || c->profiling) {
    body();
    return c->cuda(cudaGetLastError(), "sweep");
  }
  if (b.sgraph && (b.s_tries != swaptries || b.s_probg != include_probg || b.s_seed != seed)) {
    cudaStreamSynchronize(c->st);
    cudaGraphExecDestroy(b.sgraph);
    b.sgraph = nullptr;
  }
  if (!b.sgraph) {
    cudaGraph_t g;
    r = c->cuda(cudaStreamBeginCapture(c->st, cudaStreamCaptureModeThreadLocal), "capture");
    if (r) return r;
    const long long before = c->launches;
    body();
    c->launches = before;  // counted when replayed
    r = c->cuda(cudaStreamEndCapture(c->st, &g), "capture end");
    if (r) return r;
    r = c->cuda(cudaGraphInstantiate(&b.sgraph, g, 0), "graph instantiate");
    cudaGraphDestroy(g);
    if (r) return r;
    b.s_tries = swaptries;
    b.s_probg = include_probg;
    b.s_seed = seed;
  }
  r = c->cuda(cudaGraphLaunch(b.sgraph, c->st), "graph launch");
  c->launches += nk;
  c->graph_launches++;
  return r;
}

extern "C" int ima_gpu_batch_results(ima_ctx *c, int batch, double *result, int32_t *status)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  return fetch(c, c->batches[batch], result, status);
}

extern "C" int ima_gpu_batch_destroy(ima_ctx *c, int batch)
{
  if (!c || batch < 0 || batch >= (int)c->batches.size() || !c->batches[batch].live) return IMA_ERR_ARG;
  cudaStreamSynchronize(c->st);
  free_batch(c->batches[batch]);
  return IMA_OK;
}

// ======================================================================
// commit / revert
static int commit(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const uint8_t *accept,
                  bool partials, bool pdg)
{
  if (!c || n < 1 || !ci || !li || !accept) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  std::vector<int32_t> items(n);
  for (int k = 0; k < n; k++) {
    if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci[k], li[k]);
    items[k] = c->item_of(ci[k], li[k]);
  }
  if ((size_t)n > c->ccap) {
    cudaStreamSynchronize(c->st);
    cudaFree(c->d_citems);
    cudaFree(c->d_cacc);
    c->d_citems = dev_alloc<int32_t>(n, c->dev_bytes, c->st);
    c->d_cacc = dev_alloc<uint8_t>(n, c->dev_bytes, c->st);
    if (!c->d_citems || !c->d_cacc) return c->fail(IMA_ERR_NOMEM, "commit buffers");
    c->ccap = n;
  }
  int r = c->cuda(cudaMemcpyAsync(c->d_citems, items.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, c->st), "commit");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_cacc, accept, n, cudaMemcpyHostToDevice, c->st), "commit");
  if (r) return r;
  Pools P = c->pools();
  if (partials && c->d_slot64) launch_hky_commit(P, c->d_citems, c->d_cacc, n, c->st), c->launches++;
  if (pdg) launch_pdg_commit(c->d_citems, c->d_cacc, c->d_pdg_new, c->d_pdg, n, c->st), c->launches++;
  r = c->cuda(cudaGetLastError(), "commit launch");
  // the host arrays are stack-owned: wait for the copies
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "commit");
}

extern "C" int ima_gpu_commit(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const uint8_t *accept)
{
  return commit(c, n, ci, li, accept, true, true);
}

// ======================================================================
// per-call reference mirrors
extern "C" int ima_gpu_likelihoodIS(ima_ctx *c, int ci, int li, double mutrate, double *result)
{
  if (!c || !result) return IMA_ERR_ARG;
  if (!c->valid(ci, li) || c->loci[li].d.model != IMA_MODEL_IS) return c->fail(IMA_ERR_ARG, "locus %d is not infinite-sites", li);
  int32_t st = 0;
  int r = ima_gpu_eval(c, 1, &ci, &li, &mutrate, nullptr, nullptr, nullptr, IMA_PREC_FP64, result, &st);
  if (r) return r;
  if (st == IMA_EVAL_IS_FAIL) return c->fail(IMA_ERR_DATA, "Data incompatible with current genealogy, likelihood calculation failed, chain %d, locus %d", ci, li);
  return IMA_OK;
}

extern "C" int ima_gpu_likelihoodHKY(ima_ctx *c, int ci, int li, double mutrate, double kappa,
                                     int e1, int e2, int e3, int e4, double *result)
{
  if (!c || !result) return IMA_ERR_ARG;
  if (!c->valid(ci, li) || c->loci[li].d.model != IMA_MODEL_HKY) return c->fail(IMA_ERR_ARG, "locus %d is not HKY", li);
  int32_t e[4] = {e1, e2, e3, e4};
  return ima_gpu_eval(c, 1, &ci, &li, &mutrate, &kappa, e, nullptr, IMA_PREC_FAST, result, nullptr);
}

extern "C" int ima_gpu_copyfraclike(ima_ctx *c, int ci, int li)
{
  uint8_t a = 1;
  return commit(c, 1, &ci, &li, &a, true, false);
}

extern "C" int ima_gpu_storescalefactors(ima_ctx *c, int ci, int li)
{
  // scale factors travel with their partial likelihoods: committed by copyfraclike
  if (!c) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  return IMA_OK;
}

extern "C" int ima_gpu_restorescalefactors(ima_ctx *c, int ci, int li)
{
  uint8_t a = 0;
  return commit(c, 1, &ci, &li, &a, true, false);
}

extern "C" int ima_gpu_likelihoodSW(ima_ctx *c, int ci, int li, int ai, double u, double tr, double *result)
{
  if (!c || !result) return IMA_ERR_ARG;
  if (!c->valid(ci, li) || c->loci[li].d.model != IMA_MODEL_SW) return c->fail(IMA_ERR_ARG, "locus %d is not stepwise", li);
  return ima_gpu_eval(c, 1, &ci, &li, &u, &tr, nullptr, &ai, IMA_PREC_FAST, result, nullptr);
}

extern "C" int ima_gpu_get_dlikeA(ima_ctx *c, int ci, int li, int ai, double *dlikeA)
{
  if (!c || !dlikeA) return IMA_ERR_ARG;
  if (!c->valid(ci, li) || c->loci[li].d.model != IMA_MODEL_SW) return c->fail(IMA_ERR_ARG, "locus %d is not stepwise", li);
  const ItemDev &it = c->items[c->item_of(ci, li)];
  if (ai < 0 || ai >= c->loci[li].d.nlinked) return c->fail(IMA_ERR_ARG, "bad marker");
  int nl = 2 * it.n - 1;
  std::vector<double> raw(nl);
  int r = c->cuda(cudaMemcpyAsync(raw.data(), c->d_dlike + it.dl_off + (size_t)ai * nl, nl * sizeof(double), cudaMemcpyDeviceToHost, c->st), "dlikeA");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "dlikeA");
  if (r) return r;
  bool ffmt = c->dl_fast[it.al_off + (size_t)ai];
  for (int k = 0; k < nl; k++) {
    if (ffmt) {
      float2 v;
      memcpy(&v, &raw[k], sizeof(v));
      dlikeA[k] = std::isinf(v.x) ? -1e100 : (double)v.x + (double)v.y;
    } else {
      dlikeA[k] = raw[k];
    }
  }
  return IMA_OK;
}

// ======================================================================
// MC3
extern "C" int ima_gpu_setheat(ima_ctx *c, double h1, double h2, int heatmode)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (heatmode < 0 || heatmode > 2) return c->fail(IMA_ERR_ARG, "heatmode must be 0, 1 or 2");
  const int N = c->cpr;
  std::vector<double> beta(c->nchains), allb(c->nchains);
  for (int r = 0; r < c->nruns; r++)
    for (int i = 0; i < N; i++) {
      double a, b;
      if (N == 1) {
        a = b = 1.0;
      } else if (heatmode == 0) {
        a = 1.0 / (1.0 + h1 * i);
        b = 1.0 / (1.0 + (h1 < 0.05 ? 0.05 : h1) * i);
      } else if (heatmode == 1) {
        a = b = 1 - (1 - h2) * (i) * std::pow(h1, (double)(N - 1 - i)) / (double)(N - 1);
      } else {
        a = b = 1.0 - i * (1.0 / (N - 1));
      }
      if (N > 1 && (b <= 0.0 || b > 1.0))
        return c->fail(IMA_ERR_ARG, "command line heating terms have caused a heating value out of range. chain %d beta %f", i, b);
      allb[(size_t)r * N + i] = a;
      beta[(size_t)r * N + i] = b;
    }
  int rr = c->cuda(cudaMemcpyAsync(c->d_beta, beta.data(), beta.size() * 8, cudaMemcpyHostToDevice, c->st), "beta");
  rr = rr ? rr : c->cuda(cudaMemcpyAsync(c->d_allbetas, allb.data(), allb.size() * 8, cudaMemcpyHostToDevice, c->st), "allbetas");
  return rr ? rr : c->cuda(cudaStreamSynchronize(c->st), "setheat");
}

static int copy_dev(ima_ctx *c, void *dst, const void *src, size_t bytes, cudaMemcpyKind k, const char *what)
{
  if (!c || !src || !dst) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  int r = c->cuda(cudaMemcpyAsync(dst, src, bytes, k, c->st), what);
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), what);
}

extern "C" int ima_gpu_get_betas(ima_ctx *c, double *beta)
{
  return copy_dev(c, beta, c ? c->d_beta : nullptr, c ? c->nchains * 8 : 0, cudaMemcpyDeviceToHost, "betas");
}
extern "C" int ima_gpu_set_betas(ima_ctx *c, const double *beta)
{
  return copy_dev(c, c ? c->d_beta : nullptr, beta, c ? c->nchains * 8 : 0, cudaMemcpyHostToDevice, "betas");
}
extern "C" int ima_gpu_set_allbetas(ima_ctx *c, const double *allbetas)
{
  return copy_dev(c, c ? c->d_allbetas : nullptr, allbetas, c ? c->nchains * 8 : 0, cudaMemcpyHostToDevice,
                  "heat ladder");
}
extern "C" int ima_gpu_set_pdg(ima_ctx *c, const double *pdg)
{
  return copy_dev(c, c ? c->d_pdg : nullptr, pdg, c ? (size_t)c->nitems * 8 : 0, cudaMemcpyHostToDevice, "pdg");
}
extern "C" int ima_gpu_get_pdg(ima_ctx *c, double *pdg)
{
  return copy_dev(c, pdg, c ? c->d_pdg : nullptr, c ? (size_t)c->nitems * 8 : 0, cudaMemcpyDeviceToHost, "pdg");
}
extern "C" int ima_gpu_set_probg(ima_ctx *c, const double *probg)
{
  return copy_dev(c, c ? c->d_probg : nullptr, probg, c ? c->nchains * 8 : 0, cudaMemcpyHostToDevice, "probg");
}
extern "C" int ima_gpu_get_probg(ima_ctx *c, double *probg)
{
  return copy_dev(c, probg, c ? c->d_probg : nullptr, c ? c->nchains * 8 : 0, cudaMemcpyDeviceToHost, "probg");
}

extern "C" int ima_gpu_swapchains(ima_ctx *c, int swaptries, int include_probg, const double *uniforms,
                                  int stride, uint64_t seed, int32_t *used, int32_t *swap0ok)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (swaptries < 0) return c->fail(IMA_ERR_ARG, "swaptries must be >= 0");
  if (c->cpr < 2) return IMA_OK;  // the reference swaps only when numchains > 1
  int r = IMA_OK;
  if (uniforms) {
    if (stride < 1) return c->fail(IMA_ERR_ARG, "stride must be >= 1");
    size_t need = (size_t)stride * c->nruns;
    if (need > c->uni_cap) {
      cudaStreamSynchronize(c->st);
      cudaFree(c->d_uni);
      c->d_uni = dev_alloc<double>(need, c->dev_bytes, c->st);
      if (!c->d_uni) return c->fail(IMA_ERR_NOMEM, "uniform buffer");
      c->uni_cap = need;
    }
    r = c->cuda(cudaMemcpyAsync(c->d_uni, uniforms, need * 8, cudaMemcpyHostToDevice, c->st), "uniforms");
    if (r) return r;
  }
  SwapArgs a;
  a.nruns = c->nruns;
  a.cpr = c->cpr;
  a.nloci = c->nloci;
  a.swaptries = swaptries;
  a.include_probg = include_probg;
  a.stride = stride;
  a.pdg = c->d_pdg;
  a.probg = c->d_probg;
  a.beta = c->d_beta;
  a.allbetas = c->d_allbetas;
  a.uniforms = uniforms ? c->d_uni : nullptr;
  a.seed = seed;
  a.counter = c->d_ctr;
  a.used = c->d_used;
  a.swap0ok = c->d_swap0ok;
  a.swapcount = c->d_swapcount;
  a.tempcount = c->d_tempcount;
  a.S = c->d_S;
  c->launch(IMA_K_SWAP, (double)c->nitems * 8.0, [&] { launch_swap(a, c->st); });
  r = c->cuda(cudaGetLastError(), "swap launch");
  if (r) return r;
  if (used) r = r ? r : c->cuda(cudaMemcpyAsync(used, c->d_used, c->nruns * 4, cudaMemcpyDeviceToHost, c->st), "used");
  if (swap0ok) r = r ? r : c->cuda(cudaMemcpyAsync(swap0ok, c->d_swap0ok, c->nruns * 4, cudaMemcpyDeviceToHost, c->st), "swap0ok");
  if (used || swap0ok || uniforms) r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "swap");
  if (!r && used)
    for (int k = 0; k < c->nruns; k++)
      if (used[k] < 0) return c->fail(IMA_ERR_ARG, "run %d ran out of supplied uniforms", k);
  return r;
}

// The swap attempts with the caller's generator drawn one uniform at a time:
// the per-chain sums S (every locus, the expensive part) come from the
// device; the attempts, which the reference interleaves with single draws of
// its one generator stream (swapchains.cpp:549-605), run here in the order
// k_swap makes them, so a caller whose generator cannot be drawn ahead
// consumes exactly the reference's draws.
extern "C" int ima_gpu_swapchains_cb(ima_ctx *c, int swaptries, int include_probg, double (*uniform)(void *),
                                     void *arg, int32_t *used, int32_t *swap0ok)
{
  if (!c || !uniform) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  if (swaptries < 0) return c->fail(IMA_ERR_ARG, "swaptries must be >= 0");
  if (c->cpr < 2) return IMA_OK;
  SwapArgs a{};
  a.nruns = c->nruns;
  a.cpr = c->cpr;
  a.nloci = c->nloci;
  a.swaptries = 0;  // sums only
  a.include_probg = include_probg;
  a.stride = 1;
  a.pdg = c->d_pdg;
  a.probg = c->d_probg;
  a.beta = c->d_beta;
  a.allbetas = c->d_allbetas;
  a.uniforms = nullptr;
  a.counter = nullptr;
  a.used = nullptr;
  a.swap0ok = nullptr;
  a.swapcount = c->d_swapcount;
  a.tempcount = c->d_tempcount;
  a.S = c->d_S;
  c->launch(IMA_K_SWAP, (double)c->nitems * 8.0, [&] { launch_swap(a, c->st); });
  const int n = c->cpr;
  const size_t nn = (size_t)n * n, N = (size_t)c->nchains;
  std::vector<double> S(N), beta(N), allb(N);
  std::vector<int32_t> sc(nn * c->nruns), tc(nn * c->nruns);
  int r = c->cuda(cudaGetLastError(), "swap sums");
  r = r ? r : c->cuda(cudaMemcpyAsync(S.data(), c->d_S, N * 8, cudaMemcpyDeviceToHost, c->st), "sums");
  r = r ? r : c->cuda(cudaMemcpyAsync(beta.data(), c->d_beta, N * 8, cudaMemcpyDeviceToHost, c->st), "betas");
  r = r ? r : c->cuda(cudaMemcpyAsync(allb.data(), c->d_allbetas, N * 8, cudaMemcpyDeviceToHost, c->st), "betas");
  r = r ? r : c->cuda(cudaMemcpyAsync(sc.data(), c->d_swapcount, sc.size() * 4, cudaMemcpyDeviceToHost, c->st), "counts");
  r = r ? r : c->cuda(cudaMemcpyAsync(tc.data(), c->d_tempcount, tc.size() * 4, cudaMemcpyDeviceToHost, c->st), "counts");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "swap sums");
  if (r) return r;
  constexpr int SWAPDIST = 7;
  for (int run = 0; run < c->nruns; run++) {
    double *b = beta.data() + (size_t)run * n;
    const double *ab = allb.data() + (size_t)run * n, *Sr = S.data() + (size_t)run * n;
    int32_t *scr = sc.data() + run * nn, *tcr = tc.data() + run * nn;
    int k = 0, ok0 = 0;
    auto draw = [&] {
      k++;
      return uniform(arg);
    };
    auto rank_of = [&](double v) {
      for (int q = 0; q < n; q++)
        if (ab[q] == v) return q;
      return -1;
    };
    for (int t = 0; t < swaptries; t++) {
      int ci, cj, cjmin, cjrange;
      do { ci = (int)(draw() * n); } while (ci < 0 || ci >= n);
      if (n < 2 * SWAPDIST + 3) {
        cjmin = 0;
        cjrange = n;
      } else {
        cjmin = std::max(0, ci - SWAPDIST);
        cjrange = std::min(n, ci + SWAPDIST) - cjmin;
      }
      do { cj = cjmin + (int)(draw() * cjrange); } while (cj == ci || cj < 0 || cj >= n);
      const int p = rank_of(b[ci]), q = rank_of(b[cj]);
      const int hi = std::max(ci, cj), lo = std::min(ci, cj), phi = std::max(p, q), plo = std::min(p, q);
      if (p >= 0 && q >= 0) tcr[(size_t)phi * n + plo]++;
      scr[(size_t)hi * n + lo]++;
      const double w = exp((b[ci] - b[cj]) * (Sr[cj] - Sr[ci]));
      if (w >= 1.0 || w > draw()) {
        std::swap(b[ci], b[cj]);
        scr[(size_t)lo * n + hi]++;
        if (p >= 0 && q >= 0) tcr[(size_t)plo * n + phi]++;
        if (ci == 0 || cj == 0) ok0 = 1;
      }
    }
    if (used) used[run] = k;
    if (swap0ok) swap0ok[run] = ok0;
  }
  r = c->cuda(cudaMemcpyAsync(c->d_beta, beta.data(), N * 8, cudaMemcpyHostToDevice, c->st), "betas");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_swapcount, sc.data(), sc.size() * 4, cudaMemcpyHostToDevice, c->st), "counts");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_tempcount, tc.data(), tc.size() * 4, cudaMemcpyHostToDevice, c->st), "counts");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "swap");
}

extern "C" int ima_gpu_surface_retaken(ima_ctx *c, int *n)
{
  if (!c || !n) return IMA_ERR_ARG;
  *n = c->surf_retaken;
  return IMA_OK;
}

extern "C" int ima_gpu_get_swapcounts(ima_ctx *c, int run, int32_t *swapcount, int32_t *tempcount)
{
  if (!c || run < 0 || run >= c->nruns) return IMA_ERR_ARG;
  size_t nn = (size_t)c->cpr * c->cpr;
  int r = IMA_OK;
  if (swapcount) r = c->cuda(cudaMemcpyAsync(swapcount, c->d_swapcount + run * nn, nn * 4, cudaMemcpyDeviceToHost, c->st), "swapcount");
  if (tempcount) r = r ? r : c->cuda(cudaMemcpyAsync(tempcount, c->d_tempcount + run * nn, nn * 4, cudaMemcpyDeviceToHost, c->st), "tempcount");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "swapcounts");
}

// ======================================================================
// surface
extern "C" int ima_gpu_surface_load(ima_ctx *c, int G, int rowlen, const float *rows, int np, int nm,
                                    int npops, const double *lognorm)
{
  if (!c || !rows) return IMA_ERR_ARG;
  if (G < 1 || np < 0 || nm < 0 || np + nm < 1 || np + nm > 32 || rowlen < 4 * np + 3 * nm + 2 || rowlen > 64)
    return c->fail(IMA_ERR_ARG, "bad surface shape (G %d, rowlen %d, %d theta, %d m)", G, rowlen, np, nm);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->st);
  cudaFree(c->d_rows);
  cudaFree(c->d_lognorm);
  c->d_lognorm = nullptr;
  c->d_rows = dev_alloc<float>((size_t)G * rowlen, c->dev_bytes, c->st);
  if (!c->d_rows) return c->fail(IMA_ERR_NOMEM, "surface rows");
  if (lognorm) {
    c->d_lognorm = dev_alloc<double>(G, c->dev_bytes, c->st);
    if (!c->d_lognorm) return c->fail(IMA_ERR_NOMEM, "surface normalisers");
  }
  c->srows_state = 0;
  c->s_cap = (size_t)G;
  c->sG = G;
  c->srowlen = rowlen;
  c->snp = np;
  c->snm = nm;
  c->snpops = npops;
  int r = c->cuda(cudaMemcpyAsync(c->d_rows, rows, (size_t)G * rowlen * 4, cudaMemcpyHostToDevice, c->st), "rows");
  if (lognorm) r = r ? r : c->cuda(cudaMemcpyAsync(c->d_lognorm, lognorm, (size_t)G * 8, cudaMemcpyHostToDevice, c->st), "lognorm");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "surface load");
}

extern "C" int ima_gpu_surface_info(ima_ctx *c, int *G, int *np, int *nm, int *npops)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  if (G) *G = c->sG;
  if (np) *np = c->snp;
  if (nm) *nm = c->snm;
  if (npops) *npops = c->snpops;
  return IMA_OK;
}

// ---------------------------------------------------------- 1-D marginals
// genealogies [lo, hi) summed and divided by div; raw_cc as marginp reads cc
struct GRange {
  int lo, hi;
  double div;
  int raw_cc;
};

static int margin_run(ima_ctx *c, int n, const int32_t *param, const double *x, double yadjust, int logi,
                      const double *expo_mean, double *out, const GRange *rg = nullptr)
{
  const int npar = c->snp + c->snm;
  for (int k = 0; k < n; k++) {
    if (param[k] < 0 || param[k] >= npar) return c->fail(IMA_ERR_ARG, "point %d: parameter %d out of range", k, param[k]);
    if (!(x[k] > 0.0) && !(rg && x[k] >= 0.0)) return c->fail(IMA_ERR_ARG, "point %d: x must be > 0", k);
  }
  if (expo_mean)
    for (int i = 0; i < c->snm; i++)
      if (!(expo_mean[i] > 0.0)) return c->fail(IMA_ERR_ARG, "exponential prior mean %d must be > 0", i);
  const int nchunks = margin_chunks(rg ? rg->hi - rg->lo : c->sG, n);
  // one device block: param | x | means | out | partials
  const size_t bytes = 256 * 5 + (size_t)n * 4 + (size_t)n * 8 + 64 * 8 + (size_t)n * 8 + (size_t)n * nchunks * 8;
  if (bytes > c->mscratch_cap) {
    cudaFree(c->d_mscratch);
    c->d_mscratch = dev_alloc<char>(bytes, c->dev_bytes, c->st);
    if (!c->d_mscratch) return c->fail(IMA_ERR_NOMEM, "marginal scratch (%zu bytes)", bytes);
    c->mscratch_cap = bytes;
  }
  char *p = static_cast<char *>(c->d_mscratch);
  auto take = [&](size_t b) {
    char *q = p;
    p += (b + 255) / 256 * 256;
    return q;
  };
  int32_t *d_param = reinterpret_cast<int32_t *>(take((size_t)n * 4));
  double *d_x = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_mean = reinterpret_cast<double *>(take(64 * 8));
  double *d_out = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_part = reinterpret_cast<double *>(take((size_t)n * nchunks * 8));
  MarginArgs a{};
  a.G = c->sG;
  a.g_lo = rg ? rg->lo : 0;
  a.g_hi = rg ? rg->hi : c->sG;
  a.div = rg ? rg->div : c->sG;
  a.raw_cc = rg ? rg->raw_cc : 0;
  a.rowlen = c->srowlen;
  a.np = c->snp;
  a.nm = c->snm;
  a.n = n;
  a.logi = logi;
  a.yadjust = yadjust;
  a.ccp = 0;  // gsampinf layout (initialize.cpp:709-718)
  a.fcp = a.ccp + a.np;
  a.hccp = a.fcp + a.np;
  a.mcp = a.hccp + a.np;
  a.fmp = a.mcp + a.nm;
  a.qip = a.fmp + a.nm;
  a.mip = a.qip + a.np;
  a.rows = c->d_rows;
  a.param = d_param;
  a.x = d_x;
  a.expo_mean = expo_mean ? d_mean : nullptr;
  int r = c->cuda(cudaMemcpyAsync(d_param, param, (size_t)n * 4, cudaMemcpyHostToDevice, c->st), "marginal points");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_x, x, (size_t)n * 8, cudaMemcpyHostToDevice, c->st), "marginal points");
  if (expo_mean) r = r ? r : c->cuda(cudaMemcpyAsync(d_mean, expo_mean, (size_t)c->snm * 8, cudaMemcpyHostToDevice, c->st), "means");
  if (r) return r;
  int lr = 0;
  c->launch(IMA_K_MARGIN, (double)c->sG * c->srowlen * 4, [&] { lr = launch_margin(a, d_part, nchunks, d_out, c->st); });
  c->launches += 1;  // pass + merge
  if (lr) return c->fail(IMA_ERR_ARG, "marginal: unsupported shape (%d)", lr);
  r = c->cuda(cudaGetLastError(), "marginal launch");
  r = r ? r : c->cuda(cudaMemcpyAsync(out, d_out, (size_t)n * 8, cudaMemcpyDeviceToHost, c->st), "marginal values");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "marginal");
}

static int ensure_logfact(ima_ctx *c);
constexpr double EXPOMIGPLOTSCALE = 20;  // the 2NM plot scale in prior means (imamp.hpp:156)

// calc_popmig / calc_pop_expomig at n points (term k: thetai[k], mi[k], x[k])
static int popmig_run(ima_ctx *c, int n, const int32_t *thetai, const int32_t *mi, const double *x,
                      const double *theta_max, const double *mig_max, const double *mig_mean, int prob_or_like,
                      double *out, const GRange *rg = nullptr)
{
  for (int k = 0; k < n; k++) {
    if (thetai[k] < 0 || thetai[k] >= c->snp || mi[k] < 0 || mi[k] >= c->snm)
      return c->fail(IMA_ERR_ARG, "point %d: term (%d, %d) out of range", k, thetai[k], mi[k]);
    if (!(x[k] > 0.0) && !(rg && x[k] >= 0.0)) return c->fail(IMA_ERR_ARG, "point %d: x must be > 0", k);
  }
  for (int i = 0; i < c->snp; i++)
    if (!(theta_max[i] > 0.0)) return c->fail(IMA_ERR_ARG, "theta prior maximum %d must be > 0", i);
  for (int i = 0; i < c->snm; i++) {
    if (!(mig_max[i] > 0.0)) return c->fail(IMA_ERR_ARG, "migration prior maximum %d must be > 0", i);
    if (mig_mean && !(mig_mean[i] > 0.0)) return c->fail(IMA_ERR_ARG, "exponential prior mean %d must be > 0", i);
  }
  if (int r0 = ensure_logfact(c)) return r0;
  const int nchunks = popmig_chunks(rg ? rg->hi - rg->lo : c->sG, n);
  std::vector<double> hq(n), hm(n), hmean(mig_mean ? n : 0);
  for (int k = 0; k < n; k++) {
    hq[k] = theta_max[thetai[k]];
    hm[k] = mig_max[mi[k]];
    if (mig_mean) hmean[k] = mig_mean[mi[k]];
  }
  // one device block: thetai | mi | x | qmax | mmax | mmean | out | error | partials
  const size_t bytes = 256 * 9 + (size_t)n * (4 + 4 + 8 * 5) + 8 + (size_t)n * nchunks * 16;
  if (bytes > c->mscratch_cap) {
    cudaFree(c->d_mscratch);
    c->d_mscratch = dev_alloc<char>(bytes, c->dev_bytes, c->st);
    if (!c->d_mscratch) {
      c->mscratch_cap = 0;
      return c->fail(IMA_ERR_NOMEM, "2NM scratch (%zu bytes)", bytes);
    }
    c->mscratch_cap = bytes;
  }
  char *p = static_cast<char *>(c->d_mscratch);
  auto take = [&](size_t b) {
    char *q = p;
    p += (b + 255) / 256 * 256;
    return q;
  };
  int32_t *d_th = reinterpret_cast<int32_t *>(take((size_t)n * 4));
  int32_t *d_mi = reinterpret_cast<int32_t *>(take((size_t)n * 4));
  double *d_x = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_q = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_m = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_mean = reinterpret_cast<double *>(take((size_t)n * 8));
  double *d_out = reinterpret_cast<double *>(take((size_t)n * 8));
  int32_t *d_err = reinterpret_cast<int32_t *>(take(8));
  double *d_part = reinterpret_cast<double *>(take((size_t)n * nchunks * 16));
  PopmigArgs a{};
  a.G = c->sG;
  a.g_lo = rg ? rg->lo : 0;
  a.g_hi = rg ? rg->hi : c->sG;
  a.div = rg ? rg->div : c->sG;
  a.rowlen = c->srowlen;
  a.n = n;
  a.expo = mig_mean ? 1 : 0;
  a.prob_or_like = prob_or_like ? 1 : 0;
  a.ccp = 0;  // gsampinf layout (initialize.cpp:709-718)
  a.fcp = a.ccp + c->snp;
  a.hccp = a.fcp + c->snp;
  a.mcp = a.hccp + c->snp;
  a.fmp = a.mcp + c->snm;
  a.qip = a.fmp + c->snm;
  a.mip = a.qip + c->snp;
  a.rows = c->d_rows;
  a.thetai = d_th;
  a.mi = d_mi;
  a.x = d_x;
  a.qmax = d_q;
  a.mmax = d_m;
  a.mmean = mig_mean ? d_mean : nullptr;
  a.logfact = c->d_logfact;
  a.err = d_err;
  int r = c->cuda(cudaMemcpyAsync(d_th, thetai, (size_t)n * 4, cudaMemcpyHostToDevice, c->st), "2NM points");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_mi, mi, (size_t)n * 4, cudaMemcpyHostToDevice, c->st), "2NM points");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_x, x, (size_t)n * 8, cudaMemcpyHostToDevice, c->st), "2NM points");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_q, hq.data(), (size_t)n * 8, cudaMemcpyHostToDevice, c->st), "2NM priors");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_m, hm.data(), (size_t)n * 8, cudaMemcpyHostToDevice, c->st), "2NM priors");
  if (mig_mean) r = r ? r : c->cuda(cudaMemcpyAsync(d_mean, hmean.data(), (size_t)n * 8, cudaMemcpyHostToDevice, c->st), "2NM priors");
  r = r ? r : c->cuda(cudaMemsetAsync(d_err, 0, 4, c->st), "2NM status");
  if (r) return r;
  int lr = 0;
  c->launch(IMA_K_POPMIG, (double)c->sG * c->srowlen * 4, [&] { lr = launch_popmig(a, d_part, nchunks, d_out, c->st); });
  c->launches += 1;  // pass + merge
  if (lr) return c->fail(IMA_ERR_ARG, "2NM densities: unsupported shape (%d)", lr);
  int32_t err = 0;
  r = c->cuda(cudaGetLastError(), "2NM launch");
  r = r ? r : c->cuda(cudaMemcpyAsync(out, d_out, (size_t)n * 8, cudaMemcpyDeviceToHost, c->st), "2NM values");
  r = r ? r : c->cuda(cudaMemcpyAsync(&err, d_err, 4, cudaMemcpyDeviceToHost, c->st), "2NM status");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "2NM");
  if (!r && err)
    return c->fail(IMA_ERR_DATA, "2NM density: %s", err == 5 ? "a count beyond the logfact table"
                                                             : "an incomplete gamma series or fraction did not converge");
  return r;
}

extern "C" int ima_gpu_popmig(ima_ctx *c, int n, const int32_t *thetai, const int32_t *mi, const double *x,
                              const double *theta_max, const double *mig_max, const double *mig_mean,
                              int prob_or_like, double *y)
{
  if (!c || n < 1 || !thetai || !mi || !x || !theta_max || !mig_max || !y) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  if (c->snm < 1) return c->fail(IMA_ERR_STATE, "the loaded surface has no migration parameters");
  cudaSetDevice(c->device);
  return popmig_run(c, n, thetai, mi, x, theta_max, mig_max, mig_mean, prob_or_like, y);
}

extern "C" int ima_gpu_popmig_curves(ima_ctx *c, int nterms, const int32_t *thetai, const int32_t *mi, int gridsize,
                                     const double *theta_max, const double *mig_max, const double *mig_mean,
                                     int prob_or_like, double *x_out, double *y_out, double *maxx)
{
  if (!c || nterms < 1 || !thetai || !mi || gridsize < 1 || !theta_max || !mig_max || !x_out || !y_out)
    return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  if (c->snm < 1) return c->fail(IMA_ERR_STATE, "the loaded surface has no migration parameters");
  for (int t = 0; t < nterms; t++)
    if (thetai[t] < 0 || thetai[t] >= c->snp || mi[t] < 0 || mi[t] >= c->snm)
      return c->fail(IMA_ERR_ARG, "term %d: (%d, %d) out of range", t, thetai[t], mi[t]);
  cudaSetDevice(c->device);
  // pass 1: every term's scale grid (j + 0.5) pmmax / gridsize, scanned from
  // the top for the first density above 1e-9 as the reference scans it; the
  // points go to the device in batches from the top (32 per term, then 4x
  // more each round) so that a scan that stops early costs little
  const size_t npts = (size_t)nterms * gridsize;
  if (npts > (size_t)INT32_MAX) return c->fail(IMA_ERR_ARG, "too many points");
  std::vector<double> pmmax(nterms), mx(nterms, 0.0);
  std::vector<int> top(nterms, gridsize - 1);  // highest index not yet scanned
  for (int t = 0; t < nterms; t++)
    pmmax[t] = mig_mean ? EXPOMIGPLOTSCALE * mig_mean[mi[t]] : theta_max[thetai[t]] * mig_max[mi[t]] / 2.0;
  int r = IMA_OK;
  for (long long batch = 32;; batch *= 4) {
    std::vector<int32_t> th, mm, who;
    std::vector<double> x;
    for (int t = 0; t < nterms; t++) {
      if (top[t] < 0) continue;
      for (long long j = top[t]; j >= 0 && j > top[t] - batch; j--) {
        th.push_back(thetai[t]);
        mm.push_back(mi[t]);
        who.push_back(t);
        x.push_back((j + 0.5) * pmmax[t] / gridsize);
      }
    }
    if (x.empty()) break;
    std::vector<double> y(x.size());
    r = popmig_run(c, (int)x.size(), th.data(), mm.data(), x.data(), theta_max, mig_max, mig_mean, prob_or_like, y.data());
    if (r) return r;
    for (size_t k = 0; k < x.size();) {  // each term's points, top down
      const int t = who[k];
      size_t e = k;
      while (e < x.size() && who[e] == t) e++;
      for (size_t q = k; q < e && top[t] >= 0; q++) {
        if (y[q] > 1e-9) {
          mx[t] = x[q];
          top[t] = -1;
        } else if (--top[t] < 0) {
          mx[t] = pmmax[t];  // no point above 1e-9
        }
      }
      k = e;
    }
  }
  std::vector<int32_t> th(npts), mm(npts);
  std::vector<double> x(npts);
  for (int t = 0; t < nterms; t++) {
    if (maxx) maxx[t] = mx[t];
    for (int j = 0; j < gridsize; j++) {
      th[(size_t)t * gridsize + j] = thetai[t];
      mm[(size_t)t * gridsize + j] = mi[t];
      x[(size_t)t * gridsize + j] = (j + 0.5) * mx[t] / gridsize;
    }
  }
  // pass 2: the curves on [0, maxx]
  r = popmig_run(c, (int)npts, th.data(), mm.data(), x.data(), theta_max, mig_max, mig_mean, prob_or_like, y_out);
  if (r) return r;
  memcpy(x_out, x.data(), npts * 8);
  return IMA_OK;
}

extern "C" int ima_gpu_findmarginpeaks(ima_ctx *c, const double *theta_min, const double *theta_max,
                                       const double *mig_min, const double *mig_max, const double *mig_mean,
                                       int nterms, const int32_t *mpop, const int32_t *mterm, double *mlval,
                                       double *peakloc, double *migtest, double *lo95, double *hi95,
                                       double *pm_mlval, double *pm_peakloc, double *pm_test, float *holdpeakloc,
                                       int *rounds)
{
  if (!c || !theta_min || !theta_max || !mlval || !peakloc || !lo95 || !hi95 || !holdpeakloc) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  const int np = c->snp, nm = c->snm;
  if (nm > 0 && (!mig_min || !mig_max || !migtest)) return IMA_ERR_ARG;
  if (nterms < 0 || (nterms > 0 && (!mpop || !mterm || !pm_mlval || !pm_peakloc || !pm_test))) return IMA_ERR_ARG;
  for (int t = 0; t < nterms; t++)
    if (mpop[t] < 0 || mpop[t] >= np || mterm[t] < 0 || mterm[t] >= nm)
      return c->fail(IMA_ERR_ARG, "2NM term %d: (%d, %d) out of range", t, mpop[t], mterm[t]);
  for (int i = 0; i < np; i++)
    if (!(theta_max[i] > 0.0)) return c->fail(IMA_ERR_ARG, "theta prior maximum %d must be > 0", i);
  for (int i = 0; i < nm; i++) {
    if (!(mig_max[i] > 0.0)) return c->fail(IMA_ERR_ARG, "migration prior maximum %d must be > 0", i);
    if (mig_mean && !(mig_mean[i] > 0.0)) return c->fail(IMA_ERR_ARG, "exponential prior mean %d must be > 0", i);
  }
  cudaSetDevice(c->device);
  MarginPeaksIn in;
  in.G = c->sG;
  in.np = np;
  in.nm = nm;
  in.nterms = nterms;
  in.theta_min = theta_min;
  in.theta_max = theta_max;
  in.mig_min = mig_min;
  in.mig_max = mig_max;
  in.mig_mean = mig_mean;
  in.mpop = mpop;
  in.mterm = mterm;
  MarginPeaksOut out;
  out.mlval = mlval;
  out.peakloc = peakloc;
  out.migtest = migtest;
  out.lo95 = lo95;
  out.hi95 = hi95;
  out.pm_mlval = pm_mlval;
  out.pm_peakloc = pm_peakloc;
  out.pm_test = pm_test;
  out.holdpeakloc = holdpeakloc;
  // one batched launch per (kind, genealogy range) of a round
  MarginPeaksEval eval = [&](const std::vector<MarginPeaksReq> &reqs, std::vector<double> &v) -> int {
    std::vector<char> used(reqs.size(), 0);
    for (size_t k0 = 0; k0 < reqs.size(); k0++) {
      if (used[k0]) continue;
      const MarginPeaksReq &q0 = reqs[k0];
      std::vector<size_t> grp;
      for (size_t k = k0; k < reqs.size(); k++)
        if (!used[k] && reqs[k].kind == q0.kind && reqs[k].lo == q0.lo && reqs[k].hi == q0.hi) {
          used[k] = 1;
          grp.push_back(k);
        }
      const int n = (int)grp.size();
      std::vector<int32_t> idx(n), th(n), mi(n);
      std::vector<double> x(n), y(n);
      for (int k = 0; k < n; k++) {
        idx[k] = reqs[grp[k]].idx;
        x[k] = reqs[grp[k]].x;
      }
      GRange rg;
      rg.lo = q0.lo;
      rg.hi = q0.hi;
      rg.div = (double)(q0.hi - q0.lo + (q0.lo == 0));
      rg.raw_cc = q0.kind == 0;
      int r;
      if (q0.kind >= 2) {
        for (int k = 0; k < n; k++) {
          th[k] = mpop[idx[k]];
          mi[k] = mterm[idx[k]];
        }
        r = popmig_run(c, n, th.data(), mi.data(), x.data(), theta_max, mig_max, q0.kind == 2 ? mig_mean : nullptr,
                       0, y.data(), &rg);
      } else {
        if (q0.kind == 1) rg.div = (double)(q0.hi - q0.lo);  // margincalc divides by the count
        r = margin_run(c, n, idx.data(), x.data(), 0.0, q0.kind == 1, mig_mean, y.data(), &rg);
      }
      if (r) return r;
      for (int k = 0; k < n; k++) v[grp[k]] = y[k];
    }
    return IMA_OK;
  };
  int r;
  try {
    r = findmarginpeaks_run(in, eval, out);
  } catch (const std::exception &e) {  // host allocation of the search state
    return c->fail(IMA_ERR_NOMEM, "findmarginpeaks: %s", e.what());
  }
  if (rounds) *rounds = out.rounds;
  if (r == -1) return c->fail(IMA_ERR_DATA, "a peak search did not end in 20000 rounds");
  return r;
}

extern "C" int ima_gpu_margincalc(ima_ctx *c, int n, const int32_t *param, const double *x, double yadjust, int logi,
                                  const double *expo_mean, double *out)
{
  if (!c || n < 1 || !param || !x || !out) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  cudaSetDevice(c->device);
  return margin_run(c, n, param, x, yadjust, logi, expo_mean, out);
}

extern "C" int ima_gpu_fillvec(ima_ctx *c, int gridsize, const double *pmin, const double *pmax,
                               const double *expo_mean, double *x_out, double *y_out)
{
  if (!c || gridsize < 1 || !pmin || !pmax || !y_out) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  cudaSetDevice(c->device);
  const int npar = c->snp + c->snm;
  std::vector<int32_t> param;
  std::vector<double> x;
  std::vector<int> where;  // y_out index of each request
  for (int p = 0; p < npar; p++) {
    for (int j = 0; j < gridsize; j++) {
      // the grids of setup_iparams / setimigarray (initialize.cpp:189-194, :236-241)
      const double xj = pmin[p] + ((j + 0.5) * (pmax[p] - pmin[p])) / gridsize;
      if (x_out) x_out[(size_t)p * gridsize + j] = xj;
      y_out[(size_t)p * gridsize + j] = 0.0;
      // fillvec skips migration rates whose prior is (near) zero (MPRIORMIN)
      if (p >= c->snp && !(pmax[p] > 0.000001)) continue;
      param.push_back(p);
      x.push_back(xj);
      where.push_back(p * gridsize + j);
    }
  }
  if (param.empty()) return IMA_OK;
  std::vector<double> y(param.size());
  int r = margin_run(c, (int)param.size(), param.data(), x.data(), 0.0, 0, expo_mean, y.data());
  if (r) return r;
  for (size_t k = 0; k < param.size(); k++) y_out[where[k]] = y[k];
  return IMA_OK;
}

static int surf_points(ima_ctx *c, int npoints)
{
  if ((size_t)npoints <= c->spts_cap) return IMA_OK;
  cudaFree(c->d_sx);
  cudaFree(c->d_sq);
  cudaFree(c->d_sess);
  c->d_sx = dev_alloc<double>((size_t)npoints * 32, c->dev_bytes, c->st);
  c->d_sq = dev_alloc<double>(npoints, c->dev_bytes, c->st);
  c->d_sess = dev_alloc<double>(npoints, c->dev_bytes, c->st);
  if (!c->d_sx || !c->d_sq || !c->d_sess) return c->fail(IMA_ERR_NOMEM, "surface point buffers");
  c->spts_cap = npoints;
  return IMA_OK;
}

static int surf_scratch(ima_ctx *c, size_t bytes)
{
  if (bytes <= c->sscratch_cap) return IMA_OK;
  c->srows_state = 0;
  cudaFree(c->d_sscratch);
  c->d_sscratch = dev_alloc<char>(bytes, c->dev_bytes, c->st);
  if (!c->d_sscratch) return c->fail(IMA_ERR_NOMEM, "surface scratch (%zu bytes)", bytes);
  c->sscratch_cap = bytes;
  return IMA_OK;
}

extern "C" int ima_gpu_surface_eval(ima_ctx *c, int npoints, const double *x, int modeltype, int method,
                                    double *q, double *ess)
{
  if (!c || !x || !q || npoints < 1) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "call ima_gpu_surface_load first");
  if (modeltype < 0 || modeltype > 2) return c->fail(IMA_ERR_ARG, "modeltype must be 0, 1 or 2");
  const int npar = c->snp + c->snm;
  for (size_t k = 0; k < (size_t)npoints * npar; k++)
    if (!(x[k] > 0.0)) return c->fail(IMA_ERR_ARG, "parameter values must be > 0 (point %zu)", k / npar);
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->st);
  int r = surf_points(c, npoints);
  if (r) return r;
  SurfArgs a;
  a.G = c->sG;
  a.rowlen = c->srowlen;
  a.np = c->snp;
  a.nm = c->snm;
  a.npops = c->snpops;
  a.modeltype = modeltype;
  a.npoints = npoints;
  a.rows = c->d_rows;
  a.lognorm = c->d_lognorm;
  a.x = c->d_sx;
  a.q = c->d_sq;
  a.ess = c->d_sess;
  r = c->cuda(cudaMemcpyAsync(c->d_sx, x, (size_t)npoints * npar * 8, cudaMemcpyHostToDevice, c->st), "points");
  if (r) return r;
  if (method == IMA_SURF_FAST) {
    r = surf_scratch(c, surface_fast_scratch_bytes(a.G, npoints));
    if (r) return r;
    int lr = 0, nk = 1;
    c->launch(IMA_K_SURF_FAST, (double)a.G * 27 * 4 + (double)npoints * 27 * 8,
              [&] { lr = launch_surface_fast(a, c->d_sscratch, c->sscratch_cap,
                                             c->srows_state >= 1 && c->srows_model == modeltype, &nk, c->st); });
    if (lr) return c->fail(IMA_ERR_ARG, "fast surface: unsupported shape (%d)", lr);
    c->launches += nk - 1;  // one evaluation, several kernels
    if (c->srows_state < 1 || c->srows_model != modeltype) c->srows_state = 1;
    c->srows_model = modeltype;
  } else if (method == IMA_SURF_TC) {
    r = surf_scratch(c, surface_tc_scratch_bytes(a.G, npoints));
    if (r) return r;
    int lr = 0, nk = 1;
    r = c->cuda(cudaMemsetAsync(c->d_flag, 0, sizeof(int), c->st), "flag");
    if (r) return r;
    c->launch(IMA_K_SURF_TC, (double)a.G * 32 * 2 + (double)npoints * 27 * 8,
              [&] { lr = launch_surface_tc(a, c->d_sscratch, c->sscratch_cap, c->d_flag,
                                           c->srows_state == 2 && c->srows_model == modeltype, &nk,
                                           &c->surf_retaken, c->st); });
    if (lr == 5) return c->cuda(cudaGetLastError(), "tensor-core surface");
    if (lr) return c->fail(IMA_ERR_ARG, "tensor-core surface: unsupported shape (%d)", lr);
    c->launches += nk - 1;
    c->srows_state = 2;
    c->srows_model = modeltype;
    int flag = 0;
    r = c->cuda(cudaMemcpyAsync(&flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->st), "flag");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "tensor-core surface");
    if (r) return r;
    if (flag) return c->fail(IMA_ERR_TIMEOUT, "tensor-core surface: a pipeline wait ran out (stage %d)", flag);
  } else if (method == IMA_SURF_FP64) {
    r = surf_scratch(c, surface_fp64_scratch_bytes(a.G, npoints));
    if (r) return r;
    c->srows_state = 0;  // the FP64 form overwrites the scratch
    c->launch(IMA_K_SURF_FP64, (double)a.G * a.rowlen * 4, [&] { launch_surface_fp64(a, (double *)c->d_sscratch, c->st); });
    c->launches += 1;  // pass + merge
  } else if (method == IMA_SURF_COMPAT) {
    r = surf_scratch(c, surface_fp64_scratch_bytes(a.G, npoints));
    if (r) return r;
    c->srows_state = 0;
    c->launch(IMA_K_SURF_COMPAT, (double)a.G * a.rowlen * 4, [&] { launch_surface_compat(a, (double *)c->d_sscratch, c->st); });
    c->launches += (npoints + SURF_COMPAT_CONCURRENT - 1) / SURF_COMPAT_CONCURRENT - 1;
  } else {
    return c->fail(IMA_ERR_ARG, "unknown surface method %d", method);
  }
  r = c->cuda(cudaGetLastError(), "surface launch");
  r = r ? r : c->cuda(cudaMemcpyAsync(q, c->d_sq, npoints * 8, cudaMemcpyDeviceToHost, c->st), "q");
  if (ess) r = r ? r : c->cuda(cudaMemcpyAsync(ess, c->d_sess, npoints * 8, cudaMemcpyDeviceToHost, c->st), "ess");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "surface");
}

extern "C" int ima_gpu_tc_selftest(ima_ctx *c, int *mismatches, float *max_abs_err)
{
  if (!c || !mismatches || !max_abs_err) return IMA_ERR_ARG;
  cudaSetDevice(c->device);
  int r = surf_scratch(c, (size_t)256 << 10);
  if (r) return r;
  c->srows_state = 0;
  int tr = tc_selftest(c->st, c->d_sscratch, c->sscratch_cap, mismatches, max_abs_err);
  c->launches += 3;
  if (tr) return c->fail(IMA_ERR_CUDA, "tensor-core self-test failed to run (%d): %s", tr,
                         cudaGetErrorString(cudaGetLastError()));
  if (*mismatches < 0) return c->fail(IMA_ERR_TIMEOUT, "tensor-core self-test: a wait ran out (%d)", -*mismatches);
  return IMA_OK;
}

extern "C" int ima_gpu_jointp(ima_ctx *c, const double *x, int calc_ess, double *effective_n, double *q)
{
  if (!c || !x || !q) return IMA_ERR_ARG;
  double e = 0.0;
  int r = ima_gpu_surface_eval(c, 1, x, 0, IMA_SURF_COMPAT, q, &e);
  if (!r && calc_ess && effective_n) *effective_n = e;
  return r;
}

// ======================================================================
// measurement
extern "C" int ima_gpu_timer_begin(ima_ctx *c)
{
  if (!c) return IMA_ERR_ARG;
  return c->cuda(cudaEventRecord(c->t0, c->st), "timer");
}

extern "C" int ima_gpu_timer_end(ima_ctx *c, float *ms)
{
  if (!c || !ms) return IMA_ERR_ARG;
  int r = c->cuda(cudaEventRecord(c->t1, c->st), "timer");
  r = r ? r : c->cuda(cudaEventSynchronize(c->t1), "timer");
  return r ? r : c->cuda(cudaEventElapsedTime(ms, c->t0, c->t1), "timer");
}

extern "C" int ima_gpu_set_profiling(ima_ctx *c, int on)
{
  if (!c) return IMA_ERR_ARG;
  c->resolve_timings();
  c->profiling = on != 0;
  return IMA_OK;
}

extern "C" int ima_gpu_kernel_stats(ima_ctx *c, int kind, long long *launches, double *ms_total,
                                    double *bytes_total)
{
  if (!c || kind < 0 || kind >= IMA_K_COUNT) return IMA_ERR_ARG;
  c->resolve_timings();
  if (launches) *launches = c->k_launches[kind];
  if (ms_total) *ms_total = c->k_ms[kind];
  if (bytes_total) *bytes_total = c->k_bytes[kind];
  return IMA_OK;
}

extern "C" int ima_gpu_launch_count(ima_ctx *c, long long *n)
{
  if (!c || !n) return IMA_ERR_ARG;
  *n = c->launches;
  return IMA_OK;
}

extern "C" int ima_gpu_flush_l2(ima_ctx *c)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->d_flush) {
    c->flush_bytes = (size_t)512 << 20;
    if (cudaMalloc(&c->d_flush, c->flush_bytes) != cudaSuccess) {
      c->d_flush = nullptr;
      return c->fail(IMA_ERR_NOMEM, "L2 flush buffer");
    }
    c->dev_bytes += c->flush_bytes;
  }
  return c->cuda(cudaMemsetAsync(c->d_flush, c->launches & 0xff, c->flush_bytes, c->st), "flush");
}

extern "C" int ima_gpu_memory(ima_ctx *c, size_t *bytes)
{
  if (!c || !bytes) return IMA_ERR_ARG;
  *bytes = c->dev_bytes;
  return IMA_OK;
}

// ======================================================================
// genealogy weights and p(G) integrals
namespace {
int grow(ima_ctx *c, void **buf, size_t *cap, size_t bytes, const char *what)
{
  if (bytes <= *cap) return IMA_OK;
  cudaStreamSynchronize(c->st);
  cudaFree(*buf);
  *buf = nullptr;
  *cap = 0;
  size_t n = bytes + bytes / 4;
  *buf = dev_alloc<char>(n, c->dev_bytes, c->st);
  if (!*buf) return c->fail(IMA_ERR_NOMEM, "%s (%zu bytes)", what, n);
  *cap = n;
  return IMA_OK;
}

struct Carve {
  char *p;
  template <typename T>
  T *take(size_t count)
  {
    T *q = reinterpret_cast<T *>(p);
    p += (count * sizeof(T) + 255) / 256 * 256;
    return q;
  }
};

size_t carve_size(std::initializer_list<size_t> bytes)
{
  size_t s = 0;
  for (size_t b : bytes) s += (b + 255) / 256 * 256;
  return s;
}
}  // namespace

// logfact[i] = log(1) + ... + log(i) accumulated as setlogfact does
// (utilities.cpp:1406-1415), so the device table holds the host's values;
// read by the incomplete gamma functions (p(G) integrals, 2NM densities)
static int ensure_logfact(ima_ctx *c)
{
  if (c->d_logfact) return IMA_OK;
  c->d_logfact = dev_alloc<double>(TW_LF_N, c->dev_bytes, c->st);
  if (!c->d_logfact) return c->fail(IMA_ERR_NOMEM, "logfact table");
  std::vector<double> lf(TW_LF_N);
  lf[0] = 0;
  for (int i = 1; i < TW_LF_N; i++) lf[i] = lf[i - 1] + log((double)i);
  int r = c->cuda(cudaMemcpyAsync(c->d_logfact, lf.data(), sizeof(double) * TW_LF_N, cudaMemcpyHostToDevice, c->st), "logfact");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "logfact");
  if (r) {
    cudaFree(c->d_logfact);
    c->d_logfact = nullptr;
  }
  return r;
}

extern "C" int ima_gpu_set_popmodel(ima_ctx *c, int npops, int nomig, int expo, const int32_t *plist,
                                    const int32_t *droppops, const int32_t *addpop, const int32_t *pop_e,
                                    const int32_t *pop_down, int nth, const int32_t *th_off,
                                    const int32_t *th_idx, const double *th_max, const double *th_min,
                                    int nmg, const int32_t *mg_off, const int32_t *mg_idx, const double *mg_max,
                                    const double *mg_min, const double *mg_mean, int nchk,
                                    const int32_t *chk_idx)
{
  if (!c) return IMA_ERR_ARG;
  if (npops < 2 || npops > TW_MAXPOPS) return c->fail(IMA_ERR_ARG, "npops must be in 2..%d", TW_MAXPOPS);
  if (!plist || !droppops || !addpop || !pop_e || !pop_down || !th_off || !th_max || !th_min)
    return c->fail(IMA_ERR_ARG, "population model: null table");
  const int ntp = 2 * npops - 1, nsplit = npops - 1;
  TwModel h;
  memset(&h, 0, sizeof(h));
  h.npops = npops;
  h.nomig = nomig ? 1 : 0;
  h.expo = expo ? 1 : 0;
  h.T = npops * (npops + 1) / 2;
  int mm = 0;
  for (int k = 0; k <= npops; k++) {
    h.toff[k] = (int16_t)(k * npops - k * (k - 1) / 2);
    h.moff[k] = (int16_t)mm;
    if (k < nsplit) mm += (npops - k) * (npops - k);
  }
  h.M = mm;
  memset(h.plist, -1, sizeof(h.plist));
  memset(h.pos, -1, sizeof(h.pos));
  for (int k = 0; k < npops; k++)
    for (int ii = 0; ii < npops - k; ii++) {
      const int p = plist[k * npops + ii];
      if (p < 0 || p >= ntp || (ii > 0 && p <= plist[k * npops + ii - 1]))
        return c->fail(IMA_ERR_ARG, "plist[%d][%d] = %d: populations of a period must be distinct ids "
                                    "below %d in increasing order", k, ii, p, ntp);
      h.plist[k][ii] = (int8_t)p;
      h.pos[k][p] = (int8_t)ii;
    }
  for (int k = 1; k < npops; k++) {
    const int d0 = droppops[2 * k], d1 = droppops[2 * k + 1], ad = addpop[k];
    if (d0 < 0 || d0 >= ntp || d1 < 0 || d1 >= ntp || ad < 0 || ad >= ntp || h.pos[k - 1][d0] < 0 ||
        h.pos[k - 1][d1] < 0 || h.pos[k][ad] < 0 || h.pos[k - 1][ad] >= 0)
      return c->fail(IMA_ERR_ARG, "split %d (%d, %d -> %d) does not match plist", k, d0, d1, ad);
    h.droppops[k][0] = (int8_t)d0;
    h.droppops[k][1] = (int8_t)d1;
    h.addpop[k] = (int8_t)ad;
  }
  for (int p = 0; p < ntp; p++) {
    if (pop_e[p] < -1 || pop_e[p] == 0 || pop_e[p] > nsplit || pop_down[p] < -1 || pop_down[p] >= ntp)
      return c->fail(IMA_ERR_ARG, "pop_e/pop_down of population %d out of range", p);
    h.pop_e[p] = (int8_t)pop_e[p];
    h.pop_down[p] = (int8_t)pop_down[p];
  }
  if (nth < 1 || nth > TW_MAXTH || th_off[0] != 0 || th_off[nth] > TW_MAXT || (th_off[nth] > 0 && !th_idx))
    return c->fail(IMA_ERR_ARG, "theta parameter map: nth %d", nth);
  h.nth = nth;
  for (int i = 0; i <= nth; i++) {
    if (i > 0 && th_off[i] < th_off[i - 1]) return c->fail(IMA_ERR_ARG, "th_off must not decrease");
    h.th_off[i] = (int16_t)th_off[i];
  }
  for (int j = 0; j < th_off[nth]; j++) {
    if (th_idx[j] < 0 || th_idx[j] >= h.T) return c->fail(IMA_ERR_ARG, "th_idx[%d] out of range", j);
    h.th_idx[j] = (int16_t)th_idx[j];
  }
  for (int i = 0; i < nth; i++) {
    if (!(th_max[i] > th_min[i]) || th_min[i] < 0) return c->fail(IMA_ERR_ARG, "theta prior %d", i);
    h.th_max[i] = th_max[i];
    h.th_min[i] = th_min[i];
  }
  if (!nomig) {
    if (nmg < 0 || nmg > TW_MAXMG || (nmg > 0 && (!mg_off || !mg_max || !mg_min))) return c->fail(IMA_ERR_ARG, "migration parameter map: nmg %d", nmg);
    if (nmg > 0 && (mg_off[0] != 0 || mg_off[nmg] > TW_MAXM || (mg_off[nmg] > 0 && !mg_idx)))
      return c->fail(IMA_ERR_ARG, "migration parameter map offsets");
    h.nmg = nmg;
    for (int i = 0; i <= nmg && nmg > 0; i++) {
      if (i > 0 && mg_off[i] < mg_off[i - 1]) return c->fail(IMA_ERR_ARG, "mg_off must not decrease");
      h.mg_off[i] = (int16_t)mg_off[i];
    }
    for (int j = 0; nmg > 0 && j < mg_off[nmg]; j++) {
      if (mg_idx[j] < 0 || mg_idx[j] >= h.M) return c->fail(IMA_ERR_ARG, "mg_idx[%d] out of range", j);
      h.mg_idx[j] = (int16_t)mg_idx[j];
    }
    for (int i = 0; i < nmg; i++) {
      if (expo && (!mg_mean || !(mg_mean[i] > 0))) return c->fail(IMA_ERR_ARG, "migration prior mean %d", i);
      if (!expo && (!(mg_max[i] > mg_min[i]) || mg_min[i] < 0)) return c->fail(IMA_ERR_ARG, "migration prior %d", i);
      h.mg_max[i] = mg_max[i];
      h.mg_min[i] = mg_min[i];
      h.mg_mean[i] = mg_mean ? mg_mean[i] : 0.0;
    }
    if (nchk < 0 || nchk > TW_MAXM || (nchk > 0 && !chk_idx)) return c->fail(IMA_ERR_ARG, "nchk %d", nchk);
    h.nchk = nchk;
    for (int i = 0; i < nchk; i++) {
      if (chk_idx[i] < 0 || chk_idx[i] >= h.M) return c->fail(IMA_ERR_ARG, "chk_idx[%d] out of range", i);
      h.chk_idx[i] = (int16_t)chk_idx[i];
    }
  }
  cudaSetDevice(c->device);
  if (!c->d_tw) {
    c->d_tw = dev_alloc<TwModel>(1, c->dev_bytes, c->st);
    c->d_twerr = dev_alloc<int32_t>(2, c->dev_bytes, c->st);
    if (!c->d_tw || !c->d_twerr) return c->fail(IMA_ERR_NOMEM, "population model");
  }
  if (int r0 = ensure_logfact(c)) return r0;
  c->h_tw = h;
  int r = c->cuda(cudaMemcpyAsync(c->d_tw, &c->h_tw, sizeof(TwModel), cudaMemcpyHostToDevice, c->st), "population model");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "population model");
  if (r) return r;
  c->tw_ready = true;
  c->tw_ngen = 0;
  return IMA_OK;
}

static int tw_check_err(ima_ctx *c, const char *what)
{
  int32_t e[2] = {0, 0};
  int r = c->cuda(cudaMemcpyAsync(e, c->d_twerr, sizeof(e), cudaMemcpyDeviceToHost, c->st), what);
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), what);
  if (r) return r;
  static const char *why[] = {"", "a population that does not exist in that period (or a migration to the same "
                                  "population)", "a lineage count below zero", "more events than planned",
                              "an integral term the reference rejects (LogDiff order or iteration limit)",
                              "a count beyond the logfact table", "mig_off decreasing within the genealogy"};
  if (e[0]) return c->fail(e[0] == 6 ? IMA_ERR_ARG : IMA_ERR_DATA, "%s: item %d: %s", what, e[1], why[e[0] < 7 ? e[0] : 0]);
  return IMA_OK;
}

extern "C" int ima_gpu_treeweight(ima_ctx *c, int ngen, const int32_t *node_off, const int32_t *up0,
                                  const double *time, const int32_t *pop, const int32_t *mig_off,
                                  const double *mig_t, const int32_t *mig_p, const int32_t *gen_locus,
                                  const int32_t *gen_tv, int nloci, const double *hval, const int32_t *samppop,
                                  int ntv, const double *tvals, int32_t *cc, double *hcc, double *fc,
                                  int32_t *mc, double *fm, double *lens, int32_t *mignum)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  if (ngen < 1 || !node_off || !up0 || !time || !pop || !mig_off || !gen_locus || !gen_tv || nloci < 1 ||
      !hval || !samppop || ntv < 1 || !tvals)
    return c->fail(IMA_ERR_ARG, "treeweight: bad argument");
  const TwModel &h = c->h_tw;
  const int npops = h.npops, nsplit = npops - 1;
  if (node_off[0] != 0) return c->fail(IMA_ERR_ARG, "node_off[0] must be 0");
  for (int li = 0; li < nloci; li++)
    if (!(hval[li] > 0)) return c->fail(IMA_ERR_ARG, "hval[%d] must be > 0", li);
  long long Emax = 0;
  std::vector<int32_t> ev(ngen);
  for (int g = 0; g < ngen; g++) {
    const int a0 = node_off[g], nl = node_off[g + 1] - a0;
    if (nl < 1 || !(nl & 1)) return c->fail(IMA_ERR_ARG, "genealogy %d: %d nodes (need 2n-1)", g, nl);
    const int li = gen_locus[g], tv = gen_tv[g];
    if (li < 0 || li >= nloci || tv < 0 || tv >= ntv) return c->fail(IMA_ERR_ARG, "genealogy %d: locus or tvals row", g);
    int ns = 0;
    for (int p = 0; p < npops; p++) ns += samppop[(size_t)li * npops + p];
    if (ns != (nl + 1) / 2) return c->fail(IMA_ERR_ARG, "genealogy %d: %d genes, samppop of locus %d sums to %d", g, (nl + 1) / 2, li, ns);
    const long long E = (nl - 1) / 2 + (long long)(mig_off[a0 + nl] - mig_off[a0]) + nsplit;
    if (E > Emax) Emax = E;
    ev[g] = (int32_t)(E < (1 << 21) ? E : (1 << 21));
  }
  const size_t N = (size_t)node_off[ngen];
  // per genealogy here; node by node in the kernel, before any event is read
  if (mig_off[0] != 0) return c->fail(IMA_ERR_ARG, "mig_off[0] must be 0");
  for (int g = 0; g < ngen; g++)
    if (mig_off[node_off[g + 1]] < mig_off[node_off[g]])
      return c->fail(IMA_ERR_ARG, "mig_off must not decrease (genealogy %d)", g);
  const size_t Nm = (size_t)mig_off[N];
  if (Nm > 0 && (!mig_t || !mig_p)) return c->fail(IMA_ERR_ARG, "migration events without mig_t/mig_p");
  int P = 32;
  while (P < Emax) P <<= 1;
  if (P > (1 << 20) || !tw_fits(P))
    return c->fail(IMA_ERR_TOO_LARGE, "a genealogy has %lld events; at most %d fit", Emax,
                   (int)((200 * 1024 - (h.T + h.M) * 12) / 12));
  // processing order: most events first (counting sort), so that the
  // genealogies sharing a warp sweep about as many events
  std::vector<int32_t> perm(ngen), cnt((size_t)Emax + 2, 0);
  for (int g = 0; g < ngen; g++) cnt[(size_t)(Emax - ev[g])]++;
  for (size_t i = 1; i < cnt.size(); i++) cnt[i] += cnt[i - 1];
  for (int g = ngen - 1; g >= 0; g--) perm[--cnt[(size_t)(Emax - ev[g])]] = g;
  std::vector<long long> evoff(ngen + 1);
  evoff[0] = 0;
  for (int g = 0; g < ngen; g++) evoff[g + 1] = evoff[g] + ev[g];
  const size_t Etot = (size_t)evoff[ngen];
  cudaSetDevice(c->device);
  const size_t T = h.T, MM = h.M;
  const size_t inb = carve_size({ngen * 4ul, (ngen + 1) * 4ul, N * 4, N * 4, (N + 1) * 4, Nm * 4, ngen * 4ul, ngen * 4ul,
                                 (size_t)nloci * npops * 4, N * 8, Nm * 8, (size_t)ntv * nsplit * 8,
                                 (size_t)nloci * 8, (size_t)nloci * 8, (ngen + 1) * 8ul, Etot * 8, Etot * 4,
                                 ngen * 4ul});
  const size_t outb = carve_size({ngen * T * 4, ngen * MM * 4, ngen * 4ul, ngen * T * 8, ngen * T * 8,
                                  ngen * MM * 8, 2 * ngen * 8ul});
  int r = grow(c, &c->d_twin, &c->twin_cap, inb, "treeweight inputs");
  r = r ? r : grow(c, &c->d_twout, &c->twout_cap, outb, "treeweight weights");
  if (r) return r;
  Carve ci{static_cast<char *>(c->d_twin)}, co{static_cast<char *>(c->d_twout)};
  TwArgs a{};
  a.ngen = ngen;
  a.P = P;
  a.model = c->d_tw;
  a.nodes = nullptr;  // host-packed genealogies
  a.moff_start = nullptr;
  a.mbase = nullptr;
  a.len_out = nullptr;
  int32_t *d_perm = ci.take<int32_t>(ngen);
  int32_t *d_node_off = ci.take<int32_t>(ngen + 1), *d_up0 = ci.take<int32_t>(N), *d_pop = ci.take<int32_t>(N),
          *d_mig_off = ci.take<int32_t>(N + 1), *d_mig_p = ci.take<int32_t>(Nm),
          *d_gl = ci.take<int32_t>(ngen), *d_gt = ci.take<int32_t>(ngen),
          *d_sp = ci.take<int32_t>((size_t)nloci * npops);
  double *d_time = ci.take<double>(N), *d_mig_t = ci.take<double>(Nm), *d_tv = ci.take<double>((size_t)ntv * nsplit),
         *d_hlog = ci.take<double>(nloci), *d_h2 = ci.take<double>(nloci);
  long long *d_evoff = ci.take<long long>(ngen + 1);
  a.ev_t = ci.take<double>(Etot);
  a.ev_c = ci.take<uint32_t>(Etot);
  a.ev_n = ci.take<int32_t>(ngen);
  a.ev_off = d_evoff;
  std::vector<double> hl(nloci), h2(nloci);
  for (int li = 0; li < nloci; li++) {
    hl[li] = log(hval[li]);           // treeweight: hlog = log (L[li].hval)
    h2[li] = 1 / (2 * hval[li]);      // h2term = 1 / (2 * L[li].hval)
  }
  auto up = [&](void *dst, const void *src, size_t bytes) {
    if (!r && bytes) r = c->cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->st), "treeweight inputs");
  };
  up(d_perm, perm.data(), ngen * 4ul);
  up(d_node_off, node_off, (ngen + 1) * 4ul);
  up(d_up0, up0, N * 4);
  up(d_pop, pop, N * 4);
  up(d_mig_off, mig_off, (N + 1) * 4);
  up(d_mig_p, mig_p, Nm * 4);
  up(d_gl, gen_locus, ngen * 4ul);
  up(d_gt, gen_tv, ngen * 4ul);
  up(d_sp, samppop, (size_t)nloci * npops * 4);
  up(d_time, time, N * 8);
  up(d_mig_t, mig_t, Nm * 8);
  up(d_tv, tvals, (size_t)ntv * nsplit * 8);
  up(d_hlog, hl.data(), (size_t)nloci * 8);
  up(d_h2, h2.data(), (size_t)nloci * 8);
  up(d_evoff, evoff.data(), (ngen + 1) * 8ul);
  if (r) return r;
  a.perm = d_perm;
  a.node_off = d_node_off;
  a.up0 = d_up0;
  a.pop = d_pop;
  a.mig_off = d_mig_off;
  a.mig_p = d_mig_p;
  a.gen_locus = d_gl;
  a.gen_tv = d_gt;
  a.samppop = d_sp;
  a.time = d_time;
  a.mig_t = d_mig_t;
  a.tvals = d_tv;
  a.hlog = d_hlog;
  a.h2term = d_h2;
  a.cc = co.take<int32_t>(ngen * T);
  a.mc = co.take<int32_t>(ngen * MM);
  a.mignum = co.take<int32_t>(ngen);
  a.hcc = co.take<double>(ngen * T);
  a.fc = co.take<double>(ngen * T);
  a.fm = co.take<double>(ngen * MM);
  a.lens = co.take<double>(2 * (size_t)ngen);
  a.err = c->d_twerr;
  r = c->cuda(cudaMemsetAsync(c->d_twerr, 0, 8, c->st), "treeweight");
  if (r) return r;
  c->tw_ngen = 0;
  int lr = 0;
  c->launch(IMA_K_TREEWEIGHT, (double)N * 20 + (double)Nm * 12 + (double)ngen * (T * 20 + MM * 12 + 20),
            [&] { lr = launch_treeweight(a, h, c->st); });
  c->launches += 1;  // event sort + sweep
  if (lr) return c->fail(IMA_ERR_TOO_LARGE, "treeweight: shared memory for %d events", P);
  r = c->cuda(cudaGetLastError(), "treeweight launch");
  if (r) return r;
  r = tw_check_err(c, "treeweight");
  if (r) return r;
  c->tw_ngen = ngen;
  c->tw_valid.assign((size_t)ngen, 1);
  c->tw_ntv = ntv;
  c->tw_cc = a.cc;
  c->tw_mc = a.mc;
  c->tw_hcc = a.hcc;
  c->tw_fc = a.fc;
  c->tw_fm = a.fm;
  c->tw_tvals = d_tv;
  auto down = [&](void *dst, const void *src, size_t bytes) {
    if (!r && dst && bytes) r = c->cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->st), "treeweight outputs");
  };
  down(cc, a.cc, ngen * T * 4);
  down(mc, a.mc, ngen * MM * 4);
  down(mignum, a.mignum, ngen * 4ul);
  down(hcc, a.hcc, ngen * T * 8);
  down(fc, a.fc, ngen * T * 8);
  down(fm, a.fm, ngen * MM * 8);
  down(lens, a.lens, 2 * ngen * 8ul);
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "treeweight");
}

// p(G) of groups of the last weights: group i = genealogies group_off[i] ..
// group_end[i] (group_end null: group_off[i+1])
// defer: no error check, no copies back and no synchronisation here (the
// caller checks the error word after a later synchronisation)
// device copies of tree_prob_run's per-group outputs, valid until the next call
struct TpDev {
  int32_t *sc = nullptr;  // [groups][T + M] summed counts
  double *sd = nullptr;   // [groups][2T + M] summed fc, hcc, fm
  double *q = nullptr;    // [groups][nth] theta integrals
};

static int tree_prob_run(ima_ctx *c, int ngroups, const int32_t *group_off, const int32_t *group_end,
                         const double *pdg, const int32_t *group_tv, double *probg, double *q, double *m,
                         float *rows, double **d_probg = nullptr, bool defer = false, TpDev *dev = nullptr)
{
  if (!c->tw_ready || c->tw_ngen < 1) return c->fail(IMA_ERR_STATE, "call ima_gpu_treeweight first");
  if (ngroups < 1 || !group_off) return c->fail(IMA_ERR_ARG, "tree_prob: bad argument");
  const TwModel &h = c->h_tw;
  for (int i = 0; i < ngroups; i++) {
    const int e = group_end ? group_end[i] : group_off[i + 1];
    if (group_off[i] < 0 || e < group_off[i] || e > c->tw_ngen)
      return c->fail(IMA_ERR_ARG, "group %d (%d..%d) outside the %d genealogies", i, group_off[i], e, c->tw_ngen);
    for (int g = group_off[i]; g < e; g++)
      if (!c->tw_valid[g])
        return c->fail(IMA_ERR_STATE, "group %d: genealogy %d has no weights from the last weights call", i, g);
  }
  if (group_tv)
    for (int i = 0; i < ngroups; i++)
      if (group_tv[i] < 0 || group_tv[i] >= c->tw_ntv) return c->fail(IMA_ERR_ARG, "group_tv[%d] out of range", i);
  const int nth = h.nth, nmg = h.nomig ? 0 : h.nmg;
  const int rowlen = 4 * nth + 3 * nmg + 2 + h.npops - 1;  // cc fc hcc mc fm qi mi pdg probg t
  cudaSetDevice(c->device);
  const size_t G = ngroups;
  const size_t MMc = h.nomig ? 0 : h.M;
  const size_t b = carve_size({(G + 1) * 4, G * 4, G * 8, G * 8, G * nth * 8, G * (nmg ? nmg : 1) * 8,
                               G * rowlen * 4, G * (h.T + MMc) * 4, G * (2 * h.T + MMc) * 8, G * 4});
  int r = grow(c, &c->d_tpbuf, &c->tpbuf_cap, b, "tree_prob buffers");
  if (r) return r;
  Carve cv{static_cast<char *>(c->d_tpbuf)};
  TwProbArgs a{};
  a.ngroups = ngroups;
  a.group_end = nullptr;
  a.model = c->d_tw;
  int32_t *d_off = cv.take<int32_t>(G + 1), *d_tv = cv.take<int32_t>(G);
  double *d_pdg = cv.take<double>(G);
  a.group_off = d_off;
  a.group_tv = d_tv;
  a.pdg = pdg ? d_pdg : nullptr;
  a.probg = cv.take<double>(G);
  a.q = cv.take<double>(G * nth);
  a.m = cv.take<double>(G * (nmg ? nmg : 1));
  a.rows = cv.take<float>(G * rowlen);  // kept for ima_gpu_surface_append_tree_rows
  a.sc = cv.take<int32_t>(G * (h.T + MMc));
  a.sd = cv.take<double>(G * (2 * h.T + MMc));
  int32_t *d_end = cv.take<int32_t>(G);
  a.rowlen = rowlen;
  a.cc = c->tw_cc;
  a.mc = c->tw_mc;
  a.hcc = c->tw_hcc;
  a.fc = c->tw_fc;
  a.fm = c->tw_fm;
  a.tvals = c->tw_tvals;
  a.logfact = c->d_logfact;
  a.err = c->d_twerr;
  r = c->cuda(cudaMemcpyAsync(d_off, group_off, (group_end ? G : G + 1) * 4, cudaMemcpyHostToDevice, c->st), "tree_prob groups");
  if (group_end) {
    r = r ? r : c->cuda(cudaMemcpyAsync(d_end, group_end, G * 4, cudaMemcpyHostToDevice, c->st), "tree_prob groups");
    a.group_end = d_end;
  }
  if (group_tv)
    r = r ? r : c->cuda(cudaMemcpyAsync(d_tv, group_tv, G * 4, cudaMemcpyHostToDevice, c->st), "tree_prob groups");
  else
    r = r ? r : c->cuda(cudaMemsetAsync(d_tv, 0, G * 4, c->st), "tree_prob groups");
  if (pdg) r = r ? r : c->cuda(cudaMemcpyAsync(d_pdg, pdg, G * 8, cudaMemcpyHostToDevice, c->st), "tree_prob pdg");
  if (!defer) r = r ? r : c->cuda(cudaMemsetAsync(c->d_twerr, 0, 8, c->st), "tree_prob");
  if (r) return r;
  c->tp_ngroups = 0;
  c->launch(IMA_K_TREE_PROB, (double)c->tw_ngen * (h.T * 20 + h.M * 12), [&] { launch_tree_prob(a, h, c->st); });
  c->launches += 2;  // cells, parameters, final
  r = c->cuda(cudaGetLastError(), "tree_prob launch");
  if (!defer) r = r ? r : tw_check_err(c, "tree_prob");
  if (r) return r;
  c->tp_rows = a.rows;
  c->tp_ngroups = ngroups;
  c->tp_rowlen = rowlen;
  if (d_probg) *d_probg = a.probg;
  if (dev) {
    dev->sc = a.sc;
    dev->sd = a.sd;
    dev->q = a.q;
  }
  auto down = [&](void *dst, const void *src, size_t bytes) {
    if (!r && dst && bytes) r = c->cuda(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, c->st), "tree_prob outputs");
  };
  down(probg, a.probg, G * 8);
  down(q, a.q, G * nth * 8);
  if (nmg) down(m, a.m, G * nmg * 8);
  if (rows) down(rows, a.rows, G * rowlen * 4);
  if (defer) return r;
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "tree_prob");
}

extern "C" int ima_gpu_tree_prob(ima_ctx *c, int ngroups, const int32_t *group_off, const double *pdg,
                                 const int32_t *group_tv, double *probg, double *q, double *m, float *rows)
{
  if (!c) return IMA_ERR_ARG;
  return tree_prob_run(c, ngroups, group_off, nullptr, pdg, group_tv, probg, q, m, rows);
}

extern "C" int ima_gpu_surface_append_tree_rows(ima_ctx *c, int n, const int32_t *groups)
{
  if (!c || n < 1 || !groups) return IMA_ERR_ARG;
  if (c->tp_ngroups < 1) return c->fail(IMA_ERR_STATE, "call ima_gpu_tree_prob first");
  for (int i = 0; i < n; i++)
    if (groups[i] < 0 || groups[i] >= c->tp_ngroups)
      return c->fail(IMA_ERR_ARG, "groups[%d] = %d: the last tree_prob had %d chains", i, groups[i], c->tp_ngroups);
  const TwModel &h = c->h_tw;
  const int np = h.nth, nm = h.nomig ? 0 : h.nmg, rowlen = c->tp_rowlen;
  if (np + nm > 32 || rowlen > 64)
    return c->fail(IMA_ERR_ARG, "a surface holds at most 32 parameters and 64 columns (here %d, %d)", np + nm, rowlen);
  if (c->d_rows && (c->srowlen != rowlen || c->snp != np || c->snm != nm || c->snpops != h.npops))
    return c->fail(IMA_ERR_STATE, "the resident surface holds rows of another model; load or append to a new context");
  if (c->d_lognorm) return c->fail(IMA_ERR_STATE, "the resident surface has per-genealogy normalisers; rows cannot be added");
  cudaSetDevice(c->device);
  const size_t need = (size_t)(c->d_rows ? c->sG : 0) + n;
  if (need >= (size_t)(1 << 24)) return c->fail(IMA_ERR_TOO_LARGE, "surface rows beyond 2^24");
  if (!c->d_rows || need > c->s_cap) {
    size_t cap = c->s_cap ? c->s_cap * 2 : 1024;
    while (cap < need) cap *= 2;
    float *nr = dev_alloc<float>(cap * rowlen, c->dev_bytes, c->st);
    if (!nr) return c->fail(IMA_ERR_NOMEM, "surface rows (%zu)", cap);
    if (c->d_rows) {
      int r = c->cuda(cudaMemcpyAsync(nr, c->d_rows, (size_t)c->sG * rowlen * 4, cudaMemcpyDeviceToDevice, c->st), "surface grow");
      if (r) return r;
      cudaStreamSynchronize(c->st);
      cudaFree(c->d_rows);
    } else {
      c->sG = 0;
    }
    c->d_rows = nr;
    c->s_cap = cap;
    c->srowlen = rowlen;
    c->snp = np;
    c->snm = nm;
    c->snpops = h.npops;
  }
  int32_t *d_groups = nullptr;
  int r = c->cuda(cudaMallocAsync((void **)&d_groups, (size_t)n * 4, c->st), "append groups");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_groups, groups, (size_t)n * 4, cudaMemcpyHostToDevice, c->st), "append groups");
  if (r) return r;
  launch_gather_rows(c->tp_rows, rowlen, d_groups, n, c->d_rows + (size_t)c->sG * rowlen, c->st);
  c->launches += 1;
  r = c->cuda(cudaGetLastError(), "append rows");
  cudaFreeAsync(d_groups, c->st);
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "append rows");
  if (r) return r;
  c->sG += n;
  c->srows_state = 0;  // row-derived surface operands are stale
  return IMA_OK;
}

extern "C" int ima_gpu_surface_get_rows(ima_ctx *c, int start, int count, int rowlen, float *rows)
{
  if (!c || !rows || start < 0 || count < 0) return IMA_ERR_ARG;
  if (!c->d_rows) return c->fail(IMA_ERR_STATE, "no surface rows");
  if (rowlen != c->srowlen) return c->fail(IMA_ERR_ARG, "rowlen %d: the surface's rows hold %d values", rowlen, c->srowlen);
  if (start + count > c->sG) return c->fail(IMA_ERR_ARG, "rows %d..%d beyond the %d held", start, start + count, c->sG);
  cudaSetDevice(c->device);
  int r = c->cuda(cudaMemcpyAsync(rows, c->d_rows + (size_t)start * c->srowlen, (size_t)count * c->srowlen * 4,
                                  cudaMemcpyDeviceToHost, c->st), "surface rows");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "surface rows");
}

// ======================================================================
// resident population labels and the split-time update
static int labels_alloc(ima_ctx *c)
{
  if (c->d_pop) return IMA_OK;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  const int ni = c->nitems;
  const size_t nn = c->nnodes;
  size_t &B = c->dev_bytes;
  c->d_pop = dev_alloc<int32_t>(nn, B, c->st);
  c->d_moff = dev_alloc<int32_t>(nn + ni, B, c->st);
  c->d_inode_off = dev_alloc<int32_t>(ni + 1, B, c->st);
  c->d_gl = dev_alloc<int32_t>(ni, B, c->st);
  c->d_gt = dev_alloc<int32_t>(ni, B, c->st);
  c->d_moff_start = dev_alloc<int32_t>(ni, B, c->st);
  c->d_bcnt = dev_alloc<int32_t>(4 * (size_t)c->nchains, B, c->st);
  c->d_bicnt = dev_alloc<int32_t>(4 * (size_t)ni, B, c->st);
  c->d_mbase = dev_alloc<long long>(ni, B, c->st);
  c->d_len_hold = dev_alloc<double>(ni, B, c->st);
  if (!c->d_pop || !c->d_moff || !c->d_inode_off || !c->d_gl || !c->d_gt || !c->d_moff_start || !c->d_bcnt || !c->d_bicnt ||
      !c->d_mbase || !c->d_len_hold)
    return c->fail(IMA_ERR_NOMEM, "population labels");
  std::vector<int32_t> off(ni + 1), gl(ni), gt(ni), ms(ni);
  for (int i = 0; i < ni; i++) {
    off[i] = c->items[i].node_off;
    gl[i] = i % c->nloci;
    gt[i] = i / c->nloci;
    ms[i] = c->items[i].node_off + i;
    if (i > 0 && off[i] != off[i - 1] + 2 * c->items[i - 1].n - 1)
      return c->fail(IMA_ERR_STATE, "node pool is not in item order");
  }
  off[ni] = c->items[ni - 1].node_off + 2 * c->items[ni - 1].n - 1;
  int r = c->cuda(cudaMemcpyAsync(c->d_inode_off, off.data(), (ni + 1) * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_gl, gl.data(), ni * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_gt, gt.data(), ni * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_moff_start, ms.data(), ni * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "labels");
  if (r) return r;
  c->h_mbase.assign(ni, 0);
  c->h_mcnt.assign(ni, 0);
  c->h_mcap.assign(ni, 0);
  c->has_labels.assign(ni, 0);
  return IMA_OK;
}

extern "C" int ima_gpu_set_locus_pops(ima_ctx *c, const double *hval, const int32_t *samppop)
{
  if (!c || !hval || !samppop) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  const int npops = c->h_tw.npops, nl = c->nloci;
  std::vector<double> hl(nl), h2(nl);
  for (int li = 0; li < nl; li++) {
    if (!(hval[li] > 0)) return c->fail(IMA_ERR_ARG, "hval[%d] must be > 0", li);
    int ns = 0;
    for (int p = 0; p < npops; p++) ns += samppop[(size_t)li * npops + p];
    if (ns != c->loci[li].d.n) return c->fail(IMA_ERR_ARG, "locus %d: samppop sums to %d, not %d genes", li, ns, c->loci[li].d.n);
    hl[li] = log(hval[li]);
    h2[li] = 1 / (2 * hval[li]);
  }
  cudaSetDevice(c->device);
  if (!c->d_rhlog) {
    c->d_rhlog = dev_alloc<double>(nl, c->dev_bytes, c->st);
    c->d_rh2 = dev_alloc<double>(nl, c->dev_bytes, c->st);
    c->d_rsamp = dev_alloc<int32_t>((size_t)nl * TW_MAXPOPS, c->dev_bytes, c->st);
    c->d_tvr = dev_alloc<double>((size_t)c->nchains * TW_MAXPOPS, c->dev_bytes, c->st);
    if (!c->d_rhlog || !c->d_rh2 || !c->d_rsamp || !c->d_tvr) return c->fail(IMA_ERR_NOMEM, "locus populations");
  }
  int r = c->cuda(cudaMemcpyAsync(c->d_rhlog, hl.data(), nl * 8ul, cudaMemcpyHostToDevice, c->st), "locus pops");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_rh2, h2.data(), nl * 8ul, cudaMemcpyHostToDevice, c->st), "locus pops");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_rsamp, samppop, (size_t)nl * npops * 4, cudaMemcpyHostToDevice, c->st), "locus pops");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "locus pops");
  if (r) return r;
  c->h_tvr.assign((size_t)c->nchains * (npops - 1), 0.0);
  c->h_hval.assign(hval, hval + nl);
  c->h_samp.assign(samppop, samppop + (size_t)nl * npops);
  c->locus_pops = true;
  return IMA_OK;
}

extern "C" int ima_gpu_set_labels(ima_ctx *c, int n, const int32_t *ci, const int32_t *li, const int32_t *pop,
                                  const int32_t *mig_off, const double *mig_t, const int32_t *mig_p)
{
  if (!c || n < 1 || !ci || !li || !pop || !mig_off) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  cudaSetDevice(c->device);
  int r = labels_alloc(c);
  if (r) return r;
  const int ntp = 2 * c->h_tw.npops - 1;
  size_t noff = 0, moff = 0, ev = 0;
  for (int k = 0; k < n; k++) {
    if (!c->valid(ci[k], li[k])) return c->fail(IMA_ERR_ARG, "pair %d: chain %d locus %d out of range", k, ci[k], li[k]);
    const int item = c->item_of(ci[k], li[k]);
    const int nl = 2 * c->items[item].n - 1;
    const int32_t *mo = mig_off + moff;
    if (mo[0] != 0) return c->fail(IMA_ERR_ARG, "pair %d: mig_off must start at 0", k);
    for (int i = 0; i < nl; i++) {
      if (pop[noff + i] < 0 || pop[noff + i] >= ntp) return c->fail(IMA_ERR_ARG, "pair %d node %d: population %d", k, i, pop[noff + i]);
      if (mo[i + 1] < mo[i]) return c->fail(IMA_ERR_ARG, "pair %d: mig_off decreases at node %d", k, i);
    }
    const int cnt = mo[nl];
    if (cnt > 0 && (!mig_t || !mig_p)) return c->fail(IMA_ERR_ARG, "migration events without mig_t/mig_p");
    for (int j = 0; j < cnt; j++)
      if (mig_p[ev + j] < 0 || mig_p[ev + j] >= ntp) return c->fail(IMA_ERR_ARG, "pair %d: migration to population %d", k, mig_p[ev + j]);
    // room for the item's events: its own range, or a new one at the end of the pool
    if (cnt > c->h_mcap[item]) {
      if (c->mig_used + cnt > c->mig_cap) {
        size_t cap = c->mig_cap ? c->mig_cap * 2 : 4096;
        while (cap < c->mig_used + cnt) cap *= 2;
        double *nt = dev_alloc<double>(cap, c->dev_bytes, c->st);
        int32_t *np_ = dev_alloc<int32_t>(cap, c->dev_bytes, c->st);
        if (!nt || !np_) return c->fail(IMA_ERR_NOMEM, "migration events (%zu)", cap);
        if (c->mig_used) {
          r = c->cuda(cudaMemcpyAsync(nt, c->d_mig_t, c->mig_used * 8, cudaMemcpyDeviceToDevice, c->st), "events");
          r = r ? r : c->cuda(cudaMemcpyAsync(np_, c->d_mig_p, c->mig_used * 4, cudaMemcpyDeviceToDevice, c->st), "events");
          if (r) return r;
        }
        cudaStreamSynchronize(c->st);
        cudaFree(c->d_mig_t);
        cudaFree(c->d_mig_p);
        c->d_mig_t = nt;
        c->d_mig_p = np_;
        c->mig_cap = cap;
      }
      c->h_mbase[item] = (long long)c->mig_used;
      c->h_mcap[item] = cnt;
      c->mig_used += cnt;
    }
    c->h_mcnt[item] = cnt;
    const size_t no = c->items[item].node_off;
    r = c->cuda(cudaMemcpyAsync(c->d_pop + no, pop + noff, nl * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
    r = r ? r : c->cuda(cudaMemcpyAsync(c->d_moff + no + item, mo, (nl + 1) * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
    r = r ? r : c->cuda(cudaMemcpyAsync(c->d_mbase + item, &c->h_mbase[item], 8, cudaMemcpyHostToDevice, c->st), "labels");
    if (cnt) {
      r = r ? r : c->cuda(cudaMemcpyAsync(c->d_mig_t + c->h_mbase[item], mig_t + ev, cnt * 8ul, cudaMemcpyHostToDevice, c->st), "labels");
      r = r ? r : c->cuda(cudaMemcpyAsync(c->d_mig_p + c->h_mbase[item], mig_p + ev, cnt * 4ul, cudaMemcpyHostToDevice, c->st), "labels");
    }
    if (r) return r;
    c->has_labels[item] = 1;
    noff += nl;
    moff += nl + 1;
    ev += cnt;
  }
  return c->cuda(cudaStreamSynchronize(c->st), "labels");
}

extern "C" int ima_gpu_get_times(ima_ctx *c, int ci, int li, double *time, int32_t *nmig, double *mig_t)
{
  if (!c || !time) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  const int item = c->item_of(ci, li);
  const ItemDev &it = c->items[item];
  cudaSetDevice(c->device);
  int r = c->cuda(cudaMemcpyAsync(time, c->d_t64 + it.node_off, (2 * it.n - 1) * 8ul, cudaMemcpyDeviceToHost, c->st), "times");
  const int cnt = (c->d_pop && c->has_labels[item]) ? c->h_mcnt[item] : 0;
  if (nmig) *nmig = cnt;
  if (mig_t && cnt)
    r = r ? r : c->cuda(cudaMemcpyAsync(mig_t, c->d_mig_t + c->h_mbase[item], cnt * 8ul, cudaMemcpyDeviceToHost, c->st), "times");
  return r ? r : c->cuda(cudaStreamSynchronize(c->st), "times");
}

// also uploads pending host edits: the resident functions read the device pools
static int chains_ready(ima_ctx *c, int nch, const int32_t *chains)
{
  if (!c->d_pop || !c->locus_pops) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_labels and ima_gpu_set_locus_pops first");
  cudaSetDevice(c->device);
  if (int r = flush(c)) return r;
  if (int r = ensure_lengths(c)) return r;
  for (int k = 0; k < nch; k++) {
    if (chains[k] < 0 || chains[k] >= c->nchains) return c->fail(IMA_ERR_ARG, "chain %d out of range", chains[k]);
    for (int l = 0; l < k; l++)
      if (chains[l] == chains[k]) return c->fail(IMA_ERR_ARG, "chain %d listed twice", chains[k]);
    for (int li = 0; li < c->nloci; li++)
      if (!c->has_labels[c->item_of(chains[k], li)] || !c->has_tree[c->item_of(chains[k], li)])
        return c->fail(IMA_ERR_STATE, "chain %d locus %d has no genealogy or labels", chains[k], li);
  }
  return IMA_OK;
}

static void* rsel(ima_ctx *c, size_t bytes)
{
  if (bytes > c->rsel_cap) {
    cudaStreamSynchronize(c->st);
    cudaFree(c->d_rsel);
    c->d_rsel = dev_alloc<char>(bytes, c->dev_bytes, c->st);
    c->rsel_cap = c->d_rsel ? bytes : 0;
  }
  return c->d_rsel;
}

static void dev_newer(ima_ctx *c, int nch, const int32_t *chains)
{
  for (int k = 0; k < nch; k++) {
    c->dev_lo = std::min(c->dev_lo, chains[k] * c->nloci);
    c->dev_hi = std::max(c->dev_hi, chains[k] * c->nloci + c->nloci - 1);
  }
}

// the band on the device; counts stay in d_bcnt, the chain list in
// *d_chains (the caller's chains, device copy) when asked for
static int band_run(ima_ctx *c, int nch, const int32_t *chains, const int32_t *period, const double *oldt,
                    const double *newt, const double *t_u, const double *t_d, int inverse, int32_t *counts,
                    bool sync, int32_t **d_chains = nullptr)
{
  int r = IMA_OK;
  const int last = c->h_tw.npops - 1;
  std::vector<double> prm(5 * (size_t)nch);
  for (int k = 0; k < nch; k++) {
    if (period[k] < 0 || period[k] >= last) return c->fail(IMA_ERR_ARG, "period %d out of range", period[k]);
    if (!(oldt[k] > t_u[k]) || !(newt[k] > t_u[k]) || !(oldt[k] < t_d[k]) || !(newt[k] < t_d[k]))
      return c->fail(IMA_ERR_ARG, "chain %d: split times must lie inside (t_u, t_d)", chains[k]);
    prm[5 * k + 0] = period[k];
    prm[5 * k + 1] = inverse ? newt[k] : oldt[k];  // going back: from newt to oldt
    prm[5 * k + 2] = inverse ? oldt[k] : newt[k];
    prm[5 * k + 3] = t_u[k];
    prm[5 * k + 4] = t_d[k];
  }
  const int nsplit = last;
  if (c->h_tvr.size() == (size_t)c->nchains * nsplit)  // the split times the labels follow from here on
    for (int k = 0; k < nch; k++) c->h_tvr[(size_t)chains[k] * nsplit + period[k]] = inverse ? oldt[k] : newt[k];
  cudaSetDevice(c->device);
  char *buf = static_cast<char *>(rsel(c, 256 + nch * 4ul + 256 + 40ul * nch));
  if (!buf) return c->fail(IMA_ERR_NOMEM, "band buffers");
  int32_t *d_ch = reinterpret_cast<int32_t *>(buf);
  double *d_prm = reinterpret_cast<double *>(buf + (nch * 4 + 255) / 256 * 256 + 256);
  r = c->cuda(cudaMemcpyAsync(d_ch, chains, nch * 4ul, cudaMemcpyHostToDevice, c->st), "band");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_prm, prm.data(), prm.size() * 8, cudaMemcpyHostToDevice, c->st), "band");
  r = r ? r : c->cuda(cudaMemsetAsync(c->d_bcnt, 0, 16ul * nch, c->st), "band");
  if (r) return r;
  BandArgs a{};
  a.items = c->d_items;
  a.nodes = c->d_nodes;
  a.t64 = c->d_t64;
  a.tff = c->d_tff;
  a.moff = c->d_moff;
  a.mbase = c->d_mbase;
  a.mig_t = c->d_mig_t;
  a.chains = d_ch;
  a.prm = d_prm;
  a.nch = nch;
  a.nloci = c->nloci;
  a.last = last;
  a.inverse = inverse ? 1 : 0;
  a.counts = c->d_bcnt;
  a.item_counts = c->d_bicnt;
  a.len = c->d_len;
  a.len_hold = c->d_len_hold;
  int nk = 1;
  c->launch(IMA_K_TREEWEIGHT, 0.0, [&] { nk = launch_band(a, c->st); });
  c->launches += nk - 1;
  r = c->cuda(cudaGetLastError(), "band launch");
  if (!r && counts && !inverse) r = c->cuda(cudaMemcpyAsync(counts, c->d_bcnt, 16ul * nch, cudaMemcpyDeviceToHost, c->st), "band counts");
  // the parameter block is host memory of this call: wait for its copy
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "band");
  if (!r) dev_newer(c, nch, chains);
  if (d_chains) *d_chains = d_ch;
  (void)sync;
  return r;
}

extern "C" int ima_gpu_rubber_band(ima_ctx *c, int nch, const int32_t *chains, const int32_t *period,
                                   const double *oldt, const double *newt, const double *t_u, const double *t_d,
                                   int inverse, int32_t *counts)
{
  if (!c || nch < 1 || !chains || !period || !oldt || !newt || !t_u || !t_d) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  int r = chains_ready(c, nch, chains);
  if (r) return r;
  return band_run(c, nch, chains, period, oldt, newt, t_u, t_d, inverse, counts, true);
}

static int chain_weights_run(ima_ctx *c, int nch, const int32_t *chains, const double *tvals, double *probg,
                             double *q, double *m, double **d_probg, bool defer = false, TpDev *dev = nullptr)
{
  int r = IMA_OK;
  const TwModel &h = c->h_tw;
  const int npops = h.npops, nsplit = npops - 1, nl = c->nloci, ni = c->nitems;
  for (int k = 0; k < nch; k++)
    for (int s = 0; s < nsplit; s++) c->h_tvr[(size_t)chains[k] * nsplit + s] = tvals[(size_t)k * nsplit + s];
  // the chains' genealogies, most events first; event scratch per item
  std::vector<int32_t> ev(ni, 0), sel;
  long long Emax = 0;
  for (int k = 0; k < nch; k++)
    for (int li = 0; li < nl; li++) {
      const int item = c->item_of(chains[k], li);
      const long long E = c->items[item].n - 1 + (long long)c->h_mcnt[item] + nsplit;
      ev[item] = (int32_t)E;
      Emax = std::max(Emax, E);
      sel.push_back(item);
    }
  int P = 32;
  while (P < Emax) P <<= 1;
  if (P > (1 << 20) || !tw_fits(P)) return c->fail(IMA_ERR_TOO_LARGE, "a genealogy has %lld events", Emax);
  std::vector<int32_t> perm(sel.size()), cnt((size_t)Emax + 2, 0);
  for (int item : sel) cnt[(size_t)(Emax - ev[item])]++;
  for (size_t i = 1; i < cnt.size(); i++) cnt[i] += cnt[i - 1];
  for (int k = (int)sel.size() - 1; k >= 0; k--) perm[--cnt[(size_t)(Emax - ev[sel[k]])]] = sel[k];
  std::vector<long long> evoff(ni + 1, 0);
  for (int i = 0; i < ni; i++) evoff[i + 1] = evoff[i] + ev[i];
  const size_t Etot = (size_t)evoff[ni], ns = sel.size(), T = h.T, MM = h.M;
  cudaSetDevice(c->device);
  const size_t inb = carve_size({ns * 4, (ni + 1) * 8ul, Etot * 8, Etot * 4, ni * 4ul});
  const size_t outb = carve_size({ni * T * 4, ni * MM * 4, ni * 4ul, ni * T * 8, ni * T * 8, ni * MM * 8, 2ul * ni * 8});
  r = grow(c, &c->d_twin, &c->twin_cap, inb, "treeweight scratch");
  r = r ? r : grow(c, &c->d_twout, &c->twout_cap, outb, "treeweight weights");
  if (r) return r;
  Carve ci_{static_cast<char *>(c->d_twin)}, co{static_cast<char *>(c->d_twout)};
  TwArgs a{};
  a.ngen = (int)ns;
  a.P = P;
  a.model = c->d_tw;
  int32_t *d_perm = ci_.take<int32_t>(ns);
  long long *d_evoff = ci_.take<long long>(ni + 1);
  a.perm = d_perm;
  a.ev_off = d_evoff;
  a.ev_t = ci_.take<double>(Etot);
  a.ev_c = ci_.take<uint32_t>(Etot);
  a.ev_n = ci_.take<int32_t>(ni);
  a.node_off = c->d_inode_off;
  a.up0 = nullptr;
  a.nodes = c->d_nodes;
  a.time = c->d_t64;
  a.pop = c->d_pop;
  a.mig_off = c->d_moff;
  a.moff_start = c->d_moff_start;
  a.mbase = c->d_mbase;
  a.mig_t = c->d_mig_t;
  a.mig_p = c->d_mig_p;
  a.gen_locus = c->d_gl;
  a.gen_tv = c->d_gt;
  a.tvals = c->d_tvr;
  a.hlog = c->d_rhlog;
  a.h2term = c->d_rh2;
  a.samppop = c->d_rsamp;
  a.cc = co.take<int32_t>(ni * T);
  a.mc = co.take<int32_t>(ni * MM);
  a.mignum = co.take<int32_t>(ni);
  a.hcc = co.take<double>(ni * T);
  a.fc = co.take<double>(ni * T);
  a.fm = co.take<double>(ni * MM);
  a.lens = co.take<double>(2ul * ni);
  a.len_out = c->d_len;
  a.err = c->d_twerr;
  r = c->cuda(cudaMemcpyAsync(d_perm, perm.data(), ns * 4, cudaMemcpyHostToDevice, c->st), "weights");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_evoff, evoff.data(), (ni + 1) * 8ul, cudaMemcpyHostToDevice, c->st), "weights");
  r = r ? r : c->cuda(cudaMemcpyAsync(c->d_tvr, c->h_tvr.data(), c->h_tvr.size() * 8, cudaMemcpyHostToDevice, c->st), "weights");
  r = r ? r : c->cuda(cudaMemsetAsync(c->d_twerr, 0, 8, c->st), "weights");
  if (r) return r;
  c->tw_ngen = 0;
  int lr = 0;
  c->launch(IMA_K_TREEWEIGHT, 0.0, [&] { lr = launch_treeweight(a, h, c->st); });
  if (lr < 0) return c->fail(IMA_ERR_TOO_LARGE, "treeweight: shared memory for %d events", P);
  c->launches += lr - 1;
  r = c->cuda(cudaGetLastError(), "weights launch");
  if (!defer) r = r ? r : tw_check_err(c, "chain weights");
  if (r) return r;
  dev_newer(c, nch, chains);  // the lengths of these items changed on the device
  c->tw_ngen = ni;
  c->tw_valid.assign((size_t)ni, 0);
  for (int item : sel) c->tw_valid[item] = 1;
  c->tw_ntv = c->nchains;
  c->tw_cc = a.cc;
  c->tw_mc = a.mc;
  c->tw_hcc = a.hcc;
  c->tw_fc = a.fc;
  c->tw_fm = a.fm;
  c->tw_tvals = c->d_tvr;
  std::vector<int32_t> goff(nch), gend(nch);
  for (int k = 0; k < nch; k++) {
    goff[k] = chains[k] * nl;
    gend[k] = chains[k] * nl + nl;
  }
  std::vector<double> pg(nch);
  return tree_prob_run(c, nch, goff.data(), gend.data(), nullptr, chains, (probg || defer) ? probg : pg.data(), q, m,
                       nullptr, d_probg, defer, dev);
}

extern "C" int ima_gpu_chain_weights(ima_ctx *c, int nch, const int32_t *chains, const double *tvals,
                                     double *probg, double *q, double *m)
{
  if (!c || nch < 1 || !chains || !tvals) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  int r = chains_ready(c, nch, chains);
  if (r) return r;
  return chain_weights_run(c, nch, chains, tvals, probg, q, m, nullptr);
}

extern "C" int ima_gpu_changet_ry1_sweep(ima_ctx *c, int nch, const int32_t *chains, const int32_t *period,
                                         const double *oldt, const double *newt, const double *t_u, const double *t_d,
                                         const double *log_hu, const double *log_hd, const double *logU, double gbeta,
                                         const double *tvals, const double *u, const double *kappa, int precision,
                                         uint8_t *accept, double *pdgsum, double *probg)
{
  if (!c || nch < 1 || !chains || !period || !oldt || !newt || !t_u || !t_d || !log_hu || !log_hd || !logU ||
      !tvals || !u || !accept)
    return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  int r = chains_ready(c, nch, chains);
  if (r) return r;
  const int nl = c->nloci;
  int32_t *d_ch = nullptr;
  r = band_run(c, nch, chains, period, oldt, newt, t_u, t_d, 0, nullptr, false, &d_ch);
  double *d_pgnew = nullptr;
  // weights and p(G) run on while the host stages the likelihood requests;
  // their error word is read once the likelihoods have synchronised
  r = r ? r : chain_weights_run(c, nch, chains, tvals, nullptr, nullptr, nullptr, &d_pgnew, true);
  if (r) return r;
  // the chains' likelihoods (writes the per-item pdg_new pool)
  std::vector<int32_t> ci((size_t)nch * nl), li((size_t)nch * nl), st((size_t)nch * nl);
  std::vector<double> kap((size_t)nch * nl, 1.0), res((size_t)nch * nl);
  for (int k = 0; k < nch; k++)
    for (int l = 0; l < nl; l++) {
      ci[(size_t)k * nl + l] = chains[k];
      li[(size_t)k * nl + l] = l;
      if (kappa) kap[(size_t)k * nl + l] = kappa[(size_t)k * nl + l];
    }
  r = ima_gpu_eval(c, nch * nl, ci.data(), li.data(), u, kap.data(), nullptr, nullptr, precision, res.data(), st.data());
  r = r ? r : tw_check_err(c, "chain weights / p(G)");
  if (r) return r;
  for (size_t k = 0; k < st.size(); k++)
    if (st[k] == IMA_EVAL_IS_FAIL)
      return c->fail(IMA_ERR_DATA, "chain %d locus %d: data incompatible with the genealogy", ci[k], li[k]);
  // the decisions, on the device
  char *buf = static_cast<char *>(rsel(c, carve_size({nch * 4ul, 40ul * nch, 24ul * nch, 8ul * nch, nch * 1ul, 8ul * nch})));
  if (!buf) return c->fail(IMA_ERR_NOMEM, "decision buffers");
  Carve cv{buf};
  int32_t *d_ch2 = cv.take<int32_t>(nch);
  cv.take<double>(5 * (size_t)nch);  // the band's parameter block (same buffer)
  double *d_logs = cv.take<double>(3 * (size_t)nch);
  double *d_sum = cv.take<double>(nch);
  uint8_t *d_acc = cv.take<uint8_t>(nch);
  (void)d_ch;
  std::vector<double> logs(3 * (size_t)nch);
  for (int k = 0; k < nch; k++) {
    logs[k] = log_hu[k];
    logs[nch + k] = log_hd[k];
    logs[2 * nch + k] = logU[k];
  }
  r = c->cuda(cudaMemcpyAsync(d_ch2, chains, nch * 4ul, cudaMemcpyHostToDevice, c->st), "decide");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_logs, logs.data(), logs.size() * 8, cudaMemcpyHostToDevice, c->st), "decide");
  if (r) return r;
  RyArgs a{};
  a.nch = nch;
  a.nloci = nl;
  a.chains = d_ch2;
  a.counts = c->d_bcnt;
  a.lhu = d_logs;
  a.lhd = d_logs + nch;
  a.logU = d_logs + 2 * nch;
  a.probg_new = d_pgnew;
  a.gbeta = gbeta;
  a.beta = c->d_beta;
  a.probg = c->d_probg;
  a.pdg = c->d_pdg;
  a.pdg_new = c->d_pdg_new;
  a.accept = d_acc;
  a.pdgsum = d_sum;
  launch_ry_decide(a, c->st);
  c->launches++;
  r = c->cuda(cudaGetLastError(), "decide launch");
  r = r ? r : c->cuda(cudaMemcpyAsync(accept, d_acc, nch, cudaMemcpyDeviceToHost, c->st), "decisions");
  if (pdgsum) r = r ? r : c->cuda(cudaMemcpyAsync(pdgsum, d_sum, nch * 8ul, cudaMemcpyDeviceToHost, c->st), "decisions");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "decisions");
  if (r) return r;
  // commit the accepted chains' evaluations, move the others back
  std::vector<uint8_t> acc_items((size_t)nch * nl);
  std::vector<int32_t> rc, rp;
  std::vector<double> ro, rn, ru, rd;
  for (int k = 0; k < nch; k++) {
    for (int l = 0; l < nl; l++) acc_items[(size_t)k * nl + l] = accept[k];
    if (!accept[k]) {
      rc.push_back(chains[k]);
      rp.push_back(period[k]);
      ro.push_back(oldt[k]);
      rn.push_back(newt[k]);
      ru.push_back(t_u[k]);
      rd.push_back(t_d[k]);
    }
  }
  r = commit(c, nch * nl, ci.data(), li.data(), acc_items.data(), true, true);
  if (!r && !rc.empty())
    r = band_run(c, (int)rc.size(), rc.data(), rp.data(), ro.data(), rn.data(), ru.data(), rd.data(), 1, nullptr, true);
  if (!r && probg) {  // the resident p(G) of each chain after the decision
    std::vector<double> all(c->nchains);
    r = c->cuda(cudaMemcpyAsync(all.data(), c->d_probg, c->nchains * 8ul, cudaMemcpyDeviceToHost, c->st), "probg");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "probg");
    for (int k = 0; !r && k < nch; k++) probg[k] = all[chains[k]];
  }
  return r;
}

// changet_RY1's draws in the library: for each chain in order, getnewt
// (update_gtree_common.cpp:2501-2519: one uniform, a window over the prior
// range inside the neighbouring split times, reflected at its ends) and the
// acceptance uniform, from the caller's MT19937, as the reference draws
// them; the split times come from the context (ima_gpu_get_split_times).
extern "C" int ima_gpu_changet_ry1_sweep_mt(ima_ctx *c, int nch, const int32_t *chains, const int32_t *period,
                                            const double *tprior_lo, const double *tprior_hi, ima_mt19937 *rng,
                                            double gbeta, const double *u, const double *kappa, int precision,
                                            uint8_t *accept, double *pdgsum, double *probg, double *newt_out)
{
  if (!c || nch < 1 || !chains || !period || !tprior_lo || !tprior_hi || !rng || !u || !accept) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  const int npops = c->h_tw.npops, nsplit = npops - 1, last = nsplit;
  if (c->h_tvr.size() != (size_t)c->nchains * nsplit) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_locus_pops first");
  const double TIMEMAX = 1000000.0;  // imamp.hpp:129
  std::vector<double> oldt(nch), newt(nch), tu(nch), td(nch), lhu(nch), lhd(nch), logU(nch), tv((size_t)nch * nsplit);
  for (int k = 0; k < nch; k++) {
    if (chains[k] < 0 || chains[k] >= c->nchains) return c->fail(IMA_ERR_ARG, "chain %d out of range", chains[k]);
    if (period[k] < 0 || period[k] >= last) return c->fail(IMA_ERR_ARG, "period %d out of range", period[k]);
  }
  for (int k = 0; k < nch; k++) {
    const int p = period[k];
    const double *row = &c->h_tvr[(size_t)chains[k] * nsplit];
    oldt[k] = row[p];
    tu[k] = p == 0 ? 0.0 : row[p - 1];
    td[k] = p == last - 1 ? TIMEMAX : row[p + 1];
    const double tup = std::max(tprior_lo[p], tu[k]), tdp = std::min(tprior_hi[p], td[k]);
    const double twin = (tdp - tup) / (log(static_cast<double>(c->nloci) + 1) * (npops - p));
    const double U = ima_mt19937_uniform(rng);
    double nt = (oldt[k] - twin / 2) + U * twin;
    if (nt >= tdp)
      nt = 2.0 * tdp - nt;
    else if (nt <= tup)
      nt = 2.0 * tup - nt;
    newt[k] = nt;
    logU[k] = log(ima_mt19937_uniform(rng));
    lhu[k] = log((nt - tu[k]) / (oldt[k] - tu[k]));
    lhd[k] = p == last - 1 ? 0.0 : log((td[k] - nt) / (td[k] - oldt[k]));
    for (int q = 0; q < nsplit; q++) tv[(size_t)k * nsplit + q] = row[q];
    tv[(size_t)k * nsplit + p] = nt;
  }
  if (newt_out) memcpy(newt_out, newt.data(), nch * 8ul);
  return ima_gpu_changet_ry1_sweep(c, nch, chains, period, oldt.data(), newt.data(), tu.data(), td.data(), lhu.data(),
                                   lhd.data(), logU.data(), gbeta, tv.data(), u, kappa, precision, accept, pdgsum,
                                   probg);
}

// ======================================================================
// the genealogy update of the no-migration model (k_updgen.cu)
extern "C" int ima_gpu_get_genealogy(ima_ctx *c, int ci, int li, int32_t *up0, int32_t *up1, int32_t *down,
                                     double *time, int32_t *pop)
{
  if (!c) return IMA_ERR_ARG;
  if (!c->valid(ci, li)) return c->fail(IMA_ERR_ARG, "chain %d locus %d out of range", ci, li);
  const int item = c->item_of(ci, li);
  if (!c->has_tree[item]) return c->fail(IMA_ERR_STATE, "chain %d locus %d has no genealogy", ci, li);
  if (pop && !c->has_labels.size()) return c->fail(IMA_ERR_STATE, "no population labels");
  cudaSetDevice(c->device);
  const ItemDev &it = c->items[item];
  const int nl = 2 * it.n - 1;
  std::vector<NodeRec> nd(nl);
  int r = c->cuda(cudaMemcpyAsync(nd.data(), c->d_nodes + it.node_off, nl * sizeof(NodeRec), cudaMemcpyDeviceToHost, c->st), "genealogy");
  if (time) r = r ? r : c->cuda(cudaMemcpyAsync(time, c->d_t64 + it.node_off, nl * 8ul, cudaMemcpyDeviceToHost, c->st), "genealogy");
  if (pop) r = r ? r : c->cuda(cudaMemcpyAsync(pop, c->d_pop + it.node_off, nl * 4ul, cudaMemcpyDeviceToHost, c->st), "genealogy");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "genealogy");
  if (r) return r;
  for (int k = 0; k < nl; k++) {
    if (up0) up0[k] = nd[k].up0;
    if (up1) up1[k] = nd[k].up1;
    if (down) down[k] = nd[k].down;
  }
  return IMA_OK;
}

extern "C" int ima_gpu_updategenealogy_sweep(ima_ctx *c, int nch, const int32_t *chains, const double *tvals,
                                             int nsweeps, const double *u, const double *kappa,
                                             const int32_t *allele_range, double gbeta, int precision, ima_ug_rng *rng,
                                             int32_t *accepted, int32_t *topology, double *probg)
{
  if (!c || nch < 1 || !chains || !tvals || nsweeps < 0 || !u || !rng) return IMA_ERR_ARG;
  if (!c->tw_ready) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_popmodel first");
  const TwModel &h = c->h_tw;
  if (!h.nomig) return c->fail(IMA_ERR_STATE, "the genealogy update is built for the no-migration model (nomig = 1)");
  const int nl = c->nloci, nsplit = h.npops - 1, T = h.T, nth = h.nth, ni = c->nitems;
  int maxn = 0, anysw = 0;
  for (int li = 0; li < nl; li++) {
    const LocusDev &L = c->loci[li].d;
    if (L.model == IMA_MODEL_SW) {
      if (L.nlinked != 1) return c->fail(IMA_ERR_ARG, "locus %d: the genealogy update takes one-marker SW loci", li);
      if (!allele_range) return c->fail(IMA_ERR_ARG, "locus %d is SW: allele_range is needed", li);
      if (allele_range[2 * li] > allele_range[2 * li + 1]) return c->fail(IMA_ERR_ARG, "locus %d: empty allele range", li);
      anysw = 1;
    }
    maxn = std::max(maxn, L.n);
  }
  int r = chains_ready(c, nch, chains);
  if (r) return r;
  for (int k = 0; k < nch; k++)
    for (int li = 0; li < nl; li++)
      if (c->h_mcnt[c->item_of(chains[k], li)])
        return c->fail(IMA_ERR_STATE, "chain %d locus %d holds migration events", chains[k], li);
  // a full evaluation, committed: the partials and G.pdg of the genealogies
  // the sweep starts from
  const size_t np = (size_t)nch * nl;
  std::vector<int32_t> ci(np), li(np), st(np);
  std::vector<double> kap(np, 1.0), res(np);
  for (int k = 0; k < nch; k++)
    for (int l = 0; l < nl; l++) {
      ci[(size_t)k * nl + l] = chains[k];
      li[(size_t)k * nl + l] = l;
      if (kappa) kap[(size_t)k * nl + l] = kappa[(size_t)k * nl + l];
    }
  // (the SW loci in FP64: their branch terms are the state the update edits)
  for (int pass = 0; pass < 2 && !r; pass++) {
    std::vector<int32_t> pc, pl;
    std::vector<double> pu, pk;
    for (size_t k = 0; k < np; k++)
      if ((c->loci[li[k]].d.model == IMA_MODEL_SW) == (pass == 1)) {
        pc.push_back(ci[k]);
        pl.push_back(li[k]);
        pu.push_back(u[k]);
        pk.push_back(kap[k]);
      }
    if (pc.empty()) continue;
    std::vector<double> pr(pc.size());
    std::vector<int32_t> ps(pc.size());
    r = ima_gpu_eval(c, (int)pc.size(), pc.data(), pl.data(), pu.data(), pk.data(), nullptr, nullptr,
                     pass ? IMA_PREC_FP64 : precision, pr.data(), ps.data());
    for (size_t k = 0; !r && k < pc.size(); k++)
      if (ps[k] != IMA_EVAL_OK)
        return c->fail(IMA_ERR_DATA, "chain %d locus %d: the likelihood rejects the current genealogy", pc[k], pl[k]);
  }
  if (r) return r;
  {
    std::vector<uint8_t> ones(np, 1);
    r = commit(c, (int)np, ci.data(), li.data(), ones.data(), true, true);
    if (r) return r;
  }
  // the chains' weights summed afresh and their p(G), made resident
  TpDev tpd;
  std::vector<double> pg(nch);
  r = chain_weights_run(c, nch, chains, tvals, pg.data(), nullptr, nullptr, nullptr, false, &tpd);
  if (r) return r;
  {
    std::vector<double> all(c->nchains);
    r = c->cuda(cudaMemcpyAsync(all.data(), c->d_probg, c->nchains * 8ul, cudaMemcpyDeviceToHost, c->st), "probg");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "probg");
    for (int k = 0; k < nch; k++) all[chains[k]] = pg[k];
    r = r ? r : c->cuda(cudaMemcpyAsync(c->d_probg, all.data(), c->nchains * 8ul, cudaMemcpyHostToDevice, c->st), "probg");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "probg");
    if (r) return r;
  }
  // event lists of the proposed genealogies (no migrations: coalescences and splits)
  std::vector<long long> evoff(ni + 1, 0);
  long long Emax = 0;
  {
    std::vector<int32_t> ev(ni, 0);
    for (int k = 0; k < nch; k++)
      for (int l = 0; l < nl; l++) {
        const int item = c->item_of(chains[k], l);
        ev[item] = c->items[item].n - 1 + nsplit;
        Emax = std::max(Emax, (long long)ev[item]);
      }
    for (int i = 0; i < ni; i++) evoff[i + 1] = evoff[i] + ev[i];
  }
  int P = 32;
  while (P < Emax) P <<= 1;
  if (!tw_fits(P)) return c->fail(IMA_ERR_TOO_LARGE, "a genealogy has %lld events", Emax);
  // the weights kernel writes every migration cell of the model, nomig or not
  const size_t Etot = (size_t)evoff[ni], M1 = std::max(1, h.M), mx = 2 * (size_t)maxn;
  // steps in flight: a ring of per-step buffers (backups, proposal flags,
  // slide terms, acceptance uniforms); at most one sweep of loci deep, so a
  // locus's batch and weights are never rewritten before their decision ran
  const int R = std::min(4, nl);
  const size_t rn = (size_t)R * nch;
  const size_t bytes = carve_size({nch * sizeof(ima_ug_rng), nch * 4ul, np * 4, np * 4, rn * mx * sizeof(NodeRec),
                                   rn * mx * 8, rn * mx * 4, rn * mx * 2, rn * 8, rn * 4, rn * 8, rn * 8, rn * 8,
                                   rn * 16, rn * mx * 4, rn * mx * 8, rn * 8, rn * 8, rn * 8, np * 8, nl * 8ul,
                                   8, nch * T * 4ul, nch * T * 8ul, nch * T * 8ul, nch * (size_t)nth * 8, np * 4, np * 4,
                                   ni * T * 4ul, ni * M1 * 4, ni * 4ul, ni * T * 8ul, ni * T * 8ul, ni * M1 * 8,
                                   2ul * ni * 8, (ni + 1) * 8ul, Etot * 8, Etot * 4, ni * 4ul});
  r = grow(c, &c->d_ug, &c->ug_cap, bytes, "genealogy update buffers");
  if (r) return r;
  Carve cv{static_cast<char *>(c->d_ug)};
  UgArgs a{};
  a.nch = nch;
  a.nloci = nl;
  a.maxn = maxn;
  a.nsplit = nsplit;
  a.rng = cv.take<ima_ug_rng>(nch);
  int32_t *d_chains = cv.take<int32_t>(nch);
  int32_t *d_reqof = cv.take<int32_t>(np);
  int32_t *d_perm = cv.take<int32_t>(np);
  a.bk_nodes = cv.take<NodeRec>(rn * mx);
  a.bk_t = cv.take<double>(rn * mx);
  a.bk_pop = cv.take<int32_t>(rn * mx);
  a.bk_sched = cv.take<int16_t>(rn * mx);
  a.bk_len = cv.take<double>(rn);
  a.bk_nlev = cv.take<int32_t>(rn);
  a.prop = reinterpret_cast<int32_t *>(cv.take<double>(rn));
  a.slidew = cv.take<double>(rn);
  a.ustore = cv.take<double>(rn);
  a.edges = cv.take<int32_t>(4 * rn);
  a.bk_A = cv.take<int32_t>(rn * mx);
  a.bk_dl = cv.take<double>(rn * mx);
  a.swnew = cv.take<double>(rn);
  a.aterm = cv.take<double>(rn);
  a.holdsis = cv.take<double>(rn);
  double *d_ucl = cv.take<double>(np);
  int32_t *d_arange = cv.take<int32_t>(2ul * nl);
  a.err = cv.take<int32_t>(2);
  a.ag_cc = cv.take<int32_t>(nch * (size_t)T);
  a.ag_fc = cv.take<double>(nch * (size_t)T);
  a.ag_hcc = cv.take<double>(nch * (size_t)T);
  a.qint = cv.take<double>(nch * (size_t)nth);
  a.nacc = cv.take<int32_t>(np);
  a.ntopo = cv.take<int32_t>(np);
  // the proposed genealogies' weights (treeweight's outputs), by item
  TwArgs w{};
  w.cc = cv.take<int32_t>(ni * (size_t)T);
  w.mc = cv.take<int32_t>(ni * M1);
  w.mignum = cv.take<int32_t>(ni);
  w.hcc = cv.take<double>(ni * (size_t)T);
  w.fc = cv.take<double>(ni * (size_t)T);
  w.fm = cv.take<double>(ni * M1);
  w.lens = cv.take<double>(2ul * ni);
  long long *d_evoff = cv.take<long long>(ni + 1);
  w.ev_t = cv.take<double>(Etot);
  w.ev_c = cv.take<uint32_t>(Etot);
  w.ev_n = cv.take<int32_t>(ni);
  w.ngen = nch;
  w.P = P;
  w.model = c->d_tw;
  w.ev_off = d_evoff;
  w.node_off = c->d_inode_off;
  w.nodes = c->d_nodes;
  w.time = c->d_t64;
  w.pop = c->d_pop;
  w.mig_off = c->d_moff;
  w.moff_start = c->d_moff_start;
  w.mbase = c->d_mbase;
  w.mig_t = c->d_mig_t;
  w.mig_p = c->d_mig_p;
  w.gen_locus = c->d_gl;
  w.gen_tv = c->d_gt;
  w.tvals = c->d_tvr;
  w.hlog = c->d_rhlog;
  w.h2term = c->d_rh2;
  w.samppop = c->d_rsamp;
  w.len_out = c->d_len;
  w.err = c->d_twerr;
  // per-locus evaluation requests: the listed chains, full evaluations whose
  // HKY edits the proposal fills in
  if ((int)c->ugb.size() < nl) c->ugb.resize(nl);
  std::vector<int32_t> reqof(np), perm(np);
  for (int l = 0; l < nl && !r; l++) {
    for (int k = 0; k < nch; k++) perm[(size_t)l * nch + k] = c->item_of(chains[k], l);
    if (c->loci[l].d.model == IMA_MODEL_SW) continue;  // its update runs in k_ug_sw
    Batch &b = c->ugb[l];
    std::vector<int32_t> lli(nch, l);
    std::vector<double> lu(nch), lk(nch);
    for (int k = 0; k < nch; k++) {
      lu[k] = u[(size_t)k * nl + l];
      lk[k] = kap[(size_t)k * nl + l];
    }
    r = build_batch(c, b, nch, chains, lli.data(), lu.data(), lk.data(), nullptr, nullptr, precision);
    r = r ? r : init_sumlogk(c, b);
    for (int k = 0; k < nch && !r; k++) reqof[(size_t)l * nch + b.order[k]] = k;
  }
  if (r) return r;
  r = c->cuda(cudaMemcpyAsync(a.rng, rng, nch * sizeof(ima_ug_rng), cudaMemcpyHostToDevice, c->st), "generators");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_chains, chains, nch * 4ul, cudaMemcpyHostToDevice, c->st), "chains");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_reqof, reqof.data(), np * 4, cudaMemcpyHostToDevice, c->st), "requests");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_perm, perm.data(), np * 4, cudaMemcpyHostToDevice, c->st), "genealogy lists");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_evoff, evoff.data(), (ni + 1) * 8ul, cudaMemcpyHostToDevice, c->st), "events");
  r = r ? r : c->cuda(cudaMemcpyAsync(d_ucl, u, np * 8, cudaMemcpyHostToDevice, c->st), "rates");
  if (anysw)
    r = r ? r : c->cuda(cudaMemcpyAsync(d_arange, allele_range, nl * 8ul, cudaMemcpyHostToDevice, c->st), "ranges");
  r = r ? r : c->cuda(cudaMemsetAsync(a.err, 0, 8, c->st), "errors");
  r = r ? r : c->cuda(cudaMemsetAsync(c->d_twerr, 0, 8, c->st), "errors");
  r = r ? r : c->cuda(cudaMemsetAsync(a.nacc, 0, np * 4, c->st), "counts");
  r = r ? r : c->cuda(cudaMemsetAsync(a.ntopo, 0, np * 4, c->st), "counts");
  // the chains' summed weights and integrals from the fresh computation
  // (nomig: [groups][T] counts, [groups][2T] fc then hcc)
  r = r ? r : c->cuda(cudaMemcpyAsync(a.ag_cc, tpd.sc, nch * (size_t)T * 4, cudaMemcpyDeviceToDevice, c->st), "sums");
  r = r ? r : c->cuda(cudaMemcpy2DAsync(a.ag_fc, T * 8ul, tpd.sd, 2 * T * 8ul, T * 8ul, nch, cudaMemcpyDeviceToDevice, c->st), "sums");
  r = r ? r : c->cuda(cudaMemcpy2DAsync(a.ag_hcc, T * 8ul, tpd.sd + T, 2 * T * 8ul, T * 8ul, nch, cudaMemcpyDeviceToDevice, c->st), "sums");
  r = r ? r : c->cuda(cudaMemcpyAsync(a.qint, tpd.q, nch * (size_t)nth * 8, cudaMemcpyDeviceToDevice, c->st), "sums");
  if (r) return r;
  a.chains = d_chains;
  a.items = c->d_items;
  a.nodes = c->d_nodes;
  a.t64 = c->d_t64;
  a.tff = c->d_tff;
  a.pop = c->d_pop;
  a.sched = c->d_sched;
  a.nlev = c->d_nlev;
  a.len = c->d_len;
  a.is_valid = c->d_is_valid;
  a.model = c->d_tw;
  a.tvals = c->d_tvr;
  a.cc = c->tw_cc;
  a.fc = c->tw_fc;
  a.hcc = c->tw_hcc;
  a.ncc = w.cc;
  a.nfc = w.fc;
  a.nhcc = w.hcc;
  a.probg = c->d_probg;
  a.pdg = c->d_pdg;
  a.beta = c->d_beta;
  a.gbeta = gbeta;
  a.logfact = c->d_logfact;
  a.slot32 = c->d_slot32;
  a.fresh32 = c->d_fresh32;
  a.slot64 = c->d_slot64;
  a.fresh64 = c->d_fresh64;
  a.alleles = c->d_al;
  a.dlike = c->d_dlike;
  a.arange = d_arange;
  a.u_cl = d_ucl;
  if (!c->ug_sd) {
    for (cudaStream_t *q : {&c->ug_sw, &c->ug_sw2, &c->ug_sw3, &c->ug_sh, &c->ug_sh2, &c->ug_sd})
      r = r ? r : c->cuda(cudaStreamCreateWithFlags(q, cudaStreamNonBlocking), "streams");
    if (r) return r;
  }
  while ((int)c->ug_ev.size() < 16) {
    cudaEvent_t e;
    r = c->cuda(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "events");
    if (r) return r;
    c->ug_ev.push_back(e);
  }
  cudaEvent_t *evP = c->ug_ev.data(), *evW = evP + 4, *evH = evP + 8, *evD = evP + 12;
  // The steps: one locus of every listed chain at a time.  Each chain's
  // proposals follow one another on st (they share its generator), its
  // decisions on ug_sd (they share its sums); a step's weights (on three
  // streams used by turns) and its likelihoods (on two; consecutive steps
  // touch different loci) wait for its proposal, its decision for both and
  // for the previous decision.  So proposals, weights and likelihoods of
  // the next steps run while a decision does, up to R steps ahead.  After an
  // IS step the next proposal waits for the decision: an IS decision draws
  // the acceptance uniform only when the likelihood does not reject, so the
  // generator's position is known only then (an HKY proposal draws it
  // itself, next in the stream, as the reference always does).
  const UgArgs a0 = a;
  long long step = 0;
  int prev_is = 0;
  for (int s = 0; s < nsweeps && !r; s++)
    for (int l = 0; l < nl && !r; l++, step++) {
      const int slot = (int)(step % R);
      const size_t so = (size_t)slot * nch;
      Batch &b = c->ugb[l];
      UgArgs u_ = a0;
      u_.locus = l;
      u_.hky = c->loci[l].d.model == IMA_MODEL_HKY;
      u_.sw = c->loci[l].d.model == IMA_MODEL_SW;
      u_.predraw = u_.hky || u_.sw;
      u_.req = b.d_req;
      u_.req_of = d_reqof + (size_t)l * nch;
      u_.res = b.d_res;
      u_.st = b.d_st;
      u_.bk_nodes = a0.bk_nodes + so * mx;
      u_.bk_t = a0.bk_t + so * mx;
      u_.bk_pop = a0.bk_pop + so * mx;
      u_.bk_sched = a0.bk_sched + so * mx;
      u_.bk_len = a0.bk_len + so;
      u_.bk_nlev = a0.bk_nlev + so;
      u_.prop = a0.prop + 2 * so;
      u_.slidew = a0.slidew + so;
      u_.ustore = a0.ustore + so;
      u_.edges = a0.edges + 4 * so;
      u_.bk_A = a0.bk_A + so * mx;
      u_.bk_dl = a0.bk_dl + so * mx;
      u_.swnew = a0.swnew + so;
      u_.aterm = a0.aterm + so;
      u_.holdsis = a0.holdsis + so;
      if (step >= R) cudaStreamWaitEvent(c->st, evD[slot], 0);
      if (prev_is) cudaStreamWaitEvent(c->st, evD[(step - 1) % R], 0);
      c->launch(IMA_K_UG, 0.0, [&] { launch_ug_propose(u_, c->st); });
      cudaEventRecord(evP[slot], c->st);
      w.perm = d_perm + (size_t)l * nch;
      cudaStream_t sw = (step % 3 == 0) ? c->ug_sw : (step % 3 == 1 ? c->ug_sw2 : c->ug_sw3);
      cudaStreamWaitEvent(sw, evP[slot], 0);
      int lr = 0;
      c->launch(IMA_K_TREEWEIGHT, 0.0, [&] { lr = launch_treeweight(w, h, sw); }, sw);
      if (lr < 0) return c->fail(IMA_ERR_TOO_LARGE, "treeweight: shared memory for %d events", P);
      c->launches += lr - 1;
      cudaEventRecord(evW[slot], sw);
      cudaStreamWaitEvent(c->ug_sd, evW[slot], 0);
      {  // the likelihood: a stepwise locus's branch terms from its proposal's edges and allele
        cudaStream_t sh = (step & 1) ? c->ug_sh2 : c->ug_sh;
        cudaStreamWaitEvent(sh, evP[slot], 0);
        if (u_.sw) {
          c->launch(IMA_K_UG, 0.0, [&] { launch_ug_sw(u_, sh); }, sh);
        } else {
          if (!u_.hky) cudaStreamWaitEvent(sh, evW[slot], 0);  // the IS likelihood reads the new lengths
          enqueue(c, b, sh);
        }
        cudaEventRecord(evH[slot], sh);
        cudaStreamWaitEvent(c->ug_sd, evH[slot], 0);
      }
      c->launch(IMA_K_UG, 0.0, [&] { launch_ug_decide(u_, c->ug_sd); }, c->ug_sd);
      cudaEventRecord(evD[slot], c->ug_sd);
      prev_is = c->loci[l].d.model == IMA_MODEL_IS;
      r = c->cuda(cudaGetLastError(), "genealogy update launch");
    }
  if (step > 0) cudaStreamWaitEvent(c->st, evD[(step - 1) % R], 0);  // st carries on after the last decision
  // the device's genealogies are newer than the mirror from here on
  for (int k = 0; k < nch; k++) {
    c->topo_lo = std::min(c->topo_lo, chains[k] * nl);
    c->topo_hi = std::max(c->topo_hi, chains[k] * nl + nl - 1);
  }
  dev_newer(c, nch, chains);
  c->tw_ngen = 0;  // the weights of the last weights call no longer describe these genealogies
  c->tw_valid.clear();
  if (r) return r;
  int32_t e[2] = {0, 0};
  r = c->cuda(cudaMemcpyAsync(e, a.err, 8, cudaMemcpyDeviceToHost, c->st), "genealogy update");
  r = r ? r : c->cuda(cudaMemcpyAsync(rng, a.rng, nch * sizeof(ima_ug_rng), cudaMemcpyDeviceToHost, c->st), "generators");
  if (accepted) r = r ? r : c->cuda(cudaMemcpyAsync(accepted, a.nacc, np * 4, cudaMemcpyDeviceToHost, c->st), "counts");
  if (topology) r = r ? r : c->cuda(cudaMemcpyAsync(topology, a.ntopo, np * 4, cudaMemcpyDeviceToHost, c->st), "counts");
  r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "genealogy update");
  r = r ? r : tw_check_err(c, "genealogy update weights");
  if (r) return r;
  if (e[0]) {
    static const char *why[] = {"", "a slide that did not end", "a root time beyond TIMEMAX",
                                "an IS genealogy with a site no edge can carry", "an integral term the reference rejects",
                                "a genealogy that is not a tree"};
    return c->fail(IMA_ERR_DATA, "genealogy update: listed chain %d: %s", e[1], why[e[0] < 6 ? e[0] : 0]);
  }
  if (probg) {
    std::vector<double> all(c->nchains);
    r = c->cuda(cudaMemcpyAsync(all.data(), c->d_probg, c->nchains * 8ul, cudaMemcpyDeviceToHost, c->st), "probg");
    r = r ? r : c->cuda(cudaStreamSynchronize(c->st), "probg");
    for (int k = 0; !r && k < nch; k++) probg[k] = all[chains[k]];
  }
  return r;
}

// ======================================================================
// checkpoints of the resident chain state (resume a run, with the caller's
// generator state, as the reference's .mcf files and seed do)
namespace {
const char CKP_MAGIC[8] = {'I', 'M', 'A', 'C', 'K', 'P', '0', '1'};

struct CkpHeader {
  char magic[8];
  int32_t version, nloci, nchains, nitems;
  int64_t nnodes, nsched, nal;
  int32_t npops, has_labels, locus_pops, has_rng;
  int64_t nmig;
};

struct CkpFile {
  FILE *f = nullptr;
  bool ok = true;
  ~CkpFile() { if (f) fclose(f); }
  void put(const void *p, size_t bytes) { if (ok && bytes && fwrite(p, 1, bytes, f) != bytes) ok = false; }
  void get(void *p, size_t bytes) { if (ok && bytes && fread(p, 1, bytes, f) != bytes) ok = false; }
};

int dev_to_host(ima_ctx *c, void *dst, const void *src, size_t bytes)
{
  if (!bytes) return IMA_OK;
  return c->cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost), "checkpoint");
}
int host_to_dev(ima_ctx *c, void *dst, const void *src, size_t bytes)
{
  if (!bytes) return IMA_OK;
  return c->cuda(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice), "checkpoint");
}
}  // namespace

extern "C" int ima_gpu_checkpoint_write(ima_ctx *c, const char *path, const ima_mt19937 *rng)
{
  if (!c || !path) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first");
  cudaSetDevice(c->device);
  int r = c->cuda(cudaStreamSynchronize(c->st), "checkpoint");
  r = r ? r : sync_mirror(c);
  if (r) return r;
  const size_t ni = c->nitems, nn = c->nnodes;
  CkpHeader h;
  memset(&h, 0, sizeof(h));
  memcpy(h.magic, CKP_MAGIC, 8);
  h.version = 1;
  h.nloci = c->nloci;
  h.nchains = c->nchains;
  h.nitems = c->nitems;
  h.nnodes = (int64_t)nn;
  h.nsched = (int64_t)c->nsched;
  h.nal = (int64_t)c->nal;
  h.npops = c->tw_ready ? c->h_tw.npops : 0;
  h.has_labels = c->d_pop ? 1 : 0;
  h.locus_pops = c->locus_pops ? 1 : 0;
  h.has_rng = rng ? 1 : 0;
  if (h.has_labels)
    for (size_t i = 0; i < ni; i++) h.nmig += c->h_mcnt[i];
  std::vector<double> pdg(ni), probg(c->nchains), beta(c->nchains);
  r = dev_to_host(c, pdg.data(), c->d_pdg, ni * 8);
  r = r ? r : dev_to_host(c, probg.data(), c->d_probg, c->nchains * 8ul);
  r = r ? r : dev_to_host(c, beta.data(), c->d_beta, c->nchains * 8ul);
  if (r) return r;
  CkpFile F;
  F.f = fopen(path, "wb");
  if (!F.f) return c->fail(IMA_ERR_ARG, "cannot write %s", path);
  F.put(&h, sizeof(h));
  for (int li = 0; li < c->nloci; li++) {  // the loci, to check a restore against
    const int32_t sig[3] = {c->loci[li].d.model, c->loci[li].d.n, c->loci[li].d.nsites};
    F.put(sig, sizeof(sig));
  }
  F.put(c->h_nodes, nn * sizeof(NodeRec));
  F.put(c->h_t64, nn * 8);
  {  // the float-float copy the device keeps, as the device makes it
    std::vector<float2> tff(nn);
    for (size_t k = 0; k < nn; k++) {
      const float hi = (float)c->h_t64[k];
      tff[k] = make_float2(hi, (float)(c->h_t64[k] - (double)hi));
    }
    F.put(tff.data(), nn * sizeof(float2));
  }
  F.put(c->h_sched, c->nsched * sizeof(int16_t));
  F.put(c->h_nlev, ni * 4);
  F.put(c->h_len, ni * 8);
  F.put(c->h_pi, 4 * ni * 8);
  F.put(c->h_al, c->nal * 4);
  F.put(c->has_tree.data(), ni);
  F.put(pdg.data(), ni * 8);
  F.put(probg.data(), c->nchains * 8ul);
  F.put(beta.data(), c->nchains * 8ul);
  if (h.has_labels) {
    std::vector<int32_t> pop(nn), moff(nn + ni);
    std::vector<double> mt(c->mig_used);
    std::vector<int32_t> mp(c->mig_used);
    r = dev_to_host(c, pop.data(), c->d_pop, nn * 4);
    r = r ? r : dev_to_host(c, moff.data(), c->d_moff, (nn + ni) * 4);
    r = r ? r : dev_to_host(c, mt.data(), c->d_mig_t, c->mig_used * 8);
    r = r ? r : dev_to_host(c, mp.data(), c->d_mig_p, c->mig_used * 4);
    if (r) return r;
    F.put(pop.data(), nn * 4);
    F.put(moff.data(), (nn + ni) * 4);
    F.put(c->h_mcnt.data(), ni * 4);
    F.put(c->has_labels.data(), ni);
    for (size_t i = 0; i < ni; i++) {  // each item's events, compacted in item order
      F.put(mt.data() + c->h_mbase[i], (size_t)c->h_mcnt[i] * 8);
      F.put(mp.data() + c->h_mbase[i], (size_t)c->h_mcnt[i] * 4);
    }
  }
  if (h.locus_pops) {
    F.put(c->h_hval.data(), c->nloci * 8ul);
    F.put(c->h_samp.data(), c->h_samp.size() * 4);
    F.put(c->h_tvr.data(), c->h_tvr.size() * 8);
  }
  if (rng) F.put(rng, sizeof(ima_mt19937));
  if (!F.ok) return c->fail(IMA_ERR_ARG, "writing %s failed", path);
  return IMA_OK;
}

extern "C" int ima_gpu_checkpoint_read(ima_ctx *c, const char *path, ima_mt19937 *rng)
{
  if (!c || !path) return IMA_ERR_ARG;
  if (!c->nchains) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_chains first (the same loci and chains)");
  cudaSetDevice(c->device);
  CkpFile F;
  F.f = fopen(path, "rb");
  if (!F.f) return c->fail(IMA_ERR_ARG, "cannot read %s", path);
  CkpHeader h;
  F.get(&h, sizeof(h));
  const size_t ni = c->nitems, nn = c->nnodes;
  if (!F.ok || memcmp(h.magic, CKP_MAGIC, 8) || h.version != 1)
    return c->fail(IMA_ERR_DATA, "%s is not a checkpoint of this library", path);
  if (h.nloci != c->nloci || h.nchains != c->nchains || h.nitems != c->nitems || h.nnodes != (int64_t)nn ||
      h.nsched != (int64_t)c->nsched || h.nal != (int64_t)c->nal)
    return c->fail(IMA_ERR_STATE, "checkpoint of %d loci x %d chains does not match this context", h.nloci, h.nchains);
  for (int li = 0; li < c->nloci; li++) {
    int32_t sig[3];
    F.get(sig, sizeof(sig));
    if (!F.ok || sig[0] != c->loci[li].d.model || sig[1] != c->loci[li].d.n || sig[2] != c->loci[li].d.nsites)
      return c->fail(IMA_ERR_STATE, "checkpoint locus %d does not match this context's", li);
  }
  if ((h.has_labels || h.locus_pops) && (!c->tw_ready || c->h_tw.npops != h.npops))
    return c->fail(IMA_ERR_STATE, "set the population model (%d populations) before restoring", h.npops);
  if (h.nmig < 0 || h.npops < 0 || h.npops > TW_MAXPOPS) return c->fail(IMA_ERR_DATA, "%s: bad header", path);
  {  // the whole file must be there before any state is replaced
    size_t want = sizeof(h) + 12ul * c->nloci + nn * (sizeof(NodeRec) + 8 + sizeof(float2)) + c->nsched * 2 +
                  ni * (4 + 8 + 32 + 1 + 8) + c->nal * 4 + c->nchains * 16ul;
    if (h.has_labels) want += nn * 4 + (nn + ni) * 4 + ni * 5 + (size_t)h.nmig * 12;
    if (h.locus_pops) want += c->nloci * (8ul + 4ul * h.npops) + c->nchains * 8ul * (h.npops - 1);
    if (h.has_rng) want += sizeof(ima_mt19937);
    const long here = ftell(F.f);
    if (here < 0 || fseek(F.f, 0, SEEK_END) != 0) return c->fail(IMA_ERR_DATA, "%s: cannot size", path);
    const long end = ftell(F.f);
    if (end < 0 || (size_t)end != want || fseek(F.f, here, SEEK_SET) != 0)
      return c->fail(IMA_ERR_DATA, "%s holds %ld bytes, this context's checkpoint %zu", path, end, want);
  }
  // every section is read into host buffers and checked before any state
  // of the context is replaced: a bad file leaves the context as it was
  std::vector<char> nodes(nn * sizeof(NodeRec)), t64(nn * 8), tff(nn * sizeof(float2)), sched(c->nsched * 2),
      nlev(ni * 4), len(ni * 8), pi(4 * ni * 8), al(c->nal * 4);
  std::vector<uint8_t> has_tree(ni);
  std::vector<double> pdg(ni), probg(c->nchains), beta(c->nchains);
  F.get(nodes.data(), nodes.size());
  F.get(t64.data(), t64.size());
  F.get(tff.data(), tff.size());
  F.get(sched.data(), sched.size());
  F.get(nlev.data(), nlev.size());
  F.get(len.data(), len.size());
  F.get(pi.data(), pi.size());
  F.get(al.data(), al.size());
  F.get(has_tree.data(), ni);
  F.get(pdg.data(), ni * 8);
  F.get(probg.data(), c->nchains * 8ul);
  F.get(beta.data(), c->nchains * 8ul);
  if (!F.ok) return c->fail(IMA_ERR_DATA, "%s is truncated", path);
  std::vector<int32_t> pop, moff, cnt, mp;
  std::vector<uint8_t> has;
  std::vector<double> mt;
  std::vector<long long> base;
  size_t used = 0;
  if (h.has_labels) {
    pop.resize(nn);
    moff.resize(nn + ni);
    cnt.resize(ni);
    has.resize(ni);
    F.get(pop.data(), nn * 4);
    F.get(moff.data(), (nn + ni) * 4);
    F.get(cnt.data(), ni * 4);
    F.get(has.data(), ni);
    if (!F.ok) return c->fail(IMA_ERR_DATA, "%s is truncated", path);
    mt.resize((size_t)h.nmig);
    mp.resize((size_t)h.nmig);
    base.resize(ni);
    for (size_t i = 0; i < ni; i++) {
      if (cnt[i] < 0 || used + cnt[i] > (size_t)h.nmig) return c->fail(IMA_ERR_DATA, "%s: bad event counts", path);
      F.get(mt.data() + used, (size_t)cnt[i] * 8);
      F.get(mp.data() + used, (size_t)cnt[i] * 4);
      base[i] = (long long)used;
      used += cnt[i];
    }
    if (!F.ok) return c->fail(IMA_ERR_DATA, "%s is truncated", path);
    if (used != (size_t)h.nmig)
      return c->fail(IMA_ERR_DATA, "%s: event counts sum to %zu, not %d", path, used, (int)h.nmig);
  }
  std::vector<double> hval, tvr;
  std::vector<int32_t> samp;
  if (h.locus_pops) {
    hval.resize(c->nloci);
    tvr.resize((size_t)c->nchains * (h.npops - 1));
    samp.resize((size_t)c->nloci * h.npops);
    F.get(hval.data(), hval.size() * 8);
    F.get(samp.data(), samp.size() * 4);
    F.get(tvr.data(), tvr.size() * 8);
    if (!F.ok) return c->fail(IMA_ERR_DATA, "%s is truncated", path);
    for (int li = 0; li < c->nloci; li++) {
      int ns = 0;
      for (int p = 0; p < h.npops; p++) ns += samp[(size_t)li * h.npops + p];
      if (!(hval[li] > 0) || ns != c->loci[li].d.n)
        return c->fail(IMA_ERR_DATA, "%s: locus %d populations do not match its %d genes", path, li, c->loci[li].d.n);
    }
  }
  ima_mt19937 g;
  if (h.has_rng) {
    F.get(&g, sizeof(g));
    if (!F.ok) return c->fail(IMA_ERR_DATA, "%s is truncated", path);
  }
  // commit
  int r = c->cuda(cudaStreamSynchronize(c->st), "checkpoint");
  if (r) return r;
  memcpy(c->h_nodes, nodes.data(), nodes.size());
  memcpy(c->h_t64, t64.data(), t64.size());
  // the float-float times are made again from the FP64 ones at the upload
  memcpy(c->h_sched, sched.data(), sched.size());
  memcpy(c->h_nlev, nlev.data(), nlev.size());
  memcpy(c->h_len, len.data(), len.size());
  memcpy(c->h_pi, pi.data(), pi.size());
  memcpy(c->h_al, al.data(), al.size());
  c->has_tree = has_tree;
  c->tree_gen++;
  c->tw_ngen = 0;  // weights of the genealogies replaced here are gone
  c->tw_valid.clear();
  c->dev_lo = INT32_MAX;  // the file is authoritative now
  c->dev_hi = -1;
  c->topo_lo = INT32_MAX;
  c->topo_hi = -1;
  c->lpend_lo = INT32_MAX;
  c->lpend_hi = -1;
  c->dirty_lo = 0;        // upload everything with the next flush
  c->dirty_hi = (int)ni - 1;
  c->tdirty_lo = INT32_MAX;
  c->tdirty_hi = -1;
  c->evkey.valid = false;
  r = flush(c);
  r = r ? r : host_to_dev(c, c->d_pdg, pdg.data(), ni * 8);
  r = r ? r : host_to_dev(c, c->d_probg, probg.data(), c->nchains * 8ul);
  r = r ? r : host_to_dev(c, c->d_beta, beta.data(), c->nchains * 8ul);
  if (r) return r;
  if (h.has_labels) {
    r = labels_alloc(c);
    if (r) return r;
    if (used > c->mig_cap) {
      cudaFree(c->d_mig_t);
      cudaFree(c->d_mig_p);
      c->d_mig_t = dev_alloc<double>(used, c->dev_bytes, c->st);
      c->d_mig_p = dev_alloc<int32_t>(used, c->dev_bytes, c->st);
      if (!c->d_mig_t || !c->d_mig_p) return c->fail(IMA_ERR_NOMEM, "migration events");
      c->mig_cap = used;
    }
    r = host_to_dev(c, c->d_pop, pop.data(), nn * 4);
    r = r ? r : host_to_dev(c, c->d_moff, moff.data(), (nn + ni) * 4);
    r = r ? r : host_to_dev(c, c->d_mbase, base.data(), ni * 8);
    r = r ? r : host_to_dev(c, c->d_mig_t, mt.data(), used * 8);
    r = r ? r : host_to_dev(c, c->d_mig_p, mp.data(), used * 4);
    if (r) return r;
    c->mig_used = used;
    c->h_mbase = base;
    c->h_mcnt = cnt;
    c->h_mcap = cnt;
    c->has_labels = has;
  } else {
    // the restored genealogies come without labels: none of the old ones apply
    c->has_labels.assign(ni, 0);
  }
  if (h.locus_pops) {
    r = ima_gpu_set_locus_pops(c, hval.data(), samp.data());
    if (r) return r;
    c->h_tvr = tvr;
  }
  if (h.has_rng && rng) *rng = g;
  return c->cuda(cudaDeviceSynchronize(), "checkpoint");
}

extern "C" int ima_gpu_get_split_times(ima_ctx *c, double *tvals)
{
  if (!c || !tvals) return IMA_ERR_ARG;
  if (!c->tw_ready || c->h_tvr.empty()) return c->fail(IMA_ERR_STATE, "call ima_gpu_set_locus_pops first");
  memcpy(tvals, c->h_tvr.data(), c->h_tvr.size() * 8);
  return IMA_OK;
}
