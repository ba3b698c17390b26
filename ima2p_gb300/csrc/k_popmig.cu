// k_popmig.cu -- posterior densities of the population migration rate
// 2NM = theta_i m_j / 2 over the loaded genealogies: calc_popmig and, under
// an exponential migration prior, calc_pop_expomig (popmig.cpp:9-172), the
// functions print_populationmigrationrate_histograms evaluates on its grids
// (histograms.cpp:755-810).
//
// Every genealogy contributes a term with one or two incomplete gamma
// functions of x (igamma.cuh), so the work is FP64-issue bound: tens to
// hundreds of FP64 operations per (point, genealogy) pair, with iteration
// counts that vary with x.  A CTA is one warp: 32 requested points and one
// chunk of genealogies, which every lane walks in genealogy order reading
// the seven columns it needs straight from the rows (the addresses are the
// same across the warp, one broadcast load each; the rows stay in L2).  No
// barriers tie warps of unequal work together, and the grid holds many
// waves of these small CTAs so that the block scheduler balances the SMs.
// Each (point, chunk) partial has its own slot.  calc_popmig's sum
// of exp(temp1 + temp2) (terms outside +-700 skipped) is kept per chunk;
// calc_pop_expomig's eexp mantissa / decimal-exponent terms are kept per
// chunk rescaled to the chunk's largest exponent.  The merge kernel adds the
// chunks in chunk order, rescales them to the overall largest exponent, and
// divides by G and, for likelihoods, by the prior density of 2NM.  The peak
// search's forms (marginpopmig, marginpop_expomig; :181-351) sum a range of
// genealogies and divide by its length (+1 when it starts at genealogy 0).
//
// The terms are written with the reference's operation order and this file
// is compiled with -fmad=false; log, exp and pow are the device's.
#include "internal.h"
#include "igamma.cuh"
#include "eexp.cuh"

namespace {

constexpr int PM_BS = 32;  // points per CTA (one warp)
constexpr double LOG10 = 2.3025850929940456840;
constexpr int OCUTOFF = 10;

// calc_popmig's term for one genealogy (popmig.cpp:33-84): temp1 + temp2, or
// NaN when the reference would skip it.
__device__ double popmig_term(IgBase &ig, int cc, double fc, double hc, int mc, double fm, double qintg,
                              double mintg, double x, double qmax, double mmax)
{
  double temp1, temp2;
  if (fc == 0 && cc == 0 && fm > 0) {
    temp1 = LOG2 - (mc * log(fm)) - hc - qintg - mintg;
    temp2 = log(exp(ig.upper(mc, 2 * fm * x / qmax)) - exp(ig.upper(mc, mmax * fm)));
  } else if (fm == 0 && mc == 0 && fc > 0) {
    temp1 = LOG2 - (cc * log(fc)) - hc - qintg - mintg;
    temp2 = log(exp(ig.upper(cc, 2 * fc / qmax)) - exp(ig.upper(cc, fc * mmax / x)));
  } else if (fc == 0 && cc == 0 && mc == 0 && fm == 0) {
    temp1 = log(2 * log(mmax * qmax / (2 * x))) - hc - qintg - mintg;
    temp2 = 0;
  } else {
    temp1 = LOG2 + (mc * log(x)) - ((cc + mc) * log(fc + fm * x)) - hc - qintg - mintg;
    double a = ig.upper(cc + mc, 2 * (fc + fm * x) / qmax);
    double b = ig.upper(cc + mc, mmax * (fm + fc / x));
    if (a == b) {  // both saturated: the lower functions separate them
      b = ig.lower(cc + mc, 2 * (fc + fm * x) / qmax);
      a = ig.lower(cc + mc, mmax * (fm + fc / x));
    }
    if (a > b) {
      temp2 = ig.logdiff(a, b);
    } else {
      temp1 = temp2 = 0.0;  // the reference adds exp(0) for these
    }
  }
  return temp1 + temp2;
}

// calc_pop_expomig's log term for one genealogy (popmig.cpp:114-147).
__device__ double popexpo_term(IgBase &ig, int cc, double fc, double hc, int mc, double fm, double qintg,
                               double mintg, double x, double qmax, double mmean)
{
  const double temp1 = x + fc * mmean + fm * mmean * x;
  double temp2 = LOG2 - hc - log(mmean) - qintg - mintg;
  double temp3 = 2 * temp1 / (mmean * qmax);
  if (mc == 0 && cc == 0) {
    temp3 = ig.upper(0, temp3);
    temp2 += temp3;
  } else if (cc == 0) {
    temp3 = ig.upper(mc, temp3);
    temp2 += temp3 - mc * log(fm + 1 / mmean);
  } else if (mc == 0) {
    temp3 = ig.upper(cc, temp3);
    temp2 += temp3 + -cc * log(fc + x * (fm + 1 / mmean));
  } else {
    temp3 = ig.upper(mc + cc, temp3);
    temp2 += temp3 - cc * log(x) + (cc + mc) * log(mmean * x / temp1);
  }
  return temp2;
}

__global__ void __launch_bounds__(PM_BS) k_popmig(PopmigArgs a, int chunk, double *part)
{
  const int k = blockIdx.x * PM_BS + threadIdx.x;
  if (k >= a.n) return;
  const int th = a.thetai[k], mi = a.mi[k];
  const double x = a.x[k], qmax = a.qmax[k], mmax = a.mmax[k];
  const double mmean = a.expo ? a.mmean[k] : 1.0;
  const float *c_cc = a.rows + a.ccp + th, *c_fc = a.rows + a.fcp + th, *c_hc = a.rows + a.hccp + th;
  const float *c_qi = a.rows + a.qip + th, *c_mc = a.rows + a.mcp + mi, *c_fm = a.rows + a.fmp + mi;
  const float *c_mi = a.rows + a.mip + mi;
  IgBase ig{a.logfact, 0};
  double sum = 0.0;        // calc_popmig: sum of exp; expo: sum of m 10^(z - (maxz - OCUTOFF))
  int maxz = -1000000000;  // expo: the chunk's largest decimal exponent
  const int g0 = a.g_lo + blockIdx.y * chunk, g1 = min(a.g_hi, g0 + chunk);
  for (int g = g0; g < g1; g++) {
    const size_t o = (size_t)g * a.rowlen;
    const int cc = (int)__ldg(c_cc + o), mc = (int)__ldg(c_mc + o);
    const double fc = __ldg(c_fc + o), hc = __ldg(c_hc + o), fm = __ldg(c_fm + o);
    const double qintg = __ldg(c_qi + o), mintg = __ldg(c_mi + o);
    if (!a.expo) {
      const double t = popmig_term(ig, cc, fc, hc, mc, fm, qintg, mintg, x, qmax, mmax);
      if (t < 700 && t > -700) sum += exp(t);
    } else {
      const double t = popexpo_term(ig, cc, fc, hc, mc, fm, qintg, mintg, x, qmax, mmean);
      double m;
      int z;
      eexp_dev(t, &m, &z);
      if (z > maxz) {  // a new largest exponent: earlier terms rescale to it
        if (sum != 0.0) sum *= pow(10.0, (double)(maxz - z));
        maxz = z;
      }
      sum += m * pow(10.0, (double)(z - (maxz - OCUTOFF)));
    }
  }
  const size_t o = (size_t)k * gridDim.y + blockIdx.y;
  part[2 * o] = sum;
  part[2 * o + 1] = (double)maxz;
  if (ig.st) atomicCAS(a.err, 0, ig.st);
}

__global__ void k_popmig_merge(PopmigArgs a, int nchunks, const double *part, double *out)
{
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= a.n) return;
  const double *w = part + 2 * (size_t)k * nchunks;
  const double x = a.x[k], qmax = a.qmax[k], mmax = a.mmax[k];
  double sum = 0.0;
  if (!a.expo) {
    for (int c = 0; c < nchunks; c++) sum += w[2 * c];
    sum /= a.div;
    if (a.prob_or_like) {
      const double temp = 2 * (log(qmax) + log(mmax) - log(2 * x)) / (qmax * mmax);
      sum /= temp;
    }
  } else {
    const double mmean = a.mmean[k];
    int maxz = -1000000000;
    for (int c = 0; c < nchunks; c++) maxz = max(maxz, (int)w[2 * c + 1]);
    double acumm = 0.0;
    for (int c = 0; c < nchunks; c++)
      if (w[2 * c] != 0.0) acumm += w[2 * c] * pow(10.0, (double)((int)w[2 * c + 1] - maxz));
    sum = log(acumm) + (maxz - OCUTOFF) * LOG10;
    sum -= log(a.div);
    sum = exp(sum);
    if (a.prob_or_like) {
      IgBase ig{a.logfact, 0};
      const double temp = 2 * exp(ig.upper(0, 2 * x / (mmean * qmax))) / (qmax * mmean);
      sum /= temp;
      if (ig.st) atomicCAS(a.err, 0, ig.st);
    }
  }
  out[k] = sum;
}

}  // namespace

int popmig_chunks(int G, int n)
{
  // about 16 waves of one-warp CTAs (20 resident per SM at 96 registers),
  // chunks of at least 64 genealogies
  const long long rblocks = (n + PM_BS - 1) / PM_BS;
  long long nchunks = (16LL * 152 * 20 + rblocks - 1) / rblocks;
  const long long maxc = (G + 63) / 64;
  if (nchunks > maxc) nchunks = maxc;
  if (nchunks > 65535) nchunks = 65535;  // grid y limit
  return nchunks < 1 ? 1 : (int)nchunks;
}

int launch_popmig(const PopmigArgs &a, double *part, int nchunks, double *out, cudaStream_t st)
{
  const int ng = a.g_hi - a.g_lo;
  if (a.n < 1 || ng < 1) return 2;
  const int chunk = (ng + nchunks - 1) / nchunks;
  nchunks = (ng + chunk - 1) / chunk;
  k_popmig<<<dim3((a.n + PM_BS - 1) / PM_BS, nchunks), PM_BS, 0, st>>>(a, chunk, part);
  k_popmig_merge<<<(a.n + 127) / 128, 128, 0, st>>>(a, nchunks, part, out);
  return 0;
}
