/* ref_access_jf.cpp -- compiles the reference jointfind.cpp in this
 * translation unit so the harness can set jointp's model range (test only). */
#include "jointfind.cpp"
#include "ref_access.h"
void refacc_jointp_setup(int nparams_total, int modeltype)
{
  nparams = nparams_total;
  nowmodeltype = modeltype;
  nparamrange[0] = (modeltype == 2) ? numpopsizeparams : 0;
  nparamrange[1] = (modeltype == 1) ? numpopsizeparams : nparams_total;
  setuplist();
}
double refacc_jointp(double *x, double *ess) { return jointp(x, 1, ess); }

/* modelloop (jointfind.cpp:746-812) for one model: bounds as setbounds
 * (:578-590) would set them from the priors' maxima; xmap (NULL = the model
 * itself) describes a nested model as setup_mapping would (:115-130). */
void refacc_modelloop(int nparams_total, int modeltype, const double *upper, int multiplier,
                      const double *xmap, int nested_params, double *best_out, double *ess_out)
{
  nparams = nparams_total;
  nowmodeltype = modeltype;
  nparamrange[0] = (modeltype == 2) ? numpopsizeparams : 0;
  nparamrange[1] = (modeltype == 1) ? numpopsizeparams : nparams_total;
  bestvals = static_cast<double *>(malloc((nparams + 1) * sizeof(double)));
  parameter_lower_bound = static_cast<double *>(malloc(nparams * sizeof(double)));
  parameter_upper_bound = static_cast<double *>(malloc(nparams * sizeof(double)));
  for (int i = 0; i < nparams; i++) {
    parameter_lower_bound[i] = MINPARAMVAL;
    parameter_upper_bound[i] = upper[i];
  }
  popsizemultiplier = multiplier;
  depopsize = nparams * popsizemultiplier;
  pop = alt2d_alloc2Ddouble(depopsize, nparams + 1);
  trialpop = alt2d_alloc2Ddouble(depopsize, nparams + 1);
  popnest = static_cast<double *>(malloc(nparams * sizeof(double)));
  calculate_ess = 0;
  int mi = -1;
  if (xmap) {
    for (int i = 0; i < nparams; i++) holdxmaps[0][i] = xmap[i];
    nparams_nested[0] = nested_params;
    fullmodeltype[0] = modeltype;
    mi = 0;
  }
  modelloop(mi);
  if (xmap) {
    mapvals(bestvals, popnest, holdxmaps[0]);
    for (int i = 0; i < nparams; i++) best_out[i] = popnest[i];
  } else {
    for (int i = 0; i < nparams; i++) best_out[i] = bestvals[i];
  }
  best_out[nparams] = bestvals[nparams];
  *ess_out = effective_sample_size;
}
