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
