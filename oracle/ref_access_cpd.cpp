/* ref_access_cpd.cpp -- compiles the reference calc_prob_data.cpp in this
 * translation unit so the harness can read its sumlogk cache (test only). */
#include "calc_prob_data.cpp"
#include "ref_access.h"
double refacc_sumlogk(int li) { return sumlogk[li] ? *sumlogk[li] : 0.0; }
