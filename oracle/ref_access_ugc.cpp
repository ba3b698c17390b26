/* ref_access_ugc.cpp -- compiles the reference update_gtree_common.cpp in
 * this translation unit so the harness can call its file-static integral
 * terms (integrate_coalescent_term, integrate_migration_term,
 * integrate_migration_term_expo_prior; update_gtree_common.cpp:108-304)
 * directly (test only). */
#include "update_gtree_common.cpp"
#include "ref_access.h"
double refacc_icoal(int cc, double fc, double hcc, double max, double min)
{
  return integrate_coalescent_term(cc, fc, hcc, max, min);
}
double refacc_imig(int cm, double fm, double max, double min)
{
  return integrate_migration_term(cm, fm, max, min);
}
double refacc_imig_expo(int cm, double fm, double mean)
{
  return integrate_migration_term_expo_prior(cm, fm, mean);
}
