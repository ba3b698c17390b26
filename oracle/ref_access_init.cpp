/* ref_access_init.cpp -- compiles the reference initialize.cpp in this
 * translation unit so the harness can run its file-static setup_iparams
 * (initialize.cpp:202-727), which builds the theta and migration parameter
 * maps (itheta/imig wp lists) from the population tree, and its
 * set_nomigrationchecklist (:761-809) (test only). */
#include "initialize.cpp"
#include "ref_access.h"
void refacc_setup_iparams(void) { setup_iparams(); }
/* varrank (the polymorphism rank of each sampled population, which set_uvals
 * fills from the data) for ANCESTRALPOPSIZESSETTOLARGESTSAMPLED */
void refacc_set_varrank(const double *v, int n)
{
  for (int i = 0; i < n; i++) varrank[i] = v[i];
}
void refacc_set_nomigrationchecklist(void) { set_nomigrationchecklist(); }
