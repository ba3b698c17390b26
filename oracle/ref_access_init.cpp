/* ref_access_init.cpp -- compiles the reference initialize.cpp in this
 * translation unit so the harness can run its file-static setup_iparams
 * (initialize.cpp:202-727), which builds the theta and migration parameter
 * maps (itheta/imig wp lists) from the population tree (test only). */
#include "initialize.cpp"
#include "ref_access.h"
void refacc_setup_iparams(void) { setup_iparams(); }
