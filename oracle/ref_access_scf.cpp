/* ref_access_scf.cpp -- compiles the reference surface_call_functions.cpp in
 * this translation unit so the harness can call its static marginp (test
 * only). */
#include "surface_call_functions.cpp"
#include "ref_access.h"
double refacc_marginp(int param, int firsttree, int lasttree, double x) { return marginp(param, firsttree, lasttree, x, 0); }
