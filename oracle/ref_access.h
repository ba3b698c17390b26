/* ref_access.h -- accessors for reference file statics (test infrastructure). */
#ifndef REF_ACCESS_H
#define REF_ACCESS_H
double refacc_sumlogk(int li);
void refacc_jointp_setup(int nparams_total, int modeltype);
double refacc_jointp(double *x, double *ess);
void refacc_modelloop(int nparams_total, int modeltype, const double *upper, int multiplier,
                      const double *xmap, int nested_params, double *best_out, double *ess_out);
double refacc_icoal(int cc, double fc, double hcc, double max, double min);
double refacc_imig(int cm, double fm, double max, double min);
double refacc_imig_expo(int cm, double fm, double mean);
void refacc_setup_iparams(void);
void refacc_set_varrank(const double *v, int n);
void refacc_set_nomigrationchecklist(void);
double refacc_marginp(int param, int firsttree, int lasttree, double x);
#endif
