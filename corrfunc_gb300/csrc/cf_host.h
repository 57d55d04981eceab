/* cf_host.h -- host-side helpers (cf_common.c) used by the public entry points. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int cf_setup_bins(const char *fname, double *rmin, double *rmax, int *nbin, double **rupp);
void cf_formula_for_isa(int isa, int *fma_formula, int *chord_formula);

#ifdef __cplusplus
}
#endif
