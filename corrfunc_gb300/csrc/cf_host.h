/* cf_host.h -- host-side helpers (cf_common.c) used by the public entry points. */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

int cf_setup_bins(const char *fname, double *rmin, double *rmax, int *nbin, double **rupp);
void cf_formula_for_isa(int isa, int *fma_formula, int *chord_formula);
int64_t cf_getnumlines(const char *fname, char comment);
/* get_binsize (utils/gridlink_utils.c.src:31-49): cells per axis and their size */
int cf_ref_binsize(double xdiff, double xwrap, double rmax, int refine, int max_cells, double *binsize, int *nmesh);

/* MT19937 (Matsumoto & Nishimura 1998) with the 2002 seeding, seed 0 replaced by 4357: the
 * generator the reference takes from GSL (gsl_rng_mt19937, theory/vpf/countspheres_impl.c.src:188-190).
 * cf_mt_uniform returns the next 32-bit output / 2^32, as gsl_rng_uniform does for it. */
typedef struct {
    uint32_t mt[624];
    int mti;
} cf_mt19937;
void cf_mt_seed(cf_mt19937 *g, unsigned long seed);
uint32_t cf_mt_next(cf_mt19937 *g);
double cf_mt_uniform(cf_mt19937 *g);

#ifdef __cplusplus
}
#endif
