/* Exposes the test-only GSL stand-in to the oracle tests (known answers of MT19937, the linear
 * interpolant).  Built by oracle/build_ref.py into oracle/_ref/libcf_gslshim.so. */
#include <stdint.h>
#include "gsl/gsl_interp.h"
#include "gsl/gsl_rng.h"

uint32_t cf_shim_mt_nth(unsigned long seed, int n)
{
    gsl_rng *r = gsl_rng_alloc(gsl_rng_mt19937);
    gsl_rng_set(r, seed);
    uint32_t v = 0;
    for (int k = 0; k < n; k++) v = cf_shim_mt_next(r);
    gsl_rng_free(r);
    return v;
}

double cf_shim_interp(const double *xa, const double *ya, int n, double x)
{
    gsl_interp *p = gsl_interp_alloc(gsl_interp_linear, (size_t)n);
    gsl_interp_accel *a = gsl_interp_accel_alloc();
    double y = NAN;
    if (p && gsl_interp_init(p, xa, ya, (size_t)n) == 0) y = gsl_interp_eval(p, xa, ya, x, a);
    gsl_interp_free(p);
    gsl_interp_accel_free(a);
    return y;
}
