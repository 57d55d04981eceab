/* Test-only stand-in for the few GSL interpolation symbols the reference's survey counters call
 * (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:345-361,
 * mocks/DDsmu_mocks/countpairs_s_mu_mocks_impl.c.src:354-370,
 * mocks/vpf_mocks/countspheres_mocks_impl.c.src:316-366).  GSL is not installed here; this header
 * lets oracle/build_ref.py compile those reference sources unchanged, as the checker.
 *
 * Only gsl_interp_linear is provided, restated from GSL 2.x's published linear interpolant:
 * the interval is located by bisection (x_lo <= x < x_hi, the last interval for x at the upper
 * end) and y = y_lo + (x - x_lo) / (x_hi - x_lo) * (y_hi - y_lo).  Points outside the table give
 * NaN, as GSL's domain error does.  Nothing in the product includes this file. */
#ifndef CF_GSL_SHIM_INTERP_H
#define CF_GSL_SHIM_INTERP_H
#include <math.h>
#include <stddef.h>
#include <stdlib.h>

typedef struct {
    const char *name;
    unsigned int min_size;
} gsl_interp_type;

typedef struct {
    const gsl_interp_type *type;
    size_t size;
} gsl_interp;

typedef struct {
    size_t cache; /* last interval found (a hint only: every lookup bisects) */
} gsl_interp_accel;

static const gsl_interp_type cf_shim_interp_linear = {"linear", 2};
#define gsl_interp_linear (&cf_shim_interp_linear)

static inline gsl_interp_accel *gsl_interp_accel_alloc(void) { return (gsl_interp_accel *)calloc(1, sizeof(gsl_interp_accel)); }
static inline void gsl_interp_accel_free(gsl_interp_accel *a) { free(a); }

static inline gsl_interp *gsl_interp_alloc(const gsl_interp_type *T, size_t size)
{
    if (T == NULL || size < T->min_size) return NULL;
    gsl_interp *p = (gsl_interp *)calloc(1, sizeof(gsl_interp));
    if (p) {
        p->type = T;
        p->size = size;
    }
    return p;
}

static inline int gsl_interp_init(gsl_interp *interp, const double xa[], const double ya[], size_t size)
{
    (void)ya;
    if (interp == NULL || size != interp->size) return 1;
    for (size_t k = 1; k < size; k++)
        if (!(xa[k] > xa[k - 1])) return 1; /* abscissae must increase */
    return 0;
}

static inline void gsl_interp_free(gsl_interp *interp) { free(interp); }

static inline double gsl_interp_eval(const gsl_interp *interp, const double xa[], const double ya[], double x,
                                     gsl_interp_accel *a)
{
    const size_t n = interp->size;
    if (!(x >= xa[0] && x <= xa[n - 1])) return NAN;
    size_t lo = 0, hi = n - 1; /* xa[lo] <= x, and x < xa[hi] unless x is the last abscissa */
    while (hi - lo > 1) {
        const size_t mid = lo + (hi - lo) / 2;
        if (x < xa[mid]) hi = mid;
        else lo = mid;
    }
    if (a) a->cache = lo;
    const double x_lo = xa[lo], x_hi = xa[lo + 1], y_lo = ya[lo], y_hi = ya[lo + 1];
    const double dx = x_hi - x_lo;
    if (!(dx > 0.0)) return NAN;
    return y_lo + (x - x_lo) / dx * (y_hi - y_lo);
}
#endif
