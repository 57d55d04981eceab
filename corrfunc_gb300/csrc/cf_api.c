/*
 * cf_api.c -- the six public pair-counting entry points (C ABI of libcorrfunc_gb300.so).
 *
 * Each function keeps the reference's prototype, validation, side effects on the options
 * struct and result packing; the pair counting itself is handed to the CUDA engine
 * (cf_engine_run).  Finalisation (auto-correlation doubling, self pairs, averages, xi / wp
 * from the analytic random counts) follows the reference drivers cited per function.
 * All arithmetic after counting is double precision, also for float inputs.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stddef.h>
#include <stdint.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/time.h>
#include <time.h>

#include "corrfunc_gb300.h"
#include "cf_internal.h"
#include "cf_host.h"

/* per-task timings are handed over as the reference's per cell-pair records */
_Static_assert(sizeof(cf_task_time) == sizeof(struct api_cell_timings), "task timing layout");
_Static_assert(offsetof(cf_task_time, warp) == offsetof(struct api_cell_timings, tid), "task timing layout");

static double wall_now(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_REALTIME, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define CF_ERR(...)                         \
    do {                                    \
        fprintf(stderr, "Error: " __VA_ARGS__); \
        fprintf(stderr, "\n");              \
    } while (0)

/* float_type and API version checks (theory/DD/countpairs.c:46-55) */
static int check_options(const struct config_options *options, const char *fn)
{
    if (options == NULL) {
        CF_ERR("In %s> options can not be NULL", fn);
        return EXIT_FAILURE;
    }
    if (!(options->float_type == sizeof(float) || options->float_type == sizeof(double))) {
        CF_ERR("In %s> Can only handle doubles or floats. Got an array of size = %zu", fn, options->float_type);
        return EXIT_FAILURE;
    }
    if (strncmp(options->version, CF_API_VERSION, sizeof(options->version) - 1) != 0) {
        CF_ERR("Do not know this API version = `%s'. Expected version = `%s'", options->version, CF_API_VERSION);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

/* max_cells / refine-factor sanitation done at the top of every theory driver
 * (theory/DD/countpairs_impl.c.src:175-189) */
static void sanitize_lattice_options(struct config_options *options)
{
    if (options->max_cells_per_dim == 0) {
        fprintf(stderr, "Warning: Max. cells per dimension is set to 0 - resetting to `NLATMAX' = %d\n", NLATMAX);
        options->max_cells_per_dim = NLATMAX;
    }
    for (int i = 0; i < 3; i++) {
        if (options->bin_refine_factors[i] < 1) {
            fprintf(stderr, "Warning: bin refine factor along axis = %d *must* be >=1. Instead found bin refine factor =%d\n",
                    i, options->bin_refine_factors[i]);
            reset_bin_refine_factors(options);
            break;
        }
    }
}

static double wval(const void *w, int64_t j, size_t es)
{
    return es == sizeof(float) ? (double)((const float *)w)[j] : ((const double *)w)[j];
}

static double self_weight_sum(const void *w, int64_t n, size_t es)
{
    double s = 0.0;
    for (int64_t j = 0; j < n; j++) {
        const double v = wval(w, j, es);
        s += v * v;
    }
    return s;
}

static void fill_rule_box(cf_refrule *R, const struct config_options *options, double boxsize, double sx, double sz,
                          int dfl_kind, int64_t np1)
{
    memset(R, 0, sizeof(*R));
    R->kind = CF_REF_BOX;
    R->periodic = 1;
    R->boxsize[0] = R->boxsize[1] = R->boxsize[2] = boxsize;
    R->max_size[0] = sx;
    R->max_size[1] = sx;
    R->max_size[2] = sz;
    for (int a = 0; a < 3; a++) R->refine[a] = options->bin_refine_factors[a];
    R->custom_refine = (options->binning_flags & BINNING_REF_MASK) == BINNING_CUST;
    R->max_cells = options->max_cells_per_dim;
    R->dfl_kind = dfl_kind;
    R->boost_kind = CF_BOOST_XY;
    R->np1 = np1;
}

static int alloc_hist(cf_hist *H, int nbins)
{
    H->nbins = nbins;
    H->npairs = calloc((size_t)nbins, sizeof(uint64_t));
    H->avg = calloc((size_t)nbins, sizeof(double));
    H->wsum = calloc((size_t)nbins, sizeof(double));
    if (!H->npairs || !H->avg || !H->wsum) {
        free(H->npairs);
        free(H->avg);
        free(H->wsum);
        CF_ERR("could not allocate %d histogram bins", nbins);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

static void free_hist(cf_hist *H)
{
    free(H->npairs);
    free(H->avg);
    free(H->wsum);
    H->npairs = NULL;
    H->avg = NULL;
    H->wsum = NULL;
}

/* Finalisation common to all drivers: x2 for auto-correlations, self pairs when the first
 * bin starts at zero (count into self_idx, weights into flat bin 1 exactly as the reference
 * does, e.g. theory/DDrppi/countpairs_rp_pi_impl.c.src:603-642), then averages. */
static void finalize_hist(cf_hist *H, int autocorr, int first_edge_is_zero, int self_idx, int64_t n1, double self_w,
                          int need_avg, int need_w, int div_start)
{
    if (autocorr) {
        for (int i = 0; i < H->nbins; i++) {
            H->npairs[i] *= 2;
            H->avg[i] *= 2.0;
            H->wsum[i] *= 2.0;
        }
        if (first_edge_is_zero) {
            H->npairs[self_idx] += (uint64_t)n1;
            if (need_w) H->wsum[1] += self_w;
        }
    }
    for (int i = div_start; i < H->nbins; i++) {
        if (H->npairs[i] > 0) {
            if (need_avg) H->avg[i] /= (double)H->npairs[i];
            if (need_w) H->wsum[i] /= (double)H->npairs[i];
        }
    }
}

static void init_job(cf_job *J, const struct config_options *options, int mode, int autocorr)
{
    memset(J, 0, sizeof(*J));
    J->mode = mode;
    J->autocorr = autocorr;
    J->precision = cf_engine_get_precision();
    cf_formula_for_isa(options->instruction_set, &J->fma_formula, &J->chord_formula);
    J->elem_size = (int)options->float_type;
    J->need_avg = options->need_avg_sep ? 1 : 0;
}

static int read_bins(const char *binfile, double **rupp, int *nbin, double *rmin, double *rmax)
{
    if (cf_setup_bins(binfile, rmin, rmax, nbin, rupp) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!(*rmin >= 0.0 && *rmax > 0.0 && *rmin < *rmax && *nbin > 0)) {
        CF_ERR("Could not setup with R bins correctly. (rmin = %lf, rmax = %lf, with nbins = %d). "
               "Expected non-zero rmin/rmax with rmax > rmin and nbins >=1 ",
               *rmin, *rmax, *nbin);
        free(*rupp);
        *rupp = NULL;
        return EXIT_FAILURE;
    }
    if (*nbin > CF_MAX_EDGES) {
        CF_ERR("at most %d bins are supported (got %d)", CF_MAX_EDGES - 1, *nbin - 1);
        free(*rupp);
        *rupp = NULL;
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

static int check_weights(const struct extra_options *extra, int autocorr)
{
    if (extra->weight_method == NONE) return EXIT_SUCCESS;
    if (extra->weight_method != PAIR_PRODUCT) {
        CF_ERR("unknown weight method %d", (int)extra->weight_method);
        return EXIT_FAILURE;
    }
    if (extra->weights0.weights[0] == NULL || (!autocorr && extra->weights1.weights[0] == NULL)) {
        CF_ERR("pair_product weighting needs one weight array per particle set");
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

/* ========================= countpairs (DD) ========================= */
/* theory/DD/countpairs.c:34-77 + theory/DD/countpairs_impl.c.src:136-707 */
static int countpairs_impl(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2, void *Y2,
                           void *Z2, const int numthreads, const int autocorr, const char *binfile,
                           results_countpairs *results, struct config_options *options, struct extra_options *extra,
                           int on_device)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d. Expected to receive either 1 (auto-correlations) or 0 (cross-correlations)", autocorr);
        return EXIT_FAILURE;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    double *rupp = NULL, rmin, rmax;
    int nbin;
    if (read_bins(binfile, &rupp, &nbin, &rmin, &rmax) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (options->periodic && options->boxsize == BOXSIZE_NOTGIVEN) {
        fprintf(stderr, "boxsize = %g must be specified with periodic wrap. Please specify a non-zero boxsize, or zero to "
                        "detect the particle extent, or -1 to make a dimension non-periodic.\n", options->boxsize);
        free(rupp);
        return EXIT_FAILURE;
    }
    cf_job J;
    init_job(&J, options, CF_MODE_R3, autocorr);
    J.inputs_on_device = on_device;
    J.n1 = ND1;
    J.n2 = autocorr ? ND1 : ND2;
    J.x1 = X1; J.y1 = Y1; J.z1 = Z1;
    J.x2 = autocorr ? X1 : X2; J.y2 = autocorr ? Y1 : Y2; J.z2 = autocorr ? Z1 : Z2;
    J.need_weight = need_w;
    J.w1 = need_w ? extra->weights0.weights[0] : NULL;
    J.w2 = need_w ? (autocorr ? extra->weights0.weights[0] : extra->weights1.weights[0]) : NULL;
    cf_fill_rule_extent(&J.rule, options, rmax, rmax, rmax, CF_DFL_PER_AXIS, CF_BOOST_XY, ND1);
    J.rmax_xy = J.rmax_z = J.rmax_3d = rmax;
    J.nedges = nbin;
    for (int i = 0; i < nbin; i++) J.edges[i] = rupp[i] * rupp[i];
    cf_hist H;
    if (alloc_hist(&H, nbin) != EXIT_SUCCESS) {
        free(rupp);
        return EXIT_FAILURE;
    }
    if (cf_engine_run(&J, &H) != EXIT_SUCCESS) {
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    double self_w = 0.0;
    if (autocorr && need_w && rupp[0] <= 0.0) {
        if (on_device) {
            void *hw = malloc(options->float_type * (size_t)(ND1 > 0 ? ND1 : 1));
            if (hw == NULL || cf_engine_copy_to_host(hw, J.w1, options->float_type * (size_t)ND1) != EXIT_SUCCESS) {
                free(hw);
                free_hist(&H);
                free(rupp);
                return EXIT_FAILURE;
            }
            self_w = self_weight_sum(hw, ND1, options->float_type);
            free(hw);
        } else {
            self_w = self_weight_sum(J.w1, ND1, options->float_type);
        }
    }
    finalize_hist(&H, autocorr, rupp[0] <= 0.0, 1, ND1, self_w, options->need_avg_sep, need_w, 0);
    results->nbin = nbin;
    results->npairs = malloc(sizeof(uint64_t) * nbin);
    results->rupp = malloc(sizeof(double) * nbin);
    results->rpavg = calloc(nbin, sizeof(double));
    results->weightavg = calloc(nbin, sizeof(double));
    if (!results->npairs || !results->rupp || !results->rpavg || !results->weightavg) {
        free_results(results);
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    for (int i = 0; i < nbin; i++) {
        results->npairs[i] = H.npairs[i];
        results->rupp[i] = rupp[i];
        results->rpavg[i] = options->need_avg_sep ? H.avg[i] : 0.0;
        results->weightavg[i] = need_w ? H.wsum[i] : 0.0;
    }
    free_hist(&H);
    free(rupp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

int countpairs(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2, void *Y2, void *Z2,
               const int numthreads, const int autocorr, const char *binfile, results_countpairs *results,
               struct config_options *options, struct extra_options *extra)
{
    return countpairs_impl(ND1, X1, Y1, Z1, ND2, X2, Y2, Z2, numthreads, autocorr, binfile, results, options, extra, 0);
}

int cf_gpu_countpairs_device(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2, void *Y2,
                             void *Z2, const int numthreads, const int autocorr, const char *binfile,
                             results_countpairs *results, struct config_options *options,
                             struct extra_options *extra)
{
    return countpairs_impl(ND1, X1, Y1, Z1, ND2, X2, Y2, Z2, numthreads, autocorr, binfile, results, options, extra, 1);
}

/* ========================= batched DD cross-correlations ========================= */
/* No reference counterpart: many countpairs(autocorr = 0) calls against one set-2 catalogue,
 * planned once and replayed as one CUDA graph. */
struct cf_gpu_batch {
    cf_batch *eng;
    int nbatch;
    int nbin;
    double *rupp;
    int need_avg;
    int need_w;
};

int cf_gpu_batch_plan(const int nbatch, const int64_t *ND1, void *const *X1, void *const *Y1, void *const *Z1,
                      void *const *W1, const int64_t ND2, void *X2, void *Y2, void *Z2, void *W2, const char *binfile,
                      struct config_options *options, const int weight_method, const int autotune,
                      cf_gpu_batch **plan)
{
    if (plan == NULL) return EXIT_FAILURE;
    *plan = NULL;
    if (check_options(options, __func__) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (nbatch < 1 || ND1 == NULL || X1 == NULL || Y1 == NULL || Z1 == NULL) {
        CF_ERR("a batch needs at least one set-1 catalogue");
        return EXIT_FAILURE;
    }
    if (weight_method != NONE && weight_method != PAIR_PRODUCT) {
        CF_ERR("unknown weight method %d", weight_method);
        return EXIT_FAILURE;
    }
    const int need_w = weight_method == PAIR_PRODUCT;
    if (need_w && (W1 == NULL || W2 == NULL)) {
        CF_ERR("pair_product weighting needs one weight array per particle set");
        return EXIT_FAILURE;
    }
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    double *rupp = NULL, rmin, rmax;
    int nbin;
    if (read_bins(binfile, &rupp, &nbin, &rmin, &rmax) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (options->periodic && options->boxsize == BOXSIZE_NOTGIVEN) {
        fprintf(stderr, "boxsize = %g must be specified with periodic wrap. Please specify a non-zero boxsize, or zero to "
                        "detect the particle extent, or -1 to make a dimension non-periodic.\n", options->boxsize);
        free(rupp);
        return EXIT_FAILURE;
    }
    cf_job J;
    init_job(&J, options, CF_MODE_R3, 0);
    J.inputs_on_device = 1;
    J.n1 = ND1[0];
    J.n2 = ND2;
    J.x2 = X2; J.y2 = Y2; J.z2 = Z2;
    J.need_weight = need_w;
    J.w2 = need_w ? W2 : NULL;
    cf_fill_rule_extent(&J.rule, options, rmax, rmax, rmax, CF_DFL_PER_AXIS, CF_BOOST_XY, ND1[0]);
    J.rmax_xy = J.rmax_z = J.rmax_3d = rmax;
    J.nedges = nbin;
    for (int i = 0; i < nbin; i++) J.edges[i] = rupp[i] * rupp[i];
    cf_gpu_batch *P = calloc(1, sizeof(cf_gpu_batch));
    if (P == NULL) {
        free(rupp);
        return EXIT_FAILURE;
    }
    if (cf_engine_batch_plan(&J, nbatch, ND1, (const void *const *)X1, (const void *const *)Y1,
                             (const void *const *)Z1, need_w ? (const void *const *)W1 : NULL, autotune,
                             &P->eng) != EXIT_SUCCESS) {
        free(P);
        free(rupp);
        return EXIT_FAILURE;
    }
    P->nbatch = nbatch;
    P->nbin = nbin;
    P->rupp = rupp;
    P->need_avg = options->need_avg_sep ? 1 : 0;
    P->need_w = need_w;
    reset_bin_refine_factors(options);
    *plan = P;
    return EXIT_SUCCESS;
}

int cf_gpu_batch_run(cf_gpu_batch *plan, results_countpairs *results)
{
    if (plan == NULL || results == NULL) return EXIT_FAILURE;
    const int nb = plan->nbatch, nbin = plan->nbin;
    cf_hist *H = calloc((size_t)nb, sizeof(cf_hist));
    if (H == NULL) return EXIT_FAILURE;
    int rc = EXIT_SUCCESS;
    for (int b = 0; b < nb && rc == EXIT_SUCCESS; b++) rc = alloc_hist(&H[b], nbin);
    if (rc == EXIT_SUCCESS) rc = cf_engine_batch_run(plan->eng, H);
    for (int b = 0; b < nb; b++) {
        results[b].npairs = NULL;
        results[b].rupp = NULL;
        results[b].rpavg = NULL;
        results[b].weightavg = NULL;
        results[b].nbin = 0;
    }
    for (int b = 0; b < nb && rc == EXIT_SUCCESS; b++) {
        finalize_hist(&H[b], 0, plan->rupp[0] <= 0.0, 1, 0, 0.0, plan->need_avg, plan->need_w, 0);
        results_countpairs *r = &results[b];
        r->nbin = nbin;
        r->npairs = malloc(sizeof(uint64_t) * nbin);
        r->rupp = malloc(sizeof(double) * nbin);
        r->rpavg = calloc(nbin, sizeof(double));
        r->weightavg = calloc(nbin, sizeof(double));
        if (!r->npairs || !r->rupp || !r->rpavg || !r->weightavg) {
            rc = EXIT_FAILURE;
            break;
        }
        for (int i = 0; i < nbin; i++) {
            r->npairs[i] = H[b].npairs[i];
            r->rupp[i] = plan->rupp[i];
            r->rpavg[i] = plan->need_avg ? H[b].avg[i] : 0.0;
            r->weightavg[i] = plan->need_w ? H[b].wsum[i] : 0.0;
        }
    }
    if (rc != EXIT_SUCCESS)
        for (int b = 0; b < nb; b++) free_results(&results[b]);
    for (int b = 0; b < nb; b++) free_hist(&H[b]);
    free(H);
    return rc;
}

void cf_gpu_batch_free(cf_gpu_batch *plan)
{
    if (plan == NULL) return;
    cf_engine_batch_free(plan->eng);
    free(plan->rupp);
    free(plan);
}

void free_results(results_countpairs *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->rupp);
    free(results->rpavg);
    free(results->weightavg);
    results->npairs = NULL;
    results->rupp = NULL;
    results->rpavg = NULL;
    results->weightavg = NULL;
}

/* ========================= countpairs_rp_pi (DDrppi) ========================= */
/* theory/DDrppi/countpairs_rp_pi_impl.c.src:135-709 */
int countpairs_rp_pi(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2, void *Y2, void *Z2,
                     const int numthreads, const int autocorr, const char *binfile, const double pimax,
                     results_countpairs_rp_pi *results, struct config_options *options, struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d", autocorr);
        return EXIT_FAILURE;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    const int npibin = (int)pimax;
    if (npibin < 1) {
        CF_ERR("pimax = %g gives %d pi bins; pimax must be at least 1", pimax, npibin);
        return EXIT_FAILURE;
    }
    double *rupp = NULL, rpmin, rpmax;
    int nrpbin;
    if (read_bins(binfile, &rupp, &nrpbin, &rpmin, &rpmax) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (options->periodic && options->boxsize == BOXSIZE_NOTGIVEN) {
        fprintf(stderr, "boxsize = %g must be specified with periodic wrap.\n", options->boxsize);
        free(rupp);
        return EXIT_FAILURE;
    }
    const int64_t totnbins = (int64_t)(npibin + 1) * (nrpbin + 1);
    cf_job J;
    init_job(&J, options, CF_MODE_RPPI, autocorr);
    J.n1 = ND1;
    J.n2 = autocorr ? ND1 : ND2;
    J.x1 = X1; J.y1 = Y1; J.z1 = Z1;
    J.x2 = autocorr ? X1 : X2; J.y2 = autocorr ? Y1 : Y2; J.z2 = autocorr ? Z1 : Z2;
    J.need_weight = need_w;
    J.w1 = need_w ? extra->weights0.weights[0] : NULL;
    J.w2 = need_w ? (autocorr ? extra->weights0.weights[0] : extra->weights1.weights[0]) : NULL;
    cf_fill_rule_extent(&J.rule, options, rpmax, rpmax, pimax, CF_DFL_PER_AXIS, CF_BOOST_XY, ND1);
    J.rmax_xy = rpmax;
    J.rmax_z = pimax;
    J.rmax_3d = 0.0;
    J.pimax = pimax;
    J.npibin = npibin;
    J.nedges = nrpbin;
    for (int i = 0; i < nrpbin; i++) J.edges[i] = rupp[i] * rupp[i];
    cf_hist H;
    if (alloc_hist(&H, nrpbin * (npibin + 1)) != EXIT_SUCCESS) {
        free(rupp);
        return EXIT_FAILURE;
    }
    if (cf_engine_run(&J, &H) != EXIT_SUCCESS) {
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    const double self_w = (autocorr && need_w && rupp[0] <= 0.0) ? self_weight_sum(J.w1, ND1, options->float_type) : 0.0;
    finalize_hist(&H, autocorr, rupp[0] <= 0.0, npibin + 1, ND1, self_w, options->need_avg_sep, need_w, 0);
    results->nbin = nrpbin;
    results->npibin = npibin;
    results->pimax = pimax;
    results->npairs = calloc((size_t)totnbins, sizeof(uint64_t));
    results->rupp = malloc(sizeof(double) * nrpbin);
    results->rpavg = calloc((size_t)totnbins, sizeof(double));
    results->weightavg = calloc((size_t)totnbins, sizeof(double));
    if (!results->npairs || !results->rupp || !results->rpavg || !results->weightavg) {
        free_results_rp_pi(results);
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    for (int i = 0; i < nrpbin; i++) {
        results->rupp[i] = rupp[i];
        for (int j = 0; j < npibin; j++) {
            const int64_t idx = (int64_t)i * (npibin + 1) + j;
            results->npairs[idx] = H.npairs[idx];
            results->rpavg[idx] = options->need_avg_sep ? H.avg[idx] : 0.0;
            results->weightavg[idx] = need_w ? H.wsum[idx] : 0.0;
        }
    }
    free_hist(&H);
    free(rupp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_rp_pi(results_countpairs_rp_pi *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->rupp);
    free(results->rpavg);
    free(results->weightavg);
    results->npairs = NULL;
    results->rupp = NULL;
    results->rpavg = NULL;
    results->weightavg = NULL;
}

/* ========================= countpairs_s_mu (DDsmu) ========================= */
/* theory/DDsmu/countpairs_s_mu_impl.c.src:136-717 */
int countpairs_s_mu(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2, void *Y2, void *Z2,
                    const int numthreads, const int autocorr, const char *sbinfile, const double mu_max,
                    const int nmu_bins, results_countpairs_s_mu *results, struct config_options *options,
                    struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d", autocorr);
        return EXIT_FAILURE;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    double *supp = NULL, smin, smax;
    int nsbin;
    if (read_bins(sbinfile, &supp, &nsbin, &smin, &smax) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (mu_max <= 0.0 || mu_max > 1.0) {
        CF_ERR("max_mu (max. value for the cosine of the angle with line of sight) must be greater than 0 and at most 1). "
               "The passed value is max_mu = %lf. Please change it to be > 0 and <= 1.0", mu_max);
        free(supp);
        return EXIT_FAILURE;
    }
    if (nmu_bins < 1) {
        CF_ERR("Number of mu bins = %d must be at least 1", nmu_bins);
        free(supp);
        return EXIT_FAILURE;
    }
    if (options->periodic && options->boxsize == BOXSIZE_NOTGIVEN) {
        fprintf(stderr, "boxsize = %g must be specified with periodic wrap.\n", options->boxsize);
        free(supp);
        return EXIT_FAILURE;
    }
    const double pimax = smax * mu_max;
    const int64_t totnbins = (int64_t)(nmu_bins + 1) * (nsbin + 1);
    cf_job J;
    init_job(&J, options, CF_MODE_SMU, autocorr);
    J.n1 = ND1;
    J.n2 = autocorr ? ND1 : ND2;
    J.x1 = X1; J.y1 = Y1; J.z1 = Z1;
    J.x2 = autocorr ? X1 : X2; J.y2 = autocorr ? Y1 : Y2; J.z2 = autocorr ? Z1 : Z2;
    J.need_weight = need_w;
    J.w1 = need_w ? extra->weights0.weights[0] : NULL;
    J.w2 = need_w ? (autocorr ? extra->weights0.weights[0] : extra->weights1.weights[0]) : NULL;
    cf_fill_rule_extent(&J.rule, options, smax, smax, pimax, CF_DFL_NONE, CF_BOOST_NONE, ND1);
    J.rmax_xy = smax;
    J.rmax_z = pimax;
    J.rmax_3d = smax;
    J.mu_max = mu_max;
    J.npibin = nmu_bins;
    J.nedges = nsbin;
    for (int i = 0; i < nsbin; i++) J.edges[i] = supp[i] * supp[i];
    cf_hist H;
    if (alloc_hist(&H, nsbin * (nmu_bins + 1)) != EXIT_SUCCESS) {
        free(supp);
        return EXIT_FAILURE;
    }
    if (cf_engine_run(&J, &H) != EXIT_SUCCESS) {
        free_hist(&H);
        free(supp);
        return EXIT_FAILURE;
    }
    const double self_w = (autocorr && need_w && supp[0] <= 0.0) ? self_weight_sum(J.w1, ND1, options->float_type) : 0.0;
    finalize_hist(&H, autocorr, supp[0] <= 0.0, nmu_bins + 1, ND1, self_w, options->need_avg_sep, need_w, 0);
    results->nsbin = nsbin;
    results->nmu_bins = nmu_bins;
    results->mu_max = mu_max;
    results->mu_min = 0.0;
    results->npairs = calloc((size_t)totnbins, sizeof(uint64_t));
    results->supp = malloc(sizeof(double) * nsbin);
    results->savg = calloc((size_t)totnbins, sizeof(double));
    results->weightavg = calloc((size_t)totnbins, sizeof(double));
    if (!results->npairs || !results->supp || !results->savg || !results->weightavg) {
        free_results_s_mu(results);
        free_hist(&H);
        free(supp);
        return EXIT_FAILURE;
    }
    for (int i = 0; i < nsbin; i++) {
        results->supp[i] = supp[i];
        for (int j = 0; j < nmu_bins; j++) {
            const int64_t idx = (int64_t)i * (nmu_bins + 1) + j;
            results->npairs[idx] = H.npairs[idx];
            results->savg[idx] = options->need_avg_sep ? H.avg[idx] : 0.0;
            results->weightavg[idx] = need_w ? H.wsum[idx] : 0.0;
        }
    }
    free_hist(&H);
    free(supp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_s_mu(results_countpairs_s_mu *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->supp);
    free(results->savg);
    free(results->weightavg);
    results->npairs = NULL;
    results->supp = NULL;
    results->savg = NULL;
    results->weightavg = NULL;
}

/* weighted sums for the analytic RR of xi / wp (theory/xi/countpairs_xi_impl.c.src:581-596) */
static void weight_sums(const struct extra_options *extra, int need_w, int64_t nd, size_t es, double *ws, double *wss)
{
    *ws = (double)nd;
    *wss = (double)nd;
    if (need_w && extra->weight_method == PAIR_PRODUCT) {
        const void *w = extra->weights0.weights[0];
        double a = 0.0, b = 0.0;
        for (int64_t j = 0; j < nd; j++) {
            const double v = wval(w, j, es);
            a += v;
            b += v * v;
        }
        *ws = a;
        *wss = (double)nd + b;
    }
}

/* ========================= countpairs_wp ========================= */
/* theory/wp/countpairs_wp_impl.c.src:148-676 */
int countpairs_wp(const int64_t ND, void *X, void *Y, void *Z, const double boxsize, const int numthreads,
                  const char *binfile, const double pimax, results_countpairs_wp *results,
                  struct config_options *options, struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    options->periodic = 1;
    options->autocorr = 1;
    if (check_weights(extra, 1) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    double *rupp = NULL, rpmin, rpmax;
    int nrpbins;
    if (read_bins(binfile, &rupp, &nrpbins, &rpmin, &rpmax) != EXIT_SUCCESS) return EXIT_FAILURE;
    cf_job J;
    init_job(&J, options, CF_MODE_WP, 1);
    J.n1 = J.n2 = ND;
    J.x1 = J.x2 = X;
    J.y1 = J.y2 = Y;
    J.z1 = J.z2 = Z;
    J.need_weight = need_w;
    J.w1 = J.w2 = need_w ? extra->weights0.weights[0] : NULL;
    fill_rule_box(&J.rule, options, boxsize, rpmax, pimax, CF_DFL_WP, ND);
    J.rmax_xy = rpmax;
    J.rmax_z = pimax;
    J.rmax_3d = 0.0;
    J.pimax = pimax;
    J.npibin = 1;
    J.nedges = nrpbins;
    for (int i = 0; i < nrpbins; i++) J.edges[i] = rupp[i] * rupp[i];
    J.task_timer = options->c_cell_timer ? 1 : 0;
    cf_hist H;
    if (alloc_hist(&H, nrpbins) != EXIT_SUCCESS) {
        free(rupp);
        return EXIT_FAILURE;
    }
    if (cf_engine_run(&J, &H) != EXIT_SUCCESS) {
        free_hist(&H);
        free(rupp);
        free(J.task_times);
        return EXIT_FAILURE;
    }
    /* per cell-pair timings (theory/wp/countpairs_wp_impl.c.src:330-332, 433-463): on the GPU one
     * record per work-list task (an i-chunk of a lattice column against one z-window of a
     * neighbouring column), with the warp that ran it as the thread id */
    if (options->c_cell_timer && J.ntask_times > 0)
        assign_cell_timer((struct api_cell_timings *)J.task_times, J.ntask_times, options);
    free(J.task_times);
    J.task_times = NULL;
    const double self_w = (need_w && rupp[0] <= 0.0) ? self_weight_sum(J.w1, ND, options->float_type) : 0.0;
    finalize_hist(&H, 1, rupp[0] <= 0.0, 1, ND, self_w, options->need_avg_sep, need_w, 0);
    results->nbin = nrpbins;
    results->pimax = pimax;
    results->npairs = malloc(sizeof(uint64_t) * nrpbins);
    results->wp = malloc(sizeof(double) * nrpbins);
    results->rupp = malloc(sizeof(double) * nrpbins);
    results->rpavg = malloc(sizeof(double) * nrpbins);
    results->weightavg = calloc(nrpbins, sizeof(double));
    if (!results->npairs || !results->wp || !results->rupp || !results->rpavg || !results->weightavg) {
        free_results_wp(results);
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    double weightsum, weight_sqr_sum;
    weight_sums(extra, need_w, ND, options->float_type, &weightsum, &weight_sqr_sum);
    /* analytic RR and w_p (theory/wp/countpairs_wp_impl.c.src:622-660) */
    const double prefac_density_DD = weightsum * (weightsum - weightsum / ND) / (boxsize * boxsize * boxsize);
    double rlow = 0.0;
    const double twice_pimax = 2.0 * pimax;
    for (int i = 0; i < nrpbins; i++) {
        results->npairs[i] = H.npairs[i];
        results->rupp[i] = rupp[i];
        results->rpavg[i] = options->need_avg_sep ? H.avg[i] : 0.0;
        results->weightavg[i] = need_w ? H.wsum[i] : 0.0;
        double weight0 = (double)results->npairs[i];
        if (need_w && extra->weight_method == PAIR_PRODUCT) weight0 *= results->weightavg[i];
        const double vol = M_PI * (results->rupp[i] * results->rupp[i] - rlow * rlow) * twice_pimax;
        if (vol > 0.0) {
            double weightrandom = prefac_density_DD * vol;
            if (rlow <= 0.) weightrandom += weight_sqr_sum;
            results->wp[i] = (weight0 / weightrandom - 1) * twice_pimax;
        } else {
            results->wp[i] = -2.0 * twice_pimax;
        }
        rlow = results->rupp[i];
    }
    free_hist(&H);
    free(rupp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = (wall_now() - t0) * 1e9; /* nanoseconds, as the reference's wp */
    return EXIT_SUCCESS;
}

void free_results_wp(results_countpairs_wp *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->wp);
    free(results->rupp);
    free(results->rpavg);
    free(results->weightavg);
    results->npairs = NULL;
    results->wp = NULL;
    results->rupp = NULL;
    results->rpavg = NULL;
    results->weightavg = NULL;
}

/* ========================= countpairs_xi ========================= */
/* theory/xi/countpairs_xi_impl.c.src:135-643 */
int countpairs_xi(const int64_t ND, void *X, void *Y, void *Z, const double boxsize, const int numthreads,
                  const char *binfile, results_countpairs_xi *results, struct config_options *options,
                  struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    options->periodic = 1;
    options->autocorr = 1;
    if (check_weights(extra, 1) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    sanitize_lattice_options(options);
    options->sort_on_z = 1;
    double *rupp = NULL, rmin, rmax;
    int nbins;
    if (read_bins(binfile, &rupp, &nbins, &rmin, &rmax) != EXIT_SUCCESS) return EXIT_FAILURE;
    cf_job J;
    init_job(&J, options, CF_MODE_R3, 1);
    J.n1 = J.n2 = ND;
    J.x1 = J.x2 = X;
    J.y1 = J.y2 = Y;
    J.z1 = J.z2 = Z;
    J.need_weight = need_w;
    J.w1 = J.w2 = need_w ? extra->weights0.weights[0] : NULL;
    fill_rule_box(&J.rule, options, boxsize, rmax, rmax, CF_DFL_XI, ND);
    J.rmax_xy = J.rmax_z = J.rmax_3d = rmax;
    J.nedges = nbins;
    for (int i = 0; i < nbins; i++) J.edges[i] = rupp[i] * rupp[i];
    cf_hist H;
    if (alloc_hist(&H, nbins) != EXIT_SUCCESS) {
        free(rupp);
        return EXIT_FAILURE;
    }
    if (cf_engine_run(&J, &H) != EXIT_SUCCESS) {
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    const double self_w = (need_w && rupp[0] <= 0.0) ? self_weight_sum(J.w1, ND, options->float_type) : 0.0;
    finalize_hist(&H, 1, rupp[0] <= 0.0, 1, ND, self_w, options->need_avg_sep, need_w, 0);
    results->nbin = nbins;
    results->npairs = malloc(sizeof(uint64_t) * nbins);
    results->xi = malloc(sizeof(double) * nbins);
    results->rupp = malloc(sizeof(double) * nbins);
    results->ravg = malloc(sizeof(double) * nbins);
    results->weightavg = calloc(nbins, sizeof(double));
    if (!results->npairs || !results->xi || !results->rupp || !results->ravg || !results->weightavg) {
        free_results_xi(results);
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    double weightsum, weight_sqr_sum;
    weight_sums(extra, need_w, ND, options->float_type, &weightsum, &weight_sqr_sum);
    /* analytic RR and xi (theory/xi/countpairs_xi_impl.c.src:597-626) */
    const double prefac_density = weightsum * (weightsum - weightsum / ND) / (boxsize * boxsize * boxsize);
    double rlow = 0.0;
    for (int i = 0; i < nbins; i++) {
        results->npairs[i] = H.npairs[i];
        results->rupp[i] = rupp[i];
        results->ravg[i] = options->need_avg_sep ? H.avg[i] : 0.0;
        results->weightavg[i] = need_w ? H.wsum[i] : 0.0;
        double weight0 = (double)results->npairs[i];
        if (need_w && extra->weight_method == PAIR_PRODUCT) weight0 *= results->weightavg[i];
        const double vol = 4.0 / 3.0 * M_PI * (rupp[i] * rupp[i] * rupp[i] - rlow * rlow * rlow);
        if (vol > 0.0) {
            double weightrandom = prefac_density * vol;
            if (rlow <= 0.) weightrandom += weight_sqr_sum;
            results->xi[i] = (weight0 / weightrandom - 1.0);
        } else {
            results->xi[i] = -2.0;
        }
        rlow = results->rupp[i];
    }
    free_hist(&H);
    free(rupp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_xi(results_countpairs_xi *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->xi);
    free(results->rupp);
    free(results->ravg);
    free(results->weightavg);
    results->npairs = NULL;
    results->xi = NULL;
    results->rupp = NULL;
    results->ravg = NULL;
    results->weightavg = NULL;
}

/* ========================= countpairs_theta_mocks (DDtheta) ========================= */
/* RA / DEC sanity fix-ups (mocks/DDtheta_mocks/countpairs_theta_mocks_impl.c.src:42-83):
 * the reference shifts RA by +180 and DEC by -90 in place when they look like the other
 * convention. */
static int check_ra_dec(int64_t n, void *ra, void *dec, size_t es)
{
    if (n == 0) return EXIT_SUCCESS;
    if (ra == NULL || dec == NULL) {
        CF_ERR("Input arrays can not be NULL. Have RA = %p DEC = %p", ra, dec);
        return EXIT_FAILURE;
    }
    int fix_ra = 0, fix_dec = 0;
    for (int64_t i = 0; i < n; i++) {
        const double r = wval(ra, i, es), d = wval(dec, i, es);
        if (r < 0.0) fix_ra = 1;
        if (!(d <= 180.0)) {
            CF_ERR("Declination should not be more than 180. Did you swap ra and dec?");
            return EXIT_FAILURE;
        }
        if (d > 90.0) fix_dec = 1;
    }
    if (fix_ra || fix_dec) {
        if (fix_ra) fprintf(stderr, "DDtheta> Out of range values found for ra. Expected ra to be in the range [0.0,360.0]. Found ra values in [-180,180] -- fixing that\n");
        if (fix_dec) fprintf(stderr, "DDtheta> Out of range values found for dec. Expected dec to be in the range [-90.0,90.0]. Found dec values in [0,180] -- fixing that\n");
        for (int64_t i = 0; i < n; i++) {
            if (es == sizeof(float)) {
                if (fix_ra) ((float *)ra)[i] += 180.0f;
                if (fix_dec) ((float *)dec)[i] -= 90.0f;
            } else {
                if (fix_ra) ((double *)ra)[i] += 180.0;
                if (fix_dec) ((double *)dec)[i] -= 90.0;
            }
        }
    }
    return EXIT_SUCCESS;
}

#define CF_PI_OVER_180 0.017453292519943295769236907684886127134428718885417254560971

/* unit vectors on the host with libm, as the reference does
 * (mocks/DDtheta_mocks/countpairs_theta_mocks_impl.c.src:586-608) */
static int unit_vectors(int64_t n, const void *ra, const void *dec, const void *w, size_t es, double **X, double **Y,
                        double **Z, double **W)
{
    *X = malloc(sizeof(double) * (n > 0 ? n : 1));
    *Y = malloc(sizeof(double) * (n > 0 ? n : 1));
    *Z = malloc(sizeof(double) * (n > 0 ? n : 1));
    *W = w ? malloc(sizeof(double) * (n > 0 ? n : 1)) : NULL;
    if (!*X || !*Y || !*Z || (w && !*W)) return EXIT_FAILURE;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        const double r = wval(ra, i, es), d = wval(dec, i, es);
        const double cd = cos(d * CF_PI_OVER_180);
        (*X)[i] = cd * cos(r * CF_PI_OVER_180);
        (*Y)[i] = cd * sin(r * CF_PI_OVER_180);
        (*Z)[i] = sin(d * CF_PI_OVER_180);
        if (w) (*W)[i] = wval(w, i, es);
    }
    return EXIT_SUCCESS;
}

int countpairs_theta_mocks(const int64_t ND1, void *phi1, void *theta1, const int64_t ND2, void *phi2, void *theta2,
                           const int numthreads, const int autocorr, const char *binfile,
                           results_countpairs_theta *results, struct config_options *options,
                           struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d", autocorr);
        return EXIT_FAILURE;
    }
    if (ND1 == 0 || ND2 == 0) {
        /* mocks/DDtheta_mocks/countpairs_theta_mocks_impl.c.src:464-477 */
        fprintf(stderr, "Warning: Received 0 particles in at least one of the arrays. len(array1) = %lld len(array2) = %lld\n",
                (long long)ND1, (long long)ND2);
        results->npairs = NULL;
        results->theta_avg = NULL;
        results->weightavg = NULL;
        results->theta_upp = NULL;
        results->nbin = 0;
        return EXIT_SUCCESS;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    const size_t es = options->float_type;
    if (check_ra_dec(ND1, phi1, theta1, es) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!autocorr && check_ra_dec(ND2, phi2, theta2, es) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (options->max_cells_per_dim == 0) options->max_cells_per_dim = NLATMAX;
    double *theta_upp = NULL, thetamin, thetamax;
    int nthetabin;
    if (cf_setup_bins(binfile, &thetamin, &thetamax, &nthetabin, &theta_upp) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!(thetamin >= 0.0 && thetamax > 0.0 && thetamin < thetamax && thetamax <= 180.0 && nthetabin >= 1)) {
        CF_ERR("Could not setup with theta bins correctly. (thetamin = %lf, thetamax = %lf, with nbins = %d). "
               "Expected non-zero rmin/rmax with thetamax > thetamin and nbins >=1 ",
               thetamin, thetamax, nthetabin);
        free(theta_upp);
        return EXIT_FAILURE;
    }
    if (nthetabin > CF_MAX_EDGES) {
        CF_ERR("at most %d bins are supported", CF_MAX_EDGES - 1);
        free(theta_upp);
        return EXIT_FAILURE;
    }
    double *X1 = NULL, *Y1 = NULL, *Z1 = NULL, *W1 = NULL, *X2 = NULL, *Y2 = NULL, *Z2 = NULL, *W2 = NULL;
    int rc = unit_vectors(ND1, phi1, theta1, need_w ? extra->weights0.weights[0] : NULL, es, &X1, &Y1, &Z1, &W1);
    if (rc == EXIT_SUCCESS && !autocorr)
        rc = unit_vectors(ND2, phi2, theta2, need_w ? extra->weights1.weights[0] : NULL, es, &X2, &Y2, &Z2, &W2);
    cf_hist H;
    memset(&H, 0, sizeof(H));
    if (rc == EXIT_SUCCESS) rc = alloc_hist(&H, nthetabin);
    if (rc == EXIT_SUCCESS) {
        cf_job J;
        init_job(&J, options, CF_MODE_THETA, autocorr);
        J.elem_size = 8;
        J.n1 = ND1;
        J.n2 = autocorr ? ND1 : ND2;
        J.x1 = X1; J.y1 = Y1; J.z1 = Z1; J.w1 = W1;
        J.x2 = autocorr ? X1 : X2; J.y2 = autocorr ? Y1 : Y2; J.z2 = autocorr ? Z1 : Z2; J.w2 = autocorr ? W1 : W2;
        J.need_weight = need_w;
        J.rule.kind = CF_REF_NONE;
        J.nedges = nthetabin;
        for (int i = 0; i < nthetabin; i++) J.edges[i] = cos(theta_upp[i] * CF_PI_OVER_180);
        const double cmax = J.edges[nthetabin - 1];
        const double chord = sqrt(2.0 * (1.0 - cmax) + 1e-14) * (1.0 + 1e-9);
        J.rmax_xy = J.rmax_z = J.rmax_3d = chord;
        rc = cf_engine_run(&J, &H);
    }
    if (rc == EXIT_SUCCESS) {
        const double self_w = (autocorr && need_w && theta_upp[0] <= 0.0) ? self_weight_sum(W1, ND1, 8) : 0.0;
        finalize_hist(&H, autocorr, theta_upp[0] <= 0.0, 1, ND1, self_w, options->need_avg_sep, need_w, 1);
        results->nbin = nthetabin;
        results->npairs = malloc(sizeof(uint64_t) * nthetabin);
        results->theta_upp = malloc(sizeof(double) * nthetabin);
        results->theta_avg = malloc(sizeof(double) * nthetabin);
        results->weightavg = calloc(nthetabin, sizeof(double));
        if (!results->npairs || !results->theta_upp || !results->theta_avg || !results->weightavg) {
            free_results_countpairs_theta(results);
            rc = EXIT_FAILURE;
        } else {
            for (int i = 0; i < nthetabin; i++) {
                results->npairs[i] = H.npairs[i];
                results->theta_upp[i] = theta_upp[i];
                results->theta_avg[i] = options->need_avg_sep ? H.avg[i] : 0.0;
                results->weightavg[i] = need_w ? H.wsum[i] : 0.0;
            }
        }
    }
    free_hist(&H);
    free(X1); free(Y1); free(Z1); free(W1);
    free(X2); free(Y2); free(Z2); free(W2);
    free(theta_upp);
    if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_countpairs_theta(results_countpairs_theta *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->theta_upp);
    free(results->theta_avg);
    free(results->weightavg);
    results->npairs = NULL;
    results->theta_upp = NULL;
    results->theta_avg = NULL;
    results->weightavg = NULL;
}

/* ==================== countpairs_mocks (DDrppi_mocks), countpairs_mocks_s_mu (DDsmu_mocks) ==================== */
#define CF_SPEED_OF_LIGHT 299800.0 /* km/s, utils/set_cosmo_dist.h:19 */

/* (RA, DEC, cz) sanity fix-ups, in place as the reference does
 * (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:43-112; the DDsmu_mocks copy is
 * mocks/DDsmu_mocks/countpairs_s_mu_mocks_impl.c.src:44-113): RA in [-180, 180] is shifted by
 * +180, DEC in [0, 180] by -90, and redshifts (max < 10 unless the third column already is a
 * comoving distance) are multiplied by the speed of light. */
static int check_ra_dec_cz(int64_t n, void *ra, void *dec, void *cz, size_t es, int is_comoving)
{
    if (n == 0) return EXIT_SUCCESS;
    if (ra == NULL || dec == NULL || cz == NULL) {
        CF_ERR("Input arrays can not be NULL. Have RA = %p DEC = %p cz = %p", ra, dec, cz);
        return EXIT_FAILURE;
    }
    int fix_cz = 0, fix_ra = 0, fix_dec = 0;
    double max_cz = 0.0;
    for (int64_t i = 0; i < n; i++) {
        const double c = wval(cz, i, es), r = wval(ra, i, es), d = wval(dec, i, es);
        if (c > max_cz) max_cz = c;
        if (r < 0.0) fix_ra = 1;
        if (d > 90.0) fix_dec = 1;
        if (d > 180) {
            CF_ERR("theta[%lld] = %g should be less than 180 deg", (long long)i, d);
            return EXIT_FAILURE;
        }
    }
    if (max_cz < 10.0 && !is_comoving) fix_cz = 1;
    if (fix_ra) fprintf(stderr, "check_ra_dec_cz> Out of range values found for ra. Expected ra to be in the range [0.0,360.0]. Found ra values in [-180,180] -- fixing that\n");
    if (fix_dec) fprintf(stderr, "check_ra_dec_cz> Out of range values found for dec. Expected dec to be in the range [-90.0,90.0]. Found dec values in [0,180] -- fixing that\n");
    if (fix_cz) fprintf(stderr, "check_ra_dec_cz> Out of range values found for cz. Expected input to be `cz' but found `z' instead. max_cz (found in input) = %g threshold = %g\n", max_cz, 10.0);
    if (!(fix_ra || fix_dec || fix_cz)) return EXIT_SUCCESS;
    for (int64_t i = 0; i < n; i++) {
        if (es == sizeof(float)) {
            if (fix_ra) ((float *)ra)[i] += 180.0f;
            if (fix_dec) ((float *)dec)[i] -= 90.0f;
            if (fix_cz) ((float *)cz)[i] *= (float)CF_SPEED_OF_LIGHT;
        } else {
            if (fix_ra) ((double *)ra)[i] += 180.0;
            if (fix_dec) ((double *)dec)[i] -= 90.0;
            if (fix_cz) ((double *)cz)[i] *= CF_SPEED_OF_LIGHT;
        }
    }
    return EXIT_SUCCESS;
}

/* Omega_matter of the two built-in cosmologies (utils/cosmology_params.c:28-55): 1 = LasDamas,
 * 2 = Planck; both flat (Omega_Lambda = 1 - Omega_m). */
static int cosmology_omega_m(int cosmology, double *omega_m)
{
    switch (cosmology) {
    case 1: *omega_m = 0.25; return EXIT_SUCCESS;
    case 2: *omega_m = 0.302; return EXIT_SUCCESS;
    }
    fprintf(stderr, "ERROR: In init_cosmology> Cosmology=%d not implemented\n", cosmology);
    return EXIT_FAILURE;
}

/* Comoving distance table D_c(z) in Mpc/h (utils/set_cosmo_dist.c:26-67): Simpson's rule with
 * step dz = 1e-2 / max_size on 1/E(z), one sample every 1/max_size in z up to zmax.  The
 * operation order is the reference's (this file is compiled without contractions).  Returns
 * the number of samples. */
/* The table of the most recent call with the largest zmax so far, per (omega_m, max_size).  The
 * Simpson loop below visits the same z values in the same order whatever zmax is, so the table for
 * a smaller zmax is a prefix of a longer one (its entries recorded before the loop reached zmax):
 * later calls copy that prefix instead of integrating again. */
static pthread_mutex_t g_cosmo_lock = PTHREAD_MUTEX_INITIALIZER;
static struct {
    double omega_m, zmax;
    int max_size, n;
    double *z, *d;
} g_cosmo = {0.0, 0.0, 0, 0, NULL, NULL};

static int comoving_table_compute(double zmax, int max_size, double omega_m, double *zc, double *dc);

static int comoving_table(double zmax, int max_size, double omega_m, double *zc, double *dc)
{
    int n = -1;
    pthread_mutex_lock(&g_cosmo_lock);
    if (g_cosmo.z && g_cosmo.omega_m == omega_m && g_cosmo.max_size == max_size && zmax <= g_cosmo.zmax) {
        n = 0;
        while (n < g_cosmo.n && g_cosmo.z[n] < zmax) n++;
        memcpy(zc, g_cosmo.z, sizeof(double) * (size_t)n);
        memcpy(dc, g_cosmo.d, sizeof(double) * (size_t)n);
    }
    pthread_mutex_unlock(&g_cosmo_lock);
    if (n >= 0) return n;
    n = comoving_table_compute(zmax, max_size, omega_m, zc, dc);
    pthread_mutex_lock(&g_cosmo_lock);
    double *z = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1)), *d = malloc(sizeof(double) * (size_t)(n > 0 ? n : 1));
    if (z && d) {
        memcpy(z, zc, sizeof(double) * (size_t)n);
        memcpy(d, dc, sizeof(double) * (size_t)n);
        free(g_cosmo.z);
        free(g_cosmo.d);
        g_cosmo.z = z;
        g_cosmo.d = d;
        g_cosmo.n = n;
        g_cosmo.zmax = zmax;
        g_cosmo.omega_m = omega_m;
        g_cosmo.max_size = max_size;
    } else {
        free(z);
        free(d);
    }
    pthread_mutex_unlock(&g_cosmo_lock);
    return n;
}

static int comoving_table_compute(double zmax, int max_size, double omega_m, double *zc, double *dc)
{
    const double omega_l = 1.0 - omega_m;
    const double omega_k = 1.0 - omega_m - omega_l;
    const double Dh = CF_SPEED_OF_LIGHT * 0.01 / 1.0;
    const double Deltaz = 1.0 / max_size;
    const double dz = 1e-2 * Deltaz;
    const double eps = 1e-10;
    double Eint = 0.0, E2 = 1.0, z2 = Deltaz;
    int i = 0;
    for (double z = 2.0 * dz; z < zmax; z += 2.0 * dz) {
        const double E0 = E2;
        const double a1 = 1 + z - dz, a2 = 1 + z;
        const double E1 = 1.0 / sqrt(omega_m * (a1 * a1 * a1) + omega_k * (1 + z - dz) + omega_l);
        E2 = 1.0 / sqrt(omega_m * (a2 * a2 * a2) + omega_k * (1 + z) + omega_l);
        Eint += dz * (E0 + 4. * E1 + E2) / 3.;
        if (z > (z2 - eps) && z < (z2 + eps)) {
            if (i >= max_size) break;
            zc[i] = z;
            dc[i] = Eint * Dh;
            z2 += Deltaz;
            i++;
        }
    }
    return i;
}

/* Piecewise-linear interpolation of the table at x: the segment [x_k, x_k+1] with
 * x_k <= x < x_k+1 (the last segment for x = x_n-1), y = y_k + (x - x_k) / (x_k+1 - x_k) * (y_k+1 - y_k).
 * This is the evaluation order of the linear interpolant the reference takes from GSL
 * (gsl_interp_linear, used at mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:345-356).
 * Points outside the table are an error (GSL raises a domain error there). */
static int interp_linear(const double *xs, const double *ys, int n, double x, double *y)
{
    if (n < 2 || !(x >= xs[0] && x <= xs[n - 1])) return EXIT_FAILURE;
    int lo = 0, hi = n - 1;
    while (hi > lo + 1) {
        const int mid = (lo + hi) / 2;
        if (xs[mid] > x) hi = mid; else lo = mid;
    }
    const double dx = xs[lo + 1] - xs[lo];
    if (!(dx > 0.0)) return EXIT_FAILURE;
    *y = ys[lo] + (x - xs[lo]) / dx * (ys[lo + 1] - ys[lo]);
    return EXIT_SUCCESS;
}

/* Comoving Cartesian positions of one catalogue, on the host with libm as the reference does
 * (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:318-392):
 *   X = D cos(DEC) cos(RA), Y = D cos(DEC) sin(RA), Z = D sin(DEC)
 * with D the third column itself (is_comoving_dist) or D_c(cz / c) from the table. */
static int mock_positions(int64_t n, const void *ra, const void *dec, const void *cz, const void *w, size_t es,
                          const double *zc, const double *dcs, int nz, double **X, double **Y, double **Z, double **W)
{
    const size_t m = (size_t)(n > 0 ? n : 1);
    *X = malloc(sizeof(double) * m);
    *Y = malloc(sizeof(double) * m);
    *Z = malloc(sizeof(double) * m);
    *W = w ? malloc(sizeof(double) * m) : NULL;
    if (!*X || !*Y || !*Z || (w && !*W)) return EXIT_FAILURE;
    const double inv_c = 1.0 / CF_SPEED_OF_LIGHT;
    int64_t bad = -1;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
        double D = wval(cz, i, es);
        if (zc != NULL && interp_linear(zc, dcs, nz, D * inv_c, &D) != EXIT_SUCCESS) {
#pragma omp critical
            bad = (bad < 0 || i < bad) ? i : bad;
            continue;
        }
        const double r = wval(ra, i, es), d = wval(dec, i, es);
        const double cd = cos(d * CF_PI_OVER_180);  /* the value the reference computes twice */
        (*X)[i] = D * cd * cos(r * CF_PI_OVER_180);
        (*Y)[i] = D * cd * sin(r * CF_PI_OVER_180);
        (*Z)[i] = D * sin(d * CF_PI_OVER_180);
        if (w) (*W)[i] = wval(w, i, es);
    }
    if (bad >= 0) {
        CF_ERR("cz[%lld] = %g is outside the comoving-distance table (z in [%g, %g])", (long long)bad,
               wval(cz, bad, es), zc[0], zc[nz - 1]);
        return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

typedef struct {
    double *X1, *Y1, *Z1, *W1, *X2, *Y2, *Z2, *W2;
} mock_sets;

static void free_mock_sets(mock_sets *M)
{
    free(M->X1); free(M->Y1); free(M->Z1); free(M->W1);
    free(M->X2); free(M->Y2); free(M->Z2); free(M->W2);
    memset(M, 0, sizeof(*M));
}

/* Both catalogues to comoving XYZ (double).  The distance table spans z up to
 * max(cz) / c + 0.01 over both sets (countpairs_rp_pi_mocks_impl.c.src:330-343). */
static int mock_inputs(int64_t ND1, void *ra1, void *dec1, void *cz1, int64_t ND2, void *ra2, void *dec2, void *cz2,
                       int autocorr, int cosmology, const struct config_options *options,
                       const struct extra_options *extra, mock_sets *M)
{
    memset(M, 0, sizeof(*M));
    const size_t es = options->float_type;
    const int need_w = extra->weight_method != NONE;
    double *zc = NULL, *dcs = NULL;
    int nz = 0, rc = EXIT_SUCCESS;
    if (!options->is_comoving_dist) {
        double omega_m;
        if (cosmology_omega_m(cosmology, &omega_m) != EXIT_SUCCESS) return EXIT_FAILURE;
        double czmax = 0.0;
        for (int64_t i = 0; i < ND1; i++) if (wval(cz1, i, es) > czmax) czmax = wval(cz1, i, es);
        if (!autocorr)
            for (int64_t i = 0; i < ND2; i++) if (wval(cz2, i, es) > czmax) czmax = wval(cz2, i, es);
        const double zmax = czmax * (1.0 / CF_SPEED_OF_LIGHT) + 0.01;
        const int max_size = 10000;
        zc = calloc(max_size, sizeof(double));
        dcs = calloc(max_size, sizeof(double));
        if (!zc || !dcs) rc = EXIT_FAILURE;
        if (rc == EXIT_SUCCESS) nz = comoving_table(zmax, max_size, omega_m, zc, dcs);
        if (rc == EXIT_SUCCESS && nz < 2) {
            CF_ERR("comoving-distance table has %d samples (zmax = %g)", nz, zmax);
            rc = EXIT_FAILURE;
        }
    }
    if (rc == EXIT_SUCCESS)
        rc = mock_positions(ND1, ra1, dec1, cz1, need_w ? extra->weights0.weights[0] : NULL, es, zc, dcs, nz, &M->X1,
                            &M->Y1, &M->Z1, &M->W1);
    if (rc == EXIT_SUCCESS && !autocorr)
        rc = mock_positions(ND2, ra2, dec2, cz2, need_w ? extra->weights1.weights[0] : NULL, es, zc, dcs, nz, &M->X2,
                            &M->Y2, &M->Z2, &M->W2);
    free(zc);
    free(dcs);
    if (rc != EXIT_SUCCESS) free_mock_sets(M);
    return rc;
}

static void mock_job(cf_job *J, const struct config_options *options, int mode, int autocorr, int64_t ND1,
                     int64_t ND2, const mock_sets *M, int need_w, double max_sep)
{
    init_job(J, options, mode, autocorr);
    J->elem_size = 8;
    J->n1 = ND1;
    J->n2 = autocorr ? ND1 : ND2;
    J->x1 = M->X1; J->y1 = M->Y1; J->z1 = M->Z1; J->w1 = M->W1;
    J->x2 = autocorr ? M->X1 : M->X2;
    J->y2 = autocorr ? M->Y1 : M->Y2;
    J->z2 = autocorr ? M->Z1 : M->Z2;
    J->w2 = autocorr ? M->W1 : M->W2;
    J->need_weight = need_w;
    J->rule.kind = CF_REF_NONE;
    J->rmax_xy = J->rmax_z = J->rmax_3d = max_sep;
}

/* mocks/DDrppi_mocks/countpairs_rp_pi_mocks.c + countpairs_rp_pi_mocks_impl.c.src:200-847 */
int countpairs_mocks(const int64_t ND1, void *ra1, void *dec1, void *czD1, const int64_t ND2, void *ra2, void *dec2,
                     void *czD2, const int numthreads, const int autocorr, const char *binfile, const double pimax,
                     const int cosmology, results_countpairs_mocks *results, struct config_options *options,
                     struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    options->sort_on_z = 1;
    memset(results, 0, sizeof(*results));
    if (ND1 == 0 || (autocorr == 0 && ND2 == 0)) return EXIT_SUCCESS;
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d", autocorr);
        return EXIT_FAILURE;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    const size_t es = options->float_type;
    if (check_ra_dec_cz(ND1, ra1, dec1, czD1, es, options->is_comoving_dist) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!autocorr && check_ra_dec_cz(ND2, ra2, dec2, czD2, es, options->is_comoving_dist) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    sanitize_lattice_options(options);
    const int npibin = (int)pimax;
    if (npibin < 1) {
        CF_ERR("pimax = %g gives %d pi bins; pimax must be at least 1", pimax, npibin);
        return EXIT_FAILURE;
    }
    double omega_m;
    if (cosmology_omega_m(cosmology, &omega_m) != EXIT_SUCCESS) return EXIT_FAILURE;
    double *rupp = NULL, rpmin, rpmax;
    int nrpbin;
    if (cf_setup_bins(binfile, &rpmin, &rpmax, &nrpbin, &rupp) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!(rpmin > 0.0 && rpmax > 0.0 && rpmin < rpmax && nrpbin > 0) || nrpbin > CF_MAX_EDGES) {
        CF_ERR("Could not setup with R bins correctly. (rmin = %lf, rmax = %lf, with nbins = %d). Expected non-zero "
               "rmin/rmax with rmax > rmin and nbins >=1 ", rpmin, rpmax, nrpbin);
        free(rupp);
        return EXIT_FAILURE;
    }
    mock_sets M;
    if (mock_inputs(ND1, ra1, dec1, czD1, ND2, ra2, dec2, czD2, autocorr, cosmology, options, extra, &M) !=
        EXIT_SUCCESS) {
        free(rupp);
        return EXIT_FAILURE;
    }
    const int64_t totnbins = (int64_t)(npibin + 1) * (nrpbin + 1);
    cf_job J;
    mock_job(&J, options, CF_MODE_RPPI_MOCK, autocorr, ND1, ND2, &M, need_w, sqrt(rpmax * rpmax + pimax * pimax));
    J.pimax = pimax;
    J.npibin = npibin;
    J.nedges = nrpbin;
    for (int i = 0; i < nrpbin; i++) J.edges[i] = rupp[i] * rupp[i];
    cf_hist H;
    int rc = alloc_hist(&H, nrpbin * (npibin + 1));
    if (rc == EXIT_SUCCESS) rc = cf_engine_run(&J, &H);
    free_mock_sets(&M);
    if (rc != EXIT_SUCCESS) {
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    /* rpmin > 0: no self pairs (countpairs_rp_pi_mocks_impl.c.src:730-765) */
    finalize_hist(&H, autocorr, 0, npibin + 1, ND1, 0.0, options->need_avg_sep, need_w, 0);
    results->nbin = nrpbin;
    results->npibin = npibin;
    results->pimax = pimax;
    results->npairs = calloc((size_t)totnbins, sizeof(uint64_t));
    results->rupp = malloc(sizeof(double) * nrpbin);
    results->rpavg = calloc((size_t)totnbins, sizeof(double));
    results->weightavg = calloc((size_t)totnbins, sizeof(double));
    if (!results->npairs || !results->rupp || !results->rpavg || !results->weightavg) {
        free_results_mocks(results);
        free_hist(&H);
        free(rupp);
        return EXIT_FAILURE;
    }
    for (int i = 0; i < nrpbin; i++) {
        results->rupp[i] = rupp[i];
        for (int j = 0; j < npibin; j++) {
            const int64_t idx = (int64_t)i * (npibin + 1) + j;
            results->npairs[idx] = H.npairs[idx];
            results->rpavg[idx] = options->need_avg_sep ? H.avg[idx] : 0.0;
            results->weightavg[idx] = need_w ? H.wsum[idx] : 0.0;
        }
    }
    free_hist(&H);
    free(rupp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_mocks(results_countpairs_mocks *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->rupp);
    free(results->rpavg);
    free(results->weightavg);
    results->npairs = NULL;
    results->rupp = NULL;
    results->rpavg = NULL;
    results->weightavg = NULL;
}

/* mocks/DDsmu_mocks/countpairs_s_mu_mocks.c + countpairs_s_mu_mocks_impl.c.src:203-846 */
int countpairs_mocks_s_mu(const int64_t ND1, void *ra1, void *dec1, void *czD1, const int64_t ND2, void *ra2,
                          void *dec2, void *czD2, const int numthreads, const int autocorr, const char *sbinfile,
                          const double mu_max, const int nmu_bins, const int cosmology,
                          results_countpairs_mocks_s_mu *results, struct config_options *options,
                          struct extra_options *extra)
{
    (void)numthreads;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    struct extra_options dummy;
    if (extra == NULL) {
        dummy = get_extra_options(NONE);
        extra = &dummy;
    }
    options->sort_on_z = 1;
    memset(results, 0, sizeof(*results));
    if (ND1 == 0 || (autocorr == 0 && ND2 == 0)) return EXIT_SUCCESS;
    if (autocorr != 0 && autocorr != 1) {
        CF_ERR("Strange value of autocorr = %d", autocorr);
        return EXIT_FAILURE;
    }
    if (check_weights(extra, autocorr) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int need_w = extra->weight_method != NONE;
    const size_t es = options->float_type;
    if (check_ra_dec_cz(ND1, ra1, dec1, czD1, es, options->is_comoving_dist) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!autocorr && check_ra_dec_cz(ND2, ra2, dec2, czD2, es, options->is_comoving_dist) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    sanitize_lattice_options(options);
    double omega_m;
    if (cosmology_omega_m(cosmology, &omega_m) != EXIT_SUCCESS) return EXIT_FAILURE;
    double *supp = NULL, smin, smax;
    int nsbin;
    if (cf_setup_bins(sbinfile, &smin, &smax, &nsbin, &supp) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (!(smin > 0.0 && smax > 0.0 && smin < smax && nsbin > 0) || nsbin > CF_MAX_EDGES) {
        CF_ERR("Could not setup with S bins correctly. (smin = %lf, smax = %lf, with nbins = %d). Expected non-zero "
               "smin/smax with smax > smin and nbins >=1 ", smin, smax, nsbin);
        free(supp);
        return EXIT_FAILURE;
    }
    if (mu_max <= 0.0 || mu_max > 1.0) {
        CF_ERR("max_mu (max. value for the cosine of the angle with line of sight) must be greater than 0 and at most "
               "1).\nThe passed value is max_mu = %lf. Please change it to be > 0 and <= 1.0", mu_max);
        free(supp);
        return EXIT_FAILURE;
    }
    if (nmu_bins < 1) {
        CF_ERR("Number of mu bins = %d must be at least 1", nmu_bins);
        free(supp);
        return EXIT_FAILURE;
    }
    mock_sets M;
    if (mock_inputs(ND1, ra1, dec1, czD1, ND2, ra2, dec2, czD2, autocorr, cosmology, options, extra, &M) !=
        EXIT_SUCCESS) {
        free(supp);
        return EXIT_FAILURE;
    }
    const int64_t totnbins = (int64_t)(nmu_bins + 1) * (nsbin + 1);
    cf_job J;
    mock_job(&J, options, CF_MODE_SMU_MOCK, autocorr, ND1, ND2, &M, need_w, smax);
    J.mu_max = mu_max;
    J.npibin = nmu_bins;
    J.nedges = nsbin;
    for (int i = 0; i < nsbin; i++) J.edges[i] = supp[i] * supp[i];
    cf_hist H;
    int rc = alloc_hist(&H, nsbin * (nmu_bins + 1));
    if (rc == EXIT_SUCCESS) rc = cf_engine_run(&J, &H);
    free_mock_sets(&M);
    if (rc != EXIT_SUCCESS) {
        free_hist(&H);
        free(supp);
        return EXIT_FAILURE;
    }
    finalize_hist(&H, autocorr, 0, nmu_bins + 1, ND1, 0.0, options->need_avg_sep, need_w, 0);
    results->nsbin = nsbin;
    results->nmu_bins = nmu_bins;
    results->mu_max = mu_max;
    results->mu_min = 0.0;
    results->npairs = calloc((size_t)totnbins, sizeof(uint64_t));
    results->supp = malloc(sizeof(double) * nsbin);
    results->savg = calloc((size_t)totnbins, sizeof(double));
    results->weightavg = calloc((size_t)totnbins, sizeof(double));
    if (!results->npairs || !results->supp || !results->savg || !results->weightavg) {
        free_results_mocks_s_mu(results);
        free_hist(&H);
        free(supp);
        return EXIT_FAILURE;
    }
    for (int i = 0; i < nsbin; i++) {
        results->supp[i] = supp[i];
        for (int j = 0; j < nmu_bins; j++) {
            const int64_t idx = (int64_t)i * (nmu_bins + 1) + j;
            results->npairs[idx] = H.npairs[idx];
            results->savg[idx] = options->need_avg_sep ? H.avg[idx] : 0.0;
            results->weightavg[idx] = need_w ? H.wsum[idx] : 0.0;
        }
    }
    free_hist(&H);
    free(supp);
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_mocks_s_mu(results_countpairs_mocks_s_mu *results)
{
    if (results == NULL) return;
    free(results->npairs);
    free(results->supp);
    free(results->savg);
    free(results->weightavg);
    results->npairs = NULL;
    results->supp = NULL;
    results->savg = NULL;
    results->weightavg = NULL;
}

/* ========================= GB300 extensions ========================= */
/* ========================= countspheres (vpf), countspheres_mocks (vpf_mocks) ========================= */

static double **pn_matrix(int nbin, int num_pN)
{
    double **m = calloc((size_t)nbin, sizeof(double *));
    if (m == NULL) return NULL;
    for (int i = 0; i < nbin; i++) {
        m[i] = calloc((size_t)num_pN, sizeof(double));
        if (m[i] == NULL) {
            for (int k = 0; k < i; k++) free(m[k]);
            free(m);
            return NULL;
        }
    }
    return m;
}

static void pn_free(double **m, int nbin)
{
    if (m == NULL) return;
    for (int i = 0; i < nbin; i++) free(m[i]);
    free(m);
}

static void refine_check(struct config_options *options)
{
    if (options->max_cells_per_dim == 0) {
        fprintf(stderr, "Warning: Max. cells per dimension is set to 0 - resetting to `NLATMAX' = %d\n", NLATMAX);
        options->max_cells_per_dim = NLATMAX;
    }
    for (int i = 0; i < 3; i++) {
        if (options->bin_refine_factors[i] < 1) {
            fprintf(stderr, "Warning: bin refine factor along axis = %d *must* be >=1. Instead found bin refine factor =%d\n",
                    i, options->bin_refine_factors[i]);
            reset_bin_refine_factors(options);
            break;
        }
    }
}

/* theory/vpf/countspheres.c:34-77 + theory/vpf/countspheres_impl.c.src:136-479 */
int countspheres(const int64_t np, void *X, void *Y, void *Z, const double rmax, const int nbin, const int nc,
                 const int num_pN, unsigned long seed, results_countspheres *results, struct config_options *options,
                 struct extra_options *extra)
{
    (void)extra;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    if (!(rmax > 0.0 && nbin > 0 && nc > 0 && num_pN > 0)) {
        CF_ERR("Invalid input parameters. Expected rmax > 0, number of bins > 0, number of random spheres > 0, number of "
               "pN's to calculate > 0.\nFound rmax = %lf, nbin = %d nspheres = %d num_pN = %d", rmax, nbin, nc, num_pN);
        return EXIT_FAILURE;
    }
    if (np < 1) {
        CF_ERR("vpf needs at least one particle");
        return EXIT_FAILURE;
    }
    refine_check(options);
    cf_mt19937 rng;
    cf_mt_seed(&rng, seed);
    const size_t es = options->float_type;
    double *P = malloc(sizeof(double) * 3 * (size_t)np);
    if (P == NULL) return EXIT_FAILURE;
    double *px = P, *py = P + np, *pz = P + 2 * np;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    for (int64_t i = 0; i < np; i++) {
        px[i] = wval(X, i, es);
        py[i] = wval(Y, i, es);
        pz[i] = wval(Z, i, es);
        const double v[3] = {px[i], py[i], pz[i]};
        for (int a = 0; a < 3; a++) {
            if (v[a] < lo[a]) lo[a] = v[a];
            if (v[a] > hi[a]) hi[a] = v[a];
        }
    }
    if (options->periodic && options->boxsize == BOXSIZE_NOTGIVEN) {
        fprintf(stderr, "boxsize = %g must be specified with periodic wrap. Please specify a non-zero boxsize, or zero to "
                "detect the particle extent, or -1 to make a dimension non-periodic.\n", options->boxsize);
        free(P);
        return EXIT_FAILURE;
    }
    const double bsz[3] = {options->boxsize_x,
                           options->boxsize_y == BOXSIZE_NOTGIVEN ? options->boxsize : options->boxsize_y,
                           options->boxsize_z == BOXSIZE_NOTGIVEN ? options->boxsize : options->boxsize_z};
    cf_vpf_job J;
    memset(&J, 0, sizeof(J));
    double wrap[3];
    for (int a = 0; a < 3; a++) {
        wrap[a] = (options->periodic && bsz[a] > 0) ? bsz[a] : (hi[a] - lo[a]);
        double binsize;
        if (cf_ref_binsize(hi[a] - lo[a], wrap[a], rmax, options->bin_refine_factors[a], options->max_cells_per_dim,
                           &binsize, &J.nmesh[a]) != EXIT_SUCCESS) {
            free(P);
            return EXIT_FAILURE;
        }
        J.lat_min[a] = lo[a];
        J.lat_inv[a] = binsize > 0 ? 1.0 / binsize : 0.0;
        J.refine[a] = options->bin_refine_factors[a];
        J.wrap[a] = wrap[a];
    }
    double *cen = malloc(sizeof(double) * 3 * (size_t)nc);
    int *cell = malloc(sizeof(int) * 3 * (size_t)nc);
    uint64_t *cnt = calloc((size_t)nbin * num_pN, sizeof(uint64_t));
    int rc = (cen && cell && cnt) ? EXIT_SUCCESS : EXIT_FAILURE;
    const double inv_wrap[3] = {1.0 / wrap[0], 1.0 / wrap[1], 1.0 / wrap[2]};
    for (int ic = 0; rc == EXIT_SUCCESS && ic < nc;) {
        double c[3];
        for (int a = 0; a < 3; a++) c[a] = wrap[a] * cf_mt_uniform(&rng) + lo[a];
        if (!options->periodic) {
            int near = 0;
            for (int a = 0; a < 3; a++) near |= (c[a] - lo[a]) < rmax || (hi[a] - c[a]) < rmax;
            if (near) continue;
        }
        for (int a = 0; a < 3; a++) {
            int k = (int)(J.nmesh[a] * (c[a] - lo[a]) * inv_wrap[a]);
            if (k > J.nmesh[a] - 1) k--;
            if (k < 0 || k >= J.nmesh[a]) {
                CF_ERR("%c-position = %lf with index = %d should be in [0, %d)", 'x' + a, c[a], k, J.nmesh[a]);
                rc = EXIT_FAILURE;
            }
            cen[3 * ic + a] = c[a];
            cell[3 * ic + a] = k;
        }
        ic++;
    }
    if (rc == EXIT_SUCCESS) {
        J.np = np;
        J.x = px; J.y = py; J.z = pz;
        J.periodic = options->periodic ? 1 : 0;
        J.ncen = nc;
        J.cen = cen;
        J.cen_cell = cell;
        J.rmax = rmax;
        J.nbin = nbin;
        J.num_pN = num_pN;
        rc = cf_engine_vpf(&J, cnt);
    }
    if (rc == EXIT_SUCCESS) {
        results->rmax = rmax;
        results->nbin = nbin;
        results->nc = nc;
        results->num_pN = num_pN;
        results->pN = pn_matrix(nbin, num_pN);
        if (results->pN == NULL) rc = EXIT_FAILURE;
        const double inv_nc = 1.0 / (double)nc;
        for (int i = 0; rc == EXIT_SUCCESS && i < num_pN; i++)
            for (int b = 0; b < nbin; b++) results->pN[b][i] = (double)cnt[(size_t)b * num_pN + i] * inv_nc;
    }
    free(P);
    free(cen);
    free(cell);
    free(cnt);
    if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_countspheres(results_countspheres *results)
{
    if (results == NULL) return;
    pn_free(results->pN, results->nbin);
    results->pN = NULL;
    results->rmax = 0.0;
    results->nbin = 0;
    results->nc = 0;
    results->num_pN = 0;
}

/* comoving XYZ of one catalogue shifted into the bounding cube; *dmax is raised to the largest
 * distance (mocks/vpf_mocks/countspheres_mocks_impl.c.src:309-370) */
static int vpf_mock_positions(int64_t n, const void *ra, const void *dec, const void *cz, size_t es, const double *zc,
                              const double *dcs, int nz, double *X, double *Y, double *Z, double *dmax)
{
    const double inv_c = 1.0 / CF_SPEED_OF_LIGHT;
    for (int64_t i = 0; i < n; i++) {
        double D = wval(cz, i, es);
        if (zc != NULL && interp_linear(zc, dcs, nz, D * inv_c, &D) != EXIT_SUCCESS) {
            CF_ERR("cz[%lld] = %g is outside the comoving-distance table", (long long)i, wval(cz, i, es));
            return EXIT_FAILURE;
        }
        if (D > *dmax) *dmax = D;
        const double r = wval(ra, i, es), d = wval(dec, i, es);
        X[i] = D * cos(d * CF_PI_OVER_180) * cos(r * CF_PI_OVER_180);
        Y[i] = D * cos(d * CF_PI_OVER_180) * sin(r * CF_PI_OVER_180);
        Z[i] = D * sin(d * CF_PI_OVER_180);
    }
    return EXIT_SUCCESS;
}

/* mocks/vpf_mocks/countspheres_mocks.c + countspheres_mocks_impl.c.src:208-638 */
int countspheres_mocks(const int64_t Ngal, void *xgal, void *ygal, void *zgal, const int64_t Nran, void *xran,
                       void *yran, void *zran, const int threshold_neighbors, const double rmax, const int nbin,
                       const int nc, const int num_pN, const char *centers_file, const int cosmology,
                       results_countspheres_mocks *results, struct config_options *options,
                       struct extra_options *extra)
{
    (void)extra;
    const double t0 = wall_now();
    if (check_options(options, __func__) != EXIT_SUCCESS || results == NULL) return EXIT_FAILURE;
    if (!(rmax > 0.0)) { CF_ERR("rmax=%lf has to be positive", rmax); return EXIT_FAILURE; }
    if (nbin < 1) { CF_ERR("Number of bins=%d has to be at least 1", nbin); return EXIT_FAILURE; }
    if (nc < 1) { CF_ERR("Number of spheres=%d has to be at least 1", nc); return EXIT_FAILURE; }
    if (num_pN < 1) { CF_ERR("Number of pN's=%d requested must be at least 1", num_pN); return EXIT_FAILURE; }
    double omega_m;
    if (cosmology_omega_m(cosmology, &omega_m) != EXIT_SUCCESS) return EXIT_FAILURE;
    options->periodic = 0;
    const size_t es = options->float_type;
    /* centres: the file when it holds at least nc centres for spheres of at least rmax, else
     * randoms with more than threshold_neighbors randoms within rmax (then written to the file) */
    int need_randoms = 0;
    int64_t num_in_file = 0;
    FILE *fpcen = centers_file ? fopen(centers_file, "r") : NULL;
    if (fpcen != NULL) {
        double rr = 0.0;
        if (fscanf(fpcen, "%*f %*f %*f %lf", &rr) != 1) {
            CF_ERR("Could not read max. sphere radius from the centers file");
            fclose(fpcen);
            return EXIT_FAILURE;
        }
        num_in_file = cf_getnumlines(centers_file, '#');
        if (rr >= rmax && num_in_file >= nc) {
            rewind(fpcen);
        } else {
            fclose(fpcen);
            fpcen = NULL;
            num_in_file = 0;
            need_randoms = 1;
        }
    } else {
        need_randoms = 1;
    }
    if (need_randoms) {
        fpcen = centers_file ? fopen(centers_file, "w") : NULL;
        if (fpcen == NULL) {
            CF_ERR("could not open the centers file `%s' for writing", centers_file ? centers_file : "(null)");
            return EXIT_FAILURE;
        }
    }
    double *zc = NULL, *dcs = NULL;
    int nz = 0, rc = EXIT_SUCCESS;
    if (!options->is_comoving_dist) {
        double czmax = 0.0;
        for (int64_t i = 0; i < Ngal; i++) if (wval(zgal, i, es) > czmax) czmax = wval(zgal, i, es);
        if (need_randoms)
            for (int64_t i = 0; i < Nran; i++) if (wval(zran, i, es) > czmax) czmax = wval(zran, i, es);
        const double zmax = czmax * (1.0 / CF_SPEED_OF_LIGHT) + 0.01;
        zc = calloc(10000, sizeof(double));
        dcs = calloc(10000, sizeof(double));
        if (!zc || !dcs) rc = EXIT_FAILURE;
        if (rc == EXIT_SUCCESS) nz = comoving_table(zmax, 10000, omega_m, zc, dcs);
        if (rc == EXIT_SUCCESS && nz < 2) rc = EXIT_FAILURE;
    }
    const int64_t nr = need_randoms ? Nran : 0;
    double *G = malloc(sizeof(double) * 3 * (size_t)(Ngal > 0 ? Ngal : 1));
    double *R = malloc(sizeof(double) * 3 * (size_t)(nr > 0 ? nr : 1));
    if (!G || !R) rc = EXIT_FAILURE;
    double rcube = 0.0;
    if (rc == EXIT_SUCCESS)
        rc = vpf_mock_positions(Ngal, xgal, ygal, zgal, es, zc, dcs, nz, G, G + Ngal, G + 2 * Ngal, &rcube);
    if (rc == EXIT_SUCCESS && nr > 0)
        rc = vpf_mock_positions(nr, xran, yran, zran, es, zc, dcs, nz, R, R + nr, R + 2 * nr, &rcube);
    free(zc);
    free(dcs);
    rcube = rcube + 1.;
    for (int64_t i = 0; rc == EXIT_SUCCESS && i < 3 * Ngal; i++) G[i] += rcube;
    for (int64_t i = 0; rc == EXIT_SUCCESS && i < 3 * nr; i++) R[i] += rcube;
    rcube = 2.0 * rcube;
    const double inv_rcube = 1.0 / rcube;
    refine_check(options);
    cf_vpf_job J;
    memset(&J, 0, sizeof(J));
    for (int a = 0; rc == EXIT_SUCCESS && a < 3; a++) {
        double binsize;
        rc = cf_ref_binsize(rcube, 0.0, rmax, options->bin_refine_factors[a], options->max_cells_per_dim, &binsize,
                            &J.nmesh[a]);
        J.lat_min[a] = 0.0;
        J.lat_inv[a] = binsize > 0 ? 1.0 / binsize : 0.0;
        J.refine[a] = options->bin_refine_factors[a];
    }
    J.periodic = 0;
    J.rmax = rmax;
    J.nbin = nbin;
    J.num_pN = num_pN;
    /* candidate centres and their cells */
    const int64_t maxc = need_randoms ? nr : (Nran < nc ? Nran : nc);
    double *cen = malloc(sizeof(double) * 3 * (size_t)(maxc > 0 ? maxc : 1));
    int *cell = malloc(sizeof(int) * 3 * (size_t)(maxc > 0 ? maxc : 1));
    uint32_t *ngb = need_randoms ? malloc(sizeof(uint32_t) * (size_t)(maxc > 0 ? maxc : 1)) : NULL;
    if (!cen || !cell || (need_randoms && !ngb)) rc = EXIT_FAILURE;
    int64_t ncand = 0;
    for (int64_t t = 0; rc == EXIT_SUCCESS && t < maxc; t++) {
        double c[3];
        if (need_randoms) {
            c[0] = R[t];
            c[1] = R[nr + t];
            c[2] = R[2 * nr + t];
        } else {
            char buf[10000];
            double rr = 0.0;
            if (fgets(buf, sizeof buf, fpcen) == NULL) {
                CF_ERR("Could not read-in co-ordinates for the centers of the randoms spheres from file %s", centers_file);
                rc = EXIT_FAILURE;
                break;
            }
            if (sscanf(buf, "%lf %lf %lf %lf", &c[0], &c[1], &c[2], &rr) != 4) {
                CF_ERR("Read the centers from the centers file (3 positions and 1 radius)");
                rc = EXIT_FAILURE;
                break;
            }
            if (!(rr >= rmax)) {
                CF_ERR("Rmax from the center file is >= rmax");
                rc = EXIT_FAILURE;
                break;
            }
        }
        for (int a = 0; a < 3; a++) {
            int k = (int)(J.nmesh[a] * (c[a] - 0.0) * inv_rcube);
            if (k > J.nmesh[a] - 1) k--;
            if (k < 0 || k >= J.nmesh[a]) {
                fprintf(stderr, "Error in countspheres_mocks> Positions are outside grid. (X,Y,Z) = (%lf,%lf,%lf) should have "
                        "been within the range [0.0, %lf]\n", c[0], c[1], c[2], 1.0 / inv_rcube);
                rc = EXIT_FAILURE;
            }
            cen[3 * t + a] = c[a];
            cell[3 * t + a] = k;
        }
        ncand++;
    }
    /* neighbour counts of the random candidates, then the first nc with more than the threshold */
    int64_t nacc = ncand;
    if (rc == EXIT_SUCCESS && need_randoms) {
        cf_vpf_job K = J;
        K.np = nr;
        K.x = R; K.y = R + nr; K.z = R + 2 * nr;
        K.ncen = ncand;
        K.cen = cen;
        K.cen_cell = cell;
        K.nbin = 1;
        K.num_pN = 1;
        K.counts_out = ngb;
        uint64_t dummy = 0;
        rc = cf_engine_vpf(&K, &dummy);
        nacc = 0;
        for (int64_t t = 0; rc == EXIT_SUCCESS && t < ncand && nacc < nc; t++) {
            if ((int64_t)ngb[t] > threshold_neighbors) {
                for (int a = 0; a < 3; a++) {
                    cen[3 * nacc + a] = cen[3 * t + a];
                    cell[3 * nacc + a] = cell[3 * t + a];
                }
                fprintf(fpcen, "%lf \t %lf \t %lf \t %lf\n", cen[3 * nacc], cen[3 * nacc + 1], cen[3 * nacc + 2], rmax);
                nacc++;
            }
        }
    }
    if (fpcen) fclose(fpcen);
    uint64_t *cnt = calloc((size_t)nbin * num_pN, sizeof(uint64_t));
    if (rc == EXIT_SUCCESS && cnt == NULL) rc = EXIT_FAILURE;
    if (rc == EXIT_SUCCESS && nacc <= 0) {
        CF_ERR("Could not place even a single sphere within the volume. Please reduce the radius of the sphere "
               "(currently set to %lf)", rmax);
        rc = EXIT_FAILURE;
    }
    if (rc == EXIT_SUCCESS) {
        if (nacc < nc)
            fprintf(stderr, "WARNING: Could only place `%lld' out of requested `%d' spheres. Increase the random-sample "
                    "size might improve the situation\n", (long long)nacc, nc);
        J.np = Ngal;
        J.x = G; J.y = G + Ngal; J.z = G + 2 * Ngal;
        J.ncen = nacc;
        J.cen = cen;
        J.cen_cell = cell;
        rc = cf_engine_vpf(&J, cnt);
    }
    if (rc == EXIT_SUCCESS) {
        results->rmax = rmax;
        results->nbin = nbin;
        results->nc = nc;
        results->num_pN = num_pN;
        results->pN = pn_matrix(nbin, num_pN);
        if (results->pN == NULL) rc = EXIT_FAILURE;
        const double inv_nc = 1.0 / (double)nacc;
        for (int i = 0; rc == EXIT_SUCCESS && i < num_pN; i++)
            for (int b = 0; b < nbin; b++) results->pN[b][i] = (double)cnt[(size_t)b * num_pN + i] * inv_nc;
    }
    free(G);
    free(R);
    free(cen);
    free(cell);
    free(ngb);
    free(cnt);
    if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    reset_bin_refine_factors(options);
    if (options->c_api_timer) options->c_api_time = wall_now() - t0;
    return EXIT_SUCCESS;
}

void free_results_countspheres_mocks(results_countspheres_mocks *results)
{
    if (results == NULL) return;
    pn_free(results->pN, results->nbin);
    results->pN = NULL;
    results->rmax = 0.0;
    results->nbin = 0;
    results->nc = 0;
    results->num_pN = 0;
}

int cf_gpu_set_precision(int mode) { return cf_engine_set_precision(mode); }

int cf_gpu_get_precision(void) { return cf_engine_get_precision(); }

int cf_gpu_set_autotune(int on) { return cf_engine_set_autotune(on); }

int cf_gpu_get_autotune(void) { return cf_engine_get_autotune(); }

int cf_gpu_last_stats(cf_gpu_stats *out)
{
    if (out == NULL) return EXIT_FAILURE;
    cf_engine_stats s;
    if (cf_engine_last_stats(&s) != EXIT_SUCCESS) return EXIT_FAILURE;
    out->pair_kernel_ms = s.pair_kernel_ms;
    out->gridlink_ms = s.gridlink_ms;
    out->total_gpu_ms = s.total_gpu_ms;
    out->pairs_evaluated = s.pairs_evaluated;
    out->pairs_refined = s.pairs_refined;
    out->tasks = s.tasks;
    out->kernel_launches = s.kernel_launches;
    out->num_cells = s.num_cells;
    out->blocks_per_sm = s.blocks_per_sm;
    out->warps_per_block = s.warps_per_block;
    out->lane_stride = s.lane_stride;
    out->column_split = s.column_split;
    out->pairs_slow = s.pairs_slow;
    return EXIT_SUCCESS;
}

int cf_gpu_fp32_peak_tflops(double *tflops)
{
    if (tflops == NULL) return EXIT_FAILURE;
    return cf_engine_fp32_peak(tflops);
}
