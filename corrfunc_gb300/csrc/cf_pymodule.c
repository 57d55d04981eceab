/*
 * cf_pymodule.c -- CPython extension modules `_countpairs` (theory) and `_countpairs_mocks`
 * (angular mocks) over the C ABI of libcorrfunc_gb300.
 *
 * The functions take the arguments of the reference's compiled bindings -- same names, order,
 * keyword lists and argument types (theory/python_bindings/_countpairs.c:1166-1195 for
 * countpairs, :1471-1500 rp_pi, :1773-1797 wp, :2015-2038 xi, :2243-2274 s_mu;
 * mocks/python_bindings/_countpairs_mocks.c:1764-1792 theta) -- and return the same values: a
 * list of per-bin tuples and the C API time, plus the (empty) per-cell timings for wp.  On an
 * error they print the reason and return None, which the reference's Python wrappers turn into
 * RuntimeError.  Positions are 1-D float32 or float64 arrays, weights a 2-D array of shape
 * (n_weights, n_particles) of the same type.  The GIL is released around the count.
 *
 * The same source builds both modules; each .so exports the init function of its own name.
 */
#define PY_SSIZE_T_CLEAN
#include <Python.h>
#define NPY_NO_DEPRECATED_API NPY_1_7_API_VERSION
#include <numpy/arrayobject.h>

#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include "corrfunc_gb300.h"

/* ---------------- shared argument handling ---------------- */

static PyObject *fail(const char *fn, const char *why)
{
    fprintf(stderr, "corrfunc_gb300 %s: %s\n", fn, why);
    Py_RETURN_NONE;
}

/* Borrowed input arrays of one particle set and their contiguous, aligned versions. */
typedef struct {
    PyArrayObject *in[4];  /* x, y, z (z NULL for angular sets), weights (may be NULL) */
    PyObject *arr[4];      /* owned contiguous views */
    int64_t n;
    int elem;              /* 4 or 8 */
    int nweights;
} cf_pyset;

static void set_release(cf_pyset *s)
{
    for (int k = 0; k < 4; k++) {
        Py_XDECREF(s->arr[k]);
        s->arr[k] = NULL;
    }
}

/* Checks dimensions and dtypes (1-D positions, 2-D weights, float32/float64, one dtype) and
 * makes contiguous aligned views.  Returns 0, or -1 with the reason in msg. */
static int set_prepare(cf_pyset *s, int npos, char *msg, size_t msglen)
{
    int type = -1;
    s->n = -1;
    for (int k = 0; k < npos; k++) {
        PyArrayObject *a = s->in[k];
        if (PyArray_NDIM(a) != 1) {
            snprintf(msg, msglen, "ERROR: expected 1-D position arrays, found %d dimensions", PyArray_NDIM(a));
            return -1;
        }
        const int t = PyArray_TYPE(a);
        if (t != NPY_FLOAT && t != NPY_DOUBLE) {
            snprintf(msg, msglen, "TypeError: positions must be float32 or float64 arrays (found type number %d)", t);
            return -1;
        }
        if (type >= 0 && t != type) {
            snprintf(msg, msglen, "TypeError: all position arrays of a set must have the same dtype");
            return -1;
        }
        type = t;
        const int64_t n = (int64_t)PyArray_DIM(a, 0);
        if (s->n >= 0 && n != s->n) {
            snprintf(msg, msglen, "ValueError: position arrays of one set differ in length (%lld vs %lld)",
                     (long long)s->n, (long long)n);
            return -1;
        }
        s->n = n;
    }
    s->nweights = 0;
    if (s->in[3] != NULL) {
        PyArrayObject *w = s->in[3];
        if (PyArray_NDIM(w) != 2) {
            snprintf(msg, msglen, "ERROR: expected a 2-D weight array of shape (n_weights_per_particle, n_particles), "
                     "found %d dimensions", PyArray_NDIM(w));
            return -1;
        }
        if (PyArray_TYPE(w) != type) {
            snprintf(msg, msglen, "TypeError: weights must have the dtype of the positions");
            return -1;
        }
        if ((int64_t)PyArray_DIM(w, 1) != s->n) {
            snprintf(msg, msglen, "ValueError: weights hold %lld particles, positions %lld",
                     (long long)PyArray_DIM(w, 1), (long long)s->n);
            return -1;
        }
        s->nweights = (int)PyArray_DIM(w, 0);
    }
    s->elem = type == NPY_FLOAT ? 4 : 8;
    for (int k = 0; k < 4; k++) {
        if (s->in[k] == NULL) continue;
        s->arr[k] = PyArray_FromArray(s->in[k], NULL, NPY_ARRAY_IN_ARRAY);
        if (s->arr[k] == NULL) {
            PyErr_Clear();
            snprintf(msg, msglen, "TypeError: could not convert the inputs to contiguous floating-point arrays");
            return -1;
        }
    }
    return 0;
}

static void *set_data(cf_pyset *s, int k) { return s->arr[k] ? PyArray_DATA((PyArrayObject *)s->arr[k]) : NULL; }

/* weight_type string -> method; NULL means no weights */
static int weight_method(const char *name, weight_method_t *m)
{
    if (name == NULL) {
        *m = NONE;
        return 0;
    }
    return get_weight_method_by_name(name, m) == EXIT_SUCCESS ? 0 : -1;
}

/* Common preparation of the one or two sets of a pair count.  npos = 3 (x, y, z) or 2 (RA, DEC). */
static int prepare_sets(const char *fn, int autocorr, int npos, cf_pyset *s1, cf_pyset *s2, const char *wname,
                        struct extra_options *extra, int *elem)
{
    char msg[512];
    weight_method_t m;
    if (weight_method(wname, &m) != 0) {
        snprintf(msg, sizeof msg, "ValueError: unknown weight_type \"%s\"", wname);
        fail(fn, msg);
        return -1;
    }
    if (m == NONE) s1->in[3] = s2->in[3] = NULL;  /* weights are ignored without a method */
    if (set_prepare(s1, npos, msg, sizeof msg) != 0) {
        fail(fn, msg);
        return -1;
    }
    *extra = get_extra_options(m);
    if (extra->weights0.num_weights > 0 && extra->weights0.num_weights != s1->nweights) {
        snprintf(msg, sizeof msg, "ValueError: weight_type %s needs %lld weight(s) per particle, found %d", wname,
                 (long long)extra->weights0.num_weights, s1->nweights);
        fail(fn, msg);
        return -1;
    }
    if (!autocorr) {
        for (int k = 0; k < npos; k++) {
            if (s2->in[k] == NULL) {
                fail(fn, "ValueError: a cross-correlation (autocorr = 0) needs the second set of positions");
                return -1;
            }
        }
        if ((s1->in[3] == NULL) != (s2->in[3] == NULL)) {
            fail(fn, "ValueError: a cross-correlation takes weights for both sets or for neither");
            return -1;
        }
        if (set_prepare(s2, npos, msg, sizeof msg) != 0) {
            fail(fn, msg);
            return -1;
        }
        if (s2->elem != s1->elem) {
            fail(fn, "TypeError: the two sets must have the same dtype");
            return -1;
        }
    }
    for (int k = 0; k < extra->weights0.num_weights; k++) {
        extra->weights0.weights[k] = (char *)set_data(s1, 3) + (size_t)k * s1->n * s1->elem;
        if (!autocorr) extra->weights1.weights[k] = (char *)set_data(s2, 3) + (size_t)k * s2->n * s2->elem;
    }
    *elem = s1->elem;
    return 0;
}

static void refine_options(struct config_options *o, int8_t rx, int8_t ry, int8_t rz)
{
    if (rx != o->bin_refine_factors[0] || ry != o->bin_refine_factors[1] || rz != o->bin_refine_factors[2]) {
        o->bin_refine_factors[0] = rx;
        o->bin_refine_factors[1] = ry;
        o->bin_refine_factors[2] = rz;
        set_bin_refine_scheme(o, BINNING_CUST);
    }
}

static struct config_options theory_defaults(void)
{
    struct config_options o = get_config_options();
    o.verbose = 0;
    o.instruction_set = -1;
    o.periodic = 1;
    o.need_avg_sep = 0;
    o.c_api_timer = 0;
    o.copy_particles = 1;
    o.enable_min_sep_opt = 1;
    return o;
}

static PyObject *with_time(PyObject *list, const struct config_options *o)
{
    if (list == NULL) return NULL;
    PyObject *t = Py_BuildValue("(Od)", list, o->c_api_timer ? o->c_api_time : 0.0);
    Py_DECREF(list);
    return t;
}

/* ---------------- theory ---------------- */

static PyObject *py_countpairs(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"autocorr", "nthreads", "binfile", "X1", "Y1", "Z1", "weights1", "X2", "Y2", "Z2",
                         "weights2", "periodic", "verbose", "boxsize", "output_ravg", "xbin_refine_factor",
                         "ybin_refine_factor", "zbin_refine_factor", "max_cells_per_dim", "copy_particles",
                         "enable_min_sep_opt", "c_api_timer", "isa", "weight_type", NULL};
    int autocorr = 0, nthreads = 4;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = theory_defaults();
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "iisO!O!O!|O!O!O!O!O!bb(ddd)bbbbhbbbis", kw, &autocorr, &nthreads,
                                     &binfile, &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type,
                                     &s1.in[2], &PyArray_Type, &s1.in[3], &PyArray_Type, &s2.in[0], &PyArray_Type,
                                     &s2.in[1], &PyArray_Type, &s2.in[2], &PyArray_Type, &s2.in[3], &o.periodic,
                                     &o.verbose, &o.boxsize_x, &o.boxsize_y, &o.boxsize_z, &o.need_avg_sep, &rx, &ry,
                                     &rz, &o.max_cells_per_dim, &o.copy_particles, &o.enable_min_sep_opt,
                                     &o.c_api_timer, &o.instruction_set, &wname)) {
        PyErr_Clear();
        return fail("countpairs", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs", autocorr, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), autocorr ? 0 : s2.n,
                    autocorr ? NULL : set_data(&s2, 0), autocorr ? NULL : set_data(&s2, 1),
                    autocorr ? NULL : set_data(&s2, 2), nthreads, autocorr, binfile, &r, &o, &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    set_release(&s2);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    for (int i = 1; list && i < r.nbin; i++) {
        PyObject *it = Py_BuildValue("(dddkd)", r.rupp[i - 1], r.rupp[i], r.rpavg[i], (unsigned long)r.npairs[i],
                                     r.weightavg[i]);
        PyList_Append(list, it);
        Py_XDECREF(it);
    }
    free_results(&r);
    return with_time(list, &o);
}

static PyObject *py_countpairs_rp_pi(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"autocorr", "nthreads", "pimax", "binfile", "X1", "Y1", "Z1", "weights1", "X2", "Y2",
                         "Z2", "weights2", "periodic", "verbose", "boxsize", "output_rpavg", "xbin_refine_factor",
                         "ybin_refine_factor", "zbin_refine_factor", "max_cells_per_dim", "copy_particles",
                         "enable_min_sep_opt", "c_api_timer", "isa", "weight_type", NULL};
    int autocorr = 0, nthreads = 4;
    double pimax = 0.0;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = theory_defaults();
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "iidsO!O!O!|O!O!O!O!O!bb(ddd)bbbbhbbbis", kw, &autocorr,
                                     &nthreads, &pimax, &binfile, &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1],
                                     &PyArray_Type, &s1.in[2], &PyArray_Type, &s1.in[3], &PyArray_Type, &s2.in[0],
                                     &PyArray_Type, &s2.in[1], &PyArray_Type, &s2.in[2], &PyArray_Type, &s2.in[3],
                                     &o.periodic, &o.verbose, &o.boxsize_x, &o.boxsize_y, &o.boxsize_z,
                                     &o.need_avg_sep, &rx, &ry, &rz, &o.max_cells_per_dim, &o.copy_particles,
                                     &o.enable_min_sep_opt, &o.c_api_timer, &o.instruction_set, &wname)) {
        PyErr_Clear();
        return fail("countpairs_rp_pi", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs_rp_pi", autocorr, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs_rp_pi r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs_rp_pi(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), autocorr ? 0 : s2.n,
                          autocorr ? NULL : set_data(&s2, 0), autocorr ? NULL : set_data(&s2, 1),
                          autocorr ? NULL : set_data(&s2, 2), nthreads, autocorr, binfile, pimax, &r, &o, &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    set_release(&s2);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    const double dpi = pimax / r.npibin;
    for (int i = 1; list && i < r.nbin; i++) {
        for (int j = 0; j < r.npibin; j++) {
            const int b = i * (r.npibin + 1) + j;
            PyObject *it = Py_BuildValue("(ddddkd)", r.rupp[i - 1], r.rupp[i], r.rpavg[b], (j + 1) * dpi,
                                         (unsigned long)r.npairs[b], r.weightavg[b]);
            PyList_Append(list, it);
            Py_XDECREF(it);
        }
    }
    free_results_rp_pi(&r);
    return with_time(list, &o);
}

static PyObject *py_countpairs_s_mu(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"autocorr", "nthreads", "binfile", "mu_max", "nmu_bins", "X1", "Y1", "Z1", "weights1",
                         "X2", "Y2", "Z2", "weights2", "periodic", "verbose", "boxsize", "output_savg",
                         "fast_divide_and_NR_steps", "xbin_refine_factor", "ybin_refine_factor",
                         "zbin_refine_factor", "max_cells_per_dim", "copy_particles", "enable_min_sep_opt",
                         "c_api_timer", "isa", "weight_type", NULL};
    int autocorr = 0, nthreads = 4, nmu = 0;
    double mu_max = 1.0;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = theory_defaults();
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "iisdiO!O!O!|O!O!O!O!O!bb(ddd)bbbbbhbbbis", kw, &autocorr,
                                     &nthreads, &binfile, &mu_max, &nmu, &PyArray_Type, &s1.in[0], &PyArray_Type,
                                     &s1.in[1], &PyArray_Type, &s1.in[2], &PyArray_Type, &s1.in[3], &PyArray_Type,
                                     &s2.in[0], &PyArray_Type, &s2.in[1], &PyArray_Type, &s2.in[2], &PyArray_Type,
                                     &s2.in[3], &o.periodic, &o.verbose, &o.boxsize_x, &o.boxsize_y, &o.boxsize_z,
                                     &o.need_avg_sep, &o.fast_divide_and_NR_steps, &rx, &ry, &rz,
                                     &o.max_cells_per_dim, &o.copy_particles, &o.enable_min_sep_opt, &o.c_api_timer,
                                     &o.instruction_set, &wname)) {
        PyErr_Clear();
        return fail("countpairs_s_mu", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs_s_mu", autocorr, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs_s_mu r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs_s_mu(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), autocorr ? 0 : s2.n,
                         autocorr ? NULL : set_data(&s2, 0), autocorr ? NULL : set_data(&s2, 1),
                         autocorr ? NULL : set_data(&s2, 2), nthreads, autocorr, binfile, mu_max, nmu, &r, &o,
                         &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    set_release(&s2);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    const double dmu = r.mu_max / r.nmu_bins;
    for (int i = 1; list && i < r.nsbin; i++) {
        for (int j = 0; j < r.nmu_bins; j++) {
            const int b = i * (r.nmu_bins + 1) + j;
            PyObject *it = Py_BuildValue("(ddddkd)", r.supp[i - 1], r.supp[i], r.savg[b], (j + 1) * dmu,
                                         (unsigned long)r.npairs[b], r.weightavg[b]);
            PyList_Append(list, it);
            Py_XDECREF(it);
        }
    }
    free_results_s_mu(&r);
    return with_time(list, &o);
}

static PyObject *py_countpairs_wp(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"boxsize", "pimax", "nthreads", "binfile", "X", "Y", "Z", "weights", "weight_type",
                         "verbose", "output_rpavg", "xbin_refine_factor", "ybin_refine_factor",
                         "zbin_refine_factor", "max_cells_per_dim", "copy_particles", "enable_min_sep_opt",
                         "c_api_timer", "c_cell_timer", "isa", NULL};
    double boxsize = 0.0, pimax = 0.0;
    int nthreads = 4;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = theory_defaults();
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "ddisO!O!O!|O!sbbbbbhbbbbi", kw, &boxsize, &pimax, &nthreads,
                                     &binfile, &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type,
                                     &s1.in[2], &PyArray_Type, &s1.in[3], &wname, &o.verbose, &o.need_avg_sep, &rx,
                                     &ry, &rz, &o.max_cells_per_dim, &o.copy_particles, &o.enable_min_sep_opt,
                                     &o.c_api_timer, &o.c_cell_timer, &o.instruction_set)) {
        PyErr_Clear();
        return fail("countpairs_wp", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs_wp", 1, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs_wp r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs_wp(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), boxsize, nthreads, binfile, pimax,
                       &r, &o, &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    for (int i = 1; list && i < r.nbin; i++) {
        PyObject *it = Py_BuildValue("(ddddkd)", r.rupp[i - 1], r.rupp[i], r.rpavg[i], r.wp[i],
                                     (unsigned long)r.npairs[i], r.weightavg[i]);
        PyList_Append(list, it);
        Py_XDECREF(it);
    }
    free_results_wp(&r);
    /* per cell-pair timings (theory/python_bindings/_countpairs.c:1972-1983): one tuple per GPU
     * work-list task, (N1, N2, time_in_ns, first index, second index, warp) */
    PyObject *cells = PyList_New(0);
    if (o.c_cell_timer && cells) {
        const struct api_cell_timings *c = o.cell_timings;
        for (int64_t k = 0; k < o.totncells_timings; k++, c++) {
            PyObject *it = Py_BuildValue("(LLLiii)", (long long)c->N1, (long long)c->N2, (long long)c->time_in_ns,
                                         c->first_cellindex, c->second_cellindex, c->tid);
            PyList_Append(cells, it);
            Py_XDECREF(it);
        }
        free_cell_timings(&o);
    }
    PyObject *t = Py_BuildValue("(OdO)", list, o.c_api_timer ? o.c_api_time : 0.0, cells);
    Py_XDECREF(list);
    Py_XDECREF(cells);
    return t;
}

static PyObject *py_countpairs_xi(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"boxsize", "nthreads", "binfile", "X", "Y", "Z", "weights", "weight_type", "verbose",
                         "output_ravg", "xbin_refine_factor", "ybin_refine_factor", "zbin_refine_factor",
                         "max_cells_per_dim", "copy_particles", "enable_min_sep_opt", "c_api_timer", "isa", NULL};
    double boxsize = 0.0;
    int nthreads = 4;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = theory_defaults();
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "disO!O!O!|O!sbbbbbhbbbi", kw, &boxsize, &nthreads, &binfile,
                                     &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type, &s1.in[2],
                                     &PyArray_Type, &s1.in[3], &wname, &o.verbose, &o.need_avg_sep, &rx, &ry, &rz,
                                     &o.max_cells_per_dim, &o.copy_particles, &o.enable_min_sep_opt, &o.c_api_timer,
                                     &o.instruction_set)) {
        PyErr_Clear();
        return fail("countpairs_xi", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs_xi", 1, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs_xi r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs_xi(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), boxsize, nthreads, binfile, &r,
                       &o, &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    for (int i = 1; list && i < r.nbin; i++) {
        PyObject *it = Py_BuildValue("(ddddkd)", r.rupp[i - 1], r.rupp[i], r.ravg[i], r.xi[i],
                                     (unsigned long)r.npairs[i], r.weightavg[i]);
        PyList_Append(list, it);
        Py_XDECREF(it);
    }
    free_results_xi(&r);
    return with_time(list, &o);
}

/* ---------------- angular mocks ---------------- */

static PyObject *py_countpairs_theta_mocks(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"autocorr", "nthreads", "binfile", "RA1", "DEC1", "weights1", "RA2", "DEC2", "weights2",
                         "link_in_dec", "link_in_ra", "verbose", "output_thetaavg", "fast_acos",
                         "ra_refine_factor", "dec_refine_factor", "max_cells_per_dim", "copy_particles",
                         "enable_min_sep_opt", "c_api_timer", "isa", "weight_type", NULL};
    int autocorr = 0, nthreads = 1;
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = get_config_options();
    o.verbose = 0;
    o.instruction_set = -1;
    o.link_in_dec = 1;
    o.link_in_ra = 1;
    o.fast_acos = 0;
    o.c_api_timer = 0;
    o.enable_min_sep_opt = 1;
    o.copy_particles = 1;
    int8_t rr = o.bin_refine_factors[0], rd = o.bin_refine_factors[1];
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "iisO!O!|O!O!O!O!bbbbbbbhbbbis", kw, &autocorr, &nthreads,
                                     &binfile, &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type,
                                     &s1.in[3], &PyArray_Type, &s2.in[0], &PyArray_Type, &s2.in[1], &PyArray_Type,
                                     &s2.in[3], &o.link_in_dec, &o.link_in_ra, &o.verbose, &o.need_avg_sep,
                                     &o.fast_acos, &rr, &rd, &o.max_cells_per_dim, &o.copy_particles,
                                     &o.enable_min_sep_opt, &o.c_api_timer, &o.instruction_set, &wname)) {
        PyErr_Clear();
        return fail("countpairs_theta_mocks", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rr, rd, o.bin_refine_factors[2]);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countpairs_theta_mocks", autocorr, 2, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countpairs_theta r;
    int rc;
    /* the reference fixes RA/DEC ranges in place; the arrays passed are the contiguous views */
    Py_BEGIN_ALLOW_THREADS
    rc = countpairs_theta_mocks(s1.n, set_data(&s1, 0), set_data(&s1, 1), autocorr ? s1.n : s2.n,
                                autocorr ? set_data(&s1, 0) : set_data(&s2, 0),
                                autocorr ? set_data(&s1, 1) : set_data(&s2, 1), nthreads, autocorr, binfile, &r, &o,
                                &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    set_release(&s2);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = PyList_New(0);
    for (int i = 1; list && i < r.nbin; i++) {
        PyObject *it = Py_BuildValue("(dddkd)", r.theta_upp[i - 1], r.theta_upp[i], r.theta_avg[i],
                                     (unsigned long)r.npairs[i], r.weightavg[i]);
        PyList_Append(list, it);
        Py_XDECREF(it);
    }
    free_results_countpairs_theta(&r);
    return with_time(list, &o);
}

/* Shared body of countpairs_rp_pi_mocks / countpairs_s_mu_mocks: kwlists and format strings of
 * mocks/python_bindings/_countpairs_mocks.c:1124-1154 (rp_pi) and :1449-1479 (s_mu); rows
 * (low, high, avg, (j + 1) * width, npairs, weightavg) as built at :1390-1404 and :1716-1730. */
static PyObject *mocks_2d(PyObject *args, PyObject *kwargs, int smu)
{
    const char *fn = smu ? "countpairs_s_mu_mocks" : "countpairs_rp_pi_mocks";
    static char *kw_rppi[] = {"autocorr", "cosmology", "nthreads", "pimax", "binfile", "RA1", "DEC1", "CZ1",
                              "weights1", "RA2", "DEC2", "CZ2", "weights2", "is_comoving_dist", "verbose",
                              "output_rpavg", "fast_divide_and_NR_steps", "xbin_refine_factor", "ybin_refine_factor",
                              "zbin_refine_factor", "max_cells_per_dim", "copy_particles", "enable_min_sep_opt",
                              "c_api_timer", "isa", "weight_type", NULL};
    static char *kw_smu[] = {"autocorr", "cosmology", "nthreads", "mu_max", "nmu_bins", "binfile", "RA1", "DEC1",
                             "CZ1", "weights1", "RA2", "DEC2", "CZ2", "weights2", "is_comoving_dist", "verbose",
                             "output_savg", "fast_divide_and_NR_steps", "xbin_refine_factor", "ybin_refine_factor",
                             "zbin_refine_factor", "max_cells_per_dim", "copy_particles", "enable_min_sep_opt",
                             "c_api_timer", "isa", "weight_type", NULL};
    int autocorr = 1, nthreads = 4, cosmology = 1, nmu_bins = 0;
    double width_max = 0.0;  /* pimax or mu_max */
    char *binfile = NULL, *wname = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = get_config_options();
    o.is_comoving_dist = 0;
    o.verbose = 0;
    o.instruction_set = -1;
    o.periodic = 0;
    o.fast_divide_and_NR_steps = 0;
    o.c_api_timer = 0;
    o.enable_min_sep_opt = 1;
    o.copy_particles = 1;
    int8_t rx = o.bin_refine_factors[0], ry = o.bin_refine_factors[1], rz = o.bin_refine_factors[2];
    int ok;
    if (smu) {
        ok = PyArg_ParseTupleAndKeywords(args, kwargs, "iiidisO!O!O!|O!O!O!O!O!bbbbbbbhbbbis", kw_smu, &autocorr,
                                         &cosmology, &nthreads, &width_max, &nmu_bins, &binfile, &PyArray_Type,
                                         &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type, &s1.in[2], &PyArray_Type,
                                         &s1.in[3], &PyArray_Type, &s2.in[0], &PyArray_Type, &s2.in[1], &PyArray_Type,
                                         &s2.in[2], &PyArray_Type, &s2.in[3], &o.is_comoving_dist, &o.verbose,
                                         &o.need_avg_sep, &o.fast_divide_and_NR_steps, &rx, &ry, &rz,
                                         &o.max_cells_per_dim, &o.copy_particles, &o.enable_min_sep_opt,
                                         &o.c_api_timer, &o.instruction_set, &wname);
    } else {
        ok = PyArg_ParseTupleAndKeywords(args, kwargs, "iiidsO!O!O!|O!O!O!O!O!bbbbbbbhbbbis", kw_rppi, &autocorr,
                                         &cosmology, &nthreads, &width_max, &binfile, &PyArray_Type, &s1.in[0],
                                         &PyArray_Type, &s1.in[1], &PyArray_Type, &s1.in[2], &PyArray_Type, &s1.in[3],
                                         &PyArray_Type, &s2.in[0], &PyArray_Type, &s2.in[1], &PyArray_Type, &s2.in[2],
                                         &PyArray_Type, &s2.in[3], &o.is_comoving_dist, &o.verbose, &o.need_avg_sep,
                                         &o.fast_divide_and_NR_steps, &rx, &ry, &rz, &o.max_cells_per_dim,
                                         &o.copy_particles, &o.enable_min_sep_opt, &o.c_api_timer,
                                         &o.instruction_set, &wname);
    }
    if (!ok) {
        PyErr_Clear();
        return fail(fn, "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets(fn, autocorr, 3, &s1, &s2, wname, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    void *r2 = autocorr ? set_data(&s1, 0) : set_data(&s2, 0);
    void *d2 = autocorr ? set_data(&s1, 1) : set_data(&s2, 1);
    void *c2 = autocorr ? set_data(&s1, 2) : set_data(&s2, 2);
    const int64_t n2 = autocorr ? s1.n : s2.n;
    int rc;
    PyObject *list = NULL;
    if (smu) {
        results_countpairs_mocks_s_mu r;
        Py_BEGIN_ALLOW_THREADS
        rc = countpairs_mocks_s_mu(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), n2, r2, d2, c2,
                                   nthreads, autocorr, binfile, width_max, nmu_bins, cosmology, &r, &o, &extra);
        Py_END_ALLOW_THREADS
        set_release(&s1);
        set_release(&s2);
        if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
        list = PyList_New(0);
        const double dmu = width_max / (double)r.nmu_bins;
        for (int i = 1; list && r.npairs && i < r.nsbin; i++) {
            for (int j = 0; j < r.nmu_bins; j++) {
                const int b = i * (r.nmu_bins + 1) + j;
                PyObject *it = Py_BuildValue("(ddddkd)", r.supp[i - 1], r.supp[i], r.savg[b], (j + 1) * dmu,
                                             (unsigned long)r.npairs[b], r.weightavg[b]);
                PyList_Append(list, it);
                Py_XDECREF(it);
            }
        }
        free_results_mocks_s_mu(&r);
    } else {
        results_countpairs_mocks r;
        Py_BEGIN_ALLOW_THREADS
        rc = countpairs_mocks(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), n2, r2, d2, c2, nthreads,
                              autocorr, binfile, width_max, cosmology, &r, &o, &extra);
        Py_END_ALLOW_THREADS
        set_release(&s1);
        set_release(&s2);
        if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
        list = PyList_New(0);
        const double dpi = width_max / (double)r.npibin;
        for (int i = 1; list && r.npairs && i < r.nbin; i++) {
            for (int j = 0; j < r.npibin; j++) {
                const int b = i * (r.npibin + 1) + j;
                PyObject *it = Py_BuildValue("(ddddkd)", r.rupp[i - 1], r.rupp[i], r.rpavg[b], (j + 1) * dpi,
                                             (unsigned long)r.npairs[b], r.weightavg[b]);
                PyList_Append(list, it);
                Py_XDECREF(it);
            }
        }
        free_results_mocks(&r);
    }
    return with_time(list, &o);
}

static PyObject *py_countpairs_rp_pi_mocks(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    return mocks_2d(args, kwargs, 0);
}

static PyObject *py_countpairs_s_mu_mocks(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    return mocks_2d(args, kwargs, 1);
}

/* rows [rmax_k, pN[k][0], ..., pN[k][num_pN-1]] with rmax_k = (k + 1) * rmax / nbin
 * (theory/python_bindings/_countpairs.c:2674-2690) */
static PyObject *vpf_list(double **pN, double rmax, int nbin, int num_pN)
{
    PyObject *ret = PyList_New(0);
    const double rstep = rmax / (double)nbin;
    for (int b = 0; ret && b < nbin; b++) {
        PyObject *item = PyList_New(0);
        PyObject *v = Py_BuildValue("d", (b + 1) * rstep);
        PyList_Append(item, v);
        Py_XDECREF(v);
        for (int i = 0; i < num_pN; i++) {
            v = Py_BuildValue("d", pN[b][i]);
            PyList_Append(item, v);
            Py_XDECREF(v);
        }
        PyList_Append(ret, item);
        Py_XDECREF(item);
    }
    return ret;
}

/* countspheres_vpf: kwlist and format of theory/python_bindings/_countpairs.c:2552-2586 */
static PyObject *py_countspheres_vpf(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"rmax", "nbins", "nspheres", "num_pN", "seed", "X", "Y", "Z", "periodic", "verbose",
                         "boxsize", "xbin_refine_factor", "ybin_refine_factor", "zbin_refine_factor",
                         "max_cells_per_dim", "copy_particles", "c_api_timer", "isa", NULL};
    double rmax;
    int nbin, nc, num_pN;
    unsigned long seed = (unsigned long)-1;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = get_config_options();
    o.verbose = 0;
    o.periodic = 1;
    o.instruction_set = -1;
    o.copy_particles = 1;
    o.c_api_timer = 0;
    for (int k = 0; k < 3; k++) o.bin_refine_factors[k] = 1;
    int8_t rx = 1, ry = 1, rz = 1;
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "diiikO!O!O!|bb(ddd)bbbhbbi", kw, &rmax, &nbin, &nc, &num_pN, &seed,
                                     &PyArray_Type, &s1.in[0], &PyArray_Type, &s1.in[1], &PyArray_Type, &s1.in[2],
                                     &o.periodic, &o.verbose, &o.boxsize_x, &o.boxsize_y, &o.boxsize_z, &rx, &ry, &rz,
                                     &o.max_cells_per_dim, &o.copy_particles, &o.c_api_timer, &o.instruction_set)) {
        PyErr_Clear();
        return fail("countspheres_vpf", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countspheres_vpf", 1, 3, &s1, &s2, NULL, &extra, &elem) != 0) {
        set_release(&s1);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countspheres r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countspheres(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), rmax, nbin, nc, num_pN, seed, &r, &o,
                      &extra);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = vpf_list(r.pN, rmax, r.nbin, num_pN);
    free_results_countspheres(&r);
    return with_time(list, &o);
}

/* countspheres_vpf_mocks: kwlist and format of mocks/python_bindings/_countpairs_mocks.c:2067-2108 */
static PyObject *py_countspheres_vpf_mocks(PyObject *self, PyObject *args, PyObject *kwargs)
{
    (void)self;
    static char *kw[] = {"rmax", "nbins", "numSpheres", "numpN", "threshold", "centers_file", "cosmology", "X1", "Y1",
                         "Z1", "X2", "Y2", "Z2", "is_comoving_dist", "verbose", "xbin_refine_factor",
                         "ybin_refine_factor", "zbin_refine_factor", "max_cells_per_dim", "copy_particles",
                         "c_api_timer", "isa", NULL};
    double rmax;
    int nbin, nc, num_pN, threshold, cosmology = 1;
    char *centers_file = NULL;
    cf_pyset s1 = {{0}}, s2 = {{0}};
    struct config_options o = get_config_options();
    o.is_comoving_dist = 0;
    o.verbose = 0;
    o.instruction_set = -1;
    o.copy_particles = 1;
    o.c_api_timer = 0;
    for (int k = 0; k < 3; k++) o.bin_refine_factors[k] = 1;
    int8_t rx = 1, ry = 1, rz = 1;
    if (!PyArg_ParseTupleAndKeywords(args, kwargs, "diiiisiO!O!O!O!O!O!|bbbbbhbbi", kw, &rmax, &nbin, &nc, &num_pN,
                                     &threshold, &centers_file, &cosmology, &PyArray_Type, &s1.in[0], &PyArray_Type,
                                     &s1.in[1], &PyArray_Type, &s1.in[2], &PyArray_Type, &s2.in[0], &PyArray_Type,
                                     &s2.in[1], &PyArray_Type, &s2.in[2], &o.is_comoving_dist, &o.verbose, &rx, &ry,
                                     &rz, &o.max_cells_per_dim, &o.copy_particles, &o.c_api_timer,
                                     &o.instruction_set)) {
        PyErr_Clear();
        return fail("countspheres_vpf_mocks", "ArgumentError: could not parse the arguments");
    }
    refine_options(&o, rx, ry, rz);
    struct extra_options extra;
    int elem = 8;
    if (prepare_sets("countspheres_vpf_mocks", 0, 3, &s1, &s2, NULL, &extra, &elem) != 0) {
        set_release(&s1);
        set_release(&s2);
        Py_RETURN_NONE;
    }
    o.float_type = (uint8_t)elem;
    results_countspheres_mocks r;
    int rc;
    Py_BEGIN_ALLOW_THREADS
    rc = countspheres_mocks(s1.n, set_data(&s1, 0), set_data(&s1, 1), set_data(&s1, 2), s2.n, set_data(&s2, 0),
                            set_data(&s2, 1), set_data(&s2, 2), threshold, rmax, nbin, nc, num_pN, centers_file,
                            cosmology, &r, &o, NULL);
    Py_END_ALLOW_THREADS
    set_release(&s1);
    set_release(&s2);
    if (rc != EXIT_SUCCESS) Py_RETURN_NONE;
    PyObject *list = vpf_list(r.pN, rmax, r.nbin, num_pN);
    free_results_countspheres_mocks(&r);
    return with_time(list, &o);
}

/* ---------------- module tables ---------------- */

static PyMethodDef theory_methods[] = {
    {"countpairs", (PyCFunction)(void (*)(void))py_countpairs, METH_VARARGS | METH_KEYWORDS,
     "3-D pair counts DD(r) (countpairs)."},
    {"countpairs_rp_pi", (PyCFunction)(void (*)(void))py_countpairs_rp_pi, METH_VARARGS | METH_KEYWORDS,
     "Pair counts in (rp, pi) (countpairs_rp_pi)."},
    {"countpairs_wp", (PyCFunction)(void (*)(void))py_countpairs_wp, METH_VARARGS | METH_KEYWORDS,
     "Projected correlation function wp(rp) in a periodic box (countpairs_wp)."},
    {"countpairs_xi", (PyCFunction)(void (*)(void))py_countpairs_xi, METH_VARARGS | METH_KEYWORDS,
     "Correlation function xi(r) in a periodic box (countpairs_xi)."},
    {"countpairs_s_mu", (PyCFunction)(void (*)(void))py_countpairs_s_mu, METH_VARARGS | METH_KEYWORDS,
     "Pair counts in (s, mu) (countpairs_s_mu)."},
    {"countspheres_vpf", (PyCFunction)(void (*)(void))py_countspheres_vpf, METH_VARARGS | METH_KEYWORDS,
     "Counts in spheres pN(r) (countspheres)."},
    {NULL, NULL, 0, NULL}};

static PyMethodDef mocks_methods[] = {
    {"countpairs_theta_mocks", (PyCFunction)(void (*)(void))py_countpairs_theta_mocks, METH_VARARGS | METH_KEYWORDS,
     "Angular pair counts DD(theta) on the sky (countpairs_theta_mocks)."},
    {"countpairs_rp_pi_mocks", (PyCFunction)(void (*)(void))py_countpairs_rp_pi_mocks, METH_VARARGS | METH_KEYWORDS,
     "Pair counts in (rp, pi) of survey catalogues (countpairs_mocks)."},
    {"countpairs_s_mu_mocks", (PyCFunction)(void (*)(void))py_countpairs_s_mu_mocks, METH_VARARGS | METH_KEYWORDS,
     "Pair counts in (s, mu) of survey catalogues (countpairs_mocks_s_mu)."},
    {"countspheres_vpf_mocks", (PyCFunction)(void (*)(void))py_countspheres_vpf_mocks, METH_VARARGS | METH_KEYWORDS,
     "Counts in spheres of survey catalogues (countspheres_mocks)."},
    {NULL, NULL, 0, NULL}};

static struct PyModuleDef theory_module = {PyModuleDef_HEAD_INIT, "_countpairs",
                                           "GPU pair counters with the arguments of Corrfunc's _countpairs.", -1,
                                           theory_methods, NULL, NULL, NULL, NULL};
static struct PyModuleDef mocks_module = {PyModuleDef_HEAD_INIT, "_countpairs_mocks",
                                          "GPU angular pair counter with the arguments of Corrfunc's "
                                          "_countpairs_mocks.",
                                          -1, mocks_methods, NULL, NULL, NULL, NULL};

static PyObject *make_module(struct PyModuleDef *def)
{
    import_array();
    PyObject *m = PyModule_Create(def);
    if (m == NULL) return NULL;
    PyModule_AddStringConstant(m, "__version__", "2.5.3");
    return m;
}

PyMODINIT_FUNC PyInit__countpairs(void) { return make_module(&theory_module); }
PyMODINIT_FUNC PyInit__countpairs_mocks(void) { return make_module(&mocks_module); }
