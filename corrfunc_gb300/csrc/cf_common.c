/*
 * cf_common.c -- host-side helpers shared by the six entry points: bin-file parsing,
 * resolution of the reference's lattice geometry, and the double-precision formula
 * variant that the caller's reference run would use.
 */
#define _GNU_SOURCE
#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "corrfunc_gb300.h"
#include "cf_internal.h"
#include "cf_host.h"

/* Counts the lines that are neither blank nor start (after blanks) with the comment
 * character (utils/utils.c:715-745).  Returns -1 when the file cannot be opened. */
static int64_t count_data_lines(const char *fname, const char comment)
{
    char line[10000];
    FILE *fp = fopen(fname, "rt");
    if (fp == NULL) return -1;
    int64_t n = 0;
    while (fgets(line, sizeof(line), fp) != NULL) {
        const char *c = line;
        while (*c != '\0' && isspace((unsigned char)*c)) c++;
        if (*c != '\0' && *c != comment) n++;
    }
    fclose(fp);
    return n;
}

/* Bin file "low high" per line (utils/utils.c:62-106): nbin = data lines + 1,
 * rupp[0] = low of the first line, rupp[i] = high of line i, and rupp[nbin-1] = rmax. */
int cf_setup_bins(const char *fname, double *rmin, double *rmax, int *nbin, double **rupp)
{
    *rupp = NULL;
    *nbin = 0;
    if (fname == NULL) {
        fprintf(stderr, "Error: bin file name is NULL\n");
        return EXIT_FAILURE;
    }
    const int64_t nlines = count_data_lines(fname, '#');
    if (nlines < 0) {
        fprintf(stderr, "Error: Could not open bin file `%s'\n", fname);
        return EXIT_FAILURE;
    }
    *nbin = (int)nlines + 1;
    double *r = calloc((size_t)*nbin + 1, sizeof(double));
    if (r == NULL) return EXIT_FAILURE;
    FILE *fp = fopen(fname, "r");
    if (fp == NULL) {
        free(r);
        fprintf(stderr, "Error: Could not open bin file `%s'\n", fname);
        return EXIT_FAILURE;
    }
    char buf[1000];
    int index = 1;
    double lo, hi;
    *rmin = 0.0;
    while (fgets(buf, sizeof(buf), fp) != NULL) {
        if (sscanf(buf, "%lf %lf", &lo, &hi) == 2) {
            if (index == 1) {
                *rmin = lo;
                r[0] = lo;
            }
            if (index <= *nbin) r[index] = hi;
            index++;
        }
    }
    fclose(fp);
    *rmax = r[index - 1 <= *nbin ? index - 1 : *nbin];
    r[*nbin] = *rmax;
    r[*nbin - 1] = *rmax;
    *rupp = r;
    return EXIT_SUCCESS;
}

/* get_binsize (utils/gridlink_utils.c:31-49) */
static int ref_binsize(double xdiff, double xwrap, double rmax, int refine, int max_cells, double *binsize, int *nmesh)
{
    int n = (int)(refine * xdiff / rmax);
    n = n < 1 ? 1 : n;
    if (xwrap > 0 && rmax >= xwrap / 2) {
        fprintf(stderr, "Error: rmax=%f must be less than half of periodic boxize=%f to avoid double-counting particles\n",
                rmax, xwrap);
        return EXIT_FAILURE;
    }
    if (n > max_cells) n = max_cells;
    if (n < 2) n = 2;
    *binsize = xdiff / n;
    *nmesh = n;
    return EXIT_SUCCESS;
}

static int ref_gridsize(const double lo[3], const double hi[3], const double wrap[3], const double max_size[3],
                        const int refine[3], int max_cells, double binsize[3], int nmesh[3])
{
    for (int a = 0; a < 3; a++) {
        if (ref_binsize(hi[a] - lo[a], wrap[a], max_size[a], refine[a], max_cells, &binsize[a], &nmesh[a]) != EXIT_SUCCESS)
            return EXIT_FAILURE;
    }
    return EXIT_SUCCESS;
}

int cf_resolve_geometry(const cf_refrule *R, const double lo_in[3], const double hi_in[3], cf_geometry *G)
{
    memset(G, 0, sizeof(*G));
    if (R->kind == CF_REF_NONE) {
        for (int a = 0; a < 3; a++) {
            G->ref_nmesh[a] = 1;
            G->refine_used[a] = R->refine[a];
        }
        return EXIT_SUCCESS;
    }
    double lo[3], hi[3], wrap[3];
    int refine[3] = {R->refine[0], R->refine[1], R->refine[2]};
    if (R->kind == CF_REF_BOX) {
        /* xi / wp: lattice is the periodic box [0, L) on every axis */
        for (int a = 0; a < 3; a++) {
            lo[a] = 0.0;
            hi[a] = R->boxsize[a];
            wrap[a] = R->boxsize[a];
            G->periodic[a] = 1;
        }
    } else {
        for (int a = 0; a < 3; a++) {
            lo[a] = lo_in[a];
            hi[a] = hi_in[a];
            const int per = R->periodic && R->boxsize[a] >= 0;
            G->periodic[a] = per;
            wrap[a] = per ? (R->boxsize[a] > 0 ? R->boxsize[a] : (hi[a] - lo[a])) : 0.0;
        }
    }
    for (int a = 0; a < 3; a++) G->wrap[a] = wrap[a];
    if (!R->custom_refine) {
        switch (R->dfl_kind) {
        case CF_DFL_PER_AXIS:
            for (int a = 0; a < 3; a++)
                if (R->max_size[a] < 0.05 * wrap[a]) refine[a] = 1;
            break;
        case CF_DFL_XI:
            if (R->max_size[0] < 0.05 * R->boxsize[0])
                for (int a = 0; a < 3; a++) refine[a] = 1;
            break;
        case CF_DFL_WP:
            if (R->max_size[0] < 0.05 * R->boxsize[0]) refine[0] = refine[1] = 1;
            if (R->max_size[2] < 0.05 * R->boxsize[0]) refine[2] = 1;
            break;
        default:
            break;
        }
    }
    double binsize[3];
    int nmesh[3];
    if (ref_gridsize(lo, hi, wrap, R->max_size, refine, R->max_cells, binsize, nmesh) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    if (R->boost_kind == CF_BOOST_XY) {
        /* boost heuristic (theory/DD/countpairs_impl.c.src:298-332) */
        const double avg_np = ((double)R->np1) / ((double)nmesh[0] * nmesh[1] * nmesh[2]);
        int max_nmesh = nmesh[0];
        if (nmesh[1] > max_nmesh) max_nmesh = nmesh[1];
        if (nmesh[2] > max_nmesh) max_nmesh = nmesh[2];
        if ((max_nmesh <= 10 || avg_np >= 250) && max_nmesh < R->max_cells && !R->custom_refine) {
            refine[0] += 1;
            refine[1] += 1;
            if (ref_gridsize(lo, hi, wrap, R->max_size, refine, R->max_cells, binsize, nmesh) != EXIT_SUCCESS)
                return EXIT_FAILURE;
        }
    }
    for (int a = 0; a < 3; a++) {
        G->ref_min[a] = lo[a];
        G->ref_inv[a] = binsize[a] > 0 ? 1.0 / binsize[a] : 0.0;
        G->ref_nmesh[a] = nmesh[a];
        G->refine_used[a] = refine[a];
    }
    return EXIT_SUCCESS;
}

/* Which double-precision formula the reference run of the caller would evaluate.
 * The AVX512F kernels chain fused multiply-adds (theory/DD/countpairs_kernels.c.src:188-190,
 * theory/DDsmu/countpairs_s_mu_kernels.c.src:212-214); the AVX, SSE and fallback kernels sum
 * unfused products (countpairs_kernels.c.src:447,765,967).  The angular SIMD kernels use the
 * chord form cos = 1 - chord^2/2, the fallback a dot product
 * (mocks/DDtheta_mocks/countpairs_theta_mocks_kernels.c.src:147,483,1062-1066).
 * isa < 0 ("fastest") resolves to what the reference would pick on this host. */
void cf_formula_for_isa(int isa, int *fma_formula, int *chord_formula)
{
    int eff = isa;
    if (eff < 0 || eff >= 11) {
#if defined(__x86_64__) || defined(__i386__)
        __builtin_cpu_init();
        if (__builtin_cpu_supports("avx512f")) eff = 9;
        else if (__builtin_cpu_supports("avx")) eff = 7;
        else if (__builtin_cpu_supports("sse4.2")) eff = 6;
        else eff = 0;
#else
        eff = 0;
#endif
    }
    *fma_formula = eff == 9 ? 1 : 0;
    *chord_formula = (eff >= 6 && eff <= 9) ? 1 : 0;
}

int64_t cf_getnumlines(const char *fname, char comment) { return count_data_lines(fname, comment); }

int cf_ref_binsize(double xdiff, double xwrap, double rmax, int refine, int max_cells, double *binsize, int *nmesh)
{
    return ref_binsize(xdiff, xwrap, rmax, refine, max_cells, binsize, nmesh);
}

/* MT19937: state recurrence with the twist constants 0x9908b0df, tempering shifts 11, 7 / 0x9d2c5680,
 * 15 / 0xefc60000, 18, and the seeding x_i = 1812433253 (x_{i-1} ^ (x_{i-1} >> 30)) + i of the
 * published 2002 reference implementation. */
void cf_mt_seed(cf_mt19937 *g, unsigned long seed)
{
    if (seed == 0) seed = 4357;
    g->mt[0] = (uint32_t)(seed & 0xffffffffUL);
    for (int i = 1; i < 624; i++) g->mt[i] = 1812433253u * (g->mt[i - 1] ^ (g->mt[i - 1] >> 30)) + (uint32_t)i;
    g->mti = 624;
}

uint32_t cf_mt_next(cf_mt19937 *g)
{
    if (g->mti >= 624) {
        for (int k = 0; k < 624; k++) {
            const uint32_t y = (g->mt[k] & 0x80000000u) | (g->mt[(k + 1) % 624] & 0x7fffffffu);
            g->mt[k] = g->mt[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
        }
        g->mti = 0;
    }
    uint32_t y = g->mt[g->mti++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

double cf_mt_uniform(cf_mt19937 *g) { return cf_mt_next(g) / 4294967296.0; }

/* reference lattice rule of a call whose lattice spans the data extent (gridlink on the points'
 * bounding box, theory/DD/countpairs_impl.c.src:231-332) */
void cf_fill_rule_extent(cf_refrule *R, const struct config_options *options, double sx, double sy, double sz,
                         int dfl_kind, int boost_kind, int64_t np1)
{
    memset(R, 0, sizeof(*R));
    R->kind = CF_REF_EXTENT;
    R->periodic = options->periodic;
    R->boxsize[0] = options->boxsize_x;
    R->boxsize[1] = options->boxsize_y == BOXSIZE_NOTGIVEN ? options->boxsize_x : options->boxsize_y;
    R->boxsize[2] = options->boxsize_z == BOXSIZE_NOTGIVEN ? options->boxsize_x : options->boxsize_z;
    R->max_size[0] = sx;
    R->max_size[1] = sy;
    R->max_size[2] = sz;
    for (int a = 0; a < 3; a++) R->refine[a] = options->bin_refine_factors[a];
    R->custom_refine = (options->binning_flags & BINNING_REF_MASK) == BINNING_CUST;
    R->max_cells = options->max_cells_per_dim;
    R->dfl_kind = dfl_kind;
    R->boost_kind = boost_kind;
    R->np1 = np1;
}
