/*
 * cf_workunit.c -- the benchmark's work unit, on the host only.
 *
 * Built into libcorrfunc_gb300.so (where cf_reference_candidate_pairs is exported with the
 * other entry points) and, with cf_common.c, into the GPU-free libcf_workunit.so, which the
 * CPU-only measurements load so that they never map the GPU library.
 */
#define _GNU_SOURCE
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "corrfunc_gb300.h"
#include "cf_internal.h"
#include "cf_host.h"

static double wval(const void *w, int64_t j, size_t es)
{
    return es == sizeof(float) ? (double)((const float *)w)[j] : ((const double *)w)[j];
}

/* ---------------- reference-lattice work unit ----------------
 * Candidate pairs of the reference's own cell-pair list for a countpairs() call: the sum over
 * the cell pairs produced by generate_cell_pairs (utils/gridlink_impl.c.src:439-625, with the
 * default refine rule, boost, duplicate suppression and min-separation prune exactly as the
 * reference applies them) of n1*n2, or n*(n-1)/2 for a cell with itself in an auto-correlation.
 * This is the algorithmic unit "pair evaluations" is quoted in; it does not depend on how the
 * GPU tiles the work. */
typedef struct {
    int64_t n;
    double lo[3], hi[3];
} ref_cell;

static void ref_cells(int64_t np, const void *X, const void *Y, const void *Z, size_t es, const cf_geometry *G,
                      ref_cell *cells)
{
    const int nx = G->ref_nmesh[0], ny = G->ref_nmesh[1], nz = G->ref_nmesh[2];
    for (int64_t i = 0; i < np; i++) {
        const double p[3] = {wval(X, i, es), wval(Y, i, es), wval(Z, i, es)};
        int idx[3];
        for (int a = 0; a < 3; a++) {
            int c = (int)((p[a] - G->ref_min[a]) * G->ref_inv[a]);
            if (c > G->ref_nmesh[a] - 1) c--;
            if (c < 0) c = 0;
            idx[a] = c;
        }
        ref_cell *cl = &cells[((int64_t)idx[0] * ny + idx[1]) * nz + idx[2]];
        for (int a = 0; a < 3; a++) {
            if (cl->n == 0 || p[a] < cl->lo[a]) cl->lo[a] = p[a];
            if (cl->n == 0 || p[a] > cl->hi[a]) cl->hi[a] = p[a];
        }
        cl->n++;
    }
    (void)nx;
}

int cf_reference_candidate_pairs(const int64_t ND1, void *X1, void *Y1, void *Z1, const int64_t ND2, void *X2,
                                 void *Y2, void *Z2, const int autocorr, const char *binfile,
                                 struct config_options *options, uint64_t *candidates)
{
    if (options == NULL || candidates == NULL ||
        !(options->float_type == sizeof(float) || options->float_type == sizeof(double)))
        return EXIT_FAILURE;
    *candidates = 0;
    double *rupp = NULL, rmin, rmax;
    int nbin;
    if (cf_setup_bins(binfile, &rmin, &rmax, &nbin, &rupp) != EXIT_SUCCESS) return EXIT_FAILURE;
    free(rupp);
    if (!(rmin >= 0.0 && rmax > 0.0 && rmin < rmax && nbin > 0)) return EXIT_FAILURE;
    const size_t es = options->float_type;
    const int64_t n2 = autocorr ? ND1 : ND2;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int s = 0; s < (autocorr ? 1 : 2); s++) {
        const void *P[3] = {s ? X2 : X1, s ? Y2 : Y1, s ? Z2 : Z1};
        const int64_t n = s ? n2 : ND1;
        for (int64_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) {
                const double v = wval(P[a], i, es);
                if (v < lo[a]) lo[a] = v;
                if (v > hi[a]) hi[a] = v;
            }
    }
    cf_refrule R;
    cf_fill_rule_extent(&R, options, rmax, rmax, rmax, CF_DFL_PER_AXIS, CF_BOOST_XY, ND1);
    cf_geometry G;
    if (cf_resolve_geometry(&R, lo, hi, &G) != EXIT_SUCCESS) return EXIT_FAILURE;
    const int nx = G.ref_nmesh[0], ny = G.ref_nmesh[1], nz = G.ref_nmesh[2];
    const int64_t ncell = (int64_t)nx * ny * nz;
    ref_cell *c1 = calloc((size_t)ncell, sizeof(ref_cell));
    ref_cell *c2 = autocorr ? c1 : calloc((size_t)ncell, sizeof(ref_cell));
    if (!c1 || !c2) {
        free(c1);
        if (!autocorr) free(c2);
        return EXIT_FAILURE;
    }
    ref_cells(ND1, X1, Y1, Z1, es, &G, c1);
    if (!autocorr) ref_cells(n2, X2, Y2, Z2, es, &G, c2);
    const int rx = G.refine_used[0], ry = G.refine_used[1], rz = G.refine_used[2];
    const int any_per = G.periodic[0] || G.periodic[1] || G.periodic[2];
    const int dup_check = any_per && (nx < 2 * rx + 1 || ny < 2 * ry + 1 || nz < 2 * rz + 1);
    const int max_ngb = (2 * rx + 1) * (2 * ry + 1) * (2 * rz + 1);
    int64_t *seen_cell = malloc(sizeof(int64_t) * max_ngb);
    double *seen_off = malloc(sizeof(double) * 3 * max_ngb);
    uint64_t total = 0;
    const double sqr_rmax = rmax * rmax;
    for (int64_t icell = 0; icell < ncell; icell++) {
        const ref_cell *first = &c1[icell];
        if (first->n == 0) continue;
        const int iz = (int)(icell % nz), ix = (int)(icell / ((int64_t)ny * nz)), iy = (int)((icell / nz) % ny);
        int nseen = 0;
        for (int iix = -rx; iix <= rx; iix++) {
            const int ux = ix + iix;
            const int px = G.periodic[0] ? (ux + nx) % nx : ux;
            if (px < 0 || px >= nx) continue;
            const double offx = (ux >= 0 && ux < nx) ? 0.0 : (ux < 0 ? G.wrap[0] : -G.wrap[0]);
            for (int iiy = -ry; iiy <= ry; iiy++) {
                const int uy = iy + iiy;
                const int py = G.periodic[1] ? (uy + ny) % ny : uy;
                if (py < 0 || py >= ny) continue;
                const double offy = (uy >= 0 && uy < ny) ? 0.0 : (uy < 0 ? G.wrap[1] : -G.wrap[1]);
                for (int iiz = -rz; iiz <= rz; iiz++) {
                    const int uz = iz + iiz;
                    const int pz = G.periodic[2] ? (uz + nz) % nz : uz;
                    if (pz < 0 || pz >= nz) continue;
                    const double offz = (uz >= 0 && uz < nz) ? 0.0 : (uz < 0 ? G.wrap[2] : -G.wrap[2]);
                    const int64_t icell2 = pz + (int64_t)nz * py + (int64_t)nz * ny * px;
                    if ((autocorr && icell2 > icell) || c2[icell2].n == 0) continue;
                    if (dup_check) {
                        int dup = 0;
                        for (int k = 0; k < nseen; k++)
                            if (seen_cell[k] == icell2 && seen_off[3 * k] == offx && seen_off[3 * k + 1] == offy &&
                                seen_off[3 * k + 2] == offz) {
                                dup = 1;
                                break;
                            }
                        if (dup) continue;
                    }
                    const ref_cell *second = &c2[icell2];
                    if (options->enable_min_sep_opt) {
                        const double xl = first->lo[0] + offx, xh = first->hi[0] + offx;
                        const double yl = first->lo[1] + offy, yh = first->hi[1] + offy;
                        const double zl = first->lo[2] + offz, zh = first->hi[2] + offz;
                        const double mdx = iix != 0 ? ((iix < 0 ? xl : xh) - (iix < 0 ? second->hi[0] : second->lo[0])) : 0.0;
                        const double mdy = iiy != 0 ? ((iiy < 0 ? yl : yh) - (iiy < 0 ? second->hi[1] : second->lo[1])) : 0.0;
                        const double mdz = iiz != 0 ? ((iiz < 0 ? zl : zh) - (iiz < 0 ? second->hi[2] : second->lo[2])) : 0.0;
                        if (mdx * mdx + mdy * mdy + mdz * mdz >= sqr_rmax) continue;
                    }
                    if (dup_check) {
                        seen_cell[nseen] = icell2;
                        seen_off[3 * nseen] = offx;
                        seen_off[3 * nseen + 1] = offy;
                        seen_off[3 * nseen + 2] = offz;
                        nseen++;
                    }
                    if (autocorr && icell2 == icell) total += (uint64_t)first->n * (uint64_t)(first->n - 1) / 2;
                    else total += (uint64_t)first->n * (uint64_t)second->n;
                }
            }
        }
    }
    free(seen_cell);
    free(seen_off);
    free(c1);
    if (!autocorr) free(c2);
    *candidates = total;
    return EXIT_SUCCESS;
}
