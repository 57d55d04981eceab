/*
 * cf_oracle.c -- ORACLE: CPU restatement of Corrfunc 2.5.3 pair counting (test infrastructure).
 *
 * This file is test infrastructure.  Only the test-suite, the smoke check and the CPU
 * baseline leg of bench.py load it, and only as the checker; the product library never
 * links or calls it.
 *
 * It evaluates every pair (brute force, OpenMP over the first set) with exactly the
 * double-precision arithmetic of the reference kernels, so that its raw histograms equal
 * the reference's on any input where the reference's own pruning is exact:
 *
 *   - wrap: the first point of a pair is shifted by the periodic offset and the separation
 *     is  d = x_second - (x_first + off)                (theory/DD/countpairs_kernels.c.src:894-896,954)
 *     Which point is "first" follows the reference's cell-pair order: in a cross-correlation
 *     always the point of set 1; in an auto-correlation the point whose reference-lattice cell
 *     has the larger linear index (utils/gridlink_impl.c.src:525, cells with icell2 > icell are
 *     skipped), ties broken by the per-cell z order (utils/gridlink_impl.c.src:380-424).
 *     The offset is the one image (0, +L or -L) that brings the pair within L/2; for any
 *     pair inside rmax < L/2 that is the offset the reference's neighbour stencil assigns
 *     (utils/gridlink_impl.c.src:500-518).
 *   - 3-D:  r2 = (dx*dx + dy*dy) + dz*dz  (fallback, countpairs_kernels.c.src:967) or
 *           fma(dz,dz, fma(dy,dy, dx*dx)) (AVX512F, countpairs_kernels.c.src:188-190);
 *           accept rmin^2 <= r2 < rmax^2, bin = max k with r2 >= rupp_sqr[k-1] (:968-990).
 *   - rp-pi: -pimax < dz < pimax, rp2 = dx*dx + dy*dy (or fma(dy,dy,dx*dx)),
 *           pibin = (int)(|dz| * inv_dpi) clamped to npibin, index kbin*(npibin+1)+pibin
 *           (theory/DDrppi/countpairs_rp_pi_kernels.c.src:1080-1112).
 *   - wp:   rp-pi acceptance, 1-D rp bins (theory/wp/wp_kernels.c.src:1459-1486).
 *   - s-mu: s2 = (dx*dx+dy*dy) + dz*dz, reject dz*dz >= s2*mu_max^2, mu = sqrt(dz*dz/s2),
 *           mubin = (int)(mu*inv_dmu) clamped (theory/DDsmu/countpairs_s_mu_kernels.c.src:1140-1171).
 *   - theta: cos = (x2*x1 + y2*y1) + z2*z1 on unit vectors, accept cosmax < cos <= cosmin,
 *           bin = max k with cos <= cos_upp[k-1]
 *           (mocks/DDtheta_mocks/countpairs_theta_mocks_kernels.c.src:138-192).
 *
 * Outputs are the *raw* per-bin sums (each unordered auto pair counted once); the
 * finalisation (x2 for auto, self pairs, averages, xi / wp) is restated in oracle.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { CFO_R3 = 0, CFO_RPPI = 1, CFO_WP = 2, CFO_SMU = 3, CFO_THETA = 4 };

typedef struct {
    int32_t mode;
    int32_t autocorr;
    int32_t fma_formula;   /* 1: the AVX512F kernels' fused formula, 0: unfused sums */
    int32_t chord_formula; /* theta only: 1 = cos = 1 - chord^2/2 (SIMD kernels), 0 = dot product */
    int32_t periodic[3];
    int32_t nmesh[3];      /* reference lattice, used for the first-point rule of wrapped auto pairs */
    double wrap[3];
    double lat_min[3];
    double lat_inv[3];
    int32_t nedges;        /* number of rupp entries (bins 1..nedges-1 are valid, bin 0 is junk) */
    int32_t npibin;        /* rp-pi: number of pi bins; s-mu: number of mu bins */
    double pimax;          /* rp-pi / wp: pimax; s-mu: mu_max */
    const double *edges;   /* rupp_sqr (3-D, rp, s) or cos(theta_upp) (theta) */
    int32_t need_avg;
    int32_t need_weight;
    int32_t fast_acos;     /* reserved */
    int32_t pad;
} cfo_params;

static inline int ref_cell(const cfo_params *p, double x, double y, double z)
{
    int ix = (int)((x - p->lat_min[0]) * p->lat_inv[0]);
    int iy = (int)((y - p->lat_min[1]) * p->lat_inv[1]);
    int iz = (int)((z - p->lat_min[2]) * p->lat_inv[2]);
    if (ix > p->nmesh[0] - 1) ix--;
    if (iy > p->nmesh[1] - 1) iy--;
    if (iz > p->nmesh[2] - 1) iz--;
    return (ix * p->nmesh[1] + iy) * p->nmesh[2] + iz;
}

static inline double image_offset(double xa, double xb, int periodic, double L)
{
    /* offset added to point a so that (xa + off) is the image nearest to xb */
    if (!periodic || !(L > 0.0)) return 0.0;
    const double d = xb - xa;
    if (d > 0.5 * L) return L;
    if (d < -0.5 * L) return -L;
    return 0.0;
}

/* Evaluate one pair (first = a, second = b, offset applied to a).  Returns the flat bin index
 * or -1, and the separation measure used for the average. */
static inline int eval_pair(const cfo_params *p, double xa, double ya, double za,
                            double xb, double yb, double zb,
                            double ox, double oy, double oz, double *avg_term)
{
    const double *e = p->edges;
    const int nb = p->nedges;
    if (p->mode == CFO_THETA) {
        double c;
        if (p->chord_formula) {
            const double dx = xb - xa, dy = yb - ya, dz = zb - za;
            double ch2;
            if (p->fma_formula) ch2 = fma(dz, dz, fma(dy, dy, dx * dx));
            else { volatile double t = dx * dx + dy * dy; ch2 = t + dz * dz; }
            c = 1.0 - 0.5 * ch2;
        } else {
            volatile double t = xb * xa + yb * ya;
            c = t + zb * za;
        }
        if (c > e[0] || c <= e[nb - 1]) return -1;
        for (int k = nb - 1; k >= 1; k--) {
            if (c <= e[k - 1]) {
                if (p->need_avg) *avg_term = 57.29577951308232087679815481410517033240547246656432154916024 * acos(c);
                return k;
            }
        }
        return -1;
    }
    const double xpos = xa + ox, ypos = ya + oy, zpos = za + oz;
    const double dx = xb - xpos, dy = yb - ypos, dz = zb - zpos;
    if (p->mode == CFO_R3) {
        double r2;
        if (p->fma_formula) r2 = fma(dz, dz, fma(dy, dy, dx * dx));
        else { volatile double t = dx * dx + dy * dy; r2 = t + dz * dz; }
        if (r2 >= e[nb - 1] || r2 < e[0]) return -1;
        for (int k = nb - 1; k >= 1; k--) {
            if (r2 >= e[k - 1]) {
                if (p->need_avg) *avg_term = sqrt(r2);
                return k;
            }
        }
        return -1;
    }
    if (p->mode == CFO_RPPI || p->mode == CFO_WP) {
        const double pimax = p->pimax;
        if (dz <= -pimax || dz >= pimax) return -1;
        const double adz = fabs(dz);
        double r2;
        if (p->fma_formula) r2 = fma(dy, dy, dx * dx);
        else r2 = dx * dx + dy * dy;
        if (r2 >= e[nb - 1] || r2 < e[0]) return -1;
        int kbin = -1;
        for (int k = nb - 1; k >= 1; k--) {
            if (r2 >= e[k - 1]) { kbin = k; break; }
        }
        if (kbin < 0) return -1;
        if (p->need_avg) *avg_term = sqrt(r2);
        if (p->mode == CFO_WP) return kbin;
        const int npibin = p->npibin;
        const double dpi = pimax / npibin;
        const double inv_dpi = 1.0 / dpi;
        int pibin = (int)(adz * inv_dpi);
        pibin = pibin > npibin ? npibin : pibin;
        return kbin * (npibin + 1) + pibin;
    }
    /* CFO_SMU */
    {
        const double mu_max = p->pimax;
        const int nmu = p->npibin;
        const double dmu = mu_max / nmu;
        const double inv_dmu = 1.0 / dmu;
        const double sqr_mu_max = mu_max * mu_max;
        double s2, sqr_dz;
        if (p->fma_formula) {
            sqr_dz = dz * dz;
            s2 = fma(dx, dx, fma(dy, dy, sqr_dz));
        } else {
            volatile double sqr_dx_dy = dx * dx + dy * dy;
            sqr_dz = dz * dz;
            s2 = sqr_dx_dy + sqr_dz;
        }
        if (s2 >= e[nb - 1] || s2 < e[0]) return -1;
        if (sqr_dz >= s2 * sqr_mu_max) return -1;
        const double mu = sqrt(sqr_dz / s2);
        int mubin = (int)(mu * inv_dmu);
        mubin = mubin > nmu ? nmu : mubin;
        for (int k = nb - 1; k >= 1; k--) {
            if (s2 >= e[k - 1]) {
                if (p->need_avg) *avg_term = sqrt(s2);
                return k * (nmu + 1) + mubin;
            }
        }
        return -1;
    }
}

int cfo_num_bins(const cfo_params *p)
{
    if (p->mode == CFO_RPPI || p->mode == CFO_SMU) return p->nedges * (p->npibin + 1);
    return p->nedges;
}

/* Raw histograms over all pairs.  Arrays npairs/avg/wsum have cfo_num_bins(p) entries and
 * are overwritten.  w1/w2 may be NULL when need_weight == 0. */
int cfo_count(const cfo_params *p,
              int64_t n1, const double *x1, const double *y1, const double *z1, const double *w1,
              int64_t n2, const double *x2, const double *y2, const double *z2, const double *w2,
              uint64_t *npairs, double *avg, double *wsum, int nthreads)
{
    const int nbins = cfo_num_bins(p);
    if (p->autocorr) {
        n2 = n1; x2 = x1; y2 = y1; z2 = z1; w2 = w1;
    }
    memset(npairs, 0, sizeof(uint64_t) * nbins);
    memset(avg, 0, sizeof(double) * nbins);
    memset(wsum, 0, sizeof(double) * nbins);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        uint64_t *ln = calloc(nbins, sizeof(uint64_t));
        double *la = calloc(nbins, sizeof(double));
        double *lw = calloc(nbins, sizeof(double));
#pragma omp for schedule(dynamic, 64)
        for (int64_t i = 0; i < n1; i++) {
            const int64_t j0 = p->autocorr ? i + 1 : 0;
            const int cell_i = (p->autocorr && p->mode != CFO_THETA) ? ref_cell(p, x1[i], y1[i], z1[i]) : 0;
            for (int64_t j = j0; j < n2; j++) {
                /* a = set-1 point, b = set-2 point; offsets that move a next to b */
                double ox = 0.0, oy = 0.0, oz = 0.0;
                if (p->mode != CFO_THETA) {
                    ox = image_offset(x1[i], x2[j], p->periodic[0], p->wrap[0]);
                    oy = image_offset(y1[i], y2[j], p->periodic[1], p->wrap[1]);
                    oz = image_offset(z1[i], z2[j], p->periodic[2], p->wrap[2]);
                }
                int swap = 0;
                if (p->autocorr && (ox != 0.0 || oy != 0.0 || oz != 0.0)) {
                    const int cell_j = ref_cell(p, x2[j], y2[j], z2[j]);
                    if (cell_j > cell_i) swap = 1;
                    else if (cell_j == cell_i) {
                        if (z2[j] < z1[i] || (z2[j] == z1[i] && j < i)) swap = 1;
                    }
                }
                double avg_term = 0.0;
                int bin;
                if (!swap) {
                    bin = eval_pair(p, x1[i], y1[i], z1[i], x2[j], y2[j], z2[j], ox, oy, oz, &avg_term);
                } else {
                    bin = eval_pair(p, x2[j], y2[j], z2[j], x1[i], y1[i], z1[i], -ox, -oy, -oz, &avg_term);
                }
                if (bin < 0) continue;
                ln[bin]++;
                if (p->need_avg) la[bin] += avg_term;
                if (p->need_weight) lw[bin] += w1[i] * w2[j];
            }
        }
#pragma omp critical
        {
            for (int b = 0; b < nbins; b++) {
                npairs[b] += ln[b];
                avg[b] += la[b];
                wsum[b] += lw[b];
            }
        }
        free(ln);
        free(la);
        free(lw);
    }
    return 0;
}
