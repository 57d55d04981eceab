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
 *   - rp-pi and s-mu of survey catalogues (comoving XYZ, observer at the origin, no wrap):
 *           s = x2 - x1, l = x1 + x2, pi^2 = (s.l)^2 / |l|^2, rp^2 = s^2 - pi^2, mu^2 = (s.l)^2 / (|l|^2 s^2)
 *           (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_kernels.c.src:1232-1283,
 *            mocks/DDsmu_mocks/countpairs_s_mu_mocks_kernels.c.src:1173-1206), in the three
 *           formula families of those files (fallback, AVX/SSE, AVX512F).
 *   - cz -> comoving distance (utils/set_cosmo_dist.c:26-67, Simpson table; linear
 *           interpolation in z = cz / c as gsl_interp_linear evaluates it) and XYZ
 *           (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_impl.c.src:318-392): cfo_mock_xyz.
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

enum { CFO_R3 = 0, CFO_RPPI = 1, CFO_WP = 2, CFO_SMU = 3, CFO_THETA = 4, CFO_RPPI_MOCK = 5, CFO_SMU_MOCK = 6 };

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
    if (p->mode == CFO_RPPI_MOCK || p->mode == CFO_SMU_MOCK) {
        const double parx = xa + xb, pary = ya + yb, parz = za + zb;
        const double perpx = xb - xa, perpy = yb - ya, perpz = zb - za;
        double s2, sdl, l2;
        if (p->fma_formula) {
            s2 = fma(perpx, perpx, fma(perpy, perpy, perpz * perpz));
            volatile double t = parx * perpx + pary * perpy;
            sdl = fma(parz, perpz, t);
            l2 = fma(parx, parx, fma(pary, pary, parz * parz));
        } else if (p->chord_formula) {
            volatile double t1 = perpy * perpy + perpz * perpz, t2 = pary * perpy + parx * perpx,
                            t3 = pary * pary + parz * parz;
            s2 = perpx * perpx + t1;
            sdl = parz * perpz + t2;
            l2 = parx * parx + t3;
        } else {
            volatile double t1 = perpx * perpx + perpy * perpy, t2 = parx * perpx + pary * perpy,
                            t3 = parx * parx + pary * pary;
            s2 = t1 + perpz * perpz;
            sdl = t2 + parz * perpz;
            l2 = t3 + parz * parz;
        }
        const int simd = p->fma_formula || p->chord_formula;
        const double sqr_sdl = sdl * sdl;
        const int nrow = p->npibin + 1;
        double ratio, limit, inv_d;
        int kbin = -1;
        if (p->mode == CFO_RPPI_MOCK) {
            const double pimax = p->pimax, sqr_pimax = pimax * pimax;
            if (s2 >= e[nb - 1] + sqr_pimax) return -1;
            if (sqr_sdl >= l2 * sqr_pimax) return -1;
            ratio = sqr_sdl / l2;
            limit = sqr_pimax;
            inv_d = 1.0 / (pimax / p->npibin);
            const double dperp2 = s2 - ratio;
            if (dperp2 >= e[nb - 1] || dperp2 < e[0]) return -1;
            for (int k = nb - 1; k >= 1; k--) if (dperp2 >= e[k - 1]) { kbin = k; break; }
            if (p->need_avg) *avg_term = sqrt(dperp2);
        } else {
            const double mu_max = p->pimax;
            if (s2 >= e[nb - 1] || s2 < e[0]) return -1;
            ratio = sqr_sdl / (l2 * s2);
            if (ratio != ratio) return -1;
            limit = mu_max * mu_max;
            inv_d = 1.0 / (mu_max / (double)p->npibin);
            for (int k = nb - 1; k >= 1; k--) if (s2 >= e[k - 1]) { kbin = k; break; }
            if (p->need_avg) *avg_term = sqrt(s2);
        }
        if (kbin < 0) return -1;
        const double t = sqrt(ratio) * inv_d;
        if (simd) {
            if (!(ratio < limit)) return -1;
            int flat = (int)((double)(kbin * nrow) + t);
            return flat > kbin * nrow + p->npibin ? kbin * nrow + p->npibin : flat;
        }
        int b = ratio >= limit ? p->npibin : (int)t;
        b = b > p->npibin ? p->npibin : b;
        return kbin * nrow + b;
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
    if (p->mode == CFO_RPPI || p->mode == CFO_SMU || p->mode == CFO_RPPI_MOCK || p->mode == CFO_SMU_MOCK)
        return p->nedges * (p->npibin + 1);
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
    /* mocks: pairs with |dz| beyond the largest separation are rejected by the per-pair test
     * anyway; skipping them only saves time */
    double zcut = INFINITY;
    if (p->mode == CFO_RPPI_MOCK) zcut = sqrt(p->edges[p->nedges - 1] + p->pimax * p->pimax) * (1.0 + 1e-9) + 1e-300;
    if (p->mode == CFO_SMU_MOCK) zcut = sqrt(p->edges[p->nedges - 1]) * (1.0 + 1e-9) + 1e-300;
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
                if (fabs(z2[j] - z1[i]) >= zcut) continue;
                /* a = set-1 point, b = set-2 point; offsets that move a next to b */
                double ox = 0.0, oy = 0.0, oz = 0.0;
                if (p->mode != CFO_THETA && p->mode != CFO_RPPI_MOCK && p->mode != CFO_SMU_MOCK) {
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

/* ---- survey positions: cz -> comoving distance -> XYZ ---- */

/* D_c(z) table (utils/set_cosmo_dist.c:26-67): Simpson's rule on 1/E(z), step 1e-2/max_size,
 * a sample every 1/max_size; returns the number of samples. */
static int cfo_cosmo_table(double zmax, int max_size, double omega_m, double *zc, double *dc)
{
    const double OL = 1.0 - omega_m;
    const double Ok = 1.0 - omega_m - OL;
    const double Dh = 299800.0 * 0.01 / 1.0;
    const double Deltaz = 1.0 / max_size;
    const double dz = 1e-2 * Deltaz;
    double Eint = 0.0, E2 = 1.0, z2 = Deltaz;
    int n = 0;
    for (double z = 2.0 * dz; z < zmax; z += 2.0 * dz) {
        const double E0 = E2;
        const double u = 1 + z - dz, v = 1 + z;
        const double E1 = 1.0 / sqrt(omega_m * (u * u * u) + Ok * (1 + z - dz) + OL);
        E2 = 1.0 / sqrt(omega_m * (v * v * v) + Ok * (1 + z) + OL);
        Eint += dz * (E0 + 4. * E1 + E2) / 3.;
        if (z > (z2 - 1e-10) && z < (z2 + 1e-10)) {
            if (n >= max_size) break;
            zc[n] = z;
            dc[n] = Eint * Dh;
            z2 += Deltaz;
            n++;
        }
    }
    return n;
}

/* Positions of one catalogue (and, when dist is not NULL, the distances).  is_comoving: cz already holds the distance.  Otherwise the
 * table spans z up to zmax (max cz / c + 0.01 over the catalogues of the call).  Returns 0, or
 * -1 when a redshift falls outside the table. */
int cfo_mock_xyz(int64_t n, const double *ra, const double *dec, const double *cz, int is_comoving, double omega_m,
                 double zmax, double *x, double *y, double *z, double *dist)
{
    const double P = 0.017453292519943295769236907684886127134428718885417254560971;
    const int max_size = 10000;
    double *zc = NULL, *dc = NULL;
    int nz = 0;
    if (!is_comoving) {
        zc = calloc(max_size, sizeof(double));
        dc = calloc(max_size, sizeof(double));
        nz = cfo_cosmo_table(zmax, max_size, omega_m, zc, dc);
    }
    const double inv_c = 1.0 / 299800.0;
    int rc = 0;
    for (int64_t i = 0; i < n; i++) {
        double D = cz[i];
        if (!is_comoving) {
            const double zz = cz[i] * inv_c;
            if (nz < 2 || !(zz >= zc[0] && zz <= zc[nz - 1])) { rc = -1; break; }
            int lo = 0, hi = nz - 1;
            while (hi > lo + 1) {
                const int mid = (lo + hi) / 2;
                if (zc[mid] > zz) hi = mid; else lo = mid;
            }
            D = dc[lo] + (zz - zc[lo]) / (zc[lo + 1] - zc[lo]) * (dc[lo + 1] - dc[lo]);
        }
        if (dist) dist[i] = D;
        x[i] = D * cos(dec[i] * P) * cos(ra[i] * P);
        y[i] = D * cos(dec[i] * P) * sin(ra[i] * P);
        z[i] = D * sin(dec[i] * P);
    }
    free(zc);
    free(dc);
    return rc;
}

/* ---- counts in spheres (vpf) ----
 * MT19937 restated from its published description (Matsumoto & Nishimura 1998; 2002 seeding),
 * seed 0 -> 4357 and uniform = output / 2^32 as GSL's mt19937 (theory/vpf/countspheres_impl.c.src:188-190,
 * 281-283).  n uniforms into out. */
void cfo_mt_uniforms(unsigned long seed, int64_t n, double *out)
{
    uint32_t mt[624];
    if (seed == 0) seed = 4357;
    mt[0] = (uint32_t)(seed & 0xffffffffUL);
    for (int i = 1; i < 624; i++) mt[i] = 1812433253u * (mt[i - 1] ^ (mt[i - 1] >> 30)) + (uint32_t)i;
    int idx = 624;
    for (int64_t k = 0; k < n; k++) {
        if (idx >= 624) {
            for (int i = 0; i < 624; i++) {
                const uint32_t y = (mt[i] & 0x80000000u) | (mt[(i + 1) % 624] & 0x7fffffffu);
                mt[i] = mt[(i + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
            }
            idx = 0;
        }
        uint32_t y = mt[idx++];
        y ^= y >> 11;
        y ^= (y << 7) & 0x9d2c5680u;
        y ^= (y << 15) & 0xefc60000u;
        y ^= y >> 18;
        out[k] = y / 4294967296.0;
    }
}

/* Shell counts around every centre with the reference's cell walk
 * (theory/vpf/countspheres_impl.c.src:332-415: cells c + d, |d| <= refine, wrapped with the
 * centre shifted by -/+ wrap when periodic, skipped otherwise) and the fallback kernel's binning
 * (theory/vpf/vpf_kernels.c.src:281-302): r2 = dx*dx + dy*dy + dz*dz, r2 < rmax^2,
 * bin = (int)(sqrt(r2) * inv_rstep) < nbin.  Cumulative counts then fill pN[bin * num_pN + N].
 * within != NULL: instead the number of points with r2 < rmax^2 per centre. */
int cfo_vpf(int64_t np, const double *x, const double *y, const double *z, const int *nmesh, const double *lat_min,
            const double *lat_inv, const int *refine, int periodic, const double *wrap, int64_t ncen,
            const double *cen, const int *cen_cell, double rmax, int nbin, int num_pN, uint64_t *pN,
            uint32_t *within)
{
    const int64_t ncells = (int64_t)nmesh[0] * nmesh[1] * nmesh[2];
    int64_t *start = calloc((size_t)ncells + 1, sizeof(int64_t));
    int64_t *cellof = malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
    int64_t *order = malloc(sizeof(int64_t) * (size_t)(np > 0 ? np : 1));
    for (int64_t i = 0; i < np; i++) {
        const double v[3] = {x[i], y[i], z[i]};
        int c[3];
        for (int a = 0; a < 3; a++) {
            int k = (int)((v[a] - lat_min[a]) * lat_inv[a]);
            if (k > nmesh[a] - 1) k--;
            if (k < 0 || k >= nmesh[a]) { free(start); free(cellof); free(order); return -1; }
            c[a] = k;
        }
        cellof[i] = ((int64_t)c[0] * nmesh[1] + c[1]) * nmesh[2] + c[2];
        start[cellof[i] + 1]++;
    }
    for (int64_t c = 0; c < ncells; c++) start[c + 1] += start[c];
    int64_t *fill = calloc((size_t)ncells, sizeof(int64_t));
    for (int64_t i = 0; i < np; i++) order[start[cellof[i]] + fill[cellof[i]]++] = i;
    free(fill);
    const double rstep = rmax / (double)nbin, inv_rstep = 1.0 / rstep, rmax_sqr = rmax * rmax;
    int *counts = malloc(sizeof(int) * (size_t)nbin);
    if (pN) memset(pN, 0, sizeof(uint64_t) * (size_t)nbin * num_pN);
    for (int64_t ic = 0; ic < ncen; ic++) {
        memset(counts, 0, sizeof(int) * (size_t)nbin);
        uint32_t nwithin = 0;
        const int ix = cen_cell[3 * ic], iy = cen_cell[3 * ic + 1], iz = cen_cell[3 * ic + 2];
        for (int dx = -refine[0]; dx <= refine[0]; dx++) {
            int cx = ix + dx;
            double ox = 0.0;
            if (periodic) {
                if (cx >= nmesh[0]) ox = -wrap[0]; else if (cx < 0) ox = wrap[0];
                cx = ((cx % nmesh[0]) + nmesh[0]) % nmesh[0];
            } else if (cx < 0 || cx >= nmesh[0]) continue;
            const double px = cen[3 * ic] + ox;
            for (int dy = -refine[1]; dy <= refine[1]; dy++) {
                int cy = iy + dy;
                double oy = 0.0;
                if (periodic) {
                    if (cy >= nmesh[1]) oy = -wrap[1]; else if (cy < 0) oy = wrap[1];
                    cy = ((cy % nmesh[1]) + nmesh[1]) % nmesh[1];
                } else if (cy < 0 || cy >= nmesh[1]) continue;
                const double py = cen[3 * ic + 1] + oy;
                for (int dz = -refine[2]; dz <= refine[2]; dz++) {
                    int cz = iz + dz;
                    double oz = 0.0;
                    if (periodic) {
                        if (cz >= nmesh[2]) oz = -wrap[2]; else if (cz < 0) oz = wrap[2];
                        cz = ((cz % nmesh[2]) + nmesh[2]) % nmesh[2];
                    } else if (cz < 0 || cz >= nmesh[2]) continue;
                    const double pz = cen[3 * ic + 2] + oz;
                    const int64_t cell = ((int64_t)cx * nmesh[1] + cy) * nmesh[2] + cz;
                    for (int64_t k = start[cell]; k < start[cell + 1]; k++) {
                        const int64_t j = order[k];
                        const double ddx = x[j] - px, ddy = y[j] - py, ddz = z[j] - pz;
                        volatile double t = ddx * ddx + ddy * ddy;
                        const double r2 = t + ddz * ddz;
                        if (r2 >= rmax_sqr) continue;
                        nwithin++;
                        const int ib = (int)(sqrt(r2) * inv_rstep);
                        if (ib < nbin) counts[ib]++;
                    }
                }
            }
        }
        if (within) {
            within[ic] = nwithin;
            continue;
        }
        for (int b = 1; b < nbin; b++) counts[b] += counts[b - 1];
        for (int b = 0; b < nbin; b++)
            if (counts[b] < num_pN) pN[(size_t)b * num_pN + counts[b]]++;
    }
    free(counts);
    free(start);
    free(cellof);
    free(order);
    return 0;
}
