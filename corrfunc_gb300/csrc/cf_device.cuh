// cf_device.cuh -- device-side data structures and per-pair arithmetic shared by the
// GB300 pair-counting kernels.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace cf {

// One unit of pair work: up to 32 consecutive points of one lattice column ("i-chunk")
// against one contiguous range of points of a neighbouring column ("j-range") with a fixed
// periodic image.  meta packs: bits 0-5 i_count-1, bits 8/10/12 (2 bits each) image+1 per
// axis, bit 14 'images' (packed: some range has a periodic image), bit 15 'packed', bit 16 'own'
// (auto-correlation, same column, same image: count only j > i).
//
// A packed task ("item") takes its j points from a list of ranges (JRange records, one per
// split j column and periodic image) that the chunk's whole neighbourhood concatenates:
// j_begin = first record, j_end bits 0-10 = points - 1, bits 11-31 = item number m; the item
// covers list positions [m kJMax, m kJMax + points).
struct Task {
    uint32_t i_begin;
    uint32_t j_begin;
    uint32_t j_end;
    uint32_t meta;
};
constexpr uint32_t kTaskImages = 1u << 14;
constexpr uint32_t kTaskPacked = 1u << 15;

// One range of a chunk's concatenated j list: x = first j point (lattice index), y = its list
// position, z = image code (bits 0-5, as Task::meta bits 8-13) | bit 31 on the chunk's last
// record, w = list position after the range.
typedef uint4 JRange;

__host__ __device__ inline uint32_t task_meta(int icount, int mx, int my, int mz, int own)
{
    return (uint32_t)(icount - 1) | ((uint32_t)(mx + 1) << 8) | ((uint32_t)(my + 1) << 10) |
           ((uint32_t)(mz + 1) << 12) | ((uint32_t)own << 16);
}

// Sorted point record kept per lattice (SoA of these arrays).
struct Lattice {
    float4 *hi;       // x_hi, y_hi, z_hi on the per-axis grid q (exact differences), w as float
    float4 *lo;       // x - x_hi, y - y_hi, z - z_hi (float), unused
    double4_32a *dbl;     // original coordinates (x, y, z, w) in double
    int2 *ro;         // reference-lattice cell (first-point rule), index in the caller's arrays
    uint32_t *cell_start; // ncells + 1 offsets
};

// MODE_RPPI_MOCK / MODE_SMU_MOCK: rp-pi and s-mu about the pair's line of sight (comoving
// positions of a survey, observer at the origin, no periodic images).
enum { MODE_R3 = 0, MODE_RPPI = 1, MODE_WP = 2, MODE_SMU = 3, MODE_THETA = 4, MODE_RPPI_MOCK = 5, MODE_SMU_MOCK = 6 };
constexpr int kNumModes = 7;

__host__ __device__ constexpr bool mode_is_mock(int m) { return m == MODE_RPPI_MOCK || m == MODE_SMU_MOCK; }
// flat 2-D histograms (separation bin * (npibin + 1) + pi or mu bin)
__host__ __device__ constexpr bool mode_two_d(int m)
{
    return m == MODE_RPPI || m == MODE_SMU || m == MODE_RPPI_MOCK || m == MODE_SMU_MOCK;
}

struct PairArgs {
    // lattices (set 1 = i points, set 2 = j points; identical for auto-correlations)
    const float4 *hi1, *lo1;
    const double4_32a *d1;
    const int2 *ro1;  // per point: reference-lattice cell, index in the caller's arrays
    const float4 *hi2, *lo2;
    const double4_32a *d2;
    const int2 *ro2;

    const Task *tasks;
    const JRange *jrec;         // range records of packed tasks
    uint32_t ntasks;            // task count, or the work-list capacity when ntask_dev is set
    const uint32_t *ntask_dev;  // device-resident task count (batched work lists), or null
    uint32_t *task_counter;

    unsigned long long *g_cnt;  // nbins
    double *g_avg;              // nbins
    double *g_w;                // nbins
    unsigned long long *g_stats; // [0] evaluated pairs, [1] refined pairs
    const double *g_edges;      // nedges (double, reference values)
    const float *g_guard;       // 2*nedges: lo guards then hi guards
    const uint32_t *g_lut;      // bin lookup on the float bits of the classified quantity (row byte offsets)
    uint32_t trash_off;         // byte offset of the trash row (rejected / deferred pairs)
    uint32_t row_bytes;         // bytes between consecutive histogram rows (4 * lane stride)
    int lane_stride_hint;       // layout the LUT offsets were built for
    int lut_n_hint;
    int lut_shift;              // bucket = (float_bits >> lut_shift) - lut_base
    int lut_base;
    int lut_n;                  // buckets; entry lut_n is the reject entry
    uint32_t lut_mul;           // 2^(32 - lut_shift): bucket = mad.hi(bits, lut_mul, -lut_base)
    float q_floor;              // added to q in the fast path so that q = 0 stays in the table
    uint32_t lut_negbase;
    // Byte table (DD(r), xi and DDtheta with at most 127 bins): the classified quantity is
    //   q' = min(r^2 + b, cap)
    // (r^2 the squared chord for DDtheta) with b a power of two below the smallest positive edge
    // and cap the start of the first bucket beyond the last guard, so that its float bits lie in
    // [bits(b), bits(cap)] and index the table with no lower clamp.  Entry = 2 * row + flag
    // (flag: the bucket holds a guard and its pairs take the exact path).
    int lut8;
    float q_bias, q_cap;        // b, cap
    float q_cap2;               // cap of lanes 16-31: the bucket after cap (entry: the second trash row)
    // box pruning (FLT_MAX: every point kept): a j point whose FP32 squared distance (DDrppi / wp:
    // in the xy plane) to the bounding box of a chunk's points exceeds this pairs with none of
    // them in range (the top edge's separation, or the survey modes' separation cut, plus four
    // coordinate error bounds, and 1e-5 relative, squared, rounded up)
    float prune_r2;
    // DDrppi / wp: a j point whose z distance to the box is at least this (the FP32 pi rejection
    // bound) pairs with none of the chunk's points within pimax
    float prune_z;
    uint32_t lut8_base;         // bits(b) >> lut_shift (bucket 0)
    uint32_t half_row;          // half the bytes of a histogram row (entry * half_row = row offset)
    uint32_t trash_e;           // entry of a rejected pair (2 * trash row)

    int nedges;
    int guard_search_top;       // largest power of two <= nedges - 1 (0 when nedges < 2)
    int nbins;
    int npibin;                 // rp-pi: pi bins, s-mu: mu bins
    int autocorr;
    int fma_formula;
    int chord_formula;

    // image offsets per axis for image index m+1 (m = -1, 0, +1)
    float ohi[3][3];
    float olo[3][3];
    double odbl[3][3];

    // rp-pi / wp / s-mu constants (reference values and FP32 classification bands)
    double pimax;
    double inv_dpi;
    double sqr_mu_max;
    double inv_dmu;
    float pimax_lo_f, pimax_hi_f;  // guard band around pimax for |dz|
    float inv_dpi_f;
    float pibin_band;              // half-width (in pi-bin units) of the ambiguity band
    float inv_dpi256_f;            // 256 / dpi (fast pi-bin rounding)
    int pi_band_q;                 // ambiguity half-width in 1/256 pi-bin units (fast path)
    float mu_band_abs;             // absolute mu error bound numerator (divided by s)
    float mu_max_f;
    float inv_dmu_f;
    float dz_err;                  // bound on |dz_f32 - dz_ref|
    float dxy_err;                 // bound on |(dx,dy)_f32 - (dx,dy)_ref|
    // survey (mock) modes
    float s2_cut_f;                // FP32 |s|^2 at or above this: certainly beyond the largest separation
    float l2_min_f;                // FP32 |l|^2 below this (pairs near the observer): exact path
    float mu_band_rel;             // part of the mu error bound independent of |s|
    int theta_series;              // angular averages: the arcsine series is exact for all counted chords

    // fixed-point scales for the per-warp accumulators
    const float *g_ascale;      // per separation bin: fixed-point scale of the separation sums
    int rbin_div;               // flat bin / rbin_div = separation bin (npibin + 1 for 2-D histograms)
    float w_scale_f;
    double w_unscale;
    // FP64 kernel only: weight sums accumulate in double precision (per-warp rows of doubles in
    // shared memory) instead of fixed point, for weights spanning a wide range
    int w_exact;
    // per-task timer (null: off): [2 t] elapsed SM clock cycles of task t, [2 t + 1] global warp
    unsigned long long *task_clock;
    // FP64 kernel only, for points outside the reference lattice (where the reference's cell-pair
    // list can leave out pairs in range across the periodic boundary): a pair counts only where the
    // reference lattice links the two cells (ref_n cells, ref_reach neighbours per axis)
    int ref_links;
    int ref_n[3], ref_reach[3];
};

// ---------------------------------------------------------------------------------------
// Reference (double-precision) evaluation of one pair, with the first point of the pair
// shifted by the periodic offset, exactly as the reference kernels do.  Every operation uses
// an explicitly rounded intrinsic so that no fused multiply-add is introduced unless the
// formula being reproduced has one.
// Returns the flat histogram bin, or -1 when the pair is not counted.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int bin_upper(const double *e, int n, double v)
{
    // number of edges <= v (edges sorted ascending)
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (e[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int bin_theta(const double *c, int n, double v)
{
    // reference rule: largest k in [1, n-1] with v <= c[k-1]; c is descending.
    // number of leading edges with c[k] >= v
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (c[mid] >= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <int MODE>
__device__ __forceinline__ int ref_eval(const PairArgs &A, const double *se,
                                        double xa, double ya, double za,
                                        double xb, double yb, double zb,
                                        double ox, double oy, double oz, double *avg_term)
{
    const int nb = A.nedges;
    if (MODE == MODE_THETA) {
        double c;
        if (A.chord_formula) {
            const double dx = __dsub_rn(xb, xa), dy = __dsub_rn(yb, ya), dz = __dsub_rn(zb, za);
            double ch2;
            if (A.fma_formula) ch2 = __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
            else ch2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
            c = __dsub_rn(1.0, __dmul_rn(0.5, ch2));
        } else {
            c = __dadd_rn(__dadd_rn(__dmul_rn(xb, xa), __dmul_rn(yb, ya)), __dmul_rn(zb, za));
        }
        if (c > se[0] || c <= se[nb - 1]) return -1;
        const int k = bin_theta(se, nb, c);  // >= 1 since c <= se[0]
        *avg_term = 57.29577951308232087679815481410517033240547246656432154916024 * acos(c);
        return k;
    }
    if (MODE == MODE_RPPI_MOCK || MODE == MODE_SMU_MOCK) {
        // s = x_second - x_first and the (unhalved) line of sight l = x_first + x_second.  Three
        // formula families: fallback, left-to-right sums
        // (mocks/DDrppi_mocks/countpairs_rp_pi_mocks_kernels.c.src:1232-1257,
        // mocks/DDsmu_mocks/countpairs_s_mu_mocks_kernels.c.src:1173-1190); AVX / SSE, sums nested
        // to the right (rp_pi :528-563, s_mu :505-546); AVX512F, fused chains (rp_pi :210-262,
        // s_mu :202-245).  The SIMD kernels drop pi >= pimax (mu >= mu_max) and truncate the flat
        // index from the double sum bin * (n + 1) + pi / dpi (rp_pi :312-319, s_mu :289-296); the
        // fallback files those pairs in column n and truncates pi / dpi alone.
        // Swapping the two points negates s and keeps l, so every quantity is symmetric.
        const double px = __dadd_rn(xa, xb), py = __dadd_rn(ya, yb), pz = __dadd_rn(za, zb);
        const double sx = __dsub_rn(xb, xa), sy = __dsub_rn(yb, ya), sz = __dsub_rn(zb, za);
        double s2, sl, l2;
        if (A.fma_formula) {
            s2 = __fma_rn(sx, sx, __fma_rn(sy, sy, __dmul_rn(sz, sz)));
            sl = __fma_rn(pz, sz, __dadd_rn(__dmul_rn(px, sx), __dmul_rn(py, sy)));
            l2 = __fma_rn(px, px, __fma_rn(py, py, __dmul_rn(pz, pz)));
        } else if (A.chord_formula) {
            s2 = __dadd_rn(__dmul_rn(sx, sx), __dadd_rn(__dmul_rn(sy, sy), __dmul_rn(sz, sz)));
            sl = __dadd_rn(__dmul_rn(pz, sz), __dadd_rn(__dmul_rn(py, sy), __dmul_rn(px, sx)));
            l2 = __dadd_rn(__dmul_rn(px, px), __dadd_rn(__dmul_rn(py, py), __dmul_rn(pz, pz)));
        } else {
            s2 = __dadd_rn(__dadd_rn(__dmul_rn(sx, sx), __dmul_rn(sy, sy)), __dmul_rn(sz, sz));
            sl = __dadd_rn(__dadd_rn(__dmul_rn(px, sx), __dmul_rn(py, sy)), __dmul_rn(pz, sz));
            l2 = __dadd_rn(__dadd_rn(__dmul_rn(px, px), __dmul_rn(py, py)), __dmul_rn(pz, pz));
        }
        const bool simd = A.fma_formula || A.chord_formula;
        const double sl2 = __dmul_rn(sl, sl);
        const int nrow = A.npibin + 1;
        double ratio, limit;  // pi^2 or mu^2 and its upper limit
        int kbin;
        if (MODE == MODE_RPPI_MOCK) {
            const double sqr_pimax = __dmul_rn(A.pimax, A.pimax);
            if (!(s2 < __dadd_rn(se[nb - 1], sqr_pimax))) return -1;
            if (!(sl2 < __dmul_rn(l2, sqr_pimax))) return -1;
            ratio = __ddiv_rn(sl2, l2);
            limit = sqr_pimax;
            const double dperp2 = __dsub_rn(s2, ratio);
            if (dperp2 >= se[nb - 1] || dperp2 < se[0]) return -1;
            kbin = bin_upper(se, nb, dperp2);
            *avg_term = __dsqrt_rn(dperp2);
        } else {
            if (s2 >= se[nb - 1] || s2 < se[0]) return -1;
            ratio = __ddiv_rn(sl2, __dmul_rn(l2, s2));
            if (ratio != ratio) return -1;  // l = 0: points mirrored through the observer
            limit = A.sqr_mu_max;
            kbin = bin_upper(se, nb, s2);
            *avg_term = __dsqrt_rn(s2);
        }
        const double t = __dmul_rn(__dsqrt_rn(ratio), MODE == MODE_RPPI_MOCK ? A.inv_dpi : A.inv_dmu);
        if (simd) {
            if (!(ratio < limit)) return -1;
            return min(__double2int_rz(__dadd_rn((double)(kbin * nrow), t)), kbin * nrow + A.npibin);
        }
        return kbin * nrow + (ratio >= limit ? A.npibin : min(__double2int_rz(t), A.npibin));
    }
    const double xpos = __dadd_rn(xa, ox), ypos = __dadd_rn(ya, oy), zpos = __dadd_rn(za, oz);
    const double dx = __dsub_rn(xb, xpos), dy = __dsub_rn(yb, ypos), dz = __dsub_rn(zb, zpos);
    if (MODE == MODE_R3) {
        double r2;
        if (A.fma_formula) r2 = __fma_rn(dz, dz, __fma_rn(dy, dy, __dmul_rn(dx, dx)));
        else r2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
        if (r2 >= se[nb - 1] || r2 < se[0]) return -1;
        *avg_term = __dsqrt_rn(r2);
        return bin_upper(se, nb, r2);
    }
    if (MODE == MODE_RPPI || MODE == MODE_WP) {
        if (dz <= -A.pimax || dz >= A.pimax) return -1;
        double r2;
        if (A.fma_formula) r2 = __fma_rn(dy, dy, __dmul_rn(dx, dx));
        else r2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
        if (r2 >= se[nb - 1] || r2 < se[0]) return -1;
        const int kbin = bin_upper(se, nb, r2);
        *avg_term = __dsqrt_rn(r2);
        if (MODE == MODE_WP) return kbin;
        int pibin = (int)__dmul_rn(fabs(dz), A.inv_dpi);
        pibin = pibin > A.npibin ? A.npibin : pibin;
        return kbin * (A.npibin + 1) + pibin;
    }
    // MODE_SMU
    {
        const double sqr_dz = __dmul_rn(dz, dz);
        double s2;
        if (A.fma_formula) s2 = __fma_rn(dx, dx, __fma_rn(dy, dy, sqr_dz));
        else s2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), sqr_dz);
        if (s2 >= se[nb - 1] || s2 < se[0]) return -1;
        if (sqr_dz >= __dmul_rn(s2, A.sqr_mu_max)) return -1;
        const double mu = __dsqrt_rn(__ddiv_rn(sqr_dz, s2));
        int mubin = (int)__dmul_rn(mu, A.inv_dmu);
        mubin = mubin > A.npibin ? A.npibin : mubin;
        const int kbin = bin_upper(se, nb, s2);
        *avg_term = __dsqrt_rn(s2);
        return kbin * (A.npibin + 1) + mubin;
    }
}

}  // namespace cf
