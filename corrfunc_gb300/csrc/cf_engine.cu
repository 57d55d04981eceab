// cf_engine.cu -- GB300 (sm_103a) pair-counting engine.
//
// Replaces the reference's three hot stages:
//   * gridlink (utils/gridlink_impl.c.src:65-436): a device counting sort of the points into
//     a lattice of (x,y) columns x fine z slabs, in integer and FP32 arithmetic on fixed-point
//     coordinates, written as SoA records (FP32 hi/lo grid coordinates, FP64 copies,
//     reference-lattice cell and caller index);
//   * generate_cell_pairs (utils/gridlink_impl.c.src:439-625): a device-built worklist of
//     (32-point column chunk, neighbouring column z-window) tasks with periodic images, the
//     auto-correlation half stencil and a min-separation prune;
//   * the per-cell-pair kernels (theory/*/..._kernels.c.src, countpairs_theta_mocks_kernels):
//     persistent warps that classify each pair in FP32 against proven error bands around
//     every bin edge and re-evaluate only the ambiguous pairs with the reference's FP64
//     formula (or, in FP64 mode, evaluate every pair with that formula).
//
// Entry point: cf_engine_run() (C ABI, called by the C host layer).
#include <cuda_runtime.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <signal.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "cf_device.cuh"
#include "cf_internal.h"

using namespace cf;

#define CF_CUDA(call)                                                                           \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            fprintf(stderr, "corrfunc_gb300: CUDA error '%s' at %s:%d (%s)\n", cudaGetErrorString(e_), \
                    __FILE__, __LINE__, #call);                                                 \
            return EXIT_FAILURE;                                                                \
        }                                                                                       \
    } while (0)

#define CF_FAIL(...)                                                                            \
    do {                                                                                        \
        fprintf(stderr, "corrfunc_gb300: " __VA_ARGS__);                                        \
        fprintf(stderr, "\n");                                                                  \
        return EXIT_FAILURE;                                                                    \
    } while (0)

namespace {

constexpr int kChunk = 32;          // points per i-chunk (one per lane)
constexpr int kCatShift = 17;       // Task::meta bits 17-31: catalogue of a batched count
// partial j tiles above this size run padded to 32 (fully unrolled); smaller ones pair by pair
// (measured on this GPU with box pruning: 24 is 1.2 % faster than 16 and 4 % faster than 8 on
// DD(r), 1-3 % faster than 16 on the 2-D counters; 20 and 28 within 0.3 % of 24)
#ifndef CF_PAD_MIN
#define CF_PAD_MIN 24
#endif
constexpr int kPadMin = CF_PAD_MIN;
constexpr uint32_t kJMax = 2048;    // max j points per task
constexpr int kRxy = 2;             // lattice columns per rmax_xy
// z slabs per rmax_z: finer slabs trim the z windows of the work list (64 evaluates 0.9-1.2 %
// fewer pairs than 32 on DD(r) at a few hundred kB of cell offsets)
#ifndef CF_Z_SLABS
#define CF_Z_SLABS 64
#endif
constexpr int kZFine = CF_Z_SLABS;
// the FP32 pair kernel's largest block and the resident blocks of that size per SM it is compiled
// for: 2 x 512 threads caps it at 64 registers (32 resident warps per SM)
#ifndef CF_PAIR_MAX_THREADS
#define CF_PAIR_MAX_THREADS 512
#endif
#ifndef CF_PAIR_MIN_BLOCKS
#define CF_PAIR_MIN_BLOCKS 2
#endif
// DD(r) / xi / DDtheta with weights or separation averages (not both): 2 x 384 threads (up to 85
// registers, 24 warps per SM) -- measured 4 % faster on the weighted 2M x 2M cross-correlation, 8 %
// on the 300k auto-correlation with averages and 5 % on the 1M-point DDtheta with thetaavg than
// 2 x 512, which spills at 64 registers; plain counts (4 % faster) and counts with both sums (6 %)
// keep 2 x 512
#ifndef CF_PAIR_SPLIT_THETA
#define CF_PAIR_SPLIT_THETA 1  // 0: DDtheta keeps 2 x 512 throughout
#endif
constexpr int pair_max_threads(int mode, bool avg, bool w)
{
    return ((mode == MODE_R3 || (CF_PAIR_SPLIT_THETA && mode == MODE_THETA)) && avg != w && CF_PAIR_MAX_THREADS > 384)
               ? 384
               : CF_PAIR_MAX_THREADS;
}
// pairs whose table offsets are computed before their shared reductions are issued (byte-table
// DD(r) / xi / DDtheta without averages; measured on this GPU with box pruning: 16 pairs in one
// group per loop body 1.0-1.2 % faster than 8 x 2 and 32 x 1 3-10 % slower, with fewer spills)
#ifndef CF_PAIR_GROUP
#define CF_PAIR_GROUP 16
#endif
// survey modes: pairs per group and groups per unrolled loop body
#ifndef CF_MOCK_GROUP
#define CF_MOCK_GROUP 1
#endif
#ifndef CF_MOCK_UNROLL
#define CF_MOCK_UNROLL 8
#endif
constexpr int kMockUnroll = CF_MOCK_UNROLL;
// Tile loops are unrolled only partly: the full 32-pair unroll overflows the instruction cache
// once a pair's body grows (measured on this GPU: rp-pi, wp, s-mu and angular averages 1.4-2.2x,
// weighted DD(r) 13 %, DD(r) with averages 1.8x faster than the full unroll).  Angular counts
// without averages keep the full unroll.
#ifndef CF_2D_GROUP
#define CF_2D_GROUP 4
#endif
#ifndef CF_2D_UNROLL
#define CF_2D_UNROLL 2
#endif
#ifndef CF_R3_UNROLL
#define CF_R3_UNROLL 1
#endif
constexpr int kR3Unroll = CF_R3_UNROLL;

constexpr int kScanTile = 4096;
constexpr uint32_t kLutMax = 8192;  // largest bucket table (32 KB of shared memory)

// modes with an FP32 classification kernel (the others always run the FP64 kernel)
constexpr bool has_f32_path(int mode) { return mode >= 0 && mode < kNumModes; }
template <int MODE>
constexpr bool kHasF32 = has_f32_path(MODE);

// ------------------------------------------------------------------------------------
// geometry of the GPU lattice and of the reference lattice
// ------------------------------------------------------------------------------------
struct Geom {
    double origin[3];
    double hi_origin[3];  // origin of the hi / lo split (the lattice origin, or 0 for survey positions)
    double inv_s[3];
    double s[3];
    int n[3];  // n[0] x columns, n[1] y columns, n[2] z slabs
    double q[3];
    double inv_q[3];
    double ref_min[3];
    double ref_inv[3];
    int ref_n[3];
    int check_ref_bounds;
    // replays of a planned batch: points must stay inside the planned box and weights within the
    // planned maximum (the lattice and the error bounds were sized for them); violations are
    // counted in *extent_err (null: no check)
    unsigned long long *extent_err;
    double chk_lo[3], chk_hi[3];
    double chk_wmax, chk_wmin;  // planned largest |w| and smallest non-zero |w| (0: no lower check)
    // Integer view of the coordinates (the lattice kernels keep FP64 arithmetic off their common
    // path -- on this GPU the FP64 pipe issues at 1/64 of the FP32 rate -- and use it only for
    // the rare points near a reference-cell boundary).  A coordinate x becomes the fixed-point
    // integer X = round(x / 2^e_fix) modulo 2^64 (e_fix = log2(q) - 31); the differences
    // X - o_hi and X - o_cell are exact and give the hi / lo split and the cell index.
    int e_fix[3];
    unsigned long long o_hi[3], o_cell[3];  // X of hi_origin and of origin
    float q_f[3], rho_f[3];                 // q, 2^e_fix
    // fixed-point index t = umulhi(X - o_cell, cell_mul) >> cell_shift: (x - origin) / (s / cdiv)
    // in 64-bit fixed point, within eps_cell (position units) of the exact value, clamped below
    // tmax; the cell index is t / cdiv.  With two lattices of split columns in one call (the j
    // lattice's columns split every i-lattice column cdiv x cdiv, its z slabs merge cdiv i-lattice
    // slabs) both take t from the same product, so that a j-lattice cell lies inside exactly
    // one i-lattice column and slab range.  cdiv = 1, tmax = n otherwise.
    unsigned long long cell_mul[3];
    int cell_shift[3];
    double eps_cell[3];
    int cdiv[3], tmax[3];
    // order keys (okey0) of the extent checks, and of the range of coordinates that are inside
    // the reference lattice whatever the rounding of its FP64 cell index (others take the exact test)
    unsigned long long k_chk_lo[3], k_chk_hi[3], k_chk_wmax, k_chk_wmin;
    unsigned long long k_ref_lo[3], k_ref_hi[3];
    // fixed-point X of ref_min (FP32 estimate of the reference cell index)
    unsigned long long o_ref[3];
    float ref_inv_f[3], ref_tol_f[3];  // 1 / reference cell, absolute error term of the estimate
    // lo parts of the lattice records are written only for separation averages and survey modes
    int write_lo;
};

// round(x / 2^e) modulo 2^64 of a finite double / float from its bits (ties away from zero)
__host__ __device__ inline unsigned long long fix_round(unsigned long long m, int t, bool neg)
{
    unsigned long long v;
    if (t >= 0) v = t >= 64 ? 0ull : m << t;
    else v = -t >= 64 ? 0ull : ((m >> (-t - 1)) + 1ull) >> 1;
    return neg ? 0ull - v : v;
}
__host__ __device__ inline unsigned long long fix_of(double x, int e)
{
    unsigned long long b;
#ifdef __CUDA_ARCH__
    b = (unsigned long long)__double_as_longlong(x);
#else
    memcpy(&b, &x, sizeof(b));
#endif
    int E = (int)((b >> 52) & 0x7ffu);
    unsigned long long m = b & 0xfffffffffffffull;
    if (E) m |= 1ull << 52;
    else E = 1;
    return fix_round(m, E - 1075 - e, (b >> 63) != 0);
}
__host__ __device__ inline unsigned long long fix_of(float x, int e)
{
    uint32_t b;
#ifdef __CUDA_ARCH__
    b = __float_as_uint(x);
#else
    memcpy(&b, &x, sizeof(b));
#endif
    int E = (int)((b >> 23) & 0xffu);
    unsigned long long m = b & 0x7fffffu;
    if (E) m |= 1ull << 23;
    else E = 1;
    return fix_round(m, E - 150 - e, (b >> 31) != 0);
}

// U = (x - origin) / 2^e_fix as N * 2^31 + L (N the nearest integer to U / 2^31, |L| <= 2^30):
// hi = N q exactly (|N| < 2^24), lo = L 2^e_fix rounded once
__device__ __forceinline__ void fix_split(unsigned long long U, float q, float rho, float *hi, float *lo)
{
    const long long N = ((long long)U + (1ll << 30)) >> 31;
    const int L = (int)(long long)(U - ((unsigned long long)N << 31));
    *hi = (float)(int)N * q;
    *lo = (float)L * rho;
}

// order key of a double with -0 mapped to +0 (so that key order is the IEEE comparison order)
__host__ __device__ inline unsigned long long okey0(double v)
{
    unsigned long long u;
#ifdef __CUDA_ARCH__
    u = (unsigned long long)__double_as_longlong(v);
#else
    memcpy(&u, &v, sizeof(u));
#endif
    if ((u << 1) == 0) u = 0;
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

__device__ __forceinline__ unsigned long long ord_enc(double v)
{
    unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}

__host__ inline double ord_dec(unsigned long long u)
{
    u = (u & 0x8000000000000000ull) ? (u & 0x7fffffffffffffffull) : ~u;
    double d;
    memcpy(&d, &u, sizeof(d));
    return d;
}

template <typename T>
__device__ __forceinline__ double ld(const T *p, int64_t i) { return (double)p[i]; }

// Data extent.  Values are compared as order-preserving unsigned keys (integer min/max on the
// ALU pipe; double min/max would run on the slow FP64 pipe); every block folds its extremes
// (xmin, xmax, ymin, ymax, zmin, zmax, max |w|, non-finite flag) into mm[0..7] (ord_enc of the
// double values) with one atomic per slot.
__device__ __forceinline__ uint32_t okey(float v)
{
    const uint32_t u = __float_as_uint(v);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ unsigned long long okey(double v)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(v);
    return (u & 0x8000000000000000ull) ? ~u : (u | 0x8000000000000000ull);
}
__device__ __forceinline__ bool nonfinite(float v) { return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u; }
__device__ __forceinline__ bool nonfinite(double v)
{
    return (((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ffu) == 0x7ffu;
}
__device__ __forceinline__ uint32_t abskey(float v) { return __float_as_uint(v) & 0x7fffffffu; }
__device__ __forceinline__ unsigned long long abskey(double v)
{
    return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
}
__device__ __forceinline__ double key_value(uint32_t k)
{
    return (double)__uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ double key_value(unsigned long long k)
{
    return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k));
}
__device__ __forceinline__ uint32_t warp_min(uint32_t v) { return __reduce_min_sync(0xffffffffu, v); }
__device__ __forceinline__ uint32_t warp_max(uint32_t v) { return __reduce_max_sync(0xffffffffu, v); }
__device__ __forceinline__ unsigned long long warp_min(unsigned long long v)
{
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t < v ? t : v;
    }
    return v;
}
__device__ __forceinline__ unsigned long long warp_max(unsigned long long v)
{
    for (int o = 16; o; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, v, o);
        v = t > v ? t : v;
    }
    return v;
}

constexpr int kMinmaxUnroll = 4;
// extent slots of one catalogue: xmin, xmax, ymin, ymax, zmin, zmax, max |w|, non-finite flag,
// smallest non-zero |w|; catalogue s folds into mm[kMmSlots * s ...]
constexpr int kMmUsed = 9;
constexpr int kMmSlots = 16;
// initial value of extent slot k (minima start at the largest key, maxima and flags at 0)
__host__ inline unsigned long long mm_init_value(int k)
{
    k %= kMmSlots;
    return (k == 0 || k == 2 || k == 4 || k == 8) ? ~0ull : 0ull;
}
// smallest non-zero |w| of a catalogue's extent slots (0 when it has no non-zero weight)
__host__ inline double mm_wmin(const unsigned long long *mmh) { return mmh[8] == ~0ull ? 0.0 : ord_dec(mmh[8]); }

// Weight sums are 32-bit fixed-point terms at one scale per call (the largest |w1 w2| maps to
// just below 2^30), so a term's rounding error is at most 2^-30 of the largest product; terms
// much smaller than it could all round the same way.  When the largest product exceeds the
// smallest non-zero one by more than kWeightSpanFixed (then every term is still resolved to
// 2^-30 * 512 < 5e-7 of itself), the count runs the FP64 pair kernel with the weight sums in
// double precision instead.
constexpr double kWeightSpanFixed = 512.0;
__host__ inline bool weights_wide(const double wmax[2], const double wmin[2])
{
    if (!(wmin[0] > 0.0) || !(wmin[1] > 0.0)) return false;  // no non-zero products
    return wmax[0] * wmax[1] > kWeightSpanFixed * (wmin[0] * wmin[1]);
}

template <typename T>
__global__ void __launch_bounds__(256) k_minmax(const T *x, const T *y, const T *z, const T *w, int64_t n,
                                                unsigned long long *mm)
{
    using K = decltype(okey(T(0)));
    K mn[3] = {(K)~(K)0, (K)~(K)0, (K)~(K)0}, mx[3] = {0, 0, 0}, wm = 0, wn = (K)~(K)0;
    uint32_t bad = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    // kMinmaxUnroll points per iteration: all their loads are issued before the compares
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += kMinmaxUnroll * stride) {
        T c[3 * kMinmaxUnroll];
#pragma unroll
        for (int u = 0; u < kMinmaxUnroll; u++) {
            const int64_t iu = i + u * stride < n ? i + u * stride : i;  // repeats of point i are harmless
            c[3 * u] = x[iu];
            c[3 * u + 1] = y[iu];
            c[3 * u + 2] = z[iu];
        }
#pragma unroll
        for (int k = 0; k < 3 * kMinmaxUnroll; k++) {
            const int a = k % 3;
            bad |= nonfinite(c[k]) ? 1u : 0u;
            const K key = okey(c[k]);
            mn[a] = key < mn[a] ? key : mn[a];
            mx[a] = key > mx[a] ? key : mx[a];
        }
        if (w) {
#pragma unroll
            for (int u = 0; u < kMinmaxUnroll; u++) {
                const int64_t iu = i + u * stride < n ? i + u * stride : i;
                const K kw = abskey(w[iu]);
                wm = kw > wm ? kw : wm;
                wn = (kw != 0 && kw < wn) ? kw : wn;  // smallest non-zero |w|
            }
        }
    }
    __shared__ unsigned long long part[8][kMmUsed];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    K r[7];
    for (int a = 0; a < 3; a++) {
        r[2 * a] = warp_min(mn[a]);
        r[2 * a + 1] = warp_max(mx[a]);
    }
    r[6] = warp_max(wm);
    wn = warp_min(wn);
    bad = __any_sync(0xffffffffu, bad != 0) ? 1u : 0u;
    if (lane == 0) {
        for (int k = 0; k < 7; k++) part[warp][k] = (unsigned long long)r[k];
        part[warp][7] = bad;
        part[warp][8] = (unsigned long long)wn;
    }
    __syncthreads();
    // the block's extremes go straight into mm (ord_enc of the double values; one atomic each)
    if (threadIdx.x < kMmUsed) {
        const int k = threadIdx.x;
        const bool is_min = (k < 6 && (k & 1) == 0) || k == 8;
        K v = (K)part[0][k];
        for (int q = 1; q < nwarps; q++) {
            const K o = (K)part[q][k];
            v = is_min ? (o < v ? o : v) : (o > v ? o : v);
        }
        if (k == 7) {
            if (v) atomicMax(&mm[7], 1ull);
        } else if (k == 6 || k == 8) {
            if (k == 8 && v == (K)~(K)0) return;  // no non-zero weight in this block
            const double wv = key_value((K)(v | ((K)1 << (sizeof(K) * 8 - 1))));  // non-negative value
            if (k == 6) atomicMax(&mm[6], ord_enc(wv));
            else atomicMin(&mm[8], ord_enc(wv));
        } else {
            const unsigned long long e = ord_enc(key_value(v));
            if (is_min) atomicMin(&mm[k], e);
            else atomicMax(&mm[k], e);
        }
    }
}

// Cell index along axis a from the fixed-point coordinate X: (x - origin) / s by a 64-bit
// reciprocal multiply, within eps_cell (position units) of the exact value; the neighbour search
// margins cover it.  Points below the origin (none in a valid call) go to cell 0.
__device__ __forceinline__ int axis_cell(unsigned long long X, const Geom &g, int a)
{
    const unsigned long long U = X - g.o_cell[a];
    if ((long long)U < 0) return 0;
    const unsigned long long t = __umul64hi(U, g.cell_mul[a]) >> g.cell_shift[a];
    const int div = g.cdiv[a] > 1 ? g.cdiv[a] : 1;
    const unsigned long long nt = g.tmax[a] > 0 ? (unsigned long long)g.tmax[a] : (unsigned long long)g.n[a];
    const int tf = t >= nt ? (int)nt - 1 : (int)t;
    return div > 1 ? tf / div : tf;
}

// cell index of a point in the reference lattice, in the reference's FP64 arithmetic
// (utils/gridlink_impl.c.src:165-183)
__device__ __forceinline__ void ref_axis_cells(const double *ref_min, const double *ref_inv, const int *ref_n, double a,
                                               double b, double c, int *r)
{
    r[0] = (int)((a - ref_min[0]) * ref_inv[0]);
    r[1] = (int)((b - ref_min[1]) * ref_inv[1]);
    r[2] = (int)((c - ref_min[2]) * ref_inv[2]);
    for (int k = 0; k < 3; k++)
        if (r[k] > ref_n[k] - 1) r[k]--;
}

template <typename T>
__global__ void k_assign(const T *x, const T *y, const T *z, int64_t n, Geom g,
                         uint32_t *cellid, uint32_t *rank, uint32_t *count, unsigned long long *oob)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T c[3] = {x[i], y[i], z[i]};
        int ic[3];
#pragma unroll
        for (int a = 0; a < 3; a++) ic[a] = axis_cell(fix_of(c[a], g.e_fix[a]), g, a);
        const uint32_t cell = ((uint32_t)ic[0] * g.n[1] + ic[1]) * (uint32_t)g.n[2] + ic[2];
        if (g.extent_err) {
            bool in = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const unsigned long long k = okey0((double)c[a]);
                in = in && k >= g.k_chk_lo[a] && k <= g.k_chk_hi[a];
            }
            if (!in) atomicAdd(g.extent_err, 1ull);
        }
        cellid[i] = cell;
        rank[i] = atomicAdd(&count[cell], 1u);  // the point's slot within its cell
        if (g.check_ref_bounds) {
            // out-of-bounds test of the reference lattice (utils/gridlink_impl.c.src:165-183):
            // points well inside its range pass on their keys, the others take the FP64 test
            bool safe = true;
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const unsigned long long k = okey0((double)c[a]);
                safe = safe && k >= g.k_ref_lo[a] && k <= g.k_ref_hi[a];
            }
            if (!safe) {
                int r[3];
                ref_axis_cells(g.ref_min, g.ref_inv, g.ref_n, (double)c[0], (double)c[1], (double)c[2], r);
                if (r[0] < 0 || r[0] >= g.ref_n[0] || r[1] < 0 || r[1] >= g.ref_n[1] || r[2] < 0 || r[2] >= g.ref_n[2])
                    atomicAdd(oob, 1ull);
            }
        }
    }
}

// Reference-lattice cell index along axis a, equal to the reference's FP64
// (int)((x - ref_min) * ref_inv) with its clamp of the top cell: an FP32 estimate t from the
// fixed-point coordinate (|t - t_FP64| below 2^-22 |t| + 4 ref_inv 2^e_fix) decides when that
// band is non-negative and holds no integer; otherwise the FP64 expression runs.
template <typename T>
__device__ __forceinline__ int ref_axis_cell(T x, unsigned long long X, const Geom &g, int a)
{
    const unsigned long long U = X - g.o_ref[a];
    const long long N = ((long long)U + (1ll << 30)) >> 31;
    int r = -1;
    bool exact = true;
    if (N > -(1ll << 23) && N < (1ll << 23)) {
        const int L = (int)(long long)(U - ((unsigned long long)N << 31));
        const float t = ((float)(int)N * g.q_f[a] + (float)L * g.rho_f[a]) * g.ref_inv_f[a];
        const float e = fabsf(t) * 6e-7f + g.ref_tol_f[a];
        const float lo = t - e, hi = t + e;
        if (lo >= 0.f && hi < 1073741824.f && floorf(lo) == floorf(hi)) {
            r = (int)lo;
            exact = false;
        }
    }
    if (exact) r = (int)(((double)x - g.ref_min[a]) * g.ref_inv[a]);
    if (r > g.ref_n[a] - 1) r--;
    return r;
}

// key order of |w| (the sign bit cleared; integer operations only)
__device__ __forceinline__ unsigned long long abs_okey(double v)
{
    return ((unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull) | 0x8000000000000000ull;
}
__device__ __forceinline__ unsigned long long abs_okey(float v) { return abs_okey((double)v); }

// Lattice records of every point at its slot of the counting sort.  L.lo (separation averages,
// survey modes) is written only when set.
template <typename T>
__global__ void k_scatter(const T *x, const T *y, const T *z, const T *w, int64_t n, Geom g,
                          const uint32_t *cellid, const uint32_t *rank, const uint32_t *cell_start, Lattice L,
                          int ro_cat)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cellid[i];
        const uint32_t pos = cell_start[c] + rank[i];
        const T p[3] = {x[i], y[i], z[i]};
        const T wv = w ? w[i] : T(1);
        if (g.extent_err && w) {
            // a replayed batch keeps its weights inside the planned range (the scale of the weight
            // sums was chosen for it); zero weights are always inside
            const unsigned long long kw = abs_okey(wv);
            if (!(kw <= g.k_chk_wmax) || (kw > 0x8000000000000000ull && kw < g.k_chk_wmin)) atomicAdd(g.extent_err, 1ull);
        }
        float h[3], l[3];
        unsigned long long X[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            X[a] = fix_of(p[a], g.e_fix[a]);
            fix_split(X[a] - g.o_hi[a], g.q_f[a], g.rho_f[a], &h[a], &l[a]);
        }
        L.hi[pos] = make_float4(h[0], h[1], h[2], (float)wv);
        if (L.lo) L.lo[pos] = make_float4(l[0], l[1], l[2], 0.f);
        L.dbl[pos] = make_double4_32a((double)p[0], (double)p[1], (double)p[2], (double)wv);
        if (ro_cat >= 0) {
            L.ro[pos] = make_int2(ro_cat, (int)i);  // merged batch lattice: the catalogue instead
        } else {
            int r[3];
#pragma unroll
            for (int a = 0; a < 3; a++) r[a] = ref_axis_cell(p[a], X[a], g, a);
            L.ro[pos] = make_int2((r[0] * g.ref_n[1] + r[1]) * g.ref_n[2] + r[2], (int)i);
        }
    }
}

// ------------------------------------------------------------------------------------
// exclusive scan of uint32 (out has n+1 entries; out[n] = total)
// ------------------------------------------------------------------------------------
__global__ void k_scan_tile(const uint32_t *in, uint32_t *out, uint32_t n, uint32_t *blocksums)
{
    __shared__ uint32_t wsum[32];
    const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
    const int t = threadIdx.x;  // 1024 threads, 4 items each
    uint32_t v[4];
    uint32_t s = 0;
    for (int k = 0; k < 4; k++) {
        const uint32_t idx = base + t * 4 + k;
        v[k] = idx < n ? in[idx] : 0u;
        s += v[k];
    }
    // inclusive warp scan of per-thread sums
    uint32_t inc = s;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xffffffffu, inc, off);
        if ((t & 31) >= off) inc += o;
    }
    if ((t & 31) == 31) wsum[t >> 5] = inc;
    __syncthreads();
    if (t < 32) {
        uint32_t ws = wsum[t];
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, ws, off);
            if (t >= off) ws += o;
        }
        wsum[t] = ws;  // inclusive
    }
    __syncthreads();
    uint32_t run = inc - s + ((t >> 5) ? wsum[(t >> 5) - 1] : 0u);
    for (int k = 0; k < 4; k++) {
        const uint32_t idx = base + t * 4 + k;
        if (idx < n) out[idx] = run;
        run += v[k];
    }
    if (t == 1023) {
        blocksums[blockIdx.x] = run;
        if (gridDim.x == 1) out[n] = run;  // a single tile is the whole scan: write the total
    }
}

// adds the scanned tile sums (nblk + 1 entries, the last the total) and writes out[n] = total
__global__ void k_scan_add(uint32_t *out, uint32_t n, const uint32_t *offs)
{
    const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
    const uint32_t add = offs[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
        const uint32_t idx = base + k;
        if (idx < n) out[idx] += add;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) out[n] = offs[gridDim.x];
}

// ------------------------------------------------------------------------------------
// chunks (up to 32 consecutive points of one column) and tasks
// ------------------------------------------------------------------------------------
// z slab of sorted point p of a column whose slab offsets are cs[0..nz] (the last slab whose
// offset is <= p; empty slabs before it share its offset)
__device__ __forceinline__ uint32_t slab_of(const uint32_t *cs, int nz, uint32_t p)
{
    int lo = 0, hi = nz;  // cs[lo] <= p < cs[hi]
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (cs[mid] <= p) lo = mid;
        else hi = mid;
    }
    return (uint32_t)lo;
}

// The chunks of one column, walked by one warp: the column's points split into runs at every gap
// of at least `gap` empty z slabs (a chunk spanning such a gap would pull in the j points of the
// whole gap; split, its two parts' windows leave most of it out), and each run into chunks of 32
// consecutive points.  Returns the column's chunk count; with EMIT the chunks are written from
// slot o0 (slots at or beyond cap are not written and set bit 2 of *err): chunk_begin = absolute
// first point (point_base + index), chunk_info = size (bits 0-5), first and last z slab (bits
// 6-17, 18-29) and column, chunk_cat = catalogue (batched counts).  gap < 0: no splits.
template <bool EMIT>
__device__ uint32_t column_chunks(const uint32_t *cs, int nz, int gap, int col, int lane, uint32_t o0, uint32_t cap,
                                  uint32_t *err, uint32_t *chunk_begin, uint2 *chunk_info, uint32_t point_base,
                                  uint16_t *chunk_cat, uint16_t cat)
{
    uint32_t count = 0;
    auto close_run = [&](uint32_t p0, uint32_t p1) {
        const uint32_t n = (p1 - p0 + kChunk - 1) / kChunk;
        if (EMIT) {
            for (uint32_t k = lane; k < n; k += 32) {
                const uint32_t p = p0 + k * kChunk, o = o0 + count + k;
                if (o >= cap) {
                    if (err) atomicOr(err, 2u);
                    continue;
                }
                const uint32_t cnt = min((uint32_t)kChunk, p1 - p);
                chunk_begin[o] = point_base + p;
                chunk_info[o] =
                    make_uint2(cnt | (slab_of(cs, nz, p) << 6) | (slab_of(cs, nz, p + cnt - 1) << 18), (uint32_t)col);
                if (chunk_cat) chunk_cat[o] = cat;
            }
        }
        count += n;
    };
    const uint32_t a = cs[0], b = cs[nz];
    if (b == a) return 0;
    if (gap < 0) {
        close_run(a, b);
        return count;
    }
    int prev = -1;        // last non-empty slab before the current batch of 32 slabs
    uint32_t run_p0 = a;  // first point of the open run
    bool open = false;
    for (int z0 = 0; z0 < nz; z0 += 32) {
        const int z = z0 + lane;
        const bool ne = z < nz && cs[z + 1] > cs[z];
        // last non-empty slab before z: exclusive max-scan over the batch, with the carry
        int incl = ne ? z : -1;
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl = max(incl, t);
        }
        int before = __shfl_up_sync(0xffffffffu, incl, 1);
        if (lane == 0) before = -1;
        before = max(before, prev);
        uint32_t starts = __ballot_sync(0xffffffffu, ne && (before < 0 || z - before > gap));
        while (starts) {
            const int bl = __ffs(starts) - 1;
            starts &= starts - 1;
            const uint32_t ps = cs[z0 + bl];
            if (open) close_run(run_p0, ps);
            run_p0 = ps;
            open = true;
        }
        prev = max(prev, __shfl_sync(0xffffffffu, incl, 31));
    }
    if (open) close_run(run_p0, b);
    return count;
}

// chunk count of every column (one warp per column)
__global__ void k_col_chunks(const uint32_t *cell_start, int ncols, int nz, int gap, uint32_t *chunks_per_col)
{
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (c >= ncols) return;  // warp-uniform
    const uint32_t n = column_chunks<false>(cell_start + (uint32_t)c * nz, nz, gap, c, lane, 0u, 0u, nullptr, nullptr,
                                            nullptr, 0u, nullptr, 0);
    if (lane == 0) chunks_per_col[c] = n;
}

// the chunks of every column at its offset chunk_off[c] (one warp per column; cap: chunk slots)
__global__ void k_chunk_emit(const uint32_t *cell_start, int ncols, int nz, int gap, const uint32_t *chunk_off,
                             uint32_t cap, uint32_t *err, uint32_t *chunk_begin, uint2 *chunk_info,
                             uint32_t point_base, uint16_t *chunk_cat, uint16_t cat)
{
    const int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (c >= ncols) return;  // warp-uniform
    column_chunks<true>(cell_start + (uint32_t)c * nz, nz, gap, c, lane, chunk_off[c], cap, err, chunk_begin,
                        chunk_info, point_base, chunk_cat, cat);
}

// Chunk slots reserved for n1 points in ncols columns of nz slabs: a run of n points makes at
// most n/32 + 1 chunks, and a column holds at most nz / (gap + 1) + 1 runs (k runs separated by
// at least gap empty slabs take k + (k - 1) gap slabs), and no more runs than points.
static inline uint64_t chunk_slots(uint64_t n1, uint64_t ncols, int nz, int gap)
{
    const uint64_t per_col = ncols * ((uint64_t)nz / (uint64_t)(gap + 1) + 1);
    const uint64_t runs = gap < 0 ? ncols : (per_col < n1 ? per_col : n1);
    return (n1 + kChunk - 1) / kChunk + runs;
}

constexpr int kWzTab = 512;  // stencil columns whose z reach is tabulated in the task geometry

struct TaskGeom {
    int nx, ny, nz;
    int periodic[3];
    int autocorr;
    int mode;
    int reach_x, reach_y;   // neighbour columns considered per side
    double s[3];
    double rmax_xy;         // prune radius in the plane (incl. margin)
    double rmax_z;          // max |dz| (incl. margin)
    double rmax_3d;         // spherical limit (incl. margin), 0 = none
    uint32_t *error;        // set when a task would need an image beyond +-1
    // z reach in slabs of every neighbour column offset c = (dx + reach_x) * (2 reach_y + sub) +
    // dy + reach_y, -1 when the column is pruned; computed on the host (FP64) when the stencil
    // has at most kWzTab columns (ntab > 0), else by each thread
    int ntab;
    int16_t wz_tab[kWzTab];
    // columns of this lattice per chunk column and axis (a j lattice of split columns: offsets
    // dx, dy are counted from the first split column of the chunk's column, which spans 0 .. sub - 1)
    int sub;
    uint32_t j_off;  // packed tasks: lattice index of the split lattice's first point in the j arrays
    int zshift, nzj;  // packed tasks: j-lattice slab = slab >> zshift, of nzj per column
};

__device__ __forceinline__ int floordiv(int a, int b)
{
    int q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

// z reach (slabs) of neighbour column offset (dx, dy), -1 when the column is beyond reach: the
// radii against the gap between the chunk's column (offsets 0 .. sub - 1) and that column
__host__ __device__ inline int column_wz(const TaskGeom &G, int dx, int dy)
{
    const int sub = G.sub > 1 ? G.sub : 1;
    const int gx = dx < 0 ? -dx - 1 : (dx >= sub ? dx - sub : 0);
    const int gy = dy < 0 ? -dy - 1 : (dy >= sub ? dy - sub : 0);
    const double rx = (double)gx * G.s[0];
    const double ry = (double)gy * G.s[1];
    const double rho2 = rx * rx + ry * ry;
    if (rho2 >= G.rmax_xy * G.rmax_xy) return -1;
    double W = G.rmax_z;
    if (G.rmax_3d > 0.0) W = fmin(W, sqrt(fmax(0.0, G.rmax_3d * G.rmax_3d - rho2)));
    const double wz = ceil(W / G.s[2]);
    return wz > 1e9 ? 1000000000 : (int)wz;
}

// Empty z slabs at which a column's chunks are split: two and a half times the own column's z
// reach (a split there takes at least half a reach of j slabs out of every neighbour column's
// window, against one more task per column).  -1 (no splits) when the reach spans the column, or
// when the set-1 points are so dense (n1 points in ncols columns) that a column would hold 16
// points or more in such a gap on average.
static int chunk_gap(const TaskGeom &G, int64_t n1, uint32_t ncols)
{
    const int wz = column_wz(G, 0, 0);
    if (wz < 0 || wz >= G.nz) return -1;
    const int gap = 2 * wz + wz / 2;
    if ((double)n1 * gap >= 16.0 * (double)ncols * (double)G.nz) return -1;
    return gap;
}

// Tasks of one chunk against one neighbour column (dx, dy) (stencil index c): one per periodic z
// image whose window is not empty, split into ranges of at most kJMax points.  With EMIT == false
// only counted.
template <bool EMIT>
__device__ uint32_t chunk_col_tasks(const TaskGeom &G, uint32_t ib, uint2 info, const uint32_t *cs2, Task *out,
                                    uint32_t cat, uint32_t room, int dx, int dy, int c)
{
    const uint32_t icount = info.x & 63u;
    if (icount == 0) return 0;  // unused chunk slot
    if (G.autocorr && (dx < 0 || (dx == 0 && dy < 0))) return 0;  // half stencil
    const int wz = G.ntab ? (int)G.wz_tab[c] : column_wz(G, dx, dy);
    if (wz < 0) return 0;
    const int nz = G.nz;
    const int col = (int)info.y;
    const int a = (int)((info.x >> 6) & 4095u), b = (int)((info.x >> 18) & 4095u);
    const int ix = col / G.ny, iy = col % G.ny;
    // periodic images are encoded in two bits; the lattice construction keeps |m| <= 1
    // (neighbour reach < half the period), anything else is reported and skipped.
    const int ux = ix + dx;
    int mx = 0, cx = ux;
    if (G.periodic[0]) { mx = floordiv(ux, G.nx); cx = ux - mx * G.nx; }
    else if (ux < 0 || ux >= G.nx) return 0;
    const int uy = iy + dy;
    int my = 0, cy = uy;
    if (G.periodic[1]) { my = floordiv(uy, G.ny); cy = uy - my * G.ny; }
    else if (uy < 0 || uy >= G.ny) return 0;
    const bool own = G.autocorr && dx == 0 && dy == 0;
    const int klo = own ? a : a - wz;
    const int khi = b + wz;
    const int col2 = cx * G.ny + cy;
    const int mlo = G.periodic[2] ? floordiv(klo, nz) : 0;
    const int mhi = G.periodic[2] ? floordiv(khi, nz) : 0;
    if (mx < -1 || mx > 1 || my < -1 || my > 1 || mlo < -1 || mhi > 1) {
        if (G.error) atomicOr(G.error, 1u);
        return 0;
    }
    uint32_t ntask = 0;
    for (int mz = mlo; mz <= mhi; mz++) {
        int s0 = klo - mz * nz, s1 = khi - mz * nz;
        s0 = s0 < 0 ? 0 : s0;
        s1 = s1 > nz - 1 ? nz - 1 : s1;
        if (s0 > s1) continue;
        uint32_t jb = cs2[(uint32_t)col2 * nz + s0];
        const uint32_t je = cs2[(uint32_t)col2 * nz + s1 + 1];
        const bool own_img = own && mz == 0 && mx == 0 && my == 0;
        if (own_img) jb = ib;  // forward half of the own column
        if (je <= jb) continue;
        for (uint32_t p = jb; p < je; p += kJMax) {
            if (EMIT && ntask < room) {
                Task t;
                t.i_begin = ib;
                t.j_begin = p;
                t.j_end = min(je, p + kJMax);
                t.meta = task_meta((int)icount, mx, my, mz, own_img && p == jb ? 1 : 0) | (cat << kCatShift);
                out[ntask] = t;
            }
            ntask++;
        }
    }
    return ntask;
}

// One thread per (chunk slot, neighbour column): slot = x index, stencil column c = blockIdx.y;
// entry k = slot * ncoff + c.
__global__ void k_task_count(TaskGeom G, uint32_t nslots, const uint32_t *chunk_begin, const uint2 *chunk_info,
                             const uint32_t *cs2, uint32_t *ntasks)
{
    const uint32_t ny = 2 * G.reach_y + 1, ncoff = (2 * G.reach_x + 1) * ny;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (slot >= nslots) return;
    ntasks[(uint64_t)slot * ncoff + c] = chunk_col_tasks<false>(G, chunk_begin[slot], chunk_info[slot], cs2, nullptr, 0,
                                                                0, (int)(c / ny) - G.reach_x, (int)(c % ny) - G.reach_y,
                                                                (int)c);
}

// Writes the tasks of every (chunk, column) at its offset; with a capacity smaller than the total
// the tail is dropped and *overflow set (the caller resizes and runs again).  flags[1] receives
// the total (task_off[nslots * ncoff]), flags[3] the overflow.
__global__ void k_task_emit(TaskGeom G, uint32_t nslots, const uint32_t *chunk_begin, const uint2 *chunk_info,
                            const uint32_t *cs2, const uint32_t *task_off, Task *tasks, const uint16_t *chunk_cat,
                            uint32_t capacity, uint32_t *flags)
{
    const uint32_t ny = 2 * G.reach_y + 1, ncoff = (2 * G.reach_x + 1) * ny;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    if (slot == 0 && c == 0) flags[1] = task_off[(uint64_t)nslots * ncoff];
    if (slot >= nslots) return;
    const uint32_t off = task_off[(uint64_t)slot * ncoff + c];
    const uint32_t room = off < capacity ? capacity - off : 0u;
    const uint32_t n = chunk_col_tasks<true>(G, chunk_begin[slot], chunk_info[slot], cs2, tasks + off,
                                             chunk_cat ? (uint32_t)chunk_cat[slot] : 0u, room,
                                             (int)(c / ny) - G.reach_x, (int)(c % ny) - G.reach_y, (int)c);
    if (n > room) atomicOr(&flags[3], 1u);
}

// Counts and writes the tasks of every (chunk, column) in one pass: each warp reserves room for
// its tasks with one atomic on flags[1] (the running total, also past the capacity) and every
// lane writes its own at its offset; tasks beyond the capacity are dropped and flags[3] set (the
// caller resizes to flags[1] and runs again).  The order of the work list is the order in which
// warps reserve, which only changes which warp of the pair kernel takes which task.
__global__ void k_task_list(TaskGeom G, uint32_t nslots, const uint32_t *chunk_begin, const uint2 *chunk_info,
                            const uint32_t *cs2, Task *tasks, uint32_t capacity, uint32_t *flags)
{
    const uint32_t ny = 2 * G.reach_y + 1;
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x, c = blockIdx.y;
    const int lane = threadIdx.x & 31;
    const int dx = (int)(c / ny) - G.reach_x, dy = (int)(c % ny) - G.reach_y;
    const bool live = slot < nslots;
    const uint32_t ib = live ? chunk_begin[slot] : 0u;
    const uint2 info = live ? chunk_info[slot] : make_uint2(0u, 0u);
    const uint32_t n = chunk_col_tasks<false>(G, ib, info, cs2, nullptr, 0, 0, dx, dy, (int)c);
    uint32_t incl = n;  // inclusive warp scan of the task counts
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
    uint32_t base = 0;
    if (lane == 31 && total) base = atomicAdd(&flags[1], total);
    base = __shfl_sync(0xffffffffu, base, 31);
    if (n == 0) return;
    const uint32_t off = base + incl - n;
    const uint32_t room = off < capacity ? capacity - off : 0u;
    chunk_col_tasks<true>(G, ib, info, cs2, tasks + off, 0u, room, dx, dy, (int)c);
    if (n > room) atomicOr(&flags[3], 1u);
}

// The neighbourhood of one chunk in a j lattice of split columns as packed tasks (one warp per
// chunk slot).  Every split column within reach and every periodic z image of it whose window
// holds points gives one range; the chunk's ranges are concatenated into one list (records
// contiguous in recs, list positions from 0) and cut into items of kJMax positions.  An
// auto-correlation takes only the split columns of forward neighbour columns (its own column's
// pairs are listed from the i lattice).  Pass 0 counts, pass 1 writes: records and items are
// reserved with one atomic each per chunk (rec_count, flags[1]); past either capacity nothing
// is written, flags[3] is set and the counters still grow to the totals (the caller resizes
// and runs again).
static_assert(kJMax <= 2048, "an item's point count is stored in 11 bits");
constexpr int kItemWarps = 8;          // warps per block of k_item_list: one reservation per block
constexpr int kItemLanes = 4;          // lanes per chunk (they share its stencil list)
constexpr int kItemUnroll = 4;         // stencil entries per lane and step (their loads issued together)
constexpr int kItemStenShared = 4096;  // longest stencil list staged in shared memory (32 KB)

// One z image of one stencil entry (0: none): the range of the j lattice's slabs that hold
// window slabs [lo, hi] of periodic image mz, clamped to the lattice
__device__ __forceinline__ void item_window(const TaskGeom &G, int lo, int hi, int mz, int &s0, int &s1)
{
    s0 = lo - mz * G.nz;
    s1 = hi - mz * G.nz;
    s0 = s0 < 0 ? 0 : s0;
    s1 = s1 > G.nz - 1 ? G.nz - 1 : s1;
}

// The neighbourhood of every chunk in a j lattice of split columns as packed tasks: every
// stencil entry (split column within reach) and periodic z image whose window holds points is
// one range; a chunk's ranges are concatenated into one list (records contiguous, list
// positions from 0) and cut into items of kJMax positions.  kItemLanes lanes per chunk (a warp
// holds 32 / kItemLanes consecutive chunk slots, mostly of one lattice column, so that their
// cell-offset loads for one entry fall close together) share the stencil list sten[0 .. nsten):
// split-column offset (du, dv) = (low, high int16 of .x) and z reach .y, only the entries within
// reach (and, for an auto-correlation, of forward neighbour columns).  Pass 0 counts, pass 1
// writes: records and items are reserved with one atomic each per block (rec_count, flags[1]);
// past either capacity nothing is written, flags[3] is set and the counters still grow to the
// totals (the caller resizes and runs again).
__global__ void __launch_bounds__(32 * kItemWarps) k_item_list(TaskGeom G, uint32_t nslots, const uint32_t *chunk_begin,
                                                              const uint2 *chunk_info, const uint32_t *cs2,
                                                              const int2 *sten, int nsten, Task *tasks,
                                                              uint32_t task_cap, JRange *recs, uint32_t rec_cap,
                                                              uint32_t *flags, uint32_t *rec_count)
{
    __shared__ uint32_t s_rec[kItemWarps], s_item[kItemWarps], s_base[2];
    extern __shared__ int2 s_sten[];
    const int lane = threadIdx.x & 31, g = lane % kItemLanes;
    const uint32_t slot = (blockIdx.x * blockDim.x + threadIdx.x) / kItemLanes;
    const uint2 info = slot < nslots ? chunk_info[slot] : make_uint2(0u, 0u);
    const uint32_t icount = info.x & 63u;  // 0: unused chunk slot (or past the last)
    const uint32_t ib = slot < nslots ? chunk_begin[slot] : 0u;
    const int sub = G.sub, nz = G.nz;
    const int nyc = G.ny / sub;
    const int col = (int)info.y, ix = col / nyc, iy = col % nyc;
    const int a = (int)((info.x >> 6) & 4095u), b = (int)((info.x >> 18) & 4095u);
    const uint32_t meta = task_meta(icount ? (int)icount : 1, 0, 0, 0, 0) | kTaskPacked;
    // the stencil list in shared memory
    const bool sten_sh = nsten <= kItemStenShared;
    if (sten_sh)
        for (int e = threadIdx.x; e < nsten; e += blockDim.x) s_sten[e] = sten[e];
    __syncthreads();
    const int2 *stl = sten_sh ? (const int2 *)s_sten : sten;
    uint32_t nrec = 0, npts = 0;  // pass 0: this lane's ranges and points
    bool imgs = false;            // a range of the chunk has a periodic image
    uint32_t ctot = 0;            // the chunk's points (all its lanes)
    uint32_t r = 0, p = 0, rlast = 0, tb = 0;  // pass 1: next record, list position; the chunk's last record, first task
    for (int pass = 0; pass < 2; pass++) {
        auto emit = [&](uint32_t jb, uint32_t je, uint32_t img) {
            if (je <= jb) return;
            const uint32_t len = je - jb;
            if (pass == 0) {
                nrec++;
                npts += len;
                imgs = imgs || img != 0x15u;  // 0x15: no image on any axis
                return;
            }
            recs[r] = make_uint4(jb + G.j_off, p, img | (r == rlast ? 0x80000000u : 0u), p + len);
            // items whose first position falls in this range
            for (uint32_t m = (p + kJMax - 1) / kJMax; m * kJMax < p + len; m++) {
                const uint32_t cnt = min(kJMax, ctot - m * kJMax);
                Task t;
                t.i_begin = ib;
                t.j_begin = r;
                t.j_end = (cnt - 1) | (m << 11);
                t.meta = meta | (imgs ? kTaskImages : 0u);
                tasks[tb + m] = t;
            }
            r++;
            p += len;
        };
        const int nl = icount ? nsten : 0;
        for (int e0 = g; e0 < nl; e0 += kItemLanes * kItemUnroll) {
            uint32_t jbv[kItemUnroll], jev[kItemUnroll], imgv[kItemUnroll];
            int lov[kItemUnroll], hiv[kItemUnroll], cbv[kItemUnroll];
#pragma unroll
            for (int q = 0; q < kItemUnroll; q++) {
                jbv[q] = jev[q] = imgv[q] = 0;
                lov[q] = 0;
                hiv[q] = -1;
                cbv[q] = -1;
                const int e = e0 + q * kItemLanes;
                if (e >= nl) continue;
                const int2 se = stl[e];
                const int du = (int)(int16_t)(se.x & 0xffff), dv = se.x >> 16, wz = se.y;
                const int ux = ix * sub + du, uy = iy * sub + dv;
                int mx = 0, cx = ux, my = 0, cy = uy;
                if (G.periodic[0]) {
                    mx = ux < 0 ? -1 : (ux >= G.nx ? 1 : 0);
                    cx = ux - mx * G.nx;
                } else if (ux < 0 || ux >= G.nx) {
                    continue;
                }
                if (G.periodic[1]) {
                    my = uy < 0 ? -1 : (uy >= G.ny ? 1 : 0);
                    cy = uy - my * G.ny;
                } else if (uy < 0 || uy >= G.ny) {
                    continue;
                }
                const int lo = a - wz, hi = b + wz;
                if (cx < 0 || cx >= G.nx || cy < 0 || cy >= G.ny ||
                    (G.periodic[2] && (lo < -nz || hi >= 2 * nz))) {  // an image beyond +-1
                    if (pass == 0 && G.error) atomicOr(G.error, 1u);
                    continue;
                }
                cbv[q] = (cx * G.ny + cy) * G.nzj;
                lov[q] = lo;
                hiv[q] = hi;
                imgv[q] = (uint32_t)(mx + 1) | ((uint32_t)(my + 1) << 2);
                // the window's own image (mz = 0), loaded with the others of this step
                int s0, s1;
                item_window(G, lo, hi, 0, s0, s1);
                if (s0 <= s1) {
                    jbv[q] = cs2[(size_t)cbv[q] + (s0 >> G.zshift)];
                    jev[q] = cs2[(size_t)cbv[q] + (s1 >> G.zshift) + 1];
                }
            }
#pragma unroll
            for (int q = 0; q < kItemUnroll; q++) {
                if (cbv[q] < 0) continue;
                // periodic z images -1 and +1 (windows across the lattice's z ends: rare)
                if (G.periodic[2] && lov[q] < 0) {
                    int s0, s1;
                    item_window(G, lov[q], hiv[q], -1, s0, s1);
                    if (s0 <= s1)
                        emit(cs2[(size_t)cbv[q] + (s0 >> G.zshift)], cs2[(size_t)cbv[q] + (s1 >> G.zshift) + 1],
                             imgv[q]);
                }
                emit(jbv[q], jev[q], imgv[q] | (1u << 4));
                if (G.periodic[2] && hiv[q] >= nz) {
                    int s0, s1;
                    item_window(G, lov[q], hiv[q], 1, s0, s1);
                    if (s0 <= s1)
                        emit(cs2[(size_t)cbv[q] + (s0 >> G.zshift)], cs2[(size_t)cbv[q] + (s1 >> G.zshift) + 1],
                             imgv[q] | (2u << 4));
                }
            }
        }
        if (pass == 1) break;
        // the chunk's totals over its lanes, then block-wide offsets and one reservation
        uint32_t cp = npts, crec = nrec;  // inclusive scans within the chunk's lanes
        for (int o = 1; o < kItemLanes; o <<= 1) {
            const uint32_t tp = __shfl_up_sync(0xffffffffu, cp, o, kItemLanes);
            const uint32_t tr = __shfl_up_sync(0xffffffffu, crec, o, kItemLanes);
            if (g >= o) {
                cp += tp;
                crec += tr;
            }
        }
        ctot = __shfl_sync(0xffffffffu, cp, kItemLanes - 1, kItemLanes);
        const uint32_t crtot = __shfl_sync(0xffffffffu, crec, kItemLanes - 1, kItemLanes);
        imgs = ((__ballot_sync(0xffffffffu, imgs) >> (lane - g)) & ((1u << kItemLanes) - 1u)) != 0u;
        const bool big = ctot >= 0x80000000u;  // list positions must stay below 2^31
        const uint32_t myrec = big ? 0u : nrec;
        const uint32_t nitems = (g == 0 && !big) ? (ctot + kJMax - 1) / kJMax : 0u;
        uint32_t ir = myrec, it = nitems;  // inclusive scans over the warp
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t tr = __shfl_up_sync(0xffffffffu, ir, o), ti = __shfl_up_sync(0xffffffffu, it, o);
            if (lane >= o) {
                ir += tr;
                it += ti;
            }
        }
        const int warp = threadIdx.x >> 5;
        if (lane == 31) {
            s_rec[warp] = ir;
            s_item[warp] = it;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t sr = 0, si = 0;
            for (int w = 0; w < kItemWarps; w++) {
                const uint32_t cr = s_rec[w], ci = s_item[w];
                s_rec[w] = sr;
                s_item[w] = si;
                sr += cr;
                si += ci;
            }
            s_base[0] = sr ? atomicAdd(rec_count, sr) : 0u;
            s_base[1] = si ? atomicAdd(&flags[1], si) : 0u;
        }
        __syncthreads();
        if (big && g == 0) atomicOr(&flags[3], 1u);
        const uint32_t rb = s_base[0] + s_rec[warp] + ir - myrec;  // this lane's first record
        const uint32_t tfirst = s_base[1] + s_item[warp] + it - nitems;
        tb = __shfl_sync(0xffffffffu, tfirst, lane - g);                      // the chunk's first task
        const uint32_t crb = __shfl_sync(0xffffffffu, rb, lane - g);          // and first record
        const uint32_t nit = __shfl_sync(0xffffffffu, nitems, lane - g);
        const bool over = (uint64_t)crb + (big ? 0u : crtot) > rec_cap || (uint64_t)tb + nit > task_cap;
        if (big || crtot == 0) return;  // no barrier below
        if (over) {
            // reserved task slots below the capacity become empty tasks (the pair kernel runs
            // before the host sees the overflow and reads every slot below the capacity)
            if (g == 0) {
                for (uint32_t m = 0; m < nit && (uint64_t)tb + m < task_cap; m++) {
                    Task t;
                    t.i_begin = ib;
                    t.j_begin = 0;
                    t.j_end = 0;
                    t.meta = task_meta((int)icount, 0, 0, 0, 0);
                    tasks[tb + m] = t;
                }
                atomicOr(&flags[3], 1u);
            }
            return;
        }
        r = rb;
        p = cp - npts;  // this lane's first list position within the chunk
        rlast = crb + crtot - 1;
    }
}

// ------------------------------------------------------------------------------------
// pair kernels
// ------------------------------------------------------------------------------------
struct SmemLayout {
    int nedges, nbins, warps, lut_n, lane_stride;
    int nrows;  // histogram rows incl. the trash rows that absorb rejected / deferred pairs
    bool need_avg, need_w;
    int entry_words;  // 32-bit words per histogram entry: count [, avg hi, avg lo] [, w hi, w lo]
    size_t edges_off, guard_off, ascale_off, lut_off, stage_off, hist_off, per_warp_hist, per_warp_stage, total;
    size_t shift_off;  // FP32 kernels: periodic shifts of j points by image code (hi then lo, 64 float4 each)
    bool extras;       // the per-warp stage holds staged j indices, image codes and a box (packed or pruned tiles)
    size_t wd_off, per_warp_wd;  // FP64 kernel with weights: one double weight sum per row and warp
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

constexpr int kRefineQueue = 64;  // per-warp queue of pairs awaiting the FP64 re-evaluation
constexpr int kSlowQueue = 64;    // per-warp queue of pairs in flagged table buckets

struct RefineEntry {
    uint32_t i, j, meta;  // meta: image code bits 8-13 as in Task
};

// Histogram accumulators live in shared memory, one set per warp.  With lane_stride == 32 every
// lane owns a private column (no contention); for large 2-D histograms lanes share columns
// through shared atomics.  An entry is 1, 3 or 5 consecutive 32-bit words: the count, then the
// separation and weight sums as 32-bit fixed-point terms split into a signed high half (bits
// 16-31) and an unsigned low half (bits 0-15).  Only 32-bit shared reductions are used: 64-bit
// and floating-point shared atomics run several times slower on this GPU.  Odd entry sizes keep
// the private columns on distinct banks.  A column takes at most kColumnTerms terms between
// flushes into the FP64 global histogram, so neither half can overflow.
constexpr int kColumnTerms = 1 << 15;

__host__ __device__ inline SmemLayout smem_layout(int nedges, int nbins, int warps, bool f64, int lut_n, int lane_stride,
                                                  bool need_avg, bool need_w, bool store_dz, bool lo_stage,
                                                  bool packed = false, bool prune = false)
{
    SmemLayout L;
    L.need_avg = need_avg;
    L.need_w = need_w;
    L.entry_words = 1 + (need_avg ? 2 : 0) + (need_w ? 2 : 0);
    L.nedges = nedges;
    L.nbins = nbins;
    L.warps = warps;
    L.lut_n = lut_n;
    L.lane_stride = lane_stride;
    // trash rows: two for 1-D modes (a flagged byte-table entry points half a row past the first),
    // one row of 2-D cells (npibin + 1 = nbins / nedges) otherwise
    L.nrows = nbins + (store_dz && nbins > nedges ? nbins / nedges : 2);
    size_t o = 0;
    L.edges_off = o;
    o = align_up(o + sizeof(double) * nedges, 16);
    L.guard_off = o;
    o = align_up(o + sizeof(float) * 2 * nedges, 16);
    L.ascale_off = o;
    o = align_up(o + sizeof(float) * (nedges + 2), 16);
    L.lut_off = o;
    o = align_up(o + sizeof(uint32_t) * (lut_n + 1), 16);
    L.shift_off = o;
    o = align_up(o + (f64 || !packed ? 0 : 2 * 64 * sizeof(float4)), 16);
    L.stage_off = o;
    // f32: float4 hi[32] + float4 lo[32] + refine and slow queues + queue fill and counters (16
    // bytes) + the lattice index and image code of every staged j point (packed or pruned tiles)
    // + the chunk's bounding box (pruned tiles) (the lo half is laid out even where it stays
    // unused: the histogram layouts were measured with it);
    // f64: double4_32a[32] + int rc[32] + int orig[32]
    (void)lo_stage;
    L.extras = !f64 && (packed || prune);
    L.per_warp_stage = f64 ? (32 * sizeof(double4_32a) + 64 * sizeof(int))
                           : (64 * sizeof(float4) + (kRefineQueue + kSlowQueue) * sizeof(RefineEntry) + 16 +
                              (packed || prune ? 32 * sizeof(uint32_t) + 32 + 2 * sizeof(float4) : 0));
    o = align_up(o + L.per_warp_stage * warps, 16);
    L.hist_off = o;
    L.per_warp_hist = align_up((size_t)L.nrows * lane_stride * 4 * L.entry_words + 32, 16);
    o += L.per_warp_hist * warps;
    L.wd_off = o;
    L.per_warp_wd = (f64 && need_w) ? align_up(sizeof(double) * (size_t)L.nrows, 16) : 0;
    o += L.per_warp_wd * warps;
    L.total = o;
    return L;
}

struct WarpHist {
    uint32_t *e;          // entries: (row * ls + column) * ew words
    int ls;               // lane stride
    int ew;               // words per entry
    const float *ascale;  // fixed-point scale of the separation sums per separation bin (shared)
};

__device__ __forceinline__ WarpHist warp_hist(unsigned char *smem, const SmemLayout &L, int warp)
{
    WarpHist h;
    h.e = (uint32_t *)(smem + L.hist_off + L.per_warp_hist * warp);
    h.ls = L.lane_stride;
    h.ew = L.entry_words;
    h.ascale = (const float *)(smem + L.ascale_off);
    return h;
}

__device__ __forceinline__ void zero_hist(WarpHist h, const SmemLayout &L, int lane)
{
    const int n = L.nrows * h.ls * h.ew;
    for (int b = lane; b < n; b += 32) h.e[b] = 0;
}

// word offsets of the sums inside an entry
template <bool NEED_AVG>
__host__ __device__ constexpr int avg_word() { return 1; }
template <bool NEED_AVG>
__host__ __device__ constexpr int w_word() { return NEED_AVG ? 3 : 1; }

__device__ __forceinline__ void add_term(uint32_t *hi_lo, int v)
{
    atomicAdd(hi_lo, (uint32_t)(v >> 16));
    atomicAdd(hi_lo + 1, (uint32_t)v & 0xffffu);
}

template <bool NEED_AVG, bool NEED_W>
__device__ __forceinline__ void flush_hist(const PairArgs &A, WarpHist h, int lane, uint32_t cat = 0, double *wd = nullptr)
{
    __syncwarp();
    unsigned long long *g_cnt = A.g_cnt + (size_t)cat * A.nbins;
    double *g_avg = A.g_avg + (size_t)cat * A.nbins;
    double *g_w = A.g_w + (size_t)cat * A.nbins;
    for (int b = lane; b < A.nbins; b += 32) {
        unsigned long long c = 0, al = 0, wl = 0;
        long long ah = 0, wh = 0;
        for (int t = 0; t < h.ls; t++) {
            const int l = (t + lane) & (h.ls - 1);  // skewed so that the lanes hit distinct banks
            uint32_t *e = h.e + (size_t)(b * h.ls + l) * h.ew;
            c += e[0];
            e[0] = 0;
            if (NEED_AVG) {
                uint32_t *s = e + avg_word<NEED_AVG>();
                ah += (int)s[0];
                al += s[1];
                s[0] = 0;
                s[1] = 0;
            }
            if (NEED_W) {
                uint32_t *s = e + w_word<NEED_AVG>();
                wh += (int)s[0];
                wl += s[1];
                s[0] = 0;
                s[1] = 0;
            }
        }
        if (c) atomicAdd(&g_cnt[b], c);
        if (NEED_AVG) {
            const long long va = ah * 65536ll + (long long)al;
            if (va) atomicAdd(&g_avg[b], (double)va / (double)h.ascale[b / A.rbin_div]);
        }
        if (NEED_W) {
            const long long vw = wh * 65536ll + (long long)wl;
            double v = (double)vw * A.w_unscale;
            if (wd) {
                v += wd[b];
                wd[b] = 0.0;
            }
            if (v != 0.0) atomicAdd(&g_w[b], v);
        }
    }
    __syncwarp();
}

// first-point rule of the reference for wrapped auto-correlation pairs
__device__ __forceinline__ bool j_is_first(const PairArgs &A, uint32_t i, uint32_t j, double zi, double zj)
{
    const int2 ri = A.ro1[i], rj = A.ro2[j];
    if (rj.x != ri.x) return rj.x > ri.x;
    if (zj != zi) return zj < zi;
    return rj.y < ri.y;
}

// Whether the reference's cell-pair list holds reference cells ci, cj (linear indices) with the
// periodic image M of the second point: per axis the second cell is the first one's neighbour at
// an offset of at most the refine factor, wrapped across the lattice edge with the image of the
// side it leaves (utils/gridlink_impl.c.src:494-521).
__device__ __forceinline__ bool ref_linked(const PairArgs &A, int ci, int cj, int Mx, int My, int Mz)
{
    const int n1 = A.ref_n[1], n2 = A.ref_n[2];
    const int ti = ci / n2, tj = cj / n2;
    const int dz = cj - tj * n2 - (ci - ti * n2) + Mz * n2;
    const int dy = tj % n1 - ti % n1 + My * n1;
    const int dx = tj / n1 - ti / n1 + Mx * A.ref_n[0];
    return abs(dx) <= A.ref_reach[0] && abs(dy) <= A.ref_reach[1] && abs(dz) <= A.ref_reach[2];
}

template <int MODE>
__device__ __noinline__ int refine_pair(const PairArgs &A, const double *se, uint32_t i, uint32_t j,
                                        int mx, int my, int mz, double *avg_term, double *wprod)
{
    const double4_32a pi = A.d1[i], pj = A.d2[j];
    *wprod = pi.w * pj.w;
    const double ox = A.odbl[0][mx + 1], oy = A.odbl[1][my + 1], oz = A.odbl[2][mz + 1];
    if (MODE == MODE_THETA) {
        return ref_eval<MODE>(A, se, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, 0.0, 0.0, 0.0, avg_term);
    }
    const bool wrapped = (mx | my | mz) != 0;
    if (A.autocorr && wrapped && j_is_first(A, i, j, pi.z, pj.z)) {
        return ref_eval<MODE>(A, se, pj.x, pj.y, pj.z, pi.x, pi.y, pi.z, ox, oy, oz, avg_term);
    }
    return ref_eval<MODE>(A, se, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, -ox, -oy, -oz, avg_term);
}

// Angle in degrees subtended by a chord ch of the unit sphere, 2 asin(ch / 2).  For angular bins
// up to 23 degrees (ch / 2 <= 0.2) the arcsine's Maclaurin series
//   asin(x) = x (1 + x^2/6 + 3x^4/40 + 5x^6/112 + 35x^8/1152 + ...)
// truncated after the x^9 term is within 3e-9 relative of it there, well inside FP32 rounding.
template <bool SERIES>
__device__ __forceinline__ float chord_degrees(float ch)
{
    const float x = 0.5f * ch;
    if (SERIES) {
        const float x2 = x * x;
        const float p = fmaf(fmaf(fmaf(fmaf(35.f / 1152.f, x2, 5.f / 112.f), x2, 3.f / 40.f), x2, 1.f / 6.f), x2, 1.f);
        return x * p * 114.59155902616465f;
    }
    return 2.f * asinf(x) * 57.29577951308232f;
}

// LUT bucket of the classified FP32 quantity q (r^2, rp^2, s^2 or chord^2): one mad.hi on the
// float bits (bucket = (bits >> shift) - base), clamped to the reject entry lut_n.
__device__ __forceinline__ uint32_t lut_bucket(const PairArgs &A, float q)
{
    uint32_t r;
    asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(r) : "r"(__float_as_uint(q)), "r"(A.lut_mul), "r"(A.lut_negbase));
    return min(r, (uint32_t)A.lut_n);
}

// The byte table's classified quantity q' = min(r^2 + b, cap): (dx^2 + b) + dy^2 + dz^2 with one
// rounding per fused multiply-add, capped at the start of the first bucket wholly beyond the
// last guard (all farther pairs share that one reject entry, so their table loads broadcast).
// q' >= b always (b a power of two), so its bits index the table from bits(b) with no lower clamp.
// Two FP32 lanes in one 64-bit register: the paired (f32x2) arithmetic evaluates two pairs per
// instruction, each lane rounded exactly as its scalar counterpart.
__device__ __forceinline__ unsigned long long f2_pack(float a, float b)
{
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_sub(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_mul(unsigned long long a, unsigned long long b)
{
    unsigned long long r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b, unsigned long long c)
{
    unsigned long long r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}

__device__ __forceinline__ float q8(const PairArgs &A, float dx, float dy, float dz)
{
    return fminf(fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, A.q_bias))), A.q_cap);
}

// Exact FP32 classification of q against the guard bands: the bin m (1..nedges-1) with
// *amb = false when q is provably on one side of every edge, *amb = true when q lies inside an
// edge's band, or 0 when q is provably outside [rmin, rmax).
__device__ __forceinline__ int classify_q(const PairArgs &A, const float *glo, const float *ghi, float q, bool *amb)
{
    const int n = A.nedges;
    *amb = false;
    if (q < glo[0] || q >= ghi[n - 1]) return 0;
    // m = 1 + #{k in [1, n) : glo[k] <= q}; the guards are non-decreasing (binary lifting)
    int pos = 0;
    for (int step = A.guard_search_top; step > 0; step >>= 1)
        if (pos + step <= n - 1 && glo[pos + step] <= q) pos += step;
    const int m = pos + 1;
    *amb = q < ghi[m - 1];
    return m;
}

// FP32 quantities of a survey pair.  Positions are split at the observer (x = hi + lo, hi on a
// power-of-two grid): s = x_j - x_i is the exact hi difference plus the lo difference, the line of
// sight l = x_i + x_j (per i point a = hi_i + lo_i), and
//   s2 = |s|^2,  pi = |s.l| / |l|,  rp2 = |s x l|^2 / |l|^2
// (the cross product keeps rp accurate to a few ulps of |s| where s^2 - pi^2 would cancel).
template <int MODE>
__device__ __forceinline__ void mock_terms(float4 pj, float4 pjl, float xi, float yi, float zi, float xil, float yil,
                                           float zil, float ax, float ay, float az, float &s2, float &l2, float &pi,
                                           float &rp2)
{
    const float sx = (pj.x - xi) + (pjl.x - xil), sy = (pj.y - yi) + (pjl.y - yil), sz = (pj.z - zi) + (pjl.z - zil);
    const float lx = ax + (pj.x + pjl.x), ly = ay + (pj.y + pjl.y), lz = az + (pj.z + pjl.z);
    s2 = fmaf(sz, sz, fmaf(sy, sy, sx * sx));
    l2 = fmaf(lz, lz, fmaf(ly, ly, lx * lx));
    const float rl = rsqrtf(l2);
    pi = fabsf(fmaf(lz, sz, fmaf(ly, sy, lx * sx))) * rl;
    rp2 = 0.f;
    if (MODE == MODE_RPPI_MOCK) {
        const float cx = fmaf(sy, lz, -(sz * ly)), cy = fmaf(sz, lx, -(sx * lz)), cz = fmaf(sx, ly, -(sy * lx));
        rp2 = fmaf(cz, cz, fmaf(cy, cy, cx * cx)) * (rl * rl);
    }
}

// Exact FP32 classification of one candidate whose LUT bucket is flagged: guard scan and the
// 2-D bin checks.  Returns the flat bin (with its FP32 accumulator terms), -1 when the pair is
// provably not counted, or -2 when it lies inside an error band and needs the reference's FP64
// formula.
template <int MODE, bool NEED_AVG, bool NEED_W, bool LUT8>
__device__ __noinline__ int slow_candidate(const PairArgs &A, const float *glo, const float *ghi, float4 pj, float4 pjl,
                                           float xi, float yi, float zi, float xil, float yil, float zil, float wi,
                                           float ax, float ay, float az, float *favg, float *fw)
{
    if (MODE == MODE_RPPI_MOCK || MODE == MODE_SMU_MOCK) {
        float s2, l2, pi, rp2;
        mock_terms<MODE>(pj, pjl, xi, yi, zi, xil, yil, zil, ax, ay, az, s2, l2, pi, rp2);
        if (!(s2 < A.s2_cut_f)) return -1;
        if (!(l2 >= A.l2_min_f)) return -2;  // near the observer: the bands do not hold
        bool amb;
        const int m = classify_q(A, glo, ghi, fmaxf(MODE == MODE_RPPI_MOCK ? rp2 : s2, A.q_floor), &amb);
        if (m == 0) return -1;
        int pb;
        if (MODE == MODE_RPPI_MOCK) {
            if (pi >= A.pimax_hi_f) return -1;
            if (pi > A.pimax_lo_f) amb = true;
            const float tpi = pi * A.inv_dpi_f;
            pb = (int)tpi;
            const float fr = tpi - (float)pb;
            if ((pb >= 1 && fr < A.pibin_band) || (1.f - fr) < A.pibin_band) amb = true;
            if (NEED_AVG) amb = true;  // rp averages need the FP64 rp of every counted pair
        } else {
            const float inv_s = rsqrtf(fmaxf(s2, 1e-30f));
            const float mu = pi * inv_s;
            const float emu = fmaf(A.mu_band_abs, inv_s, A.mu_band_rel);
            if (mu >= A.mu_max_f + emu) return -1;
            if (mu > A.mu_max_f - emu) amb = true;
            const float tmu = mu * A.inv_dmu_f;
            pb = (int)tmu;
            const float bt = emu * A.inv_dmu_f + 4e-7f * tmu;
            const float fr = tmu - (float)pb;
            if ((pb >= 1 && fr < bt) || (1.f - fr) < bt) amb = true;
        }
        if (amb) return -2;
        pb = pb > A.npibin ? A.npibin : pb;
        if (NEED_AVG) *favg = sqrtf(s2);
        if (NEED_W) *fw = wi * pj.w;
        return m * (A.npibin + 1) + pb;
    }
    const float dx = pj.x - xi, dy = pj.y - yi, dz = pj.z - zi;
    float q;  // the fast path's expression, so that the pair lands in the same flagged bucket
    if (LUT8) q = q8(A, dx, dy, dz);
    else if (MODE == MODE_RPPI || MODE == MODE_WP) q = fmaf(dy, dy, fmaf(dx, dx, A.q_floor));
    else q = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, A.q_floor)));
    bool amb;
    const int m = classify_q(A, glo, ghi, q, &amb);
    if (m == 0) return -1;
    int bin = m;
    if (MODE == MODE_RPPI || MODE == MODE_WP) {
        const float adz = fabsf(dz);
        if (adz >= A.pimax_hi_f) return -1;
        if (adz > A.pimax_lo_f) amb = true;
        if (MODE == MODE_RPPI) {
            const float tpi = adz * A.inv_dpi_f;
            int pb = (int)tpi;
            const float fr = tpi - (float)pb;
            if ((pb >= 1 && fr < A.pibin_band) || (1.f - fr) < A.pibin_band) amb = true;
            pb = pb > A.npibin ? A.npibin : pb;
            bin = m * (A.npibin + 1) + pb;
        }
    }
    if (MODE == MODE_SMU) {
        if (!(q > 0.f)) amb = true;
        const float sqq = sqrtf(q);
        const float mu = fabsf(dz) / sqq;
        const float emu = A.mu_band_abs / sqq + 6e-7f * mu + 1e-7f;
        if (mu >= A.mu_max_f + emu) return -1;  // definitely mu >= mu_max
        if (mu > A.mu_max_f - emu) amb = true;
        const float tmu = mu * A.inv_dmu_f;
        int pb = (int)tmu;
        const float bt = emu * A.inv_dmu_f + 3e-7f * tmu;
        const float fr = tmu - (float)pb;
        if ((pb >= 1 && fr < bt) || (1.f - fr) < bt) amb = true;
        pb = pb > A.npibin ? A.npibin : pb;
        bin = m * (A.npibin + 1) + pb;
    }
    if (amb) return -2;
    if (NEED_AVG) {
        const float dxp = dx + (pjl.x - xil), dyp = dy + (pjl.y - yil), dzp = dz + (pjl.z - zil);
        if (MODE == MODE_RPPI || MODE == MODE_WP) {
            *favg = sqrtf(fmaf(dyp, dyp, dxp * dxp));
        } else if (MODE == MODE_THETA) {
            const float ch = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
            *favg = A.theta_series ? chord_degrees<true>(ch) : chord_degrees<false>(ch);
        } else {
            *favg = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
        }
    }
    if (NEED_W) *fw = wi * pj.w;
    return bin;
}

// one pair of flat bin `bin` into column entry hidx (slow path, FP64 path)
template <bool NEED_AVG, bool NEED_W>
__device__ __forceinline__ void accumulate(const PairArgs &A, WarpHist h, int bin, int hidx, double davg, double dw)
{
    uint32_t *e = h.e + (size_t)hidx * h.ew;
    atomicAdd(e, 1u);
    if (NEED_AVG) add_term(e + avg_word<NEED_AVG>(), __double2int_rn(davg * (double)h.ascale[bin / A.rbin_div]));
    if (NEED_W) add_term(e + w_word<NEED_AVG>(), __double2int_rn(dw * (double)A.w_scale_f));
}

template <int IMM>
__device__ __forceinline__ void red_shared_u32_at(uint32_t saddr, uint32_t v)
{
    asm volatile("red.shared.add.u32 [%0+%2], %1;" ::"r"(saddr), "r"(v), "n"(IMM));
}

// Fast classification of one pair.  k is the tile position (compile-time in full tiles).  The
// LUT entry is the byte offset of the histogram row the pair belongs to (a trash row when the
// pair is rejected or deferred) with bit 31 set when the pair must go through the exact slow
// path; the caller issues one unconditional conflict-free shared reduction per pair.
template <int MODE, bool NEED_AVG, bool NEED_W, bool OWN, bool SER>
__device__ __forceinline__ uint32_t pair_offset(const PairArgs &A, const float4 *__restrict__ sjhi,
                                                const float4 *__restrict__ sjlo, const uint32_t *__restrict__ lut,
                                                const float *__restrict__ ascale, int k, uint32_t jb, uint32_t i, float xi, float yi, float zi,
                                                float xil, float yil, float zil, float wis, float ax, float ay, float az,
                                                uint32_t &slow, int &vw, int &vavg, const uint32_t *__restrict__ jidx)
{
    if (MODE == MODE_RPPI_MOCK || MODE == MODE_SMU_MOCK) {
        const float4 pj = sjhi[k], pjl = sjlo[k];
        float s2, l2, pi, rp2;
        mock_terms<MODE>(pj, pjl, xi, yi, zi, xil, yil, zil, ax, ay, az, s2, l2, pi, rp2);
        const float q = fmaxf(MODE == MODE_RPPI_MOCK ? rp2 : s2, A.q_floor);
        const uint32_t e = lut[lut_bucket(A, q)];
        uint32_t off = e & 0x003fffffu, sl = e;
        // own column of an auto-correlation: only j > i (every outcome below is masked by keep;
        // pruned tiles: the staged point's own index)
        const bool keep = !OWN || (jidx ? jidx[k] : jb + (uint32_t)k) > i;
        off = keep ? off : A.trash_off;
        sl = keep ? sl : 0u;
        const bool real = off != A.trash_off;
        const bool near = keep && !(l2 >= A.l2_min_f);  // also NaN (padding far away)
        bool rej, amb;
        uint32_t add;
        if (MODE == MODE_RPPI_MOCK) {
            rej = !(pi < A.pimax_hi_f);
            amb = pi > A.pimax_lo_f || NEED_AVG;
            const int v = __float_as_int(fmaf(pi, A.inv_dpi256_f, 12582912.0f)) - 0x4B400000;
            amb = amb || (((v + A.pi_band_q) & 255) < 2 * A.pi_band_q);
            add = (uint32_t)min(v >> 8, A.npibin) * A.row_bytes;
        } else {
            const float inv_s = rsqrtf(q);
            const float mu = pi * inv_s;
            const float emu = fmaf(A.mu_band_abs, inv_s, A.mu_band_rel);
            rej = !(mu < A.mu_max_f + emu);
            const float tmu = mu * A.inv_dmu_f;
            const float rt = rintf(tmu);
            amb = (mu > A.mu_max_f - emu) || (fabsf(tmu - rt) < emu * A.inv_dmu_f + 4e-7f * tmu && rt >= 0.5f);
            add = (uint32_t)min((int)tmu, A.npibin) * A.row_bytes;
        }
        rej = !(s2 < A.s2_cut_f) || (rej && !near);
        slow = (!rej && ((sl >> 31) || near || (real && amb))) ? 0x80000000u : 0u;
        off = (real && !rej && !amb && !near) ? off + add : A.trash_off;
        if (NEED_W) vw = __float2int_rn(wis * pj.w);
        if (NEED_AVG) vavg = MODE == MODE_SMU_MOCK ? __float2int_rn(sqrtf(s2) * ascale[(e >> 22) & 0x1ffu]) : 0;
        return off;
    }
    const float4 pj = sjhi[k];
    const float dx = pj.x - xi, dy = pj.y - yi, dz = pj.z - zi;
    // q_floor (1e-30 when rmin <= 0, else 0) keeps exact-zero separations inside the table
    float q;
    if (MODE == MODE_RPPI || MODE == MODE_WP) q = fmaf(dy, dy, fmaf(dx, dx, A.q_floor));
    else q = fmaf(dz, dz, fmaf(dy, dy, fmaf(dx, dx, A.q_floor)));
    const uint32_t e = lut[lut_bucket(A, q)];
    uint32_t off = e & 0x003fffffu;  // bits 0-21: row byte offset, 22-30: separation bin, 31: flagged
    slow = e;
    if (OWN) {  // own column: only j > i (pruned tiles: the staged point's own index)
        const bool keep = (jidx ? jidx[k] : jb + (uint32_t)k) > i;
        off = keep ? off : A.trash_off;
        slow = keep ? slow : 0u;
    }
    if (MODE == MODE_RPPI || MODE == MODE_WP || MODE == MODE_SMU) {
        const float adz = fabsf(dz);
        const bool real = off != A.trash_off;  // a definite rp / s bin
        bool rej, amb;
        uint32_t add = 0;
        if (MODE == MODE_SMU) {
            const float inv_s = rsqrtf(q);
            const float mu = adz * inv_s;
            const float emu = A.mu_band_abs * inv_s + 1e-6f * mu + 1e-7f;
            rej = !(mu < A.mu_max_f + emu);
            const float tmu = mu * A.inv_dmu_f;
            const float rt = rintf(tmu);
            amb = (mu > A.mu_max_f - emu) || (fabsf(tmu - rt) < emu * A.inv_dmu_f + 4e-7f * tmu && rt >= 0.5f);
            add = (uint32_t)min((int)tmu, A.npibin) * A.row_bytes;
        } else {
            rej = !(adz < A.pimax_hi_f);
            amb = adz > A.pimax_lo_f;
            if (MODE == MODE_RPPI) {
                // round(|dz| / dpi * 256) with the 1.5*2^23 constant: pi bin and its 8-bit fraction
                const int v = __float_as_int(fmaf(adz, A.inv_dpi256_f, 12582912.0f)) - 0x4B400000;
                amb = amb || (((v + A.pi_band_q) & 255) < 2 * A.pi_band_q);
                add = (uint32_t)min(v >> 8, A.npibin) * A.row_bytes;
            }
        }
        slow = (!rej && ((slow >> 31) || (real && amb))) ? 0x80000000u : 0u;
        off = (real && !rej && !amb) ? off + add : A.trash_off;
    }
    if (NEED_W) vw = __float2int_rn(wis * pj.w);  // 32-bit term (rejected pairs saturate into the trash row)
    if (NEED_AVG) {
        const float4 pjl = sjlo[k];
        const float dxp = dx + (pjl.x - xil), dyp = dy + (pjl.y - yil), dzp = dz + (pjl.z - zil);
        float favg;
        if (MODE == MODE_RPPI || MODE == MODE_WP) {
            favg = sqrtf(fmaf(dyp, dyp, dxp * dxp));
        } else if (MODE == MODE_THETA) {
            const float ch = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
            favg = chord_degrees<SER>(ch);
        } else {
            favg = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
        }
        vavg = __float2int_rn(favg * ascale[(e >> 22) & 0x1ffu]);
    }
    return off;
}

template <int MODE, bool NEED_AVG, bool NEED_W, bool OWN, bool SER, int U>
__device__ __forceinline__ void pairs_group(const PairArgs &A, const float4 *__restrict__ sjhi,
                                            const float4 *__restrict__ sjlo, const uint32_t *__restrict__ lut,
                                            const float *__restrict__ ascale, int k0,
                                            uint32_t jb, uint32_t i, float xi, float yi, float zi, float xil, float yil,
                                            float zil, float wis, float ax, float ay, float az, uint32_t cnt_s,
                                            uint32_t &slowbits, const uint32_t *__restrict__ jidx)
{
    uint32_t off[U];
    int vw[U], va[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
        uint32_t sl;
        vw[u] = 0;
        va[u] = 0;
        off[u] = pair_offset<MODE, NEED_AVG, NEED_W, OWN, SER>(A, sjhi, sjlo, lut, ascale, k0 + u, jb, i, xi, yi, zi, xil, yil, zil,
                                                          wis, ax, ay, az, sl, vw[u], va[u], jidx);
        slowbits = __funnelshift_l(sl, slowbits, 1);  // pair k of n ends at bit n - 1 - k
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
        const uint32_t e = cnt_s + off[u];  // this lane's entry in the pair's row
        red_shared_u32_at<0>(e, 1u);
        if (NEED_AVG) {
            red_shared_u32_at<4 * avg_word<NEED_AVG>()>(e, (uint32_t)(va[u] >> 16));
            red_shared_u32_at<4 * avg_word<NEED_AVG>() + 4>(e, (uint32_t)va[u] & 0xffffu);
        }
        if (NEED_W) {
            red_shared_u32_at<4 * w_word<NEED_AVG>()>(e, (uint32_t)(vw[u] >> 16));
            red_shared_u32_at<4 * w_word<NEED_AVG>() + 4>(e, (uint32_t)vw[u] & 0xffffu);
        }
    }
}

// Byte-table fast path of a group of U pairs (DD(r), xi, DDtheta): the staged j coordinates are
// read four points per 16-byte broadcast load (the stage is laid out coordinate by coordinate),
// q' from the points, the entry from the table at byte address mad.hi(bits(q'), 2^(32 - shift),
// lut_add), the flag bit funnelled into slowbits (pair k of n ends at bit 32 - n + k), and one
// shared reduction per pair at entry * half_row + cnt_s (a flagged entry points half a row into
// the spare rows).
template <int MODE, bool NEED_AVG, bool NEED_W, bool OWN, bool SER, int U>
__device__ __forceinline__ void pairs_group8(const PairArgs &A, const float4 *__restrict__ sjhi,
                                             const float4 *__restrict__ sjlo, uint32_t lut_add,
                                             const float *__restrict__ ascale, int k0, uint32_t jb, uint32_t i, float xi,
                                             float yi, float zi, float xil, float yil, float zil, float wis,
                                             float qcap, uint32_t cnt_s, uint32_t &slowbits,
                                             const uint32_t *__restrict__ jidx = nullptr)
{
    static_assert(U % 4 == 0, "the byte-table stage is read four j points at a time");
    const float *S = (const float *)sjhi, *SL8 = (const float *)sjlo;
    const unsigned long long xi2 = f2_pack(xi, xi), yi2 = f2_pack(yi, yi), zi2 = f2_pack(zi, zi),
                             b2 = f2_pack(A.q_bias, A.q_bias);
    const unsigned long long xil2 = f2_pack(xil, xil), yil2 = f2_pack(yil, yil), zil2 = f2_pack(zil, zil);
    uint32_t addr[U];
    int vw[U], va[U];
#pragma unroll
    for (int g = 0; g < U; g += 4) {
        const int kq = k0 + g;
        const float4 X = *(const float4 *)(S + kq), Y = *(const float4 *)(S + 32 + kq),
                     Z = *(const float4 *)(S + 64 + kq);
        float4 Wj = make_float4(0.f, 0.f, 0.f, 0.f), LX = Wj, LY = Wj, LZ = Wj;
        if (NEED_W) Wj = *(const float4 *)(S + 96 + kq);
        if (NEED_AVG) {
            LX = *(const float4 *)(SL8 + kq);
            LY = *(const float4 *)(SL8 + 32 + kq);
            LZ = *(const float4 *)(SL8 + 64 + kq);
        }
        // separations and q' of the four pairs, two per paired instruction (the scalar q8 chain,
        // lane by lane)
        float qv[4], sv[4];  // q' and, with averages, the squared separation from the lo-corrected points
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const unsigned long long dx2 = f2_sub(h ? f2_pack(X.z, X.w) : f2_pack(X.x, X.y), xi2);
            const unsigned long long dy2 = f2_sub(h ? f2_pack(Y.z, Y.w) : f2_pack(Y.x, Y.y), yi2);
            const unsigned long long dz2 = f2_sub(h ? f2_pack(Z.z, Z.w) : f2_pack(Z.x, Z.y), zi2);
            const unsigned long long q2 = f2_fma(dz2, dz2, f2_fma(dy2, dy2, f2_fma(dx2, dx2, b2)));
            f2_unpack(q2, qv[2 * h], qv[2 * h + 1]);
            if (NEED_AVG) {
                // dx + (lx - xil) and the sum of squares, as the scalar form rounds them
                const unsigned long long dxp = f2_add(dx2, f2_sub(h ? f2_pack(LX.z, LX.w) : f2_pack(LX.x, LX.y), xil2));
                const unsigned long long dyp = f2_add(dy2, f2_sub(h ? f2_pack(LY.z, LY.w) : f2_pack(LY.x, LY.y), yil2));
                const unsigned long long dzp = f2_add(dz2, f2_sub(h ? f2_pack(LZ.z, LZ.w) : f2_pack(LZ.x, LZ.y), zil2));
                const unsigned long long s2 = f2_fma(dzp, dzp, f2_fma(dyp, dyp, f2_mul(dxp, dxp)));
                f2_unpack(s2, sv[2 * h], sv[2 * h + 1]);
            }
        }
#pragma unroll
        for (int v = 0; v < 4; v++) {
            const int u = g + v, k = kq + v;
            const float q = fminf(qv[v], qcap);
            uint32_t a, e;
            asm("mad.hi.u32 %0, %1, %2, %3;" : "=r"(a) : "r"(__float_as_uint(q)), "r"(A.lut_mul), "r"(lut_add));
            asm("ld.shared.u8 %0, [%1];" : "=r"(e) : "r"(a));
            if (OWN) {  // own column: only j > i (pruned tiles: the staged point's own index)
                const uint32_t jj = jidx ? jidx[k] : jb + (uint32_t)k;
                e = jj > i ? e : A.trash_e;
            }
            slowbits = __funnelshift_r(slowbits, e, 1);
            addr[u] = e * A.half_row + cnt_s;
            vw[u] = 0;
            va[u] = 0;
            if (NEED_W) {
                const float jw = v == 0 ? Wj.x : v == 1 ? Wj.y : v == 2 ? Wj.z : Wj.w;
                vw[u] = __float2int_rn(wis * jw);
            }
            if (NEED_AVG) {
                const float d = sqrtf(sv[v]);
                const float favg = MODE == MODE_THETA ? chord_degrees<SER>(d) : d;
                va[u] = __float2int_rn(favg * ascale[e >> 1]);
            }
        }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
        red_shared_u32_at<0>(addr[u], 1u);
        if (NEED_AVG) {
            red_shared_u32_at<4 * avg_word<NEED_AVG>()>(addr[u], (uint32_t)(va[u] >> 16));
            red_shared_u32_at<4 * avg_word<NEED_AVG>() + 4>(addr[u], (uint32_t)va[u] & 0xffffu);
        }
        if (NEED_W) {
            red_shared_u32_at<4 * w_word<NEED_AVG>()>(addr[u], (uint32_t)(vw[u] >> 16));
            red_shared_u32_at<4 * w_word<NEED_AVG>() + 4>(addr[u], (uint32_t)vw[u] & 0xffffu);
        }
    }
}

template <int MODE, bool NEED_AVG, bool NEED_W, bool OWN, bool SER>
__device__ __forceinline__ uint32_t tile_fast8(const PairArgs &A, const float4 *__restrict__ sjhi,
                                               const float4 *__restrict__ sjlo, uint32_t lut_add,
                                               const float *__restrict__ ascale, int nj, uint32_t jb, uint32_t i,
                                               float xi, float yi, float zi, float xil, float yil, float zil, float wis,
                                               float qcap, uint32_t cnt_s, const uint32_t *__restrict__ jidx = nullptr)
{
    uint32_t slowbits = 0;
    if (nj == 32) {
        constexpr bool kFull = MODE == MODE_THETA && !NEED_AVG;
        constexpr int kGroup = kFull ? CF_PAIR_GROUP : (NEED_AVG ? 4 : CF_PAIR_GROUP);
        constexpr int kUnroll = kFull ? 32 / CF_PAIR_GROUP : (NEED_AVG ? 2 : kR3Unroll);
#pragma unroll kUnroll
        for (int k0 = 0; k0 < 32; k0 += kGroup)
            pairs_group8<MODE, NEED_AVG, NEED_W, OWN, SER, kGroup>(A, sjhi, sjlo, lut_add, ascale, k0, jb, i, xi, yi, zi,
                                                                   xil, yil, zil, wis, qcap, cnt_s, slowbits, jidx);
    } else {
        // a partial tile, padded to a multiple of 4 points
        for (int k = 0; k < nj; k += 4)
            pairs_group8<MODE, NEED_AVG, NEED_W, OWN, SER, 4>(A, sjhi, sjlo, lut_add, ascale, k, jb, i, xi, yi, zi, xil,
                                                              yil, zil, wis, qcap, cnt_s, slowbits, jidx);
    }
    return slowbits;
}

template <int MODE, bool NEED_AVG, bool NEED_W, bool OWN, bool SER>
__device__ __forceinline__ uint32_t tile_fast(const PairArgs &A, const float4 *__restrict__ sjhi,
                                              const float4 *__restrict__ sjlo, const uint32_t *__restrict__ lut,
                                              const float *__restrict__ ascale, int nj,
                                              uint32_t jb, uint32_t i, float xi, float yi, float zi, float xil, float yil,
                                              float zil, float wis, float ax, float ay, float az, uint32_t cnt_s,
                                              const uint32_t *__restrict__ jidx = nullptr)
{
    uint32_t slowbits = 0;
    if (nj == 32) {
        // group size (pairs whose table offsets are computed before their reductions) and
        // groups per unrolled loop body, per mode
        constexpr bool kMock = mode_is_mock(MODE);
        constexpr bool kFull = MODE == MODE_THETA && !NEED_AVG;
        constexpr int kGroup = kMock ? CF_MOCK_GROUP
                               : kFull ? CF_PAIR_GROUP
                               : MODE == MODE_R3 ? (NEED_AVG ? 4 : CF_PAIR_GROUP) : CF_2D_GROUP;
        constexpr int kUnroll = kMock ? kMockUnroll
                                : kFull ? 32 / CF_PAIR_GROUP
                                : MODE == MODE_R3 ? (NEED_AVG ? 2 : kR3Unroll) : CF_2D_UNROLL;
#pragma unroll kUnroll
        for (int k0 = 0; k0 < 32; k0 += kGroup)
            pairs_group<MODE, NEED_AVG, NEED_W, OWN, SER, kGroup>(A, sjhi, sjlo, lut, ascale, k0, jb, i, xi, yi, zi, xil,
                                                                  yil, zil, wis, ax, ay, az, cnt_s, slowbits, jidx);
    } else {
        for (int k = 0; k < nj; k++)
            pairs_group<MODE, NEED_AVG, NEED_W, OWN, SER, 1>(A, sjhi, sjlo, lut, ascale, k, jb, i, xi, yi, zi, xil, yil, zil, wis,
                                                        ax, ay, az, cnt_s, slowbits, jidx);
    }
    return slowbits;
}

// Dense FP64 re-evaluation of up to 32 queued pairs (one per lane).
// (col_base >= 0: every pair goes to the column of its own i point, r.i - col_base, instead of the
// processing lane's column hl -- counts whose lanes belong to different catalogues)
template <int MODE, bool NEED_AVG, bool NEED_W>
__device__ __noinline__ void refine_batch(const PairArgs &A, const double *se, const RefineEntry *q, int count,
                                          WarpHist h, int hl, int lane, int col_base = -1)
{
    if (lane < count) {
        const RefineEntry r = q[lane];
        if (col_base >= 0) hl = (int)(r.i - (uint32_t)col_base);
        const int mx = (int)((r.meta >> 8) & 3u) - 1, my = (int)((r.meta >> 10) & 3u) - 1,
                  mz = (int)((r.meta >> 12) & 3u) - 1;
        double davg = 0.0, dw = 0.0;
        const int bin = refine_pair<MODE>(A, se, r.i, r.j, mx, my, mz, &davg, &dw);
        if (bin >= 0) accumulate<NEED_AVG, NEED_W>(A, h, bin, bin * h.ls + hl, davg, dw);
    }
    __syncwarp();
}

// Exact FP32 classification of up to 32 queued pairs in flagged buckets (one per lane; the pairs
// come from any lane and tile of the warp, so a warp spends one pass per 32 such pairs instead of
// one pass per flagged pair of its busiest lane).  Both points are re-read from the lattice
// arrays, which the warp touched a moment ago.  Pairs inside an error band move on to the FP64
// queue.
template <int MODE, bool NEED_AVG, bool NEED_W, bool LUT8>
__device__ __noinline__ void slow_batch(const PairArgs &A, const double *se, const float *glo, const float *ghi,
                                        const RefineEntry *sq, int count, RefineEntry *rq, int *rq_count, WarpHist h,
                                        int hl, int lane, unsigned long long *refined, int col_base = -1)
{
    const int hl0 = hl;
    if (lane < count) {
        const RefineEntry e = sq[lane];
        if (col_base >= 0) hl = (int)(e.i - (uint32_t)col_base);
        const int mx = (int)((e.meta >> 8) & 3u) - 1, my = (int)((e.meta >> 10) & 3u) - 1,
                  mz = (int)((e.meta >> 12) & 3u) - 1;
        const float4 pi = A.hi1[e.i];
        const float4 pj = A.hi2[e.j];
        const float xi = pi.x - A.ohi[0][mx + 1], yi = pi.y - A.ohi[1][my + 1], zi = pi.z - A.ohi[2][mz + 1];
        float xil = 0.f, yil = 0.f, zil = 0.f;
        float4 pjl = make_float4(0.f, 0.f, 0.f, 0.f);
        if (NEED_AVG || mode_is_mock(MODE)) {
            const float4 pl = A.lo1[e.i];
            xil = pl.x - A.olo[0][mx + 1];
            yil = pl.y - A.olo[1][my + 1];
            zil = pl.z - A.olo[2][mz + 1];
            pjl = A.lo2[e.j];
        }
        const float ax = xi + xil, ay = yi + yil, az = zi + zil;
        float favg = 0.f, fw = 0.f;
        const int bin = slow_candidate<MODE, NEED_AVG, NEED_W, LUT8>(A, glo, ghi, pj, pjl, xi, yi, zi, xil, yil, zil,
                                                                     pi.w, ax, ay, az, &favg, &fw);
        if (bin >= 0) {
            accumulate<NEED_AVG, NEED_W>(A, h, bin, bin * h.ls + hl, (double)favg, (double)fw);
        } else if (bin == -2) {
            const int pos = atomicAdd(rq_count, 1);
            rq[pos] = e;
            (*refined)++;
        }
    }
    __syncwarp();
    const int cnt = *rq_count;
    if (cnt >= 32) {
        refine_batch<MODE, NEED_AVG, NEED_W>(A, se, rq + (cnt - 32), 32, h, hl0, lane, col_base);
        if (lane == 0) *rq_count = cnt - 32;
        __syncwarp();
    }
}

template <int MODE, bool NEED_AVG, bool NEED_W, bool LUT8, bool PACKED>
__global__ void __launch_bounds__(pair_max_threads(MODE, NEED_AVG, NEED_W), CF_PAIR_MIN_BLOCKS)
    k_pairs_f32(PairArgs A, SmemLayout SL)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *se = (double *)(smem + SL.edges_off);
    float *glo = (float *)(smem + SL.guard_off);
    float *ghi = glo + A.nedges;
    uint32_t *lut = (uint32_t *)(smem + SL.lut_off);
    float *asc = (float *)(smem + SL.ascale_off);
    for (int k = threadIdx.x; k < A.nedges; k += blockDim.x) {
        se[k] = A.g_edges[k];
        glo[k] = A.g_guard[k];
        ghi[k] = A.g_guard[A.nedges + k];
        asc[k] = A.g_ascale[k];
    }
    // the scale entries after the last edge serve the trash rows of the byte table (index
    // nbins = nedges, and nedges + 1 for flagged entries of the last row)
    if (threadIdx.x < 2) asc[A.nedges + threadIdx.x] = 0.f;
    for (int k = threadIdx.x; k <= SL.lut_n; k += blockDim.x) lut[k] = A.g_lut[k];
    // byte table: entry address = mad.hi(bits(q'), 2^(32 - shift), lut_add)
    const uint32_t lut_add = (uint32_t)__cvta_generic_to_shared(lut) - A.lut8_base;
    // byte table: lanes 16-31 clamp to a cap bucket of their own whose entry is the second trash
    // row, so that a rejected pair of lane l and one of lane l + 16 (which share a histogram
    // column below lane stride 32) do not reduce into the same word
    // (plain counts, which run with private columns, keep the one cap: a register less)
    const float qcap_l = (NEED_AVG || NEED_W) && lane >= 16 ? A.q_cap2 : A.q_cap;
    float4 *sjhi = (float4 *)(smem + SL.stage_off + SL.per_warp_stage * warp);
    float4 *sjlo = sjhi + 32;
    RefineEntry *rq = (RefineEntry *)(sjlo + 32);
    RefineEntry *sq = rq + kRefineQueue;
    int *rq_count = (int *)(sq + kSlowQueue);
    // pairs queued for the slow path and pairs evaluated by the warp (bytes 4-7 and 8-15 of the 16
    // after the queue fill: kept off registers)
    uint32_t *qd_s = (uint32_t *)((unsigned char *)rq_count + 4);
    unsigned long long *ev_s = (unsigned long long *)((unsigned char *)rq_count + 8);
    uint32_t *sidx = (uint32_t *)((unsigned char *)rq_count + 16);  // packed tasks: staged j points'
    uint8_t *simg = (uint8_t *)(sidx + 32);                          // lattice indices and image codes
    float4 *sbox = (float4 *)(simg + 32);  // pruned tiles: the chunk's box (lo, prune radius^2), (hi, -)
    // box pruning: the unpacked byte-table kernels (DD(r), xi, DDtheta), DDrppi / wp / DDsmu and
    // the survey modes
    constexpr bool kPrune = !PACKED && (LUT8 || MODE == MODE_RPPI || MODE == MODE_WP || MODE == MODE_SMU ||
                                        mode_is_mock(MODE));
    // periodic shift of a j point by image code (bits 0-5 as Task::meta bits 8-13)
    float4 *shift_hi = (float4 *)(smem + SL.shift_off), *shift_lo = shift_hi + 64;
    if constexpr (PACKED) {
        for (int k = threadIdx.x; k < 64; k += blockDim.x) {
            const int c0 = k & 3, c1 = (k >> 2) & 3, c2 = (k >> 4) & 3;
            shift_hi[k] = make_float4(c0 < 3 ? A.ohi[0][c0] : 0.f, c1 < 3 ? A.ohi[1][c1] : 0.f,
                                      c2 < 3 ? A.ohi[2][c2] : 0.f, 0.f);
            shift_lo[k] = make_float4(c0 < 3 ? A.olo[0][c0] : 0.f, c1 < 3 ? A.olo[1][c1] : 0.f,
                                      c2 < 3 ? A.olo[2][c2] : 0.f, 0.f);
        }
    }
    int sq_n = 0;  // warp-uniform fill of the slow queue (always < 32 between tiles)
    WarpHist h = warp_hist(smem, SL, warp);
    zero_hist(h, SL, lane);
    if (lane == 0) {
        *rq_count = 0;
        *qd_s = 0u;
        *ev_s = 0ull;
    }
    const int hl = lane & (SL.lane_stride - 1);
    // shared-window address of this lane's entry in row 0; a pair's table entry is its row offset
    const uint32_t cnt_s = (uint32_t)__cvta_generic_to_shared(h.e) + 4u * h.ew * hl;
    __syncthreads();
    unsigned long long refined = 0;
    // unpacked kernels count in registers; packed ones (tighter on registers) in shared memory
    unsigned long long evaluated = 0, queued = 0;
    const uint32_t ntasks = A.ntask_dev ? min(*A.ntask_dev, A.ntasks) : A.ntasks;
    uint32_t cur_cat = 0;  // catalogue whose counts the warp's histogram holds (batched counts)
    // terms a column may have taken since the last flush: per tile 32 fast-path pairs per lane
    // sharing the column, plus at most 32 slow-queue and 32 FP64 terms
    uint32_t col_terms = 0;
    const uint32_t tile_terms = 32u * (32u / (uint32_t)SL.lane_stride) + 64u;

    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(A.task_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) break;
        const Task T = A.tasks[t];
        const long long t_start = A.task_clock ? clock64() : 0;
        const uint32_t cat = T.meta >> kCatShift;
        if (cat != cur_cat) {
            // queued pairs belong to the previous catalogue: settle them, then hand over
            __syncwarp();
            if (sq_n > 0) {
                slow_batch<MODE, NEED_AVG, NEED_W, LUT8>(A, se, glo, ghi, sq, sq_n, rq, rq_count, h, hl, lane, &refined);
                sq_n = 0;
            }
            const int rest = *rq_count;
            if (rest > 0) {
                refine_batch<MODE, NEED_AVG, NEED_W>(A, se, rq, rest, h, hl, lane);
                if (lane == 0) *rq_count = 0;
                __syncwarp();
            }
            flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat);
            cur_cat = cat;
            col_terms = 0;
        }
        const int icount = (int)(T.meta & 63u) + 1;
        const int mx = (int)((T.meta >> 8) & 3u) - 1, my = (int)((T.meta >> 10) & 3u) - 1,
                  mz = (int)((T.meta >> 12) & 3u) - 1;
        const bool own = (T.meta >> 16) & 1u;
        const uint32_t i = T.i_begin + lane;
        const bool ivalid = lane < icount;
        const float4 pi = ivalid ? A.hi1[i] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
        // j is shifted by the image offset o; equivalently shift i by -o (exact on the grid)
        const float xi = pi.x - A.ohi[0][mx + 1], yi = pi.y - A.ohi[1][my + 1], zi = pi.z - A.ohi[2][mz + 1];
        float xil = 0.f, yil = 0.f, zil = 0.f;
        constexpr bool kLo = NEED_AVG || mode_is_mock(MODE);  // survey modes always use the lo parts
        if (kLo) {
            const float4 pl = ivalid ? A.lo1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            xil = pl.x - A.olo[0][mx + 1];
            yil = pl.y - A.olo[1][my + 1];
            zil = pl.z - A.olo[2][mz + 1];
        }
        const float ax = xi + xil, ay = yi + yil, az = zi + zil;  // survey modes: the i point from the observer
        // j points: a contiguous lattice range, or (packed task) list positions of the chunk's
        // concatenated ranges, each range with its own periodic image applied to its j points
        const bool packed = PACKED && (T.meta & kTaskPacked) != 0;
        const uint32_t jbeg = packed ? (T.j_end >> 11) * kJMax : T.j_begin;
        const uint32_t jend = packed ? jbeg + (T.j_end & 2047u) + 1u : T.j_end;
        if constexpr (PACKED) {
            if (lane == 0) *ev_s += (unsigned long long)icount * (jend - jbeg);
        } else if constexpr (!kPrune) {
            evaluated += (unsigned long long)icount * (jend - jbeg);  // pruned tasks count per tile
        }
        const bool shifted = packed && (T.meta & kTaskImages) != 0;
        uint32_t jrc = T.j_begin;  // packed: the record holding list position jb
        // Box pruning (unpacked kernels of every mode but vpf): a j point farther than the prune
        // radius (the top edge's separation, or the survey modes' separation cut, plus the
        // coordinate error bounds) from the chunk's bounding box pairs with none of its points in
        // range, so it is never staged (DDrppi / wp also drop a j point whose z distance to the
        // box reaches the pi rejection bound); the points kept fill whole tiles across the
        // task's candidates.
        constexpr bool prune = kPrune;
        if constexpr (prune) {
            // the box of the valid lanes' (image-shifted) points, by order-preserving integer keys
            auto key = [](float v) { const int b = __float_as_int(v); return b ^ ((b >> 31) & 0x7fffffff); };
            auto val = [](int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); };
            const int big = 0x7f800000, small = (int)0x80800000;  // keys of +inf, -inf
            const float bxl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(xi) : big));
            const float byl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(yi) : big));
            const float bzl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(zi) : big));
            const float bxh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(xi) : small));
            const float byh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(yi) : small));
            const float bzh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(zi) : small));
            if (lane == 0) {
                sbox[0] = make_float4(bxl, byl, bzl, A.prune_r2);
                sbox[1] = make_float4(bxh, byh, bzh, A.prune_z);
            }
            __syncwarp();
        }
        for (uint32_t jb = jbeg; jb < jend;) {
            const uint32_t tile_j0 = jb;  // unpruned: the tile's first j point
            int nj = (int)min(32u, jend - jb);
            if constexpr (prune) {
                // rounds of 32 candidates until 32 points are staged or the range ends; a round
                // that overfills the stage takes its first kept points and the next round starts
                // after the last one taken
                const float4 b0 = sbox[0], b1 = sbox[1];
                float *S = (float *)sjhi, *SL8 = (float *)sjlo;
                int f = 0;
                while (f < 32 && jb < jend) {
                    const uint32_t nc = min(32u, jend - jb);
                    float4 p = make_float4(0.f, 0.f, 0.f, 0.f), pl = p;
                    bool keep = false;
                    if ((uint32_t)lane < nc) {
                        p = A.hi2[jb + lane];
                        const float dx = fmaxf(0.f, fmaxf(b0.x - p.x, p.x - b1.x));
                        const float dy = fmaxf(0.f, fmaxf(b0.y - p.y, p.y - b1.y));
                        const float dz = fmaxf(0.f, fmaxf(b0.z - p.z, p.z - b1.z));
                        // DDrppi / wp: rp from the box's xy rectangle and |dz| against the pi bound
                        keep = (MODE == MODE_RPPI || MODE == MODE_WP)
                                   ? fmaf(dy, dy, dx * dx) <= b0.w && dz < b1.w
                                   : fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= b0.w;
                        if (kLo && keep) pl = A.lo2[jb + lane];
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, keep);
                    const int room = 32 - f;
                    const int rank = __popc(m & ((1u << lane) - 1u));
                    const uint32_t taken = __ballot_sync(0xffffffffu, keep && rank < room);
                    if (keep && rank < room) {
                        const int pos = f + rank;
                        if constexpr (LUT8) {
                            S[pos] = p.x;
                            S[32 + pos] = p.y;
                            S[64 + pos] = p.z;
                            if (NEED_W) S[96 + pos] = p.w;
                            if (kLo) {
                                SL8[pos] = pl.x;
                                SL8[32 + pos] = pl.y;
                                SL8[64 + pos] = pl.z;
                            }
                        } else {
                            sjhi[pos] = p;
                            if (kLo) sjlo[pos] = pl;
                        }
                        sidx[pos] = jb + (uint32_t)lane;
                    }
                    const int nt = __popc(taken);
                    jb += (uint32_t)__popc(m) <= (uint32_t)room ? nc : (uint32_t)(32 - __clz(taken));
                    f += nt;
                }
                nj = f;
                if (nj == 0) break;  // no candidate left in reach
                evaluated += (unsigned long long)icount * (uint32_t)nj;
                // a partial tile is padded (far-away points: the reject entry) to 32 above kPadMin
                // and (byte table) to a multiple of 4 otherwise; the other tables pair a tile of
                // kPadMin points or fewer point by point
                const int njp = nj > kPadMin ? 32 : LUT8 ? ((nj + 3) & ~3) : nj;
                if (lane >= nj && lane < njp) {
                    if constexpr (LUT8) {
                        S[lane] = -1e30f;
                        S[32 + lane] = -1e30f;
                        S[64 + lane] = -1e30f;
                        if (NEED_W) S[96 + lane] = 0.f;
                        if (kLo) SL8[lane] = SL8[32 + lane] = SL8[64 + lane] = 0.f;
                    } else {
                        sjhi[lane] = make_float4(-1e30f, -1e30f, -1e30f, 0.f);
                        if (kLo) sjlo[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                }
                nj = njp;
            } else {
            uint32_t jx = jb + (uint32_t)lane, jimg = 0;  // this lane's j point (unpacked)
            if (packed) {
                // records jrc .. jrc + 31 (one per lane, cut after the chunk's last record): the
                // ranges that start inside the tile set their bit, and a lane's record is the
                // number of those starting at or before its position
                const JRange rec = A.jrec[jrc + lane];
                const uint32_t lastm = __ballot_sync(0xffffffffu, (rec.z >> 31) != 0u);
                const int nval = lastm ? __ffs(lastm) : 32;
                const uint32_t rel = rec.y - jb;
                const uint32_t bit = (lane > 0 && lane < nval && rel - 1u < 31u) ? (1u << rel) : 0u;
                const uint32_t starts = __reduce_or_sync(0xffffffffu, bit);
                const int rl = __popc(starts & (0xffffffffu >> (31 - lane)));
                const uint32_t j0 = __shfl_sync(0xffffffffu, rec.x, rl), p0 = __shfl_sync(0xffffffffu, rec.y, rl);
                jimg = __shfl_sync(0xffffffffu, rec.z, rl) & 63u;
                jx = j0 + (jb + (uint32_t)lane - p0);
                // the next tile starts in the record holding position jb + 31, or in the one after
                const int r31 = __shfl_sync(0xffffffffu, rl, 31);
                const uint32_t e31 = __shfl_sync(0xffffffffu, rec.w, r31);
                jrc += (uint32_t)r31 + (e31 == jb + 32u ? 1u : 0u);
            }
            if constexpr (PACKED) {
                // far-away padding: q overflows to +inf (the reject bucket, zero weight) against valid i
                // points and against the +1e30 stand-in of lanes without an i point alike
                float4 p = make_float4(-1e30f, -1e30f, -1e30f, 0.f), pl = make_float4(0.f, 0.f, 0.f, 0.f);
                if (lane < nj) {
                    p = A.hi2[jx];
                    if (kLo) pl = A.lo2[jx];
                    if (shifted) {
                        // j + o for image o (exact on the grid, as i - o is)
                        const float4 sh = shift_hi[jimg];
                        p.x += sh.x;
                        p.y += sh.y;
                        p.z += sh.z;
                        if (kLo) {
                            const float4 sl = shift_lo[jimg];
                            pl.x += sl.x;
                            pl.y += sl.y;
                            pl.z += sl.z;
                        }
                    }
                }
                if (packed) {
                    sidx[lane] = jx;
                    simg[lane] = (uint8_t)jimg;
                }
                if constexpr (LUT8) {
                    // byte table: the stage holds x[32] | y[32] | z[32] | w[32] (and the lo parts
                    // x[32] | y[32] | z[32]) so that one 16-byte shared load broadcasts a coordinate of
                    // four j points; a partial tile is padded to 32 points above kPadMin and to a
                    // multiple of 4 otherwise, with far-away points (q' = cap: the reject entry)
                    const int njp = nj > kPadMin ? 32 : ((nj + 3) & ~3);
                    float *S = (float *)sjhi, *SL8 = (float *)sjlo;
                    if (lane < njp) {
                        S[lane] = p.x;
                        S[32 + lane] = p.y;
                        S[64 + lane] = p.z;
                        if (NEED_W) S[96 + lane] = p.w;
                        if (kLo) {
                            SL8[lane] = pl.x;
                            SL8[32 + lane] = pl.y;
                            SL8[64 + lane] = pl.z;
                        }
                    }
                    nj = njp;
                } else {
                    // a partial tile above kPadMin runs fully unrolled on its padding
                    if (lane < nj || nj > kPadMin) {
                        sjhi[lane] = p;
                        if (kLo) sjlo[lane] = pl;
                    }
                    if (nj > kPadMin) nj = 32;
                }
            } else {
                if constexpr (LUT8) {
                    // byte table: the stage holds x[32] | y[32] | z[32] | w[32] (and the lo parts
                    // x[32] | y[32] | z[32]) so that one 16-byte shared load broadcasts a coordinate of
                    // four j points; a partial tile is padded to 32 points above kPadMin and to a
                    // multiple of 4 otherwise, with far-away points (q' = cap: the reject entry)
                    const int njp = nj > kPadMin ? 32 : ((nj + 3) & ~3);
                    float *S = (float *)sjhi, *SL8 = (float *)sjlo;
                    if (lane < njp) {
                        float4 p = make_float4(-1e30f, -1e30f, -1e30f, 0.f), pl = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (lane < nj) {
                            p = A.hi2[jb + lane];
                            if (kLo) pl = A.lo2[jb + lane];
                        }
                        S[lane] = p.x;
                        S[32 + lane] = p.y;
                        S[64 + lane] = p.z;
                        if (NEED_W) S[96 + lane] = p.w;
                        if (kLo) {
                            SL8[lane] = pl.x;
                            SL8[32 + lane] = pl.y;
                            SL8[64 + lane] = pl.z;
                        }
                    }
                    nj = njp;
                } else {
                    if (lane < nj) {
                        sjhi[lane] = A.hi2[jb + lane];
                        if (kLo) sjlo[lane] = A.lo2[jb + lane];
                    } else if (nj > kPadMin) {
                        // pad a partial tile with far-away points and run it fully unrolled: q overflows
                        // to +inf (the reject bucket, zero weight) against valid i points and against the
                        // +1e30 stand-in of lanes without an i point alike
                        sjhi[lane] = make_float4(-1e30f, -1e30f, -1e30f, 0.f);
                        if (kLo) sjlo[lane] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    if (nj > kPadMin) nj = 32;
                }
            }
            jb += 32;
            }
            __syncwarp();
            const float wi_s = pi.w * A.w_scale_f;
            uint32_t slowbits;
            if constexpr (LUT8) {
                // byte table: pair k of nj ends at bit 32 - nj + k (shifted into bit 0 of k = 0 below)
                if (MODE == MODE_THETA && NEED_AVG && A.theta_series) {
                    slowbits = own ? tile_fast8<MODE, NEED_AVG, NEED_W, true, true>(A, sjhi, sjlo, lut_add, h.ascale, nj,
                                                                                  tile_j0, i, xi, yi, zi, xil, yil, zil, wi_s, qcap_l,
                                                                                  cnt_s, prune ? sidx : nullptr)
                                   : tile_fast8<MODE, NEED_AVG, NEED_W, false, true>(A, sjhi, sjlo, lut_add, h.ascale,
                                                                                   nj, tile_j0, i, xi, yi, zi, xil, yil, zil,
                                                                                   wi_s, qcap_l, cnt_s);
                } else {
                    slowbits = own ? tile_fast8<MODE, NEED_AVG, NEED_W, true, false>(A, sjhi, sjlo, lut_add, h.ascale,
                                                                                   nj, tile_j0, i, xi, yi, zi, xil, yil, zil,
                                                                                   wi_s, qcap_l, cnt_s, prune ? sidx : nullptr)
                                   : tile_fast8<MODE, NEED_AVG, NEED_W, false, false>(A, sjhi, sjlo, lut_add, h.ascale,
                                                                                    nj, tile_j0, i, xi, yi, zi, xil, yil, zil,
                                                                                    wi_s, qcap_l, cnt_s);
                }
                slowbits >>= 32 - nj;  // pair k at bit k
            } else if (MODE == MODE_THETA && NEED_AVG && A.theta_series) {
                // angular averages by the arcsine series: a separate copy of the unrolled tile loop
                slowbits = own ? tile_fast<MODE, NEED_AVG, NEED_W, true, true>(A, sjhi, sjlo, lut, h.ascale, nj, tile_j0, i, xi,
                                                                             yi, zi, xil, yil, zil, wi_s, ax, ay, az, cnt_s,
                                                                             prune ? sidx : nullptr)
                               : tile_fast<MODE, NEED_AVG, NEED_W, false, true>(A, sjhi, sjlo, lut, h.ascale, nj, tile_j0, i, xi,
                                                                              yi, zi, xil, yil, zil, wi_s, ax, ay, az, cnt_s);
            } else {
                slowbits = own ? tile_fast<MODE, NEED_AVG, NEED_W, true, false>(A, sjhi, sjlo, lut, h.ascale, nj, tile_j0, i, xi,
                                                                              yi, zi, xil, yil, zil, wi_s, ax, ay, az, cnt_s,
                                                                              prune ? sidx : nullptr)
                               : tile_fast<MODE, NEED_AVG, NEED_W, false, false>(A, sjhi, sjlo, lut, h.ascale, nj, tile_j0, i, xi,
                                                                               yi, zi, xil, yil, zil, wi_s, ax, ay, az, cnt_s);
            }
            // candidates in flagged buckets go to the warp's slow queue, one bit per lane per round
            // (a round appends at most 32 entries, so the queue never holds more than 63)
            while (true) {
                const uint32_t want = __ballot_sync(0xffffffffu, slowbits != 0);
                if (!want) break;
                if (slowbits) {
                    const int b = (int)(__float_as_uint(__uint2float_rz(slowbits)) >> 23) - 127;
                    slowbits ^= 1u << b;
                    const int k = LUT8 ? b : nj - 1 - b;  // bit k (byte table) or n - 1 - k holds pair k
                    RefineEntry r;
                    r.i = i;
                    r.j = (packed || prune) ? sidx[k] : tile_j0 + (uint32_t)k;
                    r.meta = packed ? (T.meta & ~0x3f00u) | ((uint32_t)simg[k] << 8) : T.meta;
                    sq[sq_n + __popc(want & ((1u << lane) - 1u))] = r;
                }
                sq_n += __popc(want);
                if constexpr (PACKED) {
                    if (lane == 0) {
                        const uint32_t qd = *qd_s + (uint32_t)__popc(want);
                        if (qd >= 0x80000000u) atomicAdd(&A.g_stats[2], (unsigned long long)qd);
                        *qd_s = qd >= 0x80000000u ? 0u : qd;
                    }
                } else {
                    queued += __popc(want);
                }
                __syncwarp();
                if (sq_n >= 32) {
                    slow_batch<MODE, NEED_AVG, NEED_W, LUT8>(A, se, glo, ghi, sq + (sq_n - 32), 32, rq, rq_count, h, hl,
                                                       lane, &refined);
                    sq_n -= 32;
                }
            }
            __syncwarp();
            col_terms += tile_terms;
            if (col_terms + tile_terms > (uint32_t)kColumnTerms) {
                flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat);
                col_terms = 0;
            }
        }
        if (A.task_clock && lane == 0) {
            A.task_clock[2 * (size_t)t] = (unsigned long long)(clock64() - t_start);
            A.task_clock[2 * (size_t)t + 1] = (blockIdx.x * (blockDim.x >> 5)) + warp;
        }
    }
    __syncwarp();
    if (sq_n > 0) slow_batch<MODE, NEED_AVG, NEED_W, LUT8>(A, se, glo, ghi, sq, sq_n, rq, rq_count, h, hl, lane, &refined);
    const int rest = *rq_count;
    if (rest > 0) refine_batch<MODE, NEED_AVG, NEED_W>(A, se, rq, rest, h, hl, lane);
    flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat);
    for (int off = 16; off; off >>= 1) refined += __shfl_down_sync(0xffffffffu, refined, off);
    if (lane == 0) {
        atomicAdd(&A.g_stats[0], evaluated + *ev_s);
        atomicAdd(&A.g_stats[1], refined);
        atomicAdd(&A.g_stats[2], queued + (unsigned long long)*qd_s);
    }
}

// Flush of a warp histogram whose lanes count for different catalogues (private columns, lane
// stride 32): lane l moves its own column into catalogue cat's sums and zeroes it.
template <bool NEED_AVG, bool NEED_W>
__device__ __forceinline__ void flush_lanes(const PairArgs &A, WarpHist h, int lane, uint32_t cat)
{
    __syncwarp();
    unsigned long long *g_cnt = A.g_cnt + (size_t)cat * A.nbins;
    double *g_avg = A.g_avg + (size_t)cat * A.nbins;
    double *g_w = A.g_w + (size_t)cat * A.nbins;
    for (int b = 0; b < A.nbins; b++) {
        uint32_t *e = h.e + (size_t)(b * 32 + lane) * h.ew;
        const uint32_t c = e[0];
        if (c == 0) continue;  // no pair, so no sums either
        e[0] = 0;
        atomicAdd(&g_cnt[b], (unsigned long long)c);
        if (NEED_AVG) {
            uint32_t *s = e + avg_word<NEED_AVG>();
            const long long va = (long long)(int)s[0] * 65536ll + (long long)s[1];
            s[0] = 0;
            s[1] = 0;
            if (va) atomicAdd(&g_avg[b], (double)va / (double)h.ascale[b / A.rbin_div]);
        }
        if (NEED_W) {
            uint32_t *s = e + w_word<NEED_AVG>();
            const long long vw = (long long)(int)s[0] * 65536ll + (long long)s[1];
            s[0] = 0;
            s[1] = 0;
            const double v = (double)vw * A.w_unscale;
            if (v != 0.0) atomicAdd(&g_w[b], v);
        }
    }
    __syncwarp();
}

// Batched cross-correlations on one merged set-1 lattice (every catalogue's points sorted
// together by cell; ro1[i].x holds the catalogue of point i): a warp takes one chunk -- 32
// consecutive points of a column, from any catalogues -- and walks its neighbour columns itself
// (the ranges chunk_col_tasks would list), so the chunk's lanes keep their points, and with them
// their catalogues, until the chunk is done.  Every lane owns a histogram column (lane stride 32)
// that it flushes into its catalogue's sums.  Byte-table DD(r) only.
template <bool NEED_AVG, bool NEED_W, bool SINGLE>
__global__ void __launch_bounds__(pair_max_threads(MODE_R3, NEED_AVG, NEED_W), CF_PAIR_MIN_BLOCKS)
    k_pairs_chunks(PairArgs A, SmemLayout SL, TaskGeom G, const uint32_t *chunk_begin, const uint2 *chunk_info,
                   const uint32_t *cs2, uint32_t nchunk)
{
    constexpr int MODE = MODE_R3;
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *se = (double *)(smem + SL.edges_off);
    float *glo = (float *)(smem + SL.guard_off);
    float *ghi = glo + A.nedges;
    uint32_t *lut = (uint32_t *)(smem + SL.lut_off);
    float *asc = (float *)(smem + SL.ascale_off);
    for (int k = threadIdx.x; k < A.nedges; k += blockDim.x) {
        se[k] = A.g_edges[k];
        glo[k] = A.g_guard[k];
        ghi[k] = A.g_guard[A.nedges + k];
        asc[k] = A.g_ascale[k];
    }
    if (threadIdx.x < 2) asc[A.nedges + threadIdx.x] = 0.f;
    for (int k = threadIdx.x; k <= SL.lut_n; k += blockDim.x) lut[k] = A.g_lut[k];
    const uint32_t lut_add = (uint32_t)__cvta_generic_to_shared(lut) - A.lut8_base;
    float4 *sjhi = (float4 *)(smem + SL.stage_off + SL.per_warp_stage * warp);
    float4 *sjlo = sjhi + 32;
    RefineEntry *rq = (RefineEntry *)(sjlo + 32);
    RefineEntry *sq = rq + kRefineQueue;
    int *rq_count = (int *)(sq + kSlowQueue);
    uint32_t *sidx = (uint32_t *)((unsigned char *)rq_count + 16);  // staged j points' lattice indices,
    uint8_t *simg = (uint8_t *)(sidx + 32);                          // image codes
    float4 *sbox = (float4 *)(simg + 32);                            // and the chunk's box
    int sq_n = 0;
    WarpHist h = warp_hist(smem, SL, warp);
    zero_hist(h, SL, lane);
    if (lane == 0) *rq_count = 0;
    // batches: lane stride 32 (private columns of the lanes' catalogues); one count: any stride
    const int hl = SINGLE ? lane & (SL.lane_stride - 1) : lane;
    const uint32_t cnt_s = (uint32_t)__cvta_generic_to_shared(h.e) + 4u * h.ew * hl;
    __syncthreads();
    uint64_t evaluated = 0;
    unsigned long long refined = 0, queued = 0;
    uint32_t col_terms = 0;
    const uint32_t tile_terms = 32u + 64u;
    const int nyc = 2 * G.reach_y + 1, ncoff = (2 * G.reach_x + 1) * nyc;
    const int nz = G.nz;

    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(A.task_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= nchunk) break;
        const uint2 info = chunk_info[t];
        const int icount = (int)(info.x & 63u);
        if (icount == 0) continue;
        const uint32_t ib = chunk_begin[t];
        const uint32_t i = ib + lane;
        const bool ivalid = lane < icount;
        const float4 pi = ivalid ? A.hi1[i] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
        float4 pl = make_float4(0.f, 0.f, 0.f, 0.f);
        if (NEED_AVG && ivalid) pl = A.lo1[i];
        const uint32_t cat = (!SINGLE && ivalid) ? (uint32_t)A.ro1[i].x : 0u;
        const float wi_s = pi.w * A.w_scale_f;
        const int a = (int)((info.x >> 6) & 4095u), b = (int)((info.x >> 18) & 4095u);
        const int col = (int)info.y, ix = col / G.ny, iy = col % G.ny;
        // Box pruning: a j point farther than the prune radius from the chunk's bounding box pairs
        // with none of its points in range and is never staged.  Staged points carry their
        // range's periodic image (j + o, exact on the grid as i - o is), so the points kept from
        // every neighbour column and image fill whole tiles against the unshifted i points.
        {
            auto key = [](float v) { const int bk = __float_as_int(v); return bk ^ ((bk >> 31) & 0x7fffffff); };
            auto val = [](int k) { return __int_as_float(k ^ ((k >> 31) & 0x7fffffff)); };
            const int big = 0x7f800000, small = (int)0x80800000;  // keys of +inf, -inf
            const float bxl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(pi.x) : big));
            const float byl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(pi.y) : big));
            const float bzl = val(__reduce_min_sync(0xffffffffu, ivalid ? key(pi.z) : big));
            const float bxh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(pi.x) : small));
            const float byh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(pi.y) : small));
            const float bzh = val(__reduce_max_sync(0xffffffffu, ivalid ? key(pi.z) : small));
            if (lane == 0) {
                sbox[0] = make_float4(bxl, byl, bzl, A.prune_r2);
                sbox[1] = make_float4(bxh, byh, bzh, 0.f);
            }
            __syncwarp();
        }
        const float xi = pi.x, yi = pi.y, zi = pi.z;
        const float xil = pl.x, yil = pl.y, zil = pl.z;
        float *S = (float *)sjhi, *SL8 = (float *)sjlo;
        int f = 0;  // points staged
        const float qcap_l = (NEED_AVG || NEED_W) && SINGLE && SL.lane_stride < 32 && lane >= 16 ? A.q_cap2 : A.q_cap;
        // one tile of the staged points (njp: 32, or a partial tile's padded size); own: the own
        // column of an auto-correlation, which counts only j > i (by the staged point's index)
        auto run_tile = [&](int njp, bool own) {
            __syncwarp();
            uint32_t slowbits =
                own ? tile_fast8<MODE, NEED_AVG, NEED_W, true, false>(A, sjhi, sjlo, lut_add, h.ascale, njp, 0u, i, xi,
                                                                    yi, zi, xil, yil, zil, wi_s, qcap_l, cnt_s, sidx)
                    : tile_fast8<MODE, NEED_AVG, NEED_W, false, false>(A, sjhi, sjlo, lut_add, h.ascale, njp, 0u, i,
                                                                     xi, yi, zi, xil, yil, zil, wi_s, qcap_l, cnt_s);
            slowbits >>= 32 - njp;
            while (true) {
                const uint32_t want = __ballot_sync(0xffffffffu, slowbits != 0);
                if (!want) break;
                if (slowbits) {
                    const int bb = (int)(__float_as_uint(__uint2float_rz(slowbits)) >> 23) - 127;
                    slowbits ^= 1u << bb;
                    RefineEntry r;
                    r.i = i;
                    r.j = sidx[bb];
                    r.meta = (uint32_t)simg[bb] << 8;  // one i point per lane, the staged point's image
                    sq[sq_n + __popc(want & ((1u << lane) - 1u))] = r;
                }
                sq_n += __popc(want);
                queued += __popc(want);
                __syncwarp();
                if (sq_n >= 32) {
                    slow_batch<MODE, NEED_AVG, NEED_W, true>(A, se, glo, ghi, sq + (sq_n - 32), 32, rq, rq_count, h,
                                                             hl, lane, &refined, SINGLE ? -1 : (int)ib);
                    sq_n -= 32;
                }
            }
            __syncwarp();
            col_terms += tile_terms;
            if (col_terms + tile_terms > (uint32_t)kColumnTerms) {
                if constexpr (SINGLE) flush_hist<NEED_AVG, NEED_W>(A, h, lane, 0u);
                else flush_lanes<NEED_AVG, NEED_W>(A, h, lane, cat);
                col_terms = 0;
            }
        };
        // the staged points as a partial tile (padded with far-away points, the reject entry, to
        // 32 above kPadMin and to a multiple of 4 otherwise)
        auto run_partial = [&](bool own) {
            const int njp = f > kPadMin ? 32 : ((f + 3) & ~3);
            if (lane >= f && lane < njp) {
                S[lane] = -1e30f;
                S[32 + lane] = -1e30f;
                S[64 + lane] = -1e30f;
                if (NEED_W) S[96 + lane] = 0.f;
                if (NEED_AVG) SL8[lane] = SL8[32 + lane] = SL8[64 + lane] = 0.f;
                sidx[lane] = 0u;
            }
            run_tile(njp, own);
            f = 0;
        };
        const bool autocorr = SINGLE && A.autocorr;
        for (int c = 0; c < ncoff; c++) {
            const int dx = c / nyc - G.reach_x, dy = c % nyc - G.reach_y;
            if (autocorr && (dx < 0 || (dx == 0 && dy < 0))) continue;  // half stencil
            const bool own = autocorr && dx == 0 && dy == 0;           // forward half of the own column
            const int wz = G.ntab ? (int)G.wz_tab[c] : column_wz(G, dx, dy);
            if (wz < 0) continue;
            const int ux = ix + dx, uy = iy + dy;
            int mx = 0, cx = ux, my = 0, cy = uy;
            if (G.periodic[0]) {
                mx = floordiv(ux, G.nx);
                cx = ux - mx * G.nx;
            } else if (ux < 0 || ux >= G.nx) {
                continue;
            }
            if (G.periodic[1]) {
                my = floordiv(uy, G.ny);
                cy = uy - my * G.ny;
            } else if (uy < 0 || uy >= G.ny) {
                continue;
            }
            const int klo = own ? a : a - wz, khi = b + wz;
            const int mlo = G.periodic[2] ? floordiv(klo, nz) : 0, mhi = G.periodic[2] ? floordiv(khi, nz) : 0;
            if (mx < -1 || mx > 1 || my < -1 || my > 1 || mlo < -1 || mhi > 1) {
                if (G.error && lane == 0) atomicOr(G.error, 1u);
                continue;
            }
            const uint32_t *cs = cs2 + (uint32_t)(cx * G.ny + cy) * nz;
            for (int mz = mlo; mz <= mhi; mz++) {
                int s0 = klo - mz * nz, s1 = khi - mz * nz;
                s0 = s0 < 0 ? 0 : s0;
                s1 = s1 > nz - 1 ? nz - 1 : s1;
                if (s0 > s1) continue;
                // the own column's own image starts at the chunk's first point, in tiles of its own
                const bool ownr = own && mz == 0;
                const uint32_t jbeg = ownr ? ib : cs[s0], jend = cs[s1 + 1];
                if (jend <= jbeg) continue;
                if (ownr && f > 0) run_partial(false);
                // this range's periodic image, applied to its j points
                const float ox = A.ohi[0][mx + 1], oy = A.ohi[1][my + 1], oz = A.ohi[2][mz + 1];
                const float olx = A.olo[0][mx + 1], oly = A.olo[1][my + 1], olz = A.olo[2][mz + 1];
                const uint32_t img = (uint32_t)(mx + 1) | ((uint32_t)(my + 1) << 2) | ((uint32_t)(mz + 1) << 4);
                for (uint32_t jb = jbeg; jb < jend;) {
                    // a round of 32 candidates: the kept ones go to the stage (a round that
                    // overfills it takes its first kept points; the next starts after the last)
                    const float4 b0 = sbox[0], b1 = sbox[1];
                    const uint32_t nc = min(32u, jend - jb);
                    float4 p = make_float4(0.f, 0.f, 0.f, 0.f), q = p;
                    bool keep = false;
                    if ((uint32_t)lane < nc) {
                        p = A.hi2[jb + lane];
                        p.x += ox;
                        p.y += oy;
                        p.z += oz;
                        const float dx = fmaxf(0.f, fmaxf(b0.x - p.x, p.x - b1.x));
                        const float dy = fmaxf(0.f, fmaxf(b0.y - p.y, p.y - b1.y));
                        const float dz = fmaxf(0.f, fmaxf(b0.z - p.z, p.z - b1.z));
                        keep = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) <= b0.w;
                        if (NEED_AVG && keep) {
                            q = A.lo2[jb + lane];
                            q.x += olx;
                            q.y += oly;
                            q.z += olz;
                        }
                    }
                    const uint32_t m = __ballot_sync(0xffffffffu, keep);
                    const int room = 32 - f;
                    const int rank = __popc(m & ((1u << lane) - 1u));
                    const uint32_t taken = __ballot_sync(0xffffffffu, keep && rank < room);
                    if (keep && rank < room) {
                        const int pos = f + rank;
                        S[pos] = p.x;
                        S[32 + pos] = p.y;
                        S[64 + pos] = p.z;
                        if (NEED_W) S[96 + pos] = p.w;
                        if (NEED_AVG) {
                            SL8[pos] = q.x;
                            SL8[32 + pos] = q.y;
                            SL8[64 + pos] = q.z;
                        }
                        sidx[pos] = jb + (uint32_t)lane;
                        simg[pos] = (uint8_t)img;
                    }
                    const int nt = __popc(taken);
                    jb += (uint32_t)__popc(m) <= (uint32_t)room ? nc : (uint32_t)(32 - __clz(taken));
                    f += nt;
                    evaluated += (uint64_t)icount * (uint32_t)nt;
                    if (f == 32) {
                        run_tile(32, ownr);
                        f = 0;
                    }
                }
                if (ownr && f > 0) run_partial(true);
            }
        }
        if (f > 0) run_partial(false);
        if constexpr (SINGLE) continue;  // one catalogue: queues and columns carry over
        // the chunk's queued pairs, then every lane's column into its catalogue
        __syncwarp();
        if (sq_n > 0) {
            slow_batch<MODE, NEED_AVG, NEED_W, true>(A, se, glo, ghi, sq, sq_n, rq, rq_count, h, hl, lane, &refined,
                                                     (int)ib);
            sq_n = 0;
        }
        const int rest = *rq_count;
        if (rest > 0) {
            refine_batch<MODE, NEED_AVG, NEED_W>(A, se, rq, rest, h, hl, lane, (int)ib);
            if (lane == 0) *rq_count = 0;
            __syncwarp();
        }
        flush_lanes<NEED_AVG, NEED_W>(A, h, lane, cat);
        col_terms = 0;
    }
    if constexpr (SINGLE) {
        __syncwarp();
        if (sq_n > 0) slow_batch<MODE, NEED_AVG, NEED_W, true>(A, se, glo, ghi, sq, sq_n, rq, rq_count, h, hl, lane, &refined);
        const int rest = *rq_count;
        if (rest > 0) refine_batch<MODE, NEED_AVG, NEED_W>(A, se, rq, rest, h, hl, lane);
        flush_hist<NEED_AVG, NEED_W>(A, h, lane, 0u);
    }
    for (int off = 16; off; off >>= 1) refined += __shfl_down_sync(0xffffffffu, refined, off);
    if (lane == 0) {
        atomicAdd(&A.g_stats[0], (unsigned long long)evaluated);
        atomicAdd(&A.g_stats[1], refined);
        atomicAdd(&A.g_stats[2], queued);
    }
}

template <int MODE, bool NEED_AVG, bool NEED_W>
__global__ void __launch_bounds__(256) k_pairs_f64(PairArgs A, SmemLayout SL)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *se = (double *)(smem + SL.edges_off);
    float *asc = (float *)(smem + SL.ascale_off);
    for (int k = threadIdx.x; k < A.nedges; k += blockDim.x) {
        se[k] = A.g_edges[k];
        asc[k] = A.g_ascale[k];
    }
    double4_32a *sj = (double4_32a *)(smem + SL.stage_off + SL.per_warp_stage * warp);
    int2 *sro = (int2 *)(sj + 32);  // reference cell, caller index
    WarpHist h = warp_hist(smem, SL, warp);
    zero_hist(h, SL, lane);
    // weights over a wide range: the warp's weight sums in double, one per histogram row
    double *wd = (NEED_W && A.w_exact) ? (double *)(smem + SL.wd_off + SL.per_warp_wd * warp) : nullptr;
    if (wd)
        for (int b = lane; b < SL.nrows; b += 32) wd[b] = 0.0;
    const int hl = lane & (SL.lane_stride - 1);
    __syncthreads();
    uint64_t evaluated = 0;
    const uint32_t ntasks = A.ntask_dev ? min(*A.ntask_dev, A.ntasks) : A.ntasks;
    uint32_t cur_cat = 0;
    uint32_t col_terms = 0;
    const uint32_t tile_terms = 32u * (32u / (uint32_t)SL.lane_stride);

    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(A.task_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= ntasks) break;
        const Task T = A.tasks[t];
        const long long t_start = A.task_clock ? clock64() : 0;
        const uint32_t cat = T.meta >> kCatShift;
        if (cat != cur_cat) {
            flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat, wd);
            cur_cat = cat;
            col_terms = 0;
        }
        const int icount = (int)(T.meta & 63u) + 1;
        const int mx = (int)((T.meta >> 8) & 3u) - 1, my = (int)((T.meta >> 10) & 3u) - 1,
                  mz = (int)((T.meta >> 12) & 3u) - 1;
        const bool own = (T.meta >> 16) & 1u;
        const bool wrapped = (mx | my | mz) != 0;
        const uint32_t i = T.i_begin + lane;
        const bool ivalid = lane < icount;
        const double4_32a pi = ivalid ? A.d1[i] : make_double4_32a(0, 0, 0, 0);
        const int2 roi = ivalid ? A.ro1[i] : make_int2(0, 0);
        const int rci = roi.x, ori = roi.y;
        const double ox = A.odbl[0][mx + 1], oy = A.odbl[1][my + 1], oz = A.odbl[2][mz + 1];
        for (uint32_t jb = T.j_begin; jb < T.j_end; jb += 32) {
            const uint32_t nj = min(32u, T.j_end - jb);
            if ((uint32_t)lane < nj) {
                sj[lane] = A.d2[jb + lane];
                sro[lane] = A.ro2[jb + lane];
            }
            __syncwarp();
            if (ivalid) {
                for (uint32_t k = 0; k < nj; k++) {
                    const uint32_t j = jb + k;
                    if (own && j <= i) continue;
                    const double4_32a pj = sj[k];
                    double avg_term = 0.0;
                    int bin;
                    // points outside the reference lattice: only pairs of linked reference cells
                    if (A.ref_links && !ref_linked(A, rci, sro[k].x, mx, my, mz)) continue;
                    if (MODE != MODE_THETA && A.autocorr && wrapped &&
                        (sro[k].x > rci || (sro[k].x == rci && (pj.z < pi.z || (pj.z == pi.z && sro[k].y < ori))))) {
                        bin = ref_eval<MODE>(A, se, pj.x, pj.y, pj.z, pi.x, pi.y, pi.z, ox, oy, oz, &avg_term);
                    } else {
                        bin = ref_eval<MODE>(A, se, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, -ox, -oy, -oz, &avg_term);
                    }
                    if (bin < 0) continue;
                    if (wd) {
                        accumulate<NEED_AVG, false>(A, h, bin, bin * h.ls + hl, avg_term, 0.0);
                        atomicAdd(&wd[bin], pi.w * pj.w);
                    } else {
                        accumulate<NEED_AVG, NEED_W>(A, h, bin, bin * h.ls + hl, avg_term, pi.w * pj.w);
                    }
                }
            }
            __syncwarp();
            col_terms += tile_terms;
            if (col_terms + tile_terms > (uint32_t)kColumnTerms) {
                flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat, wd);
                col_terms = 0;
            }
        }
        evaluated += (uint64_t)icount * (T.j_end - T.j_begin);
        if (A.task_clock && lane == 0) {
            A.task_clock[2 * (size_t)t] = (unsigned long long)(clock64() - t_start);
            A.task_clock[2 * (size_t)t + 1] = (blockIdx.x * (blockDim.x >> 5)) + warp;
        }
    }
    flush_hist<NEED_AVG, NEED_W>(A, h, lane, cur_cat, wd);
    if (lane == 0) atomicAdd(&A.g_stats[0], (unsigned long long)evaluated);
}

// ------------------------------------------------------------------------------------
// FP32 FMA-pipe calibration: 8 independent dependency chains per thread keep every FMA
// lane busy; 2 FLOP per fmaf.  Used only as the measured denominator of the pair kernels'
// FP32 roofline fraction.
// ------------------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_fma_peak(float *out, int iters, float a, float b)
{
    float v[8];
    for (int k = 0; k < 8; k++) v[k] = threadIdx.x * 1e-3f + k;
    for (int it = 0; it < iters; it++) {
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = fmaf(v[k], a, b);
    }
    float s = 0.f;
    for (int k = 0; k < 8; k++) s += v[k];
    if (s == 12345.678f) out[blockIdx.x] = s;  // keeps the chains live
}

// ------------------------------------------------------------------------------------
// host side: buffers, launch helpers
// ------------------------------------------------------------------------------------
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
};

static bool injected_alloc_failure(size_t bytes);

static int ensure(DevBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return EXIT_SUCCESS;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = bytes + bytes / 4;
    if (injected_alloc_failure(want)) return EXIT_FAILURE;
    CF_CUDA(cudaMalloc(&b.p, want));
    b.cap = want;
    return EXIT_SUCCESS;
}

// pinned host staging (small uploads and the histogram read-back go through it, so none of
// those copies waits on the host); only grown between calls, after the stream has drained
struct HostBuf {
    void *p = nullptr;
    size_t cap = 0;
};

static int ensure_host(HostBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return EXIT_SUCCESS;
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = bytes + bytes / 4;
    if (injected_alloc_failure(want)) return EXIT_FAILURE;
    CF_CUDA(cudaHostAlloc(&b.p, want, cudaHostAllocDefault));
    b.cap = want;
    return EXIT_SUCCESS;
}

struct SetBufs {
    DevBuf raw[4];  // device copies of x, y, z, w as given (float or double)
    const void *in[4];  // arrays the lattice is built from: raw[] or caller-owned device arrays
    DevBuf cellid_u, count, fill, cell_start;  // fill: slot of every point within its cell
    DevBuf hi, lo, dbl, ro;
};

// Every device and pinned buffer one count uses.  Single calls share the engine's workspace;
// a batch plan owns one, so that its captured graph never sees a buffer move.
struct Workspace {
    SetBufs set[2];
    DevBuf mm, scan_tmp[4], chunk_cnt, chunk_off, chunk_begin, chunk_info, chunk_cat, ntask, task_off, tasks;
    DevBuf recs;  // range records of packed tasks (JRange)
    DevBuf sten;  // stencil list of the split j lattice (k_item_list)
    DevBuf res, tab;  // result block (ResView), bin tables (edges, guards, averages scale, lookup table)
    DevBuf task_clock;  // per-task timer records (only when asked for)
    HostBuf h_small, h_tab, h_hist, h_sten;
};

// The result block of one run, one device allocation read back by one copy (the pinned host
// copy has the same layout), nb = bins x catalogues:
//   u64 cnt[nb] | f64 avg[nb] | f64 w[nb] | u64 stats[4] | u32 flags[4] | u64 oob | u64 extent
//   | u32 recs[2]
// stats: pairs evaluated, refined, queued; flags: [0] task counter of the pair kernel, [1] tasks
// emitted, [2] periodic image beyond +-1, [3] work-list overflow; oob: points outside the
// reference lattice; extent: points / weights outside a batch plan's range; recs[0]: range
// records of packed tasks emitted.
struct ResView {
    unsigned long long *cnt;
    double *avg, *w;
    unsigned long long *stats;
    uint32_t *flags;
    unsigned long long *oob, *extent;
    uint32_t *recs;
};
static inline size_t res_bytes(size_t nb) { return sizeof(unsigned long long) * (3 * nb + 9); }
// bytes zeroed before each pair-kernel launch: the sums, the statistics and the task counter
static inline size_t res_zero_bytes(size_t nb) { return sizeof(unsigned long long) * (3 * nb + 4) + sizeof(uint32_t); }
static inline ResView res_view(void *base, size_t nb)
{
    ResView R;
    unsigned long long *u = (unsigned long long *)base;
    R.cnt = u;
    R.avg = (double *)(u + nb);
    R.w = (double *)(u + 2 * nb);
    R.stats = u + 3 * nb;
    R.flags = (uint32_t *)(u + 3 * nb + 4);
    R.oob = u + 3 * nb + 6;
    R.extent = u + 3 * nb + 7;
    R.recs = (uint32_t *)(u + 3 * nb + 8);
    return R;
}

static void release(DevBuf &b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

static void release_workspace(Workspace &W)
{
    for (int s = 0; s < 2; s++) {
        SetBufs &B = W.set[s];
        for (int k = 0; k < 4; k++) release(B.raw[k]);
        DevBuf *v[] = {&B.cellid_u, &B.count, &B.fill, &B.cell_start, &B.hi, &B.lo, &B.dbl, &B.ro};
        for (DevBuf *d : v) release(*d);
    }
    for (int k = 0; k < 4; k++) release(W.scan_tmp[k]);
    DevBuf *v[] = {&W.mm, &W.chunk_cnt, &W.chunk_off, &W.chunk_begin, &W.chunk_info, &W.chunk_cat, &W.ntask,
                   &W.task_off, &W.tasks, &W.recs, &W.sten, &W.res, &W.tab, &W.task_clock};
    for (DevBuf *d : v) release(*d);
    HostBuf *h[] = {&W.h_small, &W.h_tab, &W.h_hist, &W.h_sten};
    for (HostBuf *b : h) {
        if (b->p) cudaFreeHost(b->p);
        b->p = nullptr;
        b->cap = 0;
    }
}

struct Engine {
    bool init = false;
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8];
    Workspace ws;
    int regs_cache[kNumModes][4][2] = {};  // registers per thread of each pair kernel (0 = not queried)
    int force_ls = 0, force_warps = 0;  // FP32 pair-kernel layout chosen by the batch tuner (0 = scored)
    uint32_t task_cap0 = 0;  // first work-list capacity of a call (0 = from the lattice; CF_TASK_CAPACITY)
    int precision = CF_PRECISION_FP32_REFINE;
    int byte_table = 1;  // byte bucket table for DD(r), xi and DDtheta (CF_BYTE_TABLE=0: 32-bit table)
    int lut8_lg = 12;    // finest byte-table resolution, log2 buckets per octave (CF_BYTE_TABLE_LG)
    bool layout_packed = false;  // the current count's FP32 pair kernel takes packed tasks
    bool layout_prune = false;   // ... or may prune j points by box (byte-table modes of single counts)
    // single-count autotuner (cf_engine_set_autotune): per count shape, the fastest j-lattice
    // column split found by timing the candidates on the first count of that shape
    int autotune = 0;
    int tune_force = 0, tune_zdiv = 1;  // split forced for the count being run (0: none)
    struct TuneEntry {
        unsigned long long key;
        int split, zdiv;
    } tune[32];
    int ntune = 0, tune_next = 0;
    int clock_khz = 0;   // SM clock rate (per-task timer: cycles to nanoseconds)
    // test hooks (environment, read once): CF_TEST_FAIL_ALLOC=n makes the n-th device or pinned
    // allocation of the process fail as an out-of-memory would; CF_TEST_SIGNAL=n raises SIGINT
    // on the host just before the n-th pair-kernel launch of the process
    long fail_alloc_at = 0, alloc_count = 0;
    long test_signal = 0, pair_launches = 0;
    int launches = 0;  // kernels launched by the current call
    size_t smem_per_sm = 228 * 1024;
    int last_blocks_per_sm = 0, last_warps_per_block = 0, last_lane_stride = 0;
    cf_engine_stats last;
};

static Engine g_eng;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

static bool injected_alloc_failure(size_t bytes)
{
    if (g_eng.fail_alloc_at <= 0 || ++g_eng.alloc_count != g_eng.fail_alloc_at) return false;
    fprintf(stderr, "corrfunc_gb300: allocation of %zu bytes failed (injected by CF_TEST_FAIL_ALLOC)\n", bytes);
    return true;
}

// ------------------------------------------------------------------------------------
// Interrupts (utils/macros.h:145-167, theory/DD/countpairs_impl.c.src:31-37): while a count runs,
// SIGTERM, SIGINT and SIGHUP only set a flag (and say so on stderr); the host checks it between
// launches and returns EXIT_FAILURE.  The kernels already in flight finish (milliseconds); the
// previous handlers are restored when the call returns.
// ------------------------------------------------------------------------------------
static volatile sig_atomic_t g_signal = 0;

static void on_interrupt(int signo)
{
    g_signal = signo;
    static const char msg[] = "corrfunc_gb300: received an interrupt signal; aborting the count\n";
    const ssize_t w = write(2, msg, sizeof(msg) - 1);
    (void)w;
}

struct InterruptGuard {
    static constexpr int kN = 3;
    const int sigs[kN] = {SIGTERM, SIGINT, SIGHUP};
    struct sigaction prev[kN];
    bool saved[kN];
    InterruptGuard()
    {
        g_signal = 0;
        struct sigaction sa;
        memset(&sa, 0, sizeof(sa));
        sa.sa_handler = on_interrupt;
        sigemptyset(&sa.sa_mask);
        for (int k = 0; k < kN; k++) saved[k] = sigaction(sigs[k], &sa, &prev[k]) == 0;
    }
    ~InterruptGuard()
    {
        for (int k = 0; k < kN; k++)
            if (saved[k]) sigaction(sigs[k], &prev[k], nullptr);
    }
};

#define CF_CHECK_INTERRUPT()                                                                   \
    do {                                                                                        \
        if (g_signal) CF_FAIL("interrupted by signal %d; the count was abandoned", (int)g_signal); \
    } while (0)

static int engine_init(void)
{
    int dev = 0;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        CF_FAIL("no CUDA device available (%s); this library has no CPU fallback",
                e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
    }
    CF_CUDA(cudaGetDevice(&dev));
    if (g_eng.init && g_eng.device == dev) return EXIT_SUCCESS;
    cudaDeviceProp prop;
    CF_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (prop.major < 10) {
        CF_FAIL("device %d (%s, sm_%d%d) is not a Blackwell-class GPU; this build targets sm_103a", dev, prop.name,
                prop.major, prop.minor);
    }
    g_eng.device = dev;
    g_eng.num_sms = prop.multiProcessorCount;
    g_eng.smem_per_sm = prop.sharedMemPerMultiprocessor;
    if (cudaDeviceGetAttribute(&g_eng.clock_khz, cudaDevAttrClockRate, dev) != cudaSuccess) g_eng.clock_khz = 0;
    CF_CUDA(cudaStreamCreateWithFlags(&g_eng.stream, cudaStreamNonBlocking));
    for (int k = 0; k < 8; k++) CF_CUDA(cudaEventCreate(&g_eng.ev[k]));
    // CF_PAIR_LAYOUT="<lane stride>,<warps per block>" fixes the FP32 pair kernel's histogram
    // layout instead of the scored choice (for layout measurements)
    const char *lay = getenv("CF_PAIR_LAYOUT");
    int ls = 0, wp = 0;
    if (lay && sscanf(lay, "%d,%d", &ls, &wp) == 2 && (ls == 1 || ls == 4 || ls == 8 || ls == 16 || ls == 32) &&
        (wp == 3 || wp == 4 || wp == 6 || wp == 8 || wp == 12 || wp == 16)) {
        g_eng.force_ls = ls;
        g_eng.force_warps = wp;
    }
    // CF_TASK_CAPACITY=<n> starts every single call with a work-list buffer of n tasks (tests use
    // a small n to exercise the resize-and-rerun path)
    const char *tc = getenv("CF_TASK_CAPACITY");
    if (tc && atoi(tc) > 0) g_eng.task_cap0 = (uint32_t)atoi(tc);
    // CF_BYTE_TABLE=0 classifies DD(r), xi and DDtheta pairs with the 32-bit bucket table of the
    // other modes (for measurements; both give the same counts)
    const char *bt = getenv("CF_BYTE_TABLE");
    if (bt && atoi(bt) == 0) g_eng.byte_table = 0;
    // CF_BYTE_TABLE_LG=<4..12> caps the byte table at 2^n buckets per octave (for measurements;
    // every resolution gives the same counts)
    const char *bl = getenv("CF_BYTE_TABLE_LG");
    if (bl && atoi(bl) >= 4 && atoi(bl) <= 12) g_eng.lut8_lg = atoi(bl);
    const char *fa = getenv("CF_TEST_FAIL_ALLOC");
    if (fa && atol(fa) > 0) g_eng.fail_alloc_at = atol(fa);
    const char *ts = getenv("CF_TEST_SIGNAL");
    if (ts && atol(ts) > 0) g_eng.test_signal = atol(ts);
    g_eng.init = true;
    return EXIT_SUCCESS;
}

// exclusive scan; out must have n+1 entries
static int scan_u32(Workspace &W, const uint32_t *in, uint32_t *out, uint32_t n, int level)
{
    cudaStream_t st = g_eng.stream;
    if (n == 0) {
        CF_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
        return EXIT_SUCCESS;
    }
    if (level >= 4) CF_FAIL("scan too deep");
    const uint32_t nblk = (n + kScanTile - 1) / kScanTile;
    if (ensure(W.scan_tmp[level], sizeof(uint32_t) * (2 * (size_t)nblk + 2)) != EXIT_SUCCESS) return EXIT_FAILURE;
    uint32_t *bs = (uint32_t *)W.scan_tmp[level].p;
    uint32_t *bs_scan = bs + nblk;  // nblk+1 entries
    k_scan_tile<<<nblk, 1024, 0, st>>>(in, out, n, bs);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    if (nblk == 1) return EXIT_SUCCESS;  // the tile wrote out[n]
    if (scan_u32(W, bs, bs_scan, nblk, level + 1) != EXIT_SUCCESS) return EXIT_FAILURE;
    k_scan_add<<<nblk, 1024, 0, st>>>(out, n, bs_scan);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    return EXIT_SUCCESS;
}

static inline int grid_for(int64_t n, int threads)
{
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)g_eng.num_sms * 16;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

static double pow2_ceil(double v)
{
    if (!(v > 0.0)) return 1.0;
    return ldexp(1.0, (int)ceil(log2(v)));
}

static float f_down(double v)
{
    float f = (float)v;
    if ((double)f > v) f = nextafterf(f, -INFINITY);
    return f;
}

static float f_up(double v)
{
    float f = (float)v;
    if ((double)f < v) f = nextafterf(f, INFINITY);
    return f;
}

// extent of one catalogue folded into mm[0..7] (one pass; each block folds its extremes atomically)
template <typename T>
static int minmax_into(Workspace &W, const T *x, const T *y, const T *z, const T *w, int64_t n, unsigned long long *mm)
{
    if (n <= 0) return EXIT_SUCCESS;
    int grid = grid_for((n + kMinmaxUnroll - 1) / kMinmaxUnroll, 256);
    if (grid > 4 * g_eng.num_sms) grid = 4 * g_eng.num_sms;
    (void)W;
    k_minmax<T><<<grid, 256, 0, g_eng.stream>>>(x, y, z, w, n, mm);
    CF_CUDA(cudaGetLastError());
    g_eng.launches += 1;
    return EXIT_SUCCESS;
}

template <typename T>
static int upload_and_minmax(Workspace &W, int s, int64_t n, const void *x, const void *y, const void *z, const void *w,
                             bool on_device, unsigned long long *mm_dev)
{
    SetBufs &B = W.set[s];
    const size_t bytes = sizeof(T) * (size_t)n;
    const void *src[4] = {x, y, z, w};
    for (int k = 0; k < 4; k++) {
        B.in[k] = nullptr;
        if (k == 3 && !w) continue;
        if (on_device) {
            B.in[k] = src[k];
            continue;
        }
        if (ensure(B.raw[k], bytes) != EXIT_SUCCESS) return EXIT_FAILURE;
        CF_CUDA(cudaMemcpyAsync(B.raw[k].p, src[k], bytes, cudaMemcpyHostToDevice, g_eng.stream));
        B.in[k] = B.raw[k].p;
    }
    return minmax_into<T>(W, (const T *)B.in[0], (const T *)B.in[1], (const T *)B.in[2], (const T *)B.in[3], n,
                          mm_dev);
}

// Counting sort of one catalogue into lattice records at point offset `base` of B (whose
// per-point buffers already hold base + n points); B's per-cell arrays are reused.
// The counting sort of one catalogue into a lattice, in two halves around the scan of the cell
// occupancy: cell index and slot within the cell of every point (the occupancy counts must have
// been zeroed; several catalogues may count into one lattice), then the records at their slots
// (from record rec_base on; ro_cat >= 0: the catalogue number takes the place of the reference
// cell).  base: the catalogue's first point in the per-point cell and slot arrays.
template <typename T>
static int lattice_assign_at(SetBufs &B, int64_t n, int64_t base, const T *x, const T *y, const T *z, const Geom &g,
                             unsigned long long *oob)
{
    if (n <= 0) return EXIT_SUCCESS;
    k_assign<T><<<grid_for(n, 256), 256, 0, g_eng.stream>>>(x, y, z, n, g, (uint32_t *)B.cellid_u.p + base,
                                                           (uint32_t *)B.fill.p + base, (uint32_t *)B.count.p, oob);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    return EXIT_SUCCESS;
}

template <typename T>
static int lattice_scatter_at(SetBufs &B, int64_t n, int64_t base, int64_t rec_base, const T *x, const T *y,
                              const T *z, const T *w, const Geom &g, int ro_cat, SetBufs *RB = nullptr)
{
    if (n <= 0) return EXIT_SUCCESS;
    SetBufs &D = RB ? *RB : B;  // the record buffers (B's own unless given)
    Lattice L;
    L.hi = (float4 *)D.hi.p + rec_base;
    L.lo = g.write_lo ? (float4 *)D.lo.p + rec_base : nullptr;
    L.dbl = (double4_32a *)D.dbl.p + rec_base;
    L.ro = (int2 *)D.ro.p + rec_base;
    L.cell_start = (uint32_t *)B.cell_start.p;
    k_scatter<T><<<grid_for(n, 256), 256, 0, g_eng.stream>>>(x, y, z, w, n, g, (const uint32_t *)B.cellid_u.p + base,
                                                            (const uint32_t *)B.fill.p + base,
                                                            (const uint32_t *)B.cell_start.p, L, ro_cat);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    return EXIT_SUCCESS;
}

// (RB: the records go to RB's buffers from record rec_base on instead of B's from base)
template <typename T>
static int build_lattice_at(Workspace &W, SetBufs &B, int64_t n, int64_t base, const T *x, const T *y, const T *z,
                            const T *w, const Geom &g, uint32_t ncells, unsigned long long *oob,
                            SetBufs *RB = nullptr, int64_t rec_base = -1)
{
    cudaStream_t st = g_eng.stream;
    // per-cell occupancy; every point gets its slot within its cell from the counting atomic
    if (ensure(B.count, sizeof(uint32_t) * (size_t)ncells) ||
        ensure(B.cell_start, sizeof(uint32_t) * ((size_t)ncells + 1)))
        return EXIT_FAILURE;
    uint32_t *count = (uint32_t *)B.count.p;
    CF_CUDA(cudaMemsetAsync(count, 0, sizeof(uint32_t) * (size_t)ncells, st));
    if (n <= 0) {
        CF_CUDA(cudaMemsetAsync(B.cell_start.p, 0, sizeof(uint32_t) * ((size_t)ncells + 1), st));
        return EXIT_SUCCESS;
    }
    if (lattice_assign_at<T>(B, n, base, x, y, z, g, oob) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (scan_u32(W, count, (uint32_t *)B.cell_start.p, ncells, 0) != EXIT_SUCCESS) return EXIT_FAILURE;
    return lattice_scatter_at<T>(B, n, base, RB ? rec_base : base, x, y, z, w, g, -1, RB);
}

static int ensure_points(SetBufs &B, int64_t n)
{
    if (ensure(B.cellid_u, sizeof(uint32_t) * n) || ensure(B.fill, sizeof(uint32_t) * n) ||
        ensure(B.hi, sizeof(float4) * n) || ensure(B.lo, sizeof(float4) * n) ||
        ensure(B.dbl, sizeof(double4_32a) * n) || ensure(B.ro, sizeof(int2) * n))
        return EXIT_FAILURE;
    return EXIT_SUCCESS;
}

template <typename T>
static int build_lattice(Workspace &W, int s, int64_t n, bool has_w, const Geom &g, uint32_t ncells, unsigned long long *oob)
{
    SetBufs &B = W.set[s];
    if (ensure_points(B, n) != EXIT_SUCCESS) return EXIT_FAILURE;
    const T *x = (const T *)B.in[0], *y = (const T *)B.in[1], *z = (const T *)B.in[2];
    const T *w = has_w ? (const T *)B.in[3] : nullptr;
    return build_lattice_at<T>(W, B, n, 0, x, y, z, w, g, ncells, oob);
}

// Histogram layout / block size that keeps the most warps resident: private per-lane columns
// (conflict-free) or one shared row per warp (shared atomics), 8/4/2 warps per block.
template <int MODE, bool AVG, bool W>
static int pair_kernel_regs_t(bool f64)
{
    cudaFuncAttributes fa;
    cudaError_t rc;
    if constexpr (kHasF32<MODE>) {
        rc = f64 ? cudaFuncGetAttributes(&fa, k_pairs_f64<MODE, AVG, W>)
                 : cudaFuncGetAttributes(&fa, k_pairs_f32<MODE, AVG, W, false, false>);
    } else {
        rc = cudaFuncGetAttributes(&fa, k_pairs_f64<MODE, AVG, W>);
    }
    return rc == cudaSuccess && fa.numRegs > 0 ? fa.numRegs : 64;
}

template <int MODE>
static int pair_kernel_regs_m(bool f64, bool avg, bool w)
{
    if (avg && w) return pair_kernel_regs_t<MODE, true, true>(f64);
    if (avg) return pair_kernel_regs_t<MODE, true, false>(f64);
    if (w) return pair_kernel_regs_t<MODE, false, true>(f64);
    return pair_kernel_regs_t<MODE, false, false>(f64);
}

static int pair_kernel_regs(int mode, bool f64, bool avg, bool w)
{
    int &c = g_eng.regs_cache[mode < 0 || mode >= kNumModes ? MODE_THETA : mode][(avg ? 2 : 0) + (w ? 1 : 0)][f64 ? 1 : 0];
    if (c > 0) return c;
    switch (mode) {
    case MODE_R3: c = pair_kernel_regs_m<MODE_R3>(f64, avg, w); break;
    case MODE_RPPI: c = pair_kernel_regs_m<MODE_RPPI>(f64, avg, w); break;
    case MODE_WP: c = pair_kernel_regs_m<MODE_WP>(f64, avg, w); break;
    case MODE_SMU: c = pair_kernel_regs_m<MODE_SMU>(f64, avg, w); break;
    case MODE_RPPI_MOCK: c = pair_kernel_regs_m<MODE_RPPI_MOCK>(f64, avg, w); break;
    case MODE_SMU_MOCK: c = pair_kernel_regs_m<MODE_SMU_MOCK>(f64, avg, w); break;
    default: c = pair_kernel_regs_m<MODE_THETA>(f64, avg, w); break;
    }
    return c;
}

// Histogram layout and block size.  Lanes l and l + lane_stride share a column; the score is the
// resident warps per SM (shared memory and registers) discounted by the expected contention of
// shared columns (1 = private, 2 = 2-way, ... 32 = the whole warp on one row).
// warps of the FP32 pair kernel resident per SM with layout c (shared memory, threads, registers)
static int layout_resident(const SmemLayout &c, int mode, bool avg, bool w)
{
    if (c.total > 220 * 1024) return 0;
    (void)mode;
    const int regs = pair_kernel_regs(mode, false, avg, w);
    const int warps_by_regs = 65536 / (32 * ((regs + 7) / 8 * 8));
    int blocks = (int)(g_eng.smem_per_sm / (c.total + 1024));
    const int max_blocks_threads = 2048 / (32 * c.warps);
    if (blocks > max_blocks_threads) blocks = max_blocks_threads;
    const int max_blocks_regs = warps_by_regs / c.warps;
    if (blocks > max_blocks_regs) blocks = max_blocks_regs;
    return blocks * c.warps;
}

// resident warps weighted by the measured cost of lanes sharing histogram columns
static double lane_factor(int lane_stride)
{
    // measured: 2-way sharing costs a few per cent, 4-way about a third (64-bit weight sums)
    switch (lane_stride) {
    case 32: return 1.0;
    case 16: return 0.92;
    case 8: return 0.6;
    case 4: return 0.45;
    default: return 0.2;
    }
}
static double layout_score(const SmemLayout &c, int mode, bool avg, bool w)
{
    int resident = layout_resident(c, mode, avg, w);
    if (resident > 48) resident = 48;
    return resident * lane_factor(c.lane_stride);
}

static SmemLayout choose_layout(int mode, bool f64, bool avg, bool w, int nedges, int nbins, int lut_n)
{
    const bool pk = g_eng.layout_packed && !f64;  // a count with packed tasks
    const bool pr = g_eng.layout_prune && !f64;   // a count whose kernel may prune
    const bool dz = (mode == MODE_RPPI || mode == MODE_WP || mode == MODE_SMU || mode_is_mock(mode));
    const bool los = avg || mode_is_mock(mode);
    const bool forced = g_eng.force_ls > 0 && g_eng.force_warps > 0 && 32 * g_eng.force_warps <= pair_max_threads(mode, avg, w);
    if (!f64 && forced) {
        const SmemLayout c = smem_layout(nedges, nbins, g_eng.force_warps, f64, lut_n, g_eng.force_ls, avg, w, dz, los, pk, pr);
        if (c.total <= 220 * 1024) return c;
    }
    const int regs = pair_kernel_regs(mode, f64, avg, w);
    const int warps_by_regs = 65536 / (32 * ((regs + 7) / 8 * 8));
    SmemLayout SL = smem_layout(nedges, nbins, 8, f64, lut_n, 1, avg, w, dz, los, pk, pr);
    double best = -1.0;
    const int lstrides[5] = {32, 16, 8, 4, 1};
    const int max_warps = f64 ? 8 : pair_max_threads(mode, avg, w) / 32;
    const int wopts[3] = {max_warps, max_warps / 2, max_warps / 4};
    for (int li = 0; li < 5; li++) {
        for (int wi = 0; wi < 3; wi++) {
            const SmemLayout c = smem_layout(nedges, nbins, wopts[wi], f64, lut_n, lstrides[li], avg, w, dz, los, pk, pr);
            if (c.total > 220 * 1024) continue;
            int blocks = (int)(g_eng.smem_per_sm / (c.total + 1024));
            const int max_blocks_threads = 2048 / (32 * wopts[wi]);
            if (blocks > max_blocks_threads) blocks = max_blocks_threads;
            const int max_blocks_regs = warps_by_regs / wopts[wi];
            if (blocks > max_blocks_regs) blocks = max_blocks_regs;
            int resident = blocks * wopts[wi];
            if (resident > 48) resident = 48;
            const double score = resident * lane_factor(lstrides[li]) + 1e-3 * wopts[wi];
            if (score > best) {
                best = score;
                SL = c;
            }
        }
    }
    return SL;
}

template <int MODE, bool AVG, bool W>
static int launch_pairs_t(const PairArgs &A, bool f64, int *launched)
{
    const int nedges = A.nedges;
    SmemLayout SL = choose_layout(MODE, f64, AVG, W, nedges, A.nbins, A.lut_n);
    if (!f64 && SL.lane_stride != A.lane_stride_hint) CF_FAIL("internal: histogram layout changed after the table was built");
    // the kernel's kPrune
    const bool prunes = A.lut8 || MODE == MODE_RPPI || MODE == MODE_WP || MODE == MODE_SMU || mode_is_mock(MODE);
    if (!f64 && (A.jrec || prunes) && !SL.extras) CF_FAIL("internal: packed or pruned tiles without their stage space");
    if (SL.total > 220 * 1024) CF_FAIL("histogram too large for on-chip accumulation (%d bins)", A.nbins);
    const int threads = SL.warps * 32;
    int per_sm = 1;
    if (f64) {
        auto kern = k_pairs_f64<MODE, AVG, W>;
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, SL.total));
        if (per_sm < 1) per_sm = 1;
        kern<<<g_eng.num_sms * per_sm, threads, SL.total, g_eng.stream>>>(A, SL);
    } else if constexpr (kHasF32<MODE>) {
        auto kern = k_pairs_f32<MODE, AVG, W, false, false>;
        if constexpr (MODE == MODE_R3 || MODE == MODE_THETA) {
            if (A.lut8) kern = k_pairs_f32<MODE, AVG, W, true, false>;
        }
        // work lists with packed tasks (split j columns, DD(r) and xi only)
        if constexpr (MODE == MODE_R3) {
            if (A.jrec) kern = A.lut8 ? k_pairs_f32<MODE, AVG, W, true, true> : k_pairs_f32<MODE, AVG, W, false, true>;
        } else {
            if (A.jrec) CF_FAIL("internal: packed tasks for mode %d", MODE);
        }
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, SL.total));
        if (per_sm < 1) per_sm = 1;
        kern<<<g_eng.num_sms * per_sm, threads, SL.total, g_eng.stream>>>(A, SL);
    } else {
        CF_FAIL("internal: no FP32 pair kernel for mode %d", MODE);
    }
    CF_CUDA(cudaGetLastError());
    g_eng.launches++;
    (*launched)++;
    g_eng.last_blocks_per_sm = per_sm;
    g_eng.last_warps_per_block = SL.warps;
    g_eng.last_lane_stride = SL.lane_stride;
    g_eng.last.blocks_per_sm = per_sm;
    g_eng.last.warps_per_block = SL.warps;
    g_eng.last.lane_stride = SL.lane_stride;
    return EXIT_SUCCESS;
}

template <int MODE>
static int launch_pairs_m(const PairArgs &A, bool f64, bool avg, bool w, int *launched)
{
    if (avg && w) return launch_pairs_t<MODE, true, true>(A, f64, launched);
    if (avg) return launch_pairs_t<MODE, true, false>(A, f64, launched);
    if (w) return launch_pairs_t<MODE, false, true>(A, f64, launched);
    return launch_pairs_t<MODE, false, false>(A, f64, launched);
}

// A single DD(r) / xi count whose warps each walk a whole chunk's neighbourhood (k_pairs_chunks
// with one catalogue): no work list, and the j points kept by the box fill whole tiles across
// the chunk's neighbour columns.
template <bool AVG, bool W>
static int launch_walk_t(const PairArgs &A, const TaskGeom &G, const uint32_t *chunk_begin, const uint2 *chunk_info,
                         const uint32_t *cs2, uint32_t nchunk, int *launched)
{
    const SmemLayout SL = choose_layout(MODE_R3, false, AVG, W, A.nedges, A.nbins, A.lut_n);
    if (SL.lane_stride != A.lane_stride_hint) CF_FAIL("internal: histogram layout changed after the table was built");
    if (!SL.extras) CF_FAIL("internal: pruned tiles without their stage space");
    auto kern = k_pairs_chunks<AVG, W, true>;
    int per_sm = 1;
    CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
    CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SL.warps * 32, SL.total));
    if (per_sm < 1) per_sm = 1;
    kern<<<g_eng.num_sms * per_sm, SL.warps * 32, SL.total, g_eng.stream>>>(A, SL, G, chunk_begin, chunk_info, cs2,
                                                                            nchunk);
    CF_CUDA(cudaGetLastError());
    g_eng.launches++;
    (*launched)++;
    g_eng.last.blocks_per_sm = per_sm;
    g_eng.last.warps_per_block = SL.warps;
    g_eng.last.lane_stride = SL.lane_stride;
    return EXIT_SUCCESS;
}

static int launch_walk(const PairArgs &A, bool avg, bool w, const TaskGeom &G, const uint32_t *chunk_begin,
                       const uint2 *chunk_info, const uint32_t *cs2, uint32_t nchunk, int *launched)
{
    if (avg && w) return launch_walk_t<true, true>(A, G, chunk_begin, chunk_info, cs2, nchunk, launched);
    if (avg) return launch_walk_t<true, false>(A, G, chunk_begin, chunk_info, cs2, nchunk, launched);
    if (w) return launch_walk_t<false, true>(A, G, chunk_begin, chunk_info, cs2, nchunk, launched);
    return launch_walk_t<false, false>(A, G, chunk_begin, chunk_info, cs2, nchunk, launched);
}

static int launch_pairs(int mode, const PairArgs &A, bool f64, bool avg, bool w, int *launched)
{
    switch (mode) {
    case MODE_R3: return launch_pairs_m<MODE_R3>(A, f64, avg, w, launched);
    case MODE_RPPI: return launch_pairs_m<MODE_RPPI>(A, f64, avg, w, launched);
    case MODE_WP: return launch_pairs_m<MODE_WP>(A, f64, avg, w, launched);
    case MODE_SMU: return launch_pairs_m<MODE_SMU>(A, f64, avg, w, launched);
    case MODE_THETA: return launch_pairs_m<MODE_THETA>(A, f64, avg, w, launched);
    case MODE_RPPI_MOCK: return launch_pairs_m<MODE_RPPI_MOCK>(A, f64, avg, w, launched);
    case MODE_SMU_MOCK: return launch_pairs_m<MODE_SMU_MOCK>(A, f64, avg, w, launched);
    }
    CF_FAIL("unknown mode %d", mode);
}

// Survey modes: the FP32 classification holds for pairs with FP32 |s|^2 below s2_cut (larger
// ones are certainly beyond the largest separation and rejected) and |l| of at least twice the
// largest |s| (pairs nearer the observer go to the exact path).  S = sqrt(s2_cut) with margin.
static double mock_s2_cut(const cf_job *J, int mode)
{
    const double e = J->edges[J->nedges - 1];
    const double m2 = mode == MODE_RPPI_MOCK ? e + J->pimax * J->pimax : e;
    return m2 * (1.0 + 1e-5);
}

static double mock_smax(const cf_job *J, int mode) { return sqrt(mock_s2_cut(J, mode) * (1.0 + 1e-6)); }

// FP32 error bounds of the survey quantities (u = 2^-24, rsqrtf taken as 8 ulps, q the hi grid):
//   |s_f - s| <= u|s| + 3.5uq,  |l_f - l| <= u(2|l| + 2|s|) + 2uq  ->  |l^_f - l^| <= 6u + 2uq/|l|
//   |pi_f - pi| <= |s|(12.7u + 8u) + 3.5uq                      (mock_pi_err, with |s| <= S)
//   rp via |s x l| / |l|:  |rp_f - rp| <= D = 6uS + 4.5uq + 3u rp, relative factor eta = 25u on rp^2
//   s^2:  |s2_f - s^2| <= 5.2u s^2 + 7uq|s|
static double mock_pi_err(double S, double q)
{
    const double u = 5.9604644775390625e-08;
    return 24.0 * u * S + 4.0 * u * q + 1e-13 * S;
}

static double mock_edge_band(int mode, double e, double S, double q)
{
    const double u = 5.9604644775390625e-08;
    const double re = sqrt(fabs(e));
    if (mode == MODE_RPPI_MOCK) {
        const double D = 6.0 * u * S + 4.5 * u * q + 3.0 * u * re;
        const double eta = 25.0 * u;
        return 2.0 * (2.0 * re * D + D * D + eta * (re + D) * (re + D) + 1e-14 * (S * S + 1.0));
    }
    return 2.0 * (6.0 * u * fabs(e) + 8.0 * u * q * re + 1e-14 * (fabs(e) + 1.0));
}

// error band for an edge value e given the per-axis coordinate error bound |delta|
static double edge_band(double e, double delta)
{
    const double u = 5.9604644775390625e-08;  // 2^-24
    const double re = sqrt(fabs(e));
    return 2.0 * (3.1 * u * fabs(e) + 2.0 * re * delta + delta * delta + 1e-14 * (fabs(e) + 1.0));
}

// Error bands, guards and the bucket table of one call, built on the host into pinned memory
// and uploaded stream-ordered (no host wait); done while the lattice kernels run.
struct Tables {
    int lut_n, shift, base, ls;
    uint32_t row_bytes, trash;
    float q_floor;
    double dxy, d3;
    size_t guard_off, ascale_off, lut_off;  // byte offsets in W.tab (edges at 0)
    // byte table (lut_n then counts 32-bit words of it, less one)
    int lut8;
    float qbias, qcap, qcap2;
    uint32_t trash_e;
};

constexpr int kLut8Max = 16384;  // largest byte table (entries)

// Byte table of DD(r), xi and DDtheta (at most 127 bins): entry = 2 * row + flag for the buckets
// of q' = min(r^2 + b, cap) (r^2 the squared chord for DDtheta).  Guards are built for q': an edge
// e maps to e' = e + b (exact in double), the FP32 evaluation of q' (three roundings, each within
// u of a partial sum at most q') is within 3.1 u q' of the exact value for the hi coordinates, and
// those differ from the reference's by the coordinate bound dlim, as for the 32-bit table.
// Returns false (building nothing) when the layout chosen for it would put a flagged entry at a
// misaligned address, or the edges do not suit it.
static bool build_lut8(const cf_job *J, int mode, int nbins, bool need_w, double dlim, float *guards_h, uint8_t *lut_h,
                       Tables *T)
{
    const int ne = J->nedges;
    const double u = 5.9604644775390625e-08;
    // edges in the classified domain (r^2, or the squared chord 2 (1 - cos) for DDtheta)
    double ev[CF_MAX_EDGES];
    double epos = 0.0;
    for (int k = 0; k < ne; k++) {
        ev[k] = mode == MODE_THETA ? 2.0 * (1.0 - J->edges[k]) : J->edges[k];
        if (ev[k] > 0.0 && (epos == 0.0 || ev[k] < epos)) epos = ev[k];
    }
    if (!(epos > 0.0) || !isfinite(ev[ne - 1])) return false;
    // b: a power of two at most 1/16 of the smallest positive edge (a normal float)
    const int kb = (int)floor(log2(epos / 16.0));
    if (kb < -120 || kb > 100) return false;
    const double b = ldexp(1.0, kb);
    for (int k = 0; k < ne; k++) {
        const double e1 = ev[k] + b;
        const double re = sqrt(fabs(ev[k]));
        double band = 2.0 * (3.1 * u * e1 + 2.0 * re * dlim + dlim * dlim + 1e-14 * (e1 + 1e-30));
        if (mode == MODE_THETA) band += 8e-15;
        guards_h[k] = f_down(e1 - band);
        guards_h[ne + k] = f_up(e1 + band);
    }
    for (int k = ne - 2; k >= 0; k--) guards_h[k] = fminf(guards_h[k], guards_h[k + 1]);
    for (int k = 1; k < ne; k++) guards_h[ne + k] = fmaxf(guards_h[ne + k], guards_h[ne + k - 1]);
    const float bf = (float)b, gtop = guards_h[2 * ne - 1];
    if (!(gtop > bf) || !isfinite(gtop) || gtop > 1e36f) return false;
    uint32_t bb, bt;
    memcpy(&bb, &bf, 4);
    memcpy(&bt, &gtop, 4);
    // buckets per octave: the finest power of two (at most 2^12) that fits kLut8Max entries from
    // bucket(b) to the cap bucket
    int lg = g_eng.lut8_lg;
    while (lg > 4 && (int)((bt >> (23 - lg)) - (bb >> (23 - lg))) + 2 > kLut8Max) lg--;
    const int shift = 23 - lg;
    const int base = (int)(bb >> shift);
    const int nb = (int)(bt >> shift) + 1 - base;  // cap bucket: the first wholly beyond the last guard
    if (nb + 2 > kLut8Max) return false;
    const uint32_t bcap = (uint32_t)(base + nb) << shift, bcap2 = (uint32_t)(base + nb + 1) << shift;
    float cap, cap2;
    memcpy(&cap, &bcap, 4);
    memcpy(&cap2, &bcap2, 4);
    const int words = (nb + 2 + 3) / 4;
    // layout: a flagged entry lands half a row past the trash row, which must stay 4-byte aligned
    const int ls = choose_layout(mode, false, J->need_avg != 0, need_w, ne, nbins, words - 1).lane_stride;
    const int ew = 1 + (J->need_avg ? 2 : 0) + (need_w ? 2 : 0);
    if ((ew * ls) % 2 != 0) return false;
    const uint32_t row_bytes = (uint32_t)(4 * ew * ls);
    const float *glo = guards_h, *ghi = guards_h + ne;
    const uint32_t trash_e = (uint32_t)nbins << 1;
    int mlo = 0, mhi = 0;
    for (int t = 0; t <= nb; t++) {
        const uint32_t ulo = (uint32_t)(base + t) << shift;
        const uint32_t uhi = (((uint32_t)(base + t + 1)) << shift) - 1u;
        float vlo, vhi;
        memcpy(&vlo, &ulo, 4);
        memcpy(&vhi, &uhi, 4);
        while (mlo < ne && glo[mlo] <= vlo) mlo++;
        while (mhi < ne && glo[mhi] <= vhi) mhi++;
        uint32_t e;
        if (vhi < glo[0] || vlo >= ghi[ne - 1]) {
            e = trash_e;  // certainly below the first edge or at / beyond the last
        } else if (mlo == mhi && mlo >= 1 && mlo < ne && vlo >= ghi[mlo - 1] && vhi < ghi[ne - 1]) {
            e = (uint32_t)mlo << 1;  // certainly in bin mlo
        } else {
            e = trash_e | 1u;  // a guard band reaches into the bucket: exact path
        }
        lut_h[t] = (uint8_t)e;
    }
    for (int t = nb + 1; t < 4 * words; t++) lut_h[t] = (uint8_t)trash_e;
    // the second cap bucket (lanes 16-31 where two lanes share a column): the second trash row
    const bool cap_pair = ls < 32 && 2 * (nbins + 1) <= 255;
    if (cap_pair) lut_h[nb + 1] = (uint8_t)(2 * (nbins + 1));
    T->lut8 = 1;
    T->qbias = bf;
    T->qcap = cap;
    T->qcap2 = cap_pair ? cap2 : cap;
    T->shift = shift;
    T->base = base;
    T->lut_n = words - 1;
    T->ls = ls;
    T->row_bytes = row_bytes;
    T->trash = (uint32_t)nbins * row_bytes;
    T->trash_e = trash_e;
    T->q_floor = 0.f;
    return true;
}

// packed bin tables of one run: double edges[ne] | float guards[2 ne] | float ascale[ne] | u32 lut[]
static inline size_t tab_align(size_t v) { return (v + 15) / 16 * 16; }

static int build_tables(Workspace &W, const cf_job *J, int mode, int nbins, bool need_w, const double delta[3], Tables *T)
{
    cudaStream_t st = g_eng.stream;
    // coordinate error bounds
    const double dxy = sqrt(delta[0] * delta[0] + delta[1] * delta[1]);
    const double d3 = sqrt(dxy * dxy + delta[2] * delta[2]);
    T->dxy = dxy;
    T->d3 = d3;
    const double dlim = (mode == MODE_RPPI || mode == MODE_WP) ? dxy : d3;
    // guards: for theta the classified quantity is the squared chord 2*(1 - cos)
    const size_t ne = (size_t)J->nedges;
    T->guard_off = tab_align(sizeof(double) * ne);
    T->ascale_off = tab_align(T->guard_off + sizeof(float) * 2 * ne);
    T->lut_off = tab_align(T->ascale_off + sizeof(float) * ne);
    const size_t tab_max = T->lut_off + sizeof(uint32_t) * (kLutMax + 4);
    if (ensure_host(W.h_tab, tab_max) != EXIT_SUCCESS || ensure(W.tab, tab_max) != EXIT_SUCCESS) return EXIT_FAILURE;
    double *edges_h = (double *)W.h_tab.p;
    float *guards_h = (float *)((char *)W.h_tab.p + T->guard_off);
    float *ascale_h = (float *)((char *)W.h_tab.p + T->ascale_off);
    uint32_t *lut_h = (uint32_t *)((char *)W.h_tab.p + T->lut_off);
    memcpy(edges_h, J->edges, sizeof(double) * J->nedges);
    // fixed-point scale of the separation sums per separation bin m (values in [edge m-1, edge m)):
    // one term stays below 2^30, i.e. a relative resolution of 2^-30 of the bin's upper edge
    for (int m = 0; m < J->nedges; m++) {
        const int mm = m > 0 ? m : (J->nedges > 1 ? 1 : 0);
        double top = mode == MODE_THETA ? acos(fmax(-1.0, fmin(1.0, J->edges[mm]))) * 57.29577951308232
                                        : sqrt(fabs(J->edges[mm]));
        top = fmax(top * 1.01, 1e-30);
        int ex = 30 - (int)ceil(log2(top));
        ex = ex > 100 ? 100 : (ex < -100 ? -100 : ex);
        ascale_h[m] = (float)ldexp(1.0, ex);
    }
    T->lut8 = 0;
    T->qbias = 0.f;
    T->qcap = 0.f;
    T->qcap2 = 0.f;
    T->trash_e = 0;
    if ((mode == MODE_R3 || mode == MODE_THETA) && nbins <= 127 && g_eng.byte_table &&
        build_lut8(J, mode, nbins, need_w, dlim, guards_h, (uint8_t *)lut_h, T)) {
        CF_CUDA(cudaMemcpyAsync(W.tab.p, W.h_tab.p, T->lut_off + sizeof(uint32_t) * (T->lut_n + 1),
                                cudaMemcpyHostToDevice, st));
        return EXIT_SUCCESS;
    }
    for (int k = 0; k < J->nedges; k++) {
        double e = J->edges[k];
        double band;
        if (mode == MODE_THETA) {
            e = 2.0 * (1.0 - J->edges[k]);
            band = edge_band(e, dlim) + 8e-15;
        } else if (mode_is_mock(mode)) {
            band = mock_edge_band(mode, e, mock_smax(J, mode), fmax(delta[0], fmax(delta[1], delta[2])));
        } else {
            band = edge_band(e, dlim);
        }
        guards_h[k] = f_down(e - band);
        guards_h[J->nedges + k] = f_up(e + band);
    }
    // keep both guard arrays non-decreasing (widening a band is always safe)
    for (int k = J->nedges - 2; k >= 0; k--) guards_h[k] = fminf(guards_h[k], guards_h[k + 1]);
    for (int k = 1; k < J->nedges; k++) guards_h[J->nedges + k] = fmaxf(guards_h[J->nedges + k], guards_h[J->nedges + k - 1]);
    // bin lookup table on the float bits of the classified quantity: entry = byte offset of the
    // histogram row of the bucket's bin, or the trash row flagged (bit 31) when a guard boundary
    // (or a band) falls in the bucket
    const float qlo = fmaxf(guards_h[0], 1e-30f);
    T->q_floor = guards_h[0] <= 1e-30f ? 1e-30f : 0.f;
    const float qhi = fmaxf(guards_h[2 * J->nedges - 1], qlo);
    uint32_t blo, bhi;
    memcpy(&blo, &qlo, 4);
    memcpy(&bhi, &qhi, 4);
    // Bucket width: the finest that gives at most kLutMax buckets while the histogram layout
    // scores as well as with a table of kLutMax / 2 (same resident warps and column sharing; a
    // bucket holding a guard sends its pairs to the exact path, so finer buckets send fewer).
    auto lut_shift = [&](uint32_t limit) {
        int sh = 1;
        while (((bhi >> sh) - (blo >> sh)) + 1 > limit) sh++;
        return sh;
    };
    int shift = lut_shift(kLutMax / 2);
    {
        const int sh2 = lut_shift(kLutMax);
        const int n1 = (int)((bhi >> shift) - (blo >> shift)) + 1, n2 = (int)((bhi >> sh2) - (blo >> sh2)) + 1;
        if (sh2 < shift &&
            layout_score(choose_layout(mode, false, J->need_avg != 0, need_w, J->nedges, nbins, n2), mode, J->need_avg != 0,
                         need_w) >=
                layout_score(choose_layout(mode, false, J->need_avg != 0, need_w, J->nedges, nbins, n1), mode,
                             J->need_avg != 0, need_w))
            shift = sh2;
    }
    const int base = (int)(blo >> shift);
    const int n = (int)((bhi >> shift) - (blo >> shift)) + 1;
    // row byte offsets: the layout (private columns or shared row) is fixed before the launch
    const int ls = choose_layout(mode, false, J->need_avg != 0, need_w, J->nedges, nbins, n).lane_stride;
    const uint32_t ostride = mode_two_d(mode) ? (uint32_t)(J->npibin + 1) : 1u;
    const int ew = 1 + (J->need_avg ? 2 : 0) + (need_w ? 2 : 0);  // words per histogram entry
    const uint32_t row_bytes = (uint32_t)(4 * ew * ls);
    const uint32_t trash = (uint32_t)nbins * row_bytes;
    if ((size_t)(nbins + J->npibin + 2) * row_bytes >= (1u << 22)) CF_FAIL("internal: histogram rows beyond the table's offset field");
    const float *glo_h = guards_h, *ghi_h = guards_h + J->nedges;
    int mlo = 0, mhi = 0;  // both non-decreasing in the bucket index
    for (int t = 0; t < n; t++) {
        const uint32_t ulo = (uint32_t)(base + t) << shift;
        const uint32_t uhi = (((uint32_t)(base + t + 1)) << shift) - 1u;
        float vlo, vhi;
        memcpy(&vlo, &ulo, 4);
        memcpy(&vhi, &uhi, 4);
        while (mlo < J->nedges && glo_h[mlo] <= vlo) mlo++;
        while (mhi < J->nedges && glo_h[mhi] <= vhi) mhi++;
        const bool definite = (mlo == mhi) && mlo >= 1 && mlo < J->nedges && vlo >= ghi_h[mlo - 1] &&
                              vhi < ghi_h[J->nedges - 1];
        lut_h[t] = definite ? ((uint32_t)mlo * ostride * row_bytes | ((uint32_t)mlo << 22)) : (trash | 0x80000000u);
    }
    lut_h[n] = trash;  // reject: below the first bucket (q < rmin^2) or above the last (q >= rmax^2)
    CF_CUDA(cudaMemcpyAsync(W.tab.p, W.h_tab.p, T->lut_off + sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, st));
    T->lut_n = n;
    T->shift = shift;
    T->base = base;
    T->ls = ls;
    T->row_bytes = row_bytes;
    T->trash = trash;
    return EXIT_SUCCESS;
}

// GPU lattice over the data extent [lo, hi] (or the periodic length): columns of about rlim/2 in
// x and y, slabs of rlim_z / kZFine in z, a power-of-two FP32 grid q per axis and the coordinate error
// bound delta of the hi/lo split.
// Columns per rmax in x and y.  A task pairs a chunk of 32 set-1 points of one column with the
// z-window of each neighbour column; the candidates per chunk are the set-2 points in
//   sum over neighbour columns of  A * (e + 2 W),
// A the column area, e the z-extent of the chunk (32 points at the set-1 density, at most the
// box) and W the z reach of that column.  Dense set-1 catalogues favour narrow columns (small A),
// sparse ones wide columns (fewer neighbours, shorter chunks).
static int choose_rxy(const cf_job *J, const double ext[3])
{
    const double r = J->rmax_xy;
    double vol = 1.0;
    for (int a = 0; a < 3; a++) vol *= fmax(ext[a], 1e-300);
    const double rho1 = (double)J->n1 / vol;
    if (!(r > 0.0) || !(rho1 > 0.0) || !(ext[2] > 0.0)) return kRxy;
    double cost_of[4] = {INFINITY, INFINITY, INFINITY, INFINITY};
    for (int R = 1; R <= 3; R++) {
        const double s = r / R * (1.0 + 1e-6), A = s * s;
        const double e = fmin(kChunk / (rho1 * A), ext[2]);
        double cost = 0.0;
        for (int dx = -R; dx <= R; dx++) {
            for (int dy = -R; dy <= R; dy++) {
                const double rx = fmax(0.0, (double)(abs(dx) - 1)) * s, ry = fmax(0.0, (double)(abs(dy) - 1)) * s;
                const double d2 = rx * rx + ry * ry;
                if (d2 >= r * r) continue;
                double W = J->rmax_z;
                if (J->rmax_3d > 0.0) W = fmin(W, sqrt(fmax(0.0, J->rmax_3d * J->rmax_3d - d2)));
                cost += A * (e + 2.0 * W);
            }
        }
        cost_of[R] = cost;
    }
    int best = kRxy;  // the default unless another width is clearly cheaper
    for (int R = 1; R <= 3; R++)
        if (cost_of[R] < 0.97 * cost_of[best]) best = R;
    return best;
}

// Integer forms of the lattice geometry for the lattice kernels: fixed-point origins, the
// reference-lattice safe range and the extent-check keys.  Called after any change of origin,
// s, n, the reference lattice or the checked extent.
static void geom_keys(Geom &g)
{
    for (int a = 0; a < 3; a++) {
        g.o_hi[a] = fix_of(g.hi_origin[a], g.e_fix[a]);
        g.o_cell[a] = fix_of(g.origin[a], g.e_fix[a]);
        // reciprocal of the index step in fixed-point units S = (s / cdiv) / 2^e_fix, with the
        // largest shift k that keeps cell_mul = 2^(64+k) / S below 2^63
        if (g.cdiv[a] < 1) g.cdiv[a] = 1;
        if (g.tmax[a] < 1) g.tmax[a] = g.n[a] * g.cdiv[a];
        const double sw = g.s[a] / g.cdiv[a];
        const double S = ldexp(sw, -g.e_fix[a]);
        int k = ilogb(S) - 1;
        k = k < 0 ? 0 : (k > 63 ? 63 : k);
        const double m = ldexp(1.0, 64 + k) / S;
        g.cell_shift[a] = k;
        g.cell_mul[a] = m >= 0x1p64 ? ~0ull : (unsigned long long)m;
        // |cell - (x - origin)/s| <= t 2^-51 + 2^-k cells (rounding of the reciprocal, truncation)
        // plus the fixed-point rounding of x and of the origin (2^e_fix each)
        g.eps_cell[a] = ldexp(g.s[a] * (double)g.n[a], -50) + ldexp(sw, 1 - k) + ldexp(4.0, g.e_fix[a]);
        // coordinates in [ref_min - cell / 2, ref_min + (ref_n + 1/2) cells] get a reference cell in
        // [0, ref_n] before the reference's clamp of the top cell, whatever the FP64 rounding
        const double c = 1.0 / g.ref_inv[a];
        const double rl = g.ref_min[a] - 0.5 * c, rh = g.ref_min[a] + (g.ref_n[a] + 0.5) * c;
        if (g.ref_inv[a] > 0.0 && isfinite(c) && isfinite(rl) && isfinite(rh)) {
            g.k_ref_lo[a] = okey0(rl);
            g.k_ref_hi[a] = okey0(rh);
        } else {
            g.k_ref_lo[a] = ~0ull;  // empty: every point takes the FP64 test
            g.k_ref_hi[a] = 0ull;
        }
        g.o_ref[a] = fix_of(g.ref_min[a], g.e_fix[a]);
        const bool ref_ok = g.ref_inv[a] > 0.0 && isfinite(g.ref_inv[a]) && g.ref_inv[a] < 1e30;
        g.ref_inv_f[a] = ref_ok ? (float)g.ref_inv[a] : NAN;
        g.ref_tol_f[a] = ref_ok ? (float)(4.0 * ldexp(g.ref_inv[a], g.e_fix[a]) + 1e-30) : NAN;
        g.k_chk_lo[a] = okey0(g.chk_lo[a]);
        g.k_chk_hi[a] = okey0(g.chk_hi[a]);
    }
    g.k_chk_wmax = okey0(fabs(g.chk_wmax));
    g.k_chk_wmin = okey0(fabs(g.chk_wmin));
}

static int gpu_geometry(const cf_job *J, const cf_geometry &geo, const double lo[3], const double hi[3], Geom &g,
                        double delta[3])
{
    memset(&g, 0, sizeof(g));
    double span[3];
    const double rlim[3] = {J->rmax_xy, J->rmax_xy, J->rmax_z};
    double ext0[3];
    for (int a = 0; a < 3; a++) {
        const bool per = geo.periodic[a] && geo.wrap[a] > 0.0;
        ext0[a] = per ? geo.wrap[a] : hi[a] - lo[a];
    }
    const int rxy = choose_rxy(J, ext0);
    const int refine[3] = {rxy, rxy, kZFine};
    // estimate of the position error of the cell index (set exactly in geom_keys), and the cell
    // widening that keeps the neighbour reach at 'refine' cells with the search margins
    // (2 eps_cell per axis, the plane taking the larger of x and y) added to the radii
    double eps[3];
    for (int a = 0; a < 3; a++) eps[a] = ldexp(1.0, -40) * fmax(ext0[a], 0.0);
    const double eps_xy = fmax(eps[0], eps[1]);
    for (int a = 0; a < 3; a++) {
        const bool per = geo.periodic[a] && geo.wrap[a] > 0.0;
        double ext = hi[a] - lo[a];
        if (per) {
            // Points spanning more than the period: the reference counts them, but its cells at the
            // two ends of the axis then overlap across the periodic boundary, and its neighbour
            // pruning by cell bounds (utils/gridlink_impl.c.src:522-560, the min_dx / max_dz
            // tests of the pair kernels) drops some pairs in range there; that pruning is not
            // reproduced, so the call fails.
            if (ext > geo.wrap[a]) {
                CF_FAIL("points span %g along axis %d, more than the periodic length %g", ext, a, geo.wrap[a]);
            }
            ext = geo.wrap[a];
        }
        int n = 1;
        if (ext > 0.0 && rlim[a] > 0.0) {
            // cells slightly wider than rlim/refine so that the neighbour reach is exactly 'refine'
            const double slack = 1e-6 + 4.0 * (a < 2 ? eps_xy : eps[2]) / rlim[a];
            double nn = floor(ext / (rlim[a] / refine[a] * (1.0 + slack)));
            if (nn > 4096) nn = 4096;
            if (nn < 1) nn = 1;
            n = (int)nn;
        }
        g.n[a] = n;
        g.origin[a] = lo[a];
        g.hi_origin[a] = lo[a];
        g.s[a] = ext > 0.0 ? ext / n : 1.0;
        g.inv_s[a] = 1.0 / g.s[a];
        span[a] = fmax(ext, 1e-300) + (per ? 2.0 * geo.wrap[a] : 0.0);
        g.q[a] = pow2_ceil(span[a]) * ldexp(1.0, -23);
        if (mode_is_mock(J->mode)) {
            // survey positions keep their offset from the observer in the split (the line of sight
            // x_i + x_j is then accurate to a few ulps of its own length): |hi| <= max |x| < 2^23 q
            g.hi_origin[a] = 0.0;
            g.q[a] = pow2_ceil(fmax(fmax(fabs(lo[a]), fabs(hi[a])), 1e-300)) * ldexp(1.0, -22);
        }
        // the fixed-point step 2^e_fix = q 2^-31 stays a normal float
        if (g.q[a] < ldexp(1.0, -95)) g.q[a] = ldexp(1.0, -95);
        if (g.q[a] > ldexp(1.0, 100)) CF_FAIL("coordinates of magnitude %g are out of range", fmax(fabs(lo[a]), fabs(hi[a])));
        g.inv_q[a] = 1.0 / g.q[a];
        g.e_fix[a] = ilogb(g.q[a]) - 31;
        g.q_f[a] = (float)g.q[a];
        g.rho_f[a] = ldexpf(1.0f, g.e_fix[a]);
        const double maxabs = fmax(fabs(lo[a]), fabs(hi[a])) + (per ? geo.wrap[a] : 0.0);
        delta[a] = 1.5 * g.q[a] + ldexp(1.0, -49) * (maxabs + span[a]);
        g.ref_min[a] = geo.ref_min[a];
        g.ref_inv[a] = geo.ref_inv[a];
        g.ref_n[a] = geo.ref_nmesh[a] > 0 ? geo.ref_nmesh[a] : 1;
    }
    // cap the total number of cells (z slabs first, then columns)
    while ((double)g.n[0] * g.n[1] * g.n[2] > (double)(1u << 24) && g.n[2] > 1) {
        g.n[2] = (g.n[2] + 1) / 2;
        const double ext = (geo.periodic[2] && geo.wrap[2] > 0.0) ? geo.wrap[2] : hi[2] - lo[2];
        g.s[2] = ext > 0.0 ? ext / g.n[2] : 1.0;
        g.inv_s[2] = 1.0 / g.s[2];
    }
    while ((double)g.n[0] * g.n[1] * g.n[2] > (double)(1u << 24)) {
        for (int a = 0; a < 2; a++) {
            g.n[a] = (g.n[a] + 1) / 2;
            const double ext = (geo.periodic[a] && geo.wrap[a] > 0.0) ? geo.wrap[a] : hi[a] - lo[a];
            g.s[a] = ext > 0.0 ? ext / g.n[a] : 1.0;
            g.inv_s[a] = 1.0 / g.s[a];
        }
    }
    g.check_ref_bounds = (J->rule.kind == CF_REF_BOX) ? 1 : 0;
    geom_keys(g);
    return EXIT_SUCCESS;
}

// Neighbour-search parameters of the work list: reach in columns and the z / 3-D limits, with
// margins that cover the rounding of the cell assignment.  sub > 1: the geometry of the j lattice
// whose columns split every lattice column sub x sub (offsets counted from the chunk column's
// first split column).
static int task_geometry(const cf_job *J, const cf_geometry &geo, const Geom &g, const double lo[3], const double hi[3],
                         bool autocorr, int mode, TaskGeom &G, int sub = 1)
{
    // prune margins cover the rounding of the cell assignment only (the FP32 error bounds of the
    // pair kernels matter for classification, not for which neighbours are visited)
    double maxabs_all = 0.0;
    for (int a = 0; a < 3; a++) maxabs_all = fmax(maxabs_all, fmax(fabs(lo[a]), fabs(hi[a])) + (geo.periodic[a] ? geo.wrap[a] : 0.0));
    // ... plus twice the position error of the FP32 cell index of each point
    const double margin_xy = 1e-9 * fmax(g.s[0], g.s[1]) + 1e-13 * maxabs_all + 2.0 * fmax(g.eps_cell[0], g.eps_cell[1]);
    const double margin_z = 1e-9 * g.s[2] + 1e-13 * maxabs_all + 2.0 * g.eps_cell[2];
    memset(&G, 0, sizeof(G));
    G.sub = sub;
    G.nx = g.n[0] * sub;
    G.ny = g.n[1] * sub;
    G.nz = g.n[2];
    for (int a = 0; a < 3; a++) G.periodic[a] = geo.periodic[a] && geo.wrap[a] > 0.0;
    G.autocorr = autocorr;
    G.mode = mode;
    G.s[0] = g.s[0] / sub;
    G.s[1] = g.s[1] / sub;
    G.s[2] = g.s[2];
    G.rmax_xy = J->rmax_xy + margin_xy;
    G.rmax_z = J->rmax_z + margin_z;
    G.rmax_3d = J->rmax_3d > 0.0 ? J->rmax_3d + fmax(margin_xy, margin_z) : 0.0;
    G.reach_x = (int)ceil(G.rmax_xy / G.s[0]);
    G.reach_y = (int)ceil(G.rmax_xy / G.s[1]);
    if (G.reach_x > 64 * sub || G.reach_y > 64 * sub) CF_FAIL("internal: neighbour reach too large");
    const int ny = 2 * G.reach_y + sub, ncoff = (2 * G.reach_x + sub) * ny;
    G.ntab = 0;
    if (ncoff <= kWzTab) {
        for (int c = 0; c < ncoff; c++) {
            const int wz = column_wz(G, c / ny - G.reach_x, c % ny - G.reach_y);
            G.wz_tab[c] = (int16_t)(wz > 32767 ? 32767 : wz);
        }
        G.ntab = ncoff;
    }
    return EXIT_SUCCESS;
}

// launch grid of the task kernels: chunk slots along x, stencil columns along y
static dim3 task_grid(const TaskGeom &G, uint32_t nslots)
{
    return dim3(nslots ? (nslots + 127) / 128 : 1u, (unsigned)((2 * G.reach_x + 1) * (2 * G.reach_y + 1)));
}

// Bin, band and accumulator constants of the pair kernels (everything but the buffers).
static void pair_constants(PairArgs &A, const cf_job *J, int mode, int nbins, bool autocorr, const TaskGeom &G,
                           const cf_geometry &geo, const Geom &g, const double delta[3], const Tables &T,
                           const double wmax[2], Workspace &W)
{
    A.nedges = J->nedges;
    A.guard_search_top = 0;
    while (2 * A.guard_search_top + (A.guard_search_top == 0) <= J->nedges - 1)
        A.guard_search_top = A.guard_search_top ? 2 * A.guard_search_top : 1;
    A.nbins = nbins;
    A.npibin = J->npibin;
    A.autocorr = autocorr;
    A.fma_formula = J->fma_formula;
    A.chord_formula = J->chord_formula;
    A.theta_series = 0;
    if (mode == MODE_THETA && J->nedges > 0) {
        const double cmin = J->edges[J->nedges - 1];  // cos of the largest angle counted
        A.theta_series = 0.5 * sqrt(fmax(0.0, 2.0 * (1.0 - cmin))) <= 0.2 ? 1 : 0;
    }
    for (int a = 0; a < 3; a++) {
        for (int m = -1; m <= 1; m++) {
            const double o = (G.periodic[a]) ? m * geo.wrap[a] : 0.0;
            const double oh = rint(o * g.inv_q[a]) * g.q[a];
            A.odbl[a][m + 1] = o;
            A.ohi[a][m + 1] = (float)oh;
            A.olo[a][m + 1] = (float)(o - oh);
        }
    }
    const double dxy = T.dxy, d3 = T.d3;
    A.g_lut = (const uint32_t *)((const char *)W.tab.p + T.lut_off);
    A.g_ascale = (const float *)((const char *)W.tab.p + T.ascale_off);
    A.rbin_div = mode_two_d(mode) ? J->npibin + 1 : 1;
    A.trash_off = T.trash;
    A.row_bytes = T.row_bytes;
    A.lane_stride_hint = T.ls;
    A.lut_shift = T.shift;
    A.lut_base = T.base;
    A.lut_mul = 1u << (32 - T.shift);
    A.lut_negbase = (uint32_t)(-T.base);
    A.lut_n = T.lut_n;
    A.q_floor = T.q_floor;
    A.lut8 = T.lut8;
    A.q_bias = T.qbias;
    A.q_cap = T.qcap;
    A.lut8_base = (uint32_t)T.base;
    A.half_row = T.row_bytes / 2;
    A.trash_e = T.trash_e;
    A.q_cap2 = T.qcap2;
    A.prune_r2 = FLT_MAX;  // the pruning kernels always test the box: no radius keeps every point
    A.prune_z = FLT_MAX;
    const bool prunes = (T.lut8 && (mode == MODE_R3 || mode == MODE_THETA)) || mode == MODE_RPPI || mode == MODE_WP ||
                        mode == MODE_SMU || mode_is_mock(mode);
    if (prunes && J->nedges > 0) {
        // the largest classified value in range: r^2 (rp^2, s^2), the squared chord, or (survey
        // modes) the squared separation cut beyond which every pair is rejected
        double top = 0.0;
        for (int k = 0; k < J->nedges; k++)
            top = fmax(top, mode == MODE_THETA ? 2.0 * (1.0 - J->edges[k]) : J->edges[k]);
        if (mode_is_mock(mode)) top = mock_s2_cut(J, mode);
        const double rp = (sqrt(top) + 4.0 * d3) * (1.0 + 1e-5);
        if (isfinite(rp) && rp * rp < 1e30) A.prune_r2 = f_up(rp * rp);
    }
    A.g_edges = (const double *)W.tab.p;
    A.g_guard = (const float *)((const char *)W.tab.p + T.guard_off);
    A.dz_err = (float)(2.0 * delta[2]);
    A.dxy_err = (float)(2.0 * dxy);
    if (mode_is_mock(mode)) {
        const double S = mock_smax(J, mode), qm = fmax(delta[0], fmax(delta[1], delta[2]));
        const double u = 5.9604644775390625e-08;
        A.s2_cut_f = f_up(mock_s2_cut(J, mode));
        A.l2_min_f = f_up(4.0 * S * S * (1.0 + 1e-5));
        const double epi = mock_pi_err(S, qm);
        if (mode == MODE_RPPI_MOCK) {
            A.pimax = J->pimax;
            A.inv_dpi = 1.0 / (J->pimax / J->npibin);
            A.pimax_lo_f = f_down(J->pimax - 2.0 * epi);
            A.pimax_hi_f = f_up(J->pimax + 2.0 * epi);
            A.inv_dpi_f = (float)A.inv_dpi;
            A.pibin_band = (float)(2.0 * (epi * A.inv_dpi + 3.0 * 5.96e-8 * (double)J->npibin + 1e-12));
            A.inv_dpi256_f = (float)(A.inv_dpi * 256.0);
            A.pi_band_q = (int)ceil(A.pibin_band * 256.0) + 2;
            if ((double)J->npibin * 256.0 > 4.0e6 || A.pi_band_q > 100) A.pi_band_q = 128;  // everything slow
        } else {
            A.sqr_mu_max = J->mu_max * J->mu_max;
            A.inv_dmu = 1.0 / (J->mu_max / J->npibin);
            A.mu_max_f = (float)J->mu_max;
            A.inv_dmu_f = (float)A.inv_dmu;
            // |mu_f - mu| <= |pi_f - pi| / |s| + mu (8u + 5u + u) + 3.5uq / |s|
            A.mu_band_abs = (float)(2.0 * (4.0 * u * qm + 3.5 * u * qm));
            A.mu_band_rel = (float)(2.0 * (24.0 * u + 14.0 * u) + 1e-12);
        }
    }
    if (mode == MODE_RPPI || mode == MODE_WP) {
        A.pimax = J->pimax;
        const double dpi = J->pimax / J->npibin;
        A.inv_dpi = 1.0 / dpi;
        const double bz = 2.0 * delta[2] + 1e-14 * J->pimax;
        A.pimax_lo_f = f_down(J->pimax - 2.0 * bz);
        A.pimax_hi_f = f_up(J->pimax + 2.0 * bz);
        A.inv_dpi_f = (float)A.inv_dpi;
        // |t_f32 - t_ref| <= |dz err| * inv_dpi + FP32 rounding of the product (relative 2^-23 of t <= npibin)
        A.pibin_band = (float)(2.0 * (bz * A.inv_dpi + 3.0 * 5.96e-8 * (double)J->npibin + 1e-12));
        if (mode == MODE_WP) A.pibin_band = 0.f;
        // fast path: round(|dz| * 256 / dpi) must stay below 2^22 for the magic-constant rounding
        A.inv_dpi256_f = (float)(A.inv_dpi * 256.0);
        A.pi_band_q = (int)ceil(A.pibin_band * 256.0) + 2;
        if ((double)J->npibin * 256.0 > 4.0e6 || A.pi_band_q > 100) A.pi_band_q = 128;  // everything slow
        A.prune_z = A.pimax_hi_f;  // |dz| at or above it: rejected by the FP32 test itself
    }
    if (mode == MODE_SMU) {
        A.sqr_mu_max = J->mu_max * J->mu_max;
        const double dmu = J->mu_max / J->npibin;
        A.inv_dmu = 1.0 / dmu;
        A.mu_max_f = (float)J->mu_max;
        A.inv_dmu_f = (float)A.inv_dmu;
        A.mu_band_abs = (float)(2.0 * (delta[2] + d3) * 2.0 + 1e-12);
    }
    // weight sums: one term wi * wj stays below 2^30 (relative resolution 2^-30 of the largest product)
    const double w2 = fmax(wmax[0] * wmax[1], 1e-30) * 1.01;
    int sw = 30 - (int)ceil(log2(w2));
    if (sw > 100) sw = 100;
    A.w_scale_f = (float)ldexp(1.0, sw);
    A.w_unscale = ldexp(1.0, -sw);

}

// Split of the j lattice's columns (1: none) and its slab merge (*zdiv), DD(r) and xi only.
// CF_COLUMN_SPLIT=<split>[,<slab merge>] fixes them (read on every call).  Otherwise a cost model
// in pair evaluations per i point: the j points of every window (split columns against the
// chunk column's reach, z windows widened to whole merged slabs), padding per range, the
// packed path's per-pair overhead, the split lattice's extra build (cells, and for an
// auto-correlation a second lattice of the same points), and the box pruning of the unsplit
// byte-table kernel.  The j lattice keeps within 2^26 cells.
static int choose_split(const cf_job *J, const Geom &g, int64_t n1, int64_t n2, bool autocorr, int mode, int *zdiv)
{
    *zdiv = 1;
    if (mode != MODE_R3) return 1;
    const double cells_c = (double)g.n[0] * g.n[1] * g.n[2];
    // the j lattice within 2^26 cells, and its range records (at most one per chunk and split
    // column within reach, 16 bytes each) within 2 GB
    const double chunks = (double)n1 / kChunk + (double)g.n[0] * g.n[1];
    auto fits = [&](int sub, int zd) {
        const double rx = ceil(J->rmax_xy * sub / g.s[0]), ry = ceil(J->rmax_xy * sub / g.s[1]);
        const double recs = chunks * (2.0 * rx + sub) * (2.0 * ry + sub) * (autocorr ? 0.5 : 1.0) * 16.0;
        return cells_c * sub * sub / zd <= (double)(1u << 26) && recs <= 2.0 * (1u << 30);
    };
    if (g_eng.tune_force > 0) {  // the autotuner's candidate or its choice
        int sub = g_eng.tune_force;
        const int zd = g_eng.tune_zdiv;
        while (sub > 1 && !fits(sub, zd)) sub--;
        *zdiv = sub > 1 ? zd : 1;
        return sub;
    }
    const char *e = getenv("CF_COLUMN_SPLIT");
    if (e) {
        int sub = 1, zd = 1;
        const int k = sscanf(e, "%d,%d", &sub, &zd);
        if (k >= 1 && sub >= 1 && sub <= 4) {
            if (k < 2 || !(zd == 1 || zd == 2 || zd == 4 || zd == 8)) zd = 1;
            while (sub > 1 && !fits(sub, zd)) sub--;
            *zdiv = sub > 1 ? zd : 1;
            return sub;
        }
    }
    const double vol = g.s[0] * g.n[0] * g.s[1] * g.n[1] * g.s[2] * g.n[2];
    const double rho1 = (double)n1 / vol, rho2 = (double)(autocorr ? n1 : n2) / vol;
    const double r = J->rmax_xy, rz = J->rmax_z, r3 = J->rmax_3d;
    if (!(vol > 0.0) || !(rho1 > 0.0) || !(r > 0.0)) return 1;
    const double Ac = g.s[0] * g.s[1];
    const double ez = fmin(kChunk / (rho1 * Ac), g.s[2] * g.n[2]);  // a chunk's z span
    auto reach_w = [&](double d2) {                                     // z reach at plane distance^2
        double W = rz;
        if (r3 > 0.0) W = fmin(W, sqrt(fmax(0.0, r3 * r3 - d2)));
        return W;
    };
    const double kPad = 8.0, kItemPad = 16.0, kPackedCost = 1.12, kBuildPerPoint = 100.0, kPerCell = 7.0,
                 kPruneKeep = 0.7;
    auto windows = [&](int sub, int zd) {  // j points per i point, padding included
        const double sf0 = g.s[0] / sub, sf1 = g.s[1] / sub, Af = sf0 * sf1;
        const int rx = (int)ceil(r / sf0), ry = (int)ceil(r / sf1);
        double pts = 0.0, ranges = 0.0;
        for (int du = -rx; du <= sub - 1 + rx; du++) {
            for (int dv = -ry; dv <= sub - 1 + ry; dv++) {
                const int pdx = (int)floor((double)du / sub), pdy = (int)floor((double)dv / sub);
                const bool own = pdx == 0 && pdy == 0;
                if (autocorr && (pdx < 0 || (pdx == 0 && pdy < 0))) continue;
                const int gx = du < 0 ? -du - 1 : (du >= sub ? du - sub : 0);
                const int gy = dv < 0 ? -dv - 1 : (dv >= sub ? dv - sub : 0);
                const double d2 = (gx * sf0) * (gx * sf0) + (gy * sf1) * (gy * sf1);
                if (d2 >= r * r) continue;
                const double W = reach_w(d2);
                if (autocorr && own) {
                    // own column: forward half, from the i lattice (unsplit, unmerged slabs)
                    pts += Af * rho2 * (ez + W);
                    if (du == 0 && dv == 0) ranges += 1.0;
                    continue;
                }
                pts += Af * rho2 * (ez + 2.0 * W + (zd - 1) * g.s[2]);
                ranges += 1.0;
            }
        }
        return sub == 1 ? pts + kPad * ranges : pts + kItemPad + (autocorr ? kPad : 0.0);
    };
    // the unsplit byte-table kernel prunes j points by the chunk's bounding box (about 60-70 % of
    // its window points stay); the packed kernel of split columns does not
    const bool prunes = g_eng.byte_table && J->nedges >= 2 && J->nedges - 1 <= 127;
    double best = windows(1, 1) * (prunes ? kPruneKeep : 1.0);
    const double base = best;
    int bsub = 1, bzd = 1;
    for (int sub = 2; sub <= 4; sub++) {
        for (int zd = 1; zd <= 8; zd *= 2) {
            if (!fits(sub, zd)) continue;
            const double cells_j = ceil((double)g.n[2] / zd) * g.n[0] * g.n[1] * sub * sub;
            const double extra = (autocorr ? kBuildPerPoint : 0.0) +
                                 kPerCell * (cells_j - (autocorr ? 0.0 : cells_c)) / (double)n1;
            const double c = windows(sub, zd) * kPackedCost + extra;
            if (c < best) {
                best = c;
                bsub = sub;
                bzd = zd;
            }
        }
    }
    if (bsub > 1 && best > 0.95 * base) return 1;  // not clearly cheaper
    *zdiv = bzd;
    return bsub;
}

static int run_locked(cf_job *J, cf_hist *H)
{
    Workspace &W = g_eng.ws;
    if (engine_init() != EXIT_SUCCESS) return EXIT_FAILURE;
    cudaStream_t st = g_eng.stream;
    memset(&g_eng.last, 0, sizeof(g_eng.last));
    g_eng.launches = 0;
    g_eng.layout_packed = g_eng.layout_prune = false;
    const int mode = J->mode;
    const int nbins = mode_two_d(mode) ? J->nedges * (J->npibin + 1) : J->nedges;
    if (H->nbins != nbins) CF_FAIL("internal: histogram size mismatch (%d vs %d)", H->nbins, nbins);
    memset(H->npairs, 0, sizeof(uint64_t) * nbins);
    memset(H->avg, 0, sizeof(double) * nbins);
    memset(H->wsum, 0, sizeof(double) * nbins);
    const bool autocorr = J->autocorr != 0;
    const int64_t n1 = J->n1, n2 = autocorr ? J->n1 : J->n2;
    if (n1 <= 0 || n2 <= 0) return EXIT_SUCCESS;
    if (n1 >= (1ll << 31) || n2 >= (1ll << 31)) CF_FAIL("at most 2^31-1 points per set are supported");
    if (J->elem_size != 4 && J->elem_size != 8) CF_FAIL("element size must be 4 or 8");
    const bool isf = J->elem_size == 4;
    const bool need_w = J->need_weight != 0;

    CF_CUDA(cudaStreamSynchronize(st));  // pinned staging is reused: nothing of a failed call may be pending
    CF_CUDA(cudaEventRecord(g_eng.ev[0], st));
    // ---- upload + extent ----
    if (ensure(W.mm, sizeof(unsigned long long) * 2 * kMmSlots) != EXIT_SUCCESS) return EXIT_FAILURE;
    unsigned long long *mm = (unsigned long long *)W.mm.p;
    if (ensure_host(W.h_small, sizeof(unsigned long long) * 4 * kMmSlots) != EXIT_SUCCESS) return EXIT_FAILURE;
    unsigned long long *mm_init = (unsigned long long *)W.h_small.p;
    unsigned long long *mmh = mm_init + 2 * kMmSlots;
    for (int k = 0; k < 2 * kMmSlots; k++) mm_init[k] = mm_init_value(k);
    CF_CUDA(cudaMemcpyAsync(mm, mm_init, sizeof(unsigned long long) * 2 * kMmSlots, cudaMemcpyHostToDevice, st));
    const int nsets = autocorr ? 1 : 2;
    for (int s = 0; s < nsets; s++) {
        const int64_t n = s ? n2 : n1;
        const void *x = s ? J->x2 : J->x1, *y = s ? J->y2 : J->y1, *z = s ? J->z2 : J->z1;
        const void *w = need_w ? (s ? J->w2 : J->w1) : nullptr;
        if (!x || !y || !z || (need_w && !w)) CF_FAIL("NULL input array");
        int rc = isf ? upload_and_minmax<float>(W, s, n, x, y, z, w, J->inputs_on_device != 0, mm + kMmSlots * s)
                     : upload_and_minmax<double>(W, s, n, x, y, z, w, J->inputs_on_device != 0, mm + kMmSlots * s);
        if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    }
    const bool dev_float = isf;
    CF_CUDA(cudaMemcpyAsync(mmh, mm, sizeof(unsigned long long) * 2 * kMmSlots, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    CF_CHECK_INTERRUPT();
    double lo[3], hi[3], wmax[2] = {0, 0}, wmin[2] = {0, 0};
    for (int a = 0; a < 3; a++) {
        lo[a] = ord_dec(mmh[2 * a]);
        hi[a] = ord_dec(mmh[2 * a + 1]);
        if (nsets == 2) {
            lo[a] = fmin(lo[a], ord_dec(mmh[kMmSlots + 2 * a]));
            hi[a] = fmax(hi[a], ord_dec(mmh[kMmSlots + 2 * a + 1]));
        }
    }
    wmax[0] = ord_dec(mmh[6]);
    wmax[1] = nsets == 2 ? ord_dec(mmh[kMmSlots + 6]) : wmax[0];
    wmin[0] = mm_wmin(mmh);
    wmin[1] = nsets == 2 ? mm_wmin(mmh + kMmSlots) : wmin[0];
    if (mmh[7] != 0 || (nsets == 2 && mmh[kMmSlots + 7] != 0)) CF_FAIL("non-finite input coordinates");
    for (int a = 0; a < 3; a++) {
        if (!isfinite(lo[a]) || !isfinite(hi[a])) CF_FAIL("non-finite input coordinates");
    }
    cf_geometry geo;
    if (cf_resolve_geometry(&J->rule, lo, hi, &geo) != EXIT_SUCCESS) return EXIT_FAILURE;
    J->geom = geo;

    // ---- GPU lattice geometry ----
    Geom g;
    double delta[3];
    if (gpu_geometry(J, geo, lo, hi, g, delta) != EXIT_SUCCESS) return EXIT_FAILURE;
    const uint32_t ncols = (uint32_t)g.n[0] * g.n[1];
    const uint32_t ncells = ncols * (uint32_t)g.n[2];
    g_eng.last.num_cells = (int)ncells;

    // ---- lattices ----
    const bool w_exact = need_w && weights_wide(wmax, wmin);
    // points outside the reference lattice on a periodic axis (xi / wp lattice the box [0, L) and
    // take points up to a cell past its edges into the edge cells): the reference's cell-pair list
    // can leave out pairs in range across the periodic boundary, and every pair then takes the FP64
    // kernel, which applies the reference's cell links
    bool ref_links = false;
    for (int a = 0; a < 3; a++) {
        if (!(geo.periodic[a] && geo.wrap[a] > 0.0)) continue;
        if (J->rule.kind == CF_REF_BOX && (lo[a] < geo.ref_min[a] || hi[a] > geo.ref_min[a] + geo.wrap[a]))
            ref_links = true;
    }
    const bool f64 = g_eng.precision == CF_PRECISION_FP64 || !has_f32_path(mode) || w_exact || ref_links;
    g.write_lo = (J->need_avg != 0 || mode_is_mock(mode)) ? 1 : 0;
    // j points from a lattice whose columns split every lattice column jsub x jsub (FP32 path):
    // the neighbour windows then follow each chunk's sphere of reach more closely.  Both lattices
    // take their column from the same fixed-point index (the i lattice's is that index / jsub), so
    // a split column lies inside exactly one lattice column.
    int zdiv = 1;
    const int jsub = f64 ? 1 : choose_split(J, g, n1, n2, autocorr, mode, &zdiv);
    g_eng.layout_packed = jsub > 1;  // the histogram layouts of this count (tables and launch)
    g_eng.layout_prune = mode == MODE_R3 || mode == MODE_THETA || mode == MODE_RPPI || mode == MODE_WP || mode == MODE_SMU ||
                         mode_is_mock(mode);
    Geom gj = g;
    uint32_t ncells_j = ncells;
    if (jsub > 1) {
        // the i lattice: columns of jsub x jsub index steps; the j lattice: one column per step,
        // slabs of zdiv i-lattice slabs (the last one possibly shorter)
        g.cdiv[0] = g.cdiv[1] = jsub;
        g.cdiv[2] = 1;
        for (int a = 0; a < 3; a++) g.tmax[a] = g.n[a] * g.cdiv[a];
        geom_keys(g);
        gj = g;
        for (int a = 0; a < 2; a++) {
            gj.n[a] = g.n[a] * jsub;
            gj.s[a] = g.s[a] / jsub;
            gj.inv_s[a] = 1.0 / gj.s[a];
            gj.cdiv[a] = 1;
        }
        gj.n[2] = (g.n[2] + zdiv - 1) / zdiv;
        gj.s[2] = g.s[2] * zdiv;
        gj.inv_s[2] = 1.0 / gj.s[2];
        gj.cdiv[2] = zdiv;
        geom_keys(gj);
        if (autocorr) gj.check_ref_bounds = 0;  // the i lattice already checks these points
        ncells_j = (uint32_t)gj.n[0] * (uint32_t)gj.n[1] * (uint32_t)gj.n[2];
    }
    const bool split_auto = autocorr && jsub > 1;  // a second lattice of the same points
    if (ensure(W.res, res_bytes(nbins)) != EXIT_SUCCESS) return EXIT_FAILURE;
    const ResView R = res_view(W.res.p, nbins);
    unsigned long long *oob = R.oob;
    CF_CUDA(cudaMemsetAsync(R.flags, 0, sizeof(unsigned long long) * 5, st));  // flags, oob, extent, records
    CF_CUDA(cudaEventRecord(g_eng.ev[6], st));  // the lattice build (gridlink) proper
    // an auto-correlation's split lattice: its cells in set 2's buffers, its records after the n1
    // records of the i lattice (set 1's buffers hold both), so that the j points of the own
    // column and of the split columns index one array
    if (split_auto && ensure_points(W.set[0], 2 * n1) != EXIT_SUCCESS) return EXIT_FAILURE;
    for (int s = 0; s < nsets + (split_auto ? 1 : 0); s++) {
        const int64_t n = (s && !autocorr) ? n2 : n1;
        const Geom &gs = s == 1 ? gj : g;
        const uint32_t nc = s == 1 ? ncells_j : ncells;
        int rc;
        if (s == 1 && autocorr) {
            SetBufs &B1 = W.set[1];
            if (ensure(B1.cellid_u, sizeof(uint32_t) * n1) || ensure(B1.fill, sizeof(uint32_t) * n1)) return EXIT_FAILURE;
            const SetBufs &B0 = W.set[0];
            rc = dev_float ? build_lattice_at<float>(W, B1, n1, 0, (const float *)B0.in[0], (const float *)B0.in[1],
                                                     (const float *)B0.in[2], need_w ? (const float *)B0.in[3] : nullptr,
                                                     gs, nc, oob, &W.set[0], n1)
                           : build_lattice_at<double>(W, B1, n1, 0, (const double *)B0.in[0], (const double *)B0.in[1],
                                                      (const double *)B0.in[2], need_w ? (const double *)B0.in[3] : nullptr,
                                                      gs, nc, oob, &W.set[0], n1);
        } else {
            rc = dev_float ? build_lattice<float>(W, s, n, need_w, gs, nc, oob)
                           : build_lattice<double>(W, s, n, need_w, gs, nc, oob);
        }
        if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    }
    CF_CUDA(cudaEventRecord(g_eng.ev[7], st));
    SetBufs &S1 = W.set[0];
    SetBufs &S2 = W.set[nsets - 1];                          // j records
    SetBufs &SC = W.set[(nsets == 2 || split_auto) ? 1 : 0];  // cells of the j lattice
    Tables T;
    if (build_tables(W, J, mode, nbins, need_w, delta, &T) != EXIT_SUCCESS) return EXIT_FAILURE;
    // CF_CHUNK_WALK=1 (FP32 DD(r) / xi with the byte table and unsplit columns): the pair kernel
    // walks every chunk's neighbourhood itself instead of taking a work list.  Off by default: its
    // in-kernel cell-offset lookups cost more than the list saves (north star 1.016 ms against
    // 0.862; the weighted 2M x 2M workload 5.19 against 5.24).
    const char *cwalk = getenv("CF_CHUNK_WALK");
    const bool walk = !f64 && mode == MODE_R3 && T.lut8 && jsub == 1 && !J->task_timer && g_eng.task_cap0 == 0 &&
                      cwalk && atoi(cwalk) == 1;

    // ---- neighbour-search geometry ----
    TaskGeom G;
    if (task_geometry(J, geo, g, lo, hi, autocorr, mode, G) != EXIT_SUCCESS) return EXIT_FAILURE;
    G.error = R.flags + 2;
    const int gap = chunk_gap(G, n1, ncols);
    // split j columns: packed tasks over the split columns (Gj), and an auto-correlation's own
    // column from the i lattice (Gown: the own column alone)
    TaskGeom Gj, Gown;
    size_t rcap = 0;
    int nsten = 0;
    if (jsub > 1) {
        if (task_geometry(J, geo, g, lo, hi, autocorr, mode, Gj, jsub) != EXIT_SUCCESS) return EXIT_FAILURE;
        Gj.error = G.error;
        Gj.zshift = zdiv == 8 ? 3 : zdiv == 4 ? 2 : zdiv == 2 ? 1 : 0;
        Gj.nzj = gj.n[2];
        // the stencil list: split-column offsets within reach (an auto-correlation's forward
        // neighbour columns only; its own column is listed from the i lattice)
        const int wxs = 2 * Gj.reach_x + jsub, wys = 2 * Gj.reach_y + jsub;
        if (ensure_host(W.h_sten, sizeof(int2) * (size_t)wxs * wys) != EXIT_SUCCESS ||
            ensure(W.sten, sizeof(int2) * (size_t)wxs * wys) != EXIT_SUCCESS)
            return EXIT_FAILURE;
        int2 *hs = (int2 *)W.h_sten.p;
        for (int u = 0; u < wxs; u++) {
            for (int v = 0; v < wys; v++) {
                const int du = u - Gj.reach_x, dv = v - Gj.reach_y;
                if (autocorr) {
                    const int pdx = (int)floor((double)du / jsub), pdy = (int)floor((double)dv / jsub);
                    if (pdx < 0 || (pdx == 0 && pdy <= 0)) continue;
                }
                const int wz = column_wz(Gj, du, dv);
                if (wz < 0) continue;
                hs[nsten++] = make_int2((int)(((uint32_t)du & 0xffffu) | ((uint32_t)dv << 16)), wz);
            }
        }
        if (nsten > 0) CF_CUDA(cudaMemcpyAsync(W.sten.p, hs, sizeof(int2) * nsten, cudaMemcpyHostToDevice, st));
        Gown = G;
        Gown.reach_x = Gown.reach_y = 0;
        const int wz0 = column_wz(G, 0, 0);
        Gown.wz_tab[0] = (int16_t)(wz0 > 32767 ? 32767 : wz0);
        Gown.ntab = 1;
        Gj.j_off = split_auto ? (uint32_t)n1 : 0u;
    }

    // ---- chunks: fixed slot range (empty slots hold 0 points), no host wait ----
    const uint64_t slots = chunk_slots((uint64_t)n1, ncols, g.n[2], gap);
    if (slots > 0xffffffffull) CF_FAIL("too many chunks (%llu)", (unsigned long long)slots);
    const uint32_t max_chunks = (uint32_t)slots;
    if (ensure(W.chunk_cnt, sizeof(uint32_t) * ncols) || ensure(W.chunk_off, sizeof(uint32_t) * ((size_t)ncols + 1)) ||
        ensure(W.chunk_begin, sizeof(uint32_t) * max_chunks) || ensure(W.chunk_info, sizeof(uint2) * max_chunks))
        return EXIT_FAILURE;
    CF_CUDA(cudaMemsetAsync(W.chunk_info.p, 0, sizeof(uint2) * max_chunks, st));
    k_col_chunks<<<(ncols + 7) / 8, 256, 0, st>>>((const uint32_t *)S1.cell_start.p, (int)ncols, g.n[2], gap,
                                                  (uint32_t *)W.chunk_cnt.p);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    if (scan_u32(W, (const uint32_t *)W.chunk_cnt.p, (uint32_t *)W.chunk_off.p, ncols, 0) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    k_chunk_emit<<<(ncols + 7) / 8, 256, 0, st>>>((const uint32_t *)S1.cell_start.p, (int)ncols, g.n[2], gap,
                                                      (const uint32_t *)W.chunk_off.p, max_chunks, G.error,
                                                      (uint32_t *)W.chunk_begin.p, (uint2 *)W.chunk_info.p,
                                                      0u, nullptr, 0);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());

    // ---- tasks: listed on the device in one pass into a buffer sized from earlier calls ----
    // capacity: what this lattice needed last time, else about one task per neighbour column
    const size_t guess = (size_t)max_chunks * (2 * G.reach_x + 1) * (2 * G.reach_y + 1) * 5 / 4 + 1024;
    size_t cap = W.tasks.cap / sizeof(Task);
    if (cap < guess) cap = guess;
    if (ensure(W.tasks, sizeof(Task) * cap) != EXIT_SUCCESS) return EXIT_FAILURE;
    cap = W.tasks.cap / sizeof(Task);
    if (cap > 0xffffffffu) cap = 0xffffffffu;
    if (g_eng.task_cap0 > 0 && g_eng.task_cap0 < cap) cap = g_eng.task_cap0;
    if (jsub > 1) {
        // range records: what this lattice needed last time, else about one per split column
        // within reach (the forward half for an auto-correlation); 32 spare records stay
        // readable past the last (the pair kernel reads records 32 at a time)
        const size_t ncj = (size_t)(2 * Gj.reach_x + jsub) * (2 * Gj.reach_y + jsub);
        const size_t rguess = (size_t)max_chunks * ncj / (autocorr ? 2 : 1) + 1024;
        rcap = W.recs.cap / sizeof(JRange);
        rcap = rcap > 32 ? rcap - 32 : 0;
        if (rcap < rguess) rcap = rguess;
        if (rcap > 0xffffffffu - 32) rcap = 0xffffffffu - 32;
        if (ensure(W.recs, sizeof(JRange) * (rcap + 32)) != EXIT_SUCCESS) return EXIT_FAILURE;
        if (g_eng.task_cap0 > 0 && g_eng.task_cap0 < rcap) rcap = g_eng.task_cap0;
    }

    // ---- pair-kernel arguments ----
    PairArgs A;
    memset(&A, 0, sizeof(A));
    A.hi1 = (const float4 *)S1.hi.p;
    A.lo1 = (const float4 *)S1.lo.p;
    A.d1 = (const double4_32a *)S1.dbl.p;
    A.ro1 = (const int2 *)S1.ro.p;
    A.hi2 = (const float4 *)S2.hi.p;
    A.lo2 = (const float4 *)S2.lo.p;
    A.d2 = (const double4_32a *)S2.dbl.p;
    A.ro2 = (const int2 *)S2.ro.p;
    A.ntask_dev = R.flags + 1;  // tasks listed (capped by the capacity in the kernel)
    pair_constants(A, J, mode, nbins, autocorr, G, geo, g, delta, T, wmax, W);
    A.w_exact = w_exact ? 1 : 0;
    A.ref_links = ref_links ? 1 : 0;
    for (int a = 0; a < 3; a++) {
        A.ref_n[a] = g.ref_n[a];
        A.ref_reach[a] = geo.refine_used[a];
    }
    A.g_cnt = R.cnt;
    A.g_avg = R.avg;
    A.g_w = R.w;
    A.g_stats = R.stats;
    A.task_counter = R.flags;
    if (ensure_host(W.h_hist, res_bytes(nbins)) != EXIT_SUCCESS) return EXIT_FAILURE;
    const ResView Rh = res_view(W.h_hist.p, nbins);

    J->task_times = nullptr;
    J->ntask_times = 0;
    for (int attempt = 0; attempt < 2; attempt++) {
        A.tasks = (const Task *)W.tasks.p;
        A.jrec = jsub > 1 ? (const JRange *)W.recs.p : nullptr;
        A.ntasks = (uint32_t)cap;
        A.task_clock = nullptr;
        if (J->task_timer) {
            if (ensure(W.task_clock, 2 * sizeof(unsigned long long) * cap) != EXIT_SUCCESS) return EXIT_FAILURE;
            A.task_clock = (unsigned long long *)W.task_clock.p;
        }
        if (walk) {
            // no work list
        } else if (jsub > 1) {
            if (autocorr) {
                k_task_list<<<task_grid(Gown, max_chunks), 128, 0, st>>>(
                    Gown, max_chunks, (const uint32_t *)W.chunk_begin.p, (const uint2 *)W.chunk_info.p,
                    (const uint32_t *)S1.cell_start.p, (Task *)W.tasks.p, (uint32_t)cap, R.flags);
                g_eng.launches++;
                CF_CUDA(cudaGetLastError());
            }
            k_item_list<<<((size_t)max_chunks * kItemLanes + 32 * kItemWarps - 1) / (32 * kItemWarps), 32 * kItemWarps,
                          nsten <= kItemStenShared ? sizeof(int2) * nsten : 0, st>>>(
                Gj, max_chunks, (const uint32_t *)W.chunk_begin.p, (const uint2 *)W.chunk_info.p,
                (const uint32_t *)SC.cell_start.p, (const int2 *)W.sten.p, nsten, (Task *)W.tasks.p, (uint32_t)cap,
                (JRange *)W.recs.p, (uint32_t)rcap, R.flags, R.recs);
        } else {
            k_task_list<<<task_grid(G, max_chunks), 128, 0, st>>>(G, max_chunks, (const uint32_t *)W.chunk_begin.p,
                                                                  (const uint2 *)W.chunk_info.p,
                                                                  (const uint32_t *)S2.cell_start.p, (Task *)W.tasks.p,
                                                                  (uint32_t)cap, R.flags);
        }
        if (!walk) {
            g_eng.launches++;
            CF_CUDA(cudaGetLastError());
        }
        CF_CUDA(cudaEventRecord(g_eng.ev[1], st));
        CF_CUDA(cudaMemsetAsync(W.res.p, 0, res_zero_bytes(nbins), st));  // sums, statistics, task counter
        int launched = 0;
        if (g_eng.test_signal > 0 && ++g_eng.pair_launches == g_eng.test_signal) raise(SIGINT);
        CF_CHECK_INTERRUPT();
        CF_CUDA(cudaEventRecord(g_eng.ev[2], st));
        if (walk ? launch_walk(A, J->need_avg != 0, need_w, G, (const uint32_t *)W.chunk_begin.p,
                               (const uint2 *)W.chunk_info.p, (const uint32_t *)S2.cell_start.p, max_chunks, &launched)
                 : launch_pairs(mode, A, f64, J->need_avg != 0, need_w, &launched))
            return EXIT_FAILURE;
        CF_CUDA(cudaEventRecord(g_eng.ev[3], st));
        CF_CUDA(cudaMemcpyAsync(W.h_hist.p, W.res.p, res_bytes(nbins), cudaMemcpyDeviceToHost, st));
        CF_CUDA(cudaEventRecord(g_eng.ev[4], st));
        CF_CUDA(cudaStreamSynchronize(st));
        CF_CHECK_INTERRUPT();
        if (*Rh.oob > 0) CF_FAIL("%llu particles are out of bounds. Check periodic wrapping?", *Rh.oob);
        if (Rh.flags[2] & 2u) CF_FAIL("internal: the chunks outgrew their slots");
        if (Rh.flags[2]) CF_FAIL("internal: neighbour search needed a periodic image beyond +-1");
        if (!Rh.flags[3]) break;
        // the work list outgrew the buffer: size it exactly and run the pair kernel again
        if (attempt == 1) CF_FAIL("internal: work list overflow after resizing");
        cap = (size_t)Rh.flags[1] + 1024;
        if (ensure(W.tasks, sizeof(Task) * cap) != EXIT_SUCCESS) return EXIT_FAILURE;
        cap = W.tasks.cap / sizeof(Task);
        if (cap > 0xffffffffu) cap = 0xffffffffu;
        if (jsub > 1) {
            rcap = (size_t)Rh.recs[0] + 1024;
            if (rcap > 0xffffffffu - 32) rcap = 0xffffffffu - 32;
            if (ensure(W.recs, sizeof(JRange) * (rcap + 32)) != EXIT_SUCCESS) return EXIT_FAILURE;
        }
        CF_CUDA(cudaMemsetAsync(R.flags + 1, 0, 3 * sizeof(uint32_t), st));  // task total, image error, overflow
        CF_CUDA(cudaMemsetAsync(R.recs, 0, sizeof(uint32_t), st));           // records
    }
    g_eng.last.tasks = Rh.flags[1];
    if (J->task_timer && Rh.flags[1] > 0) {
        // per-task timings: the task list and the timer records back to the host
        const size_t nt = Rh.flags[1];
        Task *th = (Task *)malloc(sizeof(Task) * nt);
        unsigned long long *ch = (unsigned long long *)malloc(2 * sizeof(unsigned long long) * nt);
        cf_task_time *out = (cf_task_time *)calloc(nt, sizeof(cf_task_time));
        if (!th || !ch || !out) {
            free(th);
            free(ch);
            free(out);
            CF_FAIL("out of host memory for the per-task timings");
        }
        if (cudaMemcpy(th, W.tasks.p, sizeof(Task) * nt, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(ch, W.task_clock.p, 2 * sizeof(unsigned long long) * nt, cudaMemcpyDeviceToHost) != cudaSuccess) {
            free(th);
            free(ch);
            free(out);
            CF_FAIL("could not read the per-task timings back");
        }
        const double ns_per_cycle = g_eng.clock_khz > 0 ? 1e6 / g_eng.clock_khz : 1.0;
        for (size_t t = 0; t < nt; t++) {
            const bool packed = (th[t].meta & kTaskPacked) != 0;
            out[t].n1 = (int64_t)(th[t].meta & 63u) + 1;
            out[t].n2 = packed ? (int64_t)(th[t].j_end & 2047u) + 1 : (int64_t)th[t].j_end - (int64_t)th[t].j_begin;
            out[t].time_in_ns = (int64_t)((double)ch[2 * t] * ns_per_cycle);
            out[t].i_first = (int)th[t].i_begin;
            out[t].j_first = packed ? -1 : (int)th[t].j_begin;
            out[t].warp = (int)ch[2 * t + 1];
        }
        free(th);
        free(ch);
        J->task_times = out;
        J->ntask_times = (int64_t)nt;
    }
    memcpy(H->npairs, Rh.cnt, sizeof(uint64_t) * nbins);
    memcpy(H->avg, Rh.avg, sizeof(double) * nbins);
    memcpy(H->wsum, Rh.w, sizeof(double) * nbins);
    float ms_pairs = 0.f, ms_grid = 0.f, ms_total = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms_pairs, g_eng.ev[2], g_eng.ev[3]));
    CF_CUDA(cudaEventElapsedTime(&ms_grid, g_eng.ev[6], g_eng.ev[7]));  // cell index, offsets, scatter
    CF_CUDA(cudaEventElapsedTime(&ms_total, g_eng.ev[0], g_eng.ev[4]));
    g_eng.last.pair_kernel_ms = ms_pairs;
    g_eng.last.gridlink_ms = ms_grid;
    g_eng.last.total_gpu_ms = ms_total;
    g_eng.last.pairs_evaluated = Rh.stats[0];
    g_eng.last.pairs_refined = Rh.stats[1];
    g_eng.last.pairs_slow = Rh.stats[2];
    g_eng.last.kernel_launches = g_eng.launches;
    g_eng.last.column_split = jsub;
    return EXIT_SUCCESS;
}


// ------------------------------------------------------------------------------------
// batched cross-correlations: many set-1 catalogues against one set-2 catalogue
// ------------------------------------------------------------------------------------
// One plan owns its workspace.  The set-1 catalogues are sorted one after another into one
// lattice (catalogue b at point offset pbase[b]); each catalogue gets a fixed range of chunk
// slots (unused slots hold empty chunks), so the whole work list is built without host waits;
// tasks carry their catalogue in Task::meta and the pair kernel flushes its per-warp histogram
// into that catalogue's slice of the global histogram.  The sequence is run once eagerly (to
// size the work list and, optionally, to time candidate histogram layouts) and then captured
// as a CUDA graph that every run replays.
struct BatchPlan {
    Workspace W;
    cf_job J;
    int nbatch = 0, mode = MODE_R3, nbins = 0;
    bool isf = false, need_w = false;
    int64_t *n1 = nullptr, *pbase = nullptr, total1 = 0;
    const void **x1 = nullptr, **y1 = nullptr, **z1 = nullptr, **w1 = nullptr;
    uint32_t *cbase = nullptr, total_slots = 0, nentries = 0, ncols = 0, ncells = 0;
    uint32_t task_cap = 0, ntasks = 0;
    Geom g;
    TaskGeom G;
    int gap = -1;  // z-slab gap that splits the catalogues' chunks (chunk_gap)
    // one lattice for all set-1 catalogues, chunk tasks with per-lane catalogues (k_pairs_chunks);
    // else one lattice and chunk range per catalogue and the per-column work list
    bool merged = false;
    Tables T;
    PairArgs A;
    cf_geometry geo;
    double delta[3], wmax[2], wmin[2];
    bool w_exact = false;   // weight products span too wide a range for the FP32 kernel's sums
    int ls = 0, warps = 0;  // chosen FP32 layout (0: scored)
    int kernels = 0;        // kernels in one run
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev[4];
    bool events = false;
};

template <typename T>
static int batch_lattices(BatchPlan &P)
{
    Workspace &W = P.W;
    cudaStream_t st = g_eng.stream;
    const ResView R = res_view(W.res.p, (size_t)P.nbatch * P.nbins);
    unsigned long long *oob = R.oob;
    Geom g1 = P.g, g2 = P.g;
    g1.extent_err = g2.extent_err = R.extent;
    g1.chk_wmax = P.wmax[0];
    g2.chk_wmax = P.wmax[1];
    g1.chk_wmin = P.w_exact ? 0.0 : P.wmin[0];
    g2.chk_wmin = P.w_exact ? 0.0 : P.wmin[1];
    geom_keys(g1);
    geom_keys(g2);
    g1.write_lo = g2.write_lo = (P.J.need_avg != 0 || mode_is_mock(P.mode)) ? 1 : 0;
    const T *w2 = P.need_w ? (const T *)P.J.w2 : nullptr;
    if (build_lattice_at<T>(W, W.set[1], P.J.n2, 0, (const T *)P.J.x2, (const T *)P.J.y2, (const T *)P.J.z2, w2, g2,
                            P.ncells, oob) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    const int nz = P.g.n[2];
    if (P.merged) {
        // every catalogue counted into one occupancy array, one scan, every catalogue scattered
        // (points carry their catalogue), one set of chunks
        SetBufs &B = W.set[0];
        if (ensure(B.count, sizeof(uint32_t) * (size_t)P.ncells) ||
            ensure(B.cell_start, sizeof(uint32_t) * ((size_t)P.ncells + 1)))
            return EXIT_FAILURE;
        CF_CUDA(cudaMemsetAsync(B.count.p, 0, sizeof(uint32_t) * (size_t)P.ncells, st));
        for (int b = 0; b < P.nbatch; b++)
            if (lattice_assign_at<T>(B, P.n1[b], P.pbase[b], (const T *)P.x1[b], (const T *)P.y1[b],
                                     (const T *)P.z1[b], g1, oob) != EXIT_SUCCESS)
                return EXIT_FAILURE;
        if (scan_u32(W, (const uint32_t *)B.count.p, (uint32_t *)B.cell_start.p, P.ncells, 0) != EXIT_SUCCESS)
            return EXIT_FAILURE;
        for (int b = 0; b < P.nbatch; b++) {
            const T *w = P.need_w ? (const T *)P.w1[b] : nullptr;
            if (lattice_scatter_at<T>(B, P.n1[b], P.pbase[b], 0, (const T *)P.x1[b], (const T *)P.y1[b],
                                      (const T *)P.z1[b], w, g1, b) != EXIT_SUCCESS)
                return EXIT_FAILURE;
        }
        k_col_chunks<<<(P.ncols + 7) / 8, 256, 0, st>>>((const uint32_t *)B.cell_start.p, (int)P.ncols, nz, P.gap,
                                                        (uint32_t *)W.chunk_cnt.p);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
        if (scan_u32(W, (const uint32_t *)W.chunk_cnt.p, (uint32_t *)W.chunk_off.p, P.ncols, 0) != EXIT_SUCCESS)
            return EXIT_FAILURE;
        k_chunk_emit<<<(P.ncols + 7) / 8, 256, 0, st>>>((const uint32_t *)B.cell_start.p, (int)P.ncols, nz, P.gap,
                                                        (const uint32_t *)W.chunk_off.p, P.total_slots, P.G.error,
                                                        (uint32_t *)W.chunk_begin.p, (uint2 *)W.chunk_info.p, 0u,
                                                        nullptr, 0);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
        return EXIT_SUCCESS;
    }
    for (int b = 0; b < P.nbatch; b++) {
        const T *w = P.need_w ? (const T *)P.w1[b] : nullptr;
        if (build_lattice_at<T>(W, W.set[0], P.n1[b], P.pbase[b], (const T *)P.x1[b], (const T *)P.y1[b],
                                (const T *)P.z1[b], w, g1, P.ncells, oob) != EXIT_SUCCESS)
            return EXIT_FAILURE;
        if (P.n1[b] == 0) continue;
        k_col_chunks<<<(P.ncols + 7) / 8, 256, 0, st>>>((const uint32_t *)W.set[0].cell_start.p, (int)P.ncols, nz,
                                                        P.gap, (uint32_t *)W.chunk_cnt.p);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
        if (scan_u32(W, (const uint32_t *)W.chunk_cnt.p, (uint32_t *)W.chunk_off.p, P.ncols, 0) != EXIT_SUCCESS)
            return EXIT_FAILURE;
        k_chunk_emit<<<(P.ncols + 7) / 8, 256, 0, st>>>(
            (const uint32_t *)W.set[0].cell_start.p, (int)P.ncols, nz, P.gap, (const uint32_t *)W.chunk_off.p,
            P.cbase[b + 1] - P.cbase[b], P.G.error,
            (uint32_t *)W.chunk_begin.p + P.cbase[b], (uint2 *)W.chunk_info.p + P.cbase[b], (uint32_t)P.pbase[b],
            (uint16_t *)W.chunk_cat.p + P.cbase[b], (uint16_t)b);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
    }
    return EXIT_SUCCESS;
}

// Records ev on the engine stream; inside a stream capture as an external event node, so that
// replays of the graph record it too.
static int record_event(cudaEvent_t ev)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    CF_CUDA(cudaStreamIsCapturing(g_eng.stream, &cs));
    if (cs == cudaStreamCaptureStatusActive) CF_CUDA(cudaEventRecordWithFlags(ev, g_eng.stream, cudaEventRecordExternal));
    else CF_CUDA(cudaEventRecord(ev, g_eng.stream));
    return EXIT_SUCCESS;
}

// The chunk-task pair kernel of a merged batch (layout: private columns, P.warps per block).
template <bool AVG, bool W>
static int launch_chunks_t(BatchPlan &P)
{
    const int fls = g_eng.force_ls, fw = g_eng.force_warps;
    g_eng.force_ls = 32;
    g_eng.force_warps = P.warps;
    const SmemLayout SL = choose_layout(MODE_R3, false, AVG, W, P.A.nedges, P.nbins, P.A.lut_n);
    g_eng.force_ls = fls;
    g_eng.force_warps = fw;
    if (SL.lane_stride != 32 || SL.lane_stride != P.A.lane_stride_hint)
        CF_FAIL("internal: the merged batch needs private histogram columns");
    auto kern = k_pairs_chunks<AVG, W, false>;
    int per_sm = 1;
    CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
    CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, SL.warps * 32, SL.total));
    if (per_sm < 1) per_sm = 1;
    kern<<<g_eng.num_sms * per_sm, SL.warps * 32, SL.total, g_eng.stream>>>(
        P.A, SL, P.G, (const uint32_t *)P.W.chunk_begin.p, (const uint2 *)P.W.chunk_info.p,
        (const uint32_t *)P.W.set[1].cell_start.p, P.total_slots);
    CF_CUDA(cudaGetLastError());
    g_eng.launches++;
    g_eng.last.blocks_per_sm = per_sm;
    g_eng.last.warps_per_block = SL.warps;
    g_eng.last.lane_stride = 32;
    return EXIT_SUCCESS;
}

static int launch_chunks(BatchPlan &P)
{
    const bool avg = P.J.need_avg != 0, w = P.need_w;
    if (avg && w) return launch_chunks_t<true, true>(P);
    if (avg) return launch_chunks_t<true, false>(P);
    if (w) return launch_chunks_t<false, true>(P);
    return launch_chunks_t<false, false>(P);
}

// Enqueues lattices and task counts (phase 0), or task emission, pair kernel and read-back
// (phase 1), on the engine stream.  No host waits inside either phase.  A merged batch has no
// work list: phase 0 builds the lattices and chunks, phase 1 runs the chunk-task kernel.
static int batch_enqueue(BatchPlan &P, int phase, bool timing)
{
    Workspace &W = P.W;
    cudaStream_t st = g_eng.stream;
    if (phase == 0) {
        CF_CUDA(cudaMemsetAsync(res_view(W.res.p, (size_t)P.nbatch * P.nbins).flags, 0, sizeof(unsigned long long) * 4,
                                st));  // flags, oob, extent
        CF_CUDA(cudaMemsetAsync(W.chunk_info.p, 0, sizeof(uint2) * P.total_slots, st));
        const int rc = P.isf ? batch_lattices<float>(P) : batch_lattices<double>(P);
        if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
        if (P.merged) return EXIT_SUCCESS;
        k_task_count<<<task_grid(P.G, P.total_slots), 128, 0, st>>>(
            P.G, P.total_slots, (const uint32_t *)W.chunk_begin.p, (const uint2 *)W.chunk_info.p,
            (const uint32_t *)W.set[1].cell_start.p, (uint32_t *)W.ntask.p);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
        return scan_u32(W, (const uint32_t *)W.ntask.p, (uint32_t *)W.task_off.p, P.nentries, 0);
    }
    if (P.merged) {
        const size_t nbm = (size_t)P.nbatch * P.nbins;
        CF_CUDA(cudaMemsetAsync(W.res.p, 0, res_zero_bytes(nbm), st));  // sums, statistics, chunk counter
        if (timing && record_event(P.ev[1]) != EXIT_SUCCESS) return EXIT_FAILURE;
        if (launch_chunks(P) != EXIT_SUCCESS) return EXIT_FAILURE;
        if (timing && record_event(P.ev[2]) != EXIT_SUCCESS) return EXIT_FAILURE;
        CF_CUDA(cudaMemcpyAsync(W.h_hist.p, W.res.p, res_bytes(nbm), cudaMemcpyDeviceToHost, st));
        return EXIT_SUCCESS;
    }
    k_task_emit<<<task_grid(P.G, P.total_slots), 128, 0, st>>>(
        P.G, P.total_slots, (const uint32_t *)W.chunk_begin.p, (const uint2 *)W.chunk_info.p,
        (const uint32_t *)W.set[1].cell_start.p, (const uint32_t *)W.task_off.p,
        (Task *)W.tasks.p, (const uint16_t *)W.chunk_cat.p, P.task_cap, res_view(W.res.p, (size_t)P.nbatch * P.nbins).flags);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    const size_t nb = (size_t)P.nbatch * P.nbins;
    CF_CUDA(cudaMemsetAsync(W.res.p, 0, res_zero_bytes(nb), st));  // sums, statistics, task counter
    if (timing && record_event(P.ev[1]) != EXIT_SUCCESS) return EXIT_FAILURE;
    int launched = 0;
    const bool f64 = g_eng.precision == CF_PRECISION_FP64 || P.w_exact;
    const int fls = g_eng.force_ls, fw = g_eng.force_warps;
    g_eng.force_ls = P.ls;
    g_eng.force_warps = P.warps;
    const int rc = launch_pairs(P.mode, P.A, f64, P.J.need_avg != 0, P.need_w, &launched);
    g_eng.force_ls = fls;
    g_eng.force_warps = fw;
    if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    if (timing && record_event(P.ev[2]) != EXIT_SUCCESS) return EXIT_FAILURE;
    CF_CUDA(cudaMemcpyAsync(W.h_hist.p, W.res.p, res_bytes(nb), cudaMemcpyDeviceToHost, st));
    return EXIT_SUCCESS;
}

// Checks the flags of a finished run and copies catalogue b's raw sums into H[b].
static int batch_collect(BatchPlan &P, cf_hist *H)
{
    Workspace &W = P.W;
    const size_t nb = (size_t)P.nbatch * P.nbins;
    const ResView Rh = res_view(W.h_hist.p, nb);
    if (*Rh.oob > 0) CF_FAIL("%llu particles are out of bounds. Check periodic wrapping?", *Rh.oob);
    if (*Rh.extent > 0)
        CF_FAIL("%llu points or weights left the box / weight range the batch was planned for; plan again", *Rh.extent);
    if (Rh.flags[2] & 2u) CF_FAIL("internal: the chunks outgrew their slots");
    if (Rh.flags[2]) CF_FAIL("internal: neighbour search needed a periodic image beyond +-1");
    if (Rh.flags[3]) CF_FAIL("the batch work list outgrew its plan (catalogues changed since planning); plan again");
    for (int b = 0; b < P.nbatch; b++) {
        if (H[b].nbins != P.nbins) CF_FAIL("internal: histogram size mismatch");
        memcpy(H[b].npairs, Rh.cnt + (size_t)b * P.nbins, sizeof(uint64_t) * P.nbins);
        memcpy(H[b].avg, Rh.avg + (size_t)b * P.nbins, sizeof(double) * P.nbins);
        memcpy(H[b].wsum, Rh.w + (size_t)b * P.nbins, sizeof(double) * P.nbins);
    }
    g_eng.last.pairs_evaluated = Rh.stats[0];
    g_eng.last.pairs_refined = Rh.stats[1];
    g_eng.last.pairs_slow = Rh.stats[2];
    return EXIT_SUCCESS;
}

static void batch_destroy(BatchPlan *P)
{
    if (!P) return;
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->events)
        for (int k = 0; k < 4; k++) cudaEventDestroy(P->ev[k]);
    if (g_eng.stream) cudaStreamSynchronize(g_eng.stream);
    release_workspace(P->W);
    free(P->n1);
    free(P->pbase);
    free(P->cbase);
    free((void *)P->x1);
    delete P;
}

static int batch_plan_locked(const cf_job *tmpl, int nbatch, const int64_t *n1, const void *const *x1,
                             const void *const *y1, const void *const *z1, const void *const *w1, int tune,
                             BatchPlan **out)
{
    *out = nullptr;
    if (engine_init() != EXIT_SUCCESS) return EXIT_FAILURE;
    g_eng.layout_packed = false;  // batched counts take no packed tasks; both forms prune
    g_eng.layout_prune = true;
    if (nbatch < 1 || nbatch > (1 << 15) - 1) CF_FAIL("batch size %d outside [1, 32767]", nbatch);
    if (tmpl->mode != MODE_R3 || tmpl->autocorr) CF_FAIL("internal: batched counts are DD cross-correlations");
    if (tmpl->elem_size != 4 && tmpl->elem_size != 8) CF_FAIL("element size must be 4 or 8");
    if (tmpl->n2 <= 0 || tmpl->n2 >= (1ll << 31)) CF_FAIL("set 2 must hold between 1 and 2^31-1 points");
    cudaStream_t st = g_eng.stream;
    CF_CUDA(cudaStreamSynchronize(st));
    BatchPlan *P = new BatchPlan();
    P->J = *tmpl;
    P->nbatch = nbatch;
    P->isf = tmpl->elem_size == 4;
    P->need_w = tmpl->need_weight != 0;
    P->nbins = tmpl->nedges;
    P->n1 = (int64_t *)calloc(nbatch, sizeof(int64_t));
    P->pbase = (int64_t *)calloc(nbatch + 1, sizeof(int64_t));
    P->cbase = (uint32_t *)calloc(nbatch + 1, sizeof(uint32_t));
    P->x1 = (const void **)calloc(4 * (size_t)nbatch, sizeof(void *));
    if (!P->n1 || !P->pbase || !P->cbase || !P->x1) {
        batch_destroy(P);
        CF_FAIL("out of host memory");
    }
    P->y1 = P->x1 + nbatch;
    P->z1 = P->y1 + nbatch;
    P->w1 = P->z1 + nbatch;
    for (int b = 0; b < nbatch; b++) {
        if (n1[b] < 0 || (n1[b] > 0 && (!x1[b] || !y1[b] || !z1[b] || (P->need_w && !w1[b])))) {
            batch_destroy(P);
            CF_FAIL("catalogue %d: negative size or NULL array", b);
        }
        P->n1[b] = n1[b];
        P->x1[b] = x1[b];
        P->y1[b] = y1[b];
        P->z1[b] = z1[b];
        P->w1[b] = P->need_w ? w1[b] : nullptr;
        P->pbase[b + 1] = P->pbase[b] + n1[b];
    }
    P->total1 = P->pbase[nbatch];
    if (P->total1 >= (1ll << 31)) {
        batch_destroy(P);
        CF_FAIL("the batch holds %lld set-1 points; at most 2^31-1 are supported", (long long)P->total1);
    }
    Workspace &W = P->W;
    int rc = EXIT_SUCCESS;
    do {
        // ---- extent of everything (set 1 in slots 0-7, set 2 in 8-15) ----
        if ((rc = ensure(W.mm, sizeof(unsigned long long) * 2 * kMmSlots)) != EXIT_SUCCESS) break;
        if ((rc = ensure_host(W.h_small, sizeof(unsigned long long) * 4 * kMmSlots)) != EXIT_SUCCESS) break;
        unsigned long long *mm = (unsigned long long *)W.mm.p;
        unsigned long long *mm_init = (unsigned long long *)W.h_small.p, *mmh = mm_init + 2 * kMmSlots;
        for (int k = 0; k < 2 * kMmSlots; k++) mm_init[k] = mm_init_value(k);
        if (cudaMemcpyAsync(mm, mm_init, sizeof(unsigned long long) * 2 * kMmSlots, cudaMemcpyHostToDevice, st) !=
            cudaSuccess) {
            rc = EXIT_FAILURE;
            break;
        }
        for (int s = 0; s <= nbatch; s++) {
            const bool r = s == nbatch;
            const int64_t n = r ? P->J.n2 : P->n1[s];
            if (n == 0) continue;
            const void *x = r ? P->J.x2 : P->x1[s], *y = r ? P->J.y2 : P->y1[s], *z = r ? P->J.z2 : P->z1[s];
            const void *w = P->need_w ? (r ? P->J.w2 : P->w1[s]) : nullptr;
            unsigned long long *slot = mm + (r ? kMmSlots : 0);
            rc = P->isf ? minmax_into<float>(W, (const float *)x, (const float *)y, (const float *)z, (const float *)w,
                                             n, slot)
                        : minmax_into<double>(W, (const double *)x, (const double *)y, (const double *)z,
                                              (const double *)w, n, slot);
            if (rc != EXIT_SUCCESS) break;
        }
        if (rc != EXIT_SUCCESS) break;
        if (cudaMemcpyAsync(mmh, mm, sizeof(unsigned long long) * 2 * kMmSlots, cudaMemcpyDeviceToHost, st) !=
                cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            fprintf(stderr, "corrfunc_gb300: CUDA error '%s' while measuring the batch extent\n",
                    cudaGetErrorString(cudaGetLastError()));
            rc = EXIT_FAILURE;
            break;
        }
        double lo[3], hi[3];
        for (int a = 0; a < 3; a++) {
            lo[a] = fmin(ord_dec(mmh[2 * a]), ord_dec(mmh[kMmSlots + 2 * a]));
            hi[a] = fmax(ord_dec(mmh[2 * a + 1]), ord_dec(mmh[kMmSlots + 2 * a + 1]));
        }
        P->wmax[0] = ord_dec(mmh[6]);
        P->wmax[1] = ord_dec(mmh[kMmSlots + 6]);
        P->wmin[0] = mm_wmin(mmh);
        P->wmin[1] = mm_wmin(mmh + kMmSlots);
        P->w_exact = P->need_w && weights_wide(P->wmax, P->wmin);
        if (mmh[7] != 0 || mmh[kMmSlots + 7] != 0) {
            fprintf(stderr, "corrfunc_gb300: non-finite input coordinates\n");
            rc = EXIT_FAILURE;
            break;
        }
        bool finite = true;
        for (int a = 0; a < 3; a++) finite = finite && isfinite(lo[a]) && isfinite(hi[a]);
        if (!finite) {
            fprintf(stderr, "corrfunc_gb300: non-finite input coordinates\n");
            rc = EXIT_FAILURE;
            break;
        }
        if ((rc = cf_resolve_geometry(&P->J.rule, lo, hi, &P->geo)) != EXIT_SUCCESS) break;
        P->J.geom = P->geo;
        // the GPU lattice of a periodic axis spans the whole box when the data lie in [0, L], so
        // that replays may move points anywhere inside it
        double glo[3], ghi[3];
        for (int a = 0; a < 3; a++) {
            const bool per = P->geo.periodic[a] && P->geo.wrap[a] > 0.0;
            const bool inbox = per && lo[a] >= 0.0 && hi[a] <= P->geo.wrap[a];
            glo[a] = inbox ? 0.0 : lo[a];
            ghi[a] = inbox ? P->geo.wrap[a] : hi[a];
        }
        P->J.n1 = (P->total1 + nbatch - 1) / nbatch;  // column width follows the mean catalogue density
        if ((rc = gpu_geometry(&P->J, P->geo, glo, ghi, P->g, P->delta)) != EXIT_SUCCESS) break;
        for (int a = 0; a < 3; a++) {
            const bool per = P->geo.periodic[a] && P->geo.wrap[a] > 0.0;
            P->g.chk_lo[a] = glo[a];
            P->g.chk_hi[a] = per ? glo[a] + P->geo.wrap[a] : ghi[a];
        }
        geom_keys(P->g);
        P->ncols = (uint32_t)P->g.n[0] * P->g.n[1];
        P->ncells = P->ncols * (uint32_t)P->g.n[2];
        g_eng.last.num_cells = (int)P->ncells;

        // ---- buffers ----
        if ((rc = task_geometry(&P->J, P->geo, P->g, glo, ghi, false, MODE_R3, P->G)) != EXIT_SUCCESS) break;
        P->gap = chunk_gap(P->G, P->J.n1, P->ncols);
        // the merged form wherever the byte table and private histogram columns fit (FP32
        // classification; CF_BATCH_MERGED=0 keeps one lattice per catalogue, for measurements)
        P->merged = false;
        const int mw = pair_max_threads(MODE_R3, P->J.need_avg != 0, P->need_w) / 32;
        const char *bm = getenv("CF_BATCH_MERGED");
        if (g_eng.precision == CF_PRECISION_FP32_REFINE && !P->w_exact && g_eng.byte_table && P->nbins <= 126 &&
            !(bm && atoi(bm) == 0)) {
            for (int wv = mw; wv >= 1 && !P->merged && rc == EXIT_SUCCESS; wv /= 2) {
                g_eng.force_ls = 32;
                g_eng.force_warps = wv;
                Tables Tm;
                rc = build_tables(W, &P->J, MODE_R3, P->nbins, P->need_w, P->delta, &Tm);
                g_eng.force_ls = 0;
                g_eng.force_warps = 0;
                if (rc == EXIT_SUCCESS && Tm.lut8 && Tm.ls == 32) {
                    P->merged = true;
                    P->T = Tm;
                    P->ls = 32;
                    P->warps = wv;
                }
            }
            if (rc != EXIT_SUCCESS) break;
        }
        uint64_t slots = 0;
        if (P->merged) {
            P->gap = chunk_gap(P->G, P->total1, P->ncols);
            slots = chunk_slots((uint64_t)P->total1, P->ncols, P->g.n[2], P->gap);
            for (int b = 0; b <= nbatch; b++) P->cbase[b] = 0;
            if (slots <= 0xfffffff0ull) P->cbase[nbatch] = (uint32_t)slots;
        } else {
            for (int b = 0; b < nbatch; b++) {
                slots += P->n1[b] > 0 ? chunk_slots((uint64_t)P->n1[b], P->ncols, P->g.n[2], P->gap) : 0;
                if (slots > 0xfffffff0ull) break;
                P->cbase[b + 1] = (uint32_t)slots;
            }
        }
        if (slots > 0xfffffff0ull) {
            fprintf(stderr, "corrfunc_gb300: too many chunks in the batch\n");
            rc = EXIT_FAILURE;
            break;
        }
        P->total_slots = P->cbase[nbatch];
        const size_t nb = (size_t)nbatch * P->nbins;
        if ((rc = ensure_points(W.set[0], P->total1 > 0 ? P->total1 : 1)) != EXIT_SUCCESS ||
            (rc = ensure_points(W.set[1], P->J.n2)) != EXIT_SUCCESS ||
            (rc = ensure(W.res, res_bytes(nb))) != EXIT_SUCCESS ||
            (rc = ensure(W.chunk_cnt, sizeof(uint32_t) * P->ncols)) != EXIT_SUCCESS ||
            (rc = ensure(W.chunk_off, sizeof(uint32_t) * ((size_t)P->ncols + 1))) != EXIT_SUCCESS ||
            (rc = ensure(W.chunk_begin, sizeof(uint32_t) * ((size_t)P->total_slots + 1))) != EXIT_SUCCESS ||
            (rc = ensure(W.chunk_info, sizeof(uint2) * ((size_t)P->total_slots + 1))) != EXIT_SUCCESS ||
            (rc = ensure(W.chunk_cat, sizeof(uint16_t) * ((size_t)P->total_slots + 1))) != EXIT_SUCCESS ||
            (rc = ensure_host(W.h_hist, res_bytes(nb))) != EXIT_SUCCESS)
            break;
        P->nentries = P->merged ? 0u : P->total_slots * (uint32_t)((2 * P->G.reach_x + 1) * (2 * P->G.reach_y + 1));
        if ((rc = ensure(W.ntask, sizeof(uint32_t) * ((size_t)P->nentries + 1))) != EXIT_SUCCESS ||
            (rc = ensure(W.task_off, sizeof(uint32_t) * ((size_t)P->nentries + 2))) != EXIT_SUCCESS)
            break;
        P->G.error = res_view(W.res.p, nb).flags + 2;
        if (!P->merged && (rc = build_tables(W, &P->J, MODE_R3, P->nbins, P->need_w, P->delta, &P->T)) != EXIT_SUCCESS)
            break;

        // ---- eager run: size the work list ----
        if ((rc = batch_enqueue(*P, 0, false)) != EXIT_SUCCESS) break;
        if (P->merged) {
            P->ntasks = 0;
            P->task_cap = 0;
        } else {
            uint32_t *cnt_h = (uint32_t *)(mmh + kMmSlots);
            if (cudaMemcpyAsync(cnt_h, (uint32_t *)W.task_off.p + P->nentries, sizeof(uint32_t),
                                cudaMemcpyDeviceToHost, st) != cudaSuccess ||
                cudaStreamSynchronize(st) != cudaSuccess) {
                fprintf(stderr, "corrfunc_gb300: CUDA error '%s' while building the batch work list\n",
                        cudaGetErrorString(cudaGetLastError()));
                rc = EXIT_FAILURE;
                break;
            }
            P->ntasks = *cnt_h;
            // room for replays on catalogues of the same sizes whose points moved: twice the planned
            // work list plus eight tasks per chunk of set 1 (a replay that still outgrows it fails)
            P->task_cap = 2 * P->ntasks + 8 * (uint32_t)((P->total1 + kChunk - 1) / kChunk) + 1024;
            if ((rc = ensure(W.tasks, sizeof(Task) * (size_t)P->task_cap)) != EXIT_SUCCESS) break;
        }

        PairArgs &A = P->A;
        memset(&A, 0, sizeof(A));
        A.hi1 = (const float4 *)W.set[0].hi.p;
        A.lo1 = (const float4 *)W.set[0].lo.p;
        A.d1 = (const double4_32a *)W.set[0].dbl.p;
        A.ro1 = (const int2 *)W.set[0].ro.p;
        A.hi2 = (const float4 *)W.set[1].hi.p;
        A.lo2 = (const float4 *)W.set[1].lo.p;
        A.d2 = (const double4_32a *)W.set[1].dbl.p;
        A.ro2 = (const int2 *)W.set[1].ro.p;
        A.tasks = P->merged ? nullptr : (const Task *)W.tasks.p;
        A.ntasks = P->task_cap;
        A.ntask_dev = P->merged ? nullptr : (const uint32_t *)W.task_off.p + P->nentries;
        pair_constants(A, &P->J, MODE_R3, P->nbins, false, P->G, P->geo, P->g, P->delta, P->T, P->wmax, W);
        A.w_exact = P->w_exact ? 1 : 0;
        {
            const ResView R = res_view(W.res.p, nb);
            A.g_cnt = R.cnt;
            A.g_avg = R.avg;
            A.g_w = R.w;
            A.g_stats = R.stats;
            A.task_counter = R.flags;
        }
        for (int k = 0; k < 4; k++)
            if (cudaEventCreate(&P->ev[k]) != cudaSuccess) rc = EXIT_FAILURE;
        if (rc != EXIT_SUCCESS) break;
        P->events = true;
        if ((rc = batch_enqueue(*P, 1, false)) != EXIT_SUCCESS) break;
        if (cudaStreamSynchronize(st) != cudaSuccess) {
            fprintf(stderr, "corrfunc_gb300: CUDA error '%s' in the batch pair kernel\n",
                    cudaGetErrorString(cudaGetLastError()));
            rc = EXIT_FAILURE;
            break;
        }
        {
            const ResView Rh = res_view(W.h_hist.p, nb);
            if (*Rh.oob > 0 || *Rh.extent > 0 || Rh.flags[2] || Rh.flags[3]) {
                fprintf(stderr, "corrfunc_gb300: batch planning failed (out-of-bounds points or work-list error)\n");
                rc = EXIT_FAILURE;
                break;
            }
        }

        // ---- tuner: time the FP32 layouts that fit, keep the fastest ----
        if (tune && g_eng.precision == CF_PRECISION_FP32_REFINE && !P->w_exact) {
            const int cand_ls[3] = {32, 16, 8};
            const int cand_w[3] = {mw, mw / 2, mw / 4};
            float best = 1e30f;
            int best_ls = 0, best_w = 0;
            // (a merged batch keeps private columns: lane stride 32 only)
            for (int li = 0; li < (P->merged ? 1 : 3) && rc == EXIT_SUCCESS; li++) {
                for (int wi = 0; wi < 3 && rc == EXIT_SUCCESS; wi++) {
                    const SmemLayout c = smem_layout(P->J.nedges, P->nbins, cand_w[wi], false, P->T.lut_n, cand_ls[li],
                                                     P->J.need_avg != 0, P->need_w, false, P->J.need_avg != 0);
                    if (c.total > 220 * 1024) continue;
                    g_eng.force_ls = cand_ls[li];
                    g_eng.force_warps = cand_w[wi];
                    Tables T2;
                    if ((rc = build_tables(W, &P->J, MODE_R3, P->nbins, P->need_w, P->delta, &T2)) != EXIT_SUCCESS) break;
                    P->T = T2;
                    pair_constants(A, &P->J, MODE_R3, P->nbins, false, P->G, P->geo, P->g, P->delta, P->T, P->wmax, W);
                    P->ls = cand_ls[li];
                    P->warps = cand_w[wi];
                    float ms = 0.f;
                    for (int rep = 0; rep < 2 && rc == EXIT_SUCCESS; rep++) {
                        if ((rc = batch_enqueue(*P, 1, true)) != EXIT_SUCCESS) break;
                        if (cudaStreamSynchronize(st) != cudaSuccess ||
                            cudaEventElapsedTime(&ms, P->ev[1], P->ev[2]) != cudaSuccess) {
                            fprintf(stderr, "corrfunc_gb300: CUDA error while tuning the batch layout\n");
                            rc = EXIT_FAILURE;
                        }
                    }
                    if (rc == EXIT_SUCCESS && ms < best) {
                        best = ms;
                        best_ls = cand_ls[li];
                        best_w = cand_w[wi];
                    }
                }
            }
            g_eng.force_ls = 0;
            g_eng.force_warps = 0;
            if (rc != EXIT_SUCCESS) break;
            P->ls = best_ls;
            P->warps = best_w;
            g_eng.force_ls = best_ls;
            g_eng.force_warps = best_w;
            Tables T2;
            rc = build_tables(W, &P->J, MODE_R3, P->nbins, P->need_w, P->delta, &T2);
            g_eng.force_ls = 0;
            g_eng.force_warps = 0;
            if (rc != EXIT_SUCCESS) break;
            P->T = T2;
            pair_constants(A, &P->J, MODE_R3, P->nbins, false, P->G, P->geo, P->g, P->delta, P->T, P->wmax, W);
            if (cudaStreamSynchronize(st) != cudaSuccess) {
                rc = EXIT_FAILURE;
                break;
            }
        }

        // ---- capture the whole sequence as one graph ----
        const int launches0 = g_eng.launches;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed) != cudaSuccess) {
            fprintf(stderr, "corrfunc_gb300: cannot capture the batch graph\n");
            rc = EXIT_FAILURE;
            break;
        }
        int rc0 = record_event(P->ev[0]);
        if (rc0 == EXIT_SUCCESS) rc0 = batch_enqueue(*P, 0, false);
        if (rc0 == EXIT_SUCCESS) rc0 = batch_enqueue(*P, 1, true);
        if (rc0 == EXIT_SUCCESS) rc0 = record_event(P->ev[3]);
        const cudaError_t ec = cudaStreamEndCapture(st, &P->graph);
        if (rc0 != EXIT_SUCCESS || ec != cudaSuccess) {
            fprintf(stderr, "corrfunc_gb300: capturing the batch graph failed (%s)\n", cudaGetErrorString(ec));
            rc = EXIT_FAILURE;
            break;
        }
        P->kernels = g_eng.launches - launches0;
        if (cudaGraphInstantiate(&P->exec, P->graph, 0) != cudaSuccess) {
            fprintf(stderr, "corrfunc_gb300: instantiating the batch graph failed\n");
            rc = EXIT_FAILURE;
            break;
        }
    } while (0);
    if (rc != EXIT_SUCCESS) {
        g_eng.force_ls = 0;
        g_eng.force_warps = 0;
        batch_destroy(P);
        return EXIT_FAILURE;
    }
    *out = P;
    return EXIT_SUCCESS;
}

static int batch_run_locked(BatchPlan *P, cf_hist *H)
{
    g_eng.layout_packed = false;  // batched counts take no packed tasks; both forms prune
    g_eng.layout_prune = true;
    if (engine_init() != EXIT_SUCCESS) return EXIT_FAILURE;
    cudaStream_t st = g_eng.stream;
    CF_CUDA(cudaStreamSynchronize(st));
    memset(&g_eng.last, 0, sizeof(g_eng.last));
    CF_CHECK_INTERRUPT();
    CF_CUDA(cudaGraphLaunch(P->exec, st));
    CF_CUDA(cudaStreamSynchronize(st));
    CF_CHECK_INTERRUPT();
    if (batch_collect(*P, H) != EXIT_SUCCESS) return EXIT_FAILURE;
    float ms_total = 0.f, ms_pairs = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms_total, P->ev[0], P->ev[3]));
    CF_CUDA(cudaEventElapsedTime(&ms_pairs, P->ev[1], P->ev[2]));
    g_eng.last.total_gpu_ms = ms_total;
    g_eng.last.pair_kernel_ms = ms_pairs;
    g_eng.last.gridlink_ms = ms_total - ms_pairs;
    g_eng.last.tasks = P->ntasks;
    g_eng.last.kernel_launches = P->kernels;
    g_eng.last.num_cells = (int)P->ncells;
    g_eng.last.lane_stride = P->ls;
    g_eng.last.warps_per_block = P->warps;
    return EXIT_SUCCESS;
}

// ------------------------------------------------------------------------------------
// counts in spheres (vpf): the points are sorted by their cell of the reference lattice; one
// warp per sphere centre walks the same neighbour cells as the reference
// (theory/vpf/countspheres_impl.c.src:332-415, mocks/vpf_mocks/countspheres_mocks_impl.c.src:
// 520-548), with the same periodic shifts of the centre, and bins the FP64 distances into
// shells exactly as the fallback kernels do (theory/vpf/vpf_kernels.c.src:281-302,
// mocks/vpf_mocks/vpf_mocks_kernels.c.src:294-332).
// ------------------------------------------------------------------------------------
struct VpfLattice {
    int n[3];
    double lo[3], inv[3];
};

__global__ void k_vpf_cells(const double *x, const double *y, const double *z, int64_t np, VpfLattice L,
                            uint32_t *cellid, uint32_t *count, unsigned long long *oob)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
        const double v[3] = {x[i], y[i], z[i]};
        int c[3];
        bool bad = false;
        for (int a = 0; a < 3; a++) {
            const double t = __dmul_rn(__dsub_rn(v[a], L.lo[a]), L.inv[a]);
            int k = (t > -2.0e9 && t < 2.0e9) ? __double2int_rz(t) : -1;
            if (k > L.n[a] - 1) k--;
            if (k < 0 || k >= L.n[a]) {
                bad = true;
                k = 0;
            }
            c[a] = k;
        }
        if (bad) atomicAdd(oob, 1ull);
        const uint32_t cell = ((uint32_t)c[0] * (uint32_t)L.n[1] + (uint32_t)c[1]) * (uint32_t)L.n[2] + (uint32_t)c[2];
        cellid[i] = cell;
        atomicAdd(&count[cell], 1u);
    }
}

__global__ void k_vpf_scatter(const double *x, const double *y, const double *z, int64_t np, const uint32_t *cellid,
                              const uint32_t *cell_start, uint32_t *fill, double4_32a *pts)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < np; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cellid[i];
        const uint32_t pos = cell_start[c] + atomicAdd(&fill[c], 1u);
        pts[pos] = make_double4_32a(x[i], y[i], z[i], 0.0);
    }
}

struct VpfArgs {
    const double4_32a *pts;
    const uint32_t *cell_start;
    const double *cen;
    const int *cen_cell;
    int64_t ncen;
    int n[3];
    int refine[3];
    int periodic;
    double wrap[3];
    double rmax_sqr, inv_rstep;
    int nbin, num_pN;
    unsigned long long *pN;
    uint32_t *within;  // per-centre neighbour counts (r^2 < rmax^2) instead of pN, or null
};

// neighbour cell index and centre shift along one axis; false when a non-periodic lattice has no
// such cell
__device__ __forceinline__ bool vpf_axis(const VpfArgs &A, int a, int c, int d, int *cell, double *off)
{
    int k = c + d;
    *off = 0.0;
    if (A.periodic) {
        if (k >= A.n[a]) *off = -A.wrap[a];
        else if (k < 0) *off = A.wrap[a];
        k %= A.n[a];
        if (k < 0) k += A.n[a];
    } else if (k < 0 || k >= A.n[a]) {
        return false;
    }
    *cell = k;
    return true;
}

__global__ void __launch_bounds__(256) k_vpf(VpfArgs A)
{
    extern __shared__ uint32_t s_shell[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t *cnt = s_shell + (size_t)warp * A.nbin;
    const int64_t nw = (int64_t)gridDim.x * (blockDim.x >> 5);
    for (int64_t c = (int64_t)blockIdx.x * (blockDim.x >> 5) + warp; c < A.ncen; c += nw) {
        for (int b = lane; b < A.nbin; b += 32) cnt[b] = 0;
        __syncwarp();
        const double xc = A.cen[3 * c], yc = A.cen[3 * c + 1], zc = A.cen[3 * c + 2];
        const int ix = A.cen_cell[3 * c], iy = A.cen_cell[3 * c + 1], iz = A.cen_cell[3 * c + 2];
        for (int dx = -A.refine[0]; dx <= A.refine[0]; dx++) {
            int cx;
            double ox;
            if (!vpf_axis(A, 0, ix, dx, &cx, &ox)) continue;
            const double px = __dadd_rn(xc, ox);
            for (int dy = -A.refine[1]; dy <= A.refine[1]; dy++) {
                int cy;
                double oy;
                if (!vpf_axis(A, 1, iy, dy, &cy, &oy)) continue;
                const double py = __dadd_rn(yc, oy);
                for (int dz = -A.refine[2]; dz <= A.refine[2]; dz++) {
                    int cz;
                    double oz;
                    if (!vpf_axis(A, 2, iz, dz, &cz, &oz)) continue;
                    const double pz = __dadd_rn(zc, oz);
                    const uint32_t cell = ((uint32_t)cx * (uint32_t)A.n[1] + (uint32_t)cy) * (uint32_t)A.n[2] + (uint32_t)cz;
                    const uint32_t j1 = A.cell_start[cell + 1];
                    for (uint32_t j = A.cell_start[cell] + lane; j < j1; j += 32) {
                        const double4_32a p = A.pts[j];
                        const double ddx = __dsub_rn(p.x, px), ddy = __dsub_rn(p.y, py), ddz = __dsub_rn(p.z, pz);
                        const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)), __dmul_rn(ddz, ddz));
                        if (r2 >= A.rmax_sqr) continue;
                        if (A.within) {
                            atomicAdd(&cnt[0], 1u);
                            continue;
                        }
                        const int ib = __double2int_rz(__dmul_rn(__dsqrt_rn(r2), A.inv_rstep));
                        if (ib < A.nbin) atomicAdd(&cnt[ib], 1u);
                    }
                }
            }
        }
        __syncwarp();
        if (A.within) {
            if (lane == 0) A.within[c] = cnt[0];
        } else if (lane == 0) {
            uint32_t cum = 0;
            for (int b = 0; b < A.nbin; b++) {
                cum += cnt[b];
                if (cum < (uint32_t)A.num_pN) atomicAdd(&A.pN[(size_t)b * A.num_pN + cum], 1ull);
            }
        }
        __syncwarp();
    }
}

struct VpfBufs {
    DevBuf xyz, cellid, count, fill, cell_start, pts, cen, cen_cell, pN, oob, within;
    HostBuf h_out;
};
static VpfBufs g_vpf;

static int vpf_locked(const cf_vpf_job *J, uint64_t *pN)
{
    if (engine_init() != EXIT_SUCCESS) return EXIT_FAILURE;
    cudaStream_t st = g_eng.stream;
    g_eng.launches = 0;
    memset(&g_eng.last, 0, sizeof(g_eng.last));
    const size_t npn = (size_t)J->nbin * J->num_pN;
    memset(pN, 0, sizeof(uint64_t) * npn);
    if (J->nbin < 1 || J->num_pN < 1 || J->nbin > 4096) CF_FAIL("vpf: 1 <= nbin <= 4096 and num_pN >= 1 are supported");
    if (J->np < 0 || J->np >= (1ll << 31) || J->ncen < 0) CF_FAIL("vpf: unsupported sizes");
    double ncells_d = 1.0;
    for (int a = 0; a < 3; a++) {
        if (J->nmesh[a] < 1) CF_FAIL("vpf: empty lattice");
        ncells_d *= J->nmesh[a];
    }
    if (ncells_d > (double)(1u << 30)) CF_FAIL("vpf: lattice of %.0f cells is too large", ncells_d);
    const uint32_t ncells = (uint32_t)ncells_d;
    const int64_t np = J->np;
    VpfBufs &B = g_vpf;
    if (ensure(B.xyz, sizeof(double) * 3 * (size_t)(np > 0 ? np : 1)) || ensure(B.cellid, sizeof(uint32_t) * (size_t)(np > 0 ? np : 1)) ||
        ensure(B.count, sizeof(uint32_t) * ncells) || ensure(B.fill, sizeof(uint32_t) * ncells) ||
        ensure(B.cell_start, sizeof(uint32_t) * ((size_t)ncells + 1)) ||
        ensure(B.pts, sizeof(double4_32a) * (size_t)(np > 0 ? np : 1)) ||
        ensure(B.cen, sizeof(double) * 3 * (size_t)(J->ncen > 0 ? J->ncen : 1)) ||
        ensure(B.cen_cell, sizeof(int) * 3 * (size_t)(J->ncen > 0 ? J->ncen : 1)) ||
        ensure(B.pN, sizeof(unsigned long long) * npn) || ensure(B.oob, sizeof(unsigned long long)) ||
        ensure(B.within, sizeof(uint32_t) * (size_t)(J->ncen > 0 ? J->ncen : 1)) ||
        ensure_host(B.h_out, sizeof(unsigned long long) * (npn + 1)))
        return EXIT_FAILURE;
    CF_CUDA(cudaEventRecord(g_eng.ev[0], st));
    double *dx = (double *)B.xyz.p, *dy = dx + np, *dz = dy + np;
    if (np > 0) {
        CF_CUDA(cudaMemcpyAsync(dx, J->x, sizeof(double) * np, cudaMemcpyHostToDevice, st));
        CF_CUDA(cudaMemcpyAsync(dy, J->y, sizeof(double) * np, cudaMemcpyHostToDevice, st));
        CF_CUDA(cudaMemcpyAsync(dz, J->z, sizeof(double) * np, cudaMemcpyHostToDevice, st));
    }
    if (J->ncen > 0) {
        CF_CUDA(cudaMemcpyAsync(B.cen.p, J->cen, sizeof(double) * 3 * J->ncen, cudaMemcpyHostToDevice, st));
        CF_CUDA(cudaMemcpyAsync(B.cen_cell.p, J->cen_cell, sizeof(int) * 3 * J->ncen, cudaMemcpyHostToDevice, st));
    }
    CF_CUDA(cudaMemsetAsync(B.count.p, 0, sizeof(uint32_t) * ncells, st));
    CF_CUDA(cudaMemsetAsync(B.fill.p, 0, sizeof(uint32_t) * ncells, st));
    CF_CUDA(cudaMemsetAsync(B.pN.p, 0, sizeof(unsigned long long) * npn, st));
    CF_CUDA(cudaMemsetAsync(B.oob.p, 0, sizeof(unsigned long long), st));
    VpfLattice L;
    for (int a = 0; a < 3; a++) {
        L.n[a] = J->nmesh[a];
        L.lo[a] = J->lat_min[a];
        L.inv[a] = J->lat_inv[a];
    }
    if (np > 0) {
        const int grid = grid_for(np, 256);
        k_vpf_cells<<<grid, 256, 0, st>>>(dx, dy, dz, np, L, (uint32_t *)B.cellid.p, (uint32_t *)B.count.p,
                                          (unsigned long long *)B.oob.p);
        CF_CUDA(cudaGetLastError());
        g_eng.launches++;
    }
    if (scan_u32(g_eng.ws, (const uint32_t *)B.count.p, (uint32_t *)B.cell_start.p, ncells, 0) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    if (np > 0) {
        k_vpf_scatter<<<grid_for(np, 256), 256, 0, st>>>(dx, dy, dz, np, (const uint32_t *)B.cellid.p,
                                                          (const uint32_t *)B.cell_start.p, (uint32_t *)B.fill.p,
                                                          (double4_32a *)B.pts.p);
        CF_CUDA(cudaGetLastError());
        g_eng.launches++;
    }
    CF_CUDA(cudaEventRecord(g_eng.ev[1], st));
    VpfArgs A;
    A.pts = (const double4_32a *)B.pts.p;
    A.cell_start = (const uint32_t *)B.cell_start.p;
    A.cen = (const double *)B.cen.p;
    A.cen_cell = (const int *)B.cen_cell.p;
    A.ncen = J->ncen;
    for (int a = 0; a < 3; a++) {
        A.n[a] = J->nmesh[a];
        A.refine[a] = J->refine[a];
        A.wrap[a] = J->wrap[a];
    }
    A.periodic = J->periodic;
    A.rmax_sqr = J->rmax * J->rmax;
    A.inv_rstep = 1.0 / (J->rmax / (double)J->nbin);
    A.nbin = J->nbin;
    A.num_pN = J->num_pN;
    A.pN = (unsigned long long *)B.pN.p;
    A.within = J->counts_out ? (uint32_t *)B.within.p : nullptr;
    CF_CUDA(cudaEventRecord(g_eng.ev[2], st));
    if (J->ncen > 0) {
        const size_t smem = sizeof(uint32_t) * 8 * (size_t)J->nbin;
        CF_CUDA(cudaFuncSetAttribute(k_vpf, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int64_t blocks = (J->ncen + 7) / 8;
        const int64_t cap = (int64_t)g_eng.num_sms * 8;
        if (blocks > cap) blocks = cap;
        k_vpf<<<(int)blocks, 256, smem, st>>>(A);
        CF_CUDA(cudaGetLastError());
        g_eng.launches++;
    }
    CF_CUDA(cudaEventRecord(g_eng.ev[3], st));
    unsigned long long *h = (unsigned long long *)B.h_out.p;
    CF_CUDA(cudaMemcpyAsync(h, B.pN.p, sizeof(unsigned long long) * npn, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(h + npn, B.oob.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    if (J->counts_out && J->ncen > 0)
        CF_CUDA(cudaMemcpyAsync(J->counts_out, B.within.p, sizeof(uint32_t) * J->ncen, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaEventRecord(g_eng.ev[4], st));
    CF_CUDA(cudaStreamSynchronize(st));
    CF_CHECK_INTERRUPT();
    if (h[npn] > 0) CF_FAIL("%llu particles are out of bounds. Check periodic wrapping?", h[npn]);
    for (size_t k = 0; k < npn; k++) pN[k] = h[k];
    float ms_pairs = 0.f, ms_grid = 0.f, ms_total = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms_pairs, g_eng.ev[2], g_eng.ev[3]));
    CF_CUDA(cudaEventElapsedTime(&ms_grid, g_eng.ev[0], g_eng.ev[1]));
    CF_CUDA(cudaEventElapsedTime(&ms_total, g_eng.ev[0], g_eng.ev[4]));
    g_eng.last.pair_kernel_ms = ms_pairs;
    g_eng.last.gridlink_ms = ms_grid;
    g_eng.last.total_gpu_ms = ms_total;
    g_eng.last.num_cells = (int)ncells;
    g_eng.last.kernel_launches = g_eng.launches;
    return EXIT_SUCCESS;
}

}  // namespace

// Shape of a count for the autotuner: everything but the coordinate values (sizes, mode,
// options, the reference-lattice rule, radii and bin edges), FNV-1a over their bytes.
static unsigned long long tune_key(const cf_job *J)
{
    unsigned long long h = 1469598103934665603ull;
    auto mix = [&](const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        for (size_t k = 0; k < n; k++) h = (h ^ c[k]) * 1099511628211ull;
    };
    const int ints[7] = {J->mode, J->autocorr, J->elem_size, J->need_avg, J->need_weight, J->nedges, J->npibin};
    mix(ints, sizeof(ints));
    mix(&J->n1, sizeof(J->n1));
    mix(&J->n2, sizeof(J->n2));
    mix(&J->rule.kind, sizeof(J->rule.kind));
    mix(&J->rule.periodic, sizeof(J->rule.periodic));
    mix(J->rule.boxsize, sizeof(J->rule.boxsize));
    mix(J->rule.refine, sizeof(J->rule.refine));
    const double radii[3] = {J->rmax_xy, J->rmax_z, J->rmax_3d};
    mix(radii, sizeof(radii));
    mix(J->edges, sizeof(double) * (size_t)(J->nedges > 0 ? J->nedges : 0));
    return h;
}

// A count under the autotuner: the first count of a shape runs with each j-lattice column split
// (1, 2, 3, 4; slabs merged in pairs when split) twice, keeps the split whose second device time
// is the shortest for later counts of that shape, and returns the results of a run with it.
static int run_tuned(cf_job *J, cf_hist *H)
{
    const unsigned long long key = tune_key(J);
    int split = 0, zdiv = 1;
    for (int k = 0; k < g_eng.ntune; k++) {
        if (g_eng.tune[k].key == key) {
            split = g_eng.tune[k].split;
            zdiv = g_eng.tune[k].zdiv;
        }
    }
    int rc = EXIT_SUCCESS;
    if (split == 0) {
        const int cand[4][2] = {{1, 1}, {2, 2}, {3, 2}, {4, 2}};
        double best = INFINITY;
        int last = 0;
        for (int c = 0; c < 4 && rc == EXIT_SUCCESS; c++) {
            g_eng.tune_force = cand[c][0];
            g_eng.tune_zdiv = cand[c][1];
            for (int rep = 0; rep < 2 && rc == EXIT_SUCCESS; rep++) rc = run_locked(J, H);
            if (rc != EXIT_SUCCESS || g_eng.last.column_split != cand[c][0]) continue;  // not allowed here
            last = cand[c][0];
            if (g_eng.last.total_gpu_ms < best) {
                best = g_eng.last.total_gpu_ms;
                split = cand[c][0];
                zdiv = cand[c][1];
            }
        }
        g_eng.tune_force = 0;
        if (rc != EXIT_SUCCESS) return rc;
        if (split == 0) split = 1;
        auto &E = g_eng.tune[g_eng.tune_next];
        E.key = key;
        E.split = split;
        E.zdiv = zdiv;
        g_eng.tune_next = (g_eng.tune_next + 1) % 32;
        if (g_eng.ntune < 32) g_eng.ntune++;
        if (last == split) return EXIT_SUCCESS;  // H holds the chosen form's results
    }
    g_eng.tune_force = split;
    g_eng.tune_zdiv = zdiv;
    rc = run_locked(J, H);
    g_eng.tune_force = 0;
    return rc;
}

extern "C" int cf_engine_run(cf_job *job, cf_hist *out)
{
    pthread_mutex_lock(&g_lock);
    InterruptGuard guard;
    // the autotuner covers the FP32 path of DD(r) and xi (the counts with split j columns)
    const bool tuned = g_eng.autotune && job->mode == MODE_R3 && g_eng.precision == CF_PRECISION_FP32_REFINE &&
                       !job->task_timer;
    const int rc = tuned ? run_tuned(job, out) : run_locked(job, out);
    pthread_mutex_unlock(&g_lock);
    return rc;
}

extern "C" int cf_engine_set_autotune(int on)
{
    pthread_mutex_lock(&g_lock);
    g_eng.autotune = on ? 1 : 0;
    if (!on) g_eng.ntune = g_eng.tune_next = 0;  // forget the shapes
    pthread_mutex_unlock(&g_lock);
    return EXIT_SUCCESS;
}

extern "C" int cf_engine_get_autotune(void) { return g_eng.autotune; }

extern "C" int cf_engine_vpf(const cf_vpf_job *job, uint64_t *pN)
{
    pthread_mutex_lock(&g_lock);
    InterruptGuard guard;
    const int rc = vpf_locked(job, pN);
    pthread_mutex_unlock(&g_lock);
    return rc;
}

extern "C" int cf_engine_set_precision(int mode)
{
    if (mode != CF_PRECISION_FP32_REFINE && mode != CF_PRECISION_FP64) return EXIT_FAILURE;
    pthread_mutex_lock(&g_lock);
    g_eng.precision = mode;
    pthread_mutex_unlock(&g_lock);
    return EXIT_SUCCESS;
}

extern "C" int cf_engine_get_precision(void) { return g_eng.precision; }

extern "C" int cf_engine_to_device(const void *src, size_t bytes, void **dev)
{
    pthread_mutex_lock(&g_lock);
    int rc = engine_init();
    void *p = nullptr;
    if (rc == EXIT_SUCCESS && cudaMalloc(&p, bytes ? bytes : 16) != cudaSuccess) rc = EXIT_FAILURE;
    if (rc == EXIT_SUCCESS && bytes && cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice) != cudaSuccess) rc = EXIT_FAILURE;
    pthread_mutex_unlock(&g_lock);
    if (rc != EXIT_SUCCESS) {
        if (p) cudaFree(p);
        fprintf(stderr, "corrfunc_gb300: could not copy %zu bytes to the device\n", bytes);
        return EXIT_FAILURE;
    }
    *dev = p;
    return EXIT_SUCCESS;
}

extern "C" void cf_engine_free_device(void *dev)
{
    if (dev) cudaFree(dev);
}

extern "C" int cf_engine_copy_to_host(void *dst, const void *src, size_t bytes)
{
    CF_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
    return EXIT_SUCCESS;
}

extern "C" int cf_engine_fp32_peak(double *tflops)
{
    pthread_mutex_lock(&g_lock);
    int rc = engine_init();
    if (rc == EXIT_SUCCESS) {
        rc = [&]() -> int {
            DevBuf tmp;
            if (ensure(tmp, 4096 * sizeof(float)) != EXIT_SUCCESS) return EXIT_FAILURE;
            const int blocks = g_eng.num_sms * 8, threads = 256, iters = 1 << 16;
            const float a = 0.999999f, b = 1e-7f;
            k_fma_peak<<<blocks, threads, 0, g_eng.stream>>>((float *)tmp.p, 256, a, b);  // warm-up
            CF_CUDA(cudaEventRecord(g_eng.ev[0], g_eng.stream));
            k_fma_peak<<<blocks, threads, 0, g_eng.stream>>>((float *)tmp.p, iters, a, b);
            CF_CUDA(cudaEventRecord(g_eng.ev[1], g_eng.stream));
            CF_CUDA(cudaEventSynchronize(g_eng.ev[1]));
            float ms = 0.f;
            CF_CUDA(cudaEventElapsedTime(&ms, g_eng.ev[0], g_eng.ev[1]));
            cudaFree(tmp.p);
            *tflops = (double)blocks * threads * iters * 8.0 * 2.0 / (ms * 1e-3) / 1e12;
            return EXIT_SUCCESS;
        }();
    }
    pthread_mutex_unlock(&g_lock);
    return rc;
}

extern "C" int cf_engine_last_stats(cf_engine_stats *out)
{
    if (!out) return EXIT_FAILURE;
    pthread_mutex_lock(&g_lock);
    *out = g_eng.last;
    pthread_mutex_unlock(&g_lock);
    return EXIT_SUCCESS;
}

extern "C" int cf_engine_batch_plan(const cf_job *tmpl, int nbatch, const int64_t *n1, const void *const *x1,
                                    const void *const *y1, const void *const *z1, const void *const *w1, int tune,
                                    cf_batch **out)
{
    pthread_mutex_lock(&g_lock);
    BatchPlan *P = nullptr;
    const int rc = batch_plan_locked(tmpl, nbatch, n1, x1, y1, z1, w1, tune, &P);
    pthread_mutex_unlock(&g_lock);
    *out = (cf_batch *)P;
    return rc;
}

extern "C" int cf_engine_batch_run(cf_batch *plan, cf_hist *out)
{
    if (!plan || !out) return EXIT_FAILURE;
    pthread_mutex_lock(&g_lock);
    InterruptGuard guard;
    const int rc = batch_run_locked((BatchPlan *)plan, out);
    pthread_mutex_unlock(&g_lock);
    return rc;
}

extern "C" void cf_engine_batch_free(cf_batch *plan)
{
    if (!plan) return;
    pthread_mutex_lock(&g_lock);
    batch_destroy((BatchPlan *)plan);
    pthread_mutex_unlock(&g_lock);
}
