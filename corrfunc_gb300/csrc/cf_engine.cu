// cf_engine.cu -- GB300 (sm_103a) pair-counting engine.
//
// Replaces the reference's three hot stages:
//   * gridlink (utils/gridlink_impl.c.src:65-436): a device counting sort of the points into
//     a lattice of (x,y) columns x fine z slabs, written as SoA records (FP32 hi/lo grid
//     coordinates, FP64 copies, reference-lattice cell ids);
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
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

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
constexpr uint32_t kJMax = 2048;    // max j points per task
constexpr int kRxy = 2;             // lattice columns per rmax_xy
constexpr int kZFine = 8;           // z slabs per rmax_z
constexpr uint64_t kFlushPairs = 1ull << 22;  // per-warp accumulator flush interval
constexpr int kScanTile = 4096;

// ------------------------------------------------------------------------------------
// geometry of the GPU lattice and of the reference lattice
// ------------------------------------------------------------------------------------
struct Geom {
    double origin[3];
    double inv_s[3];
    double s[3];
    int n[3];  // n[0] x columns, n[1] y columns, n[2] z slabs
    double q[3];
    double inv_q[3];
    double ref_min[3];
    double ref_inv[3];
    int ref_n[3];
    int check_ref_bounds;
};

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

// min/max of x,y,z (slots 0..5: xmin,xmax,ymin,ymax,zmin,zmax) and max |w| (slot 6)
template <typename T>
__global__ void k_minmax(const T *x, const T *y, const T *z, const T *w, int64_t n,
                         unsigned long long *mm)
{
    double v[7] = {INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY, 0.0};
    bool bad = false;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = ld(x, i), b = ld(y, i), c = ld(z, i);
        if (!isfinite(a) || !isfinite(b) || !isfinite(c)) bad = true;
        v[0] = fmin(v[0], a); v[1] = fmax(v[1], a);
        v[2] = fmin(v[2], b); v[3] = fmax(v[3], b);
        v[4] = fmin(v[4], c); v[5] = fmax(v[5], c);
        if (w) v[6] = fmax(v[6], fabs(ld(w, i)));
    }
    for (int off = 16; off; off >>= 1) {
        for (int k = 0; k < 7; k++) {
            const double o = __shfl_down_sync(0xffffffffu, v[k], off);
            v[k] = (k & 1) || k == 6 ? fmax(v[k], o) : fmin(v[k], o);
        }
    }
    if (bad) atomicMax(&mm[7], 1ull);
    if ((threadIdx.x & 31) == 0) {
        for (int k = 0; k < 7; k++) {
            const unsigned long long e = ord_enc(v[k]);
            if ((k & 1) || k == 6) atomicMax(&mm[k], e); else atomicMin(&mm[k], e);
        }
    }
}

__device__ __forceinline__ int axis_cell(double c, const Geom &g, int a)
{
    int i = (int)floor((c - g.origin[a]) * g.inv_s[a]);
    i = i < 0 ? 0 : i;
    i = i >= g.n[a] ? g.n[a] - 1 : i;
    return i;
}

template <typename T>
__global__ void k_assign(const T *x, const T *y, const T *z, int64_t n, Geom g,
                         uint32_t *cellid, uint32_t *count, unsigned long long *oob)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const double a = ld(x, i), b = ld(y, i), c = ld(z, i);
        const int ix = axis_cell(a, g, 0), iy = axis_cell(b, g, 1), iz = axis_cell(c, g, 2);
        const uint32_t cell = ((uint32_t)ix * g.n[1] + iy) * (uint32_t)g.n[2] + iz;
        cellid[i] = cell;
        atomicAdd(&count[cell], 1u);
        if (g.check_ref_bounds) {
            // out-of-bounds test of the reference lattice (utils/gridlink_impl.c.src:165-183)
            int rx = (int)((a - g.ref_min[0]) * g.ref_inv[0]);
            int ry = (int)((b - g.ref_min[1]) * g.ref_inv[1]);
            int rz = (int)((c - g.ref_min[2]) * g.ref_inv[2]);
            if (rx > g.ref_n[0] - 1) rx--;
            if (ry > g.ref_n[1] - 1) ry--;
            if (rz > g.ref_n[2] - 1) rz--;
            if (rx < 0 || rx >= g.ref_n[0] || ry < 0 || ry >= g.ref_n[1] || rz < 0 || rz >= g.ref_n[2])
                atomicAdd(oob, 1ull);
        }
    }
}

__device__ __forceinline__ void split_hi_lo(double u, double q, double inv_q, float *hi, float *lo)
{
    const double h = rint(u * inv_q) * q;  // exact: q is a power of two
    *hi = (float)h;                        // exact: |h| / q < 2^24
    *lo = (float)(u - h);
}

template <typename T>
__global__ void k_scatter(const T *x, const T *y, const T *z, const T *w, int64_t n, Geom g,
                          const uint32_t *cellid, const uint32_t *cell_start, uint32_t *fill,
                          Lattice L)
{
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cellid[i];
        const uint32_t pos = cell_start[c] + atomicAdd(&fill[c], 1u);
        const double a = ld(x, i), b = ld(y, i), cz = ld(z, i);
        const double wv = w ? ld(w, i) : 1.0;
        float hx, hy, hz, lx, ly, lz;
        split_hi_lo(a - g.origin[0], g.q[0], g.inv_q[0], &hx, &lx);
        split_hi_lo(b - g.origin[1], g.q[1], g.inv_q[1], &hy, &ly);
        split_hi_lo(cz - g.origin[2], g.q[2], g.inv_q[2], &hz, &lz);
        L.hi[pos] = make_float4(hx, hy, hz, (float)wv);
        L.lo[pos] = make_float4(lx, ly, lz, 0.f);
        L.dbl[pos] = make_double4_32a(a, b, cz, wv);
        int rx = (int)((a - g.ref_min[0]) * g.ref_inv[0]);
        int ry = (int)((b - g.ref_min[1]) * g.ref_inv[1]);
        int rz = (int)((cz - g.ref_min[2]) * g.ref_inv[2]);
        if (rx > g.ref_n[0] - 1) rx--;
        if (ry > g.ref_n[1] - 1) ry--;
        if (rz > g.ref_n[2] - 1) rz--;
        L.refcell[pos] = (rx * g.ref_n[1] + ry) * g.ref_n[2] + rz;
        L.orig[pos] = (int)i;
        L.cellid[pos] = c;
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
    }
}

__global__ void k_scan_add(uint32_t *out, uint32_t n, const uint32_t *offs)
{
    const uint32_t base = blockIdx.x * (uint32_t)kScanTile;
    const uint32_t add = offs[blockIdx.x];
    for (int k = threadIdx.x; k < kScanTile; k += blockDim.x) {
        const uint32_t idx = base + k;
        if (idx < n) out[idx] += add;
    }
}

__global__ void k_set_total(uint32_t *out, uint32_t n, const uint32_t *blocksum_scan, uint32_t nblk)
{
    // blocksum_scan holds the exclusive scan (nblk+1 entries, last = total)
    out[n] = blocksum_scan[nblk];
}

__global__ void k_write_total_single(uint32_t *out, uint32_t n, const uint32_t *blocksums)
{
    out[n] = blocksums[0];
}

// ------------------------------------------------------------------------------------
// chunks (32 consecutive points of one column) and tasks
// ------------------------------------------------------------------------------------
__global__ void k_col_chunks(const uint32_t *cell_start, int ncols, int nz, uint32_t *chunks_per_col)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    const uint32_t a = cell_start[(uint32_t)c * nz], b = cell_start[(uint32_t)(c + 1) * nz];
    chunks_per_col[c] = (b - a + kChunk - 1) / kChunk;
}

__global__ void k_chunk_emit(const uint32_t *cell_start, int ncols, int nz, const uint32_t *chunk_off,
                             uint32_t *chunk_begin, uint32_t *chunk_count)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncols) return;
    const uint32_t a = cell_start[(uint32_t)c * nz], b = cell_start[(uint32_t)(c + 1) * nz];
    uint32_t o = chunk_off[c];
    for (uint32_t p = a; p < b; p += kChunk, o++) {
        chunk_begin[o] = p;
        chunk_count[o] = min((uint32_t)kChunk, b - p);
    }
}

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
};

__device__ __forceinline__ int floordiv(int a, int b)
{
    int q = a / b;
    if ((a % b != 0) && ((a < 0) != (b < 0))) q--;
    return q;
}

// Enumerates the tasks of one chunk.  With emit == false it only counts them.
template <bool EMIT>
__device__ uint32_t chunk_tasks(const TaskGeom &G, uint32_t ib, uint32_t icount, const uint32_t *cellid1,
                                const uint32_t *cs2, Task *out)
{
    const uint32_t c0 = cellid1[ib], c1 = cellid1[ib + icount - 1];
    const int nz = G.nz;
    const int col = (int)(c0 / nz);
    const int a = (int)(c0 % nz), b = (int)(c1 % nz);
    const int ix = col / G.ny, iy = col % G.ny;
    uint32_t ntask = 0;
    // periodic images are encoded in two bits; the lattice construction keeps |m| <= 1
    // (neighbour reach < half the period), anything else is reported and skipped.

    for (int dx = -G.reach_x; dx <= G.reach_x; dx++) {
        const int ux = ix + dx;
        int mx = 0, cx = ux;
        if (G.periodic[0]) { mx = floordiv(ux, G.nx); cx = ux - mx * G.nx; }
        else if (ux < 0 || ux >= G.nx) continue;
        for (int dy = -G.reach_y; dy <= G.reach_y; dy++) {
            if (G.autocorr && (dx < 0 || (dx == 0 && dy < 0))) continue;  // half stencil
            const int uy = iy + dy;
            int my = 0, cy = uy;
            if (G.periodic[1]) { my = floordiv(uy, G.ny); cy = uy - my * G.ny; }
            else if (uy < 0 || uy >= G.ny) continue;
            const double rx = fmax(0.0, (double)(abs(dx) - 1)) * G.s[0];
            const double ry = fmax(0.0, (double)(abs(dy) - 1)) * G.s[1];
            const double rho2 = rx * rx + ry * ry;
            if (rho2 >= G.rmax_xy * G.rmax_xy) continue;
            double W = G.rmax_z;
            if (G.rmax_3d > 0.0) W = fmin(W, sqrt(fmax(0.0, G.rmax_3d * G.rmax_3d - rho2)));
            const int wz = (int)ceil(W / G.s[2]);
            const bool own = G.autocorr && dx == 0 && dy == 0;
            const int klo = own ? a : a - wz;
            const int khi = b + wz;
            const int col2 = cx * G.ny + cy;
            const int mlo = G.periodic[2] ? floordiv(klo, nz) : 0;
            const int mhi = G.periodic[2] ? floordiv(khi, nz) : 0;
            if (mx < -1 || mx > 1 || my < -1 || my > 1 || mlo < -1 || mhi > 1) {
                if (G.error) atomicOr(G.error, 1u);
                continue;
            }
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
                    if (EMIT) {
                        Task t;
                        t.i_begin = ib;
                        t.j_begin = p;
                        t.j_end = min(je, p + kJMax);
                        t.meta = task_meta((int)icount, mx, my, mz, own_img && p == jb ? 1 : 0);
                        out[ntask] = t;
                    }
                    ntask++;
                }
            }
        }
    }
    return ntask;
}

__global__ void k_task_count(TaskGeom G, uint32_t nchunks, const uint32_t *chunk_begin, const uint32_t *chunk_count,
                             const uint32_t *cellid1, const uint32_t *cs2, uint32_t *ntasks)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    ntasks[k] = chunk_tasks<false>(G, chunk_begin[k], chunk_count[k], cellid1, cs2, nullptr);
}

__global__ void k_task_emit(TaskGeom G, uint32_t nchunks, const uint32_t *chunk_begin, const uint32_t *chunk_count,
                            const uint32_t *cellid1, const uint32_t *cs2, const uint32_t *task_off, Task *tasks)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nchunks) return;
    chunk_tasks<true>(G, chunk_begin[k], chunk_count[k], cellid1, cs2, tasks + task_off[k]);
}

// ------------------------------------------------------------------------------------
// pair kernels
// ------------------------------------------------------------------------------------
struct SmemLayout {
    int nedges, nbins, warps;
    size_t edges_off, guard_off, stage_off, hist_off, per_warp_hist, per_warp_stage, total;
};

__host__ __device__ inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

__host__ __device__ inline SmemLayout smem_layout(int nedges, int nbins, int warps, bool f64)
{
    SmemLayout L;
    L.nedges = nedges;
    L.nbins = nbins;
    L.warps = warps;
    size_t o = 0;
    L.edges_off = o;
    o = align_up(o + sizeof(double) * nedges, 16);
    L.guard_off = o;
    o = align_up(o + sizeof(float) * 2 * nedges, 16);
    L.stage_off = o;
    // f32: float4 hi[32] + float4 lo[32]; f64: double4_32a[32] + int rc[32] + int orig[32]
    L.per_warp_stage = f64 ? (32 * sizeof(double4_32a) + 64 * sizeof(int)) : (64 * sizeof(float4));
    o = align_up(o + L.per_warp_stage * warps, 16);
    L.hist_off = o;
    L.per_warp_hist = align_up((size_t)nbins * (8 + 8 + 4), 16);
    o += L.per_warp_hist * warps;
    L.total = o;
    return L;
}

struct WarpHist {
    unsigned long long *avg;
    unsigned long long *w;
    uint32_t *cnt;
};

__device__ __forceinline__ WarpHist warp_hist(unsigned char *smem, const SmemLayout &L, int warp)
{
    unsigned char *p = smem + L.hist_off + L.per_warp_hist * warp;
    WarpHist h;
    h.avg = (unsigned long long *)p;
    h.w = (unsigned long long *)(p + 8 * (size_t)L.nbins);
    h.cnt = (uint32_t *)(p + 16 * (size_t)L.nbins);
    return h;
}

template <bool NEED_AVG, bool NEED_W>
__device__ __forceinline__ void flush_hist(const PairArgs &A, WarpHist h, int lane)
{
    for (int b = lane; b < A.nbins; b += 32) {
        const uint32_t c = h.cnt[b];
        if (c) {
            atomicAdd(&A.g_cnt[b], (unsigned long long)c);
            h.cnt[b] = 0;
        }
        if (NEED_AVG) {
            const long long v = (long long)h.avg[b];
            if (v) {
                atomicAdd(&A.g_avg[b], (double)v * A.avg_unscale);
                h.avg[b] = 0;
            }
        }
        if (NEED_W) {
            const long long v = (long long)h.w[b];
            if (v) {
                atomicAdd(&A.g_w[b], (double)v * A.w_unscale);
                h.w[b] = 0;
            }
        }
    }
    __syncwarp();
}

__device__ __forceinline__ int guard_upper(const float *glo, int n, float v)
{
    // number of lower guards <= v
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (glo[mid] <= v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// first-point rule of the reference for wrapped auto-correlation pairs
__device__ __forceinline__ bool j_is_first(const PairArgs &A, uint32_t i, uint32_t j, double zi, double zj)
{
    const int ri = A.rc1[i], rj = A.rc2[j];
    if (rj != ri) return rj > ri;
    if (zj != zi) return zj < zi;
    return A.or2[j] < A.or1[i];
}

template <int MODE>
__device__ __forceinline__ int refine_pair(const PairArgs &A, const double *se, uint32_t i, uint32_t j,
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

template <int MODE, bool NEED_AVG, bool NEED_W>
__global__ void __launch_bounds__(256) k_pairs_f32(PairArgs A, SmemLayout SL)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *se = (double *)(smem + SL.edges_off);
    float *glo = (float *)(smem + SL.guard_off);
    float *ghi = glo + A.nedges;
    for (int k = threadIdx.x; k < A.nedges; k += blockDim.x) {
        se[k] = A.g_edges[k];
        glo[k] = A.g_guard[k];
        ghi[k] = A.g_guard[A.nedges + k];
    }
    float4 *sjhi = (float4 *)(smem + SL.stage_off + SL.per_warp_stage * warp);
    float4 *sjlo = sjhi + 32;
    WarpHist h = warp_hist(smem, SL, warp);
    for (int b = lane; b < A.nbins; b += 32) {
        h.cnt[b] = 0;
        h.avg[b] = 0;
        h.w[b] = 0;
    }
    __syncthreads();
    const float g_lo0 = glo[0];
    const float g_hiN = ghi[A.nedges - 1];
    const int nedges = A.nedges;
    uint64_t since_flush = 0, evaluated = 0;
    unsigned long long refined = 0;

    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(A.task_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= A.ntasks) break;
        const Task T = A.tasks[t];
        const int icount = (int)(T.meta & 63u) + 1;
        const int mx = (int)((T.meta >> 8) & 3u) - 1, my = (int)((T.meta >> 10) & 3u) - 1,
                  mz = (int)((T.meta >> 12) & 3u) - 1;
        const bool own = (T.meta >> 16) & 1u;
        const uint32_t i = T.i_begin + lane;
        const bool ivalid = lane < icount;
        float4 pi = ivalid ? A.hi1[i] : make_float4(1e30f, 1e30f, 1e30f, 0.f);
        // j is shifted by the image offset o; equivalently shift i by -o (exact on the grid)
        const float xi = pi.x - A.ohi[0][mx + 1], yi = pi.y - A.ohi[1][my + 1], zi = pi.z - A.ohi[2][mz + 1];
        float xil = 0.f, yil = 0.f, zil = 0.f;
        if (NEED_AVG) {
            const float4 pl = ivalid ? A.lo1[i] : make_float4(0.f, 0.f, 0.f, 0.f);
            xil = pl.x - A.olo[0][mx + 1];
            yil = pl.y - A.olo[1][my + 1];
            zil = pl.z - A.olo[2][mz + 1];
        }
        for (uint32_t jb = T.j_begin; jb < T.j_end; jb += 32) {
            const uint32_t nj = min(32u, T.j_end - jb);
            if ((uint32_t)lane < nj) {
                sjhi[lane] = A.hi2[jb + lane];
                if (NEED_AVG) sjlo[lane] = A.lo2[jb + lane];
            }
            __syncwarp();
            for (uint32_t k = 0; k < nj; k++) {
                const float4 pj = sjhi[k];
                const float dx = pj.x - xi, dy = pj.y - yi, dz = pj.z - zi;
                float r2;
                if (MODE == MODE_RPPI || MODE == MODE_WP) {
                    r2 = fmaf(dy, dy, dx * dx);
                    if (fabsf(dz) >= A.pimax_hi_f) continue;
                } else {
                    r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                }
                if (!(r2 >= g_lo0 && r2 < g_hiN)) continue;
                const uint32_t j = jb + k;
                if (own && j <= i) continue;
                // ---- candidate inside the outer guards: classify ----
                const int m = guard_upper(glo, nedges, r2);
                bool amb = r2 < ghi[m - 1];
                int bin = m;
                if (MODE == MODE_RPPI || MODE == MODE_WP) {
                    const float adz = fabsf(dz);
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
                float favg = 0.f;
                if (MODE == MODE_SMU) {
                    if (!(r2 > 0.f)) amb = true;
                    const float s = sqrtf(r2);
                    const float mu = fabsf(dz) / s;
                    const float emu = A.mu_band_abs / s + 6e-7f * mu + 1e-7f;
                    if (mu >= A.mu_max_f + emu) continue;  // definitely mu >= mu_max
                    if (mu > A.mu_max_f - emu) amb = true;
                    const float tmu = mu * A.inv_dmu_f;
                    int pb = (int)tmu;
                    const float bt = emu * A.inv_dmu_f + 3e-7f * tmu;
                    const float fr = tmu - (float)pb;
                    if ((pb >= 1 && fr < bt) || (1.f - fr) < bt) amb = true;
                    pb = pb > A.npibin ? A.npibin : pb;
                    bin = m * (A.npibin + 1) + pb;
                }
                double davg = 0.0, dw = 0.0;
                bool use_double = false;
                if (amb) {
                    refined++;
                    bin = refine_pair<MODE>(A, se, i, j, mx, my, mz, &davg, &dw);
                    if (bin < 0) continue;
                    use_double = true;
                } else if (NEED_AVG) {
                    const float4 pjl = sjlo[k];
                    const float dxp = dx + (pjl.x - xil), dyp = dy + (pjl.y - yil), dzp = dz + (pjl.z - zil);
                    if (MODE == MODE_RPPI || MODE == MODE_WP) {
                        favg = sqrtf(fmaf(dyp, dyp, dxp * dxp));
                    } else if (MODE == MODE_THETA) {
                        const float ch = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
                        favg = 2.f * asinf(0.5f * ch) * 57.29577951308232f;
                    } else {
                        favg = sqrtf(fmaf(dzp, dzp, fmaf(dyp, dyp, dxp * dxp)));
                    }
                }
                atomicAdd(&h.cnt[bin], 1u);
                if (NEED_AVG) {
                    const long long v = use_double ? __double2ll_rn(davg * (double)A.avg_scale_f)
                                                   : __float2ll_rn(favg * A.avg_scale_f);
                    atomicAdd(&h.avg[bin], (unsigned long long)v);
                }
                if (NEED_W) {
                    const long long v = use_double ? __double2ll_rn(dw * (double)A.w_scale_f)
                                                   : __float2ll_rn((pi.w * pj.w) * A.w_scale_f);
                    atomicAdd(&h.w[bin], (unsigned long long)v);
                }
            }
            __syncwarp();
        }
        const uint64_t np = (uint64_t)icount * (T.j_end - T.j_begin);
        since_flush += np;
        evaluated += np;
        if (since_flush > kFlushPairs) {
            flush_hist<NEED_AVG, NEED_W>(A, h, lane);
            since_flush = 0;
        }
    }
    flush_hist<NEED_AVG, NEED_W>(A, h, lane);
    for (int off = 16; off; off >>= 1) refined += __shfl_down_sync(0xffffffffu, refined, off);
    if (lane == 0) {
        atomicAdd(&A.g_stats[0], (unsigned long long)evaluated);
        atomicAdd(&A.g_stats[1], refined);
    }
}

template <int MODE, bool NEED_AVG, bool NEED_W>
__global__ void __launch_bounds__(256) k_pairs_f64(PairArgs A, SmemLayout SL)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *se = (double *)(smem + SL.edges_off);
    for (int k = threadIdx.x; k < A.nedges; k += blockDim.x) se[k] = A.g_edges[k];
    double4_32a *sj = (double4_32a *)(smem + SL.stage_off + SL.per_warp_stage * warp);
    int *srcell = (int *)(sj + 32);
    int *sorig = srcell + 32;
    WarpHist h = warp_hist(smem, SL, warp);
    for (int b = lane; b < A.nbins; b += 32) {
        h.cnt[b] = 0;
        h.avg[b] = 0;
        h.w[b] = 0;
    }
    __syncthreads();
    uint64_t since_flush = 0, evaluated = 0;
    const double avg_scale = (double)A.avg_scale_f, w_scale = (double)A.w_scale_f;

    while (true) {
        uint32_t t = 0;
        if (lane == 0) t = atomicAdd(A.task_counter, 1u);
        t = __shfl_sync(0xffffffffu, t, 0);
        if (t >= A.ntasks) break;
        const Task T = A.tasks[t];
        const int icount = (int)(T.meta & 63u) + 1;
        const int mx = (int)((T.meta >> 8) & 3u) - 1, my = (int)((T.meta >> 10) & 3u) - 1,
                  mz = (int)((T.meta >> 12) & 3u) - 1;
        const bool own = (T.meta >> 16) & 1u;
        const bool wrapped = (mx | my | mz) != 0;
        const uint32_t i = T.i_begin + lane;
        const bool ivalid = lane < icount;
        const double4_32a pi = ivalid ? A.d1[i] : make_double4_32a(0, 0, 0, 0);
        const int rci = ivalid ? A.rc1[i] : 0;
        const int ori = ivalid ? A.or1[i] : 0;
        const double ox = A.odbl[0][mx + 1], oy = A.odbl[1][my + 1], oz = A.odbl[2][mz + 1];
        for (uint32_t jb = T.j_begin; jb < T.j_end; jb += 32) {
            const uint32_t nj = min(32u, T.j_end - jb);
            if ((uint32_t)lane < nj) {
                sj[lane] = A.d2[jb + lane];
                srcell[lane] = A.rc2[jb + lane];
                sorig[lane] = A.or2[jb + lane];
            }
            __syncwarp();
            if (ivalid) {
                for (uint32_t k = 0; k < nj; k++) {
                    const uint32_t j = jb + k;
                    if (own && j <= i) continue;
                    const double4_32a pj = sj[k];
                    double avg_term = 0.0;
                    int bin;
                    if (MODE != MODE_THETA && A.autocorr && wrapped &&
                        (srcell[k] > rci || (srcell[k] == rci && (pj.z < pi.z || (pj.z == pi.z && sorig[k] < ori))))) {
                        bin = ref_eval<MODE>(A, se, pj.x, pj.y, pj.z, pi.x, pi.y, pi.z, ox, oy, oz, &avg_term);
                    } else {
                        bin = ref_eval<MODE>(A, se, pi.x, pi.y, pi.z, pj.x, pj.y, pj.z, -ox, -oy, -oz, &avg_term);
                    }
                    if (bin < 0) continue;
                    atomicAdd(&h.cnt[bin], 1u);
                    if (NEED_AVG) atomicAdd(&h.avg[bin], (unsigned long long)__double2ll_rn(avg_term * avg_scale));
                    if (NEED_W) atomicAdd(&h.w[bin], (unsigned long long)__double2ll_rn(pi.w * pj.w * w_scale));
                }
            }
            __syncwarp();
        }
        const uint64_t np = (uint64_t)icount * (T.j_end - T.j_begin);
        since_flush += np;
        evaluated += np;
        if (since_flush > kFlushPairs) {
            flush_hist<NEED_AVG, NEED_W>(A, h, lane);
            since_flush = 0;
        }
    }
    flush_hist<NEED_AVG, NEED_W>(A, h, lane);
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

static int ensure(DevBuf &b, size_t bytes)
{
    if (bytes == 0) bytes = 16;
    if (b.cap >= bytes) return EXIT_SUCCESS;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = bytes + bytes / 4;
    CF_CUDA(cudaMalloc(&b.p, want));
    b.cap = want;
    return EXIT_SUCCESS;
}

struct SetBufs {
    DevBuf raw[4];  // device copies of x, y, z, w as given (float or double)
    const void *in[4];  // arrays the lattice is built from: raw[] or caller-owned device arrays
    DevBuf cellid_u, count, fill, cell_start;
    DevBuf hi, lo, dbl, refcell, orig, cellid;
};

struct Engine {
    bool init = false;
    int device = -1;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[6];
    SetBufs set[2];
    DevBuf mm, oob, scan_tmp[4], chunk_cnt, chunk_off, chunk_begin, chunk_count, ntask, task_off, tasks;
    DevBuf hist_cnt, hist_avg, hist_w, stats, counter, edges, guards;
    int precision = CF_PRECISION_FP32_REFINE;
    int launches = 0;  // kernels launched by the current call
    cf_engine_stats last;
};

static Engine g_eng;
static pthread_mutex_t g_lock = PTHREAD_MUTEX_INITIALIZER;

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
    CF_CUDA(cudaStreamCreateWithFlags(&g_eng.stream, cudaStreamNonBlocking));
    for (int k = 0; k < 6; k++) CF_CUDA(cudaEventCreate(&g_eng.ev[k]));
    g_eng.init = true;
    return EXIT_SUCCESS;
}

// exclusive scan; out must have n+1 entries
static int scan_u32(const uint32_t *in, uint32_t *out, uint32_t n, int level)
{
    cudaStream_t st = g_eng.stream;
    if (n == 0) {
        CF_CUDA(cudaMemsetAsync(out, 0, sizeof(uint32_t), st));
        return EXIT_SUCCESS;
    }
    if (level >= 4) CF_FAIL("scan too deep");
    const uint32_t nblk = (n + kScanTile - 1) / kScanTile;
    if (ensure(g_eng.scan_tmp[level], sizeof(uint32_t) * (2 * (size_t)nblk + 2)) != EXIT_SUCCESS) return EXIT_FAILURE;
    uint32_t *bs = (uint32_t *)g_eng.scan_tmp[level].p;
    uint32_t *bs_scan = bs + nblk;  // nblk+1 entries
    k_scan_tile<<<nblk, 1024, 0, st>>>(in, out, n, bs);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    if (nblk == 1) {
        k_write_total_single<<<1, 1, 0, st>>>(out, n, bs);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
        return EXIT_SUCCESS;
    }
    if (scan_u32(bs, bs_scan, nblk, level + 1) != EXIT_SUCCESS) return EXIT_FAILURE;
    k_scan_add<<<nblk, 1024, 0, st>>>(out, n, bs_scan);
    g_eng.launches++;
    k_set_total<<<1, 1, 0, st>>>(out, n, bs_scan, nblk);
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

template <typename T>
static int upload_and_minmax(int s, int64_t n, const void *x, const void *y, const void *z, const void *w,
                             bool on_device, unsigned long long *mm_dev)
{
    SetBufs &B = g_eng.set[s];
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
    k_minmax<T><<<grid_for(n, 256), 256, 0, g_eng.stream>>>((const T *)B.in[0], (const T *)B.in[1],
                                                            (const T *)B.in[2], (const T *)B.in[3], n, mm_dev);
    CF_CUDA(cudaGetLastError());
    g_eng.launches++;
    return EXIT_SUCCESS;
}

template <typename T>
static int build_lattice(int s, int64_t n, bool has_w, const Geom &g, uint32_t ncells, unsigned long long *oob)
{
    SetBufs &B = g_eng.set[s];
    cudaStream_t st = g_eng.stream;
    if (ensure(B.cellid_u, sizeof(uint32_t) * n) || ensure(B.count, sizeof(uint32_t) * ncells) ||
        ensure(B.fill, sizeof(uint32_t) * ncells) || ensure(B.cell_start, sizeof(uint32_t) * ((size_t)ncells + 1)) ||
        ensure(B.hi, sizeof(float4) * n) || ensure(B.lo, sizeof(float4) * n) || ensure(B.dbl, sizeof(double4_32a) * n) ||
        ensure(B.refcell, sizeof(int) * n) || ensure(B.orig, sizeof(int) * n) || ensure(B.cellid, sizeof(uint32_t) * n))
        return EXIT_FAILURE;
    CF_CUDA(cudaMemsetAsync(B.count.p, 0, sizeof(uint32_t) * ncells, st));
    CF_CUDA(cudaMemsetAsync(B.fill.p, 0, sizeof(uint32_t) * ncells, st));
    const T *x = (const T *)B.in[0], *y = (const T *)B.in[1], *z = (const T *)B.in[2];
    const T *w = has_w ? (const T *)B.in[3] : nullptr;
    const int grid = grid_for(n, 256);
    k_assign<T><<<grid, 256, 0, st>>>(x, y, z, n, g, (uint32_t *)B.cellid_u.p, (uint32_t *)B.count.p, oob);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    if (scan_u32((const uint32_t *)B.count.p, (uint32_t *)B.cell_start.p, ncells, 0) != EXIT_SUCCESS) return EXIT_FAILURE;
    Lattice L;
    L.hi = (float4 *)B.hi.p;
    L.lo = (float4 *)B.lo.p;
    L.dbl = (double4_32a *)B.dbl.p;
    L.refcell = (int *)B.refcell.p;
    L.orig = (int *)B.orig.p;
    L.cellid = (uint32_t *)B.cellid.p;
    L.cell_start = (uint32_t *)B.cell_start.p;
    k_scatter<T><<<grid, 256, 0, st>>>(x, y, z, w, n, g, (const uint32_t *)B.cellid_u.p,
                                       (const uint32_t *)B.cell_start.p, (uint32_t *)B.fill.p, L);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    return EXIT_SUCCESS;
}

template <int MODE, bool AVG, bool W>
static int launch_pairs_t(const PairArgs &A, bool f64, int *launched)
{
    const int nedges = A.nedges;
    int warps = 8;
    SmemLayout SL = smem_layout(nedges, A.nbins, warps, f64);
    while (SL.total > 200 * 1024 && warps > 1) {
        warps >>= 1;
        SL = smem_layout(nedges, A.nbins, warps, f64);
    }
    if (SL.total > 220 * 1024) CF_FAIL("histogram too large for on-chip accumulation (%d bins)", A.nbins);
    const int threads = warps * 32;
    int per_sm = 1;
    if (f64) {
        auto kern = k_pairs_f64<MODE, AVG, W>;
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, SL.total));
        if (per_sm < 1) per_sm = 1;
        kern<<<g_eng.num_sms * per_sm, threads, SL.total, g_eng.stream>>>(A, SL);
        g_eng.launches++;
    } else {
        auto kern = k_pairs_f32<MODE, AVG, W>;
        CF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SL.total));
        CF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, threads, SL.total));
        if (per_sm < 1) per_sm = 1;
        kern<<<g_eng.num_sms * per_sm, threads, SL.total, g_eng.stream>>>(A, SL);
        g_eng.launches++;
    }
    CF_CUDA(cudaGetLastError());
    (*launched)++;
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

static int launch_pairs(int mode, const PairArgs &A, bool f64, bool avg, bool w, int *launched)
{
    switch (mode) {
    case MODE_R3: return launch_pairs_m<MODE_R3>(A, f64, avg, w, launched);
    case MODE_RPPI: return launch_pairs_m<MODE_RPPI>(A, f64, avg, w, launched);
    case MODE_WP: return launch_pairs_m<MODE_WP>(A, f64, avg, w, launched);
    case MODE_SMU: return launch_pairs_m<MODE_SMU>(A, f64, avg, w, launched);
    case MODE_THETA: return launch_pairs_m<MODE_THETA>(A, f64, avg, w, launched);
    }
    CF_FAIL("unknown mode %d", mode);
}

// error band for an edge value e given the per-axis coordinate error bound |delta|
static double edge_band(double e, double delta)
{
    const double u = 5.9604644775390625e-08;  // 2^-24
    const double re = sqrt(fabs(e));
    return 2.0 * (3.1 * u * fabs(e) + 2.0 * re * delta + delta * delta + 1e-14 * (fabs(e) + 1.0));
}

static int run_locked(cf_job *J, cf_hist *H)
{
    if (engine_init() != EXIT_SUCCESS) return EXIT_FAILURE;
    cudaStream_t st = g_eng.stream;
    memset(&g_eng.last, 0, sizeof(g_eng.last));
    g_eng.launches = 0;
    const int mode = J->mode;
    const bool two_d = (mode == MODE_RPPI || mode == MODE_SMU);
    const int nbins = two_d ? J->nedges * (J->npibin + 1) : J->nedges;
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

    CF_CUDA(cudaEventRecord(g_eng.ev[0], st));
    // ---- upload + extent ----
    if (ensure(g_eng.mm, sizeof(unsigned long long) * 16) != EXIT_SUCCESS) return EXIT_FAILURE;
    unsigned long long *mm = (unsigned long long *)g_eng.mm.p;
    unsigned long long mm_init[16];
    for (int k = 0; k < 16; k++) mm_init[k] = (k % 8 == 6 || k % 8 == 7 || (k % 8) % 2 == 1) ? 0ull : ~0ull;
    CF_CUDA(cudaMemcpyAsync(mm, mm_init, sizeof(mm_init), cudaMemcpyHostToDevice, st));
    const int nsets = autocorr ? 1 : 2;
    for (int s = 0; s < nsets; s++) {
        const int64_t n = s ? n2 : n1;
        const void *x = s ? J->x2 : J->x1, *y = s ? J->y2 : J->y1, *z = s ? J->z2 : J->z1;
        const void *w = need_w ? (s ? J->w2 : J->w1) : nullptr;
        if (!x || !y || !z || (need_w && !w)) CF_FAIL("NULL input array");
        int rc = isf ? upload_and_minmax<float>(s, n, x, y, z, w, J->inputs_on_device != 0, mm + 8 * s)
                     : upload_and_minmax<double>(s, n, x, y, z, w, J->inputs_on_device != 0, mm + 8 * s);
        if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    }
    const bool dev_float = isf;
    unsigned long long mmh[16];
    CF_CUDA(cudaMemcpyAsync(mmh, mm, sizeof(mmh), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    double lo[3], hi[3], wmax[2] = {0, 0};
    for (int a = 0; a < 3; a++) {
        lo[a] = ord_dec(mmh[2 * a]);
        hi[a] = ord_dec(mmh[2 * a + 1]);
        if (nsets == 2) {
            lo[a] = fmin(lo[a], ord_dec(mmh[8 + 2 * a]));
            hi[a] = fmax(hi[a], ord_dec(mmh[8 + 2 * a + 1]));
        }
    }
    wmax[0] = ord_dec(mmh[6]);
    wmax[1] = nsets == 2 ? ord_dec(mmh[14]) : wmax[0];
    if (mmh[7] != 0 || (nsets == 2 && mmh[15] != 0)) CF_FAIL("non-finite input coordinates");
    for (int a = 0; a < 3; a++) {
        if (!isfinite(lo[a]) || !isfinite(hi[a])) CF_FAIL("non-finite input coordinates");
    }
    cf_geometry geo;
    if (cf_resolve_geometry(&J->rule, lo, hi, &geo) != EXIT_SUCCESS) return EXIT_FAILURE;
    J->geom = geo;

    // ---- GPU lattice geometry ----
    Geom g;
    memset(&g, 0, sizeof(g));
    const double rlim[3] = {J->rmax_xy, J->rmax_xy, J->rmax_z};
    const int refine[3] = {kRxy, kRxy, kZFine};
    double span[3], delta[3];
    for (int a = 0; a < 3; a++) {
        const bool per = geo.periodic[a] && geo.wrap[a] > 0.0;
        double ext = hi[a] - lo[a];
        if (per) {
            if (ext > geo.wrap[a] * (1.0 + 1e-12)) {
                CF_FAIL("points span %g along axis %d, more than the periodic length %g", ext, a, geo.wrap[a]);
            }
            ext = geo.wrap[a];
        }
        int n = 1;
        if (ext > 0.0 && rlim[a] > 0.0) {
            // cells slightly wider than rlim/refine so that the neighbour reach is exactly 'refine'
            double nn = floor(ext / (rlim[a] / refine[a] * (1.0 + 1e-6)));
            if (nn > 4096) nn = 4096;
            if (nn < 1) nn = 1;
            n = (int)nn;
        }
        g.n[a] = n;
        g.origin[a] = lo[a];
        g.s[a] = ext > 0.0 ? ext / n : 1.0;
        g.inv_s[a] = 1.0 / g.s[a];
        span[a] = fmax(ext, 1e-300) + (per ? 2.0 * geo.wrap[a] : 0.0);
        g.q[a] = pow2_ceil(span[a]) * ldexp(1.0, -23);
        g.inv_q[a] = 1.0 / g.q[a];
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
    const uint32_t ncols = (uint32_t)g.n[0] * g.n[1];
    const uint32_t ncells = ncols * (uint32_t)g.n[2];
    g_eng.last.num_cells = (int)ncells;

    // ---- lattices ----
    if (ensure(g_eng.oob, sizeof(unsigned long long)) != EXIT_SUCCESS) return EXIT_FAILURE;
    unsigned long long *oob = (unsigned long long *)g_eng.oob.p;
    CF_CUDA(cudaMemsetAsync(oob, 0, sizeof(unsigned long long), st));
    for (int s = 0; s < nsets; s++) {
        const int64_t n = s ? n2 : n1;
        int rc = dev_float ? build_lattice<float>(s, n, need_w, g, ncells, oob)
                           : build_lattice<double>(s, n, need_w, g, ncells, oob);
        if (rc != EXIT_SUCCESS) return EXIT_FAILURE;
    }
    SetBufs &S1 = g_eng.set[0];
    SetBufs &S2 = g_eng.set[nsets - 1];

    // ---- chunks ----
    if (ensure(g_eng.chunk_cnt, sizeof(uint32_t) * ncols) || ensure(g_eng.chunk_off, sizeof(uint32_t) * ((size_t)ncols + 1)))
        return EXIT_FAILURE;
    k_col_chunks<<<(ncols + 255) / 256, 256, 0, st>>>((const uint32_t *)S1.cell_start.p, (int)ncols, g.n[2],
                                                      (uint32_t *)g_eng.chunk_cnt.p);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    if (scan_u32((const uint32_t *)g_eng.chunk_cnt.p, (uint32_t *)g_eng.chunk_off.p, ncols, 0) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    const uint32_t max_chunks = (uint32_t)((n1 + kChunk - 1) / kChunk + ncols);
    if (ensure(g_eng.chunk_begin, sizeof(uint32_t) * max_chunks) || ensure(g_eng.chunk_count, sizeof(uint32_t) * max_chunks))
        return EXIT_FAILURE;
    k_chunk_emit<<<(ncols + 255) / 256, 256, 0, st>>>((const uint32_t *)S1.cell_start.p, (int)ncols, g.n[2],
                                                      (const uint32_t *)g_eng.chunk_off.p,
                                                      (uint32_t *)g_eng.chunk_begin.p, (uint32_t *)g_eng.chunk_count.p);
    g_eng.launches++;
    CF_CUDA(cudaGetLastError());
    uint32_t nchunks = 0;
    unsigned long long oob_h = 0;
    CF_CUDA(cudaMemcpyAsync(&nchunks, (uint32_t *)g_eng.chunk_off.p + ncols, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(&oob_h, oob, sizeof(oob_h), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    if (oob_h > 0) CF_FAIL("%llu particles are out of bounds. Check periodic wrapping?", oob_h);
    if (nchunks > max_chunks) CF_FAIL("internal: chunk count overflow");

    // ---- tasks ----
    if (ensure(g_eng.counter, sizeof(uint32_t) * 4) != EXIT_SUCCESS) return EXIT_FAILURE;
    CF_CUDA(cudaMemsetAsync(g_eng.counter.p, 0, sizeof(uint32_t) * 4, st));
    // prune margins cover FP64 rounding of the cell assignment only (the FP32 error bounds
    // matter for classification, not for which neighbours are visited)
    double maxabs_all = 0.0;
    for (int a = 0; a < 3; a++) maxabs_all = fmax(maxabs_all, fmax(fabs(lo[a]), fabs(hi[a])) + (geo.periodic[a] ? geo.wrap[a] : 0.0));
    const double margin_xy = 1e-9 * fmax(g.s[0], g.s[1]) + 1e-13 * maxabs_all;
    const double margin_z = 1e-9 * g.s[2] + 1e-13 * maxabs_all;
    TaskGeom G;
    memset(&G, 0, sizeof(G));
    G.nx = g.n[0];
    G.ny = g.n[1];
    G.nz = g.n[2];
    for (int a = 0; a < 3; a++) G.periodic[a] = geo.periodic[a] && geo.wrap[a] > 0.0;
    G.autocorr = autocorr;
    G.mode = mode;
    G.s[0] = g.s[0];
    G.s[1] = g.s[1];
    G.s[2] = g.s[2];
    G.rmax_xy = J->rmax_xy + margin_xy;
    G.rmax_z = J->rmax_z + margin_z;
    G.rmax_3d = J->rmax_3d > 0.0 ? J->rmax_3d + fmax(margin_xy, margin_z) : 0.0;
    G.reach_x = (int)ceil(G.rmax_xy / g.s[0]);
    G.reach_y = (int)ceil(G.rmax_xy / g.s[1]);
    if (G.reach_x > 64 || G.reach_y > 64) CF_FAIL("internal: neighbour reach too large");
    G.error = (uint32_t *)g_eng.counter.p + 2;
    if (ensure(g_eng.ntask, sizeof(uint32_t) * ((size_t)nchunks + 1)) ||
        ensure(g_eng.task_off, sizeof(uint32_t) * ((size_t)nchunks + 2)))
        return EXIT_FAILURE;
    if (nchunks > 0) {
        k_task_count<<<(nchunks + 127) / 128, 128, 0, st>>>(G, nchunks, (const uint32_t *)g_eng.chunk_begin.p,
                                                            (const uint32_t *)g_eng.chunk_count.p,
                                                            (const uint32_t *)S1.cellid.p,
                                                            (const uint32_t *)S2.cell_start.p, (uint32_t *)g_eng.ntask.p);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
    }
    if (scan_u32((const uint32_t *)g_eng.ntask.p, (uint32_t *)g_eng.task_off.p, nchunks, 0) != EXIT_SUCCESS)
        return EXIT_FAILURE;
    uint32_t ntasks = 0, task_err = 0;
    CF_CUDA(cudaMemcpyAsync(&ntasks, (uint32_t *)g_eng.task_off.p + nchunks, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(&task_err, G.error, sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaStreamSynchronize(st));
    if (task_err) CF_FAIL("internal: neighbour search needed a periodic image beyond +-1");
    if (ensure(g_eng.tasks, sizeof(Task) * ((size_t)ntasks + 1)) != EXIT_SUCCESS) return EXIT_FAILURE;
    if (nchunks > 0) {
        k_task_emit<<<(nchunks + 127) / 128, 128, 0, st>>>(G, nchunks, (const uint32_t *)g_eng.chunk_begin.p,
                                                           (const uint32_t *)g_eng.chunk_count.p,
                                                           (const uint32_t *)S1.cellid.p, (const uint32_t *)S2.cell_start.p,
                                                           (const uint32_t *)g_eng.task_off.p, (Task *)g_eng.tasks.p);
        g_eng.launches++;
        CF_CUDA(cudaGetLastError());
    }
    g_eng.last.tasks = ntasks;
    CF_CUDA(cudaEventRecord(g_eng.ev[1], st));

    // ---- pair-kernel arguments ----
    PairArgs A;
    memset(&A, 0, sizeof(A));
    A.hi1 = (const float4 *)S1.hi.p;
    A.lo1 = (const float4 *)S1.lo.p;
    A.d1 = (const double4_32a *)S1.dbl.p;
    A.rc1 = (const int *)S1.refcell.p;
    A.or1 = (const int *)S1.orig.p;
    A.hi2 = (const float4 *)S2.hi.p;
    A.lo2 = (const float4 *)S2.lo.p;
    A.d2 = (const double4_32a *)S2.dbl.p;
    A.rc2 = (const int *)S2.refcell.p;
    A.or2 = (const int *)S2.orig.p;
    A.tasks = (const Task *)g_eng.tasks.p;
    A.ntasks = ntasks;
    A.nedges = J->nedges;
    A.nbins = nbins;
    A.npibin = J->npibin;
    A.autocorr = autocorr;
    A.fma_formula = J->fma_formula;
    A.chord_formula = J->chord_formula;
    for (int a = 0; a < 3; a++) {
        for (int m = -1; m <= 1; m++) {
            const double o = (G.periodic[a]) ? m * geo.wrap[a] : 0.0;
            const double oh = rint(o * g.inv_q[a]) * g.q[a];
            A.odbl[a][m + 1] = o;
            A.ohi[a][m + 1] = (float)oh;
            A.olo[a][m + 1] = (float)(o - oh);
        }
    }
    // coordinate error bounds
    const double dxy = sqrt(delta[0] * delta[0] + delta[1] * delta[1]);
    const double d3 = sqrt(dxy * dxy + delta[2] * delta[2]);
    const double dlim = (mode == MODE_RPPI || mode == MODE_WP) ? dxy : d3;
    // guards: for theta the classified quantity is the squared chord 2*(1 - cos)
    if (ensure(g_eng.edges, sizeof(double) * J->nedges) || ensure(g_eng.guards, sizeof(float) * 2 * J->nedges))
        return EXIT_FAILURE;
    float guards_h[2 * CF_MAX_EDGES];
    for (int k = 0; k < J->nedges; k++) {
        double e = J->edges[k];
        double band;
        if (mode == MODE_THETA) {
            e = 2.0 * (1.0 - J->edges[k]);
            band = edge_band(e, dlim) + 8e-15;
        } else {
            band = edge_band(e, dlim);
        }
        guards_h[k] = f_down(e - band);
        guards_h[J->nedges + k] = f_up(e + band);
    }
    // keep both guard arrays non-decreasing (widening a band is always safe)
    for (int k = J->nedges - 2; k >= 0; k--) guards_h[k] = fminf(guards_h[k], guards_h[k + 1]);
    for (int k = 1; k < J->nedges; k++) guards_h[J->nedges + k] = fmaxf(guards_h[J->nedges + k], guards_h[J->nedges + k - 1]);
    CF_CUDA(cudaMemcpyAsync(g_eng.edges.p, J->edges, sizeof(double) * J->nedges, cudaMemcpyHostToDevice, st));
    CF_CUDA(cudaMemcpyAsync(g_eng.guards.p, guards_h, sizeof(float) * 2 * J->nedges, cudaMemcpyHostToDevice, st));
    A.g_edges = (const double *)g_eng.edges.p;
    A.g_guard = (const float *)g_eng.guards.p;
    A.dz_err = (float)(2.0 * delta[2]);
    A.dxy_err = (float)(2.0 * dxy);
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
    }
    if (mode == MODE_SMU) {
        A.sqr_mu_max = J->mu_max * J->mu_max;
        const double dmu = J->mu_max / J->npibin;
        A.inv_dmu = 1.0 / dmu;
        A.mu_max_f = (float)J->mu_max;
        A.inv_dmu_f = (float)A.inv_dmu;
        A.mu_band_abs = (float)(2.0 * (delta[2] + d3) * 2.0 + 1e-12);
    }
    // fixed-point accumulator scales: one term must stay below 2^40
    double avg_max = 1.0;
    if (mode == MODE_THETA) avg_max = 180.0;
    else avg_max = sqrt(fabs(J->edges[J->nedges - 1])) * 1.01 + 1e-300;
    const int sa = 40 - (int)ceil(log2(avg_max));
    A.avg_scale_f = (float)ldexp(1.0, sa);
    A.avg_unscale = ldexp(1.0, -sa);
    const double w2 = fmax(wmax[0] * wmax[1], 1e-30) * 1.01;
    int sw = 40 - (int)ceil(log2(w2));
    if (sw > 100) sw = 100;
    A.w_scale_f = (float)ldexp(1.0, sw);
    A.w_unscale = ldexp(1.0, -sw);

    if (ensure(g_eng.hist_cnt, sizeof(unsigned long long) * nbins) || ensure(g_eng.hist_avg, sizeof(double) * nbins) ||
        ensure(g_eng.hist_w, sizeof(double) * nbins) || ensure(g_eng.stats, sizeof(unsigned long long) * 4) ||
        ensure(g_eng.counter, sizeof(uint32_t) * 4))
        return EXIT_FAILURE;
    CF_CUDA(cudaMemsetAsync(g_eng.hist_cnt.p, 0, sizeof(unsigned long long) * nbins, st));
    CF_CUDA(cudaMemsetAsync(g_eng.hist_avg.p, 0, sizeof(double) * nbins, st));
    CF_CUDA(cudaMemsetAsync(g_eng.hist_w.p, 0, sizeof(double) * nbins, st));
    CF_CUDA(cudaMemsetAsync(g_eng.stats.p, 0, sizeof(unsigned long long) * 4, st));
    CF_CUDA(cudaMemsetAsync(g_eng.counter.p, 0, sizeof(uint32_t) * 4, st));
    A.g_cnt = (unsigned long long *)g_eng.hist_cnt.p;
    A.g_avg = (double *)g_eng.hist_avg.p;
    A.g_w = (double *)g_eng.hist_w.p;
    A.g_stats = (unsigned long long *)g_eng.stats.p;
    A.task_counter = (uint32_t *)g_eng.counter.p;

    int launched = 0;
    CF_CUDA(cudaEventRecord(g_eng.ev[2], st));
    if (ntasks > 0) {
        const bool f64 = g_eng.precision == CF_PRECISION_FP64;
        if (launch_pairs(mode, A, f64, J->need_avg != 0, need_w, &launched) != EXIT_SUCCESS) return EXIT_FAILURE;
    }
    CF_CUDA(cudaEventRecord(g_eng.ev[3], st));
    unsigned long long stats_h[4];
    CF_CUDA(cudaMemcpyAsync(H->npairs, g_eng.hist_cnt.p, sizeof(uint64_t) * nbins, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(H->avg, g_eng.hist_avg.p, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(H->wsum, g_eng.hist_w.p, sizeof(double) * nbins, cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaMemcpyAsync(stats_h, g_eng.stats.p, sizeof(stats_h), cudaMemcpyDeviceToHost, st));
    CF_CUDA(cudaEventRecord(g_eng.ev[4], st));
    CF_CUDA(cudaStreamSynchronize(st));
    float ms_pairs = 0.f, ms_grid = 0.f, ms_total = 0.f;
    CF_CUDA(cudaEventElapsedTime(&ms_pairs, g_eng.ev[2], g_eng.ev[3]));
    CF_CUDA(cudaEventElapsedTime(&ms_grid, g_eng.ev[0], g_eng.ev[1]));
    CF_CUDA(cudaEventElapsedTime(&ms_total, g_eng.ev[0], g_eng.ev[4]));
    g_eng.last.pair_kernel_ms = ms_pairs;
    g_eng.last.gridlink_ms = ms_grid;
    g_eng.last.total_gpu_ms = ms_total;
    g_eng.last.pairs_evaluated = stats_h[0];
    g_eng.last.pairs_refined = stats_h[1];
    g_eng.last.kernel_launches = g_eng.launches;
    (void)launched;
    return EXIT_SUCCESS;
}

}  // namespace

extern "C" int cf_engine_run(cf_job *job, cf_hist *out)
{
    pthread_mutex_lock(&g_lock);
    const int rc = run_locked(job, out);
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
