// cf_noalloc.cu -- DD(r) cross-correlation by direct summation that allocates no memory.
//
// Who this is for: callers that must not allocate inside the call -- a service whose device
// memory is carved out up front and must not grow, a caller that runs next to latency-sensitive
// work and cannot afford the device-wide synchronisation a cudaMalloc/cudaFree may bring, or a
// host process under a hard memory budget.  The regular entry points build a lattice and a work
// list whose size depends on the catalogues, so they allocate (and cache) device buffers; this
// one does not.
//
// What it computes: the reference's countpairs() cross-correlation (autocorr = 0) in double
// precision -- npairs per bin, optionally the mean separation and the mean pair_product weight --
// by evaluating every pair of the two catalogues with the reference's own formula (the same
// exact FP64 evaluation the FP64 pair kernel of the engine uses, theory/DD/countpairs_kernels.c.src:
// dx = x2 - (x1 + off), r^2 summed as the caller's instruction set would).  With periodic
// wrapping the offset `off` is the one periodic image that can bring the pair within rmax,
// which is the image the reference's lattice pairs it under.  Cost grows as ND1 * ND2: it is
// meant for small catalogues (a few tens of thousands of points).
//
// Scratch: one file-scope device array (kScratchDoubles doubles, 4 KB) holding the squared bin
// edges and the per-bin count / sum accumulators.  Its address is looked up once per device with
// cudaGetSymbolAddress and kept for the life of the process, so a cudaDeviceReset, or another
// context made current on the same device, is not supported after the first call.  Each call
// copies the squared edges and zeros over the accumulators itself before counting, so nothing
// has to be cleared beforehand; after the call the array holds that call's raw sums.

#include <cuda_runtime.h>
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "cf_device.cuh"
#include "cf_host.h"

using namespace cf;

namespace {

constexpr int kMaxEdges = 128;                     // bin edges (nbin) accepted by this entry point
constexpr int kScratchDoubles = 4 * kMaxEdges;     // squared edges | counts | r sums | weight sums
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

struct DirectArgs {
    const double *x1, *y1, *z1, *w1;
    const double *x2, *y2, *z2, *w2;
    int64_t n1, n2;
    int64_t j_per_block;  // j range of one blockIdx.y, a multiple of kThreads
    double box[3], half[3];
};

// Every pair (i in set 1, j in set 2); one i per thread, the j of a block staged in shared memory.
// Counts and sums are gathered per block in shared memory and added to the scratch histogram.
template <bool RAVG, bool W, bool PERIODIC>
__global__ void __launch_bounds__(kThreads) k_cross_direct(PairArgs A, DirectArgs D, double *scratch)
{
    __shared__ double se[kMaxEdges];
    __shared__ unsigned long long hcnt[kMaxEdges];
    __shared__ double hr[kMaxEdges], hw[kMaxEdges];
    __shared__ double4_32a sj[kThreads];
    const int nb = A.nedges;
    for (int k = threadIdx.x; k < nb; k += kThreads) {
        se[k] = scratch[k];
        hcnt[k] = 0;
        hr[k] = 0.0;
        hw[k] = 0.0;
    }
    const int64_t i = (int64_t)blockIdx.x * kThreads + threadIdx.x;
    const bool iv = i < D.n1;
    const double xi = iv ? D.x1[i] : 0.0, yi = iv ? D.y1[i] : 0.0, zi = iv ? D.z1[i] : 0.0;
    const double wi = (W && iv) ? D.w1[i] : 0.0;
    const int64_t j0 = (int64_t)blockIdx.y * D.j_per_block;
    const int64_t j1 = min(D.n2, j0 + D.j_per_block);
    __syncthreads();
    for (int64_t jt = j0; jt < j1; jt += kThreads) {
        const int64_t j = jt + threadIdx.x;
        if (j < j1) {
            double4_32a p;
            p.x = D.x2[j];
            p.y = D.y2[j];
            p.z = D.z2[j];
            p.w = W ? D.w2[j] : 0.0;
            sj[threadIdx.x] = p;
        }
        __syncthreads();
        const int nt = (int)min((int64_t)kThreads, j1 - jt);
        if (iv) {
            for (int t = 0; t < nt; t++) {
                const double4_32a p = sj[t];
                double ox = 0.0, oy = 0.0, oz = 0.0;
                if (PERIODIC) {
                    const double dx = p.x - xi, dy = p.y - yi, dz = p.z - zi;
                    ox = dx > D.half[0] ? D.box[0] : (dx < -D.half[0] ? -D.box[0] : 0.0);
                    oy = dy > D.half[1] ? D.box[1] : (dy < -D.half[1] ? -D.box[1] : 0.0);
                    oz = dz > D.half[2] ? D.box[2] : (dz < -D.half[2] ? -D.box[2] : 0.0);
                }
                double r = 0.0;
                const int bin = ref_eval<MODE_R3>(A, se, xi, yi, zi, p.x, p.y, p.z, ox, oy, oz, &r);
                if (bin >= 0) {
                    atomicAdd(&hcnt[bin], 1ull);
                    if (RAVG) atomicAdd(&hr[bin], r);
                    if (W) atomicAdd(&hw[bin], wi * p.w);
                }
            }
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < nb; k += kThreads) {
        if (hcnt[k]) {
            atomicAdd((unsigned long long *)&scratch[kMaxEdges + k], hcnt[k]);
            if (RAVG) atomicAdd(&scratch[2 * kMaxEdges + k], hr[k]);
            if (W) atomicAdd(&scratch[3 * kMaxEdges + k], hw[k]);
        }
    }
}

template <bool RAVG, bool W>
cudaError_t launch_direct(bool periodic, dim3 grid, cudaStream_t st, const PairArgs &A, const DirectArgs &D,
                          double *scratch)
{
    if (periodic) k_cross_direct<RAVG, W, true><<<grid, kThreads, 0, st>>>(A, D, scratch);
    else k_cross_direct<RAVG, W, false><<<grid, kThreads, 0, st>>>(A, D, scratch);
    return cudaGetLastError();
}

pthread_mutex_t g_setup_lock = PTHREAD_MUTEX_INITIALIZER;
double *g_scratch_ptr[kMaxDevices];
int g_num_sms[kMaxDevices];

#define NA_FAIL(...)                                                                            \
    do {                                                                                        \
        fprintf(stderr, "corrfunc_gb300: cf_gpu_countpairs_cross_noalloc: " __VA_ARGS__);      \
        fprintf(stderr, "\n");                                                                  \
        return EXIT_FAILURE;                                                                    \
    } while (0)

#define NA_CUDA(call)                                                                           \
    do {                                                                                        \
        const cudaError_t e_ = (call);                                                          \
        if (e_ != cudaSuccess) NA_FAIL("CUDA error '%s' (%s)", cudaGetErrorString(e_), #call);  \
    } while (0)

// Set-up, once per device, with that device current: the device address of the scratch array.
int scratch_for_device(int dev, double **ptr, int *sms)
{
    if (dev < 0 || dev >= kMaxDevices) NA_FAIL("device ordinal %d is beyond the %d supported", dev, kMaxDevices);
    pthread_mutex_lock(&g_setup_lock);
    if (g_scratch_ptr[dev] == NULL) {
        void *p = NULL;
        const cudaError_t rc = cudaGetSymbolAddress((void **)&p, g_noalloc_scratch);
        int n = 0;
        const cudaError_t rc2 =
            rc == cudaSuccess ? cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) : rc;
        if (rc != cudaSuccess || rc2 != cudaSuccess || p == NULL) {
            pthread_mutex_unlock(&g_setup_lock);
            NA_FAIL("cannot find the scratch array on device %d: %s", dev,
                    cudaGetErrorString(rc != cudaSuccess ? rc : rc2));
        }
        g_num_sms[dev] = n > 0 ? n : 1;
        g_scratch_ptr[dev] = (double *)p;
    }
    *ptr = g_scratch_ptr[dev];
    *sms = g_num_sms[dev];
    pthread_mutex_unlock(&g_setup_lock);
    return EXIT_SUCCESS;
}

}  // namespace

extern "C" int cf_gpu_countpairs_cross_noalloc(const int64_t ND1, const double *X1, const double *Y1, const double *Z1,
                                               const double *W1, const int64_t ND2, const double *X2,
                                               const double *Y2, const double *Z2, const double *W2, const int nedges,
                                               const double *edges, const int periodic, const double boxsize_x,
                                               const double boxsize_y, const double boxsize_z,
                                               const int instruction_set, uint64_t *npairs, double *ravg,
                                               double *weightavg, void *stream)
{
    // ---- argument checks (before any CUDA call) ----
    if (nedges < 2 || nedges > kMaxEdges)
        NA_FAIL("nedges = %d is outside [2, %d]: this entry point keeps its histogram in a fixed %d-edge scratch "
                "array; use countpairs() for more bins",
                nedges, kMaxEdges, kMaxEdges);
    if (edges == NULL || npairs == NULL) NA_FAIL("edges and npairs must not be NULL");
    if (ND1 < 0 || ND2 < 0 || ND1 >= ((int64_t)1 << 31) || ND2 >= ((int64_t)1 << 31))
        NA_FAIL("ND1 = %lld and ND2 = %lld must lie in [0, 2^31)", (long long)ND1, (long long)ND2);
    if ((ND1 > 0 && (!X1 || !Y1 || !Z1)) || (ND2 > 0 && (!X2 || !Y2 || !Z2)))
        NA_FAIL("NULL coordinate array");
    if ((W1 == NULL) != (W2 == NULL)) NA_FAIL("give weights for both sets or for neither");
    for (int k = 0; k < nedges; k++) {
        if (!(edges[k] >= 0.0) || !isfinite(edges[k])) NA_FAIL("bin edge %d = %g is not a finite value >= 0", k, edges[k]);
        if (k > 0 && !(edges[k] > edges[k - 1])) NA_FAIL("bin edges must increase (edge %d = %g)", k, edges[k]);
    }
    const double rmax = edges[nedges - 1];
    const double box[3] = {boxsize_x, boxsize_y, boxsize_z};
    if (periodic) {
        // every axis wraps: the reference's per-axis "no wrap" value (-1) is not supported here
        for (int a = 0; a < 3; a++) {
            if (!(box[a] > 0.0) || !isfinite(box[a]))
                NA_FAIL("periodic wrapping needs a positive, finite box size on every axis (axis %d: %g)", a, box[a]);
            if (!(rmax < 0.49 * box[a]))
                NA_FAIL("rmax = %g must stay below 0.49 times the box size (%g) along every axis", rmax, box[a]);
        }
    }

    // ---- set-up (first call on a device) ----
    int dev = 0;
    NA_CUDA(cudaGetDevice(&dev));
    double *scratch = NULL;
    int sms = 1;
    if (scratch_for_device(dev, &scratch, &sms) != EXIT_SUCCESS) return EXIT_FAILURE;
    cudaStream_t st = (cudaStream_t)stream;

    // ---- squared edges in, accumulators zeroed: one copy from this stack buffer ----
    double hbuf[kScratchDoubles];
    memset(hbuf, 0, sizeof(hbuf));
    for (int k = 0; k < nedges; k++) hbuf[k] = edges[k] * edges[k];
    NA_CUDA(cudaMemcpyAsync(scratch, hbuf, sizeof(hbuf), cudaMemcpyHostToDevice, st));

    if (ND1 > 0 && ND2 > 0) {
        PairArgs A;
        memset(&A, 0, sizeof(A));
        A.nedges = nedges;
        int chord = 0;
        cf_formula_for_isa(instruction_set, &A.fma_formula, &chord);
        DirectArgs D;
        memset(&D, 0, sizeof(D));
        D.x1 = X1; D.y1 = Y1; D.z1 = Z1; D.w1 = W1;
        D.x2 = X2; D.y2 = Y2; D.z2 = Z2; D.w2 = W2;
        D.n1 = ND1;
        D.n2 = ND2;
        for (int a = 0; a < 3; a++) {
            D.box[a] = box[a];
            D.half[a] = 0.5 * box[a];
        }
        const int64_t gx = (ND1 + kThreads - 1) / kThreads;
        const int64_t jt = (ND2 + kThreads - 1) / kThreads;  // j tiles
        int64_t gy = (4 * (int64_t)sms + gx - 1) / gx;         // about four blocks per SM
        if (gy > jt) gy = jt;
        if (gy > 65535) gy = 65535;
        if (gy < 1) gy = 1;
        D.j_per_block = (jt + gy - 1) / gy * kThreads;
        gy = (ND2 + D.j_per_block - 1) / D.j_per_block;
        if (gx > 0x7fffffff) NA_FAIL("too many points in set 1");
        const dim3 grid((unsigned)gx, (unsigned)gy);
        const bool want_r = ravg != NULL, want_w = W1 != NULL && weightavg != NULL;
        cudaError_t rc;
        if (want_r && want_w) rc = launch_direct<true, true>(periodic != 0, grid, st, A, D, scratch);
        else if (want_r) rc = launch_direct<true, false>(periodic != 0, grid, st, A, D, scratch);
        else if (want_w) rc = launch_direct<false, true>(periodic != 0, grid, st, A, D, scratch);
        else rc = launch_direct<false, false>(periodic != 0, grid, st, A, D, scratch);
        NA_CUDA(rc);
    }

    // ---- raw sums back into the stack buffer, then the reference's normalisation ----
    NA_CUDA(cudaMemcpyAsync(hbuf, scratch, sizeof(hbuf), cudaMemcpyDeviceToHost, st));
    NA_CUDA(cudaStreamSynchronize(st));
    const uint64_t *cnt = (const uint64_t *)(hbuf + kMaxEdges);
    for (int k = 0; k < nedges; k++) {
        npairs[k] = cnt[k];
        if (ravg) ravg[k] = cnt[k] > 0 ? hbuf[2 * kMaxEdges + k] / (double)cnt[k] : 0.0;
        if (weightavg) weightavg[k] = (W1 && cnt[k] > 0) ? hbuf[3 * kMaxEdges + k] / (double)cnt[k] : 0.0;
    }
    return EXIT_SUCCESS;
}
