/*
 * corrfunc_gb300.h -- C ABI of the GB300 pair-counting library (libcorrfunc_gb300.so).
 *
 * Every entry point below is a drop-in for the Corrfunc 2.5.3 public C function of the
 * same name: same prototype, same option/extra/result struct layouts (byte for byte), same
 * bin-file format, same return convention (EXIT_SUCCESS / EXIT_FAILURE with a message on
 * stderr), same ownership rules (positions and weights belong to the caller; result arrays
 * are malloc'ed by the library and released by the matching free_results_* call).
 *
 * The counting itself runs on one CUDA GPU.  There is no CPU fallback: when no usable GPU
 * is present the entry points fail with EXIT_FAILURE.
 *
 * Struct layouts follow utils/defs.h:53-156 (config_options, 1024 bytes),
 * utils/defs.h:357-419 (weight_struct / extra_options, 1024 bytes) and the per-module
 * result structs cited beside each declaration.  The layouts are checked by
 * CF_STATIC_ASSERT below and by the test suite against the reference headers.
 */
#pragma once

#include <stdint.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The reference stringifies the quoted VERSION macro (utils/defs.h:25, common.mk:175), so the
 * version field of config_options holds the seven characters "2.5.3" including the quotes. */
#define CF_API_VERSION "\"2.5.3\""

#if defined(__cplusplus)
#define CF_STATIC_ASSERT(c, m) static_assert(c, #m)
#else
#define CF_STATIC_ASSERT(c, m) _Static_assert(c, #m)
#endif

/* ---------------- instruction-set tags (utils/cpu_features.h:20-34) ----------------
 * The GPU library has one code path.  The tag is kept only because it selects which
 * double-precision formula the reference evaluates (fused multiply-add chain on AVX512F,
 * unfused sums elsewhere), and the GPU reproduces the formula the caller's reference run
 * would have used so that pair counts stay identical. */
typedef enum {
    DEFAULT = -42,
    FALLBACK = 0,
    SSE = 1, SSE2 = 2, SSE3 = 3, SSSE3 = 4, SSE4 = 5, SSE42 = 6,
    AVX = 7, AVX2 = 8, AVX512F = 9, ARM64 = 10,
    NUM_ISA
} isa;

#define BINNING_REF_MASK 0x0000000F
#define BINNING_ORD_MASK 0x000000F0
#define BINNING_DFL 0x0
#define BINNING_CUST 0x1

#define NLATMAX 100
#define OPTIONS_HEADER_SIZE 1024
#define EXTRA_OPTIONS_HEADER_SIZE 1024
#define MAX_NUM_WEIGHTS 10
#define BOXSIZE_NOTGIVEN (-2.)

/* Per cell-pair timing record (utils/defs.h:37-45). */
struct api_cell_timings {
    int64_t N1;
    int64_t N2;
    int64_t time_in_ns;
    int first_cellindex;
    int second_cellindex;
    int tid;
};

/* Runtime options, identical layout to utils/defs.h:53-156. */
struct config_options {
    union {
        double boxsize;
        double boxsize_x;
    };
    double boxsize_y;
    double boxsize_z;
    struct {
        double OMEGA_M;
        double OMEGA_B;
        double OMEGA_L;
        double HUBBLE;
        double LITTLE_H;
        double SIGMA_8;
        double NS;
    };
    double c_api_time;
    struct api_cell_timings *cell_timings;
    int64_t totncells_timings;
    size_t float_type;
    int32_t instruction_set;
    char version[32];
    uint8_t verbose;
    uint8_t c_api_timer;
    uint8_t c_cell_timer;
    uint8_t need_avg_sep;
    uint8_t autocorr;
    uint8_t periodic;
    uint8_t sort_on_z;
    uint8_t is_comoving_dist;
    uint8_t link_in_dec;
    uint8_t link_in_ra;
    uint8_t fast_divide_and_NR_steps;
    uint8_t fast_acos;
    uint8_t enable_min_sep_opt;
    int8_t bin_refine_factors[3];
    uint16_t max_cells_per_dim;
    uint8_t copy_particles;
    uint8_t use_heap_sort;
    union {
        uint32_t binning_flags;
        uint8_t bin_masks[4];
    };
    uint8_t reserved[OPTIONS_HEADER_SIZE - 33 * sizeof(char) - sizeof(size_t) - 11 * sizeof(double) -
                     3 * sizeof(int) - sizeof(uint16_t) - 16 * sizeof(uint8_t) -
                     sizeof(struct api_cell_timings *) - sizeof(int64_t)];
};
CF_STATIC_ASSERT(sizeof(struct config_options) == OPTIONS_HEADER_SIZE, config_options_must_be_1024_bytes);

/* Weight arrays (utils/defs.h:357-361): weights[w] points at num_particles values. */
typedef struct {
    void *weights[MAX_NUM_WEIGHTS];
    int64_t num_weights;
} weight_struct;

/* Pair-weighting methods (utils/defs.h:363-367).  PAIR_PRODUCT = w_i * w_j. */
typedef enum {
    NONE = -42,
    PAIR_PRODUCT = 0,
    NUM_WEIGHT_TYPE
} weight_method_t;

/* Extra options (utils/defs.h:395-402). */
struct extra_options {
    weight_struct weights0;
    weight_struct weights1;
    weight_method_t weight_method;
    uint8_t reserved[EXTRA_OPTIONS_HEADER_SIZE - 2 * sizeof(weight_struct) - sizeof(weight_method_t)];
};
CF_STATIC_ASSERT(sizeof(struct extra_options) == EXTRA_OPTIONS_HEADER_SIZE, extra_options_must_be_1024_bytes);

/* ---------------- result structs ---------------- */

/* theory/DD/countpairs.h:20-26 */
typedef struct {
    uint64_t *npairs;
    double *rupp;
    double *rpavg;
    double *weightavg;
    int nbin;
} results_countpairs;

/* theory/DDrppi/countpairs_rp_pi.h: 2-D layout npairs[i*(npibin+1) + j] */
typedef struct {
    uint64_t *npairs;
    double *rupp;
    double *rpavg;
    double *weightavg;
    double pimax;
    int nbin;
    int npibin;
} results_countpairs_rp_pi;

/* theory/DDsmu/countpairs_s_mu.h: 2-D layout npairs[i*(nmu_bins+1) + j] */
typedef struct {
    uint64_t *npairs;
    double *supp;
    double *savg;
    double mu_max;
    double mu_min;
    double *weightavg;
    int nsbin;
    int nmu_bins;
} results_countpairs_s_mu;

/* theory/wp/countpairs_wp.h */
typedef struct {
    uint64_t *npairs;
    double *wp;
    double *rupp;
    double *rpavg;
    double *weightavg;
    double pimax;
    int nbin;
} results_countpairs_wp;

/* theory/xi/countpairs_xi.h */
typedef struct {
    uint64_t *npairs;
    double *xi;
    double *rupp;
    double *ravg;
    double *weightavg;
    int nbin;
} results_countpairs_xi;

/* mocks/DDtheta_mocks/countpairs_theta_mocks.h */
typedef struct {
    uint64_t *npairs;
    double *theta_upp;
    double *theta_avg;
    double *weightavg;
    int nbin;
} results_countpairs_theta;

/* mocks/DDrppi_mocks/countpairs_rp_pi_mocks.h:19-27: 2-D layout npairs[i*(npibin+1) + j] */
typedef struct {
    uint64_t *npairs;
    double *rupp;
    double *rpavg;
    double *weightavg;
    double pimax;
    int nbin;
    int npibin;
} results_countpairs_mocks;

/* mocks/DDsmu_mocks/countpairs_s_mu_mocks.h:19-28: 2-D layout npairs[i*(nmu_bins+1) + j] */
typedef struct {
    uint64_t *npairs;
    double *supp;
    double *savg;
    double mu_max;
    double mu_min;
    double *weightavg;
    int nsbin;
    int nmu_bins;
} results_countpairs_mocks_s_mu;

/* theory/vpf/countspheres.h:20-26: pN[bin][N], bin = sphere radius (bin + 1) * rmax / nbin */
typedef struct {
    double **pN;
    double rmax;
    int nbin;
    int nc;
    int num_pN;
} results_countspheres;

/* mocks/vpf_mocks/countspheres_mocks.h:20-26 */
typedef struct {
    double **pN;
    double rmax;
    int nbin;
    int nc;
    int num_pN;
} results_countspheres_mocks;

/* ---------------- entry points ---------------- */

/* Replaces countpairs(), theory/DD/countpairs.h:28-35 (3-D DD(r) counts). */
int countpairs(const int64_t ND1, void *X1, void *Y1, void *Z1,
               const int64_t ND2, void *X2, void *Y2, void *Z2,
               const int numthreads, const int autocorr, const char *binfile,
               results_countpairs *results, struct config_options *options,
               struct extra_options *extra);
/* Replaces free_results(), theory/DD/countpairs.h:37. */
void free_results(results_countpairs *results);

/* Replaces countpairs_rp_pi(), theory/DDrppi/countpairs_rp_pi.h (DD(rp, pi) counts). */
int countpairs_rp_pi(const int64_t ND1, void *X1, void *Y1, void *Z1,
                     const int64_t ND2, void *X2, void *Y2, void *Z2,
                     const int numthreads, const int autocorr, const char *binfile,
                     const double pimax, results_countpairs_rp_pi *results,
                     struct config_options *options, struct extra_options *extra);
/* Replaces free_results_rp_pi(), theory/DDrppi/countpairs_rp_pi.h. */
void free_results_rp_pi(results_countpairs_rp_pi *results);

/* Replaces countpairs_s_mu(), theory/DDsmu/countpairs_s_mu.h (DD(s, mu) counts). */
int countpairs_s_mu(const int64_t ND1, void *X1, void *Y1, void *Z1,
                    const int64_t ND2, void *X2, void *Y2, void *Z2,
                    const int numthreads, const int autocorr, const char *sbinfile,
                    const double mu_max, const int nmu_bins, results_countpairs_s_mu *results,
                    struct config_options *options, struct extra_options *extra);
/* Replaces free_results_s_mu(), theory/DDsmu/countpairs_s_mu.h. */
void free_results_s_mu(results_countpairs_s_mu *results);

/* Replaces countpairs_wp(), theory/wp/countpairs_wp.h (projected w_p(rp), periodic auto). */
int countpairs_wp(const int64_t ND1, void *X1, void *Y1, void *Z1, const double boxsize,
                  const int numthreads, const char *binfile, const double pimax,
                  results_countpairs_wp *result, struct config_options *options,
                  struct extra_options *extra);
/* Replaces free_results_wp(), theory/wp/countpairs_wp.h. */
void free_results_wp(results_countpairs_wp *results);

/* Replaces countpairs_xi(), theory/xi/countpairs_xi.h (xi(r), periodic auto). */
int countpairs_xi(const int64_t ND1, void *X1, void *Y1, void *Z1, const double boxsize,
                  const int numthreads, const char *binfile, results_countpairs_xi *results,
                  struct config_options *options, struct extra_options *extra);
/* Replaces free_results_xi(), theory/xi/countpairs_xi.h. */
void free_results_xi(results_countpairs_xi *results);

/* Replaces countpairs_theta_mocks(), mocks/DDtheta_mocks/countpairs_theta_mocks.h
 * (angular DD(theta) on the sky, RA = phi, DEC = theta, in degrees). */
int countpairs_theta_mocks(const int64_t ND1, void *phi1, void *theta1,
                           const int64_t ND2, void *phi2, void *theta2,
                           const int numthreads, const int autocorr, const char *binfile,
                           results_countpairs_theta *results, struct config_options *options,
                           struct extra_options *extra);
/* Replaces free_results_countpairs_theta(), mocks/DDtheta_mocks/countpairs_theta_mocks.h. */
void free_results_countpairs_theta(results_countpairs_theta *results);

/* Replaces countpairs_mocks(), mocks/DDrppi_mocks/countpairs_rp_pi_mocks.h:29-37: DD(rp, pi) of
 * a survey catalogue (RA, DEC in degrees; cz in km/s, or the comoving distance in Mpc/h when
 * options->is_comoving_dist is set), rp and pi about each pair's line of sight, cosmology 1
 * (LasDamas) or 2 (Planck) for cz -> distance.  RA/DEC/cz are fixed up in place exactly where
 * the reference fixes them (RA in [-180, 180], DEC in [0, 180], redshifts instead of cz). */
int countpairs_mocks(const int64_t ND1, void *theta1, void *phi1, void *czD1,
                     const int64_t ND2, void *theta2, void *phi2, void *czD2,
                     const int numthreads, const int autocorr, const char *binfile, const double pimax,
                     const int cosmology, results_countpairs_mocks *results, struct config_options *options,
                     struct extra_options *extra);
/* Replaces free_results_mocks(), mocks/DDrppi_mocks/countpairs_rp_pi_mocks.h:39. */
void free_results_mocks(results_countpairs_mocks *results);

/* Replaces countpairs_mocks_s_mu(), mocks/DDsmu_mocks/countpairs_s_mu_mocks.h:30-40: DD(s, mu) of
 * a survey catalogue, mu the cosine of the angle between s and the pair's line of sight. */
int countpairs_mocks_s_mu(const int64_t ND1, void *theta1, void *phi1, void *czD1,
                          const int64_t ND2, void *theta2, void *phi2, void *czD2,
                          const int numthreads, const int autocorr, const char *sbinfile, const double mu_max,
                          const int nmu_bins, const int cosmology, results_countpairs_mocks_s_mu *results,
                          struct config_options *options, struct extra_options *extra);
/* Replaces free_results_mocks_s_mu(), mocks/DDsmu_mocks/countpairs_s_mu_mocks.h:42. */
void free_results_mocks_s_mu(results_countpairs_mocks_s_mu *results);

/* Replaces countspheres(), theory/vpf/countspheres.h:29-35: counts in spheres (void probability
 * function and pN) of a 3-D point set; nc centres drawn from MT19937(seed) as the reference draws
 * them from GSL's mt19937, counts on the GPU. */
int countspheres(const int64_t np, void *X, void *Y, void *Z, const double rmax, const int nbin, const int nc,
                 const int num_pN, unsigned long seed, results_countspheres *results,
                 struct config_options *options, struct extra_options *extra);
/* Replaces free_results_countspheres(), theory/vpf/countspheres.h:37. */
void free_results_countspheres(results_countspheres *results);

/* Replaces countspheres_mocks(), mocks/vpf_mocks/countspheres_mocks.h:28-36: counts in spheres of a
 * survey catalogue, centres read from centers_file or drawn from the randoms (and then written to
 * centers_file), as the reference does. */
int countspheres_mocks(const int64_t Ngal, void *xgal, void *ygal, void *zgal,
                       const int64_t Nran, void *xran, void *yran, void *zran,
                       const int threshold_neighbors, const double rmax, const int nbin, const int nc,
                       const int num_pN, const char *centers_file, const int cosmology,
                       results_countspheres_mocks *results, struct config_options *options,
                       struct extra_options *extra);
/* Replaces free_results_countspheres_mocks(), mocks/vpf_mocks/countspheres_mocks.h:38. */
void free_results_countspheres_mocks(results_countspheres_mocks *results);

/* ---------------- particle-file readers (io/io.h:15-16) ----------------
 * Replace read_positions() / read_columns_into_array(), io/io.c:29-284: fast-food ("f"),
 * ASCII ("a") or CSV ("c") files; num_fields arrays of size 4 or 8 bytes per value, malloc'ed
 * (the caller frees them); returns the number of particles or -1. */
int64_t read_positions(const char *filename, const char *format, const size_t size, const int num_fields, ...);
int64_t read_columns_into_array(const char *filename, const char *format, const size_t size, const int num_fields,
                                void **data);

/* ---------------- GB300 extensions (no reference counterpart) ----------------
 * Counting precision of the GPU engine.  CF_PRECISION_FP32_REFINE (default) classifies
 * every pair in FP32 and re-evaluates in FP64, with the reference's formula, the pairs
 * whose FP32 value lies within a proven error bound of a bin edge; CF_PRECISION_FP64
 * evaluates every pair in FP64.  Both give identical npairs. */
#define CF_PRECISION_FP32_REFINE 0
#define CF_PRECISION_FP64 1
int cf_gpu_set_precision(int mode);
int cf_gpu_get_precision(void);

/* Single-count autotuner (off by default; the GPU's counterpart of the reference's
 * find_fastest_wp_bin_refs, Corrfunc/theory/wp.py:17): with it on, the first DD(r) / xi count of
 * each shape (sizes, mode, options, box, radii, bin edges) in this process runs with each split of
 * the j lattice's columns (1-4) twice and keeps the split with the shortest device time for the
 * later counts of that shape (up to 32 shapes); counts are identical for every split.  Turning it
 * off forgets the shapes.  No reference counterpart in the C API. */
int cf_gpu_set_autotune(int on);
int cf_gpu_get_autotune(void);

/* Kernel statistics of the last call on this thread (for benchmarking): pair-kernel time
 * measured with CUDA events, lattice-build time, and the number of evaluated / refined pairs. */
typedef struct {
    double pair_kernel_ms;
    double gridlink_ms;  /* single counts: the lattice build proper (cell index, offsets, scatter) */
    double total_gpu_ms; /* the whole count on the device, extent read-back and work list included */
    uint64_t pairs_evaluated;
    uint64_t pairs_refined;
    uint64_t tasks;
    int kernel_launches;
    int num_cells;
    int blocks_per_sm;   /* launch shape of the last pair kernel */
    int warps_per_block;
    int lane_stride;     /* lanes l and l + lane_stride share one histogram column (32 = private) */
    int column_split;    /* j-lattice columns per lattice column and axis (1: unsplit) */
    uint64_t pairs_slow; /* pairs in flagged table buckets (exact FP32 classification) */
} cf_gpu_stats;
int cf_gpu_last_stats(cf_gpu_stats *out);

/* countpairs() with X1..Z2 and the weight arrays of `extra` already resident on the current CUDA
 * device (device pointers); nothing is copied host to device.  No reference counterpart: it lets
 * a caller that keeps catalogues in GPU memory skip the upload. */
int cf_gpu_countpairs_device(const int64_t ND1, void *X1, void *Y1, void *Z1,
                             const int64_t ND2, void *X2, void *Y2, void *Z2,
                             const int numthreads, const int autocorr, const char *binfile,
                             results_countpairs *results, struct config_options *options,
                             struct extra_options *extra);

/* Batched DD(r) cross-correlations: nbatch set-1 catalogues, each against the same set-2
 * catalogue, with the same bins and options.  No reference counterpart: it replaces nbatch
 * countpairs(..., autocorr = 0, ...) calls (jackknife / bootstrap subsamples against one random
 * catalogue) and gives results[b] exactly as that call would.
 *
 *   ND1[b], X1[b], Y1[b], Z1[b], W1[b]  catalogue b, device pointers (float or double as
 *          options->float_type); W1 / W2 are read only with weight_method = PAIR_PRODUCT.
 *   X2 .. W2  the set-2 catalogue, device pointers.
 *   autotune  non-zero: time the pair kernel's histogram layouts while planning, keep the fastest.
 *
 * cf_gpu_batch_plan measures the data, builds every lattice and the merged work list once,
 * checks it, and captures the whole count (lattices, work list, one pair-kernel launch for all
 * catalogues, read-back) as a CUDA graph.  cf_gpu_batch_run replays that graph on the arrays the
 * plan was made with -- their contents may change between runs, their sizes may not -- and fills
 * results[0 .. nbatch-1] (release each with free_results).  cf_gpu_batch_free releases the plan. */
typedef struct cf_gpu_batch cf_gpu_batch;
int cf_gpu_batch_plan(const int nbatch, const int64_t *ND1, void *const *X1, void *const *Y1, void *const *Z1,
                      void *const *W1, const int64_t ND2, void *X2, void *Y2, void *Z2, void *W2,
                      const char *binfile, struct config_options *options, const int weight_method,
                      const int autotune, cf_gpu_batch **plan);
int cf_gpu_batch_run(cf_gpu_batch *plan, results_countpairs *results);
void cf_gpu_batch_free(cf_gpu_batch *plan);

/* Measured FP32 fused-multiply-add throughput of the current device in TFLOP/s (a calibration
 * kernel; denominator of the pair kernels' FP32 roofline fraction).  No reference counterpart. */
int cf_gpu_fp32_peak_tflops(double *tflops);

/* Extension (no counterpart in the reference): read_columns_into_array() followed by a copy of
 * every field into a new device buffer (device_fields[i], released with cf_gpu_free_device), for
 * cf_gpu_countpairs_device.  Returns the number of particles or -1. */
int64_t cf_gpu_read_positions_device(const char *filename, const char *format, const size_t size, const int num_fields,
                                     void **device_fields);
void cf_gpu_free_device(void *device_ptr);

/* The algorithmic work unit of countpairs(): the number of candidate pairs the reference's own
 * lattice and cell-pair list (utils/gridlink_impl.c.src:65-625) would evaluate for these
 * arguments.  Host arrays; runs on the CPU.  No reference counterpart. */
int cf_reference_candidate_pairs(const int64_t ND1, void *X1, void *Y1, void *Z1,
                                 const int64_t ND2, void *X2, void *Y2, void *Z2,
                                 const int autocorr, const char *binfile,
                                 struct config_options *options, uint64_t *candidates);

/* DD(r) cross-correlation (autocorr = 0) of two catalogues resident on the current CUDA device,
 * by direct summation over all ND1 * ND2 pairs in double precision, for callers that must not
 * allocate memory inside the call (device memory reserved up front, no cudaMalloc/cudaFree and
 * the synchronisation they may bring, no host heap).  No counterpart in the reference.
 *
 *   X1..W2     device pointers to double arrays; W1 and W2 both NULL (no weights) or both set
 *              (pair_product weights).
 *   edges      host array of the nedges bin edges as a bin file lists them (rmin, then each
 *              upper edge); 2 <= nedges <= 128, larger values are rejected with an error.
 *   periodic   minimum-image wrapping on all three axes with the given box sizes, each of which
 *              must be positive (the reference's per-axis -1, "no wrap on this axis", is rejected
 *              with an error); needs rmax < 0.49 * box size along every axis.
 *   instruction_set  the reference isa whose double-precision formula the counts follow
 *              (AVX512F chains fused multiply-adds, the others do not; < 0 picks this host's).
 *   npairs, ravg, weightavg  caller-provided host arrays of nedges entries (ravg / weightavg
 *              may be NULL); entry k counts edges[k-1] <= r < edges[k], entry 0 stays 0, and
 *              averages are normalised as countpairs() does.
 *   stream     the cudaStream_t to run on (NULL: the default stream); the call returns after
 *              the stream has drained.
 *
 * Scratch is a fixed 4 KB device array inside the library.  The first call on each device looks
 * up its address; the address is kept for the life of the process: after the first call, neither
 * cudaDeviceReset nor another context made current on that device is supported.  No call may be
 * made while its stream is being captured into a CUDA graph: every call copies its edges from a
 * host buffer and synchronises the stream, which a capture does not allow.  Each call
 * writes the squared edges and zeros over the accumulators itself, so nothing has to be cleared
 * beforehand.  All calls on one device share that array: calls that overlap in time (two host
 * threads, or two streams) race and corrupt each other's counts, so serialise them.  Cost grows
 * as ND1 * ND2, so this is meant for small catalogues. */
int cf_gpu_countpairs_cross_noalloc(const int64_t ND1, const double *X1, const double *Y1, const double *Z1,
                                    const double *W1, const int64_t ND2, const double *X2, const double *Y2,
                                    const double *Z2, const double *W2, const int nedges, const double *edges,
                                    const int periodic, const double boxsize_x, const double boxsize_y,
                                    const double boxsize_z, const int instruction_set, uint64_t *npairs,
                                    double *ravg, double *weightavg, void *stream);

/* ---------------- header-only helpers (utils/defs.h:158-346, 369-419) ----------------
 * Callers compile these themselves, exactly as with the reference header. */

static inline void set_bin_refine_scheme(struct config_options *options, const int8_t flag)
{
    options->binning_flags = (options->binning_flags & ~BINNING_REF_MASK) | (flag & BINNING_REF_MASK);
}

static inline void reset_bin_refine_scheme(struct config_options *options)
{
    set_bin_refine_scheme(options, BINNING_DFL);
}

static inline int8_t get_bin_refine_scheme(struct config_options *options)
{
    return (int8_t)(options->binning_flags & BINNING_REF_MASK);
}

static inline void set_bin_refine_factors(struct config_options *options, const int bin_refine_factors[3])
{
    for (int i = 0; i < 3; i++) {
        int8_t f = (int8_t)bin_refine_factors[i];
        if (bin_refine_factors[i] > INT8_MAX) {
            fprintf(stderr, "Warning: bin refine factor[%d] can be at most %d. Found %d instead\n", i,
                    INT8_MAX, bin_refine_factors[i]);
            f = 1;
        }
        options->bin_refine_factors[i] = f;
    }
    reset_bin_refine_scheme(options);
}

static inline void set_custom_bin_refine_factors(struct config_options *options, const int bin_refine_factors[3])
{
    set_bin_refine_factors(options, bin_refine_factors);
    set_bin_refine_scheme(options, BINNING_CUST);
}

static inline void reset_bin_refine_factors(struct config_options *options)
{
    options->bin_refine_factors[0] = 2;
    options->bin_refine_factors[1] = 2;
    options->bin_refine_factors[2] = 1;
    reset_bin_refine_scheme(options);
}

static inline void set_max_cells(struct config_options *options, const int max)
{
    if (max <= 0) {
        fprintf(stderr, "Warning: Max. cells per dimension was requested to be set to a negative number = %d...returning\n", max);
        return;
    }
    if (max > INT16_MAX) {
        fprintf(stderr, "Warning: Max cells per dimension is a 2-byte integer and can not hold supplied value of %d.\n", max);
    }
    options->max_cells_per_dim = (uint16_t)max;
}

static inline void reset_max_cells(struct config_options *options)
{
    options->max_cells_per_dim = NLATMAX;
}

/* Defaults as the reference's get_config_options() built with the theory.options /
 * mocks.options defaults (PERIODIC, ENABLE_MIN_SEP_OPT, COPY_PARTICLES, double precision). */
static inline struct config_options get_config_options(void)
{
    struct config_options options;
    memset(&options, 0, sizeof(options));
    snprintf(options.version, sizeof(options.version) - 1, "%s", CF_API_VERSION);
    options.boxsize_x = BOXSIZE_NOTGIVEN;
    options.boxsize_y = BOXSIZE_NOTGIVEN;
    options.boxsize_z = BOXSIZE_NOTGIVEN;
    options.float_type = sizeof(double);
    options.verbose = 0;
    options.periodic = 1;
    options.instruction_set = -1; /* let the library pick the host's fastest formula */
    options.link_in_dec = 1;
    options.link_in_ra = 1;
    options.enable_min_sep_opt = 1;
    options.copy_particles = 1;
    options.totncells_timings = 0;
    options.cell_timings = NULL;
    reset_max_cells(&options);
    reset_bin_refine_factors(&options);
    return options;
}

/* per cell-pair timer storage (utils/defs.h:438-473): the library fills options->cell_timings
 * (totncells_timings records) when options->c_cell_timer is set; the caller releases it */
static inline void free_cell_timings(struct config_options *options)
{
    if (options->totncells_timings > 0 && options->cell_timings != NULL) free(options->cell_timings);
    options->cell_timings = NULL;
    options->totncells_timings = 0;
}

static inline void allocate_cell_timer(struct config_options *options, const int64_t num_cell_pairs)
{
    if (options->totncells_timings >= num_cell_pairs) return;
    free_cell_timings(options);
    options->cell_timings = (struct api_cell_timings *)calloc((size_t)num_cell_pairs, sizeof(*options->cell_timings));
    if (options->cell_timings == NULL)
        fprintf(stderr, "Warning: In %s> Could not allocate memory to store the API timings per cell.\n", __func__);
    else
        options->totncells_timings = num_cell_pairs;
}

static inline void assign_cell_timer(struct api_cell_timings *cell_timings, const int64_t num_cell_pairs,
                                     struct config_options *options)
{
    allocate_cell_timer(options, num_cell_pairs);
    if (options->totncells_timings >= num_cell_pairs)
        memmove(options->cell_timings, cell_timings, sizeof(struct api_cell_timings) * (size_t)num_cell_pairs);
}

static inline int get_num_weights_by_method(const weight_method_t method)
{
    return method == PAIR_PRODUCT ? 1 : 0;
}

static inline int get_weight_method_by_name(const char *name, weight_method_t *method)
{
    if (name == NULL || strcmp(name, "") == 0) {
        *method = NONE;
        return EXIT_SUCCESS;
    }
    if (strcmp(name, "pair_product") == 0 || strcmp(name, "p") == 0) {
        *method = PAIR_PRODUCT;
        return EXIT_SUCCESS;
    }
    return EXIT_FAILURE;
}

static inline struct extra_options get_extra_options(const weight_method_t weight_method)
{
    struct extra_options extra;
    memset(&extra, 0, sizeof(extra));
    extra.weight_method = weight_method;
    extra.weights0.num_weights = get_num_weights_by_method(weight_method);
    extra.weights1.num_weights = extra.weights0.num_weights;
    return extra;
}

#ifdef __cplusplus
}
#endif
