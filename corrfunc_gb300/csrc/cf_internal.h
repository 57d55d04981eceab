/*
 * cf_internal.h -- interface between the C host layer (cf_api.c, cf_common.c) and the
 * CUDA engine (cf_engine.cu).  Plain C types only.
 */
#pragma once
#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pair-separation kinds.  Each one is a family of reference kernels. */
enum {
    CF_MODE_R3 = 0,    /* 3-D r^2 bins: countpairs (DD) and countpairs_xi */
    CF_MODE_RPPI = 1,  /* rp^2 bins x linear |pi| bins: countpairs_rp_pi */
    CF_MODE_WP = 2,    /* rp^2 bins with |pi| < pimax: countpairs_wp */
    CF_MODE_SMU = 3,   /* s^2 bins x linear mu bins: countpairs_s_mu */
    CF_MODE_THETA = 4, /* angular bins on unit vectors: countpairs_theta_mocks */
    CF_MODE_RPPI_MOCK = 5, /* rp^2 x pi bins about each pair's line of sight: countpairs_mocks */
    CF_MODE_SMU_MOCK = 6   /* s^2 x mu bins about each pair's line of sight: countpairs_mocks_s_mu */
};

#define CF_MAX_EDGES 512

#ifndef CF_PRECISION_FP32_REFINE
#define CF_PRECISION_FP32_REFINE 0
#define CF_PRECISION_FP64 1
#endif

/* How the reference builds its lattice for one call; resolved against the data extent by
 * cf_resolve_geometry() once the engine has measured it.  The resolved lattice fixes which
 * point of a wrapped auto-correlation pair the reference shifts, and (for xi / wp, whose
 * lattice is the fixed box) which points it rejects as out of bounds. */
enum { CF_REF_NONE = 0, CF_REF_EXTENT = 1, CF_REF_BOX = 2 };
enum { CF_DFL_PER_AXIS = 0, CF_DFL_XI = 1, CF_DFL_WP = 2, CF_DFL_NONE = 3 };
enum { CF_BOOST_XY = 0, CF_BOOST_NONE = 1 };

typedef struct {
    int kind;            /* CF_REF_* */
    int periodic;        /* options->periodic */
    double boxsize[3];   /* options->boxsize_x/_y/_z with y/z defaulted to x (or the box for xi/wp) */
    double max_size[3];  /* cell size limit per axis handed to gridlink (rmax, rmax, pimax ...) */
    int refine[3];       /* options->bin_refine_factors at call time */
    int custom_refine;   /* binning scheme is BINNING_CUST */
    int max_cells;       /* options->max_cells_per_dim */
    int dfl_kind;        /* CF_DFL_* */
    int boost_kind;      /* CF_BOOST_* */
    int64_t np1;         /* ND1, for the boost heuristic */
} cf_refrule;

typedef struct {
    int periodic[3];
    double wrap[3];
    double ref_min[3];
    double ref_inv[3];
    int ref_nmesh[3];
    int refine_used[3];
} cf_geometry;

/* Restates the wrap / refine / gridlink-size logic of the reference drivers
 * (theory/DD/countpairs_impl.c.src:231-332, theory/xi/countpairs_xi_impl.c.src:211-262,
 * theory/wp/countpairs_wp_impl.c.src:236-290, utils/gridlink_utils.c.src:31-49).
 * lo/hi: data extent (both sets).  Returns EXIT_FAILURE (message on stderr) where the
 * reference would fail. */
int cf_resolve_geometry(const cf_refrule *rule, const double lo[3], const double hi[3], cf_geometry *out);

/* The rule of a call whose reference lattice spans the data extent (cf_common.c); options is a
 * struct config_options (corrfunc_gb300.h). */
struct config_options;
void cf_fill_rule_extent(cf_refrule *R, const struct config_options *options, double sx, double sy, double sz,
                         int dfl_kind, int boost_kind, int64_t np1);

typedef struct {
    int mode;
    int autocorr;
    int precision;       /* CF_PRECISION_FP32_REFINE or CF_PRECISION_FP64 */
    int fma_formula;     /* evaluate the double-precision formula of the reference's AVX512F kernels */
    int chord_formula;   /* theta: cos = 1 - chord^2/2 (SIMD kernels) instead of the dot product */
    int elem_size;       /* 4 or 8: element type of the position / weight arrays */
    int inputs_on_device; /* x/y/z/w are device pointers on the current device (no host copy) */

    int64_t n1, n2;
    const void *x1, *y1, *z1, *w1;  /* host arrays (w1 may be NULL) */
    const void *x2, *y2, *z2, *w2;  /* ignored when autocorr */

    cf_refrule rule;     /* resolved by the engine once the extent is known */
    cf_geometry geom;    /* output: the resolved geometry (filled by cf_engine_run) */

    /* separation limits that bound the neighbour search */
    double rmax_xy;      /* max separation in the (x,y) plane (3-D: rmax; rp-pi: rpmax; theta: chord) */
    double rmax_z;       /* max |dz| (3-D: rmax; rp-pi: pimax; s-mu: min(smax, smax*mu_max)) */
    double rmax_3d;      /* spherical limit, or 0 when the mode has none (rp-pi / wp) */

    int nedges;          /* number of bin edges incl. the junk-bin lower edge */
    double edges[CF_MAX_EDGES]; /* squared separations (R3/RPPI/WP/SMU) or cos(theta) (THETA) */
    double pimax;        /* RPPI / WP */
    int npibin;          /* RPPI: pi bins; SMU: mu bins */
    double mu_max;       /* SMU */

    int need_avg;
    int need_weight;

    /* per-task timings (the GPU's analogue of the reference's per cell-pair timer): when set,
     * the engine returns a malloc'd array of ntask_times records in task_times (caller frees) */
    int task_timer;
    struct cf_task_time *task_times;
    int64_t ntask_times;
} cf_job;

/* One work-list task's timing: the i-chunk size and the j-range length, the warp's elapsed time
 * on it, the first sorted point of each, and the global warp that ran it (the layout of the
 * reference's struct api_cell_timings). */
typedef struct cf_task_time {
    int64_t n1, n2, time_in_ns;
    int i_first, j_first, warp;
} cf_task_time;

typedef struct {
    int nbins;           /* total flat bins: nedges, or nedges*(npibin+1) for 2-D modes */
    uint64_t *npairs;    /* caller-allocated, nbins entries each */
    double *avg;         /* sum of separations (r, rp, s, or theta in degrees) */
    double *wsum;        /* sum of w1*w2 */
} cf_hist;

int cf_engine_run(cf_job *job, cf_hist *out);

/* Batched DD cross-correlations: nbatch set-1 catalogues (device arrays) against the set-2
 * catalogue of tmpl, planned once (extent, lattices, work list, optional layout tuning, CUDA
 * graph capture) and replayed by cf_engine_batch_run into out[0..nbatch-1] (raw sums). */
typedef struct cf_batch cf_batch;
int cf_engine_batch_plan(const cf_job *tmpl, int nbatch, const int64_t *n1, const void *const *x1,
                         const void *const *y1, const void *const *z1, const void *const *w1, int tune,
                         cf_batch **out);
int cf_engine_batch_run(cf_batch *plan, cf_hist *out);
void cf_engine_batch_free(cf_batch *plan);
/* Counts in spheres (vpf).  Points (double, host) are binned into the reference lattice
 * (cell = (int)((x - lat_min) * lat_inv), clamped down at the top, as gridlink assigns them);
 * every centre walks the neighbour cells c + d, |d_a| <= refine[a], of its given cell: periodic
 * lattices wrap the index and shift the centre by -/+ wrap, others skip cells outside.  Shell
 * counts of (int)(sqrt(r^2) / rstep) for r^2 < rmax^2, cumulated over shells, fill
 * pN[bin * num_pN + N] (counts of centres with exactly N points within (bin + 1) * rstep). */
typedef struct {
    int64_t np;
    const double *x, *y, *z;
    int nmesh[3];
    double lat_min[3];
    double lat_inv[3];
    int refine[3];
    int periodic;
    double wrap[3];
    int64_t ncen;
    const double *cen;    /* 3 * ncen: x, y, z */
    const int *cen_cell;  /* 3 * ncen: cell index per axis */
    double rmax;
    int nbin;
    int num_pN;
    /* when set: instead of pN, the number of points with r^2 < rmax^2 around every centre
     * (the neighbour count of count_neighbors, mocks/vpf_mocks/countspheres_mocks_impl.c.src:140-206) */
    uint32_t *counts_out;
} cf_vpf_job;
int cf_engine_vpf(const cf_vpf_job *J, uint64_t *pN);

int cf_engine_set_precision(int mode);
int cf_engine_set_autotune(int on);
int cf_engine_get_autotune(void);
int cf_engine_get_precision(void);

typedef struct {
    double pair_kernel_ms;
    double gridlink_ms;
    double total_gpu_ms;
    uint64_t pairs_evaluated;
    uint64_t pairs_refined;
    uint64_t tasks;
    int kernel_launches;
    int num_cells;
    int blocks_per_sm;
    int warps_per_block;
    int lane_stride;
    int column_split;
    uint64_t pairs_slow;
} cf_engine_stats;
int cf_engine_last_stats(cf_engine_stats *out);
int cf_engine_fp32_peak(double *tflops);
int cf_engine_copy_to_host(void *dst, const void *src, size_t bytes);
/* new device buffer holding a copy of bytes of host memory; and its release */
int cf_engine_to_device(const void *src, size_t bytes, void **dev);
void cf_engine_free_device(void *dev);

#ifdef __cplusplus
}
#endif
