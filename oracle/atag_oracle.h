/*
 * atag_oracle.h — CPU restatement of the reference AprilTag quad-detection
 * path (carbotaniuman/sycl-apriltag-test).  TEST INFRASTRUCTURE ONLY: the
 * oracle is the parity checker for the CUDA path and the timed CPU baseline;
 * it is never linked into, loaded by or called from the product library.
 *
 * Parity pinning: the kernel stages (threshold, segmentation, boundaries,
 * fit_lines, do_indexing) and the record helpers are checked against golden
 * vectors produced by the reference's own sources (compiled from the
 * reference tree by oracle/refshim, see tests/golden/make_golden.py).  The
 * oneDPL glue between kernels (copy_if, sort_by_key, reduce_by_segment,
 * scans, sorts) is restated from its documented semantics; where the
 * reference's order is unspecified (sort ties) a total order is fixed:
 *   pair sort    : (key, packed point)
 *   theta sort   : (cluster, theta, packed point)
 *   corner sort  : (cluster asc, error desc, point index asc)
 */
#ifndef ATAG_ORACLE_H
#define ATAG_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/atag.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Intermediates and results of one frame. */
typedef struct oracle_result {
    int width, height;             /* after decimation */
    uint8_t *decimated;            /* w*h */
    uint8_t *thresholded;          /* w*h */
    uint32_t *labels;              /* w*h */
    uint32_t *sizes;               /* w*h */
    size_t n_points;               /* P after compaction */
    atag_boundary_point *points;   /* P, sorted by (key, packed) */
    uint64_t *keys;                /* P */
    size_t n_bounds;               /* C */
    atag_cluster_bounds *bounds;   /* C, one per distinct key, key order */
    uint64_t *bound_keys;          /* C */
    size_t n_filtered;             /* C_f */
    atag_cluster_bounds *filtered; /* C_f */
    uint64_t *filtered_keys;       /* C_f */
    atag_cluster_extents *extents; /* C_f */
    size_t n_cluster_points;       /* P_f */
    atag_cluster_point *cluster_points; /* P_f sorted (cluster, theta, packed) */
    uint32_t *cluster_indices;     /* P_f */
    atag_line_fit_point *line_fit; /* P_f per-cluster inclusive prefix sums */
    atag_corner *found_corners;    /* P_f dense (zero where no corner) */
    size_t n_corners;              /* K */
    atag_corner *corners;          /* K sorted (cluster asc, error desc, index asc) */
    size_t n_peak_extents;         /* C_p */
    atag_peak_extents *peak_extents; /* C_p */
    atag_fitted_quad *fitted;      /* C_p */
    size_t n_quads;                /* Q */
    atag_quad_corners *quads;      /* Q */
} oracle_result;

void oracle_config_default(atag_config *cfg);

/* --- record helpers (the reference include/ headers) --- */
float oracle_calc_theta(atag_boundary_point p, float cx, float cy);
float oracle_bounds_cx(const atag_cluster_bounds *b);
float oracle_bounds_cy(const atag_cluster_bounds *b);
float oracle_bounds_dot(const atag_cluster_bounds *b);
atag_cluster_bounds oracle_bounds_from_point(atag_boundary_point p, uint32_t start);
atag_cluster_bounds oracle_reduce_bounds(const atag_cluster_bounds *a, const atag_cluster_bounds *b);
int oracle_valid_blob(const atag_cluster_bounds *b, size_t width, size_t height, const atag_config *cfg);
atag_line_fit_point oracle_initial_linefit(atag_cluster_point p, uint32_t width, uint32_t height,
                                           const uint8_t *grey);
void oracle_get_moment(const atag_line_fit_point *points, size_t points_size, size_t i0, size_t i1,
                       atag_line_fit_point *out, size_t *n_out);
void oracle_fit_line(const atag_line_fit_point *m, size_t num_in_moment, float *line_params,
                     float *err, float *mse);
void oracle_combination_decode(uint32_t num, uint32_t out[4]);
float oracle_hypotf(float a, float b);

/* --- stages --- */
void oracle_decimate(const uint8_t *src, int src_w, int src_h, int factor, uint8_t *dst);
/* Colour removal + decimation: pixel (f x, f y) of a src_w x src_h image of
 * `format` (ATAG_PIX_*, include/atag.h) with rows src_pitch bytes apart (0 =
 * packed), to one grey byte; dst is (src_w / f) x (src_h / f). */
void oracle_to_grey(const uint8_t *src, int src_w, int src_h, int src_pitch, int format, int factor,
                    uint8_t *dst);
void oracle_threshold(const uint8_t *grey, int w, int h, int min_white_black_diff,
                      uint8_t *extrema, uint8_t *filtered, uint8_t *out);
/* scratch may be NULL (then allocated internally); labels/sizes w*h. */
void oracle_segmentation(const uint8_t *thr, int w, int h, uint32_t *scratch, uint32_t *labels,
                         uint32_t *sizes);
/* Dense 4-plane output; points/keys of 4*w*h must be pre-filled 0 / 0xFF. */
void oracle_find_boundaries(const uint32_t *labels, const uint32_t *sizes, int w, int h,
                            int min_component_size, atag_boundary_point *points, uint64_t *keys);
/* Literal restatement of the work-group windowed kernel (fit_quad.cpp:153-375). */
void oracle_fit_lines_windowed(const atag_line_fit_point *points, const uint32_t *cluster_indices,
                               const atag_cluster_extents *extents, size_t points_size,
                               atag_corner *found_corners);
/* Per-cluster cyclic formulation, proven equal to the windowed one. */
void oracle_fit_lines_cyclic(const atag_line_fit_point *points, const uint32_t *cluster_indices,
                             const atag_cluster_extents *extents, size_t n_clusters,
                             atag_corner *found_corners);
void oracle_do_indexing(const atag_peak_extents *extents, size_t extents_count,
                        const atag_corner *corners, const atag_line_fit_point *points,
                        const atag_cluster_extents *cluster_extents, const atag_config *cfg,
                        atag_fitted_quad *fitted);
size_t oracle_process_fitted_quads(const atag_fitted_quad *fitted, size_t n, const atag_config *cfg,
                                   atag_quad_corners *out);

/* Whole path on one source frame. Returns 0 on success. */
int oracle_detect(const uint8_t *src, int src_w, int src_h, const atag_config *cfg,
                  oracle_result *res);
void oracle_free(oracle_result *res);

/* Batch evaluation of the record helpers (golden-vector checks). */
void oracle_eval_bounds(const atag_cluster_bounds *b, const atag_boundary_point *p, size_t n, size_t w,
                        size_t h, float *cx, float *cy, float *theta, float *dot, uint8_t *valid);
void oracle_eval_linefit(const atag_cluster_point *p, size_t n, uint32_t w, uint32_t h, const uint8_t *img,
                         atag_line_fit_point *out);
void oracle_eval_fit_line(const atag_line_fit_point *m, const uint64_t *nim, size_t n, float *lp, float *err,
                          float *mse);
void oracle_eval_get_moment(const atag_line_fit_point *pre, size_t np, const uint64_t *ranges, size_t n,
                            atag_line_fit_point *out, uint64_t *nout);

/* Throughput helper for the CPU baseline: runs oracle_detect on n frames
 * with up to `threads` OpenMP threads; writes each frame's quad count.
 * Returns the number of threads used. */
int oracle_detect_many(const uint8_t *const *srcs, const int *src_w, const int *src_h, size_t n,
                       const atag_config *cfg, int threads, uint32_t *n_quads);

#ifdef __cplusplus
}
#endif

#endif
