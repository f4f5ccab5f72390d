/*
 * atag.h — C ABI of the GB300 AprilTag quad-detection path.
 *
 * Every entry point is stream-ordered: it enqueues work on `stream` and
 * returns without waiting for the device, unless its comment says it
 * synchronises.  All pointers named d_* are device pointers; h_* are host
 * pointers.  No entry point allocates device memory except
 * atag_detector_create when it is given no workspace.
 *
 * The record structs below are layout-identical to the reference's records
 * (include/boundary_point.h, include/cluster_bounds.h,
 * include/line_fit_point.h, include/fit_quad.h of the reference project), so
 * dumps of either side compare byte for byte.
 *
 * Constraints shared with the reference (notes.txt:11-16):
 *   width and height after decimation are multiples of 4, at most 4096
 *   (14-bit packed coordinates, include/boundary_point.h:20).
 */
#ifndef ATAG_H
#define ATAG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Opaque CUDA stream handle; binary-compatible with cudaStream_t. */
typedef struct CUstream_st *atag_stream_t;

/* ------------------------------------------------------------------ */
/* Status codes.  The reference has no error reporting at all.        */
/* ------------------------------------------------------------------ */
typedef enum atag_status {
    ATAG_OK = 0,
    ATAG_ERR_INVALID_ARGUMENT = 1, /* bad dimensions, null pointer, size  */
    ATAG_ERR_CUDA = 2,             /* a CUDA runtime call failed          */
    ATAG_ERR_CAPACITY = 3,         /* a device-side capacity overflowed   */
    ATAG_ERR_ITERATION_CAP = 4,    /* a bounded union-find loop gave up   */
    ATAG_ERR_NO_DEVICE = 5,        /* no CUDA device / wrong architecture */
    ATAG_ERR_OUT_OF_MEMORY = 6     /* workspace too small / cudaMalloc    */
} atag_status;

/* Device-side status word bits (atag_frame_stats.status). */
#define ATAG_DEVFLAG_POINT_OVERFLOW 0x1u   /* more boundary points than capacity */
#define ATAG_DEVFLAG_PAIR_OVERFLOW 0x2u    /* pair hash table (or output) full   */
#define ATAG_DEVFLAG_CLUSTER_OVERFLOW 0x4u /* more filtered clusters than cap    */
#define ATAG_DEVFLAG_UF_ITERATION_CAP 0x8u /* union-find merge loop cap hit      */
#define ATAG_DEVFLAG_QUAD_OVERFLOW 0x10u   /* more quads than output capacity    */
#define ATAG_DEVFLAG_SORT_OVERFLOW 0x20u   /* cluster larger than sort capacity  */

/* ------------------------------------------------------------------ */
/* Records (layout-identical to the reference).                       */
/* ------------------------------------------------------------------ */

/* BoundaryPoint, include/boundary_point.h:32-96.
 * packed_x = [HALF_PIXEL:2 | VALUE:14], packed_y = [COLOR_DIR:1 | 0:1 | VALUE:14] */
typedef struct atag_boundary_point {
    uint16_t packed_x;
    uint16_t packed_y;
} atag_boundary_point;

/* ClusterPoint, include/boundary_point.h:100-149 (slope = calc_theta). */
typedef struct atag_cluster_point {
    uint16_t packed_x;
    uint16_t packed_y;
    float slope;
} atag_cluster_point;

/* ClusterExtents, include/cluster_bounds.h:9-12. */
typedef struct atag_cluster_extents {
    uint32_t start;
    uint32_t count;
} atag_cluster_extents;

/* ClusterBounds, include/cluster_bounds.h:14-67 (coordinates are 2x). */
typedef struct atag_cluster_bounds {
    uint16_t x_min, x_max, y_min, y_max;
    int32_t gx_sum, gy_sum;
    int64_t pxgx_pygy_sum;
    uint32_t start, count;
} atag_cluster_bounds;

/* LineFitPoint, include/line_fit_point.h:11-48 (a, b unused). */
typedef struct atag_line_fit_point {
    int64_t Mx, My, Mxx, Myy, Mxy, W, a, b;
} atag_line_fit_point;

/* PeakExtents, include/fit_quad.h:9-12. */
typedef struct atag_peak_extents {
    uint32_t start;
    uint32_t count;
} atag_peak_extents;

/* Corner, include/fit_quad.h:21-25. */
typedef struct atag_corner {
    uint32_t line_fit_point_index;
    uint16_t cluster_index;
    float error;
} atag_corner;

/* FittedQuad, include/fit_quad.h:27-31. */
typedef struct atag_fitted_quad {
    atag_line_fit_point moments[4];
    uint16_t num_in_moments[4];
    uint16_t indices[4];
} atag_fitted_quad;

/* QuadCorners, include/fit_quad.h:33-37.  blob_index is left unset by the
 * reference; here it holds the index of the FittedQuad it came from. */
typedef struct atag_quad_corners {
    float corners[4][2];
    uint8_t reversed_border;
    uint8_t pad_[3];
    uint32_t blob_index;
} atag_quad_corners;

/* ------------------------------------------------------------------ */
/* Configuration: every constant the reference hard-codes.  Defaults  */
/* (atag_config_default) reproduce the reference.                     */
/* ------------------------------------------------------------------ */
typedef struct atag_config {
    int32_t decimate;              /* point-sampling factor (>=1); reference: absent (1) */
    int32_t min_white_black_diff;  /* threshold.cpp:86: "max-min < 5" -> 127            */
    int32_t min_component_size;    /* find_boundaries.cpp:82,98,143: sizes >= 25         */
    int32_t min_cluster_pixels;    /* cluster_bounds.h:89: 5 (and the fixed 24 gate)     */
    int32_t tag_width;             /* cluster_bounds.h:86: bbox area gate (2x coords)    */
    int32_t normal_border;         /* cluster_bounds.h:87                                */
    int32_t reversed_border;       /* cluster_bounds.h:88                                */
    float max_line_fit_mse;        /* fit_quad.cpp:7                                     */
    float critical_angle_deg;      /* 10: cos() of it is taken in double, then rounded to
                                      float for do_indexing (fit_quad.cpp:399) and kept
                                      double for the corner check (main.cpp:1039)     */
    int32_t min_tag_width;         /* main.cpp:1037: area >= 0.95 * w^2                  */
    int32_t compat_peak_index;     /* 1: index cluster extents by peak-cluster position
                                      exactly like fit_quad.cpp:405-408 (default);
                                      0: index by the corner's own cluster             */
} atag_config;

void atag_config_default(atag_config *cfg);

/* Per-frame counters written by the device (one struct per frame). */
typedef struct atag_frame_stats {
    uint32_t width, height;      /* after decimation                       */
    uint32_t n_points;           /* P   boundary points (after size gate)  */
    uint32_t n_pairs;            /* C   distinct cluster pairs             */
    uint32_t n_clusters;         /* C_f clusters passing ValidBlobFilter   */
    uint32_t n_cluster_points;   /* P_f points in those clusters           */
    uint32_t n_corners;          /* K   corner peaks                       */
    uint32_t n_peak_clusters;    /* C_p clusters with >= 1 peak            */
    uint32_t n_fitted;           /* FittedQuads written (nonzero indices)  */
    uint32_t n_quads;            /* Q   quads after geometric rejection    */
    uint32_t status;             /* ATAG_DEVFLAG_* bits                    */
    uint32_t reserved[5];
} atag_frame_stats;

/* ------------------------------------------------------------------ */
/* Library                                                            */
/* ------------------------------------------------------------------ */
const char *atag_status_string(atag_status s);
/* Message of the last failing call on this host thread ("" if none). */
const char *atag_last_error(void);
/* Checks for an sm_103 device and loads the kernels.  Idempotent. */
atag_status atag_init(void);
/* Number of kernel launches this library has issued since load (all streams). */
uint64_t atag_launch_count(void);

/* ------------------------------------------------------------------ */
/* Stage entry points: drop-ins for the reference's device functions. */
/* ------------------------------------------------------------------ */

/* Point-sampling decimation dst(x,y) = src(f*x, f*y); dst is
 * (src_w/f) x (src_h/f).  The reference has none (notes.txt:18-21). */
atag_status atag_decimate(const uint8_t *d_src, size_t src_width, size_t src_height,
                          size_t factor, uint8_t *d_dst, atag_stream_t stream);

/* Input pixel formats.  Colour is removed the way the reference's loader
 * does it (stbi_load(..., STBI_grey), src/main.cpp:264-265): luma
 * (77 r + 150 g + 29 b) >> 8, alpha ignored (include/stb_image.h:1834-1836);
 * grey + alpha keeps the grey byte.  Planar YUV inputs pass their Y plane
 * as ATAG_PIX_GREY8. */
typedef enum atag_pixel_format {
    ATAG_PIX_GREY8 = 0,
    ATAG_PIX_RGB8 = 1,
    ATAG_PIX_RGBA8 = 2,
    ATAG_PIX_BGR8 = 3,
    ATAG_PIX_BGRA8 = 4,
    ATAG_PIX_GREYA8 = 5
} atag_pixel_format;

/* Colour removal and point-sampling decimation in one pass (notes.txt
 * steps 1-2): dst(x,y) = grey(src(f*x, f*y)); src rows are src_pitch bytes
 * apart (0 = width * bytes per pixel). */
atag_status atag_convert_grey(const uint8_t *d_src, size_t src_width, size_t src_height, size_t src_pitch,
                              int format, size_t factor, uint8_t *d_dst, atag_stream_t stream);

/* Replaces threshold_image (include/threshold.h:6-10, src/threshold.cpp:3-98).
 * d_extrema / d_filtered_extrema are 2 bytes per 4x4 tile (min, max) and may
 * be NULL: the fused kernel keeps them in shared memory and only writes them
 * when asked. */
atag_status atag_threshold_image(const uint8_t *d_grayscale, uint8_t *d_extrema,
                                 uint8_t *d_filtered_extrema, uint8_t *d_thresholded,
                                 size_t width, size_t height, atag_stream_t stream);

/* Replaces image_segmentation (include/segmentation.h:11-15,
 * src/segmentation.cpp:95-392).  labels: u32 per pixel, bit 31 = white,
 * low 31 bits = min slot index of the component (255: even slot y*w+x of the
 * 2x2 block, 0: odd slot), 127 -> 0.  sizes: u32[width*height], pixel count
 * of each component at its root index, 0 elsewhere.  label_scratch:
 * u32[width*height] union-find forest.  sizes_elem is unused, as in the
 * reference. */
atag_status atag_image_segmentation(const uint8_t *d_thresholded, uint32_t *d_label_scratch,
                                    uint32_t *d_labels, uint32_t *d_sizes, size_t sizes_elem,
                                    size_t width, size_t height, atag_stream_t stream);

/* Same as atag_image_segmentation, for callers that must not allocate device
 * memory (no counterpart in the reference).  The union-find forest lives in
 * a 2,097,152-word array inside the library (8 MiB per GPU, held until the
 * process exits) instead of a caller buffer; frames larger than 2,097,152
 * pixels are rejected with ATAG_ERR_INVALID_ARGUMENT.  The first call on
 * each device looks up that array's device address, so make it before any
 * stream capture.  All calls share the array: calls that overlap on the GPU
 * race and must be serialised by the caller.  Allocates nothing. */
atag_status atag_image_segmentation_noalloc(const uint8_t *d_thresholded, uint32_t *d_labels,
                                            uint32_t *d_sizes, size_t width, size_t height,
                                            atag_stream_t stream);

/* Replaces find_boundaries (include/find_boundaries.h:8-12,
 * src/find_boundaries.cpp:10-155): the dense 4-plane output at
 * plane*w*h + y*w + x.  The caller pre-fills points with 0 and blob_labels
 * with 0xFF, as src/main.cpp:312-315 does. */
atag_status atag_find_boundaries(const uint32_t *d_labels, const uint32_t *d_sizes,
                                 atag_boundary_point *d_points, uint64_t *d_blob_labels,
                                 size_t width, size_t height, atag_stream_t stream);

/* Replaces fit_lines (include/fit_quad.h:46-49, src/fit_quad.cpp:153-375).
 * points: per-cluster inclusive prefix sums of line-fit moments.  The
 * caller pre-zeroes found_corners (src/main.cpp:316-317).  Unlike the
 * reference this does not block the host. */
atag_status atag_fit_lines(const atag_line_fit_point *d_points, const uint16_t *d_cluster_indices,
                           const atag_cluster_extents *d_cluster_extents, size_t points_size,
                           atag_corner *d_found_corners, atag_stream_t stream);

/* Replaces do_indexing (include/fit_quad.h:51-55, src/fit_quad.cpp:392-535),
 * including its cluster_extents[peak position] indexing.  The caller
 * pre-zeroes fitted (src/main.cpp:318-319).  Does not block the host. */
atag_status atag_do_indexing(const atag_peak_extents *d_extents, size_t extents_count,
                             const atag_corner *d_compacted_corners,
                             const atag_line_fit_point *d_points,
                             const atag_cluster_extents *d_cluster_extents,
                             atag_fitted_quad *d_fitted, atag_stream_t stream);

/* Replaces the host function process_fitted_quads (src/main.cpp:1035-1162)
 * up to, not including, tag decoding: refit the four lines, intersect them
 * in FP64, reject by area and angle.  Runs on the device; quads whose four
 * indices are zero are skipped.  *d_count receives the number written. */
atag_status atag_process_fitted_quads(const atag_fitted_quad *d_fitted, size_t fitted_count,
                                      size_t width, size_t height, const atag_config *cfg,
                                      atag_quad_corners *d_quads, size_t quads_capacity,
                                      uint32_t *d_count, atag_stream_t stream);

/* Replaces the oneDPL glue of stages 4-11 (src/main.cpp:467-801): compaction
 * of the dense boundary planes (point != 0), the sort by pair key, the
 * per-pair ClusterBounds reduction, ValidBlobFilter, the point-to-cluster
 * map with calc_theta, the (cluster, slope) sort, compute_initial_linefit
 * and the segmented prefix sum of the line-fit moments.  Inputs are the
 * outputs of atag_find_boundaries (4 planes of width*height entries) and the
 * grey image compute_initial_linefit samples.  Outputs (device arrays the
 * caller allocates; entries past the counts are left untouched):
 *   pair_bounds / pair_keys  (optional, NULL to skip) every pair's bounds
 *                            and key in key order, up to pair_capacity;
 *   filtered_bounds, filtered_keys (optional), cluster_extents
 *                            the clusters that pass the filter, up to
 *                            cluster_capacity (at most 65535: the cluster
 *                            index is 16 bits, src/main.cpp:641);
 *   cluster_points, cluster_indices, line_fit_points
 *                            their points sorted by (cluster, slope), up to
 *                            point_capacity;
 *   counts                   n_points (P), n_pairs (C), n_clusters (C_f),
 *                            n_cluster_points (P_f) and status (ATAG_DEVFLAG_*:
 *                            a capacity that was too small).
 * Ties of the reference's unstable sorts are fixed by the packed point.
 * Scratch memory is the caller's workspace of atag_cluster_workspace_size
 * bytes.  Stream-ordered; the counts stay on the device. */
typedef struct atag_cluster_outputs {
    atag_cluster_bounds *pair_bounds;
    uint64_t *pair_keys;
    size_t pair_capacity;
    atag_cluster_bounds *filtered_bounds;
    uint64_t *filtered_keys;
    atag_cluster_extents *cluster_extents;
    size_t cluster_capacity;
    atag_cluster_point *cluster_points;
    uint16_t *cluster_indices;
    atag_line_fit_point *line_fit_points;
    size_t point_capacity;
    atag_frame_stats *counts;
} atag_cluster_outputs;

atag_status atag_cluster_workspace_size(size_t width, size_t height, size_t cluster_capacity,
                                        size_t point_capacity, size_t *bytes);
atag_status atag_cluster(const atag_boundary_point *d_points, const uint64_t *d_blob_labels,
                         const uint8_t *d_grayscale, size_t width, size_t height, void *d_workspace,
                         size_t workspace_bytes, const atag_cluster_outputs *outputs, atag_stream_t stream);

/* Replaces stages 13-15 (src/main.cpp:832-907): the corners of
 * atag_fit_lines whose error is not 0, sorted by (cluster, error
 * descending; ties by point index), and one PeakExtents {first corner,
 * count} per cluster that has corners.  d_cluster_extents are the
 * cluster_count extents atag_cluster wrote (fit_lines writes each
 * cluster's corners inside its extent).  d_counts (3 words) receives the
 * corner count K, the PeakExtents count C_p and a status word: corners past
 * corner_capacity and extents past extents_capacity are dropped and set
 * ATAG_DEVFLAG_QUAD_OVERFLOW.  Scratch memory is the caller's workspace of
 * atag_corner_peaks_workspace_size bytes.  Stream-ordered. */
atag_status atag_corner_peaks_workspace_size(size_t cluster_count, size_t *bytes);
atag_status atag_corner_peaks(const atag_corner *d_found_corners, const atag_cluster_extents *d_cluster_extents,
                              size_t cluster_count, void *d_workspace, size_t workspace_bytes,
                              atag_corner *d_compacted_corners, size_t corner_capacity,
                              atag_peak_extents *d_peak_extents, size_t extents_capacity, uint32_t *d_counts,
                              atag_stream_t stream);

/* Host helpers of the reference, evaluated on the host with the device's
 * roundings (int64 products wrap; hypotf is the double-precision root
 * rounded to float, as the reference's host library computes it). */

/* get_moment (include/fit_quad.h:39-41, src/fit_quad.cpp:15-35): the moment
 * of the cyclic range [i0, i1] of one cluster's prefix sums
 * h_points[0 .. points_size); i0 == i1 gives zero and a count of 0.  The a
 * and b fields come from the leading operand, as the reference's copy does.
 * Indices at or past points_size are refused. */
atag_status atag_get_moment(const atag_line_fit_point *h_points, size_t points_size, size_t i0, size_t i1,
                            atag_line_fit_point *h_moment, size_t *h_num_in_moment);

/* fit_line (include/fit_quad.h:43-44, src/fit_quad.cpp:37-105): line
 * parameters (centroid x, y, unit normal x, y), error and mean squared
 * error of a moment of num_in_moment points; any output may be NULL. */
atag_status atag_fit_line(const atag_line_fit_point *h_moment, size_t num_in_moment, float *h_line_params,
                          float *h_err, float *h_mse);

/* compute_initial_linefit (include/line_fit_point.h:50-86): one point's
 * moment contribution, weighted by 1 + (int)hypotf of the central
 * difference of the grey image at (rx/2, rx/2) (the reference samples row
 * rx/2, not ry/2). */
atag_line_fit_point atag_compute_initial_linefit(atag_cluster_point p, uint32_t width, uint32_t height,
                                                 const uint8_t *h_greyscaled);

/* ------------------------------------------------------------------ */
/* Whole-path detector (replaces src/main.cpp:322-1024 stages 1-16 and */
/* the corner intersection).                                          */
/* ------------------------------------------------------------------ */
typedef struct atag_detector atag_detector;

/* One frame of a batch: the source image before colour removal and
 * decimation, `format` an atag_pixel_format (0: grey), rows src_pitch
 * bytes apart (0: packed).  A zero-initialised tail means a packed grey
 * image. */
typedef struct atag_frame {
    const uint8_t *d_grey;
    uint32_t src_width, src_height;
    uint32_t format;
    uint32_t src_pitch;
} atag_frame;

/* Bytes of device workspace a detector needs for up to max_frames frames
 * whose decimated sizes sum to at most max_total_pixels (and none exceeds
 * max_width x max_height after decimation). */
atag_status atag_workspace_size(const atag_config *cfg, size_t max_width, size_t max_height,
                                size_t max_frames, size_t max_total_pixels, size_t *bytes);

/* Creates a detector.  If d_workspace is NULL the detector allocates (and
 * later frees) its own workspace of atag_workspace_size bytes; otherwise the
 * caller's buffer of at least that size is used and nothing is allocated. */
atag_status atag_detector_create(const atag_config *cfg, size_t max_width, size_t max_height,
                                 size_t max_frames, size_t max_total_pixels, void *d_workspace,
                                 size_t workspace_bytes, atag_detector **out);
atag_status atag_detector_destroy(atag_detector *det);

/* Detects quads in n frames at once.  Writes up to quads_capacity quads per
 * frame to d_quads + f*quads_capacity and the frame's counters to
 * d_stats[f].  Stream-ordered, no host synchronisation: every stage sizes
 * its grid from upper bounds and reads its counts on the device, so the
 * call can be captured in a CUDA graph.  A captured call keeps its own copy
 * of the frame table, so its graph detects the captured frames on every
 * replay, whatever eager calls the detector makes in between; up to 16
 * different captured tables per detector (identical ones share a copy),
 * after which a capture fails with ATAG_ERR_CAPACITY until
 * atag_detector_release_captures.  Replays and eager calls share the
 * detector's workspace: they must not overlap on the GPU. */
atag_status atag_detect_batch(atag_detector *det, const atag_frame *h_frames, size_t n_frames,
                              atag_quad_corners *d_quads, size_t quads_capacity,
                              atag_frame_stats *d_stats, atag_stream_t stream);

/* Single frame convenience form of atag_detect_batch. */
atag_status atag_detect(atag_detector *det, const uint8_t *d_grey, size_t src_width,
                        size_t src_height, atag_quad_corners *d_quads, size_t quads_capacity,
                        atag_frame_stats *d_stats, atag_stream_t stream);

/* Host-buffer form: copies h_grey to the device, detects, copies the quads
 * and counters back and synchronises the stream.  *h_n_quads receives the
 * quad count (quads beyond quads_capacity are dropped and flagged). */
atag_status atag_detect_host(atag_detector *det, const uint8_t *h_grey, size_t src_width,
                             size_t src_height, atag_quad_corners *h_quads,
                             size_t quads_capacity, atag_frame_stats *h_stats,
                             atag_stream_t stream);

/* Intermediate buffers of the last detect call, for parity checks and
 * debugging.  Pointers are device pointers into the workspace and stay
 * valid until the next detect call.  Counts are in atag_frame_stats. */
typedef struct atag_frame_views {
    const uint8_t *decimated;                   /* w*h                              */
    const uint8_t *thresholded;                 /* w*h                              */
    const uint32_t *labels;                     /* w*h                              */
    const uint32_t *sizes;                      /* w*h                              */
    const uint64_t *pair_points;                /* (pair slot << 32) | packed point, for
                                                   pairs still under the size limit   */
    uint32_t n_pair_points;                     /* entries in pair_points           */
    uint32_t pair_capacity;                     /* slots of the pair hash table:    */
    const uint64_t *pair_keys;                  /*   key (~0 = empty)               */
    const uint32_t *pair_count;                 /*   points                         */
    const uint32_t *pair_bbox;                  /*   x_min, x_max, y_min, y_max     */
    const int32_t *pair_gsum;                   /*   gx_sum, gy_sum                 */
    const int64_t *pair_pxgx;                   /*   pxgx_pygy_sum                  */
    const uint64_t *cluster_keys;               /* n_clusters pair keys, ascending  */
    const atag_cluster_bounds *cluster_bounds;  /* n_clusters (start = position among
                                                   all pairs' points in key order)  */
    const atag_cluster_extents *cluster_extents;/* n_clusters                       */
    const atag_cluster_point *cluster_points;   /* n_cluster_points, sorted         */
    const atag_line_fit_point *line_fit_points; /* n_cluster_points prefix sums     */
    const uint32_t *peak_count;                 /* n_clusters: peaks per cluster    */
    const atag_corner *peaks;                   /* n_clusters x 10: best peaks      */
    const uint32_t *peak_clusters;              /* n_peak_clusters: rank -> cluster */
    const atag_peak_extents *peak_extents;      /* n_peak_clusters                  */
    const atag_fitted_quad *fitted;             /* n_peak_clusters (by rank)        */
    uint32_t point_capacity;                    /* entries of pair_points           */
    uint32_t cluster_capacity;                  /* filtered clusters                */
    uint32_t cluster_point_capacity;            /* points of filtered clusters      */
    uint32_t reserved_;
} atag_frame_views;

/* Selects the CUDA device this library launches on for the calling host
 * thread (the library keeps its own CUDA runtime state). */
atag_status atag_use_device(int ordinal);

atag_status atag_detector_views(const atag_detector *det, size_t frame, atag_frame_views *out);

/* Per-frame capacities and iteration caps below the ones the detector sizes
 * for itself, for callers that bound a frame's work and for exercising the
 * device status flags.  0 keeps a field's default; values above the default
 * are clipped to it, so a limit never needs more workspace.  Work past a
 * capacity is dropped and flagged in atag_frame_stats.status; nothing is
 * written past it.  Applies to later detect calls. */
typedef struct atag_limits {
    uint32_t point_capacity;         /* listed boundary points (ATAG_DEVFLAG_POINT_OVERFLOW)        */
    uint32_t pair_capacity;          /* pair table slots, rounded down to a power of two
                                        (ATAG_DEVFLAG_PAIR_OVERFLOW)                              */
    uint32_t cluster_capacity;       /* filtered clusters (ATAG_DEVFLAG_CLUSTER_OVERFLOW)           */
    uint32_t cluster_point_capacity; /* points of filtered clusters (ATAG_DEVFLAG_CLUSTER_OVERFLOW) */
    uint32_t uf_iteration_cap;       /* parents one frame-wide union-find walk follows and retries of
                                        one union (ATAG_DEVFLAG_UF_ITERATION_CAP); the default is
                                        the bound the CCL tile count gives for a w x h frame,
                                        2 + 160 ceil(w / 64) ceil(h / 16)                       */
    uint32_t reserved[3];
} atag_limits;
atag_status atag_detector_set_limits(atag_detector *det, const atag_limits *limits);

/* Subpixel refinement of the detected corners (no counterpart in the
 * reference, whose corners are the FP64 intersections of its line fits,
 * src/main.cpp:1059-1099).  When enabled, later detect calls end with one
 * more stage that replaces each quad's corners, in place, by
 * atag_refine_forward's refined corners computed on the frame's grey image
 * (as value / 255); a corner whose adjacent edge lines are nearly parallel
 * keeps its position.  Off by default: the quads are then the reference's. */
atag_status atag_detector_set_refinement(atag_detector *det, int enable);

/* Frees the frame-table copies held for captured calls; call it once every
 * graph captured from this detector has been destroyed. */
atag_status atag_detector_release_captures(atag_detector *det);

/* Intermediates of later detect calls.  By default a detector writes only
 * what its own later stages read: labels in full, parents at even rows and
 * component sizes at the root slots; and once a pair's point count is over
 * ValidBlobFilter's maximum, its later points are no longer summed (its
 * pair_count, pair_bbox, pair_gsum and pair_pxgx stop growing; it is
 * rejected all the same).  keep != 0 makes it also write the rest of the
 * reference's scratch and sizes arrays (parents compressed to roots, block
 * information words, zero sizes away from roots:
 * src/segmentation.cpp:309-389), as atag_image_segmentation does, and sum
 * every pair in full, so that atag_detector_views shows them complete. */
atag_status atag_detector_keep_intermediates(atag_detector *det, int keep);

/* ------------------------------------------------------------------ */
/* Subpixel corner refinement (no counterpart in the reference, which  */
/* stops at the corners of process_fitted_quads, src/main.cpp:1035).    */
/* ------------------------------------------------------------------ */
/* Per quad and edge (corner i -> corner i+1): 16 positions along the edge,
 * 4 bilinear taps of the FP32 image across it at -1.5, -0.5, 0.5, 1.5 px
 * (64 samples), an edge point per position offset along the normal by the
 * strength-weighted mean of the tap differences, a weighted line fit of the
 * 16 points (weight: edge strength + 1e-6, so a flat edge keeps its line) (FP32 moments about the edge midpoint, FP64 2x2 eigen-solve),
 * and refined corner i = intersection of edge lines i-1 and i (FP64).
 * corners/refined: n_quads x 4 x 2 floats (x, y); residual: n_quads x 4
 * (weight sum times the smallest covariance eigenvalue: the weighted
 * line-fit residual); samples: n_quads x 4 x 64 (may be NULL). */
atag_status atag_refine_forward(const float *d_image, size_t width, size_t height, const float *d_corners,
                                size_t n_quads, float *d_refined, float *d_residual, float *d_samples,
                                atag_stream_t stream);
/* Adjoint of atag_refine_forward: given dL/d(refined) and dL/d(residual)
 * (either may be NULL = zero), writes dL/d(corners) (n_quads x 8),
 * dL/d(samples) (n_quads x 4 x 64, may be NULL) and accumulates dL/d(image)
 * into d_grad_image (width x height, may be NULL; caller zeroes it). */
atag_status atag_refine_backward(const float *d_image, size_t width, size_t height, const float *d_corners,
                                 size_t n_quads, const float *d_grad_refined, const float *d_grad_residual,
                                 float *d_grad_corners, float *d_grad_samples, float *d_grad_image,
                                 atag_stream_t stream);

/* ------------------------------------------------------------------ */
/* Tag pose from quad corners (no counterpart in the reference; a      */
/* downstream consumer of its quads).                                  */
/* ------------------------------------------------------------------ */
/* Corner i of a quad is taken as the image of the tag-plane point
 * (tag_size / 2) * c_i, c = (-1,-1), (1,-1), (1,1), (-1,1), z = 0: for a tag
 * seen upright from the front (tag z axis pointing away from the camera)
 * that is top-left, top-right, bottom-right, bottom-left, clockwise on a
 * y-down image.  A quad wound the other way is taken in the order 0, 3, 2,
 * 1 and flagged.  Without decoding the tag's rotation by multiples of 90
 * degrees is unknown; the corner order fixes it.  Pinhole camera without
 * distortion: x = fx X / Z + cx, y = fy Y / Z + cy; camera point
 * = R * tag point + t. */
#define ATAG_POSE_REORDERED 0x1u  /* corners were wound the other way         */
#define ATAG_POSE_DEGENERATE 0x2u /* no homography or no pose in front of the
                                     camera; R, t, H and reproj_rms are zero   */
typedef struct atag_pose {
    double R[9];         /* row-major rotation, tag frame -> camera frame   */
    double t[3];         /* translation, in the unit of tag_size            */
    double H[9];         /* row-major homography tag plane (X, Y, 1) ->
                            pixel (x, y, 1) of the refined pose, H[8] = 1   */
    double reproj_rms;   /* RMS corner reprojection error in pixels         */
    uint32_t iterations; /* accepted Levenberg-Marquardt steps              */
    uint32_t status;     /* ATAG_POSE_* bits                                */
} atag_pose;

/* One pose per quad, FP64: homography of the unit square onto the quad in
 * closed form, initial pose from its columns (polar-orthogonalised
 * rotation), then up to max_iterations Levenberg-Marquardt trials on the
 * pixel reprojection error of the four corners (20 is plenty; 0 keeps the
 * homography's pose).  Corner q's eight floats (x0, y0,
 * .. x3, y3) start at byte q * corner_stride of d_corners: 40 for an array
 * of atag_quad_corners, 32 for packed corners such as atag_refine_forward's
 * output. */
atag_status atag_estimate_pose(const float *d_corners, size_t corner_stride, size_t n_quads, double fx,
                               double fy, double cx, double cy, double tag_size, uint32_t max_iterations,
                               atag_pose *d_poses, atag_stream_t stream);

/* ------------------------------------------------------------------ */
/* Reading tags: each quad's bits against a code family.  The reference */
/* hands each quad to the AprilTag library's quad_decode_task with       */
/* tag36h11 and the detector defaults plus quad_decimate = 1            */
/* (src/quad_decoding.cpp:46-75); that library and its family tables    */
/* are not in the reference tree, so the family is an argument, in the  */
/* library's own terms.                                                  */
/* ------------------------------------------------------------------ */
#define ATAG_DECODE_REORDERED 0x1u    /* corners were wound the other way        */
#define ATAG_DECODE_DEGENERATE 0x2u   /* no homography, or part of the tag
                                         projects behind the camera            */
#define ATAG_DECODE_LOW_CONTRAST 0x4u /* white minus black grey model at the tag
                                         centre below min_contrast, or a model
                                         without enough samples: no bits read  */

/* A tag family as the AprilTag library describes one: bit i of a code
 * (code bit nbits - 1 - i) is the cell (bit_x[i], bit_y[i]) of a grid whose
 * cells 0 .. width_at_border - 1 span the outer edge of the black border
 * (cells may lie outside it: coordinates are signed); total_width cells
 * span the whole tag (the sharpening grid, at most 16).  The layout must
 * carry bit cells onto bit cells under quarter turns, as the library's
 * families do.  A code with bits at or above nbits never matches. */
typedef struct atag_tag_family {
    uint32_t nbits;           /* 1..64                                          */
    uint32_t width_at_border; /* at least 3                                     */
    uint32_t total_width;     /* total_width - width_at_border even             */
    uint32_t reversed_border; /* 1: the border is white on black                */
    const int8_t *h_bit_x;    /* host arrays of nbits cell coordinates          */
    const int8_t *h_bit_y;
    const uint64_t *d_codes;  /* device array of n_codes codes                  */
    uint32_t n_codes;
    uint32_t max_hamming;     /* largest accepted distance (bits corrected)     */
} atag_tag_family;

/* The library's detector parameters that decoding reads. */
typedef struct atag_decode_params {
    float decode_sharpening;  /* 0.25                                           */
    int32_t refine_edges;     /* 1: refine each edge before reading             */
    int32_t quad_decimate;    /* 1: edge search +-(quad_decimate + 1) px        */
    float min_contrast;       /* 0: reject when the white model is not brighter */
} atag_decode_params;
void atag_decode_params_default(atag_decode_params *params);

typedef struct atag_decoded {
    uint64_t code;           /* bits read, before any rotation (bit nbits-1-i = bit i) */
    int32_t id;              /* index of the matched code, -1 if none            */
    uint32_t hamming;        /* distance to the nearest code over the 4 turns    */
    uint32_t rotation;       /* quarter turns of the read grid that give the match */
    uint32_t status;         /* ATAG_DECODE_* bits                               */
    float decision_margin;   /* min(mean value of white bits, mean magnitude of
                                black bits), after sharpening                    */
    float black, white;      /* grey models at the tag centre                    */
    float corners[4][2];     /* the edge-refined corners; for a match, turned so
                                that corner 0 is the tag's first corner          */
    uint32_t reserved;
} atag_decoded;

/* Per quad (corners as for atag_estimate_pose, used as given, as the
 * reference passes its QuadCorners to the library): a quad wound the other
 * way is read with corners 0, 3, 2, 1 and flagged; the edges are refined
 * (params->refine_edges); the homography of the tag square [-1, 1]^2 onto
 * the quad; planar grey models (least squares) of the white ring just
 * outside the black border and of the border, from nearest-pixel samples
 * one per cell along each side; each bit's bilinear sample (pixel centres
 * at +0.5) minus the models' mean, sharpened by decode_sharpening times the
 * 4-neighbour Laplacian of the bit grid, bit = value > 0; the decision
 * margin; the code and quarter turn with the smallest Hamming distance
 * (ties: fewer turns, then the lower index), accepted at most max_hamming
 * with a decision margin of at least 0.  params may be NULL (defaults).
 * corner_stride: 40 for detector output, 32 for packed corners; pitch 0 =
 * width. */
atag_status atag_decode_quads(const uint8_t *d_image, size_t width, size_t height, size_t pitch,
                              const float *d_corners, size_t corner_stride, size_t n_quads,
                              const atag_tag_family *family, const atag_decode_params *params,
                              atag_decoded *d_out, atag_stream_t stream);

/* Launch shapes of the detector's kernels.  Every choice gives the same
 * results; only the speed changes.  atag_detector_create starts from the
 * defaults below; the autotuner (sycl-apriltag-test_gb300/atag/autotune.py)
 * picks them per GPU and workload. */
typedef struct atag_tuning {
    int32_t ccl_tile_rows;        /* 8, 16 or 32 rows of 2x2 blocks per CCL tile (16) */
    int32_t boundary_tile_rows;   /* 8 or 16 pixel rows per boundary tile (16)      */
    int32_t small_cluster_max;    /* clusters up to this size use the 128-thread
                                     kernel, larger ones the 512-thread one
                                     (1..2048, default 2048)                        */
    int32_t small_ctas_per_sm;    /* persistent CTAs of the small-cluster kernel (8) */
    int32_t large_ctas_divisor;   /* large-cluster CTAs = SMs / divisor (2)         */
    int32_t index_ctas_per_sm;    /* CTAs of the combination search per SM (8)      */
    int32_t batch_lanes;          /* a batch runs as this many sub-batches on
                                     concurrent streams (1..4, default 2)           */
} atag_tuning;

atag_status atag_detector_get_tuning(const atag_detector *det, atag_tuning *out);
atag_status atag_detector_set_tuning(atag_detector *det, const atag_tuning *tuning);

/* Stage timing.  When set, every later detect call records events[i] (a
 * cudaEvent_t) on its stream just before stage i and events[ATAG_STAGE_COUNT]
 * after the last, so cudaEventElapsedTime(events[i], events[i+1]) is stage
 * i's device time.  Pass NULL / 0 to stop.  The reference prints cumulative
 * per-stage wall times instead (src/main.cpp:330-977). */
#define ATAG_STAGE_COUNT 16
atag_status atag_detector_set_stage_events(atag_detector *det, void *const *events, size_t n_events);
/* Name of stage i (e.g. "ccl_local"), or NULL past the last. */
const char *atag_stage_name(int stage);

#ifdef __cplusplus
}
#endif

#endif /* ATAG_H */
