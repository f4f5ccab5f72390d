// atag_kernels.cuh — per-frame device descriptors and kernel declarations.
#pragma once

#include "atag_device.cuh"

namespace atag {

// Everything a kernel needs to know about one frame: its size and where its
// buffers live in the workspace.  A batch is an array of these in device
// memory; kernels pick their frame from blockIdx.y (pixel stages),
// blockIdx.x (boundary points) or a flattened work index (cluster stages).
struct FrameDesc {
    // sizes
    uint32_t width, height;            // after decimation
    uint32_t factor;                   // decimation factor
    uint32_t src_stride;               // source row pitch in bytes
    uint32_t src_format;               // atag_pixel_format of the source
    // pixel buffers
    const uint8_t* src;                // source frame (before decimation)
    uint8_t* grey;                     // decimated grey frame (== src when grey and factor 1)
    uint8_t* thr;                      // thresholded
    uint8_t* extrema;                  // optional tile min/max (2 B / tile)
    uint8_t* filtered_extrema;         // optional dilated min/max
    uint32_t* scratch;                 // union-find forest (w*h)
    uint32_t* labels;                  // w*h
    uint32_t* sizes;                   // w*h
    atag_boundary_point* dense_points; // optional 4 planes (drop-in find_boundaries)
    uint64_t* dense_keys;              // optional 4 planes
    // boundary points grouped by pair (fused path)
    unsigned long long* points;        // (pair slot << 32) | packed point
    uint32_t point_cap;
    // pair hash table
    uint32_t pair_cap;                 // power of two
    unsigned long long* pair_keys;     // EMPTY = ~0
    uint4* pair_bbox;                  // x_min, x_max, y_min, y_max (2x coords)
    int2* pair_gsum;                   // gx_sum, gy_sum
    unsigned long long* pair_pxgx;     // pxgx_pygy_sum
    uint32_t* pair_count;
    uint32_t* pair_cluster;            // slot -> filtered cluster index or INVALID
    // filtered clusters (sorted by pair key)
    uint32_t cluster_cap;
    unsigned long long* cluster_keys;
    atag_cluster_bounds* cluster_bounds;
    atag_cluster_extents* cluster_extents;
    float2* cluster_center;            // (cx, cy)
    uint32_t* cluster_cursor;
    uint32_t* peak_count;              // per cluster
    atag_corner* peaks;                // per cluster x 10
    uint32_t* peak_clusters;           // rank q -> cluster
    atag_peak_extents* peak_extents;   // rank q -> {start, count}
    atag_fitted_quad* fitted;          // per rank q
    atag_quad_corners* quad_tmp;       // per rank q
    uint32_t* quad_ok;                 // per rank q
    // cluster points
    uint32_t cpoint_cap;
    unsigned long long* sortbuf;       // (theta key << 32) | packed
    atag_cluster_point* cluster_points;
    atag_line_fit_point* line_fit;
    float* errbuf;                     // 2 floats per point (big clusters)
    uint32_t* cluster_work;            // small clusters from the front, large from the back
    uint32_t* cluster_runs;            // first run (CE_RUN points) of each cluster
    // outputs
    atag_quad_corners* quads;
    uint32_t quad_cap;
    atag_frame_stats* stats;
    uint32_t* counters;                // per-frame work counters (see Counter)
    // DEAD_PAIRS keys (EMPTY = ~0) of pairs whose running point count is
    // already above the cluster size limit; null when not tracked
    unsigned long long* dead_pairs;
    // iteration cap of the frame-wide union-find loops (0: the bound the
    // tile count gives, see k_pixels.cu)
    uint32_t uf_cap;
    // optional (stage entry point): every pair's ClusterBounds and key in
    // key order, up to pair_out_cap entries; null in the fused path
    atag_cluster_bounds* pair_bounds_out;
    unsigned long long* pair_keys_out;
    uint32_t pair_out_cap;
    // 1: write the reference's complete segmentation arrays (every parent
    // compressed to its root, block information words at odd rows, zero
    // sizes away from roots).  0 (fused batches): only what later stages
    // read, i.e. parents at even rows and sizes at the roots.
    uint32_t stage_outputs;
    // Tile CCL edge records (ccl_edge_words(tile rows) words per CCL tile,
    // see k_pixels.cu): the tile roots and cross-tile links of each tile's
    // edge blocks, written by the tile pass and read by the border pass.
    // Null: the border pass reads the thresholded image and the forest.
    uint32_t* edges;
};

// Words of one CCL tile's edge record (tiles of 32 blocks x `rows` block
// rows): per edge block a (255 slot, 0 slot) pair of tile roots whose bits
// 24-27 hold that forest's P, Q, R, S links: the top row [0, 32), the
// bottom row [32, 64), the left column [64, 64 + rows), the right column
// [64 + rows, 64 + 2 rows).
__host__ __device__ constexpr uint32_t ccl_edge_words(uint32_t rows) { return 2 * (64 + 2 * rows); }

// The frames a launch works on: a device table (batches) or one descriptor
// passed by value (stage entry points, which must not allocate).  Kernels
// receive it as a __grid_constant__ parameter, so `one` is read in place.
struct FrameSet {
    const FrameDesc* table;
    FrameDesc one;
    __device__ __forceinline__ const FrameDesc& get(uint32_t i) const { return table ? table[i] : one; }
};

// per-frame counters (FrameDesc::counters[...])
enum Counter : uint32_t {
    CNT_POINTS = 0,      // boundary points written
    CNT_STATUS = 1,      // ATAG_DEVFLAG_* bits
    CNT_CLUSTERS = 2,    // filtered clusters
    CNT_PEAKCLU = 3,     // clusters with peaks
    CNT_WORK = 4,        // work-queue cursor
    CNT_ALLPOINTS = 5,   // boundary points found (list entries of pairs already
                         // known to exceed the cluster size limit are skipped)
    CNT_SMALL = 6,       // clusters of at most CF_SMALL_CAP points
    CNT_LARGE = 7,       // larger clusters
    CNT_RUNS = 8,        // runs of up to CE_RUN points of one cluster
    CNT_COUNT = 9
};

constexpr uint32_t DEAD_PAIRS = 2;

// Cluster-sort kernel shapes: most clusters are small and run several per SM
// on 128 threads (up to 16 keys per thread), large ones get a 512-thread CTA
// (up to 32 keys per thread); both sort in registers and shared memory (a
// padded array of kpad_size(cap) keys).  Clusters larger than CF_LARGE_CAP
// (4K frames only) radix-sort in global memory with per-warp counters.
constexpr uint32_t CF_SMALL_THREADS = 128, CF_SMALL_CAP = CF_SMALL_THREADS * 16;
constexpr uint32_t CF_LARGE_THREADS = 512, CF_LARGE_CAP = CF_LARGE_THREADS * 32;
constexpr uint32_t CF_SMALL_SMEM = kpad_size(CF_SMALL_CAP) * 8;
constexpr uint32_t CF_LARGE_SMEM = kpad_size(CF_LARGE_CAP) * 8 + (CF_LARGE_THREADS / 32) * 256 * 4;
// Shared memory of the small-cluster kernel for clusters of at most `cap`
// points: the sorts work on whole powers of two of at least 2 keys per
// thread.
__host__ __device__ constexpr uint32_t cf_small_smem(uint32_t cap) {
    uint32_t k = CF_SMALL_THREADS * 2;
    while (k < cap) k <<= 1;
    return kpad_size(k) * 8;
}
// Window errors / filter / peaks: one warp per run of up to CE_RUN
// consecutive points of one cluster.
constexpr uint32_t CE_RUN = 256;

// Batch-wide prefix offsets of up to four per-frame counters.
struct BatchOffsets {
    uint32_t which[4];
    uint32_t* offsets[4];      // n_frames + 1 entries each, or null
    uint32_t* work_counters;   // one queue cursor per used entry, reset to 0
};

struct PipelineParams {
    int min_white_black_diff;
    uint32_t min_component_size;
    uint32_t min_cluster_pixels;
    uint32_t tag_width;
    int normal_border, reversed_border;
    float max_line_fit_mse;
    float cos_critical_f;      // float(cos(angle)) for do_indexing
    double cos_critical_d;     // cos(angle) for the corner check
    double min_area;           // 0.95 * min_tag_width^2
    int compat_peak_index;
};

// k_pixels.cu
__global__ void k_decimate(const __grid_constant__ FrameSet fs);
__global__ void k_threshold(const __grid_constant__ FrameSet fs, int min_diff, int write_extrema);
// CCL tiles of 32 x 8 or 32 x 16 blocks (2x2 pixels)
__global__ void k_ccl_local_r8(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_local_r16(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_r8(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_local_r32(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_r16(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_r32(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_edges_r8(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_edges_r16(const __grid_constant__ FrameSet fs);
__global__ void k_ccl_border_edges_r32(const __grid_constant__ FrameSet fs);
// final labelling: grid (cdiv(w / 4, CCL_FINAL_THREADS), h / 2, frames) of
// CCL_FINAL_THREADS threads, one pair of 2x2 blocks per thread
constexpr int CCL_FINAL_THREADS = 128;
__global__ void k_ccl_final(const __grid_constant__ FrameSet fs);
__global__ void k_boundaries_dense(const __grid_constant__ FrameSet fs, uint32_t min_size);

// k_quads.cu (drop-in stage kernels)
__global__ void k_fit_lines_windowed(const atag_line_fit_point* points, const uint16_t* cluster_indices,
                                     const atag_cluster_extents* extents, size_t n, atag_corner* found);
__global__ void k_do_indexing(const atag_peak_extents* extents, size_t count, const atag_corner* corners,
                              const atag_line_fit_point* points, const atag_cluster_extents* cluster_extents,
                              float max_mse, float cos_critical, atag_fitted_quad* fitted);
__global__ void k_process_quads(const atag_fitted_quad* fitted, size_t count, PipelineParams p,
                                atag_quad_corners* out, size_t cap, uint32_t* count_out);

// k_cluster.cu (fused path)
__global__ void k_reset_frames(const __grid_constant__ FrameSet fs);
// boundary tiles of 64 x 8 or 64 x 16 pixels
__global__ void k_boundaries_pairs_r8(const __grid_constant__ FrameSet fs, uint32_t min_size);
__global__ void k_boundaries_pairs_r16(const __grid_constant__ FrameSet fs, uint32_t min_size);
__global__ void k_pairs_finalize(const __grid_constant__ FrameSet fs, PipelineParams p, uint32_t small_max);
__global__ void k_scatter_points(const __grid_constant__ FrameSet fs);
__global__ void k_cluster_sort_small(const __grid_constant__ FrameSet fs, const uint32_t* work_offsets,
                                     uint32_t n_frames, uint32_t* work_counter, uint32_t sort_cap);
__global__ void k_cluster_sort_large(const __grid_constant__ FrameSet fs, const uint32_t* work_offsets,
                                     uint32_t n_frames, uint32_t* work_counter);
__global__ void k_cluster_errors(const __grid_constant__ FrameSet fs, const uint32_t* run_offsets,
                                 uint32_t n_frames, uint32_t* work_counter);
__global__ void k_cluster_peaks(const __grid_constant__ FrameSet fs, const uint32_t* cluster_offsets,
                                uint32_t n_frames);
__global__ void k_peaks_scan(const __grid_constant__ FrameSet fs, PipelineParams p);
__global__ void k_batch_offsets(const __grid_constant__ FrameSet fs, uint32_t n_frames, BatchOffsets a);
__global__ void k_index_quads(const __grid_constant__ FrameSet fs, const uint32_t* work_offsets, uint32_t n_frames,
                              PipelineParams p);
__global__ void k_compact_quads(const __grid_constant__ FrameSet fs);

// k_refine.cu: refinement of the detector's quads in place (optional stage)
__global__ void k_refine_detected(const __grid_constant__ FrameSet fs);

// k_stage_cluster.cu (stage entry points over the dense boundary planes)
__global__ void k_planes_pairs(const __grid_constant__ FrameSet fs, const uint32_t* __restrict__ points,
                               const unsigned long long* __restrict__ keys, uint32_t n);
__global__ void k_planes_scatter(const __grid_constant__ FrameSet fs, const uint32_t* __restrict__ points,
                                 const unsigned long long* __restrict__ keys, uint32_t n);
__global__ void k_stage_cluster_out(const __grid_constant__ FrameSet fs, uint16_t* cluster_indices,
                                    unsigned long long* cluster_keys_out);
// corner peaks (stages 13-15): per-cluster counts, offsets and sorted corners
constexpr uint32_t PK_SORT_CAP = 16384;  // corners of one cluster (at most half its points)
constexpr uint32_t PK_SMEM = PK_SORT_CAP * 8;
__global__ void k_peaks_count(const atag_corner* __restrict__ found, const atag_cluster_extents* __restrict__ ext,
                              uint32_t n_clusters, uint32_t* __restrict__ counts);
__global__ void k_peaks_offsets(const uint32_t* __restrict__ counts, uint32_t n_clusters,
                                uint32_t* __restrict__ offsets, atag_peak_extents* __restrict__ peak_extents,
                                uint32_t extents_cap, uint32_t corner_cap, uint32_t* __restrict__ d_counts);
__global__ void k_peaks_sort(const atag_corner* __restrict__ found, const atag_cluster_extents* __restrict__ ext,
                             uint32_t n_clusters, const uint32_t* __restrict__ counts,
                             const uint32_t* __restrict__ offsets, atag_corner* __restrict__ out,
                             uint32_t corner_cap, uint32_t* __restrict__ d_counts);

}  // namespace atag
