// atag.hpp — C++ drop-in layer over the C ABI (atag.h) that keeps the
// reference's function names and argument order (include/threshold.h,
// include/segmentation.h, include/find_boundaries.h, include/fit_quad.h of
// the reference project), with a cudaStream_t in place of the sycl::queue
// and no dependency list (stream order replaces the event list).
//
// Differences from the reference, all deliberate:
//   * every call returns atag_status instead of a sycl::event, and errors
//     (bad sizes, no device) are reported instead of ignored;
//   * fit_lines and do_indexing do not block the host (the reference calls
//     .wait() inside them, src/fit_quad.cpp:374,534);
//   * extrema / filtered_extrema of threshold_image may be null.
#pragma once

#include <cuda_runtime_api.h>

#include <stdexcept>
#include <string>
#include <tuple>

#include "atag.h"

namespace atag {

using BoundaryPoint = atag_boundary_point;
using ClusterPoint = atag_cluster_point;
using ClusterExtents = atag_cluster_extents;
using ClusterBounds = atag_cluster_bounds;
using LineFitPoint = atag_line_fit_point;
using PeakExtents = atag_peak_extents;
using Corner = atag_corner;
using FittedQuad = atag_fitted_quad;
using QuadCorners = atag_quad_corners;

// Mask to get the pixel colour / the label value (segmentation.h:6-9).
constexpr uint32_t LABEL_PIXEL_MASK = 0x80000000u;
constexpr uint32_t LABEL_VALUE_MASK = 0x7FFFFFFFu;

inline atag_stream_t as_stream(cudaStream_t s) { return reinterpret_cast<atag_stream_t>(s); }

// threshold_image, include/threshold.h:6-10 (extrema are (min, max) byte pairs per 4x4 tile)
inline atag_status threshold_image(cudaStream_t q, const uint8_t* grayscale, uint8_t* extrema,
                                   uint8_t* filtered_extrema, uint8_t* thresholded, size_t width,
                                   size_t height) {
    return atag_threshold_image(grayscale, extrema, filtered_extrema, thresholded, width, height, as_stream(q));
}

// image_segmentation, include/segmentation.h:11-15
inline atag_status image_segmentation(cudaStream_t q, const uint8_t* thresholded, uint32_t* label_scratch,
                                      uint32_t* labels, uint32_t* sizes, size_t sizes_elem, size_t width,
                                      size_t height) {
    return atag_image_segmentation(thresholded, label_scratch, labels, sizes, sizes_elem, width, height,
                                   as_stream(q));
}

// find_boundaries, include/find_boundaries.h:8-12 (dense 4-plane output)
inline atag_status find_boundaries(cudaStream_t q, const uint32_t* labels, const uint32_t* sizes,
                                   BoundaryPoint* points, uint64_t* blob_labels, size_t width, size_t height) {
    return atag_find_boundaries(labels, sizes, points, blob_labels, width, height, as_stream(q));
}

// fit_lines, include/fit_quad.h:46-49
inline atag_status fit_lines(cudaStream_t q, const LineFitPoint* points, const uint16_t* cluster_indices,
                             const ClusterExtents* cluster_extents, size_t points_size, Corner* found_corners) {
    return atag_fit_lines(points, cluster_indices, cluster_extents, points_size, found_corners, as_stream(q));
}

// do_indexing, include/fit_quad.h:51-55
inline atag_status do_indexing(cudaStream_t q, const PeakExtents* extents, size_t extents_count,
                               const Corner* compacted_corners, const LineFitPoint* points,
                               const ClusterExtents* cluster_extents, FittedQuad* fitted) {
    return atag_do_indexing(extents, extents_count, compacted_corners, points, cluster_extents, fitted,
                            as_stream(q));
}

// get_moment, include/fit_quad.h:39-41 (host)
inline std::tuple<LineFitPoint, size_t> get_moment(const LineFitPoint* points, size_t points_size, size_t i0,
                                                   size_t i1) {
    LineFitPoint m{};
    size_t n = 0;
    if (atag_get_moment(points, points_size, i0, i1, &m, &n) != ATAG_OK)
        throw std::out_of_range(std::string("get_moment: ") + atag_last_error());
    return std::make_tuple(m, n);
}

// fit_line, include/fit_quad.h:43-44 (host)
inline void fit_line(LineFitPoint moment, size_t num_in_moment, float* line_params, float* err, float* mse) {
    atag_fit_line(&moment, num_in_moment, line_params, err, mse);
}

// compute_initial_linefit, include/line_fit_point.h:50-52 (host)
inline LineFitPoint compute_initial_linefit(ClusterPoint p, uint32_t width, uint32_t height,
                                            const uint8_t* greyscaled) {
    return atag_compute_initial_linefit(p, width, height, greyscaled);
}

// Stages 4-11 of src/main.cpp:467-801 (the oneDPL glue between
// find_boundaries and fit_lines); counts stay on the device.
inline atag_status cluster(cudaStream_t q, const BoundaryPoint* points, const uint64_t* blob_labels,
                           const uint8_t* grayscale, size_t width, size_t height, void* workspace,
                           size_t workspace_bytes, const atag_cluster_outputs& outputs) {
    return atag_cluster(points, blob_labels, grayscale, width, height, workspace, workspace_bytes, &outputs,
                        as_stream(q));
}

// Stages 13-15 of src/main.cpp:832-907 (between fit_lines and do_indexing).
inline atag_status corner_peaks(cudaStream_t q, const Corner* found_corners, const ClusterExtents* cluster_extents,
                                size_t cluster_count, void* workspace, size_t workspace_bytes,
                                Corner* compacted_corners, size_t corner_capacity, PeakExtents* peak_extents,
                                size_t extents_capacity, uint32_t* d_counts) {
    return atag_corner_peaks(found_corners, cluster_extents, cluster_count, workspace, workspace_bytes,
                             compacted_corners, corner_capacity, peak_extents, extents_capacity, d_counts,
                             as_stream(q));
}

// process_fitted_quads, src/main.cpp:1035 (up to, not including, decode_quads)
inline atag_status process_fitted_quads(cudaStream_t q, const FittedQuad* fitted, size_t count, size_t width,
                                        size_t height, QuadCorners* out, size_t capacity, uint32_t* d_count,
                                        const atag_config* cfg = nullptr) {
    return atag_process_fitted_quads(fitted, count, width, height, cfg, out, capacity, d_count, as_stream(q));
}

// Corner refinement as a forward/backward pair with the contract of
// torch.autograd.Function: forward saves what backward needs in a context,
// backward maps output gradients to input gradients.
struct RefineContext {
    const float* image = nullptr;
    size_t width = 0, height = 0;
    const float* corners = nullptr;
    size_t n_quads = 0;
};

struct CornerRefine {
    static atag_status forward(RefineContext& ctx, cudaStream_t q, const float* image, size_t width, size_t height,
                               const float* corners, size_t n_quads, float* refined, float* residual,
                               float* samples = nullptr) {
        ctx = RefineContext{image, width, height, corners, n_quads};
        return atag_refine_forward(image, width, height, corners, n_quads, refined, residual, samples, as_stream(q));
    }
    static atag_status backward(const RefineContext& ctx, cudaStream_t q, const float* grad_refined,
                                const float* grad_residual, float* grad_corners, float* grad_samples = nullptr,
                                float* grad_image = nullptr) {
        return atag_refine_backward(ctx.image, ctx.width, ctx.height, ctx.corners, ctx.n_quads, grad_refined,
                                    grad_residual, grad_corners, grad_samples, grad_image, as_stream(q));
    }
};

// Tag pose per quad (no counterpart in the reference): corner_stride is
// sizeof(QuadCorners) for detector output, 8 floats for packed corners.
inline atag_status estimate_pose(cudaStream_t q, const float* corners, size_t corner_stride, size_t n_quads,
                                 double fx, double fy, double cx, double cy, double tag_size, atag_pose* poses,
                                 uint32_t max_iterations = 20) {
    return atag_estimate_pose(corners, corner_stride, n_quads, fx, fy, cx, cy, tag_size, max_iterations, poses,
                              as_stream(q));
}

// Reads each quad's bits against a tag family described as the AprilTag
// library describes its families (the reference's decode_quads,
// src/quad_decoding.cpp:84-128, with the family as an argument).
inline atag_status decode_quads(cudaStream_t q, const uint8_t* image, size_t width, size_t height,
                                const float* corners, size_t corner_stride, size_t n_quads,
                                const atag_tag_family& family, atag_decoded* out,
                                const atag_decode_params* params = nullptr, size_t pitch = 0) {
    return atag_decode_quads(image, width, height, pitch, corners, corner_stride, n_quads, &family, params, out,
                             as_stream(q));
}

// RAII owner of an atag_detector (the whole path of src/main.cpp:322-1024).
class Detector {
public:
    Detector(size_t max_width, size_t max_height, size_t max_frames = 1, size_t max_total_pixels = 0,
             const atag_config* cfg = nullptr, void* d_workspace = nullptr, size_t workspace_bytes = 0) {
        atag_status s = atag_detector_create(cfg, max_width, max_height, max_frames, max_total_pixels, d_workspace,
                                             workspace_bytes, &det_);
        if (s != ATAG_OK) throw std::runtime_error(std::string("atag_detector_create: ") + atag_last_error());
    }
    ~Detector() { atag_detector_destroy(det_); }
    Detector(const Detector&) = delete;
    Detector& operator=(const Detector&) = delete;

    atag_status detect(cudaStream_t q, const uint8_t* d_grey, size_t width, size_t height, QuadCorners* d_quads,
                       size_t capacity, atag_frame_stats* d_stats) {
        return atag_detect(det_, d_grey, width, height, d_quads, capacity, d_stats, as_stream(q));
    }
    atag_status detect_batch(cudaStream_t q, const atag_frame* frames, size_t n, QuadCorners* d_quads,
                             size_t capacity, atag_frame_stats* d_stats) {
        return atag_detect_batch(det_, frames, n, d_quads, capacity, d_stats, as_stream(q));
    }
    atag_detector* handle() const { return det_; }

private:
    atag_detector* det_ = nullptr;
};

}  // namespace atag
