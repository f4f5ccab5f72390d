// k_quads.cu — drop-in kernels for the reference's fit_lines and do_indexing,
// and the corner intersection of process_fitted_quads moved to the device.
#include "atag_kernels.cuh"
#include "atag_quads.cuh"

namespace atag {

// ---------------------------------------------------------------------------
// fit_lines (fit_quad.cpp:153-375), restated warp-per-work-group: 32 lanes
// hold points x = 24 g - 3 ... 24 g + 28 and lanes 4..27 decide corners.
// The work-group barriers become __syncwarp.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(128) k_fit_lines_windowed(const atag_line_fit_point* __restrict__ points,
                                                            const uint16_t* __restrict__ cidx,
                                                            const atag_cluster_extents* __restrict__ extents,
                                                            size_t n, atag_corner* __restrict__ found) {
    constexpr int WG = 32, PPE = 3, EO = 4;
    __shared__ uint16_t s_ci[4][WG];
    __shared__ atag_cluster_extents s_ce[4][WG];
    __shared__ float s_es[4][WG], s_ed[4][WG], s_fs[4][WG], s_fd[4][WG];
    const int wid = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t group = (size_t)blockIdx.x * 4 + wid;
    const size_t groups = (n + 23) / 24;
    if (group >= groups) return;
    const long long x = (long long)group * (WG - 2 * EO) + lane - PPE;
    const long long xc = x < 0 ? 0 : (x > (long long)n - 1 ? (long long)n - 1 : x);
    const uint16_t ci = cidx[xc];
    const atag_cluster_extents ce = extents[ci];
    s_ci[wid][lane] = ci;
    s_ce[wid][lane] = ce;
    __syncwarp();
    s_es[wid][lane] = window_error(points, ce.start, ce.count, x);
    int their = lane;
    if (lane >= EO && s_ci[wid][lane - EO] != ci) their = lane - EO;
    if (lane < WG - EO && s_ci[wid][lane + EO] != ci) their = lane + EO;
    if (their != lane) {
        atag_cluster_extents te = s_ce[wid][their];
        s_ed[wid][lane] = window_error(points, te.start, te.count, x);
    } else {
        s_ed[wid][lane] = __int_as_float(0x7fc00000);
    }
    __syncwarp();
    if (lane >= PPE && lane < WG - PPE) {
        float acc = 0.0f, dacc = 0.0f;
#pragma unroll
        for (int i = 0; i < 7; i++) {
            int t = lane + i - PPE;
            float f = filter_tap(i);
            if (s_ci[wid][t] == ci) {
                acc = __fadd_rn(acc, __fmul_rn(s_es[wid][t], f));
                dacc = __fadd_rn(dacc, __fmul_rn(s_ed[wid][t], f));
            } else {
                dacc = __fadd_rn(dacc, __fmul_rn(s_es[wid][t], f));
                acc = __fadd_rn(acc, __fmul_rn(s_ed[wid][t], f));
            }
        }
        s_fs[wid][lane] = acc;
        s_fd[wid][lane] = dacc;
    }
    __syncwarp();
    if (lane < EO || lane >= WG - EO) return;
    if (x < 0 || x >= (long long)n) return;
    const float cur = s_fs[wid][lane];
    const bool gb = cur > (s_ci[wid][lane - 1] == ci ? s_fs : s_fd)[wid][lane - 1];
    const bool ga = cur > (s_ci[wid][lane + 1] == ci ? s_fs : s_fd)[wid][lane + 1];
    if (gb && ga) {
        atag_corner c;
        c.line_fit_point_index = (uint32_t)(x - ce.start);
        c.cluster_index = ci;
        c.error = cur;
        found[x] = c;
    }
}

// ---------------------------------------------------------------------------
// do_indexing (fit_quad.cpp:392-535): one 256-thread CTA per peak extent,
// one thread per combination number; cluster_extents is indexed by the
// extent's position, exactly as the reference does.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_do_indexing(const atag_peak_extents* __restrict__ extents, size_t count,
                                                     const atag_corner* __restrict__ corners,
                                                     const atag_line_fit_point* __restrict__ points,
                                                     const atag_cluster_extents* __restrict__ cluster_extents,
                                                     float max_mse, float cos_critical,
                                                     atag_fitted_quad* __restrict__ fitted) {
    __shared__ SegmentTable T[8];  // one per warp
    const uint32_t wid = threadIdx.x >> 5;
    for (size_t q = (size_t)blockIdx.x * 8 + wid; q < count; q += (size_t)gridDim.x * 8) {
        const atag_peak_extents pe = extents[q];
        const atag_cluster_extents ce = cluster_extents[q];
        index_one_cluster(pe.count, corners + pe.start, points + ce.start, ce.count, max_mse, cos_critical, T[wid],
                          fitted + q);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// process_fitted_quads (main.cpp:1035-1162) up to tag decoding, on one CTA
// with an ordered compaction.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_process_quads(const atag_fitted_quad* __restrict__ fitted, size_t count,
                                                       PipelineParams p, atag_quad_corners* __restrict__ out,
                                                       size_t cap, uint32_t* __restrict__ count_out) {
    __shared__ uint32_t red[33];
    uint32_t base = 0;
    for (size_t c0 = 0; c0 < count; c0 += blockDim.x) {
        size_t i = c0 + threadIdx.x;
        atag_quad_corners qc;
        bool ok = false;
        if (i < count) ok = quad_corners(fitted[i], p, (uint32_t)i, &qc);
        uint32_t total;
        uint32_t pos = block_exclusive_scan_u32(ok ? 1u : 0u, red, &total);
        if (ok && base + pos < cap) out[base + pos] = qc;
        base += total;
    }
    if (threadIdx.x == 0) *count_out = base < cap ? base : (uint32_t)cap;
}

}  // namespace atag
