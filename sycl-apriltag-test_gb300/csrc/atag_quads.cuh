// atag_quads.cuh — the combination search of do_indexing and the corner
// intersection of process_fitted_quads, shared by the drop-in kernels and
// the fused per-cluster pipeline.
#pragma once

#include "atag_kernels.cuh"

namespace atag {

struct Combination {
    float err;              // +inf when the combination is invalid
    Moment m[4];
    uint16_t nim[4];
    uint16_t idx[4];
};

// sort_4, fit_quad.cpp:377-389
__device__ __forceinline__ void sort_4(unsigned long long a[4]) {
    auto sw = [&](int i, int j) {
        if (!(a[i] < a[j])) { unsigned long long t = a[i]; a[i] = a[j]; a[j] = t; }
    };
    sw(0, 1); sw(2, 3); sw(0, 2); sw(1, 3); sw(1, 2);
}

// One combination of do_indexing (fit_quad.cpp:404-503).  `cpts` points at
// the prefix sums of the cluster whose extents the caller chose.  A NaN
// total (only reachable through wrapped moments) counts as invalid, which is
// what taking the minimum with `<` does on the host.
__device__ __forceinline__ Combination evaluate_combination(uint32_t n, atag_peak_extents pe,
                                                            const atag_corner* __restrict__ corners,
                                                            const atag_line_fit_point* __restrict__ cpts,
                                                            uint32_t ccount, float max_mse, float cos_critical) {
    Combination c;
    c.err = __int_as_float(0x7f800000);
#pragma unroll
    for (int s = 0; s < 4; s++) { c.m[s] = Moment{0, 0, 0, 0, 0, 0}; c.nim[s] = 0; c.idx[s] = 0; }
    uint32_t m = pe.count < 10u ? pe.count : 10u;
    if (n >= n_choose_4(m)) return c;
    uint32_t d[4];
    combination_decode(n, d);
    unsigned long long lfi[4];
#pragma unroll
    for (int j = 0; j < 4; j++) lfi[j] = corners[pe.start + d[j]].line_fit_point_index;
    sort_4(lfi);
    float total = 0.0f, p01[4], p12[4];
    bool valid = true;
#pragma unroll
    for (int s = 0; s < 4; s++) {
        unsigned long long nim;
        Moment mo = get_moment(cpts, ccount, lfi[s], lfi[(s + 1) & 3], &nim);
        float e, mse;
        fit_line(mo, nim, s == 0 ? p01 : (s == 1 ? p12 : nullptr), &e, &mse);
        valid &= mse <= max_mse;
        c.m[s] = mo;
        c.nim[s] = (uint16_t)nim;
        total = __fadd_rn(total, e);
    }
    float dot = __fadd_rn(__fmul_rn(p01[2], p12[2]), __fmul_rn(p01[3], p12[3]));
    valid &= fabsf(dot) <= cos_critical;
#pragma unroll
    for (int j = 0; j < 4; j++) c.idx[j] = (uint16_t)lfi[j];
    if (valid && !isnan(total)) c.err = total;
    return c;
}

__device__ __forceinline__ uint32_t block_min_u32(uint32_t v, uint32_t* red) {
    v = __reduce_min_sync(0xffffffffu, v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        uint32_t x = lane < nw ? red[lane] : 0xFFFFFFFFu;
        x = __reduce_min_sync(0xffffffffu, x);
        if (lane == 0) red[0] = x;
    }
    __syncthreads();
    return red[0];
}

// do_indexing for one peak cluster on one warp.  The 210 combinations of
// up to 10 peaks only ever fit the 90 ordered segments between two of those
// peaks, so each segment is fitted once (the same get_moment/fit_line calls
// as the per-combination form, hence the same bits) and every combination
// sums four table entries in the reference's order (fit_quad.cpp:445-498).
// The choice is the reference's: the lowest total error, then the smallest
// combination number within 0.1 of it (fit_quad.cpp:501-519).  The lane
// that owns the chosen combination writes *out (its moments recomputed by
// the same calls); every lane returns the chosen number, or -1.
struct SegmentTable {
    float err[10][10], mse[10][10], lp[10][10][4];
    uint32_t idx[10];        // line_fit_point_index of peak rank r
};

__device__ __forceinline__ int index_one_cluster(uint32_t count, const atag_corner* __restrict__ corners,
                                                 const atag_line_fit_point* __restrict__ cpts, uint32_t ccount,
                                                 float max_mse, float cos_critical, SegmentTable& T,
                                                 atag_fitted_quad* out) {
    constexpr int PER = (210 + 31) / 32;  // combinations per lane
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t m = count < 10u ? count : 10u;
    const uint32_t ncomb = n_choose_4(m);
    if (ncomb == 0) return -1;
    if (lane < m) T.idx[lane] = corners[lane].line_fit_point_index;
    __syncwarp();
    for (uint32_t s = lane; s < m * m; s += 32) {
        const uint32_t a = s / m, b = s % m;
        if (a == b) continue;
        const unsigned long long i0 = T.idx[a], i1 = T.idx[b];
        unsigned long long nim;
        const Moment mo = get_moment(cpts, ccount, i0, i1, &nim);
        float e, mse;
        fit_line(mo, nim, i0 < i1 ? T.lp[a][b] : nullptr, &e, &mse);
        T.err[a][b] = e;
        T.mse[a][b] = mse;
    }
    __syncwarp();
    // the ranks of combination n in line-fit index order (sort_4,
    // fit_quad.cpp:437)
    auto ranks = [&](uint32_t n, uint32_t (&r)[4]) {
        uint32_t d[4];
        combination_decode(n, d);
        unsigned long long v[4];
#pragma unroll
        for (int j = 0; j < 4; j++) v[j] = ((unsigned long long)T.idx[d[j]] << 8) | d[j];
        sort_4(v);
#pragma unroll
        for (int j = 0; j < 4; j++) r[j] = (uint32_t)(v[j] & 0xFF);
    };
    float errs[PER];
    uint32_t low_key = float_order_key(__int_as_float(0x7f800000));
#pragma unroll
    for (int t = 0; t < PER; t++) {
        const uint32_t n = lane + 32u * t;
        float err = __int_as_float(0x7f800000);
        if (n < ncomb) {
            uint32_t r[4];
            ranks(n, r);
            float total = 0.0f;
            bool valid = true;
#pragma unroll
            for (int j = 0; j < 4; j++) {
                const uint32_t a = r[j], b = r[(j + 1) & 3];
                valid &= T.mse[a][b] <= max_mse;
                total = __fadd_rn(total, T.err[a][b]);
            }
            const float* p01 = T.lp[r[0]][r[1]];
            const float* p12 = T.lp[r[1]][r[2]];
            const float dot = __fadd_rn(__fmul_rn(p01[2], p12[2]), __fmul_rn(p01[3], p12[3]));
            valid &= fabsf(dot) <= cos_critical;
            if (valid && !isnan(total)) err = total;
        }
        errs[t] = err;
        low_key = min(low_key, float_order_key(err));
    }
    low_key = __reduce_min_sync(0xFFFFFFFFu, low_key);
    const float lowest = float_from_order_key(low_key);
    if (isinf(lowest) && lowest > 0) return -1;
    uint32_t first = 0xFFFFFFFFu;
#pragma unroll
    for (int t = PER - 1; t >= 0; t--)  // (double)(err - lowest) < 0.1, in float
        if (__fsub_rn(errs[t], lowest) < 0x1.99999ap-4f) first = lane + 32u * t;
    const uint32_t chosen = __reduce_min_sync(0xFFFFFFFFu, first);
    if (chosen == 0xFFFFFFFFu) return -1;
    if (lane == (chosen & 31u)) {
        uint32_t r[4];
        ranks(chosen, r);
#pragma unroll
        for (int j = 0; j < 4; j++) {
            const uint32_t a = r[j], b = r[(j + 1) & 3];
            unsigned long long nim;
            const Moment mo = get_moment(cpts, ccount, T.idx[a], T.idx[b], &nim);
            store_moment(&out->moments[j], mo);
            out->num_in_moments[j] = (uint16_t)nim;
            out->indices[j] = (uint16_t)T.idx[a];
        }
    }
    return (int)chosen;
}

__device__ __forceinline__ void write_fitted(atag_fitted_quad* out, const Combination& c) {
#pragma unroll
    for (int s = 0; s < 4; s++) store_moment(&out->moments[s], c.m[s]);
#pragma unroll
    for (int s = 0; s < 4; s++) {
        out->num_in_moments[s] = c.nim[s];
        out->indices[s] = c.idx[s];
    }
}

// process_fitted_quads body (main.cpp:1042-1161) for one FittedQuad.
__device__ __forceinline__ bool quad_corners(const atag_fitted_quad& fq, const PipelineParams& p, uint32_t index,
                                             atag_quad_corners* out) {
    if (!(fq.indices[0] != 0 || fq.indices[1] != 0 || fq.indices[2] != 0 || fq.indices[3] != 0)) return false;
    float lines[4][4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        float e, mse;
        fit_line(load_moment(&fq.moments[i]), fq.num_in_moments[i], lines[i], &e, &mse);
    }
    float cs[4][2];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int j = (i + 1) & 3;
        double A00 = (double)lines[i][3], A01 = -(double)lines[j][3];
        double A10 = -(double)lines[i][2], A11 = (double)lines[j][2];
        double B0 = (double)__fadd_rn(-lines[i][0], lines[j][0]);
        double B1 = (double)__fadd_rn(-lines[i][1], lines[j][1]);
        double det = __dsub_rn(__dmul_rn(A00, A11), __dmul_rn(A10, A01));
        double W00 = __ddiv_rn(A11, det), W01 = __ddiv_rn(-A01, det);
        if (fabs(det) < 0.001) return false;
        double L0 = __dadd_rn(__dmul_rn(W00, B0), __dmul_rn(W01, B1));
        cs[i][0] = __double2float_rn(__dadd_rn((double)lines[i][0], __dmul_rn(L0, A00)));
        cs[i][1] = __double2float_rn(__dadd_rn((double)lines[i][1], __dmul_rn(L0, A10)));
    }
    {
        float area = 0.0f, len[3], pp;
        const int ia[3] = {0, 1, 2}, ib[3] = {1, 2, 0};
#pragma unroll
        for (int i = 0; i < 3; i++)
            len[i] = hypot_f(__fsub_rn(cs[ib[i]][0], cs[ia[i]][0]), __fsub_rn(cs[ib[i]][1], cs[ia[i]][1]));
        pp = __fdiv_rn(__fadd_rn(__fadd_rn(len[0], len[1]), len[2]), 2.0f);
        float t = __fmul_rn(pp, __fsub_rn(pp, len[0]));
        t = __fmul_rn(t, __fsub_rn(pp, len[1]));
        t = __fmul_rn(t, __fsub_rn(pp, len[2]));
        area = __fadd_rn(area, __fsqrt_rn(t));
        const int ja[3] = {2, 3, 0}, jb[3] = {3, 0, 2};
#pragma unroll
        for (int i = 0; i < 3; i++)
            len[i] = hypot_f(__fsub_rn(cs[jb[i]][0], cs[ja[i]][0]), __fsub_rn(cs[jb[i]][1], cs[ja[i]][1]));
        pp = __fdiv_rn(__fadd_rn(__fadd_rn(len[0], len[1]), len[2]), 2.0f);
        t = __fmul_rn(pp, __fsub_rn(pp, len[0]));
        t = __fmul_rn(t, __fsub_rn(pp, len[1]));
        t = __fmul_rn(t, __fsub_rn(pp, len[2]));
        area = __fadd_rn(area, __fsqrt_rn(t));
        if ((double)area < p.min_area) return false;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        int i0 = i, i1 = (i + 1) & 3, i2 = (i + 2) & 3;
        float dx1 = __fsub_rn(cs[i1][0], cs[i0][0]);
        float dy1 = __fsub_rn(cs[i1][1], cs[i0][1]);
        float dx2 = __fsub_rn(cs[i2][0], cs[i1][0]);
        float dy2 = __fsub_rn(cs[i2][1], cs[i1][1]);
        float num = __fadd_rn(__fmul_rn(dx1, dx2), __fmul_rn(dy1, dy2));
        float s1 = __fadd_rn(__fmul_rn(dx1, dx1), __fmul_rn(dy1, dy1));
        float s2 = __fadd_rn(__fmul_rn(dx2, dx2), __fmul_rn(dy2, dy2));
        float cosd = __fdiv_rn(num, __fsqrt_rn(__fmul_rn(s1, s2)));
        if (fabs((double)cosd) > p.cos_critical_d || __fmul_rn(dx1, dy2) < __fmul_rn(dy1, dx2)) return false;
    }
#pragma unroll
    for (int i = 0; i < 4; i++) {
        out->corners[i][0] = cs[i][0];
        out->corners[i][1] = cs[i][1];
    }
    out->reversed_border = (uint8_t)p.reversed_border;
    out->pad_[0] = out->pad_[1] = out->pad_[2] = 0;
    out->blob_index = index;
    return true;
}

}  // namespace atag
