// atag_device.cuh — device-side arithmetic shared by every kernel.
//
// Each float/double operation is spelled with an explicit round-to-nearest
// intrinsic (__fadd_rn, __fmul_rn, __fdiv_rn, __dsqrt_rn, ...) so that nvcc
// can neither contract a multiply-add into an FMA nor pick an approximate
// division: the results are the IEEE results of the operations as written in
// the reference (C++ semantics, one rounding per operation).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/atag.h"

namespace atag {

constexpr uint32_t LABEL_PIXEL_MASK = 0x80000000u;  // segmentation.h:7
constexpr uint32_t LABEL_VALUE_MASK = 0x7FFFFFFFu;  // segmentation.h:9
constexpr uint16_t COLOR_DIR_MASK = 0x8000u;        // boundary_point.h:18
constexpr uint16_t COORD_VALUE_MASK = 0x3FFFu;      // boundary_point.h:20
constexpr uint32_t INVALID = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// Wrapping int64 arithmetic (the reference's int64 products may overflow at
// 4K; two's-complement wrap is what the hardware does).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ long long wmul(long long a, long long b) {
    return (long long)((unsigned long long)a * (unsigned long long)b);
}
__host__ __device__ __forceinline__ long long wadd(long long a, long long b) {
    return (long long)((unsigned long long)a + (unsigned long long)b);
}
__host__ __device__ __forceinline__ long long wsub(long long a, long long b) {
    return (long long)((unsigned long long)a - (unsigned long long)b);
}

// ---------------------------------------------------------------------------
// hypotf of the reference's host library: the squares formed exactly in
// double, summed with one rounding to 53 bits, the square root rounded to 53
// bits and then to float: R24(sqrt(R53(a^2 + b^2))) (the second rounding of
// the root is innocuous: 53 >= 2*24 + 2).  FP64 runs at a small fraction of
// the FP32/INT32 rate on this GPU, so the same roundings are carried out in
// integer arithmetic:
//   * |a| >= |b| = m_a 2^e_a, m_b 2^e_b with 24-bit integer significands;
//   * a^2 + b^2 = (m_a^2 2^d + m_b^2) 2^(2 e_b), d = 2 (e_a - e_b), formed
//     exactly in two 64-bit words (d < 56; for d >= 56, m_b^2 lies below the
//     53-bit rounding position of m_a^2 2^d and the result is |a|);
//   * rounded to a 53-bit significand M (to nearest, ties to even);
//   * M scaled by an even power of two into [2^60, 2^62), its integer square
//     root r (31 bits, Newton's method from a float estimate, then exact
//     correction) and the remainder M - r^2 decide the rounding of r to 24
//     bits (a remainder of 0 at the half-way point is a tie, to even).
// Subnormal, huge (>= 2^63) and non-finite inputs never occur on the path;
// they take the FP64 route.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t f2u(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    __builtin_memcpy(&u, &f, 4);
    return u;
#endif
}
__host__ __device__ __forceinline__ float u2f(uint32_t u) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(u);
#else
    float f;
    __builtin_memcpy(&f, &u, 4);
    return f;
#endif
}
__host__ __device__ __forceinline__ int clz64(unsigned long long v) {
#ifdef __CUDA_ARCH__
    return __clzll((long long)v);
#else
    return v ? __builtin_clzll(v) : 64;
#endif
}
__host__ __device__ __forceinline__ float hypot_f_fp64(float a, float b) {
#ifdef __CUDA_ARCH__
    double da = (double)a, db = (double)b;
    return __double2float_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(da, da), __dmul_rn(db, db))));
#else
    const double da = (double)a, db = (double)b;
    volatile double p = da * da, q = db * db;  // exact squares, no contraction
    volatile double s = p + q;
    return (float)__builtin_sqrt(s);
#endif
}
// floor(sqrt(m)) for m in [2^60, 2^62), with 32-bit conversions only (the
// 64-bit ones issue on the FP64 pipe): a float estimate from the top 32
// bits (relative error < 2^-22, so within 2^10 of the root), one Newton
// step on the exact integer residual, then exact +-1 correction.
__host__ __device__ __forceinline__ unsigned long long isqrt_2_60(unsigned long long m) {
    const uint32_t mh = (uint32_t)(m >> 30);  // [2^30, 2^32)
    const uint32_t r0 = (uint32_t)(sqrtf((float)mh) * 32768.0f);
    const long long e = (long long)(m - (unsigned long long)r0 * r0);
    const float ef = (float)(int)(e >> 20) * 1048576.0f + (float)(uint32_t)(e & 0xFFFFF);
    const int d = (int)rintf(ef / (2.0f * (float)r0));
    unsigned long long u = (unsigned long long)((long long)r0 + d);
    while (u * u > m) u--;
    while ((u + 1) * (u + 1) <= m) u++;
    return u;
}
__host__ __device__ __forceinline__ float u64_to_f32_rn(unsigned long long u) {
    if (u < (1ull << 24)) return (float)(uint32_t)u;
    const int L = 64 - clz64(u), sh = L - 24;  // sh >= 1
    unsigned long long m = u >> sh;
    const unsigned long long rem = u & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
    int e = sh;
    if (rem > half || (rem == half && (m & 1ull))) {
        m++;
        if (m >> 24) {
            m >>= 1;
            e++;
        }
    }
    return u2f((uint32_t)(e + 23 + 127) << 23 | ((uint32_t)m & 0x7FFFFFu));
}
__host__ __device__ __forceinline__ float i64_to_f32_rn(long long v) {
    const unsigned long long u = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
    const float f = u64_to_f32_rn(u);
    return v < 0 ? -f : f;
}
__host__ __device__ __forceinline__ float hypot_f(float a, float b) {
    uint32_t x = f2u(a) & 0x7FFFFFFFu, y = f2u(b) & 0x7FFFFFFFu;
    if (x < y) {
        const uint32_t t = x;
        x = y;
        y = t;
    }
    if (y == 0) return u2f(x);
    if (x < 0x00800000u || x >= 0x5F000000u) return hypot_f_fp64(a, b);
    const int ex = (int)(x >> 23) - 150;
    const int ey = (y >> 23) ? (int)(y >> 23) - 150 : -149;
    const unsigned long long mx = (x & 0x7FFFFFu) | 0x800000u;
    const unsigned long long my = (y >> 23) ? ((y & 0x7FFFFFu) | 0x800000u) : (y & 0x7FFFFFu);
    const int d = 2 * (ex - ey);
    if (d >= 56) return u2f(x);
    // S = hi:lo = mx^2 2^d + my^2, in units of 2^(2 ey)
    const unsigned long long A = mx * mx, B = my * my;
    unsigned long long lo = (A << d) + B;
    unsigned long long hi = (d ? (A >> (64 - d)) : 0ull) + (lo < B ? 1ull : 0ull);
    int E = 2 * ey;
    const int L = hi ? 128 - clz64(hi) : 64 - clz64(lo);
    unsigned long long M;
    if (L <= 53) {
        M = lo;
    } else {
        const int sh = L - 53;  // 1..50
        M = (lo >> sh) | (hi << (64 - sh));
        const unsigned long long rem = lo & ((1ull << sh) - 1ull), half = 1ull << (sh - 1);
        E += sh;
        if (rem > half || (rem == half && (M & 1ull))) {
            M++;
            if (M >> 53) {
                M >>= 1;
                E++;
            }
        }
    }
    // M 2^E, M < 2^53: scale into [2^60, 2^62) with an even exponent
    int s = 62 - (64 - clz64(M));
    if ((E - s) & 1) s--;
    const unsigned long long Mn = M << s;
    E -= s;
    const unsigned long long r = isqrt_2_60(Mn);  // [2^30, 2^31)
    unsigned long long q = r >> 7;
    const uint32_t low = (uint32_t)(r & 127u);
    if (low > 64u || (low == 64u && (r * r != Mn || (q & 1ull)))) q++;
    int k = E / 2 + 7;  // value = q 2^k
    if (q >> 24) {
        q >>= 1;
        k++;
    }
    return u2f((uint32_t)(k + 23 + 127) << 23 | ((uint32_t)q & 0x7FFFFFu));
}

// bytes per pixel of an atag_pixel_format (0 for an unknown format)
__host__ __device__ __forceinline__ uint32_t pixel_bytes(uint32_t format) {
    switch (format) {
    case ATAG_PIX_GREY8: return 1;
    case ATAG_PIX_GREYA8: return 2;
    case ATAG_PIX_RGB8: case ATAG_PIX_BGR8: return 3;
    case ATAG_PIX_RGBA8: case ATAG_PIX_BGRA8: return 4;
    default: return 0;
    }
}

// ---------------------------------------------------------------------------
// BoundaryPoint helpers (boundary_point.h).  COORDINATE_HALF_PIXEL_MASK is 0
// (boundary_point.h:16), so dx() == 1 and dy() == 0 for every point.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t bp_xd(uint32_t packed) {  // x_with_dx()
    return (2u * (packed & COORD_VALUE_MASK) + 1u) & 0xFFFFu;
}
__host__ __device__ __forceinline__ uint32_t bp_yd(uint32_t packed) {  // y_with_dy()
    return (2u * ((packed >> 16) & COORD_VALUE_MASK)) & 0xFFFFu;
}
__host__ __device__ __forceinline__ int bp_gx(uint32_t packed) {
    return ((packed >> 16) & COLOR_DIR_MASK) ? 1 : -1;
}
__host__ __device__ __forceinline__ int bp_gy(uint32_t) { return 0; }

// calc_theta, boundary_point.h:48-61
__device__ __forceinline__ float calc_theta(uint32_t packed, float cx, float cy) {
    float dx = __fsub_rn((float)bp_xd(packed), cx);
    float dy = __fsub_rn((float)bp_yd(packed), cy);
    float quadrant;
    if (dx > 0) quadrant = dy > 0 ? 65536.0f : 0.0f;
    else quadrant = dy > 0 ? 131072.0f : -65536.0f;
    if ((dx > 0) == (dy > 0)) return __fadd_rn(quadrant, __fdiv_rn(dy, dx));
    return __fsub_rn(quadrant, __fdiv_rn(dx, dy));
}

// ClusterBounds::cx/cy, cluster_bounds.h:47-49
__device__ __forceinline__ float bounds_cx(uint32_t xmin, uint32_t xmax) {
    float h = __fmul_rn((float)(xmin + xmax), 0.5f);
    return __double2float_rn(__dadd_rn((double)h, 0.05118));
}
__device__ __forceinline__ float bounds_cy(uint32_t ymin, uint32_t ymax) {
    float h = __fmul_rn((float)(ymin + ymax), 0.5f);
    return __double2float_rn(__dadd_rn((double)h, -0.028581));
}
// ClusterBounds::dot, cluster_bounds.h:51-66
__device__ __forceinline__ float bounds_dot(uint32_t xmin, uint32_t xmax, uint32_t ymin, uint32_t ymax,
                                            int gx_sum, int gy_sum, long long pxgx) {
    uint32_t sx = xmin + xmax, sy = ymin + ymax;
    int t = (int)(sx * (uint32_t)gx_sum + sy * (uint32_t)gy_sum);
    float cxcy = __double2float_rn(__dmul_rn((double)t, 0.5));
    float gxc = __double2float_rn(__dmul_rn(0.05118, (double)__int2float_rn(gx_sum)));
    float gyc = __double2float_rn(__dmul_rn(-0.028581, (double)__int2float_rn(gy_sum)));
    float r = __fmul_rn(2.0f, i64_to_f32_rn(pxgx));
    r = __fsub_rn(r, cxcy);
    r = __fsub_rn(r, gxc);
    r = __fsub_rn(r, gyc);
    return r;
}

// ValidBlobFilter, cluster_bounds.h:85-120
struct FilterParams {
    uint32_t min_cluster_pixels;
    uint32_t max_cluster_pixels;  // 2 * (2 w + 2 h)
    uint32_t tag_width;
    int normal_border, reversed_border;
};
__device__ __forceinline__ bool valid_blob(const FilterParams& f, uint32_t count, uint32_t xmin,
                                           uint32_t xmax, uint32_t ymin, uint32_t ymax, int gx_sum,
                                           int gy_sum, long long pxgx) {
    if (count < f.min_cluster_pixels) return false;
    if (count < 24) return false;
    if (count > f.max_cluster_pixels) return false;
    if ((uint32_t)((int)(xmax - xmin) * (int)(ymax - ymin)) < f.tag_width) return false;
    bool reversed = bounds_dot(xmin, xmax, ymin, ymax, gx_sum, gy_sum, pxgx) < 0.0f;
    if (!f.reversed_border && reversed) return false;
    if (!f.normal_border && !reversed) return false;
    return true;
}

// ---------------------------------------------------------------------------
// Line-fit moments (line_fit_point.h, fit_quad.cpp:15-105)
// ---------------------------------------------------------------------------
// Single-precision operations rounded to nearest on both sides: the device
// spells each one as its _rn intrinsic (never contracted into an FMA), the
// host build compiles plain operators with -ffp-contract=off.
__host__ __device__ __forceinline__ float rn_add(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
__host__ __device__ __forceinline__ float rn_sub(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
__host__ __device__ __forceinline__ float rn_mul(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
__host__ __device__ __forceinline__ float rn_div(float a, float b) {
#ifdef __CUDA_ARCH__
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}

struct Moment {
    long long Mx, My, Mxx, Myy, Mxy, W;
};

__host__ __device__ __forceinline__ Moment load_moment(const atag_line_fit_point* p) {
    const longlong2* q = reinterpret_cast<const longlong2*>(p);
    longlong2 a = q[0], b = q[1], c = q[2];
    return Moment{a.x, a.y, b.x, b.y, c.x, c.y};
}
__host__ __device__ __forceinline__ void store_moment(atag_line_fit_point* p, const Moment& m) {
    longlong2* q = reinterpret_cast<longlong2*>(p);
    q[0] = make_longlong2(m.Mx, m.My);
    q[1] = make_longlong2(m.Mxx, m.Myy);
    q[2] = make_longlong2(m.Mxy, m.W);
    q[3] = make_longlong2(0, 0);
}
__host__ __device__ __forceinline__ Moment m_add(Moment a, const Moment& b) {
    a.Mx = wadd(a.Mx, b.Mx); a.My = wadd(a.My, b.My); a.Mxx = wadd(a.Mxx, b.Mxx);
    a.Myy = wadd(a.Myy, b.Myy); a.Mxy = wadd(a.Mxy, b.Mxy); a.W = wadd(a.W, b.W);
    return a;
}
__host__ __device__ __forceinline__ Moment m_sub(Moment a, const Moment& b) {
    a.Mx = wsub(a.Mx, b.Mx); a.My = wsub(a.My, b.My); a.Mxx = wsub(a.Mxx, b.Mxx);
    a.Myy = wsub(a.Myy, b.Myy); a.Mxy = wsub(a.Mxy, b.Mxy); a.W = wsub(a.W, b.W);
    return a;
}

// Integer floor(sqrt(v)) for v < 2^17: equals (int64)hypotf(gx, gy) for the
// central differences of a u8 image (line_fit_point.h:70-75).
__host__ __device__ __forceinline__ uint32_t isqrt_small(uint32_t v) {
#ifdef __CUDA_ARCH__
    uint32_t r = (uint32_t)__fsqrt_rn((float)v);
#else
    uint32_t r = (uint32_t)sqrtf((float)v);
#endif
    while (r * r > v) r--;
    while ((r + 1) * (r + 1) <= v) r++;
    return r;
}

// compute_initial_linefit, line_fit_point.h:50-86 (weight row rx/2, sic).
__host__ __device__ __forceinline__ uint32_t grey_at(const uint8_t* __restrict__ grey, size_t i) {
#ifdef __CUDA_ARCH__
    return __ldg(grey + i);
#else
    return grey[i];
#endif
}
__host__ __device__ __forceinline__ Moment initial_linefit(uint32_t packed, uint32_t width, uint32_t height,
                                                           const uint8_t* __restrict__ grey) {
    long long rx = (long long)bp_xd(packed) + 1;
    long long ry = (long long)bp_yd(packed) + 1;
    uint32_t x = (uint32_t)(rx / 2);
    uint32_t y = (uint32_t)(rx / 2);
    long long W = 1;
    if (x > 0 && x + 1 < width && y > 0 && y + 1 < height) {
        int gx = (int)grey_at(grey, (size_t)y * width + x + 1) - (int)grey_at(grey, (size_t)y * width + x - 1);
        int gy = (int)grey_at(grey, (size_t)(y + 1) * width + x) - (int)grey_at(grey, (size_t)(y - 1) * width + x);
        W += (long long)isqrt_small((uint32_t)(gx * gx + gy * gy));
    }
    return Moment{W * rx, W * ry, W * rx * rx, W * ry * ry, W * rx * ry, W};
}

// The inputs of compute_initial_linefit packed as rx | ry << 16 | W << 32
// (rx, ry <= 8193, W <= 362), so a cluster's moments can be rebuilt from
// shared memory without touching the image again.
__device__ __forceinline__ unsigned long long linefit_rxyw(uint32_t packed, uint32_t width, uint32_t height,
                                                           const uint8_t* __restrict__ grey) {
    uint32_t rx = bp_xd(packed) + 1;
    uint32_t ry = bp_yd(packed) + 1;
    uint32_t x = rx / 2, y = rx / 2;
    uint32_t W = 1;
    if (x > 0 && x + 1 < width && y > 0 && y + 1 < height) {
        int gx = (int)__ldg(grey + (size_t)y * width + x + 1) - (int)__ldg(grey + (size_t)y * width + x - 1);
        int gy = (int)__ldg(grey + (size_t)(y + 1) * width + x) - (int)__ldg(grey + (size_t)(y - 1) * width + x);
        W += isqrt_small((uint32_t)(gx * gx + gy * gy));
    }
    return (unsigned long long)rx | ((unsigned long long)ry << 16) | ((unsigned long long)W << 32);
}
__device__ __forceinline__ Moment moment_of(unsigned long long v) {
    long long rx = (long long)(v & 0xFFFF), ry = (long long)((v >> 16) & 0xFFFF), W = (long long)(v >> 32);
    return Moment{W * rx, W * ry, W * rx * rx, W * ry * ry, W * rx * ry, W};
}

// get_moment, fit_quad.cpp:15-35 over a prefix-sum array of one cluster.
__host__ __device__ __forceinline__ Moment get_moment(const atag_line_fit_point* points, unsigned long long n,
                                             unsigned long long i0, unsigned long long i1,
                                             unsigned long long* total) {
    Moment r{0, 0, 0, 0, 0, 0};
    *total = 0;
    if (i0 < i1) {
        *total = i1 - i0 + 1;
        r = load_moment(points + i1);
        if (i0 > 0) r = m_sub(r, load_moment(points + i0 - 1));
    } else if (i1 < i0) {
        *total = n - i0 + i1 + 1;
        r = load_moment(points + (n - 1));
        r = m_sub(r, load_moment(points + i0 - 1));
        r = m_add(r, load_moment(points + i1));
    }
    return r;
}

// fit_line, fit_quad.cpp:37-105.
__host__ __device__ __forceinline__ void fit_line(const Moment& m, unsigned long long num_in_moment, float* lp,
                                         float* err, float* mse) {
    long long Csxx = wsub(wmul(m.Mxx, m.W), wmul(m.Mx, m.Mx));
    long long Csxy = wsub(wmul(m.Mxy, m.W), wmul(m.Mx, m.My));
    long long Csyy = wsub(wmul(m.Myy, m.W), wmul(m.My, m.My));
    long long cf = wmul(wmul(m.W, m.W), 4);
    const float dxy = i64_to_f32_rn(wsub(Csxx, Csyy)), cxy2 = i64_to_f32_rn(wmul(2, Csxy));
    float sdist = hypot_f(dxy, cxy2);
    float num = rn_sub(i64_to_f32_rn(wadd(Csxx, Csyy)), sdist);
    float eig = rn_div(num, i64_to_f32_rn(wmul(cf, 2)));
    if (lp) {
        float nx1 = rn_sub(dxy, sdist);
        float ny1 = cxy2;
        float nx2 = ny1;
        float ny2 = rn_sub(i64_to_f32_rn(wsub(Csyy, Csxx)), sdist);
        float M1 = rn_add(rn_mul(nx1, nx1), rn_mul(ny1, ny1));
        float M2 = rn_add(rn_mul(nx2, nx2), rn_mul(ny2, ny2));
        float nx, ny;
        if (M1 > M2) { nx = nx1; ny = ny1; } else { nx = nx2; ny = ny2; }
        float w2 = i64_to_f32_rn(wmul(m.W, 2));
        lp[0] = rn_div(i64_to_f32_rn(m.Mx), w2);
        lp[1] = rn_div(i64_to_f32_rn(m.My), w2);
        float length = hypot_f(nx, ny);
        if (fabsf(length) < 0x1.19799ap-40f) {  // (double)|length| < 1e-12, in float
            lp[2] = 0.0f;
            lp[3] = 0.0f;
        } else {
            lp[2] = rn_div(nx, length);
            lp[3] = rn_div(ny, length);
        }
    }
    if (err) *err = rn_mul(u64_to_f32_rn(num_in_moment), eig);
    if (mse) *mse = eig;
}

// Error of the window [i-k, i+k] around global point x, fit_quad.cpp:202-225.
__device__ __forceinline__ float window_error(const atag_line_fit_point* points, uint32_t start,
                                              uint32_t count, long long x) {
    unsigned long long k = count / 12;
    if (k > 20) k = 20;
    if (k < 2) return __int_as_float(0x7fc00000);
    unsigned long long i0 = (unsigned long long)((long long)count + x - (long long)start - (long long)k) % count;
    unsigned long long i1 = (unsigned long long)((long long)count + x - (long long)start + (long long)k) % count;
    unsigned long long n;
    Moment m = get_moment(points + start, count, i0, i1, &n);
    float e;
    fit_line(m, n, nullptr, &e, nullptr);
    return e;
}

// window_error for a point at cluster-local index i of a cluster of n > 2k
// points whose prefix sums start at `points` (same arithmetic, no modulo).
__device__ __forceinline__ float window_error_local(const atag_line_fit_point* points, uint32_t n, uint32_t k,
                                                    uint32_t i) {
    if (k < 2) return __int_as_float(0x7fc00000);
    uint32_t i0 = i >= k ? i - k : i + n - k;
    uint32_t i1 = i + k < n ? i + k : i + k - n;
    unsigned long long cnt;
    Moment m = get_moment(points, n, i0, i1, &cnt);
    float e;
    fit_line(m, cnt, nullptr, &e, nullptr);
    return e;
}

// 7-tap low-pass filter, fit_quad.cpp:10-13
__device__ __forceinline__ float filter_tap(int i) {
    switch (i) {
    case 0: case 6: return 0x1.6c0504p-7f;
    case 1: case 5: return 0x1.152aaap-3f;
    case 2: case 4: return 0x1.368b3p-1f;
    default: return 0x1p+0f;
    }
}

// Combinatorial number system decode of n < 210 into 4 descending indices
// below 10 (combinadics.h:36-53 with Combinadics<uint8_t,15,4,16>).
__device__ __forceinline__ void combination_decode(uint32_t num, uint32_t out[4]) {
    // C(c, k) for c = 0..9, k = 4..1
    const uint32_t c4[10] = {0, 0, 0, 0, 1, 5, 15, 35, 70, 126};
    const uint32_t c3[10] = {0, 0, 0, 1, 4, 10, 20, 35, 56, 84};
    const uint32_t c2[10] = {0, 0, 1, 3, 6, 10, 15, 21, 28, 36};
    int c = 9;
    while (c > 0 && c4[c] > num) c--;
    num -= c4[c];
    out[0] = c;
    c = 9;
    while (c > 0 && c3[c] > num) c--;
    num -= c3[c];
    out[1] = c;
    c = 9;
    while (c > 0 && c2[c] > num) c--;
    num -= c2[c];
    out[2] = c;
    out[3] = num;
}
__host__ __device__ __forceinline__ uint32_t n_choose_4(uint32_t n) {
    return n < 4 ? 0 : n * (n - 1) * (n - 2) * (n - 3) / 24;
}

// Order-preserving map float -> uint32 (for radix/bitonic keys).
__device__ __forceinline__ uint32_t float_order_key(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float float_from_order_key(uint32_t k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// ---------------------------------------------------------------------------
// Block-wide helpers
// ---------------------------------------------------------------------------

// Ascending bitonic sort of n 64-bit keys (n arbitrary): the "flip" form of
// the network, where every comparator points upward, so a missing partner
// beyond n behaves as +infinity and is simply skipped.
__device__ __forceinline__ void bitonic_sort_u64(unsigned long long* keys, uint32_t n) {
    uint32_t npow = 1, lg = 0;
    while (npow < n) {
        npow <<= 1;
        lg++;
    }
    for (uint32_t lk = 1; lk <= lg; lk++) {
        // flip step of the merge of blocks of k = 2^lk
        const uint32_t lh = lk - 1, hmask = (1u << lh) - 1u;
        for (uint32_t t = threadIdx.x; t < npow / 2; t += blockDim.x) {
            const uint32_t base = (t >> lh) << lk, r = t & hmask;
            const uint32_t i = base + r, j = base + ((1u << lk) - 1u - r);
            if (j < n) {
                unsigned long long a = keys[i], b = keys[j];
                if (a > b) { keys[i] = b; keys[j] = a; }
            }
        }
        __syncthreads();
        for (int lj = (int)lk - 2; lj >= 0; lj--) {
            const uint32_t jm = (1u << lj) - 1u;
            for (uint32_t t = threadIdx.x; t < npow / 2; t += blockDim.x) {
                const uint32_t i = ((t >> lj) << (lj + 1)) + (t & jm), p = i + (1u << lj);
                if (p < n) {
                    unsigned long long a = keys[i], b = keys[p];
                    if (a > b) { keys[i] = b; keys[p] = a; }
                }
            }
            __syncthreads();
        }
    }
}

__device__ __forceinline__ unsigned long long warp_max_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        unsigned long long w = __shfl_xor_sync(0xffffffffu, v, o);
        v = w > v ? w : v;
    }
    return v;
}
__device__ __forceinline__ uint32_t warp_sum_u32(uint32_t v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Block reductions through a caller-provided shared array of 32 slots.
__device__ __forceinline__ unsigned long long block_max_u64(unsigned long long v, unsigned long long* red) {
    v = warp_max_u64(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        unsigned long long x = lane < nw ? red[lane] : 0ull;
        x = warp_max_u64(x);
        if (lane == 0) red[0] = x;
    }
    __syncthreads();
    return red[0];
}
__device__ __forceinline__ uint32_t block_sum_u32(uint32_t v, uint32_t* red) {
    v = warp_sum_u32(v);
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        uint32_t x = lane < nw ? red[lane] : 0u;
        x = warp_sum_u32(x);
        if (lane == 0) red[0] = x;
    }
    __syncthreads();
    return red[0];
}

// Block exclusive scan of uint32 (returns the exclusive prefix; *total gets
// the block total).  `red` holds 33 slots.
__device__ __forceinline__ uint32_t block_exclusive_scan_u32(uint32_t v, uint32_t* red, uint32_t* total) {
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) red[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t s = lane < nw ? red[lane] : 0u;
        uint32_t t = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        red[lane] = t - s;  // exclusive prefix of warp totals
        if (lane == 31) red[32] = t;
    }
    __syncthreads();
    uint32_t r = red[wid] + x - v;
    *total = red[32];
    return r;
}

// Shared-memory key arrays of the cluster sorts keep one spare slot after
// every 16 keys: a warp whose lanes touch 2 to 16 consecutive keys each
// (sorted runs, per-lane segments) then hits distinct banks.
__host__ __device__ constexpr uint32_t kpad(uint32_t i) { return i + (i >> 4); }
__host__ __device__ constexpr uint32_t kpad_size(uint32_t n) { return n + n / 16; }

// ---------------------------------------------------------------------------
// Bitonic sort of T*K 64-bit keys held K per thread in registers.  On exit
// thread t holds elements [t K, t K + K) of the ascending order.  Element e
// lives in register e % K of thread e / K: compare distances below K are
// register swaps, distances up to a warp are shuffles, longer ones go
// through `xch` (T*K keys of shared memory, laid out r * T + t).
// ---------------------------------------------------------------------------
template <int K, int J>
__device__ __forceinline__ void bitonic_regs_stage(unsigned long long (&v)[K], int base, int k) {
#pragma unroll
    for (int r = 0; r < K; r++) {
        if ((r ^ J) > r) {
            const int p = r ^ J;
            const bool asc = ((base + r) & k) == 0;
            const unsigned long long a = v[r], b = v[p];
            const bool sw = (a > b) == asc;
            v[r] = sw ? b : a;
            v[p] = sw ? a : b;
        }
    }
}

template <int T, int K>
__device__ __forceinline__ void bitonic_sort_regs(unsigned long long (&v)[K], unsigned long long* xch) {
    const int tid = threadIdx.x, base = tid * K;
    for (int k = 2; k <= T * K; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j >= K) {
                const int pj = j / K;
                const bool keep_min = ((tid & pj) == 0) == ((tid & (k / K)) == 0);
                if (pj < 32) {
#pragma unroll
                    for (int r = 0; r < K; r++) {
                        const unsigned long long o = __shfl_xor_sync(0xFFFFFFFFu, v[r], pj);
                        v[r] = keep_min ? (o < v[r] ? o : v[r]) : (o > v[r] ? o : v[r]);
                    }
                } else {
                    __syncthreads();  // the previous exchange has been read
#pragma unroll
                    for (int r = 0; r < K; r++) xch[r * T + tid] = v[r];
                    __syncthreads();
#pragma unroll
                    for (int r = 0; r < K; r++) {
                        const unsigned long long o = xch[r * T + (tid ^ pj)];
                        v[r] = keep_min ? (o < v[r] ? o : v[r]) : (o > v[r] ? o : v[r]);
                    }
                }
            } else if (j == 1) {
                bitonic_regs_stage<K, 1>(v, base, k);
            } else if (j == 2) {
                if constexpr (K > 2) bitonic_regs_stage<K, 2>(v, base, k);
            } else if (j == 4) {
                if constexpr (K > 4) bitonic_regs_stage<K, 4>(v, base, k);
            } else if (j == 8) {
                if constexpr (K > 8) bitonic_regs_stage<K, 8>(v, base, k);
            } else if (j == 16) {
                if constexpr (K > 16) bitonic_regs_stage<K, 16>(v, base, k);
            }
        }
    }
}

// Sorts src[0, n) (global memory, n <= T*K) into dst[kpad(i)] (shared memory
// of kpad_size(T*K) keys, also used for the exchange); all threads of the
// CTA call it.
template <int T, int K>
__device__ __forceinline__ void sort_keys_regs(const unsigned long long* __restrict__ src, uint32_t n,
                                               unsigned long long* dst) {
    static_assert(K <= 32 && (K & (K - 1)) == 0, "K must be a power of two up to 32");
    unsigned long long v[K];
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = (uint32_t)(r * T) + threadIdx.x;  // coalesced; the order is sorted away
        v[r] = e < n ? src[e] : ~0ull;
    }
    bitonic_sort_regs<T, K>(v, dst);
    __syncthreads();
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = threadIdx.x * K + r;
        if (e < n) dst[kpad(e)] = v[r];
    }
    __syncthreads();
}

// Block merge sort of src[0, n) (global memory, n <= T*K) into dst[kpad(i)]
// (shared memory of kpad_size(T*K) keys).  Each thread sorts K keys in
// registers, then log2(T) rounds merge pairs of sorted runs, doubling their
// length: a thread finds where its K outputs start on the merge path of its
// two runs (binary search along the diagonal, ties taken from the first
// run) and merges K keys serially.  Its work is O(n log(n / K)) against the
// O(n log^2 n) of a bitonic network, which pays from about 8 keys per thread.
template <int T, int K>
__device__ __forceinline__ void merge_sort_keys(const unsigned long long* __restrict__ src, uint32_t n,
                                                unsigned long long* dst) {
    static_assert(K >= 2 && K <= 32 && (K & (K - 1)) == 0, "K must be a power of two in [2, 32]");
    unsigned long long v[K];
#pragma unroll
    for (int r = 0; r < K; r++) {
        const uint32_t e = (uint32_t)(r * T) + threadIdx.x;  // coalesced; the order is sorted away
        v[r] = e < n ? src[e] : ~0ull;
    }
#pragma unroll
    for (int k = 2; k <= K; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int r = 0; r < K; r++) {
                const int p = r ^ j;
                if (p > r) {
                    const unsigned long long a = v[r], b = v[p];
                    const bool sw = (a > b) == ((r & k) == 0);
                    v[r] = sw ? b : a;
                    v[p] = sw ? a : b;
                }
            }
    const uint32_t tid = threadIdx.x;
    // rounds whose pairs of runs belong to one warp only need that warp
    // in step; wider rounds synchronise the CTA
#pragma unroll 1
    for (uint32_t width = 1; width < (uint32_t)T; width <<= 1) {
#pragma unroll
        for (int r = 0; r < K; r++) dst[kpad(tid * K + r)] = v[r];
        if (2 * width <= 32) __syncwarp();
        else __syncthreads();
        const uint32_t g0 = tid & ~(2 * width - 1), L = width * K;
        const uint32_t a0 = g0 * K, b0 = a0 + L, d = (tid - g0) * K;
        uint32_t lo = d > L ? d - L : 0u, hi = d < L ? d : L;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (dst[kpad(a0 + mid)] <= dst[kpad(b0 + d - 1 - mid)]) lo = mid + 1;
            else hi = mid;
        }
        uint32_t i = lo, j = d - lo;
        unsigned long long a = i < L ? dst[kpad(a0 + i)] : 0ull;
        unsigned long long b = j < L ? dst[kpad(b0 + j)] : 0ull;
#pragma unroll
        for (int k = 0; k < K; k++) {
            const bool ta = j >= L || (i < L && a <= b);
            v[k] = ta ? a : b;
            if (k + 1 < K) {
                i += ta ? 1u : 0u;
                j += ta ? 0u : 1u;
                const uint32_t ni = ta ? i : j;
                const unsigned long long nv = ni < L ? dst[kpad((ta ? a0 : b0) + ni)] : 0ull;
                a = ta ? nv : a;
                b = ta ? b : nv;
            }
        }
        if (2 * width <= 32) __syncwarp();
        else __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < K; r++) dst[kpad(tid * K + r)] = v[r];
    __syncthreads();
}

// Lanes of the warp whose 8-bit digit equals this lane's, among the lanes
// with `valid` set: eight ballots (match.any on 32 distinct values is much
// slower on this GPU).
__device__ __forceinline__ unsigned match_digit8(uint32_t d, bool valid) {
    unsigned m = __ballot_sync(0xFFFFFFFFu, valid);
#pragma unroll
    for (int b = 0; b < 8; b++) {
        const bool bit = (d >> b) & 1u;
        const unsigned bb = __ballot_sync(0xFFFFFFFFu, bit);
        m &= bit ? bb : ~bb;
    }
    return m;
}

// Stable LSD radix sort of n 64-bit keys for a CTA of THREADS threads, 8
// bits per pass.  Each warp owns a contiguous range of the input so the
// scatter keeps input order within a digit; passes where every key has the
// same digit are skipped.  `hist` holds THREADS/32 x 256 counters, `red` 33
// slots.  Returns the buffer that holds the sorted keys (a or b).  (Sorting
// on the theta half alone and ordering ties afterwards does not pay: theta
// carries a quadrant offset of 2^16, so it has 7 fractional bits there and
// long runs of equal values.)
template <uint32_t THREADS>
__device__ __forceinline__ unsigned long long* block_radix_sort_u64(unsigned long long* a, unsigned long long* b,
                                                                   uint32_t n, uint32_t* hist, uint32_t* red,
                                                                   uint32_t* s_flag) {
    constexpr uint32_t W = THREADS / 32;
    constexpr uint32_t PER = W * 256 / THREADS;  // scan entries per thread
    const uint32_t w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lo = (uint32_t)((unsigned long long)n * w / W), hi = (uint32_t)((unsigned long long)n * (w + 1) / W);
    for (int pass = 0; pass < 8; pass++) {
        const int sh = pass * 8;
        __syncthreads();  // every thread is done with the previous pass's flag and counters
        for (uint32_t i = threadIdx.x; i < W * 256; i += THREADS) hist[i] = 0;
        if (threadIdx.x == 0) *s_flag = 0;
        __syncthreads();
        // warp-aggregated counts: lanes with equal digits add once (keys of
        // one cluster share their high digits, which would serialise)
        for (uint32_t base = lo; base < hi; base += 32) {
            const uint32_t i = base + lane;
            const bool v = i < hi;
            const uint32_t d = v ? (uint32_t)((a[i] >> sh) & 255) : 0u;
            const unsigned m = match_digit8(d, v);
            if (v && (int)lane == __ffs(m) - 1) hist[w * 256 + d] += (uint32_t)__popc(m);
            __syncwarp();
        }
        __syncthreads();
        for (uint32_t d = threadIdx.x; d < 256; d += THREADS) {
            uint32_t t = 0;
#pragma unroll
            for (uint32_t ww = 0; ww < W; ww++) t += hist[ww * 256 + d];
            if (t == n) *s_flag = 1;  // all keys share this digit: the pass is the identity
        }
        __syncthreads();
        if (*s_flag) continue;
        // exclusive scan in (digit, warp) order; PER consecutive entries per thread
        uint32_t vals[PER], sum = 0;
        const uint32_t L0 = threadIdx.x * PER;
#pragma unroll
        for (uint32_t e = 0; e < PER; e++) {
            const uint32_t L = L0 + e, d = L / W, ww = L % W;
            vals[e] = hist[ww * 256 + d];
            sum += vals[e];
        }
        uint32_t total;
        uint32_t run = block_exclusive_scan_u32(sum, red, &total);
        __syncthreads();
#pragma unroll
        for (uint32_t e = 0; e < PER; e++) {
            const uint32_t L = L0 + e, d = L / W, ww = L % W;
            hist[ww * 256 + d] = run;
            run += vals[e];
        }
        __syncthreads();
        for (uint32_t base = lo; base < hi; base += 32) {
            const uint32_t i = base + lane;
            const bool v = i < hi;
            const unsigned long long key = v ? a[i] : 0ull;
            const uint32_t d = (uint32_t)((key >> sh) & 255);
            const unsigned m = match_digit8(d, v);
            const uint32_t rank = __popc(m & ((1u << lane) - 1u));
            const uint32_t p = v ? hist[w * 256 + d] : 0u;
            __syncwarp();
            if (v) {
                b[p + rank] = key;
                if ((int)lane == __ffs(m) - 1) hist[w * 256 + d] = p + __popc(m);
            }
            __syncwarp();
        }
        __syncthreads();
        unsigned long long* t = a;
        a = b;
        b = t;
    }
    return a;
}

}  // namespace atag
