// k_decode.cu — reading tags: each quad's bit grid matched against a code
// family that the caller describes the way the AprilTag library describes
// its families (bits at per-bit cell coordinates).
//
// The reference hands each quad to the AprilTag library's quad_decode_task
// with tag36h11 and the detector defaults plus quad_decimate = 1
// (src/quad_decoding.cpp:46-75).  The library is not in the reference tree;
// this kernel follows its published decoding algorithm (Olson 2011; Wang &
// Olson 2016; Krogius, Haggenmiller & Olson 2019) with its documented
// defaults (edge refinement on, decode sharpening 0.25):
//   1. edge refinement: per edge, max(16, |edge| / 8) points along it; at
//      each, quarter-pixel positions -r .. r along the outward normal
//      (r = quad_decimate + 1), the grey step between the pixels one pixel
//      either side (truncated coordinates - 0.5) weighted by its square
//      where it rises outward, gives the edge's offset; a line through the
//      offset points; corners at the intersections of adjacent lines
//      (kept when the 2x2 determinant is at most 1e-3);
//   2. homography of the tag square [-1, 1]^2 onto the quad (closed form,
//      Heckbert 1989);
//   3. grey models: least-squares planes over the white ring just outside
//      the black border and over the border, nearest-pixel samples, one per
//      cell along each side; rejected when white minus black at the centre
//      is below min_contrast;
//   4. each bit: bilinear sample at its cell centre (pixel centres at
//      +0.5) minus the models' mean, on a total_width^2 grid, sharpened by
//      decode_sharpening times the 4-neighbour Laplacian; bit = value > 0;
//   5. decision margin = min(mean value of the white bits, mean magnitude
//      of the black bits), counts starting at 1;
//   6. the code and quarter turn with the smallest Hamming distance
//      (ties: fewer turns, lower index), accepted at most max_hamming with a
//      non-negative decision margin.
// Beyond the library: a quad wound the other way is read with corners 0, 3,
// 2, 1 (flagged); the refinement's normal points outward by the quad's
// signed area; a projection behind the camera (z <= 0) marks the quad
// degenerate.
//
// One warp per quad, FP64 throughout: lanes take the refinement's points,
// the grey-model samples, the bits, the grid cells and the codes.
#include <vector>

#include "atag_internal.h"
#include "atag_kernels.cuh"

namespace atag {
namespace {

constexpr int DECODE_WARPS = 4;
constexpr int MAX_TW = 16;  // total_width limit: the value grid lives in shared memory

struct FamilyDesc {
    int8_t bit_x[64], bit_y[64];
    uint8_t perm[64];  // one quarter turn: bit i takes bit perm[i]
    int nbits, width_at_border, total_width, reversed_border;
    uint32_t n_codes, max_hamming;
};

struct DecodeParams {
    double sharpening, min_contrast;
    int refine, quad_decimate;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

struct Homography {
    double a, b, c, d, e, f, g, h;
    bool ok;
};

__device__ __forceinline__ Homography make_homography(const double* px, const double* py) {
    Homography H;
    const double sx = px[0] - px[1] + px[2] - px[3], sy = py[0] - py[1] + py[2] - py[3];
    const double dx1 = px[1] - px[2], dx2 = px[3] - px[2], dy1 = py[1] - py[2], dy2 = py[3] - py[2];
    const double den = dx1 * dy2 - dx2 * dy1;
    const double ref = fabs(dx1) + fabs(dx2) + fabs(dy1) + fabs(dy2);
    H.ok = fabs(den) > 1e-12 * ref * ref;
    if (!H.ok) return H;
    H.g = (sx * dy2 - dx2 * sy) / den;
    H.h = (dx1 * sy - sx * dy1) / den;
    H.a = px[1] - px[0] + H.g * px[1];
    H.b = px[3] - px[0] + H.h * px[3];
    H.c = px[0];
    H.d = py[1] - py[0] + H.g * py[1];
    H.e = py[3] - py[0] + H.h * py[3];
    H.f = py[0];
    return H;
}

// tag coordinates -> pixel; false behind the camera
__device__ __forceinline__ bool project(const Homography& H, double tx, double ty, double* x, double* y) {
    const double u = 0.5 * (tx + 1.0), v = 0.5 * (ty + 1.0);
    const double z = H.g * u + H.h * v + 1.0;
    if (!(z > 0.0)) return false;
    *x = (H.a * u + H.b * v + H.c) / z;
    *y = (H.d * u + H.e * v + H.f) / z;
    return true;
}

__device__ __forceinline__ double det3(double a00, double a01, double a02, double a10, double a11, double a12,
                                       double a20, double a21, double a22) {
    return a00 * (a11 * a22 - a12 * a21) - a01 * (a10 * a22 - a12 * a20) + a02 * (a10 * a21 - a11 * a20);
}

// least-squares plane from the sums of x^2, xy, x, y^2, y, n and of xv, yv, v
struct Plane {
    double c0, c1, c2;
    bool ok;
};
__device__ __forceinline__ Plane solve_plane(const double* s) {
    // s: xx, xy, x, yy, y, n, xv, yv, v
    const double A00 = s[0], A01 = s[1], A02 = s[2], A11 = s[3], A12 = s[4], A22 = s[5];
    const double B0 = s[6], B1 = s[7], B2 = s[8];
    Plane P;
    const double d = det3(A00, A01, A02, A01, A11, A12, A02, A12, A22);
    P.ok = s[5] >= 3.0 && fabs(d) > 1e-12;
    if (!P.ok) return P;
    P.c0 = det3(B0, A01, A02, B1, A11, A12, B2, A12, A22) / d;
    P.c1 = det3(A00, B0, A02, A01, B1, A12, A02, B2, A22) / d;
    P.c2 = det3(A00, A01, B0, A01, A11, B1, A02, A12, B2) / d;
    return P;
}

__device__ __forceinline__ double value_for_pixel(const uint8_t* __restrict__ img, int w, int h, size_t pitch,
                                                  double px, double py) {
    const double fx = floor(px - 0.5), cx = ceil(px - 0.5), fy = floor(py - 0.5), cy = ceil(py - 0.5);
    if (fx < 0.0 || cx >= (double)w || fy < 0.0 || cy >= (double)h) return -1.0;
    const int x1 = (int)fx, x2 = (int)cx, y1 = (int)fy, y2 = (int)cy;
    const double x = px - 0.5 - fx, y = py - 0.5 - fy;
    const double v1 = img[(size_t)y1 * pitch + x1], v2 = img[(size_t)y1 * pitch + x2];
    const double v3 = img[(size_t)y2 * pitch + x1], v4 = img[(size_t)y2 * pitch + x2];
    return v1 * (1 - x) * (1 - y) + v2 * x * (1 - y) + v3 * (1 - x) * y + v4 * x * y;
}

// C's conversion of a double to int (toward zero), as a double-range test
__device__ __forceinline__ bool trunc_in(double v, int n, int* out) {
    const double t = trunc(v);
    if (!(t >= 0.0 && t < (double)n)) return false;
    *out = (int)t;
    return true;
}

// Step 1, lanes over the refinement points of each edge.
__device__ void refine_edges(const uint8_t* __restrict__ img, int w, int h, size_t pitch, double* px, double* py,
                             bool reversed, int quad_decimate) {
    const int lane = threadIdx.x & 31;
    double L[4][4];
    bool valid[4];
    for (int e = 0; e < 4; e++) {
        const int a = e, b = (e + 1) & 3;
        double nx = py[b] - py[a], ny = -(px[b] - px[a]);
        const double mag = sqrt(nx * nx + ny * ny);
        nx /= mag;
        ny /= mag;
        if (reversed) {
            nx = -nx;
            ny = -ny;
        }
        const int nsamples = max(16, (int)(mag / 8.0));
        const double rng = (double)(quad_decimate + 1);
        const int nsteps = 8 * (quad_decimate + 1) + 1;
        double m[6] = {0, 0, 0, 0, 0, 0};  // x, y, xx, xy, yy, n
        for (int s = lane; s < nsamples; s += 32) {
            const double alpha = (1.0 + s) / (nsamples + 1);
            const double x0 = alpha * px[a] + (1.0 - alpha) * px[b];
            const double y0 = alpha * py[a] + (1.0 - alpha) * py[b];
            double Mn = 0.0, Mc = 0.0;
            for (int k = 0; k < nsteps; k++) {
                const double n = -rng + 0.25 * k;
                int x1, y1, x2, y2;
                if (!trunc_in(x0 + (n + 1.0) * nx - 0.5, w, &x1) || !trunc_in(y0 + (n + 1.0) * ny - 0.5, h, &y1))
                    continue;
                if (!trunc_in(x0 + (n - 1.0) * nx - 0.5, w, &x2) || !trunc_in(y0 + (n - 1.0) * ny - 0.5, h, &y2))
                    continue;
                const double g1 = img[(size_t)y1 * pitch + x1], g2 = img[(size_t)y2 * pitch + x2];
                if (g1 < g2) continue;
                const double wgt = (g2 - g1) * (g2 - g1);
                Mn += wgt * n;
                Mc += wgt;
            }
            if (Mc == 0.0) continue;
            const double n0 = Mn / Mc;
            const double bx = x0 + n0 * nx, by = y0 + n0 * ny;
            m[0] += bx;
            m[1] += by;
            m[2] += bx * bx;
            m[3] += bx * by;
            m[4] += by * by;
            m[5] += 1.0;
        }
#pragma unroll
        for (int k = 0; k < 6; k++) m[k] = warp_sum(m[k]);
        valid[e] = m[5] > 0.0;
        if (valid[e]) {
            const double N = m[5], Ex = m[0] / N, Ey = m[1] / N;
            const double Cxx = m[2] / N - Ex * Ex, Cxy = m[3] / N - Ex * Ey, Cyy = m[4] / N - Ey * Ey;
            const double th = 0.5 * atan2(-2.0 * Cxy, Cyy - Cxx);
            L[e][0] = Ex;
            L[e][1] = Ey;
            L[e][2] = cos(th);
            L[e][3] = sin(th);
        }
    }
    double qx[4], qy[4];
    for (int i = 0; i < 4; i++) {
        qx[i] = px[i];
        qy[i] = py[i];
    }
    for (int i = 0; i < 4; i++) {
        const int j = (i + 1) & 3;
        if (!valid[i] || !valid[j]) continue;
        const double A00 = L[i][3], A01 = -L[j][3], A10 = -L[i][2], A11 = L[j][2];
        const double B0 = L[j][0] - L[i][0], B1 = L[j][1] - L[i][1];
        const double det = A00 * A11 - A10 * A01;
        if (fabs(det) > 0.001) {
            const double L0 = (A11 * B0 - A01 * B1) / det;
            qx[j] = L[i][0] + L0 * A00;
            qy[j] = L[i][1] + L0 * A10;
        }
    }
    for (int i = 0; i < 4; i++) {
        px[i] = qx[i];
        py[i] = qy[i];
    }
}

__device__ __forceinline__ unsigned long long rotate_code(unsigned long long c, const FamilyDesc& F) {
    const int lane = threadIdx.x & 31, n = F.nbits;
    unsigned long long out = 0;
    for (int base = 0; base < n; base += 32) {
        const int i = base + lane;
        const bool bit = i < n && ((c >> (n - 1 - F.perm[i < n ? i : 0])) & 1ull);
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, bit);
        for (unsigned m = bal; m; m &= m - 1) {
            const int k = base + __ffs(m) - 1;
            out |= 1ull << (n - 1 - k);
        }
    }
    return out;
}

__global__ void __launch_bounds__(32 * DECODE_WARPS) k_decode_quads(
    const uint8_t* __restrict__ img, int w, int h, size_t pitch, const uint8_t* __restrict__ quads, size_t stride,
    uint32_t n, const unsigned long long* __restrict__ codes, const __grid_constant__ FamilyDesc F,
    DecodeParams prm, atag_decoded* __restrict__ out) {
    __shared__ double s_vals[DECODE_WARPS][MAX_TW * MAX_TW];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const uint32_t q = blockIdx.x * DECODE_WARPS + wid;
    if (q >= n) return;  // warp-uniform
    double* vals = s_vals[wid];
    const float* cf = reinterpret_cast<const float*>(quads + (size_t)q * stride);
    double px[4], py[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        px[i] = (double)cf[2 * i];
        py[i] = (double)cf[2 * i + 1];
    }
    atag_decoded R;
    memset(&R, 0, sizeof R);
    R.id = -1;
    R.hamming = 0xFFFFFFFFu;
    double area2 = 0.0;
#pragma unroll
    for (int i = 0; i < 4; i++) area2 += px[i] * py[(i + 1) & 3] - px[(i + 1) & 3] * py[i];
    if (area2 < 0.0) {
        double t = px[1];
        px[1] = px[3];
        px[3] = t;
        t = py[1];
        py[1] = py[3];
        py[3] = t;
        R.status |= ATAG_DECODE_REORDERED;
    }
    auto finish = [&]() {
        if (lane == 0) {
#pragma unroll
            for (int i = 0; i < 4; i++) {
                R.corners[i][0] = (float)px[i];
                R.corners[i][1] = (float)py[i];
            }
            out[q] = R;
        }
    };
    Homography H = make_homography(px, py);
    if (!H.ok) {
        R.status |= ATAG_DECODE_DEGENERATE;
        finish();
        return;
    }
    if (prm.refine) {
        refine_edges(img, w, h, pitch, px, py, F.reversed_border != 0, prm.quad_decimate);
        H = make_homography(px, py);
        if (!H.ok) {
            R.status |= ATAG_DECODE_DEGENERATE;
            finish();
            return;
        }
    }
    // 3. grey models: 8 sides x W samples, lanes over them
    const int Wb = F.width_at_border, T = F.total_width;
    double sw[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0}, sb[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool behind = false;
    for (int k = lane; k < 8 * Wb; k += 32) {
        const int pat = k / Wb, i = k % Wb;
        // (x0, y0, dx, dy, white) of the eight sides
        const double x0 = pat == 0 ? -0.5 : pat == 1 ? 0.5 : pat == 2 ? Wb + 0.5 : pat == 3 ? Wb - 0.5 : 0.5;
        const double y0 = pat < 4 ? 0.5 : pat == 4 ? -0.5 : pat == 5 ? 0.5 : pat == 6 ? Wb + 0.5 : Wb - 0.5;
        const bool vertical = pat < 4, white = (pat & 1) == 0;
        const double tx = 2.0 * ((x0 + (vertical ? 0 : i)) / Wb - 0.5);
        const double ty = 2.0 * ((y0 + (vertical ? i : 0)) / Wb - 0.5);
        double x, y;
        if (!project(H, tx, ty, &x, &y)) {
            behind = true;
            continue;
        }
        const double tix = trunc(x), tiy = trunc(y);
        if (tix < 0.0 || tiy < 0.0 || tix >= (double)w || tiy >= (double)h) continue;
        const double v = img[(size_t)(int)tiy * pitch + (int)tix];
        double* s = white ? sw : sb;
        s[0] += tx * tx; s[1] += tx * ty; s[2] += tx; s[3] += ty * ty; s[4] += ty; s[5] += 1.0;
        s[6] += tx * v; s[7] += ty * v; s[8] += v;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) {
        sw[k] = warp_sum(sw[k]);
        sb[k] = warp_sum(sb[k]);
    }
    if (__any_sync(0xFFFFFFFFu, behind)) {
        R.status |= ATAG_DECODE_DEGENERATE;
        finish();
        return;
    }
    const Plane PW = solve_plane(sw), PB = solve_plane(sb);
    if (!PW.ok || !PB.ok) {
        R.status |= ATAG_DECODE_LOW_CONTRAST;
        finish();
        return;
    }
    R.white = (float)PW.c2;
    R.black = (float)PB.c2;
    const double contrast = F.reversed_border ? PB.c2 - PW.c2 : PW.c2 - PB.c2;
    if (!(contrast >= prm.min_contrast)) {
        R.status |= ATAG_DECODE_LOW_CONTRAST;
        finish();
        return;
    }
    // 4. bit values on the total_width grid
    const int m = (Wb - T) / 2;
    for (int k = lane; k < T * T; k += 32) vals[k] = 0.0;
    __syncwarp();
    for (int i = lane; i < F.nbits; i += 32) {
        const int bx = F.bit_x[i], by = F.bit_y[i];
        const double tx = 2.0 * ((bx + 0.5) / Wb - 0.5), ty = 2.0 * ((by + 0.5) / Wb - 0.5);
        double x, y;
        if (!project(H, tx, ty, &x, &y)) {
            behind = true;
            continue;
        }
        const double v = value_for_pixel(img, w, h, pitch, x, y);
        if (v == -1.0) continue;
        const double thr = 0.5 * ((PB.c0 * tx + PB.c1 * ty + PB.c2) + (PW.c0 * tx + PW.c1 * ty + PW.c2));
        vals[(by - m) * T + (bx - m)] = v - thr;
    }
    if (__any_sync(0xFFFFFFFFu, behind)) {
        R.status |= ATAG_DECODE_DEGENERATE;
        finish();
        return;
    }
    __syncwarp();
    // sharpening, then the bits and their scores
    double sharp[MAX_TW * MAX_TW / 32];
    for (int k = lane, j = 0; k < T * T; k += 32, j++) {
        const int y = k / T, x = k % T;
        double acc = 4.0 * vals[k];
        if (y > 0) acc -= vals[k - T];
        if (y + 1 < T) acc -= vals[k + T];
        if (x > 0) acc -= vals[k - 1];
        if (x + 1 < T) acc -= vals[k + 1];
        sharp[j] = vals[k] + prm.sharpening * acc;
    }
    __syncwarp();
    for (int k = lane, j = 0; k < T * T; k += 32, j++) vals[k] = sharp[j];
    __syncwarp();
    unsigned long long code = 0;
    double ws = 0.0, bs = 0.0, wn = 0.0, bn = 0.0;
    const int nb = F.nbits;
    for (int base = 0; base < nb; base += 32) {
        const int i = base + lane;
        bool bit = false;
        if (i < nb) {
            const double v = vals[(F.bit_y[i] - m) * T + (F.bit_x[i] - m)];
            bit = v > 0.0;
            if (bit) {
                ws += v;
                wn += 1.0;
            } else {
                bs -= v;
                bn += 1.0;
            }
        }
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, bit);
        for (unsigned mm = bal; mm; mm &= mm - 1) code |= 1ull << (nb - 1 - (base + __ffs(mm) - 1));
    }
    ws = warp_sum(ws);
    bs = warp_sum(bs);
    wn = warp_sum(wn) + 1.0;
    bn = warp_sum(bn) + 1.0;
    const double margin = fmin(ws / wn, bs / bn);
    R.code = code;
    R.decision_margin = (float)margin;
    // 6. nearest code over the four quarter turns: (distance, turns, index)
    unsigned long long best = ~0ull;
    unsigned long long r = code;
    for (int k = 0; k < 4; k++) {
        for (uint32_t i = lane; i < F.n_codes; i += 32) {
            const unsigned long long hd = (unsigned long long)__popcll(r ^ codes[i]);
            const unsigned long long key = (hd << 40) | ((unsigned long long)k << 32) | i;
            best = key < best ? key : best;
        }
        r = rotate_code(r, F);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long v = __shfl_xor_sync(0xFFFFFFFFu, best, o);
        best = v < best ? v : best;
    }
    if (best != ~0ull) {
        R.hamming = (uint32_t)(best >> 40);
        const uint32_t turns = (uint32_t)(best >> 32) & 0xFFu;
        if (R.hamming <= F.max_hamming && margin >= 0.0) {
            R.id = (int32_t)(uint32_t)best;
            R.rotation = turns;
            double rx[4], ry[4];
            for (int i = 0; i < 4; i++) {
                rx[i] = px[(i + turns) & 3];
                ry[i] = py[(i + turns) & 3];
            }
            for (int i = 0; i < 4; i++) {
                px[i] = rx[i];
                py[i] = ry[i];
            }
        }
    }
    finish();
}

}  // namespace
}  // namespace atag

using namespace atag;

extern "C" void atag_decode_params_default(atag_decode_params* p) {
    p->decode_sharpening = 0.25f;
    p->refine_edges = 1;
    p->quad_decimate = 1;
    p->min_contrast = 0.0f;
}

extern "C" atag_status atag_decode_quads(const uint8_t* d_image, size_t width, size_t height, size_t pitch,
                                         const float* d_corners, size_t corner_stride, size_t n_quads,
                                         const atag_tag_family* family, const atag_decode_params* params,
                                         atag_decoded* d_out, atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (!family) return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: null family");
    if (n_quads == 0) return ATAG_OK;
    if (!d_image || !d_corners || !d_out || (family->n_codes && !family->d_codes) || !family->h_bit_x ||
        !family->h_bit_y)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: null pointer");
    if (width < 2 || height < 2 || width > (size_t)INT32_MAX || height > (size_t)INT32_MAX)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: image smaller than 2x2 or too large");
    if (pitch == 0) pitch = width;
    if (pitch < width) return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: pitch below width");
    if (corner_stride < 8 * sizeof(float) || corner_stride % 4)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: corner stride below 32 bytes or not a multiple of 4");
    if (reinterpret_cast<uintptr_t>(d_corners) % 4 || reinterpret_cast<uintptr_t>(d_out) % 8 ||
        reinterpret_cast<uintptr_t>(family->d_codes) % 8)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: misaligned corners, codes or output");
    if (n_quads > (size_t)UINT32_MAX || family->n_codes > (1u << 24))
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: too many quads or codes");
    const int nb = (int)family->nbits, W = (int)family->width_at_border, T = (int)family->total_width;
    if (nb < 1 || nb > 64 || W < 3 || T < 1 || T > MAX_TW || (W - T) % 2 != 0)
        return set_error(ATAG_ERR_INVALID_ARGUMENT,
                         "decode_quads: family needs 1..64 bits, width_at_border >= 3, total_width <= 16 with "
                         "total_width - width_at_border even");
    FamilyDesc F;
    memset(&F, 0, sizeof F);
    F.nbits = nb;
    F.width_at_border = W;
    F.total_width = T;
    F.reversed_border = family->reversed_border ? 1 : 0;
    F.n_codes = family->n_codes;
    F.max_hamming = family->max_hamming;
    const int m = (W - T) / 2;
    // every bit's cell must lie on the grid, be used once, and a quarter turn
    // must carry the bit cells onto bit cells (the families are symmetric)
    std::vector<int> at((size_t)T * T, -1);
    for (int i = 0; i < nb; i++) {
        const int x = family->h_bit_x[i], y = family->h_bit_y[i];
        if (x - m < 0 || x - m >= T || y - m < 0 || y - m >= T || at[(size_t)(y - m) * T + (x - m)] >= 0)
            return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: bit cell off the tag grid or used twice");
        at[(size_t)(y - m) * T + (x - m)] = i;
        F.bit_x[i] = (int8_t)x;
        F.bit_y[i] = (int8_t)y;
    }
    for (int i = 0; i < nb; i++) {
        const int sx = W - 1 - F.bit_y[i], sy = F.bit_x[i];
        const int j = (sx - m >= 0 && sx - m < T && sy - m >= 0 && sy - m < T) ? at[(size_t)(sy - m) * T + (sx - m)] : -1;
        if (j < 0) return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: the bit layout is not symmetric under quarter turns");
        F.perm[i] = (uint8_t)j;
    }
    atag_decode_params p;
    if (params) p = *params; else atag_decode_params_default(&p);
    if (p.quad_decimate < 1 || p.quad_decimate > 8)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: quad_decimate must be 1..8");
    DecodeParams prm{(double)p.decode_sharpening, (double)p.min_contrast, p.refine_edges ? 1 : 0, p.quad_decimate};
    const uint32_t n = (uint32_t)n_quads;
    k_decode_quads<<<(n + DECODE_WARPS - 1) / DECODE_WARPS, 32 * DECODE_WARPS, 0, (cudaStream_t)stream>>>(
        d_image, (int)width, (int)height, pitch, reinterpret_cast<const uint8_t*>(d_corners), corner_stride, n,
        reinterpret_cast<const unsigned long long*>(family->d_codes), F, prm, d_out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ATAG_OK : set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
}
