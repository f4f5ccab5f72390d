// k_decode.cu — reading the bit grid of each quad and matching it against a
// code family supplied by the caller.
//
// The reference hands each quad to the AprilTag library's quad_decode_task
// with the tag36h11 family (src/quad_decoding.cpp:46-128); that library and
// its family tables are not part of the reference tree, so the family is an
// argument here.  Layout of a tag (as the library's families, e.g. 36h11):
// D x D data cells inside a one-cell black border, inside a white quiet
// zone; the detected quad is the outer edge of the black border.
//
// Per quad, one thread:
//   1. a quad wound the other way (negative signed area) is taken in the
//      order 0, 3, 2, 1, so that the grid is read unmirrored;
//   2. the projective map of the unit square onto the quad in closed form
//      (Heckbert 1989); grid cell (r, c) of the (D + 2)-cell square has its
//      centre at ((c + 0.5) / (D + 2), (r + 0.5) / (D + 2));
//   3. bilinear samples (pixel centres at integer coordinates, clamped to
//      the image): black level = mean over the 4 (D + 1) border cells, white
//      level = mean over the 4 (D + 2) cells of the ring just outside;
//      threshold = their mean; fewer than min_contrast grey levels between
//      them: no decode;
//   4. data bit (r, c) = sample > threshold, code bit D^2 - 1 - (D r + c);
//   5. the family code and rotation (0..3 quarter turns of the grid) with
//      the smallest Hamming distance, first code and rotation on ties;
//      accepted at most max_hamming.
#include "atag_internal.h"
#include "atag_kernels.cuh"

namespace atag {
namespace {

constexpr uint32_t DECODE_THREADS = 32;

__device__ __forceinline__ double sample(const uint8_t* __restrict__ img, int w, int h, size_t pitch, double x,
                                         double y) {
    x = fmin(fmax(x, 0.0), (double)(w - 1));
    y = fmin(fmax(y, 0.0), (double)(h - 1));
    int x0 = (int)floor(x), y0 = (int)floor(y);
    x0 = min(x0, w - 2);
    y0 = min(y0, h - 2);
    const double fx = x - x0, fy = y - y0;
    const uint8_t* p = img + (size_t)y0 * pitch + x0;
    const double a = p[0], b = p[1], c = p[pitch], d = p[pitch + 1];
    return (1.0 - fy) * ((1.0 - fx) * a + fx * b) + fy * ((1.0 - fx) * c + fx * d);
}

// a quarter turn of a D x D bit grid (bit D^2 - 1 - (D r + c) is cell r, c):
// cell (r, c) of the result is cell (D - 1 - c, r) of the input
__device__ __forceinline__ unsigned long long rotate90(unsigned long long v, int D) {
    unsigned long long o = 0;
    const int n = D * D;
    for (int r = 0; r < D; r++)
        for (int c = 0; c < D; c++) {
            const int src = (D - 1 - c) * D + r;
            if ((v >> (n - 1 - src)) & 1ull) o |= 1ull << (n - 1 - (r * D + c));
        }
    return o;
}

__global__ void __launch_bounds__(DECODE_THREADS) k_decode_quads(const uint8_t* __restrict__ img, int w, int h,
                                                                 size_t pitch, const uint8_t* __restrict__ quads,
                                                                 size_t stride, uint32_t n,
                                                                 const unsigned long long* __restrict__ codes,
                                                                 uint32_t n_codes, int D, uint32_t max_hamming,
                                                                 double min_contrast, atag_decoded* __restrict__ out) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float* cf = reinterpret_cast<const float*>(quads + (size_t)q * stride);
    double px[4], py[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        px[i] = (double)cf[2 * i];
        py[i] = (double)cf[2 * i + 1];
    }
    atag_decoded R{};
    R.id = -1;
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
    const double sx = px[0] - px[1] + px[2] - px[3], sy = py[0] - py[1] + py[2] - py[3];
    const double dx1 = px[1] - px[2], dx2 = px[3] - px[2], dy1 = py[1] - py[2], dy2 = py[3] - py[2];
    const double den = dx1 * dy2 - dx2 * dy1;
    const double ref = fabs(dx1) + fabs(dx2) + fabs(dy1) + fabs(dy2);
    if (!(fabs(den) > 1e-12 * ref * ref)) {
        R.status |= ATAG_DECODE_DEGENERATE;
        out[q] = R;
        return;
    }
    const double g = (sx * dy2 - dx2 * sy) / den, hh = (dx1 * sy - sx * dy1) / den;
    const double a = px[1] - px[0] + g * px[1], b = px[3] - px[0] + hh * px[3], c = px[0];
    const double d = py[1] - py[0] + g * py[1], e = py[3] - py[0] + hh * py[3], f = py[0];
    const double cells = (double)(D + 2);
    auto at = [&](double cc, double rr) {  // grid cell coordinates (column, row) -> sample
        const double u = cc / cells, v = rr / cells;
        const double z = g * u + hh * v + 1.0;
        return sample(img, w, h, pitch, (a * u + b * v + c) / z, (d * u + e * v + f) / z);
    };
    // black border cells and the white ring just outside, walked side by side
    double black = 0.0, white = 0.0;
    for (int k = 0; k < D + 1; k++) {
        const double s = k + 0.5, t = D + 2 - k - 0.5;
        black += at(s, 0.5) + at(D + 1.5, s) + at(t, D + 1.5) + at(0.5, t);
    }
    for (int k = 0; k < D + 2; k++) {
        const double s = k + 0.5, t = D + 2 - k - 0.5;
        white += at(s, -0.5) + at(D + 2.5, s) + at(t, D + 2.5) + at(-0.5, t);
    }
    black /= 4.0 * (D + 1);
    white /= 4.0 * (D + 2);
    R.black = (float)black;
    R.white = (float)white;
    if (!(white - black >= min_contrast)) {
        R.status |= ATAG_DECODE_LOW_CONTRAST;
        out[q] = R;
        return;
    }
    const double thr = 0.5 * (black + white);
    const int nb = D * D;
    unsigned long long obs = 0;
    double margin = 1e300;
    for (int r = 0; r < D; r++)
        for (int cc = 0; cc < D; cc++) {
            const double v = at(cc + 1.5, r + 1.5);
            if (v > thr) obs |= 1ull << (nb - 1 - (r * D + cc));
            margin = fmin(margin, fabs(v - thr));
        }
    R.code = obs;
    R.margin = (float)margin;
    uint32_t best = 0xFFFFFFFFu;
    int best_id = -1, best_rot = 0;
    unsigned long long rot = obs;
    for (int k = 0; k < 4; k++) {
        for (uint32_t i = 0; i < n_codes; i++) {
            const uint32_t hd = (uint32_t)__popcll(rot ^ codes[i]);
            if (hd < best) {
                best = hd;
                best_id = (int)i;
                best_rot = k;
            }
        }
        rot = rotate90(rot, D);
    }
    R.hamming = best;
    if (best_id >= 0 && best <= max_hamming) {
        R.id = best_id;
        R.rotation = (uint32_t)best_rot;
    }
    out[q] = R;
}

}  // namespace
}  // namespace atag

using namespace atag;

extern "C" atag_status atag_decode_quads(const uint8_t* d_image, size_t width, size_t height, size_t pitch,
                                         const float* d_corners, size_t corner_stride, size_t n_quads,
                                         const uint64_t* d_codes, size_t n_codes, uint32_t data_side,
                                         uint32_t max_hamming, double min_contrast, atag_decoded* d_out,
                                         atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (n_quads == 0) return ATAG_OK;
    if (!d_image || !d_corners || !d_out || (n_codes && !d_codes))
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: null pointer");
    if (width < 2 || height < 2 || width > (size_t)INT32_MAX || height > (size_t)INT32_MAX)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: image smaller than 2x2 or too large");
    if (pitch == 0) pitch = width;
    if (pitch < width) return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: pitch below width");
    if (corner_stride < 8 * sizeof(float) || corner_stride % 4)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: corner stride below 32 bytes or not a multiple of 4");
    if (reinterpret_cast<uintptr_t>(d_corners) % 4 || reinterpret_cast<uintptr_t>(d_out) % 8 ||
        reinterpret_cast<uintptr_t>(d_codes) % 8)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: misaligned corners, codes or output");
    if (data_side < 2 || data_side > 8)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: data_side must be 2..8 (at most 64 bits)");
    if (n_quads > (size_t)UINT32_MAX || n_codes > (size_t)UINT32_MAX)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "decode_quads: too many quads or codes");
    const uint32_t n = (uint32_t)n_quads;
    k_decode_quads<<<(n + DECODE_THREADS - 1) / DECODE_THREADS, DECODE_THREADS, 0, (cudaStream_t)stream>>>(
        d_image, (int)width, (int)height, pitch, reinterpret_cast<const uint8_t*>(d_corners), corner_stride, n,
        reinterpret_cast<const unsigned long long*>(d_codes), (uint32_t)n_codes, (int)data_side, max_hamming,
        min_contrast, d_out);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ATAG_OK : set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
}
