// k_pose.cu — tag pose from quad corners (a downstream consumer of the
// detector's quads; the reference stops at the corners of
// process_fitted_quads, src/main.cpp:1035-1162, and has no pose stage).
//
// Per quad, one thread, FP64 throughout:
//   1. corners to normalised camera coordinates, ((x - cx) / fx, (y - cy) / fy);
//      corner i is the image of the tag-plane point (s/2) c_i,
//      c = (-1,-1), (1,-1), (1,1), (-1,1); a quad wound the other way (negative
//      signed area in pixel coordinates) is taken in the order 0, 3, 2, 1;
//   2. the projective map of the unit square onto the quad in closed form
//      (Heckbert, "Fundamentals of Texture Mapping and Image Warping", 1989:
//      square-to-quadrilateral mapping), composed with the map of the tag
//      plane onto the unit square, gives H ~ [r1 r2 t];
//   3. scale from the mean norm of the first two columns, sign such that the
//      tag is in front of the camera, R0 = [r1 r2 r1 x r2] made orthogonal by
//      the Newton iteration for the polar factor, X <- (X + X^-T) / 2
//      (Higham, "Computing the polar decomposition", 1986);
//   4. Levenberg-Marquardt on the pixel reprojection error of the four
//      corners over the six pose parameters (rotation updated as
//      R <- exp([w]x) R): normal equations with the diagonal scaled by
//      1 + mu, mu from 1e-9, times 10 after a step that does not lower the
//      error (dropped; stop above 1e9), divided by 10 after one that does
//      (kept); up to max_iterations trials.
#include "atag_internal.h"
#include "atag_kernels.cuh"

namespace atag {
namespace {

struct M3 {
    double m[9];  // row-major
};

__device__ __forceinline__ double det3(const M3& a) {
    const double* m = a.m;
    return m[0] * (m[4] * m[8] - m[5] * m[7]) - m[1] * (m[3] * m[8] - m[5] * m[6]) +
           m[2] * (m[3] * m[7] - m[4] * m[6]);
}

// polar factor of a 3x3 matrix with positive determinant
__device__ M3 orthogonalise(M3 x) {
    for (int it = 0; it < 32; it++) {
        const double* m = x.m;
        // cofactor matrix / det = inverse transpose
        M3 c;
        c.m[0] = m[4] * m[8] - m[5] * m[7];
        c.m[1] = m[5] * m[6] - m[3] * m[8];
        c.m[2] = m[3] * m[7] - m[4] * m[6];
        c.m[3] = m[2] * m[7] - m[1] * m[8];
        c.m[4] = m[0] * m[8] - m[2] * m[6];
        c.m[5] = m[1] * m[6] - m[0] * m[7];
        c.m[6] = m[1] * m[5] - m[2] * m[4];
        c.m[7] = m[2] * m[3] - m[0] * m[5];
        c.m[8] = m[0] * m[4] - m[1] * m[3];
        const double id = 1.0 / (m[0] * c.m[0] + m[1] * c.m[1] + m[2] * c.m[2]);
        double change = 0.0;
#pragma unroll
        for (int k = 0; k < 9; k++) {
            const double v = 0.5 * (m[k] + c.m[k] * id);
            change = fmax(change, fabs(v - m[k]));
            x.m[k] = v;
        }
        if (change < 1e-15) break;
    }
    return x;
}

__device__ __forceinline__ M3 matmul(const M3& a, const M3& b) {
    M3 r;
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
        for (int j = 0; j < 3; j++)
            r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}

// exp([w]x) by Rodrigues' formula
__device__ M3 so3_exp(double wx, double wy, double wz) {
    const double t2 = wx * wx + wy * wy + wz * wz, t = sqrt(t2);
    double a, b;
    if (t < 1e-8) {
        a = 1.0 - t2 / 6.0;
        b = 0.5 - t2 / 24.0;
    } else {
        a = sin(t) / t;
        b = (1.0 - cos(t)) / t2;
    }
    M3 r;
    r.m[0] = 1.0 - b * (wy * wy + wz * wz);
    r.m[1] = -a * wz + b * wx * wy;
    r.m[2] = a * wy + b * wx * wz;
    r.m[3] = a * wz + b * wx * wy;
    r.m[4] = 1.0 - b * (wx * wx + wz * wz);
    r.m[5] = -a * wx + b * wy * wz;
    r.m[6] = -a * wy + b * wx * wz;
    r.m[7] = a * wx + b * wy * wz;
    r.m[8] = 1.0 - b * (wx * wx + wy * wy);
    return r;
}

struct Cam {
    double fx, fy, cx, cy;
};

// sum of squared pixel reprojection errors of the four corners; false if a
// corner is not in front of the camera
__device__ bool reproj_cost(const M3& R, const double t[3], const double ox[4], const double oy[4],
                            const double px[4], const double py[4], const Cam& c, double* cost) {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const double X = R.m[0] * ox[i] + R.m[1] * oy[i] + t[0];
        const double Y = R.m[3] * ox[i] + R.m[4] * oy[i] + t[1];
        const double Z = R.m[6] * ox[i] + R.m[7] * oy[i] + t[2];
        if (!(Z > 0.0)) return false;
        const double ex = c.fx * X / Z + c.cx - px[i], ey = c.fy * Y / Z + c.cy - py[i];
        s += ex * ex + ey * ey;
    }
    *cost = s;
    return true;
}

// Solves the symmetric positive definite 6x6 system A x = b (A packed
// row-major, full) by Cholesky; false if A is not positive definite.
__device__ bool solve6(double A[36], double b[6], double x[6]) {
    double inv[6];  // reciprocals of L's diagonal
#pragma unroll
    for (int j = 0; j < 6; j++) {
        double d = A[6 * j + j];
#pragma unroll
        for (int k = 0; k < j; k++) d -= A[6 * j + k] * A[6 * j + k];
        if (!(d > 0.0)) return false;
        inv[j] = 1.0 / sqrt(d);
#pragma unroll
        for (int i = j + 1; i < 6; i++) {
            double v = A[6 * i + j];
#pragma unroll
            for (int k = 0; k < j; k++) v -= A[6 * i + k] * A[6 * j + k];
            A[6 * i + j] = v * inv[j];
        }
    }
#pragma unroll
    for (int i = 0; i < 6; i++) {
        double v = b[i];
#pragma unroll
        for (int k = 0; k < i; k++) v -= A[6 * i + k] * x[k];
        x[i] = v * inv[i];
    }
#pragma unroll
    for (int i = 5; i >= 0; i--) {
        double v = x[i];
#pragma unroll
        for (int k = i + 1; k < 6; k++) v -= A[6 * k + i] * x[k];
        x[i] = v * inv[i];
    }
    return true;
}

constexpr double POSE_DAMPING = 1e-9, POSE_MAX_DAMPING = 1e9;

// One thread per quad in 32-thread CTAs: the FP64 work of a few thousand
// quads spreads over every SM rather than filling a few.
constexpr uint32_t POSE_THREADS = 32;

__global__ void __launch_bounds__(POSE_THREADS) k_estimate_pose(const uint8_t* __restrict__ corners, size_t stride,
                                                       uint32_t n, Cam c, double tag_size, uint32_t max_iter,
                                                       atag_pose* __restrict__ out) {
    const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const float* cf = reinterpret_cast<const float*>(corners + (size_t)q * stride);
    double px[4], py[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        px[i] = (double)cf[2 * i];
        py[i] = (double)cf[2 * i + 1];
    }
    atag_pose P{};
    // winding: positive shoelace area in pixel coordinates is the tag order
    double area2 = 0.0;
#pragma unroll
    for (int i = 0; i < 4; i++) area2 += px[i] * py[(i + 1) & 3] - px[(i + 1) & 3] * py[i];
    if (area2 < 0.0) {
        double tx = px[1], ty = py[1];
        px[1] = px[3]; py[1] = py[3];
        px[3] = tx; py[3] = ty;
        P.status |= ATAG_POSE_REORDERED;
    }
    // normalised coordinates
    double nx[4], ny[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        nx[i] = (px[i] - c.cx) / c.fx;
        ny[i] = (py[i] - c.cy) / c.fy;
    }
    // unit square (0,0), (1,0), (1,1), (0,1) -> corners 0..3
    const double sx = nx[0] - nx[1] + nx[2] - nx[3], sy = ny[0] - ny[1] + ny[2] - ny[3];
    const double dx1 = nx[1] - nx[2], dx2 = nx[3] - nx[2], dy1 = ny[1] - ny[2], dy2 = ny[3] - ny[2];
    const double den = dx1 * dy2 - dx2 * dy1;
    const double scale_ref = fabs(dx1) + fabs(dx2) + fabs(dy1) + fabs(dy2);
    if (!(fabs(den) > 1e-14 * scale_ref * scale_ref) || !(tag_size > 0.0)) {
        P.status |= ATAG_POSE_DEGENERATE;
        out[q] = P;
        return;
    }
    const double g = (sx * dy2 - dx2 * sy) / den, h = (dx1 * sy - sx * dy1) / den;
    M3 Hu;  // columns: u, v, 1
    Hu.m[0] = nx[1] - nx[0] + g * nx[1];
    Hu.m[1] = nx[3] - nx[0] + h * nx[3];
    Hu.m[2] = nx[0];
    Hu.m[3] = ny[1] - ny[0] + g * ny[1];
    Hu.m[4] = ny[3] - ny[0] + h * ny[3];
    Hu.m[5] = ny[0];
    Hu.m[6] = g;
    Hu.m[7] = h;
    Hu.m[8] = 1.0;
    // tag plane (X, Y) -> unit square: u = X / s + 1/2, v = Y / s + 1/2
    double h1[3], h2[3], h3[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        h1[r] = Hu.m[3 * r] / tag_size;
        h2[r] = Hu.m[3 * r + 1] / tag_size;
        h3[r] = 0.5 * Hu.m[3 * r] + 0.5 * Hu.m[3 * r + 1] + Hu.m[3 * r + 2];
    }
    double lam = 0.5 * (sqrt(h1[0] * h1[0] + h1[1] * h1[1] + h1[2] * h1[2]) +
                        sqrt(h2[0] * h2[0] + h2[1] * h2[1] + h2[2] * h2[2]));
    if (!(lam > 0.0)) {
        P.status |= ATAG_POSE_DEGENERATE;
        out[q] = P;
        return;
    }
    if (h3[2] < 0.0) lam = -lam;
    M3 R;
    double t[3];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        R.m[3 * r] = h1[r] / lam;
        R.m[3 * r + 1] = h2[r] / lam;
        t[r] = h3[r] / lam;
    }
    R.m[2] = R.m[3] * R.m[7] - R.m[6] * R.m[4];
    R.m[5] = R.m[6] * R.m[1] - R.m[0] * R.m[7];
    R.m[8] = R.m[0] * R.m[4] - R.m[3] * R.m[1];
    if (!(det3(R) > 0.0)) {
        P.status |= ATAG_POSE_DEGENERATE;
        out[q] = P;
        return;
    }
    R = orthogonalise(R);

    const double hs = 0.5 * tag_size;
    const double ox[4] = {-hs, hs, hs, -hs}, oy[4] = {-hs, -hs, hs, hs};
    double cost;
    if (!reproj_cost(R, t, ox, oy, px, py, c, &cost)) {
        P.status |= ATAG_POSE_DEGENERATE;
        out[q] = P;
        return;
    }
    uint32_t it = 0;
    double mu = POSE_DAMPING;
    for (uint32_t trial = 0; trial < max_iter; trial++) {
        double A[36], b[6];
#pragma unroll
        for (int k = 0; k < 36; k++) A[k] = 0.0;
#pragma unroll
        for (int k = 0; k < 6; k++) b[k] = 0.0;
#pragma unroll
        for (int i = 0; i < 4; i++) {
            const double a0 = R.m[0] * ox[i] + R.m[1] * oy[i], a1 = R.m[3] * ox[i] + R.m[4] * oy[i],
                         a2 = R.m[6] * ox[i] + R.m[7] * oy[i];
            const double X = a0 + t[0], Y = a1 + t[1], Z = a2 + t[2];
            const double iz = 1.0 / Z;
            const double ex = c.fx * X * iz + c.cx - px[i], ey = c.fy * Y * iz + c.cy - py[i];
            // d(pixel)/dP
            const double ux = c.fx * iz, uz = -c.fx * X * iz * iz, vy = c.fy * iz, vz = -c.fy * Y * iz * iz;
            // dP/dw = -[a]x = [[0, a2, -a1], [-a2, 0, a0], [a1, -a0, 0]], dP/dt = I
            double ju[6], jv[6];
            ju[0] = uz * a1;
            ju[1] = ux * a2 - uz * a0;
            ju[2] = -ux * a1;
            ju[3] = ux;
            ju[4] = 0.0;
            ju[5] = uz;
            jv[0] = -vy * a2 + vz * a1;
            jv[1] = -vz * a0;
            jv[2] = vy * a0;
            jv[3] = 0.0;
            jv[4] = vy;
            jv[5] = vz;
#pragma unroll
            for (int r = 0; r < 6; r++) {
                b[r] -= ju[r] * ex + jv[r] * ey;
#pragma unroll
                for (int k = 0; k < 6; k++) A[6 * r + k] += ju[r] * ju[k] + jv[r] * jv[k];
            }
        }
#pragma unroll
        for (int r = 0; r < 6; r++) A[7 * r] *= 1.0 + mu;
        double d[6];
        M3 Rn;
        double tn[3], cn = 0.0;
        bool better = false;
        if (solve6(A, b, d)) {
            Rn = matmul(so3_exp(d[0], d[1], d[2]), R);
            tn[0] = t[0] + d[3];
            tn[1] = t[1] + d[4];
            tn[2] = t[2] + d[5];
            better = reproj_cost(Rn, tn, ox, oy, px, py, c, &cn) && cn < cost;
        }
        if (!better) {  // drop the step, damp more
            mu *= 10.0;
            if (mu > POSE_MAX_DAMPING) break;
            continue;
        }
        R = Rn;
        t[0] = tn[0];
        t[1] = tn[1];
        t[2] = tn[2];
        cost = cn;
        mu = fmax(mu * 0.1, POSE_DAMPING);
        it++;
        const double step = fabs(d[0]) + fabs(d[1]) + fabs(d[2]) + (fabs(d[3]) + fabs(d[4]) + fabs(d[5])) / tag_size;
        if (step < 1e-12) break;
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P.R[k] = R.m[k];
    P.t[0] = t[0];
    P.t[1] = t[1];
    P.t[2] = t[2];
    // pixel homography of the tag plane: K [r1 r2 t], scaled to h33 = 1
    double Hp[9];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        Hp[3 * r] = R.m[3 * r];
        Hp[3 * r + 1] = R.m[3 * r + 1];
        Hp[3 * r + 2] = t[r];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        Hp[k] = c.fx * Hp[k] + c.cx * Hp[6 + k];
        Hp[3 + k] = c.fy * Hp[3 + k] + c.cy * Hp[6 + k];
    }
#pragma unroll
    for (int k = 0; k < 9; k++) P.H[k] = Hp[k] / Hp[8];
    P.reproj_rms = sqrt(cost / 4.0);
    P.iterations = it;
    out[q] = P;
}

}  // namespace
}  // namespace atag

using namespace atag;

extern "C" atag_status atag_estimate_pose(const float* d_corners, size_t corner_stride, size_t n_quads, double fx,
                                          double fy, double cx, double cy, double tag_size, uint32_t max_iterations,
                                          atag_pose* d_poses, atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (n_quads == 0) return ATAG_OK;
    if (!d_corners || !d_poses) return set_error(ATAG_ERR_INVALID_ARGUMENT, "estimate_pose: null pointer");
    if (corner_stride < 8 * sizeof(float) || corner_stride % 4)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "estimate_pose: corner stride below 32 bytes or not a multiple of 4");
    if (reinterpret_cast<uintptr_t>(d_corners) % 4 || reinterpret_cast<uintptr_t>(d_poses) % 8)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "estimate_pose: misaligned corners or poses");
    if (!(fx > 0.0) || !(fy > 0.0) || !(tag_size > 0.0))
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "estimate_pose: focal lengths and tag size must be positive");
    if (n_quads > (size_t)UINT32_MAX) return set_error(ATAG_ERR_INVALID_ARGUMENT, "estimate_pose: too many quads");
    const uint32_t n = (uint32_t)n_quads;
    k_estimate_pose<<<(n + POSE_THREADS - 1) / POSE_THREADS, POSE_THREADS, 0, (cudaStream_t)stream>>>(reinterpret_cast<const uint8_t*>(d_corners),
                                                                      corner_stride, n, Cam{fx, fy, cx, cy}, tag_size,
                                                                      max_iterations, d_poses);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ATAG_OK : set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
}
