// k_refine.cu — subpixel corner refinement: forward and hand-written adjoint.
//
// The reference stops at the corners of process_fitted_quads
// (src/main.cpp:1035-1162); this stage (new, no counterpart there) refines
// them on an FP32 image the way AprilTag refines edges:
//
//   for each edge e = corner a -> corner b (d = (b-a)/|b-a|, n = (-d_y, d_x)):
//     for j in 0..15:  p_j = a + t_j (b - a),  t_j = (j + 0.5) / 16
//       4 taps across the edge: v_jk = I(p_j + u_k n), u = (-1.5,-0.5,0.5,1.5)
//       (bilinear, clamped to the image: 64 samples per edge)
//       g_m = v_j(m+1) - v_jm, w_m = g_m^2, Omega_j = sum w_m,
//       o_j = (sum w_m c_m) / (Omega_j + eps), c = (-1, 0, 1)
//       edge point q_j = p_j + o_j n with weight W_j = Omega_j + eps
//     weighted line fit of (q_j, W_j): moments in FP32 about the edge
//     midpoint, covariance eigen-solve in FP64: centroid m_e, direction
//     u_e = (cos phi, sin phi), phi = atan2(2 cxy, cxx - cyy) / 2,
//     residual r_e = sum_j W_j d_j^2, d_j the distance of q_j to the line
//     (= S0 * lambda_min, computed in a second pass without cancellation)
//   refined corner i = intersection of lines of edges i-1 and i (FP64).
//
// Forward writes the refined corners, the residuals and the 256 sampled
// intensities per quad; backward recomputes the forward and propagates
// dL/d(refined corners) and dL/d(residuals) to dL/d(corners), dL/d(samples)
// and, optionally, dL/d(image) (scattered through the bilinear weights).
// One 128-thread CTA per quad, one warp per edge, two samples per lane.
#include "atag_internal.h"
#include "atag_kernels.cuh"

namespace atag {
namespace {

constexpr int RF_POS = 16, RF_TAPS = 4;
constexpr float RF_EPS = 1e-6f;
__device__ __constant__ float RF_U[4] = {-1.5f, -0.5f, 0.5f, 1.5f};

struct Bilinear {
    float v, gx, gy;  // value and its spatial gradient
};

// Pixel sources: an FP32 image, or the detector's u8 grey frame read as
// value / 255 (the same numbers as the FP32-normalised image).
struct F32Image {
    const float* __restrict__ p;
    __device__ __forceinline__ float operator[](size_t i) const { return __ldg(p + i); }
};
struct U8Image {
    const uint8_t* __restrict__ p;
    __device__ __forceinline__ float operator[](size_t i) const { return __fdiv_rn((float)__ldg(p + i), 255.0f); }
};

template <class Img>
__device__ __forceinline__ Bilinear bilinear(const Img& img, int w, int h, float x, float y) {
    const float xc = fminf(fmaxf(x, 0.0f), (float)(w - 1)), yc = fminf(fmaxf(y, 0.0f), (float)(h - 1));
    const bool inx = x > 0.0f && x < (float)(w - 1), iny = y > 0.0f && y < (float)(h - 1);
    int x0 = (int)floorf(xc), y0 = (int)floorf(yc);
    x0 = min(x0, w - 2);
    y0 = min(y0, h - 2);
    const float fx = xc - (float)x0, fy = yc - (float)y0;
    const float i00 = img[(size_t)y0 * w + x0], i01 = img[(size_t)y0 * w + x0 + 1];
    const float i10 = img[(size_t)(y0 + 1) * w + x0], i11 = img[(size_t)(y0 + 1) * w + x0 + 1];
    Bilinear b;
    b.v = (1.0f - fy) * ((1.0f - fx) * i00 + fx * i01) + fy * ((1.0f - fx) * i10 + fx * i11);
    b.gx = inx ? (1.0f - fy) * (i01 - i00) + fy * (i11 - i10) : 0.0f;
    b.gy = iny ? (1.0f - fx) * (i10 - i00) + fx * (i11 - i01) : 0.0f;
    return b;
}

__device__ __forceinline__ void bilinear_scatter(float* __restrict__ gimg, int w, int h, float x, float y, float g) {
    const float xc = fminf(fmaxf(x, 0.0f), (float)(w - 1)), yc = fminf(fmaxf(y, 0.0f), (float)(h - 1));
    int x0 = min((int)floorf(xc), w - 2), y0 = min((int)floorf(yc), h - 2);
    const float fx = xc - (float)x0, fy = yc - (float)y0;
    atomicAdd(gimg + (size_t)y0 * w + x0, g * (1.0f - fx) * (1.0f - fy));
    atomicAdd(gimg + (size_t)y0 * w + x0 + 1, g * fx * (1.0f - fy));
    atomicAdd(gimg + (size_t)(y0 + 1) * w + x0, g * (1.0f - fx) * fy);
    atomicAdd(gimg + (size_t)(y0 + 1) * w + x0 + 1, g * fx * fy);
}

// Per-edge geometry and the line fit of one warp.
struct EdgeLine {
    double mx, my, ux, uy, r;                       // line and residual
    double S0, Sx, Sy, Sxx, Syy, Sxy;               // moments about (ox, oy)
    double ox, oy;
    double cxx, cyy, cxy, phi, R, lam;
};

struct LaneState {
    // position j = lane / 2 owns taps 2*(lane&1) .. +1
    float ax, ay, bx, by, dx, dy, nx, ny, len, t;
    Bilinear s[2];
    float sx[2], sy[2];
    // position-level values (valid on even lanes)
    float v[4], gd[3], w[3], Om, Nn, o, W;
    float sa;              // (t_j - 1/2) |b - a|: q_j - midpoint = sa d + o n
    float nux, nuy, dist;  // normal of the fitted line, distance of q_j to it
};

template <class Img>
__device__ __forceinline__ void edge_forward(const Img& img, int iw, int ih, float ax, float ay, float bx,
                                             float by, LaneState& L, EdgeLine& E) {
    const int lane = threadIdx.x & 31, j = lane >> 1, half = lane & 1;
    L.ax = ax; L.ay = ay; L.bx = bx; L.by = by;
    const float Dx = bx - ax, Dy = by - ay;
    L.len = fmaxf(sqrtf(Dx * Dx + Dy * Dy), 1e-6f);
    L.dx = Dx / L.len;
    L.dy = Dy / L.len;
    L.nx = -L.dy;
    L.ny = L.dx;
    L.t = ((float)j + 0.5f) / (float)RF_POS;
    const float px = ax + L.t * Dx, py = ay + L.t * Dy;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const float u = RF_U[2 * half + i];
        L.sx[i] = px + u * L.nx;
        L.sy[i] = py + u * L.ny;
        L.s[i] = bilinear(img, iw, ih, L.sx[i], L.sy[i]);
    }
    // gather the 4 taps of position j on its even lane
    const float o0 = __shfl_xor_sync(0xffffffffu, L.s[0].v, 1), o1 = __shfl_xor_sync(0xffffffffu, L.s[1].v, 1);
    L.v[0] = half ? o0 : L.s[0].v;
    L.v[1] = half ? o1 : L.s[1].v;
    L.v[2] = half ? L.s[0].v : o0;
    L.v[3] = half ? L.s[1].v : o1;
    L.Om = 0.0f;
    L.Nn = 0.0f;
#pragma unroll
    for (int m = 0; m < 3; m++) {
        L.gd[m] = L.v[m + 1] - L.v[m];
        L.w[m] = L.gd[m] * L.gd[m];
        L.Om += L.w[m];
        L.Nn += L.w[m] * (float)(m - 1);
    }
    L.o = L.Nn / (L.Om + RF_EPS);
    L.W = L.Om + RF_EPS;  // a contrast-free edge falls back to the unrefined line
    // moments about the edge midpoint, one contribution per position; the
    // point is taken relative to the midpoint in the edge's own frame
    // ((j - 7.5) / 16 is exact), not as a difference of image coordinates
    const float ox = 0.5f * (ax + bx), oy = 0.5f * (ay + by);
    L.sa = ((float)j - 0.5f * (RF_POS - 1)) / (float)RF_POS * L.len;
    const float X = L.sa * L.dx + L.o * L.nx, Y = L.sa * L.dy + L.o * L.ny, Wc = half ? 0.0f : L.W;
    float m6[6] = {Wc, Wc * X, Wc * Y, Wc * X * X, Wc * Y * Y, Wc * X * Y};
#pragma unroll
    for (int k = 0; k < 6; k++)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) m6[k] += __shfl_xor_sync(0xffffffffu, m6[k], off);
    // FP64 eigen-solve of the 2x2 covariance (every lane, identical values)
    E.ox = ox; E.oy = oy;
    E.S0 = fmax((double)m6[0], 1e-30);
    E.Sx = m6[1]; E.Sy = m6[2]; E.Sxx = m6[3]; E.Syy = m6[4]; E.Sxy = m6[5];
    const double mx = E.Sx / E.S0, my = E.Sy / E.S0;
    E.cxx = E.Sxx / E.S0 - mx * mx;
    E.cyy = E.Syy / E.S0 - my * my;
    E.cxy = E.Sxy / E.S0 - mx * my;
    E.phi = 0.5 * atan2(2.0 * E.cxy, E.cxx - E.cyy);
    const double h2 = 0.5 * (E.cxx - E.cyy);
    E.R = sqrt(h2 * h2 + E.cxy * E.cxy);
    E.lam = 0.5 * (E.cxx + E.cyy) - E.R;
    E.mx = (double)ox + mx;
    E.my = (double)oy + my;
    E.ux = cos(E.phi);
    E.uy = sin(E.phi);
    // residual sum W_j d_j^2 of the perpendicular distances to the fitted
    // line, in a second pass (S0 * lambda_min from the moments would
    // cancel), in the edge frame: d_j = sa (d.nu) + o (n.nu) - (m.nu), whose
    // terms are small where the line runs along the edge
    const double nux = -E.uy, nuy = E.ux;
    L.nux = (float)nux;
    L.nuy = (float)nuy;
    const float cs = (float)((double)L.dx * nux + (double)L.dy * nuy);
    const float cn = (float)((double)L.nx * nux + (double)L.ny * nuy);
    const float c0 = (float)(mx * nux + my * nuy);
    L.dist = L.sa * cs + L.o * cn - c0;
    float rr = half ? 0.0f : L.W * L.dist * L.dist;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) rr += __shfl_xor_sync(0xffffffffu, rr, off);
    E.r = rr;
}

// Intersection of line A (m_A + alpha u_A) with line B, FP64.
__device__ __forceinline__ void intersect(const EdgeLine& A, const EdgeLine& B, double& cx, double& cy, double& alpha,
                                          double& P, double& Q) {
    const double Dx = B.mx - A.mx, Dy = B.my - A.my;
    P = B.ux * Dy - B.uy * Dx;
    Q = B.ux * A.uy - B.uy * A.ux;
    alpha = P / Q;
    cx = A.mx + alpha * A.ux;
    cy = A.my + alpha * A.uy;
}

}  // namespace

__global__ void __launch_bounds__(128) k_refine_forward(const float* __restrict__ img, int iw, int ih,
                                                        const float* __restrict__ corners, int nq,
                                                        float* __restrict__ refined, float* __restrict__ residual,
                                                        float* __restrict__ samples) {
    __shared__ EdgeLine lines[4];
    const int q = blockIdx.x;
    if (q >= nq) return;
    const int e = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const float* c = corners + (size_t)q * 8;
    const int e1 = (e + 1) & 3;
    LaneState L;
    EdgeLine E;
    edge_forward(F32Image{img}, iw, ih, c[2 * e], c[2 * e + 1], c[2 * e1], c[2 * e1 + 1], L, E);
    if (samples) {
        const int j = lane >> 1, half = lane & 1;
        float* s = samples + ((size_t)q * 4 + e) * (RF_POS * RF_TAPS) + j * RF_TAPS + 2 * half;
        s[0] = L.s[0].v;
        s[1] = L.s[1].v;
    }
    if (lane == 0) {
        lines[e] = E;
        if (residual) residual[(size_t)q * 4 + e] = (float)E.r;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        const int i = threadIdx.x;
        double cx, cy, alpha, P, Q;
        intersect(lines[(i + 3) & 3], lines[i], cx, cy, alpha, P, Q);
        refined[(size_t)q * 8 + 2 * i] = (float)cx;
        refined[(size_t)q * 8 + 2 * i + 1] = (float)cy;
    }
}

// Refinement of the detector's own quads, in place, as the last stage of a
// detect call: the frame's u8 grey image, read as value / 255, gives the
// same refined corners as atag_refine_forward on the FP32-normalised image.
// A corner whose two edge lines are nearly parallel (|sin| of their angle
// at most 1e-3) keeps its unrefined position.  Frame blockIdx.x; its quads
// blockIdx.y, blockIdx.y + gridDim.y, ...
__global__ void __launch_bounds__(128) k_refine_detected(const __grid_constant__ FrameSet fs) {
    __shared__ EdgeLine lines[4];
    __shared__ float s_c[8];
    const FrameDesc& F = fs.get(blockIdx.x);
    const uint32_t nq = min(F.stats->n_quads, F.quad_cap);
    const U8Image img{F.grey};
    const int e = threadIdx.x >> 5, lane = threadIdx.x & 31, e1 = (e + 1) & 3;
    for (uint32_t q = blockIdx.y; q < nq; q += gridDim.y) {
        atag_quad_corners* qc = F.quads + q;
        if (threadIdx.x < 8) s_c[threadIdx.x] = qc->corners[threadIdx.x >> 1][threadIdx.x & 1];
        __syncthreads();
        LaneState L;
        EdgeLine E;
        edge_forward(img, (int)F.width, (int)F.height, s_c[2 * e], s_c[2 * e + 1], s_c[2 * e1], s_c[2 * e1 + 1], L, E);
        if (lane == 0) lines[e] = E;
        __syncthreads();
        if (threadIdx.x < 4) {
            const int i = threadIdx.x;
            double cx, cy, alpha, P, Q;
            intersect(lines[(i + 3) & 3], lines[i], cx, cy, alpha, P, Q);
            if (fabs(Q) > 1e-3 && isfinite(cx) && isfinite(cy)) {
                qc->corners[i][0] = (float)cx;
                qc->corners[i][1] = (float)cy;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(128) k_refine_backward(const float* __restrict__ img, int iw, int ih,
                                                         const float* __restrict__ corners, int nq,
                                                         const float* __restrict__ g_refined,
                                                         const float* __restrict__ g_residual,
                                                         float* __restrict__ g_corners, float* __restrict__ g_samples,
                                                         float* __restrict__ g_image) {
    __shared__ EdgeLine lines[4];
    __shared__ double gm[4][2], gu[4][2];   // adjoints of each line's centroid and direction
    __shared__ float gc[4][2];              // adjoints of the input corners
    const int q = blockIdx.x;
    if (q >= nq) return;
    const int e = threadIdx.x >> 5, lane = threadIdx.x & 31, j = lane >> 1, half = lane & 1;
    const float* c = corners + (size_t)q * 8;
    const int e1 = (e + 1) & 3;
    LaneState L;
    EdgeLine E;
    edge_forward(F32Image{img}, iw, ih, c[2 * e], c[2 * e + 1], c[2 * e1], c[2 * e1 + 1], L, E);
    if (lane == 0) lines[e] = E;
    if (threadIdx.x < 8) {
        (&gm[0][0])[threadIdx.x] = 0.0;
        (&gu[0][0])[threadIdx.x] = 0.0;
        (&gc[0][0])[threadIdx.x] = 0.0f;
    }
    __syncthreads();
    // corner i = intersection(line i-1 (A), line i (B))
    if (threadIdx.x == 0) {
        for (int i = 0; i < 4; i++) {
            const int a = (i + 3) & 3, b = i;
            const EdgeLine &A = lines[a], &B = lines[b];
            double cx, cy, alpha, P, Q;
            intersect(A, B, cx, cy, alpha, P, Q);
            const double gcx = g_refined ? (double)g_refined[(size_t)q * 8 + 2 * i] : 0.0;
            const double gcy = g_refined ? (double)g_refined[(size_t)q * 8 + 2 * i + 1] : 0.0;
            gm[a][0] += gcx;
            gm[a][1] += gcy;
            gu[a][0] += alpha * gcx;
            gu[a][1] += alpha * gcy;
            const double ga = gcx * A.ux + gcy * A.uy;
            const double gP = ga / Q, gQ = -ga * P / (Q * Q);
            const double Dx = B.mx - A.mx, Dy = B.my - A.my;
            // P = uBx Dy - uBy Dx
            gu[b][0] += gP * Dy;
            gu[b][1] += -gP * Dx;
            const double gDx = -gP * B.uy, gDy = gP * B.ux;
            // Q = uBx uAy - uBy uAx
            gu[b][0] += gQ * A.uy;
            gu[b][1] += -gQ * A.ux;
            gu[a][0] += -gQ * B.uy;
            gu[a][1] += gQ * B.ux;
            gm[b][0] += gDx;
            gm[b][1] += gDy;
            gm[a][0] -= gDx;
            gm[a][1] -= gDy;
        }
    }
    __syncthreads();
    // line adjoint -> moment adjoints (all lanes compute the same doubles)
    const double gr = g_residual ? (double)g_residual[(size_t)q * 4 + e] : 0.0;
    const double gphi = -sin(E.phi) * gu[e][0] + cos(E.phi) * gu[e][1];
    const double Xc = E.cxx - E.cyy, Yc = 2.0 * E.cxy, den = Xc * Xc + Yc * Yc;
    double gcxx = 0, gcyy = 0, gcxy = 0;
    if (den > 1e-300) {
        gcxy += gphi * Xc / den;
        gcxx += -0.5 * gphi * Yc / den;
        gcyy -= -0.5 * gphi * Yc / den;
    }
    // the residual's gradient needs no path through the line: the line
    // minimises sum W d^2, so only q_j and W_j move it (envelope theorem)
    double gS0 = 0.0;
    const double mx = E.Sx / E.S0, my = E.Sy / E.S0;
    const double gmx = gm[e][0] - 2.0 * mx * gcxx - my * gcxy;
    const double gmy = gm[e][1] - 2.0 * my * gcyy - mx * gcxy;
    const double gSxx = gcxx / E.S0, gSyy = gcyy / E.S0, gSxy = gcxy / E.S0;
    const double gSx = gmx / E.S0, gSy = gmy / E.S0;
    gS0 += -(E.Sxx * gcxx + E.Syy * gcyy + E.Sxy * gcxy + E.Sx * gmx + E.Sy * gmy) / (E.S0 * E.S0);
    // moments -> edge point q_j and weight W_j (even lanes own position j)
    const float X = L.sa * L.dx + L.o * L.nx, Y = L.sa * L.dy + L.o * L.ny;
    const float grf = (float)gr;
    float gW = (float)(gS0 + gSx * X + gSy * Y + gSxx * X * X + gSyy * Y * Y + gSxy * X * Y) +
               grf * L.dist * L.dist;
    float gqx = (float)(L.W * (gSx + 2.0 * gSxx * X + gSxy * Y)) + grf * 2.0f * L.W * L.dist * L.nux;
    float gqy = (float)(L.W * (gSy + 2.0 * gSyy * Y + gSxy * X)) + grf * 2.0f * L.W * L.dist * L.nuy;
    // X = q_x - o_x with q = p + o n and o the midpoint (the forward
    // evaluates the same quantity as sa d_x + o n_x)
    float gox = -gqx, goy = -gqy;
    float gpx = gqx, gpy = gqy;
    const float go = gqx * L.nx + gqy * L.ny;
    float gnx = L.o * gqx, gny = L.o * gqy;
    const float den_o = L.Om + RF_EPS;
    const float gN = go / den_o;
    const float gOm = gW - go * L.Nn / (den_o * den_o);
    float gv[4] = {0, 0, 0, 0};
#pragma unroll
    for (int m = 0; m < 3; m++) {
        const float gw = gN * (float)(m - 1) + gOm;
        const float ggd = 2.0f * L.gd[m] * gw;
        gv[m + 1] += ggd;
        gv[m] -= ggd;
    }
    if (half) {  // only even lanes carry position-level adjoints
        gpx = gpy = gnx = gny = gox = goy = 0.0f;
        gv[0] = gv[1] = gv[2] = gv[3] = 0.0f;
    }
    if (lane == 0) {  // the line's centroid is origin + S_x / S_0: direct path to the origin
        gox += (float)gm[e][0];
        goy += (float)gm[e][1];
    }
    // hand the adjoints of taps 2, 3 to the odd lane
    const float t2 = __shfl_xor_sync(0xffffffffu, gv[2], 1), t3 = __shfl_xor_sync(0xffffffffu, gv[3], 1);
    const float gs0 = half ? t2 : gv[0], gs1 = half ? t3 : gv[1];
    if (g_samples) {
        float* s = g_samples + ((size_t)q * 4 + e) * (RF_POS * RF_TAPS) + j * RF_TAPS + 2 * half;
        s[0] = gs0;
        s[1] = gs1;
    }
    // samples -> sample positions -> p_j, n
    const float gsv[2] = {gs0, gs1};
#pragma unroll
    for (int i = 0; i < 2; i++) {
        const float u = RF_U[2 * half + i];
        const float gx = gsv[i] * L.s[i].gx, gy = gsv[i] * L.s[i].gy;
        gpx += gx;
        gpy += gy;
        gnx += u * gx;
        gny += u * gy;
        if (g_image) bilinear_scatter(g_image, iw, ih, L.sx[i], L.sy[i], gsv[i]);
    }
    // p = a + t (b - a); origin = (a + b) / 2; n = (-d_y, d_x), d = (b - a) / |b - a|
    float gax = (1.0f - L.t) * gpx + 0.5f * gox, gay = (1.0f - L.t) * gpy + 0.5f * goy;
    float gbx = L.t * gpx + 0.5f * gox, gby = L.t * gpy + 0.5f * goy;
    const float gdx = gny, gdy = -gnx;
    const float dd = L.dx * gdx + L.dy * gdy;
    const float gDx = (gdx - L.dx * dd) / L.len, gDy = (gdy - L.dy * dd) / L.len;
    gax -= gDx; gay -= gDy; gbx += gDx; gby += gDy;
    float acc[4] = {gax, gay, gbx, gby};
#pragma unroll
    for (int k = 0; k < 4; k++)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], off);
    if (lane == 0) {
        atomicAdd(&gc[e][0], acc[0]);
        atomicAdd(&gc[e][1], acc[1]);
        atomicAdd(&gc[e1][0], acc[2]);
        atomicAdd(&gc[e1][1], acc[3]);
    }
    __syncthreads();
    if (threadIdx.x < 8) g_corners[(size_t)q * 8 + threadIdx.x] = (&gc[0][0])[threadIdx.x];
}

}  // namespace atag

using namespace atag;

extern "C" atag_status atag_refine_forward(const float* d_image, size_t width, size_t height, const float* d_corners,
                                           size_t n_quads, float* d_refined, float* d_residual, float* d_samples,
                                           atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (!d_image || !d_corners || !d_refined) return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_forward: null pointer");
    if (width < 2 || height < 2) return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_forward: image smaller than 2x2");
    if (n_quads == 0) return ATAG_OK;
    if (n_quads > (size_t)INT32_MAX) return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_forward: too many quads");
    k_refine_forward<<<(unsigned)n_quads, 128, 0, (cudaStream_t)stream>>>(d_image, (int)width, (int)height, d_corners,
                                                                          (int)n_quads, d_refined, d_residual, d_samples);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ATAG_OK : set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
}

extern "C" atag_status atag_refine_backward(const float* d_image, size_t width, size_t height, const float* d_corners,
                                            size_t n_quads, const float* d_grad_refined, const float* d_grad_residual,
                                            float* d_grad_corners, float* d_grad_samples, float* d_grad_image,
                                            atag_stream_t stream) {
    atag_status st = atag_init();
    if (st) return st;
    if (!d_image || !d_corners || !d_grad_corners)
        return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_backward: null pointer");
    if (width < 2 || height < 2) return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_backward: image smaller than 2x2");
    if (n_quads == 0) return ATAG_OK;
    if (n_quads > (size_t)INT32_MAX) return set_error(ATAG_ERR_INVALID_ARGUMENT, "refine_backward: too many quads");
    k_refine_backward<<<(unsigned)n_quads, 128, 0, (cudaStream_t)stream>>>(d_image, (int)width, (int)height,
                                                                           d_corners, (int)n_quads, d_grad_refined,
                                                                           d_grad_residual, d_grad_corners,
                                                                           d_grad_samples, d_grad_image);
    count_launch();
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ATAG_OK : set_error(ATAG_ERR_CUDA, cudaGetErrorString(e));
}
