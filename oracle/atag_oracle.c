/*
 * atag_oracle.c — CPU restatement of the reference quad-detection path.
 * TEST INFRASTRUCTURE ONLY (parity checker and timed CPU baseline); the
 * product library never links or calls it.
 *
 * Build flags matter: -ffp-contract=off and no fast-math, so that every
 * float operation below rounds exactly once, as written.  The CUDA kernels
 * use the same operation order with explicit round-to-nearest intrinsics.
 *
 * Citations are file:line in the reference project.
 */
#include "atag_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define LABEL_PIXEL_MASK 0x80000000u
#define LABEL_VALUE_MASK 0x7FFFFFFFu
#define COLOR_DIR_MASK 0x8000u
#define COORD_VALUE_MASK 0x3FFFu

void oracle_config_default(atag_config *c) {
    c->decimate = 1;
    c->min_white_black_diff = 5;
    c->min_component_size = 25;
    c->min_cluster_pixels = 5;
    c->tag_width = 4;
    c->normal_border = 1;
    c->reversed_border = 0;
    c->max_line_fit_mse = 10.0f;
    c->critical_angle_deg = 10.0f;
    c->min_tag_width = 8;
    c->compat_peak_index = 1;
}

/* hypotf: the square root of the exactly-formed sum of squares, computed in
 * double and rounded once to float.  (float)x*(double)x is exact, so this
 * is sqrt_rn(a^2 + b^2 rounded to double) rounded to float. */
float oracle_hypotf(float a, float b) {
    double da = a, db = b;
    return (float)sqrt(da * da + db * db);
}

/* ------------------------------------------------------------------ */
/* Records: include/boundary_point.h, cluster_bounds.h, line_fit_point.h */
/* ------------------------------------------------------------------ */

/* COORDINATE_HALF_PIXEL_MASK is (1<<15)&(1<<14) == 0 (boundary_point.h:16),
 * so extract_half_pixel() is always RIGHT: dx() == 1, dy() == 0. */
static inline int bp_dx(void) { return 1; }
static inline int bp_dy(void) { return 0; }
static inline int bp_b2w(uint16_t packed_y) { return (packed_y & COLOR_DIR_MASK) != 0; }
static inline uint16_t bp_xd(uint16_t packed_x) {
    return (uint16_t)(2 * (packed_x & COORD_VALUE_MASK) + bp_dx());
}
static inline uint16_t bp_yd(uint16_t packed_y) {
    return (uint16_t)(2 * (packed_y & COORD_VALUE_MASK) + bp_dy());
}
static inline int bp_gx(uint16_t packed_y) { return bp_b2w(packed_y) ? bp_dx() : -bp_dx(); }
static inline int bp_gy(uint16_t packed_y) { return bp_b2w(packed_y) ? bp_dy() : -bp_dy(); }

/* boundary_point.h:48-61 */
float oracle_calc_theta(atag_boundary_point p, float cx, float cy) {
    static const float quadrants[2][2] = {{-1 * (1 << 16), 1 << 17}, {0, 1 << 16}};
    float dx = (float)bp_xd(p.packed_x) - cx;
    float dy = (float)bp_yd(p.packed_y) - cy;
    float quadrant = quadrants[dx > 0][dy > 0];
    if ((dx > 0) == (dy > 0)) {
        return quadrant + dy / dx;
    }
    return quadrant - dx / dy;
}

/* cluster_bounds.h:47: int * 0.5f is float, + 0.05118 is a double add,
 * the return rounds to float. */
float oracle_bounds_cx(const atag_cluster_bounds *b) {
    float h = (float)(b->x_min + b->x_max) * 0.5f;
    return (float)((double)h + 0.05118);
}
/* cluster_bounds.h:49 */
float oracle_bounds_cy(const atag_cluster_bounds *b) {
    float h = (float)(b->y_min + b->y_max) * 0.5f;
    return (float)((double)h + -0.028581);
}
/* cluster_bounds.h:51-66.  The int products wrap as on the device. */
float oracle_bounds_dot(const atag_cluster_bounds *b) {
    uint32_t sx = (uint32_t)(b->x_min + b->x_max);
    uint32_t sy = (uint32_t)(b->y_min + b->y_max);
    int32_t t = (int32_t)(sx * (uint32_t)b->gx_sum + sy * (uint32_t)b->gy_sum);
    float cx_cy_contrib = (float)((double)t * 0.5);
    float gx_contrib = (float)(0.05118 * (double)(float)b->gx_sum);
    float gy_contrib = (float)(-0.028581 * (double)(float)b->gy_sum);
    float r = 2.0f * (float)b->pxgx_pygy_sum;
    r = r - cx_cy_contrib;
    r = r - gx_contrib;
    r = r - gy_contrib;
    return r;
}

/* cluster_bounds.h:28-45 */
atag_cluster_bounds oracle_bounds_from_point(atag_boundary_point p, uint32_t start) {
    atag_cluster_bounds b;
    uint16_t xd = bp_xd(p.packed_x), yd = bp_yd(p.packed_y);
    b.x_min = b.x_max = xd;
    b.y_min = b.y_max = yd;
    b.gx_sum = bp_gx(p.packed_y);
    b.gy_sum = bp_gy(p.packed_y);
    b.pxgx_pygy_sum = (int64_t)xd * (int64_t)bp_gx(p.packed_y) + (int64_t)yd * (int64_t)bp_gy(p.packed_y);
    b.start = start;
    b.count = 1;
    return b;
}

/* cluster_bounds.h:69-83 */
atag_cluster_bounds oracle_reduce_bounds(const atag_cluster_bounds *a, const atag_cluster_bounds *b) {
    atag_cluster_bounds o;
    o.x_min = a->x_min < b->x_min ? a->x_min : b->x_min;
    o.x_max = a->x_max > b->x_max ? a->x_max : b->x_max;
    o.y_min = a->y_min < b->y_min ? a->y_min : b->y_min;
    o.y_max = a->y_max > b->y_max ? a->y_max : b->y_max;
    o.start = a->start < b->start ? a->start : b->start;
    o.count = a->count + b->count;
    o.pxgx_pygy_sum = (int64_t)((uint64_t)a->pxgx_pygy_sum + (uint64_t)b->pxgx_pygy_sum);
    o.gx_sum = (int32_t)((uint32_t)a->gx_sum + (uint32_t)b->gx_sum);
    o.gy_sum = (int32_t)((uint32_t)a->gy_sum + (uint32_t)b->gy_sum);
    return o;
}

/* ValidBlobFilter, cluster_bounds.h:85-120 */
int oracle_valid_blob(const atag_cluster_bounds *b, size_t width, size_t height,
                      const atag_config *cfg) {
    size_t max_cluster_pixels = 2 * (2 * width + 2 * height);
    if (b->count < (uint32_t)cfg->min_cluster_pixels) return 0;
    if (b->count < 24) return 0;
    if (b->count > max_cluster_pixels) return 0;
    if ((size_t)((int)(b->x_max - b->x_min) * (int)(b->y_max - b->y_min)) < (size_t)cfg->tag_width)
        return 0;
    int quad_reversed_border = oracle_bounds_dot(b) < 0.0;
    if (!cfg->reversed_border && quad_reversed_border) return 0;
    if (!cfg->normal_border && !quad_reversed_border) return 0;
    return 1;
}

/* Integer square root floor(sqrt(v)). */
static uint32_t isqrt_u32(uint32_t v) {
    uint32_t r = (uint32_t)sqrt((double)v);
    while (r * r > v) r--;
    while ((r + 1) * (r + 1) <= v) r++;
    return r;
}

/* compute_initial_linefit, line_fit_point.h:50-86.  The weight pixel uses
 * row rx/2 (sic, :58-59).  1 + (int64)hypotf(gx, gy) equals
 * 1 + isqrt(gx^2 + gy^2) for |g| <= 255 (no integer lies within float
 * rounding of sqrt(k^2 - 1)); the isqrt form is used on both sides. */
atag_line_fit_point oracle_initial_linefit(atag_cluster_point p, uint32_t width, uint32_t height,
                                           const uint8_t *grey) {
    int64_t rx = (int64_t)bp_xd(p.packed_x) + 1;
    int64_t ry = (int64_t)bp_yd(p.packed_y) + 1;
    uint32_t x = (uint32_t)(rx / 2);
    uint32_t y = (uint32_t)(rx / 2);
    int64_t W = 1;
    if (x > 0 && x + 1 < width && y > 0 && y + 1 < height) {
        int gx = (int)grey[y * width + x + 1] - (int)grey[y * width + x - 1];
        int gy = (int)grey[(y + 1) * width + x] - (int)grey[(y - 1) * width + x];
        W += (int64_t)isqrt_u32((uint32_t)(gx * gx + gy * gy));
    }
    atag_line_fit_point o;
    o.Mx = W * rx;
    o.My = W * ry;
    o.Mxx = W * rx * rx;
    o.Myy = W * ry * ry;
    o.Mxy = W * rx * ry;
    o.W = W;
    o.a = 0;
    o.b = 0;
    return o;
}

static inline void lfp_add(atag_line_fit_point *a, const atag_line_fit_point *b) {
    a->Mx = (int64_t)((uint64_t)a->Mx + (uint64_t)b->Mx);
    a->My = (int64_t)((uint64_t)a->My + (uint64_t)b->My);
    a->Mxx = (int64_t)((uint64_t)a->Mxx + (uint64_t)b->Mxx);
    a->Myy = (int64_t)((uint64_t)a->Myy + (uint64_t)b->Myy);
    a->Mxy = (int64_t)((uint64_t)a->Mxy + (uint64_t)b->Mxy);
    a->W = (int64_t)((uint64_t)a->W + (uint64_t)b->W);
}
static inline void lfp_sub(atag_line_fit_point *a, const atag_line_fit_point *b) {
    a->Mx = (int64_t)((uint64_t)a->Mx - (uint64_t)b->Mx);
    a->My = (int64_t)((uint64_t)a->My - (uint64_t)b->My);
    a->Mxx = (int64_t)((uint64_t)a->Mxx - (uint64_t)b->Mxx);
    a->Myy = (int64_t)((uint64_t)a->Myy - (uint64_t)b->Myy);
    a->Mxy = (int64_t)((uint64_t)a->Mxy - (uint64_t)b->Mxy);
    a->W = (int64_t)((uint64_t)a->W - (uint64_t)b->W);
}

/* get_moment, fit_quad.cpp:15-35 (size_t arithmetic wraps as written). */
void oracle_get_moment(const atag_line_fit_point *points, size_t points_size, size_t i0, size_t i1,
                       atag_line_fit_point *out, size_t *n_out) {
    atag_line_fit_point r;
    memset(&r, 0, sizeof r);
    size_t total = 0;
    if (i0 < i1) {
        total = i1 - i0 + 1;
        r = points[i1];
        if (i0 > 0) lfp_sub(&r, &points[i0 - 1]);
    } else if (i1 < i0) {
        total = points_size - i0 + i1 + 1;
        r = points[points_size - 1];
        lfp_sub(&r, &points[i0 - 1]);
        lfp_add(&r, &points[i1]);
    }
    r.a = 0;
    r.b = 0;
    *out = r;
    *n_out = total;
}

static inline int64_t wmul(int64_t a, int64_t b) { return (int64_t)((uint64_t)a * (uint64_t)b); }
static inline int64_t wsub(int64_t a, int64_t b) { return (int64_t)((uint64_t)a - (uint64_t)b); }
static inline int64_t wadd(int64_t a, int64_t b) { return (int64_t)((uint64_t)a + (uint64_t)b); }

/* fit_line, fit_quad.cpp:37-105.  int64 products wrap (two's complement). */
void oracle_fit_line(const atag_line_fit_point *m, size_t num_in_moment, float *line_params,
                     float *err, float *mse) {
    int64_t Csxx = wsub(wmul(m->Mxx, m->W), wmul(m->Mx, m->Mx));
    int64_t Csxy = wsub(wmul(m->Mxy, m->W), wmul(m->Mx, m->My));
    int64_t Csyy = wsub(wmul(m->Myy, m->W), wmul(m->My, m->My));
    int64_t correction_factor = wmul(wmul(m->W, m->W), 4);
    float sdist = oracle_hypotf((float)wsub(Csxx, Csyy), (float)wmul(2, Csxy));
    float num = (float)wadd(Csxx, Csyy) - sdist;
    float eig_err = num / (float)wmul(correction_factor, 2);
    if (line_params) {
        float nx1 = (float)wsub(Csxx, Csyy) - sdist;
        float ny1 = (float)wmul(2, Csxy);
        float nx2 = (float)wmul(2, Csxy);
        float ny2 = (float)wsub(Csyy, Csxx) - sdist;
        float M1 = nx1 * nx1;
        M1 = M1 + ny1 * ny1;
        float M2 = nx2 * nx2;
        M2 = M2 + ny2 * ny2;
        float nx, ny;
        if (M1 > M2) {
            nx = nx1;
            ny = ny1;
        } else {
            nx = nx2;
            ny = ny2;
        }
        line_params[0] = (float)m->Mx / (float)wmul(m->W, 2);
        line_params[1] = (float)m->My / (float)wmul(m->W, 2);
        float length = oracle_hypotf(nx, ny);
        if (fabs(length) < 1e-12) {
            line_params[2] = 0;
            line_params[3] = 0;
        } else {
            line_params[2] = nx / length;
            line_params[3] = ny / length;
        }
    }
    if (err) *err = (float)num_in_moment * eig_err;
    if (mse) *mse = eig_err;
}

/* Combinatorial number system decode (combinadics.h:36-53 with K=4): the
 * largest c0 with C(c0,4) <= n, then C(c1,3) <= n - C(c0,4), ... */
static const uint32_t BINOM[5][16] = {
    {1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1},
    {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15},
    {0, 0, 1, 3, 6, 10, 15, 21, 28, 36, 45, 55, 66, 78, 91, 105},
    {0, 0, 0, 1, 4, 10, 20, 35, 56, 84, 120, 165, 220, 286, 364, 455},
    {0, 0, 0, 0, 1, 5, 15, 35, 70, 126, 210, 330, 495, 715, 1001, 1365},
};
void oracle_combination_decode(uint32_t num, uint32_t out[4]) {
    for (int i = 0; i < 4; i++) {
        const uint32_t *row = BINOM[4 - i];
        int c = 15;
        while (c > 0 && row[c] > num) c--;
        num -= row[c];
        out[i] = (uint32_t)c;
    }
}
static uint32_t n_choose_4(uint32_t n) { return BINOM[4][n]; }

/* ------------------------------------------------------------------ */
/* Stage a0: decimation (absent in the reference; point sampling).    */
/* ------------------------------------------------------------------ */
void oracle_decimate(const uint8_t *src, int src_w, int src_h, int f, uint8_t *dst) {
    int w = src_w / f, h = src_h / f;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) dst[(size_t)y * w + x] = src[(size_t)y * f * src_w + (size_t)x * f];
}

/* Colour removal (notes.txt step 1).  The reference removes colour when it
 * loads its input: stbi_load(..., STBI_grey) (src/main.cpp:264-265), i.e.
 * stb's luma y = (77 r + 150 g + 29 b) >> 8 for 3 and 4 channels, alpha
 * ignored (include/stb_image.h:1834-1836, 1899-1915), and the grey channel
 * of grey + alpha.  BGR orders swap r and b. */
static int pixel_bytes(int format) {
    switch (format) {
    case ATAG_PIX_GREY8: return 1;
    case ATAG_PIX_GREYA8: return 2;
    case ATAG_PIX_RGB8: case ATAG_PIX_BGR8: return 3;
    case ATAG_PIX_RGBA8: case ATAG_PIX_BGRA8: return 4;
    }
    return 0;
}
static uint8_t luma(int r, int g, int b) { return (uint8_t)((r * 77 + g * 150 + b * 29) >> 8); }

void oracle_to_grey(const uint8_t *src, int src_w, int src_h, int src_pitch, int format, int f, uint8_t *dst) {
    const int bpp = pixel_bytes(format);
    const size_t pitch = src_pitch ? (size_t)src_pitch : (size_t)src_w * bpp;
    const int w = src_w / f, h = src_h / f;
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const uint8_t *p = src + (size_t)y * f * pitch + (size_t)x * f * bpp;
            uint8_t v;
            switch (format) {
            case ATAG_PIX_RGB8: case ATAG_PIX_RGBA8: v = luma(p[0], p[1], p[2]); break;
            case ATAG_PIX_BGR8: case ATAG_PIX_BGRA8: v = luma(p[2], p[1], p[0]); break;
            default: v = p[0]; break; /* grey, grey + alpha */
            }
            dst[(size_t)y * w + x] = v;
        }
}

/* ------------------------------------------------------------------ */
/* Stage a1: threshold.cpp:8-95                                       */
/* ------------------------------------------------------------------ */
void oracle_threshold(const uint8_t *g, int w, int h, int min_diff, uint8_t *extrema,
                      uint8_t *filtered, uint8_t *out) {
    int tw = w / 4, th = h / 4;
    uint8_t *ext = extrema ? extrema : (uint8_t *)malloc((size_t)tw * th * 2);
    uint8_t *flt = filtered ? filtered : (uint8_t *)malloc((size_t)tw * th * 2);
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            uint8_t mn = 255, mx = 0;
            for (int i = 0; i < 4; i++)
                for (int j = 0; j < 4; j++) {
                    uint8_t v = g[(size_t)(ty * 4 + i) * w + tx * 4 + j];
                    if (v < mn) mn = v;
                    if (v > mx) mx = v;
                }
            ext[((size_t)ty * tw + tx) * 2 + 0] = mn;
            ext[((size_t)ty * tw + tx) * 2 + 1] = mx;
        }
    for (int ty = 0; ty < th; ty++)
        for (int tx = 0; tx < tw; tx++) {
            uint8_t mn = 255, mx = 0;
            for (int i = -1; i <= 1; i++)
                for (int j = -1; j <= 1; j++) {
                    int yy = ty + i, xx = tx + j;
                    if (xx < 0 || xx >= tw || yy < 0 || yy >= th) continue;
                    uint8_t a = ext[((size_t)yy * tw + xx) * 2 + 0];
                    uint8_t b = ext[((size_t)yy * tw + xx) * 2 + 1];
                    if (a < mn) mn = a;
                    if (b > mx) mx = b;
                }
            flt[((size_t)ty * tw + tx) * 2 + 0] = mn;
            flt[((size_t)ty * tw + tx) * 2 + 1] = mx;
        }
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const uint8_t *f = &flt[((size_t)(y / 4) * tw + x / 4) * 2];
            uint8_t mn = f[0], mx = f[1];
            uint8_t comp = (uint8_t)(mn + (mx - mn) / 2);
            uint8_t v = g[(size_t)y * w + x];
            uint8_t o;
            if (mx - mn < min_diff)
                o = 127;
            else
                o = v > comp ? 255 : 0;
            out[(size_t)y * w + x] = o;
        }
    if (!extrema) free(ext);
    if (!filtered) free(flt);
}

/* ------------------------------------------------------------------ */
/* Stage a2/a3: BKE CCL, segmentation.cpp:47-389, union_find.h:19-77  */
/* ------------------------------------------------------------------ */
enum {
    TL255 = 1 << 0, TR255 = 1 << 1, BL255 = 1 << 2, BR255 = 1 << 3,
    MU_P = 1 << 4, MU_Q = 1 << 5, MU_R = 1 << 6, MU_S = 1 << 7,
    TL0 = 1 << 8, TR0 = 1 << 9, BL0 = 1 << 10, BR0 = 1 << 11,
};

static uint32_t uf_find(const uint32_t *buf, uint32_t n) {
    while (buf[n] != n) n = buf[n];
    return n;
}
/* merge: link the larger root under the smaller (union_find.h:50-77). */
static void uf_merge(uint32_t *buf, uint32_t a, uint32_t b) {
    a = uf_find(buf, a);
    b = uf_find(buf, b);
    if (a < b)
        buf[b] = a;
    else if (b < a)
        buf[a] = b;
}

void oracle_segmentation(const uint8_t *thr, int w, int h, uint32_t *scratch_in, uint32_t *labels,
                         uint32_t *sizes) {
    size_t W = (size_t)w, N = (size_t)w * h;
    uint32_t *s = scratch_in ? scratch_in : (uint32_t *)malloc(N * sizeof(uint32_t));
    /* INITIALIZATION (:101-262) */
    for (int y = 0; y < h; y += 2)
        for (int x = 0; x < w; x += 2) {
            size_t id = (size_t)y * W + x;
            uint16_t info = 0;
            uint32_t check = 0;
            uint8_t v;
            v = thr[id];
            if (v == 255) { check |= 0x777; info |= TL255; }
            else if (v == 0) { check |= 0x777; info |= TL0; }
            v = thr[id + 1];
            if (v == 255) { check |= 0x777 << 1; info |= TR255; }
            else if (v == 0) { check |= 0x777 << 1; info |= TR0; }
            v = thr[id + W];
            if (v == 255) { check |= 0x777 << 4; info |= BL255; }
            else if (v == 0) { check |= 0x777 << 4; info |= BL0; }
            v = thr[id + W + 1];
            if (v == 255) info |= BR255;
            else if (v == 0) info |= BR0;
            if (x == 0) check &= 0xEEEE;
            else if (x + 2 >= w) check &= 0x7777;
            if (y == 0) check &= 0xFFF0;
            else if (y + 2 >= h) check &= 0x0FFF;
            int64_t off255 = 0, off0 = 1;
            static const int tdy[6] = {-1, -1, -1, -1, 0, 1};
            static const int tdx[6] = {-1, 0, 1, 2, -1, -1};
            static const int tbit[6] = {0, 1, 2, 3, 4, 8};
            static const int tkind[6] = {MU_P, MU_Q, MU_Q, MU_R, MU_S, MU_S};
            for (int t = 0; t < 6; t++) {
                if (!(check & (1u << tbit[t]))) continue;
                uint8_t tp = thr[(size_t)((int64_t)id + (int64_t)tdy[t] * (int64_t)W + tdx[t])];
                int64_t off;
                switch (tkind[t]) {
                case MU_P: off = -2 * (int64_t)W - 2; break;
                case MU_Q: off = -2 * (int64_t)W; break;
                case MU_R: off = -2 * (int64_t)W + 2; break;
                default: off = -2; break;
                }
                if (tp == 255) {
                    if (off255 == 0) off255 = off;
                    else info |= (uint16_t)tkind[t];
                } else if (tp == 0) {
                    if (off0 == 1) off0 = off + 1;
                    else info |= (uint16_t)(tkind[t] << 8);
                }
            }
            s[id] = (uint32_t)((int64_t)id + off255);
            s[id + 1] = (uint32_t)((int64_t)id + off0);
            s[id + W] = info;
        }
    /* MERGE (:269-306); the compressions (:265,309) do not change roots. */
    for (int y = 0; y < h; y += 2)
        for (int x = 0; x < w; x += 2) {
            size_t id = (size_t)y * W + x;
            uint16_t info = (uint16_t)s[id + W];
            if (info & MU_Q) uf_merge(s, id, id - 2 * W);
            if (info & MU_R) uf_merge(s, id, id - 2 * W + 2);
            if (info & MU_S) uf_merge(s, id, id - 2);
            if (info & (MU_Q << 8)) uf_merge(s, id + 1, id - 2 * W + 1);
            if (info & (MU_R << 8)) uf_merge(s, id + 1, id - 2 * W + 3);
            if (info & (MU_S << 8)) uf_merge(s, id + 1, id - 1);
        }
    /* COMPRESSION (:73-91, :309) */
    for (int y = 0; y < h; y += 2)
        for (int x = 0; x < w; x += 2) {
            size_t id = (size_t)y * W + x;
            s[id] = uf_find(s, id);
            s[id + 1] = uf_find(s, id + 1);
        }
    /* FINAL_LABELLING (:316-389) with all N sizes zeroed (H3). */
    memset(sizes, 0, N * sizeof(uint32_t));
    for (int y = 0; y < h; y += 2)
        for (int x = 0; x < w; x += 2) {
            size_t id = (size_t)y * W + x;
            uint32_t l255 = s[id], l0 = s[id + 1];
            uint16_t info = (uint16_t)s[id + W];
            uint32_t c255 = (uint32_t)__builtin_popcount(info & 0xF);
            uint32_t c0 = (uint32_t)__builtin_popcount(info & 0xF00);
            if (c255) sizes[l255] += c255;
            if (c0) sizes[l0] += c0;
            uint32_t tl = (info & TL255) ? (LABEL_PIXEL_MASK | l255) : (info & TL0) ? l0 : 0;
            uint32_t tr = (info & TR255) ? (LABEL_PIXEL_MASK | l255) : (info & TR0) ? l0 : 0;
            uint32_t bl = (info & BL255) ? (LABEL_PIXEL_MASK | l255) : (info & BL0) ? l0 : 0;
            uint32_t br = (info & BR255) ? (LABEL_PIXEL_MASK | l255) : (info & BR0) ? l0 : 0;
            labels[id] = tl;
            labels[id + 1] = tr;
            labels[id + W] = bl;
            labels[id + W + 1] = br;
        }
    if (!scratch_in) free(s);
}

/* ------------------------------------------------------------------ */
/* Stage a4: find_boundaries.cpp:10-155 (dense planes)                */
/* ------------------------------------------------------------------ */
static inline uint32_t lab_at(const uint32_t *labels, int w, int h, int y, int x) {
    if (x < 0 || y < 0 || x >= w || y >= h) return 0;
    return labels[(size_t)y * w + x];
}

void oracle_find_boundaries(const uint32_t *labels, const uint32_t *sizes, int w, int h,
                            int min_size, atag_boundary_point *points, uint64_t *keys) {
    size_t N = (size_t)w * h;
    /* Column x == 0 is never processed: every work-group's local x == 0 is a
     * halo-only work-item (find_boundaries.cpp:36,66-69). */
    for (int y = 0; y < h; y++)
        for (int x = 1; x < w; x++) {
            uint32_t p = labels[(size_t)y * w + x];
            uint32_t lp = p & LABEL_VALUE_MASK;
            int small_p = sizes[lp] < (uint32_t)min_size;
            uint32_t cp = p & LABEL_PIXEL_MASK;
            size_t idx = (size_t)y * w + x;
            for (int t = 0; t < 4; t++) {
                static const int dy[4] = {0, 1, 1, 1}, dx[4] = {1, -1, 0, 1};
                if (t == 1) {
                    uint32_t left = lab_at(labels, w, h, y, x - 1);
                    uint32_t down = lab_at(labels, w, h, y + 1, x);
                    int would_dup = (left & LABEL_PIXEL_MASK) != (down & LABEL_PIXEL_MASK) &&
                                    sizes[left & LABEL_VALUE_MASK] >= (uint32_t)min_size &&
                                    sizes[down & LABEL_VALUE_MASK] >= (uint32_t)min_size;
                    if (would_dup) continue;
                }
                uint32_t q = lab_at(labels, w, h, y + dy[t], x + dx[t]);
                uint32_t cq = q & LABEL_PIXEL_MASK;
                if (cq == cp) continue;
                uint32_t lq = q & LABEL_VALUE_MASK;
                int small_q = sizes[lq] < (uint32_t)min_size;
                if (small_p || small_q) continue;
                atag_boundary_point bp;
                bp.packed_x = (uint16_t)(x | (t << 14));
                bp.packed_y = (uint16_t)(cq > cp ? (COLOR_DIR_MASK | (uint32_t)y) : (uint32_t)y);
                uint64_t lo = lp < lq ? lp : lq, hi = lp < lq ? lq : lp;
                points[(size_t)t * N + idx] = bp;
                keys[(size_t)t * N + idx] = (lo << 32) | hi;
            }
        }
}

/* ------------------------------------------------------------------ */
/* Stage a16: fit_lines                                               */
/* ------------------------------------------------------------------ */
static const float FILTER_DATA[7] = {0x1.6c0504p-7f, 0x1.152aaap-3f, 0x1.368b3p-1f, 0x1p+0f,
                                     0x1.368b3p-1f, 0x1.152aaap-3f, 0x1.6c0504p-7f};

/* error of the window [i-k, i+k] around cluster-local position `pos`
 * (fit_quad.cpp:202-225): k = min(20, count/12), NaN when k < 2. */
static float window_error(const atag_line_fit_point *points, atag_cluster_extents e, int64_t x) {
    size_t k = e.count / 12;
    if (k > 20) k = 20;
    if (k < 2) return NAN;
    size_t i0 = (size_t)((int64_t)e.count + x - (int64_t)e.start - (int64_t)k) % e.count;
    size_t i1 = (size_t)((int64_t)e.count + x - (int64_t)e.start + (int64_t)k) % e.count;
    atag_line_fit_point m;
    size_t n;
    oracle_get_moment(points + e.start, e.count, i0, i1, &m, &n);
    float err;
    oracle_fit_line(&m, n, NULL, &err, NULL);
    return err;
}

/* Literal restatement of fit_quad.cpp:153-375: work-groups of 32 with 24
 * corner-finding work-items, "same"/"diff" cluster error arrays. */
void oracle_fit_lines_windowed(const atag_line_fit_point *points, const uint32_t *cidx,
                               const atag_cluster_extents *extents, size_t n,
                               atag_corner *found) {
    enum { WG = 32, PPE = 3, EO = 4 };
    size_t groups = (n + 23) / 24;
    for (size_t g = 0; g < groups; g++) {
        uint32_t lci[WG];
        atag_cluster_extents lce[WG];
        float es[WG], ed[WG], fs[WG], fd[WG];
        int64_t xs[WG];
        for (int l = 0; l < WG; l++) {
            int64_t x = (int64_t)g * (WG - 2 * EO) + l - PPE;
            xs[l] = x;
            int64_t xc = x < 0 ? 0 : (x > (int64_t)n - 1 ? (int64_t)n - 1 : x);
            lci[l] = cidx[xc];
            lce[l] = extents[lci[l]];
        }
        for (int l = 0; l < WG; l++) {
            es[l] = window_error(points, lce[l], xs[l]);
            int their = l;
            if (l >= EO && lci[l - EO] != lci[l]) their = l - EO;
            if (l < WG - EO && lci[l + EO] != lci[l]) their = l + EO;
            ed[l] = their != l ? window_error(points, lce[their], xs[l]) : NAN;
        }
        for (int l = PPE; l < WG - PPE; l++) {
            float acc = 0.0f, dacc = 0.0f;
            for (int i = 0; i < 7; i++) {
                int t = l + i - PPE;
                if (lci[t] == lci[l]) {
                    acc = acc + es[t] * FILTER_DATA[i];
                    dacc = dacc + ed[t] * FILTER_DATA[i];
                } else {
                    dacc = dacc + es[t] * FILTER_DATA[i];
                    acc = acc + ed[t] * FILTER_DATA[i];
                }
            }
            fs[l] = acc;
            fd[l] = dacc;
        }
        for (int l = EO; l < WG - EO; l++) {
            int64_t x = xs[l];
            if (x < 0 || x >= (int64_t)n) continue;
            float cur = fs[l];
            int gb = cur > (lci[l - 1] == lci[l] ? fs : fd)[l - 1];
            int ga = cur > (lci[l + 1] == lci[l] ? fs : fd)[l + 1];
            if (gb && ga) {
                atag_corner c;
                c.line_fit_point_index = (uint32_t)(x - lce[l].start);
                c.cluster_index = (uint16_t)lci[l];
                c.error = cur;
                found[x] = c;
            }
        }
    }
}

/* Per-cluster formulation: errors and the 7-tap filter wrap cyclically
 * inside each cluster; global point 0 is never a corner. */
void oracle_fit_lines_cyclic(const atag_line_fit_point *points, const uint32_t *cidx,
                             const atag_cluster_extents *extents, size_t n_clusters,
                             atag_corner *found) {
    (void)cidx;
    for (size_t c = 0; c < n_clusters; c++) {
        atag_cluster_extents e = extents[c];
        size_t n = e.count;
        float *err = (float *)malloc(n * sizeof(float));
        float *flt = (float *)malloc(n * sizeof(float));
        for (size_t i = 0; i < n; i++) err[i] = window_error(points, e, (int64_t)(e.start + i));
        for (size_t i = 0; i < n; i++) {
            float acc = 0.0f;
            for (int j = 0; j < 7; j++) acc = acc + err[(i + n + j - 3) % n] * FILTER_DATA[j];
            flt[i] = acc;
        }
        for (size_t i = 0; i < n; i++) {
            if (e.start + i == 0) continue;
            float cur = flt[i];
            if (cur > flt[(i + n - 1) % n] && cur > flt[(i + 1) % n]) {
                atag_corner k;
                k.line_fit_point_index = (uint32_t)i;
                k.cluster_index = (uint16_t)c;
                k.error = cur;
                found[e.start + i] = k;
            }
        }
        free(err);
        free(flt);
    }
}

/* ------------------------------------------------------------------ */
/* Stage a19: do_indexing, fit_quad.cpp:377-535                       */
/* ------------------------------------------------------------------ */
static void sort_4(size_t a[4]) {
#define SW(i, j)                                                                                   \
    if (!(a[i] < a[j])) {                                                                          \
        size_t t = a[i];                                                                           \
        a[i] = a[j];                                                                               \
        a[j] = t;                                                                                  \
    }
    SW(0, 1) SW(2, 3) SW(0, 2) SW(1, 3) SW(1, 2)
#undef SW
}

void oracle_do_indexing(const atag_peak_extents *pe, size_t count, const atag_corner *corners,
                        const atag_line_fit_point *points, const atag_cluster_extents *ce,
                        const atag_config *cfg, atag_fitted_quad *fitted) {
    float cos_critical_rad = (float)cos((double)cfg->critical_angle_deg * M_PI / 180);
    for (size_t q = 0; q < count; q++) {
        atag_peak_extents peak = pe[q];
        atag_cluster_extents cur =
            cfg->compat_peak_index ? ce[q] : ce[corners[peak.start].cluster_index];
        uint32_t m = peak.count < 10 ? peak.count : 10;
        uint32_t ncomb = n_choose_4(m);
        float errs[256];
        atag_fitted_quad cand[256];
        float lowest = INFINITY;
        for (uint32_t n = 0; n < 256; n++) {
            int valid = n < ncomb;
            float total = 0.0f;
            atag_fitted_quad fq;
            memset(&fq, 0, sizeof fq);
            if (valid) {
                uint32_t idx[4];
                oracle_combination_decode(n, idx);
                size_t lfi[4];
                for (int j = 0; j < 4; j++) lfi[j] = corners[peak.start + idx[j]].line_fit_point_index;
                sort_4(lfi);
                float p01[4], p12[4];
                for (int s = 0; s < 4; s++) {
                    atag_line_fit_point mo;
                    size_t nim;
                    oracle_get_moment(points + cur.start, cur.count, lfi[s], lfi[(s + 1) & 3], &mo, &nim);
                    float e, mse;
                    oracle_fit_line(&mo, nim, s == 0 ? p01 : s == 1 ? p12 : NULL, &e, &mse);
                    valid &= mse <= cfg->max_line_fit_mse;
                    fq.moments[s] = mo;
                    fq.num_in_moments[s] = (uint16_t)nim;
                    total = total + e;
                }
                float dot = p01[2] * p12[2];
                dot = dot + p01[3] * p12[3];
                valid &= fabsf(dot) <= cos_critical_rad;
                for (int j = 0; j < 4; j++) fq.indices[j] = (uint16_t)lfi[j];
            }
            errs[n] = valid ? total : INFINITY;
            cand[n] = fq;
            if (errs[n] < lowest) lowest = errs[n];
        }
        if (lowest == INFINITY) continue;
        for (uint32_t n = 0; n < 256; n++) {
            if ((double)(errs[n] - lowest) < 0.1) {
                fitted[q] = cand[n];
                break;
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Stage a20: process_fitted_quads, main.cpp:1035-1162                */
/* ------------------------------------------------------------------ */
size_t oracle_process_fitted_quads(const atag_fitted_quad *fitted, size_t nq, const atag_config *cfg,
                                   atag_quad_corners *out) {
    size_t nout = 0;
    double cos_critical = cos((double)cfg->critical_angle_deg * M_PI / 180);
    double min_area = 0.95 * cfg->min_tag_width * cfg->min_tag_width;
    for (size_t qi = 0; qi < nq; qi++) {
        const atag_fitted_quad *quad = &fitted[qi];
        if (!(quad->indices[0] != 0 || quad->indices[1] != 0 || quad->indices[2] != 0 ||
              quad->indices[3] != 0))
            continue;
        atag_quad_corners c;
        memset(&c, 0, sizeof c);
        c.reversed_border = (uint8_t)cfg->reversed_border;
        c.blob_index = (uint32_t)qi;
        float lines[4][4];
        for (int i = 0; i < 4; i++) {
            float e, mse;
            oracle_fit_line(&quad->moments[i], quad->num_in_moments[i], lines[i], &e, &mse);
        }
        int bad = 0;
        for (int i = 0; i < 4; i++) {
            int j = (i + 1) & 3;
            double A00 = lines[i][3], A01 = -lines[j][3];
            double A10 = -lines[i][2], A11 = lines[j][2];
            double B0 = (double)(-lines[i][0] + lines[j][0]);
            double B1 = (double)(-lines[i][1] + lines[j][1]);
            double det = A00 * A11;
            det = det - A10 * A01;
            double W00 = A11 / det, W01 = -A01 / det;
            if (fabs(det) < 0.001) {
                bad = 1;
                break;
            }
            double L0 = W00 * B0;
            L0 = L0 + W01 * B1;
            double t0 = L0 * A00, t1 = L0 * A10;
            c.corners[i][0] = (float)((double)lines[i][0] + t0);
            c.corners[i][1] = (float)((double)lines[i][1] + t1);
        }
        if (bad) continue;
        {
            float area = 0, length[3], p;
            for (int i = 0; i < 3; i++) {
                int a = i, b = (i + 1) % 3;
                length[i] = oracle_hypotf(c.corners[b][0] - c.corners[a][0],
                                          c.corners[b][1] - c.corners[a][1]);
            }
            p = (length[0] + length[1] + length[2]) / 2;
            {
                float t = p * (p - length[0]);
                t = t * (p - length[1]);
                t = t * (p - length[2]);
                area = area + sqrtf(t);
            }
            static const int idxs[4] = {2, 3, 0, 2};
            for (int i = 0; i < 3; i++) {
                int a = idxs[i], b = idxs[i + 1];
                length[i] = oracle_hypotf(c.corners[b][0] - c.corners[a][0],
                                          c.corners[b][1] - c.corners[a][1]);
            }
            p = (length[0] + length[1] + length[2]) / 2;
            {
                float t = p * (p - length[0]);
                t = t * (p - length[1]);
                t = t * (p - length[2]);
                area = area + sqrtf(t);
            }
            if (area < min_area) continue;
        }
        {
            int reject = 0;
            for (int i = 0; i < 4; i++) {
                int i0 = i, i1 = (i + 1) & 3, i2 = (i + 2) & 3;
                float dx1 = c.corners[i1][0] - c.corners[i0][0];
                float dy1 = c.corners[i1][1] - c.corners[i0][1];
                float dx2 = c.corners[i2][0] - c.corners[i1][0];
                float dy2 = c.corners[i2][1] - c.corners[i1][1];
                float num = dx1 * dx2;
                num = num + dy1 * dy2;
                float s1 = dx1 * dx1;
                s1 = s1 + dy1 * dy1;
                float s2 = dx2 * dx2;
                s2 = s2 + dy2 * dy2;
                float cos_dtheta = num / sqrtf(s1 * s2);
                if (fabs((double)cos_dtheta) > cos_critical || dx1 * dy2 < dy1 * dx2) {
                    reject = 1;
                    break;
                }
            }
            if (reject) continue;
        }
        out[nout++] = c;
    }
    return nout;
}

/* ------------------------------------------------------------------ */
/* Glue: main.cpp:467-970 (oneDPL stages)                             */
/* ------------------------------------------------------------------ */
typedef struct {
    uint64_t key;
    uint32_t packed;
} key_point;

static int cmp_key_point(const void *a, const void *b) {
    const key_point *x = (const key_point *)a, *y = (const key_point *)b;
    if (x->key != y->key) return x->key < y->key ? -1 : 1;
    if (x->packed != y->packed) return x->packed < y->packed ? -1 : 1;
    return 0;
}

typedef struct {
    uint32_t cluster;
    float theta;
    uint32_t packed;
} theta_point;

static int cmp_theta_point(const void *a, const void *b) {
    const theta_point *x = (const theta_point *)a, *y = (const theta_point *)b;
    if (x->cluster != y->cluster) return x->cluster < y->cluster ? -1 : 1;
    if (x->theta < y->theta) return -1;
    if (y->theta < x->theta) return 1;
    if (x->packed != y->packed) return x->packed < y->packed ? -1 : 1;
    return 0;
}

static int cmp_corner(const void *a, const void *b) {
    const atag_corner *x = (const atag_corner *)a, *y = (const atag_corner *)b;
    if (x->cluster_index != y->cluster_index) return x->cluster_index < y->cluster_index ? -1 : 1;
    if (x->error > y->error) return -1;
    if (y->error > x->error) return 1;
    if (x->line_fit_point_index != y->line_fit_point_index)
        return x->line_fit_point_index < y->line_fit_point_index ? -1 : 1;
    return 0;
}

static inline uint32_t pack_u32(atag_boundary_point p) {
    return (uint32_t)p.packed_x | ((uint32_t)p.packed_y << 16);
}
static inline atag_boundary_point unpack_u32(uint32_t v) {
    atag_boundary_point p;
    p.packed_x = (uint16_t)(v & 0xFFFF);
    p.packed_y = (uint16_t)(v >> 16);
    return p;
}

int oracle_detect(const uint8_t *src, int src_w, int src_h, const atag_config *cfg,
                  oracle_result *r) {
    memset(r, 0, sizeof *r);
    int f = cfg->decimate < 1 ? 1 : cfg->decimate;
    int w = src_w / f, h = src_h / f;
    if (w < 4 || h < 4 || (w % 4) || (h % 4) || w > 4096 || h > 4096) return -1;
    size_t N = (size_t)w * h;
    r->width = w;
    r->height = h;
    r->decimated = (uint8_t *)malloc(N);
    if (f == 1)
        memcpy(r->decimated, src, N);
    else
        oracle_decimate(src, src_w, src_h, f, r->decimated);
    const uint8_t *grey = r->decimated;

    /* stage 1 */
    r->thresholded = (uint8_t *)malloc(N);
    oracle_threshold(grey, w, h, cfg->min_white_black_diff, NULL, NULL, r->thresholded);
    /* stage 2 */
    r->labels = (uint32_t *)malloc(N * 4);
    r->sizes = (uint32_t *)malloc(N * 4);
    oracle_segmentation(r->thresholded, w, h, NULL, r->labels, r->sizes);
    /* stage 3 + D1 (copy_if keeps plane-major order) */
    atag_boundary_point *dense_p = (atag_boundary_point *)calloc(4 * N, sizeof(atag_boundary_point));
    uint64_t *dense_k = (uint64_t *)malloc(4 * N * sizeof(uint64_t));
    memset(dense_k, 0xFF, 4 * N * sizeof(uint64_t));
    oracle_find_boundaries(r->labels, r->sizes, w, h, cfg->min_component_size, dense_p, dense_k);
    size_t P = 0;
    for (size_t i = 0; i < 4 * N; i++)
        if (pack_u32(dense_p[i]) != 0) P++;
    key_point *kp = (key_point *)malloc((P ? P : 1) * sizeof(key_point));
    P = 0;
    for (size_t i = 0; i < 4 * N; i++)
        if (pack_u32(dense_p[i]) != 0) {
            kp[P].key = dense_k[i];
            kp[P].packed = pack_u32(dense_p[i]);
            P++;
        }
    free(dense_p);
    free(dense_k);
    /* D2 sort_by_key (ties by packed point) */
    qsort(kp, P, sizeof(key_point), cmp_key_point);
    r->n_points = P;
    r->points = (atag_boundary_point *)malloc((P ? P : 1) * sizeof(atag_boundary_point));
    r->keys = (uint64_t *)malloc((P ? P : 1) * sizeof(uint64_t));
    for (size_t i = 0; i < P; i++) {
        r->points[i] = unpack_u32(kp[i].packed);
        r->keys[i] = kp[i].key;
    }
    free(kp);
    /* D3 reduce_by_segment -> ClusterBounds */
    size_t C = 0;
    for (size_t i = 0; i < P; i++)
        if (i == 0 || r->keys[i] != r->keys[i - 1]) C++;
    r->n_bounds = C;
    r->bounds = (atag_cluster_bounds *)malloc((C ? C : 1) * sizeof(atag_cluster_bounds));
    r->bound_keys = (uint64_t *)malloc((C ? C : 1) * sizeof(uint64_t));
    {
        size_t c = (size_t)-1;
        for (size_t i = 0; i < P; i++) {
            atag_cluster_bounds b = oracle_bounds_from_point(r->points[i], (uint32_t)i);
            if (i == 0 || r->keys[i] != r->keys[i - 1]) {
                c++;
                r->bounds[c] = b;
                r->bound_keys[c] = r->keys[i];
            } else {
                r->bounds[c] = oracle_reduce_bounds(&r->bounds[c], &b);
            }
        }
    }
    /* D4 ValidBlobFilter */
    size_t Cf = 0;
    for (size_t c = 0; c < C; c++)
        if (oracle_valid_blob(&r->bounds[c], w, h, cfg)) Cf++;
    r->n_filtered = Cf;
    r->filtered = (atag_cluster_bounds *)malloc((Cf ? Cf : 1) * sizeof(atag_cluster_bounds));
    r->filtered_keys = (uint64_t *)malloc((Cf ? Cf : 1) * sizeof(uint64_t));
    r->extents = (atag_cluster_extents *)malloc((Cf ? Cf : 1) * sizeof(atag_cluster_extents));
    Cf = 0;
    for (size_t c = 0; c < C; c++)
        if (oracle_valid_blob(&r->bounds[c], w, h, cfg)) {
            r->filtered[Cf] = r->bounds[c];
            r->filtered_keys[Cf] = r->bound_keys[c];
            Cf++;
        }
    /* D6 exclusive scan of counts -> ClusterExtents */
    {
        uint32_t s = 0;
        for (size_t c = 0; c < Cf; c++) {
            r->extents[c].start = s;
            r->extents[c].count = r->filtered[c].count;
            s += r->filtered[c].count;
        }
    }
    /* D5 points -> clusters + theta; D7 sort (cluster, theta, packed) */
    size_t Pf = 0;
    for (size_t c = 0; c < Cf; c++) Pf += r->filtered[c].count;
    theta_point *tp = (theta_point *)malloc((Pf ? Pf : 1) * sizeof(theta_point));
    {
        size_t k = 0;
        for (size_t c = 0; c < Cf; c++) {
            const atag_cluster_bounds *b = &r->filtered[c];
            float cx = oracle_bounds_cx(b), cy = oracle_bounds_cy(b);
            for (uint32_t i = b->start; i < b->start + b->count; i++) {
                tp[k].cluster = (uint32_t)c;
                tp[k].theta = oracle_calc_theta(r->points[i], cx, cy);
                tp[k].packed = pack_u32(r->points[i]);
                k++;
            }
        }
    }
    qsort(tp, Pf, sizeof(theta_point), cmp_theta_point);
    r->n_cluster_points = Pf;
    r->cluster_points = (atag_cluster_point *)malloc((Pf ? Pf : 1) * sizeof(atag_cluster_point));
    r->cluster_indices = (uint32_t *)malloc((Pf ? Pf : 1) * sizeof(uint32_t));
    for (size_t i = 0; i < Pf; i++) {
        atag_boundary_point p = unpack_u32(tp[i].packed);
        r->cluster_points[i].packed_x = p.packed_x;
        r->cluster_points[i].packed_y = p.packed_y;
        r->cluster_points[i].slope = tp[i].theta;
        r->cluster_indices[i] = tp[i].cluster;
    }
    free(tp);
    /* D8 initial line fit + D9 segmented inclusive scan */
    r->line_fit = (atag_line_fit_point *)malloc((Pf ? Pf : 1) * sizeof(atag_line_fit_point));
    for (size_t i = 0; i < Pf; i++) {
        r->line_fit[i] = oracle_initial_linefit(r->cluster_points[i], (uint32_t)w, (uint32_t)h, grey);
        if (i > 0 && r->cluster_indices[i] == r->cluster_indices[i - 1])
            lfp_add(&r->line_fit[i], &r->line_fit[i - 1]);
    }
    /* K10 fit_lines (dense corners, pre-zeroed) */
    r->found_corners = (atag_corner *)calloc(Pf ? Pf : 1, sizeof(atag_corner));
    if (Pf) oracle_fit_lines_cyclic(r->line_fit, r->cluster_indices, r->extents, Cf, r->found_corners);
    /* D10 compact (error != 0), D11 sort, D12 peak extents */
    size_t K = 0;
    for (size_t i = 0; i < Pf; i++)
        if (r->found_corners[i].error != 0) K++;
    r->n_corners = K;
    r->corners = (atag_corner *)malloc((K ? K : 1) * sizeof(atag_corner));
    K = 0;
    for (size_t i = 0; i < Pf; i++)
        if (r->found_corners[i].error != 0) r->corners[K++] = r->found_corners[i];
    qsort(r->corners, K, sizeof(atag_corner), cmp_corner);
    size_t Cp = 0;
    for (size_t i = 0; i < K; i++)
        if (i == 0 || r->corners[i].cluster_index != r->corners[i - 1].cluster_index) Cp++;
    r->n_peak_extents = Cp;
    r->peak_extents = (atag_peak_extents *)malloc((Cp ? Cp : 1) * sizeof(atag_peak_extents));
    {
        size_t c = (size_t)-1;
        for (size_t i = 0; i < K; i++) {
            if (i == 0 || r->corners[i].cluster_index != r->corners[i - 1].cluster_index) {
                c++;
                r->peak_extents[c].start = (uint32_t)i;
                r->peak_extents[c].count = 0;
            }
            r->peak_extents[c].count++;
        }
    }
    /* K11 do_indexing (fitted pre-zeroed) */
    r->fitted = (atag_fitted_quad *)calloc(Cp ? Cp : 1, sizeof(atag_fitted_quad));
    oracle_do_indexing(r->peak_extents, Cp, r->corners, r->line_fit, r->extents, cfg, r->fitted);
    /* H1 process_fitted_quads */
    r->quads = (atag_quad_corners *)malloc((Cp ? Cp : 1) * sizeof(atag_quad_corners));
    r->n_quads = oracle_process_fitted_quads(r->fitted, Cp, cfg, r->quads);
    return 0;
}

void oracle_free(oracle_result *r) {
    free(r->decimated);
    free(r->thresholded);
    free(r->labels);
    free(r->sizes);
    free(r->points);
    free(r->keys);
    free(r->bounds);
    free(r->bound_keys);
    free(r->filtered);
    free(r->filtered_keys);
    free(r->extents);
    free(r->cluster_points);
    free(r->cluster_indices);
    free(r->line_fit);
    free(r->found_corners);
    free(r->corners);
    free(r->peak_extents);
    free(r->fitted);
    free(r->quads);
    memset(r, 0, sizeof *r);
}

/* ------------------------------------------------------------------ */
/* Batch evaluation of the record helpers (golden-vector checks).     */
/* ------------------------------------------------------------------ */
void oracle_eval_bounds(const atag_cluster_bounds *b, const atag_boundary_point *p, size_t n, size_t w,
                        size_t h, float *cx, float *cy, float *theta, float *dot, uint8_t *valid) {
    atag_config cfg;
    oracle_config_default(&cfg);
    for (size_t i = 0; i < n; i++) {
        cx[i] = oracle_bounds_cx(&b[i]);
        cy[i] = oracle_bounds_cy(&b[i]);
        theta[i] = oracle_calc_theta(p[i], cx[i], cy[i]);
        dot[i] = oracle_bounds_dot(&b[i]);
        valid[i] = (uint8_t)oracle_valid_blob(&b[i], w, h, &cfg);
    }
}

void oracle_eval_linefit(const atag_cluster_point *p, size_t n, uint32_t w, uint32_t h, const uint8_t *img,
                         atag_line_fit_point *out) {
    for (size_t i = 0; i < n; i++) out[i] = oracle_initial_linefit(p[i], w, h, img);
}

void oracle_eval_fit_line(const atag_line_fit_point *m, const uint64_t *nim, size_t n, float *lp, float *err,
                          float *mse) {
    for (size_t i = 0; i < n; i++) oracle_fit_line(&m[i], (size_t)nim[i], &lp[4 * i], &err[i], &mse[i]);
}

void oracle_eval_get_moment(const atag_line_fit_point *pre, size_t np, const uint64_t *ranges, size_t n,
                            atag_line_fit_point *out, uint64_t *nout) {
    for (size_t i = 0; i < n; i++) {
        size_t c;
        oracle_get_moment(pre, np, (size_t)ranges[2 * i], (size_t)ranges[2 * i + 1], &out[i], &c);
        nout[i] = c;
    }
}

int oracle_detect_many(const uint8_t *const *srcs, const int *src_w, const int *src_h, size_t n,
                       const atag_config *cfg, int threads, uint32_t *n_quads) {
    int used = 1;
#ifdef _OPENMP
    if (threads < 1) threads = omp_get_max_threads();
    used = threads;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
#endif
    for (long i = 0; i < (long)n; i++) {
        oracle_result r;
        if (oracle_detect(srcs[i], src_w[i], src_h[i], cfg, &r) == 0)
            n_quads[i] = (uint32_t)r.n_quads;
        else
            n_quads[i] = 0xFFFFFFFFu;
        oracle_free(&r);
    }
    (void)threads;
    return used;
}
