"""CPU restatement (Python, FP64) of reading tags, atag_decode_quads.

TEST INFRASTRUCTURE ONLY: tests import this as the checker; the product
path is the CUDA kernel (csrc/k_decode.cu).

The reference hands each detected quad to the AprilTag library's
quad_decode_task with the tag36h11 family and the library's detector
defaults plus quad_decimate = 1 (src/quad_decoding.cpp:46-75).  That
library (github.com/carbotaniuman/apriltag, pinned by the reference's
CMakeLists.txt:12-16 at a8b2f9639765162f2ac12a608d785ceb97deee6b) is not in
the reference tree, so parity with it is UNPINNED.  The steps below
restate its published decoding algorithm (Olson 2011; Wang & Olson 2016;
Krogius, Haggenmiller & Olson 2019) and its documented defaults
(refine_edges on, decode_sharpening 0.25):

1. edge refinement: per edge, max(16, |edge| / 8) points spread along it;
   at each, positions -r .. r (r = quad_decimate + 1) in quarter-pixel steps
   along the outward normal; the grey step between the pixels one pixel
   beyond and one pixel before a position (each at the truncated
   coordinate - 0.5), kept where it rises outward (falls, for a reversed
   border), weighted by its square, gives the edge's offset; a line fit
   through those points (normal angle 0.5 atan2(-2 Cxy, Cyy - Cxx)); the
   corners move to the intersections of adjacent lines unless the 2x2
   determinant is at most 1e-3;
2. the homography of the tag square [-1, 1]^2 onto the quad, corners
   (-1,-1), (1,-1), (1,1), (-1,1);
3. grey models: a plane I = a x + b y + c (tag coordinates, least squares)
   fitted to the white ring just outside the black border and one to the
   border itself, sampled at the nearest pixels (truncated coordinates) of
   width_at_border points along each side; the tag is rejected when white
   minus black at its centre is below min_contrast (0: white must not be
   darker), the other way round for a reversed border;
4. each data bit: the bilinear sample at its cell centre (pixel centres at
   +0.5, -1 outside the image: left at 0) minus the mean of the two models
   there, on a total_width x total_width grid; the grid sharpened by
   decode_sharpening times its 4-neighbour Laplacian; bit = value > 0,
   code bit nbits - 1 - i = bit i;
5. decision margin = min(mean positive value over the white bits, mean
   magnitude over the black bits), each count starting at 1;
6. the code and quarter turn with the smallest Hamming distance (ties: the
   fewer turns, then the lower index), accepted at most max_hamming with a
   decision margin of at least 0; the corners are reported rotated so that
   corner 0 is the tag's first corner.

The library's own choices where this one differs or adds: a quad wound the
other way (negative signed area) is read with corners 0, 3, 2, 1 and
flagged; the refinement's normal is oriented outward by the quad's signed
area; a projection behind the camera (z <= 0) marks the quad degenerate.
"""
import math

import numpy as np

REORDERED, DEGENERATE, LOW_CONTRAST = 0x1, 0x2, 0x4

SHARPEN = (0.0, -1.0, 0.0, -1.0, 4.0, -1.0, 0.0, -1.0, 0.0)


def _pix(img, x, y):
    return float(img[y, x])


def refine_edges(img, p, reversed_border=False, quad_decimate=1):
    """Step 1: the refined corners (4 x 2 floats) of a quad wound with
    positive signed area."""
    h, w = img.shape
    lines = []
    for e in range(4):
        a, b = e, (e + 1) & 3
        nx, ny = p[b][1] - p[a][1], -(p[b][0] - p[a][0])
        mag = math.sqrt(nx * nx + ny * ny)
        nx, ny = nx / mag, ny / mag
        if reversed_border:
            nx, ny = -nx, -ny
        nsamples = max(16, int(mag / 8.0))
        Mx = My = Mxx = Mxy = Myy = N = 0.0
        rng = float(quad_decimate + 1)
        for s in range(nsamples):
            alpha = (1.0 + s) / (nsamples + 1)
            x0 = alpha * p[a][0] + (1.0 - alpha) * p[b][0]
            y0 = alpha * p[a][1] + (1.0 - alpha) * p[b][1]
            Mn = Mc = 0.0
            for k in range(int(round(8 * rng)) + 1):
                n = -rng + 0.25 * k
                x1, y1 = int(x0 + (n + 1.0) * nx - 0.5), int(y0 + (n + 1.0) * ny - 0.5)
                if x1 < 0 or x1 >= w or y1 < 0 or y1 >= h:
                    continue
                x2, y2 = int(x0 + (n - 1.0) * nx - 0.5), int(y0 + (n - 1.0) * ny - 0.5)
                if x2 < 0 or x2 >= w or y2 < 0 or y2 >= h:
                    continue
                g1, g2 = _pix(img, x1, y1), _pix(img, x2, y2)
                if g1 < g2:
                    continue
                wgt = (g2 - g1) * (g2 - g1)
                Mn += wgt * n
                Mc += wgt
            if Mc == 0.0:
                continue
            n0 = Mn / Mc
            bx, by = x0 + n0 * nx, y0 + n0 * ny
            Mx += bx
            My += by
            Mxx += bx * bx
            Mxy += bx * by
            Myy += by * by
            N += 1.0
        if N == 0.0:
            lines.append(None)
            continue
        Ex, Ey = Mx / N, My / N
        Cxx, Cxy, Cyy = Mxx / N - Ex * Ex, Mxy / N - Ex * Ey, Myy / N - Ey * Ey
        th = 0.5 * math.atan2(-2.0 * Cxy, Cyy - Cxx)
        lines.append((Ex, Ey, math.cos(th), math.sin(th)))
    out = [list(map(float, c)) for c in p]
    for i in range(4):
        j = (i + 1) & 3
        if lines[i] is None or lines[j] is None:
            continue
        A00, A01 = lines[i][3], -lines[j][3]
        A10, A11 = -lines[i][2], lines[j][2]
        B0, B1 = lines[j][0] - lines[i][0], lines[j][1] - lines[i][1]
        det = A00 * A11 - A10 * A01
        if abs(det) > 0.001:
            L0 = (A11 * B0 - A01 * B1) / det
            out[j] = [lines[i][0] + L0 * A00, lines[i][1] + L0 * A10]
    return out


class _Homography:
    """Step 2: tag square [-1, 1]^2 -> quad, in closed form (Heckbert 1989)
    through the unit square."""

    def __init__(self, p):
        px, py = [c[0] for c in p], [c[1] for c in p]
        sx, sy = px[0] - px[1] + px[2] - px[3], py[0] - py[1] + py[2] - py[3]
        dx1, dx2, dy1, dy2 = px[1] - px[2], px[3] - px[2], py[1] - py[2], py[3] - py[2]
        den = dx1 * dy2 - dx2 * dy1
        ref = abs(dx1) + abs(dx2) + abs(dy1) + abs(dy2)
        self.ok = abs(den) > 1e-12 * ref * ref
        if not self.ok:
            return
        self.g, self.h = (sx * dy2 - dx2 * sy) / den, (dx1 * sy - sx * dy1) / den
        self.a, self.b, self.c = px[1] - px[0] + self.g * px[1], px[3] - px[0] + self.h * px[3], px[0]
        self.d, self.e, self.f = py[1] - py[0] + self.g * py[1], py[3] - py[0] + self.h * py[3], py[0]
        self.behind = False

    def project(self, tx, ty):
        u, v = 0.5 * (tx + 1.0), 0.5 * (ty + 1.0)
        z = self.g * u + self.h * v + 1.0
        if not z > 0.0:
            self.behind = True
            return 0.0, 0.0
        return (self.a * u + self.b * v + self.c) / z, (self.d * u + self.e * v + self.f) / z


class _GreyModel:
    """Least-squares plane I = a x + b y + c over (x, y, I) samples."""

    def __init__(self):
        self.A = np.zeros((3, 3))
        self.B = np.zeros(3)
        self.n = 0

    def add(self, x, y, v):
        r = np.array([x, y, 1.0])
        self.A += np.outer(r, r)
        self.B += r * v
        self.n += 1

    def solve(self):
        if self.n < 3:
            return False
        A = self.A
        det = (A[0, 0] * (A[1, 1] * A[2, 2] - A[1, 2] * A[2, 1]) - A[0, 1] * (A[1, 0] * A[2, 2] - A[1, 2] * A[2, 0]) +
               A[0, 2] * (A[1, 0] * A[2, 1] - A[1, 1] * A[2, 0]))
        if not abs(det) > 1e-12:
            return False
        self.C = solve3(A, self.B)
        return True

    def at(self, x, y):
        return self.C[0] * x + self.C[1] * y + self.C[2]


def solve3(A, B):
    """Cramer's rule for a 3x3 system (the kernel does the same)."""
    def det3(m):
        return (m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1]) - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0]) +
                m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]))
    d = det3(A)
    out = []
    for k in range(3):
        m = [[(B[r] if c == k else A[r][c]) for c in range(3)] for r in range(3)]
        out.append(det3(m) / d)
    return out


def value_for_pixel(img, px, py):
    """Bilinear sample with pixel centres at +0.5; -1 outside the image."""
    h, w = img.shape
    x1, x2 = math.floor(px - 0.5), math.ceil(px - 0.5)
    y1, y2 = math.floor(py - 0.5), math.ceil(py - 0.5)
    if x1 < 0 or x2 >= w or y1 < 0 or y2 >= h:
        return -1.0
    x, y = px - 0.5 - x1, py - 0.5 - y1
    v1, v2 = float(img[y1, x1]), float(img[y1, x2])
    v3, v4 = float(img[y2, x1]), float(img[y2, x2])
    return v1 * (1 - x) * (1 - y) + v2 * x * (1 - y) + v3 * (1 - x) * y + v4 * x * y


def rotation_perm(bit_x, bit_y, W):
    where = {(int(x), int(y)): j for j, (x, y) in enumerate(zip(bit_x, bit_y))}
    return [where[(W - 1 - int(y), int(x))] for x, y in zip(bit_x, bit_y)]


def rotate(code, perm, n):
    out = 0
    for i, j in enumerate(perm):
        if (code >> (n - 1 - j)) & 1:
            out |= 1 << (n - 1 - i)
    return out


def decode_one(img, corners, layout, codes, max_hamming=2, sharpening=0.25, refine=True, quad_decimate=1,
               min_contrast=0.0, reversed_border=False):
    """Steps 1-6 for one quad; `layout` has bit_x, bit_y, width_at_border
    and total_width.  Returns a dict with the fields of atag_decoded."""
    p = [[float(v) for v in c] for c in np.asarray(corners, np.float64)]
    out = {"code": 0, "id": -1, "hamming": 0xFFFFFFFF, "rotation": 0, "status": 0, "decision_margin": 0.0,
           "black": 0.0, "white": 0.0, "corners": np.array(p)}
    area2 = sum(p[i][0] * p[(i + 1) & 3][1] - p[(i + 1) & 3][0] * p[i][1] for i in range(4))
    if area2 < 0.0:
        p[1], p[3] = p[3], p[1]
        out["status"] |= REORDERED
    H = _Homography(p)
    if not H.ok:
        out["status"] |= DEGENERATE
        return out
    if refine:
        p = refine_edges(img, p, reversed_border, quad_decimate)
        H = _Homography(p)
        if not H.ok:
            out["status"] |= DEGENERATE
            return out
    out["corners"] = np.array(p)
    h, w = img.shape
    Wb, T = layout.width_at_border, layout.total_width
    white, black = _GreyModel(), _GreyModel()
    patterns = [(-0.5, 0.5, 0, 1, white), (0.5, 0.5, 0, 1, black), (Wb + 0.5, 0.5, 0, 1, white),
                (Wb - 0.5, 0.5, 0, 1, black), (0.5, -0.5, 1, 0, white), (0.5, 0.5, 1, 0, black),
                (0.5, Wb + 0.5, 1, 0, white), (0.5, Wb - 0.5, 1, 0, black)]
    for x0, y0, dx, dy, model in patterns:
        for i in range(Wb):
            tx = 2.0 * ((x0 + i * dx) / Wb - 0.5)
            ty = 2.0 * ((y0 + i * dy) / Wb - 0.5)
            px, py = H.project(tx, ty)
            ix, iy = int(px), int(py)
            if ix < 0 or iy < 0 or ix >= w or iy >= h:
                continue
            model.add(tx, ty, float(img[iy, ix]))
    if H.behind:
        out["status"] |= DEGENERATE
        return out
    if not (white.solve() and black.solve()):
        out["status"] |= LOW_CONTRAST
        return out
    wc, bc = white.at(0.0, 0.0), black.at(0.0, 0.0)
    out.update(black=bc, white=wc)
    contrast = (bc - wc) if reversed_border else (wc - bc)
    if not contrast >= min_contrast:
        out["status"] |= LOW_CONTRAST
        return out
    m = (Wb - T) // 2
    vals = [0.0] * (T * T)
    n = len(layout.bit_x)
    for i in range(n):
        bx, by = int(layout.bit_x[i]), int(layout.bit_y[i])
        tx = 2.0 * ((bx + 0.5) / Wb - 0.5)
        ty = 2.0 * ((by + 0.5) / Wb - 0.5)
        px, py = H.project(tx, ty)
        v = value_for_pixel(img, px, py)
        if v == -1.0:
            continue
        thr = 0.5 * (black.at(tx, ty) + white.at(tx, ty))
        vals[(by - m) * T + (bx - m)] = v - thr
    if H.behind:
        out["status"] |= DEGENERATE
        return out
    sharp = list(vals)
    for y in range(T):
        for x in range(T):
            acc = 0.0
            for i in range(3):
                for j in range(3):
                    yy, xx = y + i - 1, x + j - 1
                    if 0 <= yy < T and 0 <= xx < T:
                        acc += vals[yy * T + xx] * SHARPEN[i * 3 + j]
            sharp[y * T + x] = vals[y * T + x] + sharpening * acc
    code = 0
    ws, bs, wn, bn = 0.0, 0.0, 1, 1
    for i in range(n):
        bx, by = int(layout.bit_x[i]), int(layout.bit_y[i])
        v = sharp[(by - m) * T + (bx - m)]
        code <<= 1
        if v > 0.0:
            ws += v
            wn += 1
            code |= 1
        else:
            bs -= v
            bn += 1
    margin = min(ws / wn, bs / bn)
    out.update(code=code, decision_margin=margin)
    perm = rotation_perm(layout.bit_x, layout.bit_y, Wb)
    best = None
    r = code
    for k in range(4):
        for idx, c in enumerate(codes):
            hd = bin(r ^ int(c)).count("1")
            key = (hd, k, idx)
            if best is None or key < best:
                best = key
        r = rotate(r, perm, n)
    if best is not None:
        out["hamming"] = best[0]
        if best[0] <= max_hamming and margin >= 0.0:
            out["id"], out["rotation"] = best[2], best[1]
            k = best[1]
            out["corners"] = np.array([p[(i + k) & 3] for i in range(4)])
    return out
