"""CPU restatement (numpy, FP64) of reading tags, atag_decode_quads.

TEST INFRASTRUCTURE ONLY: tests import this as the checker; the product
path is the CUDA kernel (csrc/k_decode.cu).

Parity unpinned against the reference: the reference hands each quad to the
AprilTag library's quad_decode_task with tag36h11
(src/quad_decoding.cpp:46-128), and neither that library nor its family
tables are in the reference tree.  This restatement is pinned instead to
tags of a seeded random code family rendered with known codes, corner order
and winding (tests/test_decode_ref.py).

Steps, per quad (the kernel's): winding (negative signed area: corners
0, 3, 2, 1); closed-form projective map of the unit square onto the quad
(Heckbert 1989); bilinear samples at cell centres of the (D + 2)-cell grid,
pixel centres at integer coordinates, clamped to the image; black level =
mean of the 4 (D + 1) border cells, white level = mean of the 4 (D + 2)
cells of the ring just outside (corner cells left out); threshold halfway;
bit = sample > threshold; nearest code over four quarter turns.
"""
import math

import numpy as np

REORDERED, DEGENERATE, LOW_CONTRAST = 0x1, 0x2, 0x4


def _sample(img, x, y):
    h, w = img.shape
    x = min(max(x, 0.0), float(w - 1))
    y = min(max(y, 0.0), float(h - 1))
    x0, y0 = min(int(math.floor(x)), w - 2), min(int(math.floor(y)), h - 2)
    fx, fy = x - x0, y - y0
    a, b = float(img[y0, x0]), float(img[y0, x0 + 1])
    c, d = float(img[y0 + 1, x0]), float(img[y0 + 1, x0 + 1])
    return (1.0 - fy) * ((1.0 - fx) * a + fx * b) + fy * ((1.0 - fx) * c + fx * d)


def rotate90(v, D):
    """Cell (r, c) of the result is cell (D - 1 - c, r) of v."""
    n = D * D
    o = 0
    for r in range(D):
        for c in range(D):
            src = (D - 1 - c) * D + r
            if (v >> (n - 1 - src)) & 1:
                o |= 1 << (n - 1 - (r * D + c))
    return o


def decode_one(img, corners, codes, D=6, max_hamming=2, min_contrast=10.0):
    px = [float(v) for v in np.asarray(corners, np.float64)[:, 0]]
    py = [float(v) for v in np.asarray(corners, np.float64)[:, 1]]
    out = {"code": 0, "id": -1, "hamming": 0, "rotation": 0, "status": 0, "black": 0.0, "white": 0.0, "margin": 0.0}
    area2 = sum(px[i] * py[(i + 1) % 4] - px[(i + 1) % 4] * py[i] for i in range(4))
    if area2 < 0.0:
        px[1], px[3] = px[3], px[1]
        py[1], py[3] = py[3], py[1]
        out["status"] |= REORDERED
    sx, sy = px[0] - px[1] + px[2] - px[3], py[0] - py[1] + py[2] - py[3]
    dx1, dx2, dy1, dy2 = px[1] - px[2], px[3] - px[2], py[1] - py[2], py[3] - py[2]
    den = dx1 * dy2 - dx2 * dy1
    ref = abs(dx1) + abs(dx2) + abs(dy1) + abs(dy2)
    if not abs(den) > 1e-12 * ref * ref:
        out["status"] |= DEGENERATE
        return out
    g, hh = (sx * dy2 - dx2 * sy) / den, (dx1 * sy - sx * dy1) / den
    a, b, c = px[1] - px[0] + g * px[1], px[3] - px[0] + hh * px[3], px[0]
    d, e, f = py[1] - py[0] + g * py[1], py[3] - py[0] + hh * py[3], py[0]
    cells = float(D + 2)

    def at(cc, rr):
        u, v = cc / cells, rr / cells
        z = g * u + hh * v + 1.0
        return _sample(img, (a * u + b * v + c) / z, (d * u + e * v + f) / z)

    black = sum(at(k + 0.5, 0.5) + at(D + 1.5, k + 0.5) + at(D + 2 - k - 0.5, D + 1.5) + at(0.5, D + 2 - k - 0.5)
                for k in range(D + 1))
    white = sum(at(k + 0.5, -0.5) + at(D + 2.5, k + 0.5) + at(D + 2 - k - 0.5, D + 2.5) + at(-0.5, D + 2 - k - 0.5)
                for k in range(D + 2))
    black /= 4.0 * (D + 1)
    white /= 4.0 * (D + 2)
    out.update(black=black, white=white)
    if not white - black >= min_contrast:
        out["status"] |= LOW_CONTRAST
        return out
    thr = 0.5 * (black + white)
    n = D * D
    obs, margin = 0, math.inf
    for r in range(D):
        for cc in range(D):
            v = at(cc + 1.5, r + 1.5)
            if v > thr:
                obs |= 1 << (n - 1 - (r * D + cc))
            margin = min(margin, abs(v - thr))
    out.update(code=obs, margin=margin)
    best, best_id, best_rot, rot = None, -1, 0, obs
    for k in range(4):
        for i, code in enumerate(codes):
            hd = bin(rot ^ int(code)).count("1")
            if best is None or hd < best:
                best, best_id, best_rot = hd, i, k
        rot = rotate90(rot, D)
    out["hamming"] = best if best is not None else 0xFFFFFFFF
    if best is not None and best <= max_hamming:
        out.update(id=best_id, rotation=best_rot)
    return out


def random_family(n, seed, D=6, min_distance=8):
    """Seeded random codes whose pairwise distances over all quarter turns
    (and each code to its own turns) are at least min_distance: a stand-in
    family for tests."""
    rng = np.random.default_rng(seed)
    codes = []
    while len(codes) < n:
        c = int(rng.integers(0, 1 << (D * D), dtype=np.uint64))
        rots = [c]
        for _ in range(3):
            rots.append(rotate90(rots[-1], D))
        if any(bin(rots[0] ^ r).count("1") < min_distance for r in rots[1:]):
            continue
        if any(bin(r ^ o).count("1") < min_distance for r in rots for o in codes):
            continue
        codes.append(c)
    return codes


def code_bits(code, D=6):
    """The D x D bit grid (True = white) of a code."""
    n = D * D
    return np.array([[(code >> (n - 1 - (r * D + c))) & 1 for c in range(D)] for r in range(D)], bool)
