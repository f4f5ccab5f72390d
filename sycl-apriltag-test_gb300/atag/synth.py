"""Seeded synthetic frames for the benchmark and parity workloads.

The reference ships no dataset and no benchmark; frames are rendered here
from a seed so that every run sees the same pixels:

* background: uniform noise in [90, 170] plus a linear illumination
  gradient of +-40 in a random direction;
* fiducials: a 10x10-cell square (1-cell white outer border, 1-cell black
  border, 6x6 random interior bits with p = 0.5), side drawn from a range,
  rotated U(0, 360 deg) and tilted up to 40 deg through a perspective
  homography;
* clutter: filled rectangles, ellipses and line segments with random
  intensity in [0, 255] and size in [4, 120] px;
* Gaussian blur, additive Gaussian noise, clip to [0, 255], salt-and-pepper.

Everything is numpy; a 1920x1080 frame with 40 fiducials and 300 clutter
shapes renders in well under a second.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class FrameSpec:
    width: int
    height: int
    n_fiducials: int = 8
    side_range: tuple = (30, 150)
    n_clutter: int = 0
    blur_sigma: tuple = (0.8, 0.8)
    noise_sigma: tuple = (4.0, 4.0)
    salt_pepper: float = 0.0
    max_tilt_deg: float = 40.0


# The workloads named by the benchmark configurations.
CONFIGS = {
    "vga": FrameSpec(640, 480, 8, (30, 150), 0, (0.8, 0.8), (4.0, 4.0)),
    "1080p": FrameSpec(1920, 1080, 40, (16, 300), 300, (0.5, 1.5), (2.0, 8.0)),
    "4k": FrameSpec(3840, 2160, 150, (12, 400), 3000, (0.5, 1.5), (2.0, 8.0), 0.005),
}
BATCH_SIZES = [(640, 480), (1280, 720), (1920, 1080), (2592, 1944)]


def _homography(src, dst):
    """DLT for 4 point pairs: returns H with dst ~ H @ src."""
    A = []
    for (x, y), (u, v) in zip(src, dst):
        A.append([-x, -y, -1, 0, 0, 0, u * x, u * y, u])
        A.append([0, 0, 0, -x, -y, -1, v * x, v * y, v])
    _, _, vt = np.linalg.svd(np.asarray(A, np.float64))
    H = vt[-1].reshape(3, 3)
    return H / H[2, 2]


def _tag_quad(rng, cx, cy, side, max_tilt_deg):
    """Image-space corners of a square of `side` px after rotation and a
    perspective tilt about a random in-plane axis."""
    rot = rng.uniform(0, 2 * np.pi)
    tilt = np.deg2rad(rng.uniform(0, max_tilt_deg))
    axis = rng.uniform(0, 2 * np.pi)
    s = side / 2.0
    pts = np.array([[-s, -s, 0], [s, -s, 0], [s, s, 0], [-s, s, 0]], np.float64)
    c, si = np.cos(rot), np.sin(rot)
    Rz = np.array([[c, -si, 0], [si, c, 0], [0, 0, 1]])
    ax = np.array([np.cos(axis), np.sin(axis), 0.0])
    K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]])
    Rt = np.eye(3) + np.sin(tilt) * K + (1 - np.cos(tilt)) * (K @ K)
    P = pts @ Rz.T @ Rt.T
    f = 4.0 * side
    Z = P[:, 2] + f
    u = cx + f * P[:, 0] / Z
    v = cy + f * P[:, 1] / Z
    return np.stack([u, v], 1)


def _render_tag(img, rng, quad, bits):
    """Inverse-maps every pixel of the quad's bounding box into tag-cell
    space (10x10 cells) and paints black/white."""
    h, w = img.shape
    H = _homography(quad, np.array([[0, 0], [10, 0], [10, 10], [0, 10]], np.float64))
    x0 = int(max(0, np.floor(quad[:, 0].min())))
    x1 = int(min(w - 1, np.ceil(quad[:, 0].max())))
    y0 = int(max(0, np.floor(quad[:, 1].min())))
    y1 = int(min(h - 1, np.ceil(quad[:, 1].max())))
    if x1 <= x0 or y1 <= y0:
        return
    ys, xs = np.mgrid[y0:y1 + 1, x0:x1 + 1]
    X = xs + 0.5
    Y = ys + 0.5
    d = H[2, 0] * X + H[2, 1] * Y + H[2, 2]
    u = (H[0, 0] * X + H[0, 1] * Y + H[0, 2]) / d
    v = (H[1, 0] * X + H[1, 1] * Y + H[1, 2]) / d
    inside = (u >= 0) & (u < 10) & (v >= 0) & (v < 10)
    cu = np.clip(u.astype(np.int64), 0, 9)
    cv = np.clip(v.astype(np.int64), 0, 9)
    grid = np.full((10, 10), 255, np.uint8)
    grid[1:9, 1:9] = 0
    grid[2:8, 2:8] = np.where(bits, 255, 0).astype(np.uint8)
    val = grid[cv, cu]
    sub = img[y0:y1 + 1, x0:x1 + 1]
    sub[inside] = val[inside]


def _render_clutter(img, rng):
    h, w = img.shape
    kind = rng.integers(0, 3)
    size = rng.uniform(4, 120)
    cx, cy = rng.uniform(0, w), rng.uniform(0, h)
    val = np.float32(rng.integers(0, 256))
    r = int(np.ceil(size)) + 2
    x0, x1 = int(max(0, cx - r)), int(min(w, cx + r + 1))
    y0, y1 = int(max(0, cy - r)), int(min(h, cy + r + 1))
    if x1 <= x0 or y1 <= y0:
        return
    ys, xs = np.mgrid[y0:y1, x0:x1]
    dx, dy = xs + 0.5 - cx, ys + 0.5 - cy
    ang = rng.uniform(0, np.pi)
    c, s = np.cos(ang), np.sin(ang)
    u, v = c * dx + s * dy, -s * dx + c * dy
    if kind == 0:  # rectangle
        a, b = size / 2, rng.uniform(2, size) / 2
        mask = (np.abs(u) <= a) & (np.abs(v) <= b)
    elif kind == 1:  # ellipse
        a, b = size / 2, rng.uniform(2, size) / 2
        mask = (u / a) ** 2 + (v / b) ** 2 <= 1.0
    else:  # line segment
        th = rng.uniform(1, 4)
        mask = (np.abs(u) <= size / 2) & (np.abs(v) <= th / 2)
    img[y0:y1, x0:x1][mask] = val


def _blur(img, sigma):
    if sigma <= 0:
        return img
    r = max(1, int(np.ceil(3 * sigma)))
    k = np.exp(-0.5 * (np.arange(-r, r + 1) / sigma) ** 2)
    k = (k / k.sum()).astype(np.float32)
    out = np.zeros_like(img)
    pad = np.pad(img, ((0, 0), (r, r)), mode="edge")
    for i, kv in enumerate(k):
        out += kv * pad[:, i:i + img.shape[1]]
    pad = np.pad(out, ((r, r), (0, 0)), mode="edge")
    out2 = np.zeros_like(img)
    for i, kv in enumerate(k):
        out2 += kv * pad[i:i + img.shape[0], :]
    return out2


def border_corners(quad):
    """The outer corners of a rendered tag's black border (cells 1 and 9 of
    its 10-cell square), with pixel centres at integer coordinates: where
    the detector's quad corners should lie."""
    H = _homography(np.array([[0, 0], [10, 0], [10, 10], [0, 10]], np.float64), quad)
    inner = np.array([[1, 1, 1], [9, 1, 1], [9, 9, 1], [1, 9, 1]], np.float64)
    p = inner @ H.T
    return p[:, :2] / p[:, 2:] - 0.5


def render(spec: FrameSpec, seed: int, truth: list = None) -> np.ndarray:
    """Renders one uint8 frame of spec.height x spec.width from `seed`.
    If `truth` is a list, the border corners (border_corners) of every tag
    are appended to it in drawing order (later tags may cover earlier
    ones); the pixels do not depend on it."""
    rng = np.random.default_rng(seed)
    h, w = spec.height, spec.width
    img = rng.uniform(90, 170, size=(h, w)).astype(np.float32)
    ang = rng.uniform(0, 2 * np.pi)
    yy, xx = np.mgrid[0:h, 0:w].astype(np.float32)
    proj = (np.cos(ang) * (xx / max(w - 1, 1) - 0.5) + np.sin(ang) * (yy / max(h - 1, 1) - 0.5))
    img += (80.0 * proj).astype(np.float32)
    for _ in range(spec.n_clutter):
        _render_clutter(img, rng)
    for _ in range(spec.n_fiducials):
        side = rng.uniform(*spec.side_range)
        cx = rng.uniform(side * 0.6, max(side * 0.6 + 1, w - side * 0.6))
        cy = rng.uniform(side * 0.6, max(side * 0.6 + 1, h - side * 0.6))
        quad = _tag_quad(rng, cx, cy, side, spec.max_tilt_deg)
        bits = rng.random((6, 6)) < 0.5
        _render_tag(img, rng, quad, bits)
        if truth is not None:
            truth.append(border_corners(quad))
    img = _blur(img, rng.uniform(*spec.blur_sigma))
    img += rng.normal(0, rng.uniform(*spec.noise_sigma), size=img.shape).astype(np.float32)
    if spec.salt_pepper > 0:
        m = rng.random(img.shape) < spec.salt_pepper
        img[m] = np.where(rng.random(int(m.sum())) < 0.5, 0, 255)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8)


def batch_specs(n: int, seed: int):
    """Mixed-resolution batch: sizes from BATCH_SIZES, 0-60 fiducials and
    0-1000 clutter shapes per frame."""
    rng = np.random.default_rng(seed)
    specs = []
    for _ in range(n):
        w, h = BATCH_SIZES[rng.integers(0, len(BATCH_SIZES))]
        specs.append(FrameSpec(w, h, int(rng.integers(0, 61)), (16, 300), int(rng.integers(0, 1001)),
                               (0.5, 1.5), (2.0, 8.0)))
    return specs


# ---------------------------------------------------------------------------
# Tag families for reading tags.  A family is described the way the
# AprilTag library describes one: nbits data bits, bit i in the cell
# (bit_x[i], bit_y[i]) of a grid in which cells 0 .. width_at_border - 1
# span the outer edge of the black border, total_width cells across the
# whole tag (white quiet zone included), and codes whose bit nbits - 1 - i
# holds bit i.  The code tables of the library's families are not
# reproduced here; these are seeded stand-ins with the same geometry.
# ---------------------------------------------------------------------------
@dataclass
class TagLayout:
    bit_x: tuple
    bit_y: tuple
    width_at_border: int
    total_width: int

    @property
    def nbits(self):
        return len(self.bit_x)

    def rotation_perm(self):
        """perm[i] = j: after one quarter turn of the read grid, bit i holds
        what bit j held (cell (x, y) takes the content of cell
        (W - 1 - y, x))."""
        W = self.width_at_border
        where = {(x, y): j for j, (x, y) in enumerate(zip(self.bit_x, self.bit_y))}
        return [where[(W - 1 - y, x)] for x, y in zip(self.bit_x, self.bit_y)]

    def rotate(self, code, turns=1):
        n, perm = self.nbits, self.rotation_perm()
        for _ in range(turns % 4):
            out = 0
            for i, j in enumerate(perm):
                if (code >> (n - 1 - j)) & 1:
                    out |= 1 << (n - 1 - i)
            code = out
        return code

    def cells(self, code):
        """total_width x total_width grid of the rendered tag (True = white):
        quiet zone white, border ring black, data cells from the code, other
        inner cells white."""
        W, T = self.width_at_border, self.total_width
        m = (W - T) // 2  # grid coordinate of cell 0
        g = np.ones((T, T), bool)
        for y in range(T):
            for x in range(T):
                bx, by = x + m, y + m
                if 0 <= bx < W and 0 <= by < W and (bx in (0, W - 1) or by in (0, W - 1)):
                    g[y, x] = False
        n = self.nbits
        for i, (bx, by) in enumerate(zip(self.bit_x, self.bit_y)):
            g[by - m, bx - m] = bool((code >> (n - 1 - i)) & 1)
        return g


def classic_layout(D=6):
    """D x D data bits in row-major order inside a one-cell black border and
    a one-cell white quiet zone (width_at_border D + 2, total_width D + 4)."""
    return TagLayout(tuple(1 + i % D for i in range(D * D)), tuple(1 + i // D for i in range(D * D)), D + 2, D + 4)


def quadrant_layout(D=6):
    """The same cells as classic_layout, with the bits ordered the way the
    AprilTag 3 families order theirs: a quarter of the bits, then the same
    cells turned by one, two and three quarter turns, so that turning the
    tag shifts the code by nbits / 4 bits."""
    assert D % 2 == 0
    W = D + 2
    # one cell of every orbit under quarter turns, in row-major order
    quarter = []
    seen = set()
    for x, y in [(1 + c, 1 + r) for r in range(D) for c in range(D)]:
        orbit = [(x, y)]
        for _ in range(3):
            px, py = orbit[-1]
            orbit.append((W - 1 - py, px))
        if not seen.intersection(orbit):
            quarter.append((x, y))
            seen.update(orbit)
    cells = []
    for k in range(4):
        for x, y in quarter:
            for _ in range(k):
                x, y = y, W - 1 - x  # the cell whose content one quarter turn brings here
            cells.append((x, y))
    return TagLayout(tuple(c[0] for c in cells), tuple(c[1] for c in cells), W, D + 4)


def random_family(layout: TagLayout, n: int, seed: int, min_distance: int = 8):
    """n seeded codes whose distances to each other over all quarter turns,
    and to their own turns, are at least min_distance."""
    rng = np.random.default_rng(seed)
    nb = layout.nbits
    codes = []
    while len(codes) < n:
        c = int(rng.integers(0, 1 << nb, dtype=np.uint64)) if nb < 64 else int(rng.integers(0, 1 << 63)) * 2
        rots = [c] + [layout.rotate(c, k) for k in (1, 2, 3)]
        if any(bin(c ^ r).count("1") < min_distance for r in rots[1:]):
            continue
        if any(bin(r ^ o).count("1") < min_distance for r in rots for o in codes):
            continue
        codes.append(c)
    return codes


def _render_cells(img, quad, grid):
    """Paints a T x T cell grid (True = white) onto the image through the
    homography that maps the grid square onto `quad`."""
    h, w = img.shape
    T = grid.shape[0]
    H = _homography(quad, np.array([[0, 0], [T, 0], [T, T], [0, T]], np.float64))
    x0 = int(max(0, np.floor(quad[:, 0].min())))
    x1 = int(min(w - 1, np.ceil(quad[:, 0].max())))
    y0 = int(max(0, np.floor(quad[:, 1].min())))
    y1 = int(min(h - 1, np.ceil(quad[:, 1].max())))
    if x1 <= x0 or y1 <= y0:
        return
    ys, xs = np.mgrid[y0:y1 + 1, x0:x1 + 1]
    X, Y = xs + 0.5, ys + 0.5
    d = H[2, 0] * X + H[2, 1] * Y + H[2, 2]
    u = (H[0, 0] * X + H[0, 1] * Y + H[0, 2]) / d
    v = (H[1, 0] * X + H[1, 1] * Y + H[1, 2]) / d
    inside = (u >= 0) & (u < T) & (v >= 0) & (v < T)
    val = np.where(grid[np.clip(v.astype(np.int64), 0, T - 1), np.clip(u.astype(np.int64), 0, T - 1)], 255, 0)
    sub = img[y0:y1 + 1, x0:x1 + 1]
    sub[inside] = val[inside].astype(np.float32)


def family_frame(seed: int, layout: TagLayout, codes, n_tags: int = 12, width: int = 1280, height: int = 720,
                 blur: float = 0.6, noise: float = 2.0, max_tilt_deg: float = 30.0):
    """A frame of n_tags tags of a family on a noisy grey background.
    Returns the uint8 image and, per tag, (code index, the outer corners of
    its black border with pixel centres at integer coordinates, in the order
    that reads the tag unturned)."""
    rng = np.random.default_rng(seed)
    img = rng.uniform(100, 160, size=(height, width)).astype(np.float32)
    T, W = layout.total_width, layout.width_at_border
    m = (T - W) // 2
    tags, boxes = [], []
    while len(tags) < n_tags:
        side = rng.uniform(60, 160)
        cx, cy = rng.uniform(side, width - side), rng.uniform(side, height - side)
        if any(abs(cx - bx) < (side + bs) * 0.75 and abs(cy - by) < (side + bs) * 0.75 for bx, by, bs in boxes):
            continue
        boxes.append((cx, cy, side))
        quad = _tag_quad(rng, cx, cy, side, max_tilt_deg)
        k = int(rng.integers(0, len(codes)))
        _render_cells(img, quad, layout.cells(codes[k]))
        H = _homography(np.array([[0, 0], [T, 0], [T, T], [0, T]], np.float64), quad)
        inner = np.array([[m, m, 1], [m + W, m, 1], [m + W, m + W, 1], [m, m + W, 1]], np.float64)
        p = inner @ H.T
        tags.append((k, p[:, :2] / p[:, 2:] - 0.5))
    img = _blur(img, blur) + rng.normal(0, noise, size=img.shape).astype(np.float32)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8), tags
