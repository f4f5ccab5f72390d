import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "sycl-apriltag-test_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def ref_images():
    """The reference project's three input images (decimate.png 420x312,
    decimate4.png 960x540, decimate2.png 1920x1080), decoded."""
    with np.load(os.path.join(GOLDEN, "reference_images.npz")) as z:
        return {k: z[k] for k in z.files}


_SYNTH = {}


def synth_frame(name: str, seed: int):
    from atag import synth
    key = (name, seed)
    if key not in _SYNTH:
        _SYNTH[key] = synth.render(synth.CONFIGS[name], seed)
    return _SYNTH[key]


def small_frames():
    """Hand-sized frames for edge cases: tiny, ragged aspect, flat, noise."""
    rng = np.random.default_rng(7)
    out = {
        "4x4": rng.integers(0, 256, (4, 4), dtype=np.uint8),
        "8x12": rng.integers(0, 256, (8, 12), dtype=np.uint8),
        "flat": np.full((64, 64), 100, np.uint8),
        "noise_64": rng.integers(0, 256, (64, 64), dtype=np.uint8),
        "noise_68x132": rng.integers(0, 256, (68, 132), dtype=np.uint8),
        "checker": ((np.indices((96, 128)).sum(0) // 8) % 2 * 255).astype(np.uint8),
    }
    # blocky random pattern (large components, bridges through 2x2 blocks)
    b = rng.integers(0, 2, (20, 28)).astype(np.uint8) * 255
    out["blocky"] = np.kron(b, np.ones((4, 4), np.uint8))
    # a clean black square on white (one quad)
    sq = np.full((120, 160), 230, np.uint8)
    sq[30:90, 50:110] = 20
    sq[45:75, 65:95] = 230
    out["square"] = sq
    return out


def family_frame(seed: int, codes, n_tags: int = 12, width: int = 1280, height: int = 720, blur: float = 0.6,
                 noise: float = 2.0):
    """A frame with n_tags tags of the given code family (10 x 10 cells:
    white quiet zone, black border, 6 x 6 data bits) on a noisy grey
    background.  Returns the uint8 image and, per tag, (code index, the
    corners of the black border's outer edge with pixel centres at integer
    coordinates)."""
    import numpy as np
    from atag import synth
    from decode_ref import code_bits
    rng = np.random.default_rng(seed)
    img = rng.uniform(100, 160, size=(height, width)).astype(np.float32)
    tags, boxes = [], []
    while len(tags) < n_tags:
        side = rng.uniform(60, 160)
        cx, cy = rng.uniform(side, width - side), rng.uniform(side, height - side)
        if any(abs(cx - bx) < (side + bs) * 0.75 and abs(cy - by) < (side + bs) * 0.75 for bx, by, bs in boxes):
            continue
        boxes.append((cx, cy, side))
        quad = synth._tag_quad(rng, cx, cy, side, 30.0)  # the 10-cell square, pixel centres at +0.5
        k = int(rng.integers(0, len(codes)))
        synth._render_tag(img, rng, quad, code_bits(codes[k]))
        # the black border's outer edge is cells 1..9 of the 10-cell square
        H = synth._homography(np.array([[0, 0], [10, 0], [10, 10], [0, 10]], np.float64), quad)
        inner = np.array([[1, 1], [9, 1], [9, 9], [1, 9]], np.float64)
        p = np.c_[inner, np.ones(4)] @ H.T
        tags.append((k, p[:, :2] / p[:, 2:] - 0.5))
    img = synth._blur(img, blur) + rng.normal(0, noise, size=img.shape).astype(np.float32)
    return np.clip(np.rint(img), 0, 255).astype(np.uint8), tags
