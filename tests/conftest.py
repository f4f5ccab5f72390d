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
