"""Colour input on the GPU (colour removal fused with decimation): the
conversion stage against the oracle (itself pinned to the reference's stb
loader by tests/golden/colour.npz) for every pixel format, factor and a
padded row pitch; and detection on colour frames equal, byte for byte, to
detection on their grey conversion, alone and mixed in a batch."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, synth_frame

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PIX_GREY8, PIX_RGB8, PIX_RGBA8, PIX_BGR8, PIX_BGRA8, PIX_GREYA8 = range(6)
CHANNELS = {PIX_GREY8: 1, PIX_RGB8: 3, PIX_RGBA8: 4, PIX_BGR8: 3, PIX_BGRA8: 4, PIX_GREYA8: 2}


def _tint(grey, channels, seed):
    rng = np.random.default_rng(seed)
    g = grey.astype(np.int32)
    chans = [np.clip(g * rng.uniform(0.7, 1.15) + rng.integers(-30, 30), 0, 255) for _ in range(channels)]
    return np.stack(chans, axis=-1).astype(np.uint8)


def test_conversion_matches_oracle_for_every_format():
    from atag import stages
    rng = np.random.default_rng(3)
    for fmt, c in CHANNELS.items():
        for factor in (1, 2, 3):
            h, w = 4 * factor * 9, 4 * factor * 13
            img = rng.integers(0, 256, (h, w) if c == 1 else (h, w, c), dtype=np.uint8)
            got = stages.convert_grey(torch.from_numpy(img).cuda(), factor, fmt).cpu().numpy()
            assert np.array_equal(got, oracle.to_grey(img, factor, fmt)), (fmt, factor)


def test_conversion_with_padded_rows():
    from atag import lib
    L = lib.init()
    img = np.random.default_rng(5).integers(0, 256, (40, 48, 3), dtype=np.uint8)
    padded = np.zeros((40, 48 * 3 + 32), np.uint8)
    padded[:, : 48 * 3] = img.reshape(40, -1)
    d_src = torch.from_numpy(padded).cuda()
    out = torch.empty((20, 24), dtype=torch.uint8, device="cuda")
    s = torch.cuda.current_stream()
    lib.check(L.atag_convert_grey(d_src.data_ptr(), 48, 40, padded.shape[1], PIX_RGB8, 2, out.data_ptr(),
                                  s.cuda_stream), "convert_grey")
    assert np.array_equal(out.cpu().numpy(), oracle.to_grey(img, 2))


def test_golden_colour_images_on_the_device():
    from atag import stages
    with np.load(os.path.join(GOLDEN, "colour.npz")) as z:
        cases = {k: z[k] for k in z.files}
    for name in (k for k in cases if not k.endswith("_grey")):
        img = cases[name]
        h, w = img.shape[0] // 4 * 4, img.shape[1] // 4 * 4
        img = np.ascontiguousarray(img[:h, :w])
        got = stages.convert_grey(torch.from_numpy(img).cuda()).cpu().numpy()
        assert np.array_equal(got, cases[name + "_grey"][:h, :w]), name


@pytest.mark.parametrize("decimate", [1, 2])
def test_detection_on_colour_frames_equals_grey(decimate):
    from atag import lib
    from atag.detector import Detector
    cfg = lib.default_config(decimate=decimate)
    greys = [synth_frame("vga", 21), synth_frame("1080p", 22)]
    colours = [_tint(greys[0], 3, 1), _tint(greys[1], 4, 2)]
    converted = [oracle.to_grey(c) for c in colours]
    det = Detector(1920 // decimate, 1080 // decimate, max_frames=4, config=cfg)
    want, _ = det.detect([torch.from_numpy(g).cuda() for g in converted])
    got, st = det.detect([torch.from_numpy(c).cuda() for c in colours])
    for a, b in zip(got, want):
        assert a.tobytes() == b.tobytes()
    assert sum(len(a) for a in got) > 0
    # mixed in one batch with a grey frame and a BGR one
    bgr = colours[0][..., ::-1].copy()
    mixed = [torch.from_numpy(greys[0]).cuda(), torch.from_numpy(colours[1]).cuda(), torch.from_numpy(bgr).cuda()]
    q, _ = det.detect(mixed, formats=[PIX_GREY8, PIX_RGBA8, PIX_BGR8])
    alone_grey, _ = det.detect([torch.from_numpy(greys[0]).cuda()])
    assert q[0].tobytes() == alone_grey[0].tobytes()
    assert q[1].tobytes() == want[1].tobytes()
    assert q[2].tobytes() == want[0].tobytes()
