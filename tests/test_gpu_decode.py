"""The CUDA tag reader (atag_decode_quads) against the oracle
(oracle/decode_ref.py) on the detector's own quads of frames with tags of
seeded random code families, in the row-major and the AprilTag 3 quadrant
bit order."""
import numpy as np
import pytest

from decode_ref import decode_one

from atag import synth

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

LAYOUTS = {"classic": synth.classic_layout(6), "quadrant": synth.quadrant_layout(6)}
FAMILIES = {k: synth.random_family(L, 48, seed=1) for k, L in LAYOUTS.items()}


def _detect(img):
    from atag.detector import Detector
    det = Detector(img.shape[1], img.shape[0])
    quads, st = det.detect([torch.from_numpy(img).cuda()])
    return quads[0]


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_detected_quads_decode_as_the_oracle_reads_them(name):
    from atag import decode
    from atag.records import QUAD_CORNERS
    L, codes = LAYOUTS[name], FAMILIES[name]
    fam = decode.Family(L, codes)
    for seed in (5, 6):
        img, tags = synth.family_frame(seed, L, codes, n_tags=14)
        q = _detect(img)
        assert len(q) >= len(tags)
        rec = torch.from_numpy(np.frombuffer(q.tobytes(), np.uint8).reshape(len(q), QUAD_CORNERS.itemsize).copy())
        gi = torch.from_numpy(img).cuda()
        g = decode.to_numpy(decode.decode_quads(gi, rec.cuda(), fam))
        g2 = decode.to_numpy(decode.decode_quads(gi, torch.from_numpy(q["corners"].copy()).cuda(), fam))
        assert g.tobytes() == g2.tobytes()  # records and packed corners
        for i in range(len(q)):
            o = decode_one(img, q["corners"][i], L, codes)
            assert int(g["status"][i]) == o["status"], i
            assert np.abs(g["corners"][i] - o["corners"]).max() < 1e-3, i
            if o["status"]:
                continue
            assert abs(float(g["black"][i]) - o["black"]) < 1e-3 and abs(float(g["white"][i]) - o["white"]) < 1e-3
            assert abs(float(g["decision_margin"][i]) - o["decision_margin"]) < 1e-3
            assert int(g["code"][i]) == o["code"]
            assert int(g["id"][i]) == o["id"] and int(g["hamming"][i]) == o["hamming"]
            if o["id"] >= 0:
                assert int(g["rotation"][i]) == o["rotation"]
        ids = sorted(int(v) for v in g["id"] if v >= 0)
        # every rendered tag is read, nothing else matches the family
        assert ids == sorted(k for k, _ in tags)


def test_decoded_corners_start_at_the_tags_first_corner():
    """Whatever the detector's corner order, a matched tag's reported
    corners begin at the same physical corner: the one that reads it
    unturned."""
    from atag import decode
    L, codes = LAYOUTS["quadrant"], FAMILIES["quadrant"]
    fam = decode.Family(L, codes)
    img, tags = synth.family_frame(8, L, codes, n_tags=6)
    gi = torch.from_numpy(img).cuda()
    for k, quad in tags:
        outs = []
        for s in range(4):
            c = torch.from_numpy(np.roll(quad, s, axis=0)[None].astype(np.float32).copy()).cuda()
            d = decode.to_numpy(decode.decode_quads(gi, c, fam))[0]
            assert int(d["id"]) == k
            outs.append(d["corners"])
        for o in outs[1:]:
            assert np.abs(o - outs[0]).max() < 1e-3


def test_empty_family_and_argument_errors():
    import ctypes
    from atag import decode, lib
    from atag.records import DecodeParams, TagFamily
    L, codes = LAYOUTS["classic"], FAMILIES["classic"]
    img, _ = synth.family_frame(7, L, codes, n_tags=3)
    q = _detect(img)
    g = decode.to_numpy(decode.decode_quads(torch.from_numpy(img).cuda(), torch.from_numpy(q["corners"].copy()).cuda(),
                                            decode.Family(L, [])))
    assert np.all(g["id"] == -1)
    Lib = lib.init()
    P = ctypes.c_void_p
    c = torch.zeros((1, 4, 2), dtype=torch.float32, device="cuda")
    im = torch.zeros((8, 8), dtype=torch.uint8, device="cuda")
    out = torch.empty((1, 72), dtype=torch.uint8, device="cuda")
    fam = decode.Family(L, codes)

    def call(f, pitch=8, prm=None):
        return Lib.atag_decode_quads(P(im.data_ptr()), 8, 8, pitch, P(c.data_ptr()), 32, 1, ctypes.byref(f),
                                     ctypes.byref(prm) if prm is not None else None, P(out.data_ptr()), None)
    assert call(fam.struct()) == 0
    assert call(fam.struct(), pitch=4) != 0  # pitch below width
    bad = fam.struct()
    bad.total_width = 18  # above the 16-cell grid
    assert call(bad) != 0
    bad = fam.struct()
    bad.nbits = 65
    assert call(bad) != 0
    # a layout that a quarter turn does not carry onto itself
    bx = np.ascontiguousarray(L.bit_x, dtype=np.int8).copy()
    bx[0] = 0
    by = np.ascontiguousarray(L.bit_y, dtype=np.int8).copy()
    by[0] = 0
    bad = fam.struct()
    bad.h_bit_x, bad.h_bit_y = bx.ctypes.data, by.ctypes.data
    assert call(bad) != 0
    p = DecodeParams()
    Lib.atag_decode_params_default(ctypes.byref(p))
    p.quad_decimate = 0
    assert call(fam.struct(), prm=p) != 0
    assert isinstance(TagFamily(), ctypes.Structure)
