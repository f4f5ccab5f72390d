"""The CUDA tag reader (atag_decode_quads) against the oracle
(oracle/decode_ref.py) on the detector's own quads of frames with tags of a
seeded random code family."""
import numpy as np
import pytest

from conftest import family_frame
from decode_ref import decode_one, random_family

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

FAMILY = random_family(48, seed=1)


def _detect(img):
    from atag.detector import Detector
    det = Detector(img.shape[1], img.shape[0])
    quads, st = det.detect([torch.from_numpy(img).cuda()])
    return quads[0]


def test_detected_quads_decode_as_the_oracle_reads_them():
    from atag import decode
    from atag.records import QUAD_CORNERS
    for seed in (5, 6):
        img, tags = family_frame(seed, FAMILY, n_tags=14)
        q = _detect(img)
        assert len(q) >= len(tags)
        rec = torch.from_numpy(np.frombuffer(q.tobytes(), np.uint8).reshape(len(q), QUAD_CORNERS.itemsize).copy())
        gi = torch.from_numpy(img).cuda()
        g = decode.to_numpy(decode.decode_quads(gi, rec.cuda(), FAMILY))
        g2 = decode.to_numpy(decode.decode_quads(gi, torch.from_numpy(q["corners"].copy()).cuda(), FAMILY))
        assert g.tobytes() == g2.tobytes()  # records and packed corners
        for i in range(len(q)):
            o = decode_one(img, q["corners"][i], FAMILY)
            assert int(g["status"][i]) == o["status"]
            assert abs(float(g["black"][i]) - o["black"]) < 1e-3 and abs(float(g["white"][i]) - o["white"]) < 1e-3
            if o["margin"] > 1e-6:  # FP64 on both sides; a sample exactly at the threshold may differ
                assert int(g["code"][i]) == o["code"]
                assert int(g["id"][i]) == o["id"] and int(g["hamming"][i]) == o["hamming"]
                if o["id"] >= 0:
                    assert int(g["rotation"][i]) == o["rotation"]
        ids = sorted(int(v) for v in g["id"] if v >= 0)
        # every rendered tag is read, nothing else matches the family
        assert ids == sorted(k for k, _ in tags)


def test_empty_family_and_argument_errors():
    import ctypes
    from atag import decode, lib
    img, _ = family_frame(7, FAMILY, n_tags=3)
    q = _detect(img)
    g = decode.to_numpy(decode.decode_quads(torch.from_numpy(img).cuda(), torch.from_numpy(q["corners"].copy()).cuda(),
                                            np.zeros(0, np.uint64)))
    assert np.all(g["id"] == -1)
    L = lib.init()
    P = ctypes.c_void_p
    c = torch.zeros((1, 4, 2), dtype=torch.float32, device="cuda")
    im = torch.zeros((8, 8), dtype=torch.uint8, device="cuda")
    out = torch.empty((1, 40), dtype=torch.uint8, device="cuda")
    assert L.atag_decode_quads(P(im.data_ptr()), 8, 8, 8, P(c.data_ptr()), 32, 1, None, 0, 9, 2, 10.0,
                               P(out.data_ptr()), None) != 0  # data_side above 8
    assert L.atag_decode_quads(P(im.data_ptr()), 8, 8, 4, P(c.data_ptr()), 32, 1, None, 0, 6, 2, 10.0,
                               P(out.data_ptr()), None) != 0  # pitch below width
    assert L.atag_decode_quads(None, 8, 8, 8, P(c.data_ptr()), 32, 1, None, 0, 6, 2, 10.0,
                               P(out.data_ptr()), None) != 0
