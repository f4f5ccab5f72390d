"""CPU checks of the tag-reading oracle (oracle/decode_ref.py) on tags of a
seeded random code family rendered with known codes; the CUDA kernel is
checked against it in test_gpu_decode.py."""
import numpy as np

from conftest import family_frame
from decode_ref import DEGENERATE, LOW_CONTRAST, REORDERED, decode_one, random_family, rotate90

FAMILY = random_family(48, seed=1)


def test_family_is_well_separated():
    for i, a in enumerate(FAMILY):
        r = a
        for _ in range(4):
            for b in FAMILY[i + 1:]:
                assert bin(r ^ b).count("1") >= 8
            r = rotate90(r, 6)
        assert rotate90(rotate90(rotate90(rotate90(a, 6), 6), 6), 6) == a


def test_rendered_tags_read_back_in_every_corner_order():
    img, tags = family_frame(3, FAMILY)
    for k, quad in tags:
        rots = set()
        for s in range(4):
            d = decode_one(img, np.roll(quad, s, axis=0), FAMILY)
            assert d["id"] == k and d["hamming"] == 0 and d["status"] == 0
            assert d["white"] - d["black"] > 40 and d["margin"] > 5
            rots.add(d["rotation"])
        assert rots == {0, 1, 2, 3}
        m = decode_one(img, quad[[0, 3, 2, 1]], FAMILY)
        assert m["id"] == k and m["status"] == REORDERED


def test_unmatched_flat_and_degenerate_quads():
    img, tags = family_frame(4, FAMILY, n_tags=4)
    # a quad on the background: no contrast between border and ring
    flat = np.array([[20.0, 20.0], [60.0, 20.0], [60.0, 60.0], [20.0, 60.0]])
    bg = np.full_like(img, 128)
    assert decode_one(bg, flat, FAMILY)["status"] & LOW_CONTRAST
    line = np.array([[10.0, 10.0], [20.0, 10.0], [30.0, 10.0], [40.0, 10.0]])
    assert decode_one(img, line, FAMILY)["status"] & DEGENERATE
    # a family without the tag's code: nothing within two bits
    k, quad = tags[0]
    others = [c for i, c in enumerate(FAMILY) if i != k]
    assert decode_one(img, quad, others)["id"] == -1
