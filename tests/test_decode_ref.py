"""CPU checks of the tag-reading oracle (oracle/decode_ref.py) on tags of
seeded random code families rendered with known codes, in two bit layouts:
row-major (classic) and the quadrant order of the AprilTag 3 families,
where bits are not in row order; the CUDA kernel is checked against it in
test_gpu_decode.py."""
import numpy as np
import pytest

from decode_ref import DEGENERATE, LOW_CONTRAST, REORDERED, decode_one, rotate, rotation_perm

from atag import synth

LAYOUTS = {"classic": synth.classic_layout(6), "quadrant": synth.quadrant_layout(6)}
FAMILIES = {k: synth.random_family(L, 48, seed=1) for k, L in LAYOUTS.items()}


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_family_is_well_separated_and_turns_compose(name):
    L, fam = LAYOUTS[name], FAMILIES[name]
    perm = rotation_perm(L.bit_x, L.bit_y, L.width_at_border)
    for i, a in enumerate(fam):
        r = a
        for _ in range(4):
            for b in fam[i + 1:]:
                assert bin(r ^ b).count("1") >= 8
            assert rotate(r, perm, 36) == L.rotate(r)
            r = rotate(r, perm, 36)
        assert r == a


def test_quadrant_order_is_a_cyclic_shift():
    """In the AprilTag 3 order a quarter turn moves every bit by nbits / 4."""
    L = LAYOUTS["quadrant"]
    c = 0x9A3C5F0E1
    r = L.rotate(c)
    assert r == ((c >> 9) | (c << 27)) & ((1 << 36) - 1)


@pytest.mark.parametrize("name", sorted(LAYOUTS))
def test_rendered_tags_read_back_in_every_corner_order(name):
    L, fam = LAYOUTS[name], FAMILIES[name]
    img, tags = synth.family_frame(3, L, fam, n_tags=6)
    for k, quad in tags:
        rots = set()
        for s in range(4):
            d = decode_one(img, np.roll(quad, s, axis=0), L, fam)
            assert d["id"] == k and d["hamming"] == 0 and d["status"] == 0
            assert d["white"] - d["black"] > 40 and d["decision_margin"] > 10
            rots.add(d["rotation"])
            # the reported corners start at the tag's own first corner
            assert np.abs(d["corners"] - decode_one(img, quad, L, fam)["corners"]).max() < 1e-9
        assert rots == {0, 1, 2, 3}
        m = decode_one(img, quad[[0, 3, 2, 1]], L, fam)
        assert m["id"] == k and m["status"] == REORDERED


def test_edge_refinement_moves_corners_onto_the_edges():
    """Corners pushed up to 0.8 px off the tag come back within 0.45 px of
    where the unperturbed corners refine to; without refinement they stay."""
    L, fam = LAYOUTS["classic"], FAMILIES["classic"]
    img, tags = synth.family_frame(5, L, fam, n_tags=4)
    rng = np.random.default_rng(0)
    for k, quad in tags:
        base = decode_one(img, quad, L, fam)["corners"]
        moved = quad + rng.uniform(-0.8, 0.8, size=quad.shape)
        d = decode_one(img, moved, L, fam)
        assert d["id"] == k
        assert np.abs(d["corners"] - base).max() < 0.45
        nr = decode_one(img, moved, L, fam, refine=False)
        assert np.abs(nr["corners"] - moved).max() < 1e-9


def test_unmatched_flat_degenerate_and_behind_camera_quads():
    L, fam = LAYOUTS["classic"], FAMILIES["classic"]
    img, tags = synth.family_frame(4, L, fam, n_tags=4)
    sq = np.array([[20.0, 20.0], [60.0, 20.0], [60.0, 60.0], [20.0, 60.0]])
    bg = np.full_like(img, 128)
    # a flat patch: no contrast between the grey models
    assert decode_one(bg, sq, L, fam, min_contrast=10.0)["status"] & LOW_CONTRAST
    assert decode_one(bg, sq, L, fam)["id"] == -1
    line = np.array([[10.0, 10.0], [20.0, 10.0], [30.0, 10.0], [40.0, 10.0]])
    assert decode_one(img, line, L, fam)["status"] & DEGENERATE
    # a self-crossing quad: part of the tag square maps behind the camera
    bow = np.array([[200.0, 200.0], [260.0, 260.0], [260.0, 200.0], [200.0, 260.0]])
    assert decode_one(img, bow, L, fam, refine=False)["status"] & DEGENERATE
    # a family without the tag's code: nothing within two bits
    k, quad = tags[0]
    others = [c for i, c in enumerate(fam) if i != k]
    assert decode_one(img, quad, L, others)["id"] == -1


def test_reversed_border_reads_inverted_tags():
    """A family flagged with a reversed border (white border on black) reads
    the inverted image of its tags against the complemented codes; read as a
    normal border the same quads are rejected by the grey models."""
    L, fam = LAYOUTS["classic"], FAMILIES["classic"]
    img, tags = synth.family_frame(6, L, fam, n_tags=3)
    inv = 255 - img
    comp = [~c & ((1 << 36) - 1) for c in fam]
    for k, quad in tags:
        assert decode_one(inv, quad, L, comp, reversed_border=True)["id"] == k
        assert decode_one(inv, quad, L, comp)["status"] & LOW_CONTRAST
