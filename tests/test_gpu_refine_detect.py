"""Corner refinement inside detection (atag_detector_set_refinement): on
synthetic frames whose true tag corners the generator knows, the refined
corners lie closer to the truth than the reference path's corners (the FP64
intersections of its line fits, src/main.cpp:1059-1099), and the stage
changes nothing else."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def best_truth(c, truth):
    """(largest corner distance, true corners in the matching order) of the
    true quad closest to corners c, over corner order and winding."""
    best = (np.inf, None)
    for t in truth:
        for order in (t, t[::-1]):
            for k in range(4):
                o = np.roll(order, k, axis=0)
                d = np.linalg.norm(o - c, axis=1).max()
                if d < best[0]:
                    best = (d, o)
    return best


def paired_errors(q0, q1, truth, gate=3.0):
    """For each unrefined quad within `gate` px of a tag (not clutter or a
    covered tag): its largest corner error and that of the same quad
    refined, against the same true corners."""
    e0, e1 = [], []
    for a, b in zip(q0, q1):
        d, t = best_truth(a["corners"].astype(np.float64), truth)
        if d < gate:
            e0.append(d)
            e1.append(np.linalg.norm(b["corners"].astype(np.float64) - t, axis=1).max())
    return np.array(e0), np.array(e1)


def test_refined_corners_are_closer_to_truth():
    from atag import synth
    from atag.detector import Detector
    plain, refined = Detector(1920, 1080), Detector(1920, 1080)
    refined.set_refinement(True)
    e0, e1 = [], []
    for seed in range(4):
        truth = []
        img = synth.render(synth.CONFIGS["1080p"], 700 + seed, truth=truth)
        t = torch.from_numpy(img).cuda()
        q0, s0 = plain.detect([t])
        q1, s1 = refined.detect([t])
        # the same quads, in the same order, only their corners moved
        assert s0.tobytes() == s1.tobytes()
        assert len(q0[0]) == len(q1[0])
        assert np.array_equal(q0[0]["blob_index"], q1[0]["blob_index"])
        m0, m1 = paired_errors(q0[0], q1[0], truth)
        assert len(m0) >= 10
        e0.append(m0)
        e1.append(m1)
    e0, e1 = np.concatenate(e0), np.concatenate(e1)
    print(f"largest corner error per quad vs truth ({len(e0)} quads): unrefined median {np.median(e0):.3f} px, "
          f"mean {e0.mean():.3f}; refined median {np.median(e1):.3f} px, mean {e1.mean():.3f}; "
          f"refined closer for {np.mean(e1 < e0):.0%}")
    assert np.median(e1) < 0.75 * np.median(e0)
    assert np.mean(e1 < e0) > 0.8


def test_refinement_stage_equals_refine_forward():
    """The in-detector stage gives atag_refine_forward's corners (within
    1e-3 px) on the frame's FP32-normalised grey image."""
    from atag import refine, synth
    from atag.detector import Detector
    img = synth.render(synth.CONFIGS["1080p"], 711)
    t = torch.from_numpy(img).cuda()
    plain = Detector(1920, 1080)
    q0, _ = plain.detect([t])
    det = Detector(1920, 1080)
    det.set_refinement(True)
    q1, _ = det.detect([t])
    corners = torch.from_numpy(q0[0]["corners"].copy()).cuda()
    # value / 255 with IEEE division (numpy), as the stage reads the u8 frame
    r, _, _ = refine.refine_forward(torch.from_numpy(img.astype(np.float32) / np.float32(255.0)).cuda(), corners)
    want = r.cpu().numpy()
    got = q1[0]["corners"]
    # the same arithmetic in two instantiations; FMA contraction may differ
    same = (np.abs(got - want) < 1e-3).all(axis=2)
    kept = (got == q0[0]["corners"]).all(axis=2)  # nearly parallel edge lines
    assert np.all(same | kept)
    assert same.mean() > 0.95
