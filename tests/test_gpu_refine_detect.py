"""Corner refinement inside detection (atag_detector_set_refinement): on
synthetic frames whose true tag corners the generator knows, the refined
corners lie closer to the truth than the reference path's corners (the FP64
intersections of its line fits, src/main.cpp:1059-1099), and the stage
changes nothing else."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def match_errors(quads, truth, gate=3.0):
    """Per matched quad: the largest corner distance to its true quad (over
    the corner order and winding that fit best); quads farther than `gate`
    px from every true quad (clutter, covered tags) are left out."""
    out = []
    for q in quads:
        c = q["corners"].astype(np.float64)
        best = None
        for t in truth:
            for order in (t, t[::-1]):
                for k in range(4):
                    d = np.linalg.norm(np.roll(order, k, axis=0) - c, axis=1).max()
                    best = d if best is None or d < best else best
        if best is not None and best < gate:
            out.append(best)
    return np.array(out)


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
        m0, m1 = match_errors(q0[0], truth), match_errors(q1[0], truth)
        assert len(m0) >= 10 and len(m1) == len(m0)
        e0.append(m0)
        e1.append(m1)
    e0, e1 = np.concatenate(e0), np.concatenate(e1)
    print(f"max corner error per quad vs truth: unrefined mean {e0.mean():.3f} px, median {np.median(e0):.3f}; "
          f"refined mean {e1.mean():.3f} px, median {np.median(e1):.3f} ({len(e0)} quads)")
    assert e1.mean() < 0.75 * e0.mean()
    assert np.median(e1) < np.median(e0)


def test_refinement_stage_equals_refine_forward():
    """The in-detector stage gives atag_refine_forward's corners on the
    frame's FP32-normalised grey image."""
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
    r, _, _ = refine.refine_forward(t.float().div(255.0), corners)
    want = r.cpu().numpy()
    got = q1[0]["corners"]
    same = (got == want).all(axis=2)
    kept = (got == q0[0]["corners"]).all(axis=2)  # nearly parallel edge lines
    assert np.all(same | kept)
    assert same.mean() > 0.95
