"""The CUDA pose kernel (atag_estimate_pose) against the FP64 oracle
(oracle/pose_ref.py) and against ground-truth poses."""
import numpy as np
import pytest

from conftest import synth_frame
from pose_ref import DEGENERATE, REORDERED, estimate_pose_one, random_poses

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

CAM = (1000.0, 1000.0, 960.0, 540.0)
TAG = 0.16
# FP64 on both sides, but the kernel may contract a*b+c into one rounding:
# the homography's pose agrees to rounding; after Levenberg-Marquardt the
# minimum of a small noisy tag's reprojection error is flat, and rounding
# moves the converged pose along it by up to ~1e-8 while the error itself
# agrees to rounding.
TOL_INIT, TOL_LM = 1e-9, 1e-6


def _gpu(corners, max_iterations=20):
    from atag import pose
    c = torch.from_numpy(np.ascontiguousarray(corners, dtype=np.float32)).cuda()
    return pose.to_numpy(pose.estimate_pose(c, *CAM, TAG, max_iterations=max_iterations))


def _check(g, o, tol):
    assert int(g["status"]) == o["status"]
    if o["status"] & DEGENERATE:
        return
    assert np.max(np.abs(g["R"] - o["R"])) < tol
    assert np.max(np.abs(g["t"] - o["t"])) < tol * max(1.0, np.max(np.abs(o["t"])))
    assert np.max(np.abs(g["H"] - o["H"]) / np.maximum(1.0, np.abs(o["H"]))) < tol
    assert abs(float(g["reproj_rms"]) - o["reproj_rms"]) < 1e-9 * max(1.0, o["reproj_rms"])
    if tol == TOL_INIT:
        # the number of accepted steps along a flat minimum depends on
        # rounding, so it is compared only without iterations
        assert int(g["iterations"]) == o["iterations"]


@pytest.mark.parametrize("max_iterations", [0, 20])
def test_kernel_matches_oracle_on_noisy_corners(max_iterations):
    rng = np.random.default_rng(11)
    poses = random_poses(400, seed=11)
    corners = np.stack([c for _, _, c in poses]) + rng.normal(scale=0.4, size=(400, 4, 2))
    corners = corners.astype(np.float32)
    corners[::7] = corners[::7][:, [0, 3, 2, 1]]  # the other winding
    g = _gpu(corners, max_iterations)
    for i in range(len(corners)):
        _check(g[i], estimate_pose_one(corners[i], CAM, TAG, max_iterations), TOL_INIT if max_iterations == 0 else TOL_LM)
    assert np.all(g["status"][::7] == REORDERED)


def test_kernel_recovers_ground_truth():
    poses = random_poses(300, seed=12)
    g = _gpu(np.stack([c for _, _, c in poses]))
    for (R, t, _), p in zip(poses, g):
        assert int(p["status"]) == 0
        assert float(p["reproj_rms"]) < 1e-3  # float32 corners
        assert np.max(np.abs(p["R"] - R)) < 1e-3
        assert np.linalg.norm(p["t"] - t) < 1e-3 * np.linalg.norm(t)


def test_degenerate_quads_are_flagged_and_zeroed():
    c = np.array([[[100, 100], [200, 100], [300, 100], [150, 100]],
                  [[500, 500], [500, 500], [500, 500], [500, 500]]], np.float32)
    g = _gpu(c)
    assert np.all(g["status"] & DEGENERATE)
    assert not np.any(g["R"]) and not np.any(g["t"])


def test_detector_records_and_packed_corners_agree():
    from atag import pose
    from atag.detector import Detector
    from atag.records import QUAD_CORNERS
    det = Detector(1920, 1080)
    quads, st = det.detect([torch.from_numpy(synth_frame("1080p", 1)).cuda()])
    q = quads[0]
    assert len(q) > 10
    rec = torch.from_numpy(np.frombuffer(q.tobytes(), np.uint8).reshape(len(q), QUAD_CORNERS.itemsize).copy()).cuda()
    a = pose.to_numpy(pose.estimate_pose(rec, *CAM, TAG))
    b = _gpu(q["corners"])
    assert a.tobytes() == b.tobytes()
    assert np.count_nonzero(a["status"] & DEGENERATE) == 0


def test_invalid_arguments_raise():
    from atag import lib
    L = lib.init()
    out = torch.empty((1, 184), dtype=torch.uint8, device="cuda")
    c = torch.zeros((1, 4, 2), dtype=torch.float32, device="cuda")
    import ctypes
    P = ctypes.c_void_p
    assert L.atag_estimate_pose(P(c.data_ptr()), 30, 1, 1.0, 1.0, 0.0, 0.0, 1.0, 20, P(out.data_ptr()), None) != 0
    assert L.atag_estimate_pose(None, 32, 1, 1.0, 1.0, 0.0, 0.0, 1.0, 20, P(out.data_ptr()), None) != 0
    assert L.atag_estimate_pose(P(c.data_ptr()), 32, 1, 1.0, 1.0, 0.0, 0.0, -1.0, 20, P(out.data_ptr()), None) != 0
    assert L.atag_estimate_pose(P(c.data_ptr()), 32, 0, 1.0, 1.0, 0.0, 0.0, 1.0, 20, None, None) == 0
