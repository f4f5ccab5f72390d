"""CPU checks of the pose oracle (oracle/pose_ref.py) against ground truth:
corners projected from known poses give those poses back; the checks that
the CUDA kernel matches the oracle are in test_gpu_pose.py."""
import math

import numpy as np

from pose_ref import DEGENERATE, REORDERED, estimate_pose_one, project, random_poses, so3_exp

CAM = (1000.0, 1000.0, 960.0, 540.0)
TAG = 0.16


def _rot_err(A, B):
    """Angle of A^T B in radians, from the sine and the cosine (acos alone
    loses half the digits near zero)."""
    M = A.T @ B
    s = 0.5 * math.sqrt((M[2, 1] - M[1, 2]) ** 2 + (M[0, 2] - M[2, 0]) ** 2 + (M[1, 0] - M[0, 1]) ** 2)
    return math.atan2(s, (np.trace(M) - 1.0) / 2.0)


def test_exact_corners_give_the_pose_back():
    for R, t, c in random_poses(200, seed=1):
        p = estimate_pose_one(c, CAM, TAG)
        assert p["status"] == 0
        assert _rot_err(p["R"], R) < 1e-9
        assert np.linalg.norm(p["t"] - t) < 1e-9 * np.linalg.norm(t)
        assert p["reproj_rms"] < 1e-9
        assert abs(np.linalg.det(p["R"]) - 1.0) < 1e-12
        assert np.allclose(p["R"].T @ p["R"], np.eye(3), atol=1e-12)


def test_homography_maps_tag_plane_to_pixels():
    R, t, c = random_poses(1, seed=2)[0]
    p = estimate_pose_one(c, CAM, TAG)
    hs = TAG / 2
    for (X, Y), (x, y) in zip([(-hs, -hs), (hs, -hs), (hs, hs), (-hs, hs)], c):
        v = p["H"] @ np.array([X, Y, 1.0])
        assert abs(v[0] / v[2] - x) < 1e-6 and abs(v[1] / v[2] - y) < 1e-6
    assert p["H"][2, 2] == 1.0


def test_float32_corners_and_noise():
    rng = np.random.default_rng(3)
    for R, t, c in random_poses(100, seed=3):
        p = estimate_pose_one(c.astype(np.float32), CAM, TAG)
        assert p["reproj_rms"] < 1e-3
        noisy = c + rng.normal(scale=0.5, size=c.shape)
        p0 = estimate_pose_one(noisy, CAM, TAG, max_iterations=0)
        p1 = estimate_pose_one(noisy, CAM, TAG)
        assert p1["reproj_rms"] <= p0["reproj_rms"] + 1e-12
        assert p1["iterations"] >= 1 or p0["reproj_rms"] < 1e-9
        assert p1["reproj_rms"] < 1.5  # noise level: 8 residuals, 6 parameters
        # a small noisy tag may settle in the mirrored planar solution, which
        # fits its corners as well; a large one is well conditioned
        if np.ptp(c[:, 0]) > 300:
            assert _rot_err(p1["R"], R) < 0.05


def test_other_winding_is_reordered_to_the_same_pose():
    R, t, c = random_poses(1, seed=4)[0]
    a = estimate_pose_one(c, CAM, TAG)
    b = estimate_pose_one(c[[0, 3, 2, 1]], CAM, TAG)
    assert a["status"] == 0 and b["status"] == REORDERED
    assert _rot_err(a["R"], b["R"]) < 1e-9 and np.allclose(a["t"], b["t"], rtol=1e-9)


def test_degenerate_quads_are_flagged():
    line = np.array([[100.0, 100.0], [200.0, 100.0], [300.0, 100.0], [150.0, 100.0]])
    assert estimate_pose_one(line, CAM, TAG)["status"] & DEGENERATE
    point = np.full((4, 2), 500.0)
    assert estimate_pose_one(point, CAM, TAG)["status"] & DEGENERATE


def test_so3_exp_is_a_rotation_by_the_angle():
    w = np.array([0.3, -0.2, 0.5])
    R = so3_exp(w)
    assert np.allclose(R.T @ R, np.eye(3), atol=1e-14)
    assert abs(_rot_err(np.eye(3), R) - np.linalg.norm(w)) < 1e-12
    assert np.allclose(R @ w, w, atol=1e-14)
    assert np.allclose(project(np.eye(3), [0, 0, 1.0], CAM, TAG)[0], [960 - 80, 540 - 80])


def test_steep_tilts_and_anisotropic_cameras():
    cam = (1400.0, 1250.0, 900.0, 560.0)
    for R, t, c in random_poses(100, seed=5, max_angle_deg=80.0, cam=cam, dist=(0.3, 2.0)):
        p = estimate_pose_one(c, cam, TAG)
        assert p["status"] == 0
        assert _rot_err(p["R"], R) < 1e-8
        assert np.linalg.norm(p["t"] - t) < 1e-8 * np.linalg.norm(t)
        assert p["reproj_rms"] < 1e-8


def test_tag_size_scales_translation_only():
    R, t, c = random_poses(1, seed=6)[0]
    a = estimate_pose_one(c, CAM, TAG)
    b = estimate_pose_one(c, CAM, 2 * TAG)
    assert _rot_err(a["R"], b["R"]) < 1e-10
    assert np.allclose(b["t"], 2 * a["t"], rtol=1e-10)
