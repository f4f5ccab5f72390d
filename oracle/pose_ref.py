"""CPU restatement (numpy, FP64) of the tag pose stage, atag_estimate_pose.

TEST INFRASTRUCTURE ONLY: tests and bench.py's checks import this as the
checker; the product path is the CUDA kernel (csrc/k_pose.cu).

Parity unpinned against the reference: the reference has no pose stage (it
stops at the corners of process_fitted_quads, src/main.cpp:1035-1162).  This
restatement is pinned instead against ground truth: corners projected from
known poses (tests/test_pose_ref.py).

Steps, per quad (the same as the kernel's):
  1. winding: a negative shoelace area takes the corners in the order 0, 3, 2, 1;
  2. normalised coordinates and the closed-form projective map of the unit
     square onto the quad (Heckbert 1989), composed with the map of the tag
     plane onto the unit square;
  3. scale, sign (tag in front), R0 = [r1 r2 r1 x r2], polar factor by the
     Newton iteration X <- (X + X^-T) / 2 (Higham 1986);
  4. Levenberg-Marquardt on the pixel reprojection error, R <- exp([w]x) R:
     diagonal scaled by 1 + mu, mu from 1e-9, times 10 after a step that
     does not lower the error (dropped; stop above 1e9), divided by 10 after
     one that does (kept); up to max_iterations trials.
"""
import math

import numpy as np

REORDERED, DEGENERATE = 0x1, 0x2
DAMPING, MAX_DAMPING = 1e-9, 1e9


def _orthogonalise(x):
    for _ in range(32):
        c = np.array([
            [x[1, 1] * x[2, 2] - x[1, 2] * x[2, 1], x[1, 2] * x[2, 0] - x[1, 0] * x[2, 2],
             x[1, 0] * x[2, 1] - x[1, 1] * x[2, 0]],
            [x[0, 2] * x[2, 1] - x[0, 1] * x[2, 2], x[0, 0] * x[2, 2] - x[0, 2] * x[2, 0],
             x[0, 1] * x[2, 0] - x[0, 0] * x[2, 1]],
            [x[0, 1] * x[1, 2] - x[0, 2] * x[1, 1], x[0, 2] * x[1, 0] - x[0, 0] * x[1, 2],
             x[0, 0] * x[1, 1] - x[0, 1] * x[1, 0]]])
        d = x[0, 0] * c[0, 0] + x[0, 1] * c[0, 1] + x[0, 2] * c[0, 2]
        v = 0.5 * (x + c * (1.0 / d))
        change = np.max(np.abs(v - x))
        x = v
        if change < 1e-15:
            break
    return x


def so3_exp(w):
    t2 = float(w @ w)
    t = math.sqrt(t2)
    if t < 1e-8:
        a, b = 1.0 - t2 / 6.0, 0.5 - t2 / 24.0
    else:
        a, b = math.sin(t) / t, (1.0 - math.cos(t)) / t2
    k = np.array([[0.0, -w[2], w[1]], [w[2], 0.0, -w[0]], [-w[1], w[0], 0.0]])
    return np.eye(3) + a * k + b * (k @ k)


def _cost(R, t, obj, px, py, cam):
    fx, fy, cx, cy = cam
    P = obj @ R[:, :2].T + t
    if np.any(~(P[:, 2] > 0.0)):
        return None
    ex = fx * P[:, 0] / P[:, 2] + cx - px
    ey = fy * P[:, 1] / P[:, 2] + cy - py
    return float(np.sum(ex * ex + ey * ey))


def estimate_pose_one(corners, cam, tag_size, max_iterations=20):
    """corners: 4 x 2 pixel coordinates.  Returns a dict with R (3 x 3), t,
    H (3 x 3, H[2, 2] = 1), reproj_rms, iterations, status."""
    fx, fy, cx, cy = (float(v) for v in cam)
    px = np.asarray(corners, np.float64)[:, 0].copy()
    py = np.asarray(corners, np.float64)[:, 1].copy()
    out = {"R": np.zeros((3, 3)), "t": np.zeros(3), "H": np.zeros((3, 3)), "reproj_rms": 0.0, "iterations": 0,
           "status": 0}
    area2 = sum(px[i] * py[(i + 1) % 4] - px[(i + 1) % 4] * py[i] for i in range(4))
    if area2 < 0.0:
        px[[1, 3]] = px[[3, 1]]
        py[[1, 3]] = py[[3, 1]]
        out["status"] |= REORDERED
    nx, ny = (px - cx) / fx, (py - cy) / fy
    sx, sy = nx[0] - nx[1] + nx[2] - nx[3], ny[0] - ny[1] + ny[2] - ny[3]
    dx1, dx2, dy1, dy2 = nx[1] - nx[2], nx[3] - nx[2], ny[1] - ny[2], ny[3] - ny[2]
    den = dx1 * dy2 - dx2 * dy1
    ref = abs(dx1) + abs(dx2) + abs(dy1) + abs(dy2)
    if not abs(den) > 1e-14 * ref * ref or not tag_size > 0.0:
        out["status"] |= DEGENERATE
        return out
    g, h = (sx * dy2 - dx2 * sy) / den, (dx1 * sy - sx * dy1) / den
    Hu = np.array([[nx[1] - nx[0] + g * nx[1], nx[3] - nx[0] + h * nx[3], nx[0]],
                   [ny[1] - ny[0] + g * ny[1], ny[3] - ny[0] + h * ny[3], ny[0]],
                   [g, h, 1.0]])
    h1, h2 = Hu[:, 0] / tag_size, Hu[:, 1] / tag_size
    h3 = 0.5 * Hu[:, 0] + 0.5 * Hu[:, 1] + Hu[:, 2]
    lam = 0.5 * (math.sqrt(h1 @ h1) + math.sqrt(h2 @ h2))
    if not lam > 0.0:
        out["status"] |= DEGENERATE
        return out
    if h3[2] < 0.0:
        lam = -lam
    r1, r2, t = h1 / lam, h2 / lam, h3 / lam
    R = np.stack([r1, r2, np.cross(r1, r2)], axis=1)
    if not np.linalg.det(R) > 0.0:
        out["status"] |= DEGENERATE
        return out
    R = _orthogonalise(R)
    hs = 0.5 * tag_size
    obj = np.array([[-hs, -hs], [hs, -hs], [hs, hs], [-hs, hs]])
    cost = _cost(R, t, obj, px, py, (fx, fy, cx, cy))
    if cost is None:
        out["status"] |= DEGENERATE
        return out
    it, mu = 0, DAMPING
    for _ in range(max_iterations):
        A = np.zeros((6, 6))
        b = np.zeros(6)
        for i in range(4):
            a = R[:, :2] @ obj[i]
            X, Y, Z = a + t
            iz = 1.0 / Z
            ex, ey = fx * X * iz + cx - px[i], fy * Y * iz + cy - py[i]
            ux, uz, vy, vz = fx * iz, -fx * X * iz * iz, fy * iz, -fy * Y * iz * iz
            ju = np.array([uz * a[1], ux * a[2] - uz * a[0], -ux * a[1], ux, 0.0, uz])
            jv = np.array([-vy * a[2] + vz * a[1], -vz * a[0], vy * a[0], 0.0, vy, vz])
            b -= ju * ex + jv * ey
            A += np.outer(ju, ju) + np.outer(jv, jv)
        A[np.diag_indices(6)] *= 1.0 + mu
        try:
            L = np.linalg.cholesky(A)
        except np.linalg.LinAlgError:
            L = None
        cn = None
        if L is not None:
            d = np.linalg.solve(L.T, np.linalg.solve(L, b))
            Rn = so3_exp(d[:3]) @ R
            tn = t + d[3:]
            cn = _cost(Rn, tn, obj, px, py, (fx, fy, cx, cy))
        if cn is None or not cn < cost:
            mu *= 10.0
            if mu > MAX_DAMPING:
                break
            continue
        R, t, cost = Rn, tn, cn
        mu = max(mu * 0.1, DAMPING)
        it += 1
        if np.sum(np.abs(d[:3])) + np.sum(np.abs(d[3:])) / tag_size < 1e-12:
            break
    K = np.array([[fx, 0.0, cx], [0.0, fy, cy], [0.0, 0.0, 1.0]])
    Hp = K @ np.stack([R[:, 0], R[:, 1], t], axis=1)
    out.update(R=R, t=t, H=Hp / Hp[2, 2], reproj_rms=math.sqrt(cost / 4.0), iterations=it)
    return out


def estimate_pose(corners, cam, tag_size, max_iterations=20):
    """corners: Q x 4 x 2.  Returns a list of per-quad dicts."""
    return [estimate_pose_one(c, cam, tag_size, max_iterations) for c in np.asarray(corners)]


def project(R, t, cam, tag_size):
    """The four tag corners of a pose, in pixels (4 x 2, FP64)."""
    fx, fy, cx, cy = cam
    hs = 0.5 * tag_size
    obj = np.array([[-hs, -hs, 0.0], [hs, -hs, 0.0], [hs, hs, 0.0], [-hs, hs, 0.0]])
    P = obj @ np.asarray(R).T + np.asarray(t)
    return np.stack([fx * P[:, 0] / P[:, 2] + cx, fy * P[:, 1] / P[:, 2] + cy], axis=1)


def random_poses(n, seed, tag_size=0.16, max_angle_deg=60.0, dist=(0.4, 4.0), cam=(1000.0, 1000.0, 960.0, 540.0),
                 size=(1920, 1080)):
    """Seeded poses of a tag facing the camera (tilted up to max_angle_deg,
    any roll; its front seen, i.e. its z axis along the viewing ray) whose
    corners fall inside the image."""
    rng = np.random.default_rng(seed)
    out = []
    while len(out) < n:
        axis = rng.normal(size=3)
        axis /= np.linalg.norm(axis)
        tilt = math.radians(rng.uniform(0.0, max_angle_deg))
        ax = np.array([axis[0], axis[1], 0.0])
        ax /= max(np.linalg.norm(ax), 1e-12)
        R = so3_exp(ax * tilt) @ so3_exp(np.array([0.0, 0.0, rng.uniform(-math.pi, math.pi)]))
        z = rng.uniform(*dist)
        t = np.array([rng.uniform(-0.4, 0.4) * z, rng.uniform(-0.25, 0.25) * z, z])
        if not R[:, 2] @ t > 0.0:
            continue
        c = project(R, t, cam, tag_size)
        if np.all(c[:, 0] > 0) and np.all(c[:, 0] < size[0]) and np.all(c[:, 1] > 0) and np.all(c[:, 1] < size[1]):
            out.append((R, t, c))
    return out
