"""The hand-written refinement adjoint (atag_refine_backward) against an FP64
autograd reference of the same forward model and against central finite
differences (h = 1e-3): relative gradient error <= 1e-4 vs FP64."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

REL_TOL = 1e-4       # gradient vs FP64 autograd, per quad (2-norm)
CORNER_TOL = 1e-3    # refined corners vs FP64, pixels


def _scene(n_quads, seed, size=None, return_truth=False):
    """Dark rotated quads (half-size 12-22 px, one per 64 px grid cell, so
    no two overlap) on a noisy background, blurred, FP32 in [0, 1], and
    corner guesses perturbed from the drawn corners by up to 1.5 px."""
    from atag import synth
    rng = np.random.default_rng(seed)
    cells = int(np.ceil(np.sqrt(n_quads)))
    size = size or 64 * cells
    img = rng.uniform(0.55, 0.75, (size, size)).astype(np.float32)
    yy, xx = np.mgrid[0:size, 0:size].astype(np.float64)
    corners = []
    for k in range(n_quads):
        c = np.array([64 * (k % cells) + 32, 64 * (k // cells) + 32]) + rng.uniform(-4, 4, 2)
        s = rng.uniform(12, 22)
        th = rng.uniform(0, np.pi / 2)
        R = np.array([[np.cos(th), -np.sin(th)], [np.sin(th), np.cos(th)]])
        quad = c + (np.array([[-1, -1], [1, -1], [1, 1], [-1, 1]]) * s) @ R.T
        quad += rng.normal(0, 0.6, quad.shape)
        corners.append(quad)
        inside = np.ones_like(xx, bool)
        for i in range(4):
            a, b = quad[i], quad[(i + 1) % 4]
            inside &= (b[0] - a[0]) * (yy - a[1]) - (b[1] - a[1]) * (xx - a[0]) >= 0
        img[inside] = 0.1
    img = synth._blur(img, 1.0).astype(np.float32)
    truth = np.stack(corners).astype(np.float32)
    guess = (truth + rng.uniform(-1.5, 1.5, truth.shape)).astype(np.float32)
    return (img, guess, truth) if return_truth else (img, guess)


def _rel(a, b):
    return np.linalg.norm(a - b, axis=-1) / np.maximum(np.linalg.norm(b, axis=-1), 1e-12)


def _fp64(img, corners, g_ref, g_res):
    import refine_ref
    img64 = torch.from_numpy(img.astype(np.float64))
    c64 = torch.from_numpy(corners.astype(np.float64)).requires_grad_(True)
    refined, residual, v = refine_ref.refine(img64, c64)
    v.retain_grad()
    loss = (refined * torch.from_numpy(g_ref.astype(np.float64))).sum() + \
        (residual * torch.from_numpy(g_res.astype(np.float64))).sum()
    loss.backward()
    return refined.detach().numpy(), residual.detach().numpy(), c64.grad.numpy(), v.grad.numpy()


def test_forward_and_adjoint_match_fp64():
    from atag import refine
    img, corners = _scene(64, 3)
    rng = np.random.default_rng(5)
    g_ref = rng.normal(size=corners.shape).astype(np.float32)
    g_res = rng.normal(size=corners.shape[:2]).astype(np.float32) * 1e-2
    d_img, d_c = torch.from_numpy(img).cuda(), torch.from_numpy(corners).cuda()
    refined, residual, samples = refine.refine_forward(d_img, d_c)
    g_c, g_s, _ = refine.refine_backward(d_img, d_c, torch.from_numpy(g_ref).cuda(), torch.from_numpy(g_res).cuda())
    r64, res64, gc64, gv64 = _fp64(img, corners, g_ref, g_res)
    assert np.abs(refined.cpu().numpy() - r64).max() <= CORNER_TOL
    # residuals are sums of squared sub-pixel distances: FP32 positions give
    # them ~1e-7 absolute noise, so the bound is relative plus absolute
    assert np.allclose(residual.cpu().numpy(), res64, rtol=1e-4, atol=5e-7)
    rel_c = _rel(g_c.cpu().numpy().reshape(len(corners), 8), gc64.reshape(len(corners), 8))
    assert rel_c.max() <= REL_TOL, rel_c.max()
    rel_s = _rel(g_s.cpu().numpy().reshape(len(corners), -1), gv64.reshape(len(corners), -1))
    assert rel_s.max() <= REL_TOL, rel_s.max()


def test_adjoint_matches_central_differences_of_cuda_forward():
    from atag import refine
    img, corners = _scene(16, 11)
    d_img = torch.from_numpy(img).cuda()
    rng = np.random.default_rng(4)
    g_ref = torch.from_numpy(rng.normal(size=corners.shape).astype(np.float32)).cuda()
    c = torch.from_numpy(corners.astype(np.float64))
    h = 1e-3

    def loss(cc):
        r, _, _ = refine.refine_forward(d_img, cc.float().cuda())
        return (r.double() * g_ref.double()).sum(dim=(1, 2)).cpu().numpy()
    g_c, _, _ = refine.refine_backward(d_img, c.float().cuda(), g_ref, None)
    g_c = g_c.cpu().numpy().reshape(len(corners), 8)
    fd = np.zeros_like(g_c)
    for k in range(8):
        e = torch.zeros((4, 2), dtype=torch.float64)
        e.view(-1)[k] = h
        fd[:, k] = (loss(c + e) - loss(c - e)) / (2 * h)
    # FP32 forward differences carry ~1e-4 px noise / 2e-3: compare loosely
    rel = _rel(g_c, fd)
    assert np.median(rel) <= 2e-2, np.median(rel)


def test_autograd_function_and_image_gradient():
    from atag import refine
    img, corners = _scene(32, 21)
    d_img = torch.from_numpy(img).cuda().requires_grad_(True)
    d_c = torch.from_numpy(corners).cuda().requires_grad_(True)
    refined, residual = refine.refine(d_img, d_c)
    (refined.sum() + 1e-3 * residual.sum()).backward()
    g_c, g_s, g_i = refine.refine_backward(d_img.detach(), d_c.detach(), torch.ones_like(refined),
                                           torch.full_like(residual, 1e-3), want_image_grad=True)
    assert torch.allclose(d_c.grad, g_c)
    assert torch.allclose(d_img.grad, g_i)
    # image gradient = samples' gradients scattered through the bilinear weights
    assert abs(float(g_i.sum()) - float(g_s.sum())) <= 1e-3 * float(g_s.abs().sum())


def test_refinement_moves_perturbed_corners_toward_the_edges():
    from atag import refine
    img, guess, truth = _scene(36, 33, return_truth=True)
    d_img = torch.from_numpy(img).cuda()
    c = torch.from_numpy(guess).cuda()
    for _ in range(3):
        c, _, _ = refine.refine_forward(d_img, c)
    assert torch.isfinite(c).all()
    before = np.linalg.norm(guess - truth, axis=-1).mean()
    after = np.linalg.norm(c.cpu().numpy() - truth, axis=-1).mean()
    assert after < 0.5 * before, (before, after)
