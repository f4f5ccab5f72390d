"""CPU check of the FP64 refinement reference (oracle/refine_ref.py) that the
CUDA adjoint is compared with: its autograd gradient agrees with central
finite differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from test_gpu_refine import _scene  # noqa: E402


def test_fp64_reference_matches_central_differences():
    """Bilinear interpolation is piecewise linear, so a central difference
    whose step crosses a pixel edge sees a kink: at h = 1e-3 almost every
    coordinate agrees with the FP64 gradient to 1e-4, and at h = 1e-4 all do
    to 1e-6."""
    import refine_ref
    img, corners = _scene(8, 9)
    img64 = torch.from_numpy(img.astype(np.float64))
    c = torch.from_numpy(corners.astype(np.float64))
    rng = np.random.default_rng(2)
    g_ref = torch.from_numpy(rng.normal(size=corners.shape))

    def loss(cc):
        r, res, _ = refine_ref.refine(img64, cc)
        return float((r * g_ref).sum() + 1e-2 * res.sum())
    cg = c.clone().requires_grad_(True)
    r, res, _ = refine_ref.refine(img64, cg)
    ((r * g_ref).sum() + 1e-2 * res.sum()).backward()
    ad = cg.grad.reshape(-1).numpy()
    scale = np.abs(ad).max()
    flat = c.reshape(-1)
    for h, tol, frac in ((1e-3, 1e-4, 0.9), (1e-4, 1e-6, 1.0)):
        fd = np.zeros(flat.numel())
        for k in range(flat.numel()):
            e = torch.zeros_like(flat)
            e[k] = h
            fd[k] = (loss((flat + e).reshape(c.shape)) - loss((flat - e).reshape(c.shape))) / (2 * h)
        ok = np.abs(fd - ad) <= tol * scale
        assert ok.mean() >= frac, (h, ok.mean())


