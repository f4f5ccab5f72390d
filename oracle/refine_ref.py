"""FP64 reference of the corner refinement (TEST INFRASTRUCTURE ONLY): the
same forward model as atag_refine_forward, written with torch float64 ops so
that autograd gives the exact FP64 gradient used to check the hand-written
CUDA adjoint."""
import torch

U = (-1.5, -0.5, 0.5, 1.5)
POS = 16
EPS = 1e-6


def bilinear(img, x, y):
    H, W = img.shape
    xc = x.clamp(0, W - 1)
    yc = y.clamp(0, H - 1)
    x0 = torch.floor(xc.detach()).clamp(max=W - 2)
    y0 = torch.floor(yc.detach()).clamp(max=H - 2)
    fx, fy = xc - x0, yc - y0
    xi, yi = x0.long(), y0.long()
    i00 = img[yi, xi]
    i01 = img[yi, xi + 1]
    i10 = img[yi + 1, xi]
    i11 = img[yi + 1, xi + 1]
    return (1 - fy) * ((1 - fx) * i00 + fx * i01) + fy * ((1 - fx) * i10 + fx * i11)


def refine(img, corners):
    """img H x W, corners Q x 4 x 2 (float64).  Returns refined (Q,4,2),
    residual (Q,4) and the samples (Q,4,16,4) as a non-leaf tensor."""
    dt = corners.dtype
    a = corners
    b = corners.roll(-1, dims=1)
    D = b - a
    ln = D.norm(dim=-1).clamp_min(1e-6)
    d = D / ln[..., None]
    n = torch.stack([-d[..., 1], d[..., 0]], -1)
    t = (torch.arange(POS, dtype=dt) + 0.5) / POS
    p = a[:, :, None, :] + t[None, None, :, None] * D[:, :, None, :]
    u = torch.tensor(U, dtype=dt)
    s = p[:, :, :, None, :] + u[None, None, None, :, None] * n[:, :, None, None, :]
    v = bilinear(img, s[..., 0], s[..., 1])
    gd = v[..., 1:] - v[..., :-1]
    w = gd * gd
    Om = w.sum(-1)
    Nn = (w * torch.tensor([-1.0, 0.0, 1.0], dtype=dt)).sum(-1)
    o = Nn / (Om + EPS)
    q = p + o[..., None] * n[:, :, None, :]
    W = Om + EPS
    origin = 0.5 * (a + b)
    X = q[..., 0] - origin[:, :, None, 0]
    Y = q[..., 1] - origin[:, :, None, 1]
    S0 = W.sum(-1).clamp_min(1e-30)
    Sx, Sy = (W * X).sum(-1), (W * Y).sum(-1)
    Sxx, Syy, Sxy = (W * X * X).sum(-1), (W * Y * Y).sum(-1), (W * X * Y).sum(-1)
    mx, my = Sx / S0, Sy / S0
    cxx, cyy, cxy = Sxx / S0 - mx * mx, Syy / S0 - my * my, Sxy / S0 - mx * my
    phi = 0.5 * torch.atan2(2 * cxy, cxx - cyy)
    m = torch.stack([origin[..., 0] + mx, origin[..., 1] + my], -1)
    uu = torch.stack([torch.cos(phi), torch.sin(phi)], -1)
    # residual: weighted squared distances to the fitted line (= S0 * lambda_min)
    dist = (X - mx[..., None]) * (-uu[..., None, 1]) + (Y - my[..., None]) * uu[..., None, 0]
    residual = (W * dist * dist).sum(-1)
    A_m, A_u = m.roll(1, dims=1), uu.roll(1, dims=1)  # line of edge i-1
    B_m, B_u = m, uu                                  # line of edge i
    Dm = B_m - A_m
    P = B_u[..., 0] * Dm[..., 1] - B_u[..., 1] * Dm[..., 0]
    Q = B_u[..., 0] * A_u[..., 1] - B_u[..., 1] * A_u[..., 0]
    alpha = P / Q
    refined = A_m + alpha[..., None] * A_u
    return refined, residual, v
