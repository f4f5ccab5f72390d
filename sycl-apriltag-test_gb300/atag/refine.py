"""Subpixel corner refinement with a hand-written adjoint (CUDA), exposed as a
torch.autograd.Function.  The forward model is documented in
include/atag.h (atag_refine_forward) and csrc/k_refine.cu."""
import ctypes

import torch

from . import lib

_P = ctypes.c_void_p
SAMPLES_PER_EDGE = 64


def _ptr(t):
    return _P(t.data_ptr()) if t is not None else None


def _stream():
    return _P(torch.cuda.current_stream().cuda_stream)


def refine_forward(image: torch.Tensor, corners: torch.Tensor):
    """image: H x W float32 (CUDA); corners: Q x 4 x 2 float32.  Returns
    (refined Q x 4 x 2, residual Q x 4, samples Q x 4 x 64)."""
    L = lib.init()
    image = image.contiguous()
    corners = corners.contiguous()
    q = corners.shape[0]
    refined = torch.empty_like(corners)
    residual = torch.empty((q, 4), dtype=torch.float32, device=corners.device)
    samples = torch.empty((q, 4, SAMPLES_PER_EDGE), dtype=torch.float32, device=corners.device)
    lib.check(L.atag_refine_forward(_ptr(image), image.shape[1], image.shape[0], _ptr(corners), q, _ptr(refined),
                                    _ptr(residual), _ptr(samples), _stream()), "atag_refine_forward")
    return refined, residual, samples


def refine_backward(image, corners, grad_refined=None, grad_residual=None, want_image_grad=False):
    """Returns (dL/dcorners Q x 4 x 2, dL/dsamples Q x 4 x 64, dL/dimage or None)."""
    L = lib.init()
    image = image.contiguous()
    corners = corners.contiguous()
    q = corners.shape[0]
    g_c = torch.empty_like(corners)
    g_s = torch.empty((q, 4, SAMPLES_PER_EDGE), dtype=torch.float32, device=corners.device)
    g_i = torch.zeros_like(image) if want_image_grad else None
    gr = grad_refined.contiguous() if grad_refined is not None else None
    gres = grad_residual.contiguous() if grad_residual is not None else None
    lib.check(L.atag_refine_backward(_ptr(image), image.shape[1], image.shape[0], _ptr(corners), q, _ptr(gr),
                                     _ptr(gres), _ptr(g_c), _ptr(g_s), _ptr(g_i), _stream()), "atag_refine_backward")
    return g_c, g_s, g_i


class RefineCorners(torch.autograd.Function):
    """refined, residual = RefineCorners.apply(image, corners)"""

    @staticmethod
    def forward(ctx, image, corners):
        refined, residual, _ = refine_forward(image.detach(), corners.detach())
        ctx.save_for_backward(image, corners)
        return refined, residual

    @staticmethod
    def backward(ctx, grad_refined, grad_residual):
        image, corners = ctx.saved_tensors
        g_c, _, g_i = refine_backward(image.detach(), corners.detach(), grad_refined, grad_residual,
                                      want_image_grad=ctx.needs_input_grad[0])
        return (g_i if ctx.needs_input_grad[0] else None), (g_c if ctx.needs_input_grad[1] else None)


def refine(image, corners):
    return RefineCorners.apply(image, corners)
