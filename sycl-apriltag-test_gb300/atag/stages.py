"""The reference's stage functions over torch CUDA tensors, each a thin call
into the C ABI (include/atag.h) on the current torch stream.

Names follow the reference (threshold_image, image_segmentation,
find_boundaries, fit_lines, do_indexing, process_fitted_quads).  Record
arrays travel as raw byte tensors and are viewed with the numpy dtypes of
atag.records on the host.
"""
import ctypes

import numpy as np
import torch

from . import lib
from .records import CORNER, FITTED_QUAD, QUAD_CORNERS

_P = ctypes.c_void_p


def _stream():
    return _P(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return _P(t.data_ptr()) if t is not None else None


def to_device(arr: np.ndarray) -> torch.Tensor:
    """Copies a (record) numpy array to the device as raw bytes."""
    a = np.ascontiguousarray(arr)
    return torch.from_numpy(a.view(np.uint8).reshape(-1).copy()).cuda()


def to_host(t: torch.Tensor, dtype) -> np.ndarray:
    return t.cpu().numpy().view(np.uint8).view(dtype)


def decimate(src: torch.Tensor, factor: int) -> torch.Tensor:
    L = lib.init()
    h, w = src.shape
    out = torch.empty((h // factor, w // factor), dtype=torch.uint8, device=src.device)
    lib.check(L.atag_decimate(_ptr(src), w, h, factor, _ptr(out), _stream()), "atag_decimate")
    return out


def convert_grey(src: torch.Tensor, factor: int = 1, fmt: int = None) -> torch.Tensor:
    """Colour removal + decimation (atag_convert_grey): src is H x W (grey)
    or H x W x C (C = 2, 3, 4: grey + alpha, RGB, RGBA; `fmt` for BGR)."""
    from .detector import frame_format
    from .records import PIXEL_BYTES
    L = lib.init()
    src = src.contiguous()
    h, w = src.shape[0], src.shape[1]
    fmt = frame_format(src) if fmt is None else fmt
    out = torch.empty((h // factor, w // factor), dtype=torch.uint8, device=src.device)
    lib.check(L.atag_convert_grey(_ptr(src), w, h, w * PIXEL_BYTES[fmt], fmt, factor, _ptr(out), _stream()),
              "atag_convert_grey")
    return out


def threshold_image(grey: torch.Tensor, with_extrema: bool = False):
    """threshold_image (include/threshold.h:6-10): returns the {0,127,255}
    image, and the tile extrema (min, max) before and after dilation when
    asked."""
    L = lib.init()
    h, w = grey.shape
    thr = torch.empty_like(grey)
    ext = flt = None
    if with_extrema:
        ext = torch.empty((h // 4, w // 4, 2), dtype=torch.uint8, device=grey.device)
        flt = torch.empty_like(ext)
    lib.check(L.atag_threshold_image(_ptr(grey), _ptr(ext), _ptr(flt), _ptr(thr), w, h, _stream()),
              "atag_threshold_image")
    return (thr, ext, flt) if with_extrema else thr


def image_segmentation(thr: torch.Tensor):
    """image_segmentation (include/segmentation.h:11-15): returns (labels,
    sizes, scratch) as int32 tensors holding uint32 bit patterns."""
    L = lib.init()
    h, w = thr.shape
    labels = torch.empty((h, w), dtype=torch.int32, device=thr.device)
    sizes = torch.empty(h * w, dtype=torch.int32, device=thr.device)
    scratch = torch.empty(h * w, dtype=torch.int32, device=thr.device)
    lib.check(L.atag_image_segmentation(_ptr(thr), _ptr(scratch), _ptr(labels), _ptr(sizes), h * w, w, h,
                                        _stream()), "atag_image_segmentation")
    return labels, sizes, scratch


def find_boundaries(labels: torch.Tensor, sizes: torch.Tensor):
    """find_boundaries (include/find_boundaries.h:8-12): the dense 4-plane
    output, pre-filled with 0 (points) and 0xFF (keys) as the reference's
    caller does.  Returns (points int32 [4*N] of packed u16 pairs, keys
    int64 [4*N] of uint64 bit patterns)."""
    L = lib.init()
    h, w = labels.shape
    pts = torch.zeros(4 * h * w, dtype=torch.int32, device=labels.device)
    keys = torch.full((4 * h * w,), -1, dtype=torch.int64, device=labels.device)
    lib.check(L.atag_find_boundaries(_ptr(labels), _ptr(sizes), _ptr(pts), _ptr(keys), w, h, _stream()),
              "atag_find_boundaries")
    return pts, keys


def fit_lines(line_fit: np.ndarray, cluster_indices: np.ndarray, extents: np.ndarray) -> np.ndarray:
    """fit_lines (include/fit_quad.h:46-49) over host record arrays; returns
    the dense corner array (zero where no corner)."""
    L = lib.init()
    n = len(line_fit)
    d_lf = to_device(line_fit)
    d_ci = to_device(np.asarray(cluster_indices, dtype=np.uint16))
    d_ex = to_device(extents)
    d_out = torch.zeros(n * CORNER.itemsize, dtype=torch.uint8, device="cuda")
    lib.check(L.atag_fit_lines(_ptr(d_lf), _ptr(d_ci), _ptr(d_ex), n, _ptr(d_out), _stream()), "atag_fit_lines")
    return to_host(d_out, CORNER)


def do_indexing(peak_extents: np.ndarray, corners: np.ndarray, line_fit: np.ndarray,
                cluster_extents: np.ndarray) -> np.ndarray:
    """do_indexing (include/fit_quad.h:51-55); returns FittedQuad records."""
    L = lib.init()
    n = len(peak_extents)
    d_out = torch.zeros(max(n, 1) * FITTED_QUAD.itemsize, dtype=torch.uint8, device="cuda")
    if n:
        d_pe, d_co = to_device(peak_extents), to_device(corners)
        d_lf, d_ce = to_device(line_fit), to_device(cluster_extents)
        lib.check(L.atag_do_indexing(_ptr(d_pe), n, _ptr(d_co), _ptr(d_lf), _ptr(d_ce), _ptr(d_out), _stream()),
                  "atag_do_indexing")
    return to_host(d_out, FITTED_QUAD)[:n]


def process_fitted_quads(fitted: np.ndarray, width: int, height: int, config=None) -> np.ndarray:
    """process_fitted_quads (src/main.cpp:1035) up to decoding, on the device."""
    L = lib.init()
    cfg = config or lib.default_config()
    n = len(fitted)
    d_out = torch.zeros(max(n, 1) * QUAD_CORNERS.itemsize, dtype=torch.uint8, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_f = to_device(fitted) if n else torch.zeros(1, dtype=torch.uint8, device="cuda")
    lib.check(L.atag_process_fitted_quads(_ptr(d_f), n, width, height, ctypes.byref(cfg), _ptr(d_out), max(n, 1),
                                          _ptr(d_cnt), _stream()), "atag_process_fitted_quads")
    cnt = int(d_cnt.item())
    return to_host(d_out, QUAD_CORNERS)[:cnt]
