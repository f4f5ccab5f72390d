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
from .records import (CLUSTER_BOUNDS, CLUSTER_EXTENTS, CLUSTER_POINT, CORNER, FITTED_QUAD, FRAME_STATS,
                      LINE_FIT_POINT, PEAK_EXTENTS, QUAD_CORNERS, ClusterOutputs, ClusterPointC, LineFitPointC)

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


def _dev(a):
    """A device byte tensor of a record array (numpy arrays are copied)."""
    return a if isinstance(a, torch.Tensor) else to_device(a)


def _bytes(n, dtype, fill=0):
    return torch.full((max(int(n), 1) * np.dtype(dtype).itemsize,), fill, dtype=torch.uint8, device="cuda")


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


def fit_lines(line_fit, cluster_indices, extents, n: int = None, on_device: bool = False):
    """fit_lines (include/fit_quad.h:46-49) over n points: record arrays on
    the host (numpy) or the device (byte tensors, n given).  Returns the
    dense corner array (zero where no corner), on the device if asked."""
    L = lib.init()
    if n is None:
        n = len(line_fit)
    d_lf = _dev(line_fit)
    d_ci = cluster_indices if isinstance(cluster_indices, torch.Tensor) else \
        to_device(np.asarray(cluster_indices, dtype=np.uint16))
    d_ex = _dev(extents)
    d_out = _bytes(n, CORNER)
    if n:
        lib.check(L.atag_fit_lines(_ptr(d_lf), _ptr(d_ci), _ptr(d_ex), n, _ptr(d_out), _stream()), "atag_fit_lines")
    return d_out if on_device else to_host(d_out, CORNER)[:n]


def do_indexing(peak_extents, corners, line_fit, cluster_extents, n: int = None, on_device: bool = False):
    """do_indexing (include/fit_quad.h:51-55) over n PeakExtents; returns
    FittedQuad records (pre-zeroed, as src/main.cpp:318-319 does)."""
    L = lib.init()
    if n is None:
        n = len(peak_extents)
    d_out = _bytes(n, FITTED_QUAD)
    if n:
        d_pe, d_co = _dev(peak_extents), _dev(corners)
        d_lf, d_ce = _dev(line_fit), _dev(cluster_extents)
        lib.check(L.atag_do_indexing(_ptr(d_pe), n, _ptr(d_co), _ptr(d_lf), _ptr(d_ce), _ptr(d_out), _stream()),
                  "atag_do_indexing")
    return d_out if on_device else to_host(d_out, FITTED_QUAD)[:n]


def process_fitted_quads(fitted, width: int, height: int, config=None, n: int = None) -> np.ndarray:
    """process_fitted_quads (src/main.cpp:1035) up to decoding, on the device."""
    L = lib.init()
    cfg = config or lib.default_config()
    if n is None:
        n = len(fitted)
    d_out = _bytes(n, QUAD_CORNERS)
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_f = _dev(fitted) if n else torch.zeros(1, dtype=torch.uint8, device="cuda")
    lib.check(L.atag_process_fitted_quads(_ptr(d_f), n, width, height, ctypes.byref(cfg), _ptr(d_out), max(n, 1),
                                          _ptr(d_cnt), _stream()), "atag_process_fitted_quads")
    cnt = int(d_cnt.item())
    return to_host(d_out, QUAD_CORNERS)[:cnt]


def cluster(points: torch.Tensor, keys: torch.Tensor, grey: torch.Tensor, cluster_capacity: int = 65535,
            point_capacity: int = None, pair_capacity: int = None):
    """atag_cluster: the reference's stages 4-11 (src/main.cpp:467-801) from
    the dense planes of find_boundaries to the inputs of fit_lines.  Returns
    (dict of device byte tensors: pair_bounds, pair_keys, filtered_bounds,
    filtered_keys, cluster_extents, cluster_points, cluster_indices,
    line_fit; the counts record read back to the host, as the reference
    reads its counts between stages)."""
    L = lib.init()
    h, w = grey.shape
    N = w * h
    if point_capacity is None:
        point_capacity = min(4 * N, max(N // 2, 4096))
    if pair_capacity is None:
        pair_capacity = 65536
    size = ctypes.c_size_t()
    lib.check(L.atag_cluster_workspace_size(w, h, cluster_capacity, point_capacity, ctypes.byref(size)),
              "atag_cluster_workspace_size")
    ws = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    cc = min(cluster_capacity, 65535)
    out = {"pair_bounds": _bytes(pair_capacity, CLUSTER_BOUNDS), "pair_keys": _bytes(pair_capacity, np.uint64),
           "filtered_bounds": _bytes(cc, CLUSTER_BOUNDS), "filtered_keys": _bytes(cc, np.uint64),
           "cluster_extents": _bytes(cc, CLUSTER_EXTENTS), "cluster_points": _bytes(point_capacity, CLUSTER_POINT),
           "cluster_indices": _bytes(point_capacity, np.uint16), "line_fit": _bytes(point_capacity, LINE_FIT_POINT),
           "counts": _bytes(1, FRAME_STATS)}
    o = ClusterOutputs(_ptr(out["pair_bounds"]), _ptr(out["pair_keys"]), pair_capacity,
                       _ptr(out["filtered_bounds"]), _ptr(out["filtered_keys"]), _ptr(out["cluster_extents"]), cc,
                       _ptr(out["cluster_points"]), _ptr(out["cluster_indices"]), _ptr(out["line_fit"]),
                       point_capacity, _ptr(out["counts"]))
    lib.check(L.atag_cluster(_ptr(points), _ptr(keys), _ptr(grey), w, h, _ptr(ws), size.value, ctypes.byref(o),
                             _stream()), "atag_cluster")
    counts = to_host(out.pop("counts"), FRAME_STATS)[0]
    return out, counts


def corner_peaks(found: torch.Tensor, cluster_extents: torch.Tensor, n_clusters: int, corner_capacity: int,
                 extents_capacity: int = None):
    """atag_corner_peaks: the reference's stages 13-15 (src/main.cpp:832-907).
    Returns (compacted corners, PeakExtents) as device byte tensors and
    (K, C_p, status) read back to the host."""
    L = lib.init()
    if extents_capacity is None:
        extents_capacity = max(n_clusters, 1)
    size = ctypes.c_size_t()
    lib.check(L.atag_corner_peaks_workspace_size(n_clusters, ctypes.byref(size)), "atag_corner_peaks_workspace_size")
    ws = torch.empty(size.value, dtype=torch.uint8, device="cuda")
    d_corners = _bytes(corner_capacity, CORNER)
    d_pe = _bytes(extents_capacity, PEAK_EXTENTS)
    d_counts = torch.zeros(3, dtype=torch.int32, device="cuda")
    lib.check(L.atag_corner_peaks(_ptr(found), _ptr(cluster_extents), n_clusters, _ptr(ws), size.value,
                                  _ptr(d_corners), corner_capacity, _ptr(d_pe), extents_capacity, _ptr(d_counts),
                                  _stream()), "atag_corner_peaks")
    k, cp, status = (int(v) for v in d_counts.cpu().numpy().view(np.uint32))
    return d_corners, d_pe, (k, cp, status)


# -- host helpers (no device) -------------------------------------------------
def get_moment(prefix: np.ndarray, i0: int, i1: int):
    """get_moment (include/fit_quad.h:39-41) over one cluster's prefix sums."""
    L = lib.load()
    pre = np.ascontiguousarray(prefix, dtype=LINE_FIT_POINT)
    out = np.zeros(1, LINE_FIT_POINT)
    n = ctypes.c_size_t()
    lib.check(L.atag_get_moment(_P(pre.ctypes.data), len(pre), i0, i1, _P(out.ctypes.data), ctypes.byref(n)),
              "atag_get_moment")
    return out[0], int(n.value)


def fit_line(moment, num_in_moment: int):
    """fit_line (include/fit_quad.h:43-44): (line params[4], err, mse)."""
    L = lib.load()
    m = np.ascontiguousarray(np.asarray(moment, dtype=LINE_FIT_POINT).reshape(1))
    lp = np.zeros(4, np.float32)
    err, mse = ctypes.c_float(), ctypes.c_float()
    lib.check(L.atag_fit_line(_P(m.ctypes.data), num_in_moment, _P(lp.ctypes.data), ctypes.byref(err),
                              ctypes.byref(mse)), "atag_fit_line")
    return lp, np.float32(err.value), np.float32(mse.value)


def compute_initial_linefit(point, width: int, height: int, grey: np.ndarray) -> np.ndarray:
    """compute_initial_linefit (include/line_fit_point.h:50-86) of one
    ClusterPoint record over a host grey image."""
    L = lib.load()
    img = np.ascontiguousarray(grey, dtype=np.uint8)
    p = ClusterPointC(int(point["packed_x"]), int(point["packed_y"]), float(point["slope"]))
    r = L.atag_compute_initial_linefit(p, width, height, _P(img.ctypes.data))
    out = np.zeros(1, LINE_FIT_POINT)
    for name in LINE_FIT_POINT.names:
        out[name] = getattr(r, name)
    return out[0]
