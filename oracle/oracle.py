"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py as the parity checker and CPU
baseline.  The product package never imports it.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

# numpy mirrors of the reference records (layout-identical, see include/atag.h)
BOUNDARY_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2")])
CLUSTER_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2"), ("slope", "<f4")])
CLUSTER_EXTENTS = np.dtype([("start", "<u4"), ("count", "<u4")])
CLUSTER_BOUNDS = np.dtype([("x_min", "<u2"), ("x_max", "<u2"), ("y_min", "<u2"), ("y_max", "<u2"),
                           ("gx_sum", "<i4"), ("gy_sum", "<i4"), ("pxgx_pygy_sum", "<i8"),
                           ("start", "<u4"), ("count", "<u4")])
LINE_FIT_POINT = np.dtype([(n, "<i8") for n in ("Mx", "My", "Mxx", "Myy", "Mxy", "W", "a", "b")])
PEAK_EXTENTS = CLUSTER_EXTENTS
CORNER = np.dtype({"names": ["line_fit_point_index", "cluster_index", "error"],
                   "formats": ["<u4", "<u2", "<f4"], "offsets": [0, 4, 8], "itemsize": 12})
FITTED_QUAD = np.dtype([("moments", LINE_FIT_POINT, (4,)), ("num_in_moments", "<u2", (4,)),
                        ("indices", "<u2", (4,))])
QUAD_CORNERS = np.dtype([("corners", "<f4", (4, 2)), ("reversed_border", "u1"), ("pad_", "u1", (3,)),
                         ("blob_index", "<u4")])

assert BOUNDARY_POINT.itemsize == 4 and CLUSTER_POINT.itemsize == 8
assert CLUSTER_BOUNDS.itemsize == 32 and LINE_FIT_POINT.itemsize == 64
assert CORNER.itemsize == 12 and FITTED_QUAD.itemsize == 272 and QUAD_CORNERS.itemsize == 40


class Config(ctypes.Structure):
    _fields_ = [("decimate", ctypes.c_int32), ("min_white_black_diff", ctypes.c_int32),
                ("min_component_size", ctypes.c_int32), ("min_cluster_pixels", ctypes.c_int32),
                ("tag_width", ctypes.c_int32), ("normal_border", ctypes.c_int32),
                ("reversed_border", ctypes.c_int32), ("max_line_fit_mse", ctypes.c_float),
                ("critical_angle_deg", ctypes.c_float), ("min_tag_width", ctypes.c_int32),
                ("compat_peak_index", ctypes.c_int32)]


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t


class _Result(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int), ("height", ctypes.c_int),
                ("decimated", _P), ("thresholded", _P), ("labels", _P), ("sizes", _P),
                ("n_points", _SZ), ("points", _P), ("keys", _P),
                ("n_bounds", _SZ), ("bounds", _P), ("bound_keys", _P),
                ("n_filtered", _SZ), ("filtered", _P), ("filtered_keys", _P), ("extents", _P),
                ("n_cluster_points", _SZ), ("cluster_points", _P), ("cluster_indices", _P),
                ("line_fit", _P), ("found_corners", _P),
                ("n_corners", _SZ), ("corners", _P),
                ("n_peak_extents", _SZ), ("peak_extents", _P), ("fitted", _P),
                ("n_quads", _SZ), ("quads", _P)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("_atag_oracle_build",
                                                      os.path.join(HERE, "build_oracle.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = ctypes.CDLL(path)
        L.oracle_detect.restype = ctypes.c_int
        L.oracle_detect.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(Config),
                                    ctypes.POINTER(_Result)]
        L.oracle_free.argtypes = [ctypes.POINTER(_Result)]
        L.oracle_config_default.argtypes = [ctypes.POINTER(Config)]
        L.oracle_threshold.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P, _P]
        L.oracle_segmentation.argtypes = [_P, ctypes.c_int, ctypes.c_int, _P, _P, _P]
        L.oracle_find_boundaries.argtypes = [_P, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P, _P]
        L.oracle_decimate.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
        L.oracle_to_grey.argtypes = [_P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, _P]
        L.oracle_fit_lines_windowed.argtypes = [_P, _P, _P, _SZ, _P]
        L.oracle_fit_lines_cyclic.argtypes = [_P, _P, _P, _SZ, _P]
        L.oracle_do_indexing.argtypes = [_P, _SZ, _P, _P, _P, ctypes.POINTER(Config), _P]
        L.oracle_process_fitted_quads.restype = _SZ
        L.oracle_process_fitted_quads.argtypes = [_P, _SZ, ctypes.POINTER(Config), _P]
        L.oracle_hypotf.restype = ctypes.c_float
        L.oracle_hypotf.argtypes = [ctypes.c_float, ctypes.c_float]
        L.oracle_combination_decode.argtypes = [ctypes.c_uint32, _P]
        L.oracle_eval_bounds.argtypes = [_P, _P, _SZ, _SZ, _SZ, _P, _P, _P, _P, _P]
        L.oracle_eval_linefit.argtypes = [_P, _SZ, ctypes.c_uint32, ctypes.c_uint32, _P, _P]
        L.oracle_eval_fit_line.argtypes = [_P, _P, _SZ, _P, _P, _P]
        L.oracle_eval_get_moment.argtypes = [_P, _SZ, _P, _SZ, _P, _P]
        L.oracle_detect_many.restype = ctypes.c_int
        L.oracle_detect_many.argtypes = [_P, _P, _P, _SZ, ctypes.POINTER(Config), ctypes.c_int, _P]
        _lib = L
    return _lib


def default_config(**overrides) -> Config:
    c = Config()
    lib().oracle_config_default(ctypes.byref(c))
    for k, v in overrides.items():
        setattr(c, k, v)
    return c


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    buf = (ctypes.c_char * (n * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()


def detect(image: np.ndarray, cfg: Config = None) -> dict:
    """Runs the whole restated path on one source frame; returns every
    intermediate as numpy arrays."""
    img = np.ascontiguousarray(image, dtype=np.uint8)
    cfg = cfg or default_config()
    r = _Result()
    rc = lib().oracle_detect(_ptr(img), img.shape[1], img.shape[0], ctypes.byref(cfg), ctypes.byref(r))
    if rc != 0:
        raise ValueError(f"oracle_detect rejected a {img.shape[1]}x{img.shape[0]} frame")
    try:
        w, h = r.width, r.height
        N = w * h
        out = {
            "width": w, "height": h,
            "decimated": _arr(r.decimated, N, np.uint8).reshape(h, w),
            "thresholded": _arr(r.thresholded, N, np.uint8).reshape(h, w),
            "labels": _arr(r.labels, N, np.uint32).reshape(h, w),
            "sizes": _arr(r.sizes, N, np.uint32),
            "points": _arr(r.points, r.n_points, BOUNDARY_POINT),
            "keys": _arr(r.keys, r.n_points, np.uint64),
            "bounds": _arr(r.bounds, r.n_bounds, CLUSTER_BOUNDS),
            "bound_keys": _arr(r.bound_keys, r.n_bounds, np.uint64),
            "filtered": _arr(r.filtered, r.n_filtered, CLUSTER_BOUNDS),
            "filtered_keys": _arr(r.filtered_keys, r.n_filtered, np.uint64),
            "extents": _arr(r.extents, r.n_filtered, CLUSTER_EXTENTS),
            "cluster_points": _arr(r.cluster_points, r.n_cluster_points, CLUSTER_POINT),
            "cluster_indices": _arr(r.cluster_indices, r.n_cluster_points, np.uint32),
            "line_fit": _arr(r.line_fit, r.n_cluster_points, LINE_FIT_POINT),
            "found_corners": _arr(r.found_corners, r.n_cluster_points, CORNER),
            "corners": _arr(r.corners, r.n_corners, CORNER),
            "peak_extents": _arr(r.peak_extents, r.n_peak_extents, PEAK_EXTENTS),
            "fitted": _arr(r.fitted, r.n_peak_extents, FITTED_QUAD),
            "quads": _arr(r.quads, r.n_quads, QUAD_CORNERS),
        }
    finally:
        lib().oracle_free(ctypes.byref(r))
    return out


def threshold(grey: np.ndarray, min_diff: int = 5):
    g = np.ascontiguousarray(grey, dtype=np.uint8)
    h, w = g.shape
    ext = np.zeros((h // 4, w // 4, 2), np.uint8)
    flt = np.zeros((h // 4, w // 4, 2), np.uint8)
    out = np.zeros((h, w), np.uint8)
    lib().oracle_threshold(_ptr(g), w, h, min_diff, _ptr(ext), _ptr(flt), _ptr(out))
    return out, ext, flt


def segmentation(thr: np.ndarray):
    t = np.ascontiguousarray(thr, dtype=np.uint8)
    h, w = t.shape
    labels = np.zeros((h, w), np.uint32)
    sizes = np.zeros(h * w, np.uint32)
    lib().oracle_segmentation(_ptr(t), w, h, None, _ptr(labels), _ptr(sizes))
    return labels, sizes


def find_boundaries(labels: np.ndarray, sizes: np.ndarray, min_size: int = 25):
    lab = np.ascontiguousarray(labels, dtype=np.uint32)
    s = np.ascontiguousarray(sizes, dtype=np.uint32)
    h, w = lab.shape
    pts = np.zeros(4 * w * h, BOUNDARY_POINT)
    keys = np.full(4 * w * h, np.uint64(0xFFFFFFFFFFFFFFFF), np.uint64)
    lib().oracle_find_boundaries(_ptr(lab), _ptr(s), w, h, min_size, _ptr(pts), _ptr(keys))
    return pts, keys


def to_grey(src: np.ndarray, factor: int = 1, fmt: int = None) -> np.ndarray:
    """Colour removal + decimation (oracle_to_grey): src H x W or H x W x C."""
    src = np.ascontiguousarray(src, dtype=np.uint8)
    h, w = src.shape[0], src.shape[1]
    if fmt is None:
        fmt = 0 if src.ndim == 2 else {1: 0, 2: 5, 3: 1, 4: 2}[src.shape[2]]
    out = np.empty((h // factor, w // factor), np.uint8)
    lib().oracle_to_grey(_ptr(src), w, h, 0, fmt, factor, _ptr(out))
    return out


def decimate(src: np.ndarray, factor: int):
    s = np.ascontiguousarray(src, dtype=np.uint8)
    h, w = s.shape
    out = np.zeros((h // factor, w // factor), np.uint8)
    lib().oracle_decimate(_ptr(s), w, h, factor, _ptr(out))
    return out


def fit_lines(line_fit, cluster_indices, extents, windowed=True):
    lf = np.ascontiguousarray(line_fit)
    ci = np.ascontiguousarray(cluster_indices, dtype=np.uint32)
    ex = np.ascontiguousarray(extents)
    out = np.zeros(len(lf), CORNER)
    if len(lf):
        if windowed:
            lib().oracle_fit_lines_windowed(_ptr(lf), _ptr(ci), _ptr(ex), len(lf), _ptr(out))
        else:
            lib().oracle_fit_lines_cyclic(_ptr(lf), _ptr(ci), _ptr(ex), len(ex), _ptr(out))
    return out


def do_indexing(peak_extents, corners, line_fit, extents, cfg: Config = None):
    cfg = cfg or default_config()
    pe = np.ascontiguousarray(peak_extents)
    co = np.ascontiguousarray(corners)
    lf = np.ascontiguousarray(line_fit)
    ex = np.ascontiguousarray(extents)
    out = np.zeros(len(pe), FITTED_QUAD)
    if len(pe):
        lib().oracle_do_indexing(_ptr(pe), len(pe), _ptr(co), _ptr(lf), _ptr(ex), ctypes.byref(cfg),
                                 _ptr(out))
    return out


def process_fitted_quads(fitted, cfg: Config = None):
    cfg = cfg or default_config()
    f = np.ascontiguousarray(fitted)
    out = np.zeros(max(len(f), 1), QUAD_CORNERS)
    n = lib().oracle_process_fitted_quads(_ptr(f), len(f), ctypes.byref(cfg), _ptr(out))
    return out[:n]


def hypotf(a: float, b: float) -> float:
    return lib().oracle_hypotf(a, b)


def combination_decode(n: int):
    out = np.zeros(4, np.uint32)
    lib().oracle_combination_decode(n, _ptr(out))
    return out


def detect_many(frames, cfg: Config = None, threads: int = 0):
    """Runs oracle_detect over frames on `threads` OpenMP threads (0 = all).
    Returns (quad counts, threads used)."""
    cfg = cfg or default_config()
    frames = [np.ascontiguousarray(f, dtype=np.uint8) for f in frames]
    n = len(frames)
    ptrs = (ctypes.c_void_p * n)(*[f.ctypes.data for f in frames])
    ws = np.array([f.shape[1] for f in frames], np.int32)
    hs = np.array([f.shape[0] for f in frames], np.int32)
    nq = np.zeros(n, np.uint32)
    used = lib().oracle_detect_many(ctypes.cast(ptrs, ctypes.c_void_p), _ptr(ws), _ptr(hs), n,
                                    ctypes.byref(cfg), threads, _ptr(nq))
    return nq, used


def eval_bounds(bounds, points, width, height):
    """cx, cy, calc_theta(cx, cy), dot and ValidBlobFilter for each record."""
    b = np.ascontiguousarray(bounds)
    p = np.ascontiguousarray(points)
    n = len(b)
    cx, cy, th, dot = (np.zeros(n, np.float32) for _ in range(4))
    valid = np.zeros(n, np.uint8)
    lib().oracle_eval_bounds(_ptr(b), _ptr(p), n, width, height, _ptr(cx), _ptr(cy), _ptr(th), _ptr(dot),
                             _ptr(valid))
    return cx, cy, th, dot, valid


def eval_linefit(cluster_points, width, height, image):
    cp = np.ascontiguousarray(cluster_points)
    img = np.ascontiguousarray(image, dtype=np.uint8)
    out = np.zeros(len(cp), LINE_FIT_POINT)
    lib().oracle_eval_linefit(_ptr(cp), len(cp), width, height, _ptr(img), _ptr(out))
    return out


def eval_fit_line(moments, num_in_moment):
    m = np.ascontiguousarray(moments)
    nim = np.ascontiguousarray(num_in_moment, dtype=np.uint64)
    n = len(m)
    lp = np.zeros(4 * n, np.float32)
    err, mse = np.zeros(n, np.float32), np.zeros(n, np.float32)
    lib().oracle_eval_fit_line(_ptr(m), _ptr(nim), n, _ptr(lp), _ptr(err), _ptr(mse))
    return lp, err, mse


def eval_get_moment(prefix, ranges):
    pre = np.ascontiguousarray(prefix)
    r = np.ascontiguousarray(ranges, dtype=np.uint64)
    n = len(r) // 2
    out = np.zeros(n, LINE_FIT_POINT)
    cnt = np.zeros(n, np.uint64)
    lib().oracle_eval_get_moment(_ptr(pre), len(pre), _ptr(r), n, _ptr(out), _ptr(cnt))
    return out, cnt
