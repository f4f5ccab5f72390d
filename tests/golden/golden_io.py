"""Array names, record dtypes and the canonical digest shared by the golden
generator and the tests."""
import hashlib

import numpy as np

BOUNDARY_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2")])
CLUSTER_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2"), ("slope", "<f4")])
CLUSTER_EXTENTS = np.dtype([("start", "<u4"), ("count", "<u4")])
CLUSTER_BOUNDS = np.dtype([("x_min", "<u2"), ("x_max", "<u2"), ("y_min", "<u2"), ("y_max", "<u2"),
                           ("gx_sum", "<i4"), ("gy_sum", "<i4"), ("pxgx_pygy_sum", "<i8"),
                           ("start", "<u4"), ("count", "<u4")])
LINE_FIT_POINT = np.dtype([(n, "<i8") for n in ("Mx", "My", "Mxx", "Myy", "Mxy", "W", "a", "b")])
CORNER = np.dtype({"names": ["line_fit_point_index", "cluster_index", "error"],
                   "formats": ["<u4", "<u2", "<f4"], "offsets": [0, 4, 8], "itemsize": 12})
FITTED_QUAD = np.dtype([("moments", LINE_FIT_POINT, (4,)), ("num_in_moments", "<u2", (4,)),
                        ("indices", "<u2", (4,))])
QUAD_CORNERS = np.dtype([("corners", "<f4", (4, 2)), ("reversed_border", "u1"), ("pad_", "u1", (3,)),
                         ("blob_index", "<u4")])

PIPELINE_ARRAYS = {
    "thresholded": np.uint8, "extrema": np.uint8, "filtered_extrema": np.uint8,
    "labels": np.uint32, "sizes": np.uint32, "dense_points": BOUNDARY_POINT, "dense_keys": np.uint64,
    "points": BOUNDARY_POINT, "keys": np.uint64, "bounds": CLUSTER_BOUNDS, "bound_keys": np.uint64,
    "filtered_bounds": CLUSTER_BOUNDS, "filtered_keys": np.uint64, "extents": CLUSTER_EXTENTS,
    "cluster_points": CLUSTER_POINT, "cluster_indices": np.uint16, "line_fit": LINE_FIT_POINT,
    "found_corners": CORNER, "corners": CORNER, "peak_extents": CLUSTER_EXTENTS, "fitted": FITTED_QUAD,
    "quads": QUAD_CORNERS,
}

RECORD_ARRAYS = {
    "rec_combinadics": np.uint32, "rec_bounds": CLUSTER_BOUNDS, "rec_points": BOUNDARY_POINT,
    "rec_cx": np.float32, "rec_cy": np.float32, "rec_theta": np.float32, "rec_dot": np.float32,
    "rec_valid": np.uint8, "rec_image": np.uint8, "rec_cluster_points": CLUSTER_POINT,
    "rec_linefit": LINE_FIT_POINT, "rec_moments": LINE_FIT_POINT, "rec_num_in_moment": np.uint64,
    "rec_line_params": np.float32, "rec_err": np.float32, "rec_mse": np.float32, "rec_prefix": LINE_FIT_POINT,
    "rec_moment_range": np.uint64, "rec_moment": LINE_FIT_POINT, "rec_moment_n": np.uint64,
}


def _leaves(a):
    if a.dtype.names is None:
        return [np.ascontiguousarray(a).tobytes()]
    out = []
    for name in a.dtype.names:
        if name == "pad_":
            continue
        out += _leaves(a[name])
    return out


def digest(a) -> str:
    """SHA-256 over the fields of every record (padding excluded)."""
    a = np.asarray(a)
    h = hashlib.sha256()
    for b in _leaves(a):
        h.update(b)
    return h.hexdigest()
