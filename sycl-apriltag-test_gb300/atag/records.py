"""numpy mirrors of the C records in include/atag.h (layout-identical to the
reference's BoundaryPoint, ClusterPoint, ClusterBounds, LineFitPoint,
Corner, FittedQuad, QuadCorners)."""
import ctypes

import numpy as np

BOUNDARY_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2")])
CLUSTER_POINT = np.dtype([("packed_x", "<u2"), ("packed_y", "<u2"), ("slope", "<f4")])
CLUSTER_EXTENTS = np.dtype([("start", "<u4"), ("count", "<u4")])
PEAK_EXTENTS = CLUSTER_EXTENTS
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
FRAME_STATS = np.dtype([(n, "<u4") for n in ("width", "height", "n_points", "n_pairs", "n_clusters",
                                              "n_cluster_points", "n_corners", "n_peak_clusters",
                                              "n_fitted", "n_quads", "status")] + [("reserved", "<u4", (5,))])

POSE = np.dtype([("R", "<f8", (3, 3)), ("t", "<f8", (3,)), ("H", "<f8", (3, 3)), ("reproj_rms", "<f8"),
                 ("iterations", "<u4"), ("status", "<u4")])

DECODED = np.dtype([("code", "<u8"), ("id", "<i4"), ("hamming", "<u4"), ("rotation", "<u4"), ("status", "<u4"),
                    ("decision_margin", "<f4"), ("black", "<f4"), ("white", "<f4"), ("corners", "<f4", (4, 2)),
                    ("reserved", "<u4")])

assert POSE.itemsize == 184 and DECODED.itemsize == 72
assert BOUNDARY_POINT.itemsize == 4 and CLUSTER_POINT.itemsize == 8 and CLUSTER_EXTENTS.itemsize == 8
assert CLUSTER_BOUNDS.itemsize == 32 and LINE_FIT_POINT.itemsize == 64 and CORNER.itemsize == 12
assert FITTED_QUAD.itemsize == 272 and QUAD_CORNERS.itemsize == 40 and FRAME_STATS.itemsize == 64


class Config(ctypes.Structure):
    """atag_config; field order and types follow include/atag.h."""
    _fields_ = [("decimate", ctypes.c_int32), ("min_white_black_diff", ctypes.c_int32),
                ("min_component_size", ctypes.c_int32), ("min_cluster_pixels", ctypes.c_int32),
                ("tag_width", ctypes.c_int32), ("normal_border", ctypes.c_int32),
                ("reversed_border", ctypes.c_int32), ("max_line_fit_mse", ctypes.c_float),
                ("critical_angle_deg", ctypes.c_float), ("min_tag_width", ctypes.c_int32),
                ("compat_peak_index", ctypes.c_int32)]


# atag_pixel_format (include/atag.h)
PIX_GREY8, PIX_RGB8, PIX_RGBA8, PIX_BGR8, PIX_BGRA8, PIX_GREYA8 = range(6)
PIXEL_BYTES = {PIX_GREY8: 1, PIX_RGB8: 3, PIX_RGBA8: 4, PIX_BGR8: 3, PIX_BGRA8: 4, PIX_GREYA8: 2}


class Frame(ctypes.Structure):
    _fields_ = [("d_grey", ctypes.c_void_p), ("src_width", ctypes.c_uint32), ("src_height", ctypes.c_uint32),
                ("format", ctypes.c_uint32), ("src_pitch", ctypes.c_uint32)]


class FrameViews(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("decimated", "thresholded", "labels", "sizes", "pair_points")] + \
               [("n_pair_points", ctypes.c_uint32), ("pair_capacity", ctypes.c_uint32)] + \
               [(n, ctypes.c_void_p) for n in ("pair_keys", "pair_count", "pair_bbox", "pair_gsum", "pair_pxgx")] + \
               [(n, ctypes.c_void_p) for n in ("cluster_keys", "cluster_bounds", "cluster_extents",
                                                "cluster_points", "line_fit_points", "peak_count", "peaks",
                                                "peak_clusters", "peak_extents", "fitted")] + \
               [(n, ctypes.c_uint32) for n in ("point_capacity", "cluster_capacity", "cluster_point_capacity",
                                                "reserved_")]


class Limits(ctypes.Structure):
    """atag_limits: per-frame capacities and iteration caps (0 = default)."""
    _fields_ = [(n, ctypes.c_uint32) for n in ("point_capacity", "pair_capacity", "cluster_capacity",
                                                "cluster_point_capacity", "uf_iteration_cap")] + \
               [("reserved", ctypes.c_uint32 * 3)]

# device flag bits (atag_frame_stats.status)
DEVFLAG_POINT_OVERFLOW = 0x1
DEVFLAG_PAIR_OVERFLOW = 0x2
DEVFLAG_CLUSTER_OVERFLOW = 0x4
DEVFLAG_UF_ITERATION_CAP = 0x8
DEVFLAG_QUAD_OVERFLOW = 0x10
DEVFLAG_SORT_OVERFLOW = 0x20


class LineFitPointC(ctypes.Structure):
    """atag_line_fit_point passed by value."""
    _fields_ = [(n, ctypes.c_int64) for n in ("Mx", "My", "Mxx", "Myy", "Mxy", "W", "a", "b")]


class ClusterPointC(ctypes.Structure):
    """atag_cluster_point passed by value."""
    _fields_ = [("packed_x", ctypes.c_uint16), ("packed_y", ctypes.c_uint16), ("slope", ctypes.c_float)]


class ClusterOutputs(ctypes.Structure):
    """atag_cluster_outputs: device arrays and capacities atag_cluster writes."""
    _fields_ = [("pair_bounds", ctypes.c_void_p), ("pair_keys", ctypes.c_void_p), ("pair_capacity", ctypes.c_size_t),
                ("filtered_bounds", ctypes.c_void_p), ("filtered_keys", ctypes.c_void_p),
                ("cluster_extents", ctypes.c_void_p), ("cluster_capacity", ctypes.c_size_t),
                ("cluster_points", ctypes.c_void_p), ("cluster_indices", ctypes.c_void_p),
                ("line_fit_points", ctypes.c_void_p), ("point_capacity", ctypes.c_size_t),
                ("counts", ctypes.c_void_p)]


class TagFamily(ctypes.Structure):
    """atag_tag_family (bit cells on the host, codes on the device)."""
    _fields_ = [("nbits", ctypes.c_uint32), ("width_at_border", ctypes.c_uint32), ("total_width", ctypes.c_uint32),
                ("reversed_border", ctypes.c_uint32), ("h_bit_x", ctypes.c_void_p), ("h_bit_y", ctypes.c_void_p),
                ("d_codes", ctypes.c_void_p), ("n_codes", ctypes.c_uint32), ("max_hamming", ctypes.c_uint32)]


class DecodeParams(ctypes.Structure):
    """atag_decode_params."""
    _fields_ = [("decode_sharpening", ctypes.c_float), ("refine_edges", ctypes.c_int32),
                ("quad_decimate", ctypes.c_int32), ("min_contrast", ctypes.c_float)]


class Tuning(ctypes.Structure):
    """atag_tuning: launch shapes of the detector's kernels."""
    _fields_ = [("ccl_tile_rows", ctypes.c_int32), ("boundary_tile_rows", ctypes.c_int32),
                ("small_cluster_max", ctypes.c_int32), ("small_ctas_per_sm", ctypes.c_int32),
                ("large_ctas_divisor", ctypes.c_int32), ("index_ctas_per_sm", ctypes.c_int32),
                ("batch_lanes", ctypes.c_int32)]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}
