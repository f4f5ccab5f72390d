"""Detector: the whole quad-detection path for one frame or a batch of
frames of mixed sizes, over a workspace that torch allocates once."""
import ctypes

import numpy as np
import torch

from . import lib
from .records import (CLUSTER_BOUNDS, CLUSTER_EXTENTS, CLUSTER_POINT, CORNER, FITTED_QUAD, FRAME_STATS,
                      LINE_FIT_POINT, PEAK_EXTENTS, PIX_GREY8, PIX_GREYA8, PIX_RGB8, PIX_RGBA8, PIXEL_BYTES,
                      QUAD_CORNERS, Frame, FrameViews)


def frame_format(t):
    """atag_pixel_format implied by a frame tensor's shape."""
    if t.dim() == 2:
        return PIX_GREY8
    return {1: PIX_GREY8, 2: PIX_GREYA8, 3: PIX_RGB8, 4: PIX_RGBA8}[t.shape[2]]

_P = ctypes.c_void_p


class Detector:
    """Wraps atag_detector (include/atag.h).

    max_width/max_height bound a frame after decimation; max_frames and
    max_total_pixels bound a batch.  `enqueue` is stream-ordered and does not
    synchronise; `results` copies the quads back.
    """

    def __init__(self, max_width: int, max_height: int, max_frames: int = 1, max_total_pixels: int = 0,
                 config=None, quad_capacity: int = 1024, keep_intermediates: bool = False):
        self.L = lib.init()
        self.cfg = config or lib.default_config()
        self.max_frames = max_frames
        self.quad_capacity = quad_capacity
        size = ctypes.c_size_t()
        lib.check(self.L.atag_workspace_size(ctypes.byref(self.cfg), max_width, max_height, max_frames,
                                             max_total_pixels, ctypes.byref(size)), "atag_workspace_size")
        self.workspace = torch.empty(size.value, dtype=torch.uint8, device="cuda")
        self.handle = _P()
        lib.check(self.L.atag_detector_create(ctypes.byref(self.cfg), max_width, max_height, max_frames,
                                              max_total_pixels, _P(self.workspace.data_ptr()), size.value,
                                              ctypes.byref(self.handle)), "atag_detector_create")
        self.d_quads = torch.zeros(max_frames * quad_capacity * QUAD_CORNERS.itemsize, dtype=torch.uint8,
                                   device="cuda")
        self.d_stats = torch.zeros(max_frames * FRAME_STATS.itemsize, dtype=torch.uint8, device="cuda")
        self._frames = []
        self._n = 0
        self.keep_intermediates(keep_intermediates)

    def keep_intermediates(self, keep: bool = True):
        """With keep, later calls also write the reference's full scratch and
        sizes arrays (zeros away from component roots) and sum every pair in
        full, which `views` shows; by default only what the later stages read
        is written, and pairs already over the cluster size limit stop being
        summed."""
        lib.check(self.L.atag_detector_keep_intermediates(self.handle, 1 if keep else 0),
                  "atag_detector_keep_intermediates")

    def set_limits(self, **fields):
        """Per-frame capacities and the union-find iteration cap of later
        calls (atag_limits; 0 or absent = the detector's own sizing):
        point_capacity, pair_capacity, cluster_capacity,
        cluster_point_capacity, uf_iteration_cap."""
        from .records import Limits
        lim = Limits()
        for k, v in fields.items():
            setattr(lim, k, int(v))
        lib.check(self.L.atag_detector_set_limits(self.handle, ctypes.byref(lim)), "atag_detector_set_limits")

    def close(self):
        if self.handle:
            self.L.atag_detector_destroy(self.handle)
            self.handle = _P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def enqueue(self, frames, stream=None, formats=None):
        """Launches detection of `frames` (uint8 CUDA tensors before colour
        removal and decimation: H x W grey, or H x W x C with C = 2 grey +
        alpha, 3 RGB, 4 RGBA) on `stream` (default: torch's current stream).
        `formats` (one atag_pixel_format per frame) overrides the format
        implied by the shape, e.g. for BGR."""
        frames = [f if f.is_contiguous() else f.contiguous() for f in frames]
        n = len(frames)
        arr = (Frame * n)()
        for i, f in enumerate(frames):
            assert f.dtype == torch.uint8 and f.is_cuda and f.dim() in (2, 3)
            fmt = formats[i] if formats is not None else frame_format(f)
            arr[i].d_grey = f.data_ptr()
            arr[i].src_width = f.shape[1]
            arr[i].src_height = f.shape[0]
            arr[i].format = fmt
            arr[i].src_pitch = f.shape[1] * PIXEL_BYTES[fmt]
        s = stream if stream is not None else torch.cuda.current_stream()
        lib.check(self.L.atag_detect_batch(self.handle, arr, n, _P(self.d_quads.data_ptr()), self.quad_capacity,
                                           _P(self.d_stats.data_ptr()), _P(s.cuda_stream)), "atag_detect_batch")
        self._frames = frames
        self._n = n

    def stats(self) -> np.ndarray:
        return self.d_stats[: self._n * FRAME_STATS.itemsize].cpu().numpy().view(FRAME_STATS)

    def results(self, n_frames: int = None):
        """(list of QUAD_CORNERS arrays, stats array) of the last enqueue, or
        of the first n_frames output slots (e.g. after a graph replay)."""
        n = self._n if n_frames is None else n_frames
        st = self.d_stats[: n * FRAME_STATS.itemsize].cpu().numpy().view(FRAME_STATS)
        q = self.d_quads[: n * self.quad_capacity * QUAD_CORNERS.itemsize].cpu().numpy().view(QUAD_CORNERS)
        q = q.reshape(n, self.quad_capacity)
        return [q[i, : int(st[i]["n_quads"])].copy() for i in range(n)], st

    def set_refinement(self, enable: bool = True):
        """Later calls replace each quad's corners by their subpixel
        refinement on the frame's grey image (atag_detector_set_refinement)."""
        lib.check(self.L.atag_detector_set_refinement(self.handle, 1 if enable else 0), "atag_detector_set_refinement")

    def release_captures(self):
        """Frees the frame tables held for captured graphs (after those
        graphs are destroyed)."""
        lib.check(self.L.atag_detector_release_captures(self.handle), "atag_detector_release_captures")

    def detect(self, frames, formats=None):
        self.enqueue(frames, formats=formats)
        return self.results()

    def detect_host(self, image: np.ndarray, stream=None):
        """Host-buffer path: copy in, detect, copy out, synchronise."""
        img = np.ascontiguousarray(image, dtype=np.uint8)
        cap = min(self.quad_capacity, 4096)
        out = np.zeros(cap, QUAD_CORNERS)
        st = np.zeros(1, FRAME_STATS)
        s = stream if stream is not None else torch.cuda.current_stream()
        lib.check(self.L.atag_detect_host(self.handle, _P(img.ctypes.data), img.shape[1], img.shape[0],
                                          _P(out.ctypes.data), cap, _P(st.ctypes.data), _P(s.cuda_stream)),
                  "atag_detect_host")
        return out[: int(st[0]["n_quads"])], st[0]

    # -- launch shapes -------------------------------------------------------
    def get_tuning(self) -> dict:
        from .records import Tuning
        t = Tuning()
        lib.check(self.L.atag_detector_get_tuning(self.handle, ctypes.byref(t)), "get_tuning")
        return t.as_dict()

    def set_tuning(self, **fields):
        from .records import Tuning
        t = Tuning()
        lib.check(self.L.atag_detector_get_tuning(self.handle, ctypes.byref(t)), "get_tuning")
        for k, v in fields.items():
            setattr(t, k, int(v))
        lib.check(self.L.atag_detector_set_tuning(self.handle, ctypes.byref(t)), "set_tuning")

    # -- stage timing --------------------------------------------------------
    def set_stage_events(self, events):
        """events: lib.STAGE_COUNT + 1 torch.cuda.Event(enable_timing=True)
        (or None to stop).  Each later enqueue records them between stages."""
        if not events:
            lib.check(self.L.atag_detector_set_stage_events(self.handle, None, 0), "set_stage_events")
            self._stage_events = None
            return
        for e in events:  # torch creates the CUDA event on first record
            e.record()
        arr = (_P * len(events))(*[e.cuda_event for e in events])
        lib.check(self.L.atag_detector_set_stage_events(self.handle, arr, len(events)), "set_stage_events")
        self._stage_events = list(events)

    def stage_times_ms(self):
        """Per-stage device times of the last enqueue (needs set_stage_events;
        synchronises on the last event)."""
        ev = self._stage_events
        ev[-1].synchronize()
        return {lib.load().atag_stage_name(i).decode(): ev[i].elapsed_time(ev[i + 1])
                for i in range(len(ev) - 1)}

    # -- intermediates -------------------------------------------------------
    def _dev_bytes(self, ptr, nbytes):
        if nbytes == 0 or not ptr:
            return np.zeros(0, np.uint8)
        base = self.workspace.data_ptr()
        if base <= ptr < base + self.workspace.numel():
            off = ptr - base
            return self.workspace[off: off + nbytes].cpu().numpy()
        for f in self._frames:
            if f.data_ptr() <= ptr < f.data_ptr() + f.numel():
                off = ptr - f.data_ptr()
                return f.reshape(-1)[off: off + nbytes].cpu().numpy()
        raise ValueError("pointer outside the workspace")

    def views(self, i: int = 0) -> dict:
        """Copies frame i's intermediates to the host (numpy records).
        `sizes` is exact at component roots (the labels' values); elsewhere it
        holds the reference's zeros only on a detector that keeps
        intermediates."""
        v = FrameViews()
        lib.check(self.L.atag_detector_views(self.handle, i, ctypes.byref(v)), "atag_detector_views")
        st = self.stats()[i]
        w, h = int(st["width"]), int(st["height"])
        N = w * h
        ncl, npf, ncp = int(st["n_clusters"]), int(st["n_cluster_points"]), int(st["n_peak_clusters"])
        npts = int(v.n_pair_points)
        pc = int(v.pair_capacity)
        g = self._dev_bytes
        return {
            "stats": st,
            "capacities": {"point": int(v.point_capacity), "pair": pc, "cluster": int(v.cluster_capacity),
                           "cluster_point": int(v.cluster_point_capacity)},
            "pointers": {n: int(getattr(v, n) or 0) for n, _ in FrameViews._fields_
                         if n not in ("n_pair_points", "pair_capacity", "point_capacity", "cluster_capacity",
                                      "cluster_point_capacity", "reserved_")},
            "decimated": g(v.decimated, N).reshape(h, w),
            "thresholded": g(v.thresholded, N).reshape(h, w),
            "labels": g(v.labels, 4 * N).view(np.uint32).reshape(h, w),
            "sizes": g(v.sizes, 4 * N).view(np.uint32),
            "pair_points": g(v.pair_points, 8 * npts).view(np.uint64),
            "pair_keys": g(v.pair_keys, 8 * pc).view(np.uint64),
            "pair_count": g(v.pair_count, 4 * pc).view(np.uint32),
            "pair_bbox": g(v.pair_bbox, 16 * pc).view(np.uint32).reshape(pc, 4),
            "pair_gsum": g(v.pair_gsum, 8 * pc).view(np.int32).reshape(pc, 2),
            "pair_pxgx": g(v.pair_pxgx, 8 * pc).view(np.int64),
            "cluster_keys": g(v.cluster_keys, 8 * ncl).view(np.uint64),
            "cluster_bounds": g(v.cluster_bounds, 32 * ncl).view(CLUSTER_BOUNDS),
            "cluster_extents": g(v.cluster_extents, 8 * ncl).view(CLUSTER_EXTENTS),
            "cluster_points": g(v.cluster_points, 8 * npf).view(CLUSTER_POINT),
            "line_fit": g(v.line_fit_points, 64 * npf).view(LINE_FIT_POINT),
            "peak_count": g(v.peak_count, 4 * ncl).view(np.uint32),
            "peaks": g(v.peaks, CORNER.itemsize * 10 * ncl).view(CORNER).reshape(ncl, 10) if ncl else
            np.zeros((0, 10), CORNER),
            "peak_clusters": g(v.peak_clusters, 4 * ncp).view(np.uint32),
            "peak_extents": g(v.peak_extents, 8 * ncp).view(PEAK_EXTENTS),
            "fitted": g(v.fitted, FITTED_QUAD.itemsize * ncp).view(FITTED_QUAD),
        }
