"""ctypes binding of libatag_gb300.so (the C ABI in include/atag.h).

There is no fallback: if the library is missing or the device is not an
sm_103 GPU, every call raises AtagError.
"""
import ctypes
import os
import re

from .records import (ClusterOutputs, ClusterPointC, Config, DecodeParams, Frame, FrameViews, LineFitPointC,
                      Limits, TagFamily, Tuning)

PKG_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_ROOT, "lib", "libatag_gb300.so")
HEADER = os.path.join(os.path.dirname(PKG_ROOT), "include", "atag.h")


class AtagError(RuntimeError):
    pass


_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_U32 = ctypes.c_uint32
_ST = ctypes.c_int
_D = ctypes.c_double

_SIGNATURES = {
    "atag_config_default": (None, [ctypes.POINTER(Config)]),
    "atag_status_string": (ctypes.c_char_p, [_ST]),
    "atag_last_error": (ctypes.c_char_p, []),
    "atag_init": (_ST, []),
    "atag_use_device": (_ST, [ctypes.c_int]),
    "atag_launch_count": (ctypes.c_uint64, []),
    "atag_decimate": (_ST, [_P, _SZ, _SZ, _SZ, _P, _P]),
    "atag_convert_grey": (_ST, [_P, _SZ, _SZ, _SZ, ctypes.c_int, _SZ, _P, _P]),
    "atag_threshold_image": (_ST, [_P, _P, _P, _P, _SZ, _SZ, _P]),
    "atag_image_segmentation": (_ST, [_P, _P, _P, _P, _SZ, _SZ, _SZ, _P]),
    "atag_image_segmentation_noalloc": (_ST, [_P, _P, _P, _SZ, _SZ, _P]),
    "atag_find_boundaries": (_ST, [_P, _P, _P, _P, _SZ, _SZ, _P]),
    "atag_fit_lines": (_ST, [_P, _P, _P, _SZ, _P, _P]),
    "atag_do_indexing": (_ST, [_P, _SZ, _P, _P, _P, _P, _P]),
    "atag_process_fitted_quads": (_ST, [_P, _SZ, _SZ, _SZ, ctypes.POINTER(Config), _P, _SZ, _P, _P]),
    "atag_cluster_workspace_size": (_ST, [_SZ, _SZ, _SZ, _SZ, ctypes.POINTER(_SZ)]),
    "atag_cluster": (_ST, [_P, _P, _P, _SZ, _SZ, _P, _SZ, ctypes.POINTER(ClusterOutputs), _P]),
    "atag_corner_peaks_workspace_size": (_ST, [_SZ, ctypes.POINTER(_SZ)]),
    "atag_corner_peaks": (_ST, [_P, _P, _SZ, _P, _SZ, _P, _SZ, _P, _SZ, _P, _P]),
    "atag_get_moment": (_ST, [_P, _SZ, _SZ, _SZ, _P, ctypes.POINTER(_SZ)]),
    "atag_fit_line": (_ST, [_P, _SZ, _P, _P, _P]),
    "atag_compute_initial_linefit": (LineFitPointC, [ClusterPointC, _U32, _U32, _P]),
    "atag_workspace_size": (_ST, [ctypes.POINTER(Config), _SZ, _SZ, _SZ, _SZ, ctypes.POINTER(_SZ)]),
    "atag_detector_create": (_ST, [ctypes.POINTER(Config), _SZ, _SZ, _SZ, _SZ, _P, _SZ, ctypes.POINTER(_P)]),
    "atag_detector_destroy": (_ST, [_P]),
    "atag_detect_batch": (_ST, [_P, ctypes.POINTER(Frame), _SZ, _P, _SZ, _P, _P]),
    "atag_detect": (_ST, [_P, _P, _SZ, _SZ, _P, _SZ, _P, _P]),
    "atag_detect_host": (_ST, [_P, _P, _SZ, _SZ, _P, _SZ, _P, _P]),
    "atag_detector_views": (_ST, [_P, _SZ, ctypes.POINTER(FrameViews)]),
    "atag_detector_keep_intermediates": (_ST, [_P, ctypes.c_int]),
    "atag_detector_set_limits": (_ST, [_P, ctypes.POINTER(Limits)]),
    "atag_detector_release_captures": (_ST, [_P]),
    "atag_detector_set_refinement": (_ST, [_P, ctypes.c_int]),
    "atag_detector_set_stage_events": (_ST, [_P, ctypes.POINTER(_P), _SZ]),
    "atag_stage_name": (ctypes.c_char_p, [ctypes.c_int]),
    "atag_detector_get_tuning": (_ST, [_P, ctypes.POINTER(Tuning)]),
    "atag_detector_set_tuning": (_ST, [_P, ctypes.POINTER(Tuning)]),
    "atag_refine_forward": (_ST, [_P, _SZ, _SZ, _P, _SZ, _P, _P, _P, _P]),
    "atag_refine_backward": (_ST, [_P, _SZ, _SZ, _P, _SZ, _P, _P, _P, _P, _P, _P]),
    "atag_estimate_pose": (_ST, [_P, _SZ, _SZ, _D, _D, _D, _D, _D, _U32, _P, _P]),
    "atag_decode_quads": (_ST, [_P, _SZ, _SZ, _SZ, _P, _SZ, _SZ, ctypes.POINTER(TagFamily),
                                ctypes.POINTER(DecodeParams), _P, _P]),
    "atag_decode_params_default": (None, [ctypes.POINTER(DecodeParams)]),
}
STAGE_COUNT = 16

_lib = None


def declared_symbols():
    """Function names declared in include/atag.h."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(atag_[a-z_]+)\s*\(", text)))


def load(build_if_missing: bool = True):
    """Loads (building in-tree first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from importlib import util
        spec = util.spec_from_file_location("_atag_build", os.path.join(PKG_ROOT, "build.py"))
        mod = util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    if not os.path.exists(LIB_PATH):
        raise AtagError(f"CUDA library not built: {LIB_PATH}")
    L = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int, what: str = ""):
    if status != 0:
        L = load()
        raise AtagError(f"{what}: {L.atag_status_string(status).decode()}: {L.atag_last_error().decode()}")


def default_config(**overrides) -> Config:
    c = Config()
    load().atag_config_default(ctypes.byref(c))
    for k, v in overrides.items():
        if not hasattr(c, k):
            raise AttributeError(k)
        setattr(c, k, v)
    return c


def init(device: int = None):
    L = load()
    if device is None:
        import torch
        device = torch.cuda.current_device()
    check(L.atag_use_device(int(device)), "atag_use_device")
    check(L.atag_init(), "atag_init")
    return L


def launch_count() -> int:
    return int(load().atag_launch_count())
