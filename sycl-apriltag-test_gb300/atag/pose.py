"""Tag pose from quad corners (CUDA, FP64): the convention, camera model and
method are documented with atag_estimate_pose in include/atag.h."""
import ctypes

import numpy as np
import torch

from . import lib
from .records import POSE, QUAD_CORNERS

_P = ctypes.c_void_p
REORDERED, DEGENERATE = 0x1, 0x2


def estimate_pose(corners, fx, fy, cx, cy, tag_size, max_iterations=20, stream=None):
    """corners: a CUDA tensor of Q x 4 x 2 float32 corners, or a uint8 tensor
    of Q x 40 bytes holding atag_quad_corners records (detector output).
    Returns a uint8 CUDA tensor of Q x 184 bytes (atag_pose records); use
    `to_numpy` to read it."""
    L = lib.init()
    if corners.dtype == torch.float32:
        corners = corners.contiguous()
        if corners.dim() != 3 or tuple(corners.shape[1:]) != (4, 2):
            raise ValueError("corners must be Q x 4 x 2 float32")
        n, stride = corners.shape[0], 32
    elif corners.dtype == torch.uint8:
        corners = corners.contiguous()
        if corners.dim() != 2 or corners.shape[1] != QUAD_CORNERS.itemsize:
            raise ValueError("quad records must be Q x 40 bytes")
        n, stride = corners.shape[0], QUAD_CORNERS.itemsize
    else:
        raise ValueError("corners must be float32 corners or uint8 quad records")
    out = torch.empty((n, POSE.itemsize), dtype=torch.uint8, device=corners.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    lib.check(L.atag_estimate_pose(_P(corners.data_ptr()), stride, n, float(fx), float(fy), float(cx), float(cy),
                                   float(tag_size), int(max_iterations), _P(out.data_ptr()), _P(s.cuda_stream)),
              "atag_estimate_pose")
    return out


def to_numpy(poses: torch.Tensor) -> np.ndarray:
    """atag_pose records as a structured array (fields R, t, H, reproj_rms,
    iterations, status)."""
    return np.frombuffer(poses.cpu().numpy().tobytes(), dtype=POSE)
