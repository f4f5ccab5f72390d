"""Reading tags (CUDA): the bit grid of each quad matched against a code
family given by the caller; layout, sampling and matching are documented
with atag_decode_quads in include/atag.h."""
import ctypes

import numpy as np
import torch

from . import lib
from .records import DECODED, QUAD_CORNERS

_P = ctypes.c_void_p
REORDERED, DEGENERATE, LOW_CONTRAST = 0x1, 0x2, 0x4


def decode_quads(image, corners, codes, data_side=6, max_hamming=2, min_contrast=10.0, stream=None):
    """image: H x W uint8 CUDA tensor; corners: Q x 4 x 2 float32 or Q x 40
    uint8 quad records (CUDA); codes: int64/uint64 tensor or array of the
    family's codes.  Returns a uint8 CUDA tensor of Q x 40 bytes
    (atag_decoded records); `to_numpy` reads it."""
    L = lib.init()
    image = image.contiguous()
    if image.dtype != torch.uint8 or image.dim() != 2:
        raise ValueError("image must be H x W uint8")
    if corners.dtype == torch.float32:
        corners = corners.contiguous()
        n, stride = corners.shape[0], 32
    elif corners.dtype == torch.uint8:
        corners = corners.contiguous()
        n, stride = corners.shape[0], QUAD_CORNERS.itemsize
    else:
        raise ValueError("corners must be float32 corners or uint8 quad records")
    if not isinstance(codes, torch.Tensor):
        codes = torch.from_numpy(np.asarray(codes, dtype=np.uint64).view(np.int64))
    codes = codes.to(device=image.device, dtype=torch.int64).contiguous()
    out = torch.empty((n, DECODED.itemsize), dtype=torch.uint8, device=image.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    lib.check(L.atag_decode_quads(_P(image.data_ptr()), image.shape[1], image.shape[0], image.shape[1],
                                  _P(corners.data_ptr()), stride, n, _P(codes.data_ptr()), codes.numel(),
                                  int(data_side), int(max_hamming), float(min_contrast), _P(out.data_ptr()),
                                  _P(s.cuda_stream)), "atag_decode_quads")
    return out


def to_numpy(decoded: torch.Tensor) -> np.ndarray:
    return np.frombuffer(decoded.cpu().numpy().tobytes(), dtype=DECODED)
