"""Reading tags (CUDA): each quad's bits matched against a code family that
the caller describes the way the AprilTag library describes its families
(per-bit cell coordinates, width at the border, total width).  The steps are
documented with atag_decode_quads in include/atag.h."""
import ctypes

import numpy as np
import torch

from . import lib
from .records import DECODED, QUAD_CORNERS, DecodeParams, TagFamily

_P = ctypes.c_void_p
REORDERED, DEGENERATE, LOW_CONTRAST = 0x1, 0x2, 0x4


class Family:
    """A tag family for atag_decode_quads: `layout` has bit_x, bit_y,
    width_at_border and total_width (e.g. atag.synth.classic_layout()),
    `codes` the family's codes (bit nbits - 1 - i = bit i)."""

    def __init__(self, layout, codes, max_hamming=2, reversed_border=False, device="cuda"):
        self.layout = layout
        self.bit_x = np.ascontiguousarray(layout.bit_x, dtype=np.int8)
        self.bit_y = np.ascontiguousarray(layout.bit_y, dtype=np.int8)
        c = np.asarray([int(v) for v in codes], dtype=np.uint64)
        self.codes = torch.from_numpy(c.view(np.int64).copy()).to(device) if len(c) else \
            torch.zeros(1, dtype=torch.int64, device=device)
        self.n_codes = len(c)
        self.max_hamming = max_hamming
        self.reversed_border = reversed_border

    def struct(self):
        return TagFamily(len(self.bit_x), self.layout.width_at_border, self.layout.total_width,
                         1 if self.reversed_border else 0, self.bit_x.ctypes.data, self.bit_y.ctypes.data,
                         self.codes.data_ptr(), self.n_codes, self.max_hamming)


def default_params(**overrides):
    p = DecodeParams()
    lib.load().atag_decode_params_default(ctypes.byref(p))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def decode_quads(image, corners, family: Family, params=None, stream=None):
    """image: H x W uint8 CUDA tensor; corners: Q x 4 x 2 float32 or Q x 40
    uint8 quad records (CUDA).  Returns a uint8 CUDA tensor of Q x 72 bytes
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
    out = torch.empty((n, DECODED.itemsize), dtype=torch.uint8, device=image.device)
    s = stream if stream is not None else torch.cuda.current_stream()
    fam = family.struct()
    prm = params if params is not None else default_params()
    lib.check(L.atag_decode_quads(_P(image.data_ptr()), image.shape[1], image.shape[0], image.shape[1],
                                  _P(corners.data_ptr()), stride, n, ctypes.byref(fam), ctypes.byref(prm),
                                  _P(out.data_ptr()), _P(s.cuda_stream)), "atag_decode_quads")
    return out


def to_numpy(decoded: torch.Tensor) -> np.ndarray:
    return np.frombuffer(decoded.cpu().numpy().tobytes(), dtype=DECODED)
