"""Minimal PNG decoder (8-bit greyscale, non-interlaced) with zlib + numpy,
used to turn the reference project's input images into fixtures."""
import struct
import zlib

import numpy as np


def read_png_grey(path: str) -> np.ndarray:
    d = open(path, "rb").read()
    if d[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG")
    pos, idat, w, h = 8, b"", None, None
    while pos < len(d):
        (ln,) = struct.unpack(">I", d[pos:pos + 4])
        typ, body = d[pos + 4:pos + 8], d[pos + 8:pos + 8 + ln]
        if typ == b"IHDR":
            w, h, bd, ct, _cm, _fm, il = struct.unpack(">IIBBBBB", body)
            if bd != 8 or ct != 0 or il != 0:
                raise ValueError("only 8-bit greyscale non-interlaced PNGs")
        elif typ == b"IDAT":
            idat += body
        elif typ == b"IEND":
            break
        pos += 12 + ln
    raw = zlib.decompress(idat)
    out = np.zeros((h, w), np.uint8)
    prev = np.zeros(w, np.int32)
    stride = w + 1
    for y in range(h):
        f = raw[y * stride]
        line = np.frombuffer(raw, np.uint8, w, y * stride + 1).astype(np.int32)
        if f == 0:
            cur = line
        elif f == 2:
            cur = (line + prev) & 255
        else:
            cur = np.zeros(w, np.int32)
            for x in range(w):
                a = cur[x - 1] if x else 0
                b = prev[x]
                c = prev[x - 1] if x else 0
                if f == 1:
                    pr = a
                elif f == 3:
                    pr = (a + b) >> 1
                else:
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pr = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                cur[x] = (line[x] + pr) & 255
        out[y] = cur
        prev = cur
    return out
