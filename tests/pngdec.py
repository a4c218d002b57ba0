"""PNG reader for the tests: chunk CRCs checked, zlib inflated by Python's
zlib, the five scanline filters undone (ISO/IEC 15948 section 9)."""
from __future__ import annotations

import struct
import zlib

import numpy as np


def unfilter(raw: np.ndarray, w: int, h: int) -> np.ndarray:
    out = np.zeros((h, w * 4), np.int64)
    for y in range(h):
        f, r = int(raw[y, 0]), raw[y, 1:].astype(np.int64)
        up = out[y - 1] if y else np.zeros(w * 4, np.int64)
        assert f in (0, 1, 2, 3, 4), f
        if f == 0:
            out[y] = r
        elif f == 1:  # Sub: a running sum per channel
            out[y] = (np.cumsum(r.reshape(w, 4), axis=0) & 255).reshape(-1)
        elif f == 2:
            out[y] = (r + up) & 255
        else:
            row = [0] * (w * 4)
            rr, uu = r.tolist(), up.tolist()
            for i in range(w * 4):
                a = row[i - 4] if i >= 4 else 0
                b = uu[i]
                if f == 3:
                    pred = (a + b) >> 1
                else:
                    c = uu[i - 4] if i >= 4 else 0
                    p = a + b - c
                    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
                    pred = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
                row[i] = (rr[i] + pred) & 255
            out[y] = row
    return out.astype(np.uint8).reshape(h, w, 4)


def decode(data: bytes) -> np.ndarray:
    """RGBA8 pixels (h, w, 4) of an 8-bit RGBA, non-interlaced PNG."""
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    pos, idat, w, h = 8, b"", 0, 0
    while pos < len(data):
        n, = struct.unpack(">I", data[pos:pos + 4])
        t, c = data[pos + 4:pos + 8], data[pos + 8:pos + 8 + n]
        crc, = struct.unpack(">I", data[pos + 8 + n:pos + 12 + n])
        assert crc == zlib.crc32(t + c) & 0xFFFFFFFF
        if t == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", c[:13])
            assert (depth, ctype, interlace) == (8, 6, 0)
        elif t == b"IDAT":
            idat += c
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, w * 4 + 1)
    return unfilter(raw, w, h)
