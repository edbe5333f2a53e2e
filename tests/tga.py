"""Minimal TGA reader (uncompressed and RLE true-colour/grey) for the reference's shipped assets.

Returns rows top to bottom, channels RGB(A) like stbi_load, which the reference's texture loader
uses (Texture.cpp:215)."""
import numpy as np


def read_tga(path):
    b = open(path, "rb").read()
    id_len, cmap, itype = b[0], b[1], b[2]
    w, h, bpp, desc = b[12] | b[13] << 8, b[14] | b[15] << 8, b[16], b[17]
    if cmap != 0 or itype not in (2, 3, 10, 11):
        raise ValueError("unsupported TGA type %d" % itype)
    bp = bpp // 8
    o = 18 + id_len
    n = w * h * bp
    if itype in (2, 3):
        data = b[o:o + n]
    else:
        out = bytearray()
        while len(out) < n:
            c = b[o]
            o += 1
            cnt = (c & 0x7F) + 1
            if c & 0x80:
                out += b[o:o + bp] * cnt
                o += bp
            else:
                out += b[o:o + cnt * bp]
                o += cnt * bp
        data = bytes(out[:n])
    a = np.frombuffer(data, np.uint8).reshape(h, w, bp)
    if bp >= 3:
        a = a[..., [2, 1, 0] + ([3] if bp == 4 else [])]
    if not desc & 0x20:
        a = a[::-1]
    return np.ascontiguousarray(a)
