"""Minimal PNG writer and reader built on Python's zlib, independent of the library's decoder.

write_png produces every row filter type (0..4, cycling by row, or one fixed type) at any zlib
level (0 = stored blocks); read_png follows the PNG specification (non-interlaced, 8/16-bit, colour
types 0/2/4/6) and returns the samples unconverted, as (h, w, channels) uint8 or uint16."""
import struct
import zlib

import numpy as np

_CH = {0: 1, 2: 3, 4: 2, 6: 4}


def _chunk(t, data):
    return struct.pack(">I", len(data)) + t + data + struct.pack(">I", zlib.crc32(t + data) & 0xFFFFFFFF)


def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = np.abs(p - a), np.abs(p - b), np.abs(p - c)
    return np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, c))


def write_png(path, samples, depth=8, filt=None, level=6, trns=None):
    """samples: (h, w, c) array with c in 1..4 (grey, grey+alpha, RGB, RGBA)."""
    h, w, c = samples.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    if depth == 16:
        raw = samples.astype(">u2").tobytes()
    else:
        raw = samples.astype(np.uint8).tobytes()
    bpp = c * depth // 8
    stride = w * bpp
    rows = np.frombuffer(raw, np.uint8).reshape(h, stride).astype(np.int32)
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft = (y % 5) if filt is None else filt
        cur = rows[y]
        a = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        c_ = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        pred = [0, a, prev, (a + prev) >> 1, _paeth(a, prev, c_)][ft]
        out.append(ft)
        out += ((cur - pred) & 0xFF).astype(np.uint8).tobytes()
        prev = cur
    ihdr = struct.pack(">IIBBBBB", w, h, depth, ctype, 0, 0, 0)
    body = _chunk(b"IHDR", ihdr)
    if trns is not None:
        body += _chunk(b"tRNS", struct.pack(">" + "H" * len(trns), *trns))
    body += _chunk(b"tEXt", b"Comment\x00ancillary chunk")
    body += _chunk(b"IDAT", zlib.compress(bytes(out), level))
    body += _chunk(b"IEND", b"")
    open(path, "wb").write(b"\x89PNG\r\n\x1a\n" + body)


def read_png(path):
    b = open(path, "rb").read()
    assert b[:8] == b"\x89PNG\r\n\x1a\n"
    o, idat = 8, b""
    while o < len(b):
        n, t = struct.unpack(">I4s", b[o:o + 8])
        d = b[o + 8:o + 8 + n]
        if t == b"IHDR":
            w, h, depth, ctype, _, _, inter = struct.unpack(">IIBBBBB", d)
            assert inter == 0
        elif t == b"IDAT":
            idat += d
        o += 12 + n
    c = _CH[ctype]
    bpp = c * depth // 8
    stride = w * bpp
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(h, stride + 1)
    img = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft, s = raw[y, 0], raw[y, 1:].astype(np.int32)
        if ft == 0:
            cur = s.copy()
        elif ft == 1:  # Sub: a running sum per byte lane of the pixel
            cur = np.cumsum(s.reshape(w, bpp), axis=0).reshape(-1) & 0xFF
        elif ft == 2:
            cur = (s + prev) & 0xFF
        else:  # Average / Paeth: sequential over pixels, vectorized over the pixel's bytes
            cur = np.zeros(stride, np.int32)
            zero = np.zeros(bpp, np.int32)
            for i in range(0, stride, bpp):
                a = cur[i - bpp:i] if i else zero
                b = prev[i:i + bpp]
                cc = prev[i - bpp:i] if i else zero
                pr = (a + b) >> 1 if ft == 3 else _paeth(a, b, cc)
                cur[i:i + bpp] = (s[i:i + bpp] + pr) & 0xFF
        img[y] = cur
        prev = cur
    img = img.astype(np.uint8)
    if depth == 16:
        return img.view(">u2").reshape(h, w, c).astype(np.uint16)
    return img.reshape(h, w, c)


def write_tga(path, rgba, rle=True, top_down=False, channels=4):
    """(h, w, 4) RGBA8 -> TGA (BGR(A), RLE packets of runs and literals, bottom-up unless top_down)."""
    h, w, _ = rgba.shape
    px = rgba[..., [2, 1, 0, 3][:channels]] if channels >= 3 else rgba[..., :1]
    if not top_down:
        px = px[::-1]
    flat = px.reshape(-1, px.shape[-1])
    bp = flat.shape[1]
    hdr = bytes([0, 0, (10 if rle else 2) if bp >= 3 else (11 if rle else 3), 0, 0, 0, 0, 0, 0, 0, 0, 0,
                 w & 255, w >> 8, h & 255, h >> 8, bp * 8, (0x20 if top_down else 0) | (8 if bp == 4 else 0)])
    if not rle:
        data = flat.tobytes()
    else:
        data, i, n = bytearray(), 0, len(flat)
        while i < n:
            j = i + 1
            while j < n and j - i < 128 and np.array_equal(flat[j], flat[i]):
                j += 1
            if j - i >= 2:
                data.append(0x80 | (j - i - 1))
                data += flat[i].tobytes()
                i = j
                continue
            j = i + 1
            while j < n and j - i < 128 and not (j + 1 < n and np.array_equal(flat[j], flat[j + 1])):
                j += 1
            data.append(j - i - 1)
            data += flat[i:j].tobytes()
            i = j
    open(path, "wb").write(hdr + bytes(data))
