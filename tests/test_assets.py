"""The shipped-asset loader (Texture::initFromFile with stbi_load(..., STBI_rgb_alpha)) on the CPU:
files written by an independent encoder (tests/png.py: Python's zlib) decode to the expected RGBA8."""
import ctypes as C
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from png import read_png, write_png, write_tga
from tga import read_tga


def _decode(mmlib, path):
    import marshmallow.lib as L
    p, w, h = C.c_void_p(), C.c_int(), C.c_int()
    rc = mmlib.mm_image_decode_file(str(path).encode(), C.byref(p), C.byref(w), C.byref(h))
    if rc:
        return rc, None
    a = np.ctypeslib.as_array(C.cast(p, C.POINTER(C.c_uint8)), (h.value, w.value, 4)).copy()
    mmlib.mm_image_free(p)
    assert rc == L.MM_OK
    return rc, a


def _rgba8(samples, depth):
    s = samples >> 8 if depth == 16 else samples
    s = s.astype(np.uint8)
    h, w, c = s.shape
    out = np.full((h, w, 4), 255, np.uint8)
    if c <= 2:
        out[..., :3] = s[..., :1]
        if c == 2:
            out[..., 3] = s[..., 1]
    else:
        out[..., :c] = s
    return out


def _image(rng, h, w, c, depth):
    hi = 65536 if depth == 16 else 256
    noise = rng.integers(0, hi, (h, w, c))
    yy, xx = np.mgrid[0:h, 0:w]
    smooth = ((xx * 7 + yy * 3)[..., None] * (hi // 256)) % hi  # long matches for the LZ77 stage
    img = np.where((yy // 4 % 2 == 0)[..., None], smooth, noise)
    return img.astype(np.uint16 if depth == 16 else np.uint8)


@pytest.mark.parametrize("channels", [1, 2, 3, 4])
@pytest.mark.parametrize("depth", [8, 16])
@pytest.mark.parametrize("level", [0, 1, 9])
def test_png_decode(mmlib, tmp_path, channels, depth, level):
    rng = np.random.default_rng(channels * 100 + depth + level)
    img = _image(rng, 23, 37, channels, depth)
    f = tmp_path / "a.png"
    write_png(f, img, depth=depth, level=level)
    assert np.array_equal(read_png(f), img)  # the independent reader agrees with the writer
    rc, got = _decode(mmlib, f)
    assert rc == 0 and np.array_equal(got, _rgba8(img, depth))


def test_png_transparency_key(mmlib, tmp_path):
    img = np.zeros((4, 5, 3), np.uint8)
    img[1, 2] = (10, 20, 30)
    f = tmp_path / "k.png"
    write_png(f, img, trns=(10, 20, 30))
    rc, got = _decode(mmlib, f)
    assert rc == 0 and got[1, 2, 3] == 0 and (got[..., 3] == 0).sum() == 1


@pytest.mark.parametrize("rle", [False, True])
@pytest.mark.parametrize("top_down", [False, True])
@pytest.mark.parametrize("channels", [1, 3, 4])
def test_tga_decode(mmlib, tmp_path, rle, top_down, channels):
    rng = np.random.default_rng(channels + 2 * rle + 4 * top_down)
    rgba = _image(rng, 19, 29, 4, 8)
    if channels == 1:
        rgba[..., 1] = rgba[..., 2] = rgba[..., 0]
    if channels != 4:
        rgba[..., 3] = 255
    f = tmp_path / "a.tga"
    write_tga(f, rgba, rle=rle, top_down=top_down, channels=channels)
    rc, got = _decode(mmlib, f)
    assert rc == 0 and np.array_equal(got, rgba)
    ref = read_tga(str(f))
    assert np.array_equal(got[..., :ref.shape[2]], ref if channels != 1 else np.repeat(ref, 1, axis=2))


def test_golden_curl_through_tga(mmlib, tmp_path):
    # The reference's CurlNoiseFBM texture (a golden fixture) survives RLE TGA encode -> decode.
    g = np.fromfile(os.path.join(GOLDEN, "curl_fbm_128.rgba"), np.uint8).reshape(128, 128, 4)
    f = tmp_path / "curl.tga"
    write_tga(f, g, rle=True)
    rc, got = _decode(mmlib, f)
    assert rc == 0 and np.array_equal(got, g)


def test_decode_errors(mmlib, tmp_path):
    import marshmallow.lib as L
    img = np.arange(60, dtype=np.uint8).reshape(4, 5, 3)
    f = tmp_path / "a.png"
    write_png(f, img)
    b = bytearray(open(f, "rb").read())
    (tmp_path / "trunc.png").write_bytes(bytes(b[:-30]))
    assert _decode(mmlib, tmp_path / "trunc.png")[0] == L.MM_ERR_INVALID_ARGUMENT
    b2 = bytearray(b)
    b2[40] ^= 0xFF  # inside a chunk: CRC mismatch
    (tmp_path / "crc.png").write_bytes(bytes(b2))
    assert _decode(mmlib, tmp_path / "crc.png")[0] == L.MM_ERR_INVALID_ARGUMENT
    tga16 = bytes([0, 0, 2, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 0, 2, 0, 16, 0]) + bytes(8)
    (tmp_path / "a16.tga").write_bytes(tga16)
    assert _decode(mmlib, tmp_path / "a16.tga")[0] == L.MM_ERR_UNSUPPORTED
    assert _decode(mmlib, tmp_path / "missing.png")[0] == L.MM_ERR_INVALID_ARGUMENT


def test_shipped_assets_digests(mmlib):
    # With MM_ASSET_DIR pointing at the reference's Textures/ folder, the decoder reproduces the
    # digests recorded from independent decoders (tests/golden/make_golden.py).
    root = os.environ.get("MM_ASSET_DIR")
    if not root:
        pytest.skip("MM_ASSET_DIR not set")
    digests = json.load(open(os.path.join(GOLDEN, "asset_digests.json")))
    for name, want in digests.items():
        rc, a = _decode(mmlib, os.path.join(root, name))
        assert rc == 0 and hashlib.sha256(a.tobytes()).hexdigest() == want, name
