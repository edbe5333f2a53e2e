"""The texture unit's filter vs the oracle's restatement of it.

The march reads its density, weather and curl textures through texture objects (LINEAR, WRAP,
normalized coordinates: the reference's samplers, Texture.cpp:29-52, 315-338).  The oracle's
texture-unit sampler (oracle_glsl.h: 8-bit weights from round(256 (u N - 1/2)), integer corner
weights, 16-bit result) must return exactly what the hardware returns, so that the FP32 oracle run
with it is the hardware-filtered march the production kernels compute.  Fetches go through
mm_texture_sample on the library's own textures; every channel of every fetch must be identical.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import stream_ptr

pytestmark = pytest.mark.gpu

# Coordinate ranges of the march's fetches (compute-clouds.comp:218,223,236,238) with margin:
# weather 9 d.xz / |d| (|u| <= 9), curl 1e-4 pos.xz, low-res 2e-5 pos, hi-res 4e-4 pos for points
# within ~150 km of the camera.
RANGES = {"weather": 12.0, "curl": 16.0, "low_res": 4.0, "hi_res": 64.0}


def _coords(rng, dims, n, span, size):
    c = rng.uniform(-span, span, (n, dims)).astype(np.float32)
    # a fine sweep over two texels at the origin and at u = 1 (texel-boundary ties included)
    m = n // 4
    f = (np.arange(m) / m * 2.0).astype(np.float64)
    c[:m, 0] = ((np.arange(m) % 2) + f / size).astype(np.float32)
    return c


def _hw(cuda, lib, handle, coords):
    d_c = cuda.from_numpy(coords).cuda()
    out = cuda.empty((coords.shape[0], 4), dtype=cuda.float32, device="cuda")
    rc = lib.mm_texture_sample(handle, C.c_void_p(d_c.data_ptr()), coords.shape[0], C.c_void_p(out.data_ptr()),
                               stream_ptr(cuda))
    assert rc == 0, lib.mm_last_error_string()
    cuda.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("name", ["weather", "curl", "low_res", "hi_res"])
def test_texture_unit_equals_oracle_filter(cuda, mmlib, orc, name):
    import marshmallow as mm
    tex = mm.render.Textures(seed=0)
    try:
        host = tex.host(name)
        dims = 3 if host.ndim == 4 else 2
        size = host.shape[-2]
        coords = _coords(np.random.default_rng(7), dims, 1 << 18, RANGES[name], size)
        got = _hw(cuda, mmlib, tex.handles[name], coords)
        want = orc.sample(host, coords, filter=orc.FILTER_TEXTURE_UNIT)
        same = np.all(got.view(np.uint32) == want.view(np.uint32), axis=1)
        assert same.all(), (name, int((~same).sum()), coords[~same][:4], got[~same][:4], want[~same][:4])
        # the exact-weight filter is a different function: most fetches differ from the hardware
        exact = orc.sample(host, coords, filter=orc.FILTER_EXACT)
        print("%s: %d fetches identical; exact-weight filter differs on %.1f%% of them"
              % (name, len(coords), 100.0 * np.mean(np.any(exact != got, axis=1))))
    finally:
        tex.close()


@pytest.mark.parametrize("shape", [(64, 128, 4), (128, 32, 2), (37, 53, 4), (60, 100, 1), (16, 16, 16, 4),
                                   (8, 64, 32, 4), (28, 20, 24, 4)])
def test_texture_unit_equals_oracle_filter_random_texels(cuda, mmlib, orc, shape):
    # Random bytes in textures of other shapes (sides that are not powers of two included) and
    # channel counts.
    import marshmallow as mm
    rng = np.random.default_rng(11)
    texels = rng.integers(0, 256, shape, dtype=np.uint8)
    tex = mm.render.Textures.from_arrays({"t": texels})
    try:
        dims = 3 if texels.ndim == 4 else 2
        coords = _coords(rng, dims, 1 << 16, 8.0, shape[-2])
        got = _hw(cuda, mmlib, tex.handles["t"], coords)
        want = orc.sample(texels, coords, filter=orc.FILTER_TEXTURE_UNIT)
        same = np.all(got.view(np.uint32) == want.view(np.uint32), axis=1)
        assert same.all(), (shape, int((~same).sum()), coords[~same][:4], got[~same][:4], want[~same][:4])
    finally:
        tex.close()
