"""Texture files -> device textures (mm_texture_load_file / mm_texture_load_slices) and a render
through them.  The files are written by the test (an independent encoder) in the layout of the
reference's Textures/ folder; the reference's own assets are not needed."""
import numpy as np
import pytest

from conftest import GOLDEN
from png import write_png, write_tga

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def asset_dir(tmp_path_factory, orc):
    # A miniature asset folder: 16-bit RGBA weather PNG, 8-bit RGB night sky and curl PNGs, RLE TGA
    # slices for the two density volumes (sizes smaller than the shipped ones).
    import os

    import marshmallow.lib as L
    d = tmp_path_factory.mktemp("Textures")
    rng = np.random.default_rng(5)
    arrays = {}
    w16 = (orc.noise(L.NOISE_WEATHER, 3, 256, 256, 1, 4)[0].astype(np.uint16) << 8) | rng.integers(0, 256, (256, 256, 4))
    write_png(d / "CloudPlacement.png", w16.astype(np.uint16), depth=16)
    arrays["weather"] = (w16 >> 8).astype(np.uint8)
    os.makedirs(d / "NightSky")
    night = rng.integers(0, 256, (90, 160, 3), dtype=np.uint8)
    write_png(d / "NightSky" / "nightSky_noOrange.png", night)
    arrays["night_sky"] = np.concatenate([night, np.full((90, 160, 1), 255, np.uint8)], axis=2)
    curl = np.fromfile(GOLDEN + "/curl_fbm_128.rgba", np.uint8).reshape(128, 128, 4)
    write_png(d / "CurlNoiseFBM.png", curl[..., :3])
    arrays["curl"] = curl
    os.makedirs(d / "3DTextures" / "lowResCloudShape")
    os.makedirs(d / "3DTextures" / "hiResCloudShape")
    lo = orc.noise(L.NOISE_LOWRES, 3, 32, 32, 32, 4)
    hi = orc.noise(L.NOISE_HIRES, 3, 16, 16, 16, 4)
    hi[..., 3] = 255
    for i in range(32):
        write_tga(d / "3DTextures" / "lowResCloudShape" / ("lowResCloud(%d).tga" % i), lo[i], rle=True)
    for i in range(16):
        write_tga(d / "3DTextures" / "hiResCloudShape" / ("hiResClouds (%d).tga" % i), hi[i], rle=bool(i % 2))
    arrays["low_res"], arrays["hi_res"] = lo, hi
    files = {"weather": ("file", "CloudPlacement.png"), "night_sky": ("file", "NightSky/nightSky_noOrange.png"),
             "curl": ("file", "CurlNoiseFBM.png"), "low_res": ("slices", "3DTextures/lowResCloudShape/lowResCloud", 32),
             "hi_res": ("slices", "3DTextures/hiResCloudShape/hiResClouds ", 16)}
    return str(d), files, arrays


def test_loaded_texels_equal_the_files(cuda, mmlib, asset_dir):
    import marshmallow as mm
    root, files, arrays = asset_dir
    t = mm.render.Textures.from_assets(root, files=files)
    try:
        for name, want in arrays.items():
            assert np.array_equal(t.host(name), want), name
    finally:
        t.close()


def test_render_through_loaded_textures_matches_oracle(cuda, mmlib, orc, asset_dir):
    # Exact arithmetic + software sampler over the file-loaded set == the FP32 oracle over the same
    # texels (a 4-channel curl map, as the reference's CurlNoiseFBM.png loads).
    import marshmallow as mm
    import marshmallow.lib as L
    from gpu_util import render
    root, files, arrays = asset_dir
    t = mm.render.Textures.from_assets(root, files=files)
    r = mm.render.Renderer()
    try:
        w, h = 192, 108
        u = mm.scene.uniforms(w, h, yaw=20.0, pitch=14.0)
        rgba, dep = render(cuda, r, u, t, w, h, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
        want, wd, _ = orc.march(u, arrays, w, h)
        assert np.array_equal(rgba.view(np.uint32), want.view(np.uint32))
        assert np.array_equal(dep.view(np.uint32), wd.view(np.uint32))
        # and the night branch reads the loaded night sky
        un = mm.scene.uniforms(w, h, yaw=20.0, pitch=14.0, sun_elevation=-8.0)
        rgba, _ = render(cuda, r, un, t, w, h, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
        want, _, _ = orc.march(un, arrays, w, h)
        assert np.array_equal(rgba.view(np.uint32), want.view(np.uint32))
    finally:
        r.close()
        t.close()


def test_load_errors(cuda, mmlib, asset_dir, tmp_path):
    import ctypes as C

    import marshmallow.lib as L
    root, _, _ = asset_dir
    h = C.c_void_p()
    assert mmlib.mm_texture_load_slices((root + "/3DTextures/lowResCloudShape/lowResCloud").encode(), 33, 0,
                                        C.byref(h), None) == L.MM_ERR_INVALID_ARGUMENT  # slice 32 is missing
    assert b"lowResCloud(32).tga" in mmlib.mm_last_error_string()
    assert mmlib.mm_texture_load_file(str(tmp_path / "none.png").encode(), 0, C.byref(h), None) == \
        L.MM_ERR_INVALID_ARGUMENT
