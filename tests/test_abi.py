"""The C-ABI library loads and exports every symbol include/mm.h declares; host-only entry
points behave (no device work here)."""
import ctypes as C
import math
import os
import re

import numpy as np

from conftest import GOLDEN, REPO


def declared_functions():
    src = open(os.path.join(REPO, "include", "mm.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(mm_[a-z_0-9]+)\s*\(", src, flags=re.M)))


def test_exports_every_declared_symbol(mmlib):
    import marshmallow.lib as L
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(mmlib, n), n
    assert set(names) == set(L.SIGNATURES), set(names) ^ set(L.SIGNATURES)


def test_uniform_block_layout():
    import marshmallow.lib as L
    # std140 sizes of compute-clouds.comp:12-41 (camera 160, cameraPrev 144, sun 116->128, sky 52->64)
    assert L.check_layout() == {"camera": 160, "camera_prev": 144, "sun": 128, "sky": 64, "uniforms": 496}
    assert L.Uniforms.sun.offset == 304 and L.SunUBO.intensity.offset == 112


def test_abi_version_and_errors(mmlib):
    import marshmallow.lib as L
    assert mmlib.mm_abi_version() == 1
    assert mmlib.mm_clouds_march(None, None, None, None, None, None) == L.MM_ERR_INVALID_ARGUMENT
    assert b"null" in mmlib.mm_last_error_string()
    n = C.c_size_t()
    assert mmlib.mm_noise_texel_bytes(C.byref(L.NoiseDesc(L.NOISE_LOWRES, 0, 0, 0, 0)), C.byref(n)) == 0
    assert n.value == 128 ** 3 * 4
    assert mmlib.mm_noise_texel_bytes(C.byref(L.NoiseDesc(L.NOISE_CURL2D, 0, 0, 0, 0)), C.byref(n)) == 0
    assert n.value == 128 * 128 * 2
    assert mmlib.mm_noise_texel_bytes(C.byref(L.NoiseDesc(9, 0, 0, 0, 0)), C.byref(n)) == L.MM_ERR_INVALID_ARGUMENT
    assert mmlib.mm_noise_texel_bytes(C.byref(L.NoiseDesc(L.NOISE_LOWRES, 0, 64, 32, 64)), C.byref(n)) == 1
    assert mmlib.mm_noise_texel_bytes(C.byref(L.NoiseDesc(L.NOISE_REF_CURL, 0, 64, 64, 1)), C.byref(n)) == 1
    o = L.MarchOptions()
    assert mmlib.mm_march_options_default(C.byref(o)) == 0 and o.sampler == L.SAMPLER_HARDWARE
    assert mmlib.mm_noise_fill(None, None, 0, None) == L.MM_ERR_INVALID_ARGUMENT
    assert mmlib.mm_texture_destroy(None) == L.MM_ERR_INVALID_ARGUMENT


def test_sky_matches_reference_skymanager(mmlib):
    import json
    import marshmallow.lib as L
    ref = json.load(open(os.path.join(GOLDEN, "sky_reference.json")))
    assert len(ref) >= 40
    for r in ref:
        u = L.Uniforms()
        assert mmlib.mm_sky_from_reference_fractions(r["elevation"], r["azimuth"], r["time"], 0, C.byref(u)) == 0
        np.testing.assert_allclose(list(u.sun.direction), r["direction"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(list(u.sun.location), r["location"], rtol=1e-5, atol=0.05)
        np.testing.assert_allclose(list(u.sun.direction_basis), r["direction_basis"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(list(u.sun.color)[:3], r["color_rgb"], rtol=1e-5)
        np.testing.assert_allclose(u.sun.intensity, r["intensity"][0], rtol=1e-5, atol=1e-4)
        np.testing.assert_allclose(list(u.sky.beta_r), r["beta_r"], rtol=1e-5)
        np.testing.assert_allclose(list(u.sky.wind), r["wind"], rtol=1e-6)
        np.testing.assert_allclose(u.sky.mie_directional, r["mie_directional"][0])


def test_camera_basis(mmlib):
    import marshmallow as mm
    u = mm.scene.uniforms(1920, 1080, yaw=30.0, pitch=15.0, fov=60.0)
    v = np.array(list(u.camera.view)).reshape(4, 4)  # v[col][row]
    right, up, fwd = v[:3, 0], v[:3, 1], v[:3, 2]
    for a in (right, up, fwd):
        assert abs(np.linalg.norm(a) - 1) < 1e-6
    assert abs(right @ up) < 1e-6 and abs(right @ fwd) < 1e-6
    # The image centre looks along -forward = (cos yaw cos pitch, sin pitch, sin yaw cos pitch).
    y, p = math.radians(30), math.radians(15)
    np.testing.assert_allclose(-fwd, [math.cos(y) * math.cos(p), math.sin(p), math.sin(y) * math.cos(p)], atol=1e-6)
    assert abs(u.camera.camera_params[0] - 1920 / 1080) < 1e-6
    assert abs(u.camera.camera_params[1] - math.tan(0.5 * 0.01745 * 60)) < 1e-6


def test_camera_matches_reference_camera(mmlib):
    # tests/golden/camera_reference.json: the reference's own Camera (camera.cpp compiled unchanged)
    # built as the application builds it (near 0.1, far 1000) and pointed by lookAt at (yaw, pitch);
    # its m_forward is the reverse of the direction the image centre looks at, so the same camera is
    # mm_camera_from_angles(eye, yaw + 180, -pitch).  View and projection agree to float rounding.
    import ctypes as C
    import json
    import os

    import numpy as np

    import marshmallow.lib as L
    from conftest import GOLDEN
    recs = json.load(open(os.path.join(GOLDEN, "camera_reference.json")))
    assert len(recs) == 24
    for rec in recs:
        u = L.Uniforms()
        e = (C.c_float * 3)(*rec["eye"])
        L.check(mmlib.mm_camera_from_angles(e, rec["yaw"] + 180.0, -rec["pitch"], rec["fov"], rec["width"],
                                            rec["height"], C.byref(u)))
        v, rv = np.array(u.camera.view[:]), np.array(rec["view"])
        p, rp = np.array(u.camera.proj[:]), np.array(rec["proj"])
        assert np.abs(v - rv).max() <= 1e-6 * max(1.0, np.abs(rv).max()), rec
        assert np.abs(p - rp).max() <= 1e-6 * np.abs(rp).max(), rec
        assert abs(u.camera.camera_params[0] - rec["aspect"][0]) <= 1e-7 * rec["aspect"][0]
        assert abs(u.camera.camera_params[1] - rec["tan_half_fov"][0]) <= 1e-7 * rec["tan_half_fov"][0]


def test_plain_c_host_builds_and_runs(tmp_path, mmlib):
    # The header compiles as C99 and a C host links libmm.so and calls the host-only entry points
    # (tests/c_host/abi_host.c); no device is needed for these.
    import shutil
    import subprocess
    from marshmallow import build as mb
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        import pytest
        pytest.skip("no C compiler")
    exe = str(tmp_path / "abi_host")
    lib_dir = os.path.dirname(mb.LIB)
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"),
                    os.path.join(REPO, "tests", "c_host", "abi_host.c"), "-L", lib_dir, "-l:libmm.so",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
