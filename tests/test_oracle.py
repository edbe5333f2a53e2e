"""The CPU oracle pinned against the reference: golden vectors from the reference's own code
(compiled here by oracle/Makefile `ref`) and the shipped curl texture."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_ref_curl_matches_shipped_texture(orc):
    # ImageUtils.cpp GenerateCurlNoise == Textures/CurlNoiseFBM.tga, 0 LSB.
    golden = np.fromfile(os.path.join(GOLDEN, "curl_fbm_128.rgba"), np.uint8).reshape(128, 128, 4)
    assert np.array_equal(orc.ref_curl(), golden)


def test_ref_hash_matches_reference_build(orc):
    # hashNoise scales sinf by 43758.5453 before taking the fraction, so it inherits the last-bit
    # behaviour of the platform's sinf.  The oracle (and the GPU) use a correctly rounded sinf; the
    # reference build here uses glibc's, which is off by one ulp for ~1.5% of arguments.  Those
    # hashes then differ by one quantum of the scaled sine (2^-9 here), never in the gradient index
    # on these points, and the full texture still matches the shipped one (test above).
    lib = orc.load()
    rows = [l.split() for l in open(os.path.join(GOLDEN, "ref_hash.txt")) if not l.startswith("#")]
    assert len(rows) > 400
    differ = 0
    for x, y, z, h in rows:
        got = np.float32(lib.oracle_ref_curl_hash(float(x), float(y), float(z)))
        want = np.float32(float(h))
        assert int(12 * got) == int(12 * want)
        assert abs(float(got) - float(want)) <= 2.0 ** -8
        differ += got != want
    assert differ <= 0.03 * len(rows)


@pytest.mark.parametrize("fn,lo,hi,ref,tol_ulp", [
    (0, -80.0, 80.0, np.exp, 2), (1, -120.0, 120.0, np.exp2, 2), (4, -1.0, 1.0, np.arccos, 2),
    (5, -6.3, 6.3, np.cos, 2), (6, -6.3, 6.3, np.sin, 2), (7, -4000.0, 4000.0, np.sin, 0.5)])
def test_elementary_functions(orc, fn, lo, hi, ref, tol_ulp):
    lib = orc.load()
    xs = np.random.default_rng(fn).uniform(lo, hi, 20000).astype(np.float32)
    got = np.array([lib.oracle_mm_math(fn, float(x), 0.0) for x in xs], np.float32)
    want = ref(xs.astype(np.float64))
    ulp = np.abs(got.astype(np.float64) - want) / np.spacing(np.abs(want).astype(np.float32)).astype(np.float64)
    mask = np.abs(want) > 1e-6  # ulp is ill-defined at zeros of sin/cos
    assert ulp[mask].max() <= tol_ulp + 1e-9


def test_log2_and_pow(orc):
    lib = orc.load()
    rng = np.random.default_rng(3)
    xs = np.exp2(rng.uniform(-100, 100, 5000)).astype(np.float32)
    got = np.array([lib.oracle_mm_math(2, float(x), 0.0) for x in xs], np.float64)
    want = np.log2(xs.astype(np.float64))
    tol = np.maximum(3e-7, 1.5 * np.spacing(np.abs(want).astype(np.float32)))
    assert np.all(np.abs(got - want) <= tol)
    b = rng.uniform(0, 1000, 5000).astype(np.float32)
    e = rng.uniform(-2, 2, 5000).astype(np.float32)
    got = np.array([lib.oracle_mm_math(3, float(x), float(y)) for x, y in zip(b, e)], np.float64)
    want = np.power(b.astype(np.float64), e.astype(np.float64))
    assert np.max(np.abs(got - want) / want) < 3e-6
    assert lib.oracle_mm_math(3, 0.0, 0.8) == 0.0


def test_noise_generators_statistics(orc):
    # The seeded generators have the first two moments of the shipped Nubis textures.
    import marshmallow.lib as L
    stats = json.load(open(os.path.join(GOLDEN, "nubis_stats.json")))
    lo = orc.noise(L.NOISE_LOWRES, 0, 64, 64, 64, 4).reshape(-1, 4) / 255.0
    hi = orc.noise(L.NOISE_HIRES, 0, 32, 32, 32, 4).reshape(-1, 4) / 255.0
    assert np.allclose(lo.mean(0), stats["low_res"]["mean"], atol=0.03)
    assert np.allclose(lo.std(0), stats["low_res"]["std"], atol=0.03)
    assert np.allclose(hi.mean(0)[:3], stats["hi_res"]["mean"][:3], atol=0.03)
    assert np.all(hi[:, 3] == 0)


def test_noise_tileable_and_seeded(orc):
    import marshmallow.lib as L
    a = orc.noise(L.NOISE_WEATHER, 0, 64, 64, 1, 4)
    b = orc.noise(L.NOISE_WEATHER, 1, 64, 64, 1, 4)
    assert not np.array_equal(a, b)
    assert np.all(a[..., 1] == 0) and np.all(a[..., 3] == 255)
    # Tileable: wrapping the lattice makes opposite edges continuous (small differences).
    lo = orc.noise(L.NOISE_HIRES, 0, 32, 32, 32, 4).astype(int)
    edge = np.abs(lo[:, :, 0, :3] - lo[:, :, -1, :3]).mean()
    inner = np.abs(lo[:, :, 15, :3] - lo[:, :, 16, :3]).mean()
    assert edge < 3 * inner + 2


def test_hash_known_values(orc):
    lib = orc.load()
    # lowbias32 known values (its published reference outputs)
    assert lib.oracle_hash32(0) == 0
    assert lib.oracle_hash3(0, 0, 0, 0) == lib.oracle_hash32(lib.oracle_hash32(lib.oracle_hash32(0)))


def _small_scene(orc, size=64):
    import marshmallow as mm
    u = mm.scene.uniforms(size, size)
    import marshmallow.lib as L
    tex = {"low_res": orc.noise(L.NOISE_LOWRES, 0, 32, 32, 32, 4), "hi_res": orc.noise(L.NOISE_HIRES, 0, 16, 16, 16, 4),
           "curl": orc.noise(L.NOISE_CURL2D, 0, 64, 64, 1, 2)[0], "weather": orc.noise(L.NOISE_WEATHER, 0, 128, 128, 1, 4)[0]}
    return u, tex


def test_oracle_f32_vs_f64_within_gates(orc):
    import marshmallow as mm
    u, tex = _small_scene(orc, 96)
    a, da, ca = orc.march(u, tex, 96, 96, precision=32)
    b, db, cb = orc.march(u, tex, 96, 96, precision=64)
    e = mm.metrics.frame_errors(a, b, da, db)
    assert e["nan"] == 0
    assert e["rmse_255"] <= 1.0 and e["max_255"] <= 4.0
    assert e["depth_rel_p999"] <= 1e-3
    assert abs(int(ca[0]) - int(cb[0])) <= 0.01 * cb[0]


def test_oracle_phase16_and_sampling(orc):
    u, tex = _small_scene(orc, 64)
    full, dfull, _ = orc.march(u, tex, 64, 64)
    for phase in (0, 5, 15):
        u.sun.color[3] = float(phase)
        part, dpart, _ = orc.march(u, tex, 64, 64, pixel_mode=1)
        m = np.zeros((64, 64), bool)
        m[phase // 4::4, phase % 4::4] = True
        assert np.array_equal(part[m], full[m]) and np.all(part[~m] == 0)
    u.sun.color[3] = 0.0
    sub, _, _ = orc.march(u, tex, 64, 64, rows=(3, 64, 5), col_begin=2, col_step=3)
    assert np.array_equal(sub, full[3::5, 2::3])


def test_oracle_horizon_rays_and_night(orc):
    import marshmallow as mm
    u, tex = _small_scene(orc, 48)
    # Looking down: every ray is killed at :351-354, depth +inf, colour = background.
    u2 = mm.scene.uniforms(48, 48, pitch=-60.0)
    rgba, depth, cnt = orc.march(u2, tex, 48, 48)
    assert np.all(np.isinf(depth)) and cnt[0] == 0
    # Sun below the horizon needs the night-sky texture; with it the night branch runs.
    un = mm.scene.uniforms(48, 48, sun_elevation=-10.0)
    with pytest.raises(RuntimeError):
        orc.march(un, tex, 48, 48)
    night = np.random.default_rng(0).integers(0, 256, (64, 96, 4), dtype=np.uint8)
    tex["night_sky"] = night
    rgba, depth, _ = orc.march(un, tex, 48, 48)
    assert np.all(np.isfinite(rgba))


def test_reprojection_static_camera_is_identity(orc):
    # reproject.comp with camera == cameraPrev maps every pixel onto itself: the ten taps collapse
    # onto the pixel, so the result is the source up to the rounding of the ten-tap average.
    import marshmallow as mm
    u = mm.scene.uniforms(96, 64, yaw=30.0, pitch=12.0)
    rng = np.random.default_rng(4)
    src = rng.uniform(0, 5, (64, 96, 4)).astype(np.float32)
    dep = rng.uniform(1e3, 1e5, (64, 96)).astype(np.float32)
    out, od = orc.reproject(u, src, dep)
    assert np.allclose(out, src, rtol=2e-7, atol=0)
    assert np.array_equal(out[..., 3], src[..., 3]) and np.array_equal(od, dep)


def test_reprojection_follows_camera_motion(orc):
    # Turning the camera right by a few degrees moves the previous image left in the new frame.
    import marshmallow as mm
    prev = mm.scene.uniforms(128, 64, yaw=20.0, pitch=15.0)
    cur = mm.scene.uniforms(128, 64, yaw=23.0, pitch=15.0)
    cur.camera_prev = prev.camera_prev
    src = np.zeros((64, 128, 4), np.float32)
    src[:, 60:68, :] = 1.0  # a bright vertical band at x = 60..67 in the previous frame
    out, _ = orc.reproject(cur, src)
    cols = np.where(out[32, :, 3] > 0.5)[0]
    assert len(cols) > 0 and abs(cols.mean() - 63.5) > 2.0


def _shadow_scene(orc, w=160, h=90, **kw):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(w, h, eye=(0.0, 150.0, 0.0), pitch=-20.0, **kw)
    g = mm.scene.terrain_gbuffer(u, w, h)
    tex = {"low_res": orc.noise(L.NOISE_LOWRES, 0, 64, 64, 64, 4), "weather": orc.noise(L.NOISE_WEATHER, 0, 256, 256, 1, 4)[0]}
    return u, g, tex


def test_shadow_f32_vs_f64_and_uncovered_pixels(orc):
    # model.frag's shadow march: FP32 within 1e-4 of FP64 (a max of six densities, no accumulation);
    # pixels without a mesh fragment get 0.
    u, g, tex = _shadow_scene(orc, sun_elevation=45.0, time=5.0)
    a = orc.shadow(u, tex, g)
    b = orc.shadow(u, tex, g, precision=64)
    cov = g[..., 3] != 0
    assert 0.3 < cov.mean() < 1.0
    assert np.all(a[~cov] == 0) and (a[cov] > 0).mean() > 0.2
    assert np.all((a >= 0) & (a <= 1))
    assert np.percentile(np.abs(a - b), 99.9) <= 1e-4
    # multithreaded == single-threaded
    assert np.array_equal(orc.shadow(u, tex, g, nthreads=1), a)


def test_shadow_saturates_and_vanishes(orc):
    # Empty low-res noise: no density anywhere.  Dense noise with a stratocumulus weather map: on
    # almost every fragment a sample lands inside the layer and saturates the shadow to exactly 1
    # (:266-269).
    u, g, tex = _shadow_scene(orc, sun_elevation=60.0)
    empty = dict(tex, low_res=np.zeros_like(tex["low_res"]))
    assert np.all(orc.shadow(u, empty, g) == 0)
    dense = np.full_like(tex["low_res"], 255)
    dense[..., 1:] = 0
    weather = np.zeros_like(tex["weather"])
    weather[..., 2] = 128
    s = orc.shadow(u, {"low_res": dense, "weather": weather}, g)
    cov = g[..., 3] != 0
    assert np.all((s >= 0) & (s <= 1)) and (s[cov] == 1.0).mean() > 0.9 and np.all(s[~cov] == 0)


def test_post_chain_known_answers(orc):
    # Uniform alpha a: each god-ray tap reads a, so the term is 0.9 * 0.5 a (1 + 0.125 sum 0.99^i)
    # (god-ray.frag:56-75); the radial blur of a uniform term t is 1.1 t (radialBlur.frag:57-60).
    import marshmallow as mm
    u = mm.scene.uniforms(96, 64, yaw=0.0, pitch=15.0, sun_elevation=20.0)
    img = np.zeros((64, 96, 4), np.float32)
    img[..., :3] = np.random.default_rng(1).uniform(0, 1, (64, 96, 3))
    img[..., 3] = 0.25
    g = orc.post_pass("god_rays", u, img)
    want = 0.9 * 0.5 * 0.25 * (1 + 0.125 * sum(0.99 ** i for i in range(8)))
    assert np.allclose(g[..., 3], want, rtol=1e-6) and np.array_equal(g[..., :3], img[..., :3])
    r = orc.post_pass("radial_blur", u, g)
    k = np.array(u.sun.color[:3], np.float64) * u.sun.intensity
    assert np.allclose(r[..., :3], k * 1.1 * want + 0.5 * img[..., :3], rtol=1e-5)
    assert np.all(r[..., 3] == 1.0)
    # The chain is the passes in sequence; a mesh layer replaces the blurred sky where its a != 0.
    mesh = np.zeros_like(img)
    mesh[40:, :, :3] = 0.3
    mesh[40:, :, 3] = 1.0
    out = orc.post_chain(u, img, mesh)
    fb2 = r.copy()
    fb2[40:] = mesh[40:]
    assert np.array_equal(out, orc.post_tonemap(fb2))
    # tonemap: B,G,R,A byte order by default is a channel swap of R,G,B,A; alpha 255.
    t_rgba, t_bgra = orc.post_tonemap(fb2, bgra=0), orc.post_tonemap(fb2, bgra=1)
    assert np.array_equal(t_rgba[..., [2, 1, 0, 3]], t_bgra) and np.all(t_rgba[..., 3] == 255)
    # At the image centre the vignette vanishes: the 8-bit tonemap equals the FP64 metric tonemap.
    c = orc.tonemap(fb2[31:33, 47:49])
    assert np.max(np.abs(t_rgba[31:33, 47:49, :3].astype(int) - np.round(np.clip(c, 0, 1) * 255))) <= 1


def test_post_chain_night_skips_the_sun_passes(orc):
    # Sun below the horizon: both passes copy the colour (god-ray.frag:52-54, radialBlur.frag:41-43).
    import marshmallow as mm
    u = mm.scene.uniforms(64, 48, sun_elevation=-10.0)
    img = np.random.default_rng(2).uniform(0, 3, (48, 64, 4)).astype(np.float32)
    assert np.array_equal(orc.post_chain(u, img), orc.post_tonemap(img))


# ------------------------------------------------------------------------------------------------
# The restatement against the reference shader itself: compute-clouds.comp compiled unchanged as
# C++ on the CPU (oracle/Makefile `ref`, oracle/ref/glsl_to_cpp.py + glsl_shim.h).  Both evaluate
# the same float expressions in the same order under the same sampler definition, so they agree to
# the last few ulps of the elementary functions (libm's here, mm_math.h's in the restatement) and
# take the same branch at every march threshold on these frames.

def _shader_textures(orc, oracle_textures, u):
    import shader_golden
    return dict(oracle_textures, night_sky=shader_golden.night_sky(orc) if u.sun.direction[1] < 0 else None)


def test_oracle_matches_reference_shader_golden(orc, oracle_textures):
    import marshmallow as mm
    import shader_golden as sg
    frames = sg.frames()
    assert len(frames) == 5
    for name, u, rows, cols, ref in frames:
        t = _shader_textures(orc, oracle_textures, u)
        o32 = sg.oracle_march(orc, u, t, rows, cols, 32)
        assert sg.max_rel(o32, ref) <= 2e-4, name
        o64 = sg.oracle_march(orc, u, t, rows, cols, 64)
        e = mm.metrics.frame_errors(o64, ref)
        assert e["nan"] == 0 and e["rmse_255"] <= 1.0 and e["p999_255"] <= 4.0 and e["frac_over_4"] <= 0.002, (name, e)


def test_oracle_equals_reference_shader_with_the_same_elementary_functions(orc, oracle_textures):
    # Built with mm_math.h's exp/pow/acos/cos/sin (the restatement's), the reference shader and the
    # FP32 restatement agree bit for bit on every pixel of five frames: sky, clouds, night
    # (tests/golden/shader_clouds_mm.json).  Every operation and its order is the shader's.
    import shader_golden as sg
    frames = sg.mm_frames()
    assert len(frames) == 5
    for name, u, rows, cols, sha in frames:
        got = sg.oracle_march(orc, u, _shader_textures(orc, oracle_textures, u), rows, cols, 32)
        assert sg.digest(np.ascontiguousarray(got, np.float32)) == sha, name
        if orc.ref_clouds_mm_available():
            ys, xs = np.meshgrid(rows, cols, indexing="ij")
            ref = orc.ref_clouds_march(u, _shader_textures(orc, oracle_textures, u), xs.ravel(), ys.ravel(),
                                       mm_math=True).reshape(got.shape)
            assert np.array_equal(ref.view(np.uint32), got.view(np.uint32)), name


def test_reference_shader_build_reproduces_golden(orc, oracle_textures):
    # Where the reference shader has been compiled (`make -C oracle ref`), it reproduces the fixture.
    import shader_golden as sg
    if not orc.ref_clouds_available():
        pytest.skip("reference shader not compiled here")
    for name, u, rows, cols, ref in sg.frames():
        ys, xs = np.meshgrid(rows, cols, indexing="ij")
        got = orc.ref_clouds_march(u, _shader_textures(orc, oracle_textures, u), xs.ravel(), ys.ravel())
        assert sg.max_rel(got.reshape(ref.shape), ref) <= 1e-6, name


def test_reference_shader_rejects_pixels_outside_the_phase(orc, oracle_textures):
    import marshmallow as mm
    if not orc.ref_clouds_available():
        pytest.skip("reference shader not compiled here")
    u = mm.scene.uniforms(1920, 1080, phase=6)
    with pytest.raises(RuntimeError):
        orc.ref_clouds_march(u, oracle_textures, np.array([2, 3]), np.array([1, 1]))
    with pytest.raises(RuntimeError):
        orc.ref_clouds_march(u, oracle_textures, np.array([1922]), np.array([1]))


def test_oracle_matches_reference_shader_on_shipped_textures(orc, mmlib):
    # The shipped Nubis textures (MM_ASSET_DIR = the reference's Textures/ folder), several poses.
    import marshmallow as mm
    import shader_golden as sg
    from test_assets import _decode
    root = os.environ.get("MM_ASSET_DIR")
    if not root or not orc.ref_clouds_available():
        pytest.skip("needs MM_ASSET_DIR and the compiled reference shader")

    def image(name):
        rc, a = _decode(mmlib, os.path.join(root, name))
        assert rc == 0, name
        return a

    t = {"weather": image("CloudPlacement.png"), "night_sky": image("NightSky/nightSky_noOrange.png"),
         "curl": image("CurlNoiseFBM.png"),
         "low_res": np.stack([image("3DTextures/lowResCloudShape/lowResCloud(%d).tga" % i) for i in range(128)]),
         "hi_res": np.stack([image("3DTextures/hiResCloudShape/hiResClouds (%d).tga" % i) for i in range(32)])}
    poses = [dict(yaw=0.0, pitch=15.0, sun_elevation=30.0, phase=0),
             dict(yaw=75.0, pitch=3.0, sun_elevation=8.0, time=120.0, phase=9),
             dict(yaw=210.0, pitch=30.0, sun_elevation=55.0, time=600.0, phase=14),
             dict(yaw=330.0, pitch=6.0, sun_elevation=-15.0, phase=7)]
    for pose in poses:
        u = mm.scene.uniforms(1920, 1080, **pose)
        p = pose["phase"]
        rows, cols = np.arange(p // 4, 1080, 16), np.arange(p % 4, 1920, 16)
        ys, xs = np.meshgrid(rows, cols, indexing="ij")
        ref = orc.ref_clouds_march(u, t, xs.ravel(), ys.ravel()).reshape(len(rows), len(cols), 4)
        o32 = sg.oracle_march(orc, u, t, rows, cols, 32)
        assert sg.max_rel(o32, ref) <= 2e-4, pose
        if orc.ref_clouds_mm_available():
            ref_mm = orc.ref_clouds_march(u, t, xs.ravel(), ys.ravel(), mm_math=True).reshape(o32.shape)
            assert np.array_equal(ref_mm.view(np.uint32), o32.view(np.uint32)), pose


# The other passes against their shaders compiled the same way.  Reprojection is bit-identical (the
# restatement sums cameraPrev.view * p in glm's pairwise order, one of the orders GLSL allows).  The
# post passes differ only where the shader samples texColor at its own fragUV: the restatement takes
# the texel (the filter's weights are zero at a texel centre on the GPU's fixed-point filter), the
# shim's float-weight sampler lands ~1e-5 of a texel off the centre and mixes in that much of the
# neighbour.  The shadow is recovered from the shaded colour (see oracle.ref_model_shadow).

def _post_bound(src, channels):
    """Error bound of the centre fetch: 3e-5 of the largest input value of each channel."""
    return 3e-5 * np.abs(src[..., channels]).reshape(-1, len(channels)).max(0) + 1e-7


def test_reprojection_matches_reference_shader_golden(orc):
    import shader_golden as sg
    import marshmallow.lib as L
    z = sg.passes()
    for k, (case, ub, want) in enumerate(zip(sg.REPROJECT_CASES, z["reproject_uniforms"], z["reproject_digests"])):
        u = L.Uniforms.from_buffer_copy(ub.tobytes())
        got, _ = orc.reproject(u, sg.pattern(case[1], case[0], k))
        assert sg.digest(got) == str(want), case


def test_post_passes_match_reference_shader_golden(orc):
    import shader_golden as sg
    import marshmallow.lib as L
    z = sg.passes()
    u = L.Uniforms.from_buffer_copy(z["post_uniforms"].tobytes())
    w, h = sg.POST_SIZE
    src = sg.pattern(h, w, 11)
    g = orc.post_pass("god_rays", u, src)
    assert np.array_equal(g[..., :3], src[..., :3])
    assert np.all(np.abs(g[..., 3] - z["god_ray_alpha"]) <= _post_bound(src, [3]))
    assert z["god_ray_alpha"].max() > 0.3  # the sun is in view
    b = orc.post_pass("radial_blur", u, g)
    assert np.all(np.abs(b[..., :3] - z["radial_blur_rgb"]) <= 0.5 * _post_bound(g, [0, 1, 2]))
    t = orc.post_tonemap(src)[..., :3].astype(int)
    d = np.abs(t - z["tonemap_rgb"].astype(int))
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3


def test_shadow_matches_reference_shader_golden(orc, oracle_textures):
    import shader_golden as sg
    import marshmallow.lib as L
    z = sg.passes()
    u = L.Uniforms.from_buffer_copy(z["shadow_uniforms"].tobytes())
    got = orc.shadow(u, oracle_textures, z["shadow_world_pos"])
    want = z["shadow"]
    fin = np.isfinite(want)
    assert (want[fin] > 0).mean() > 0.2  # the G-buffer has cloud shadow to check
    assert np.abs(got[fin] - want[fin]).max() <= 1e-6
    assert np.all(got[~fin] >= 0.5 - 1e-6)


def _need(available):
    if not available:
        pytest.skip("reference shader not compiled here")


@pytest.mark.parametrize("k", range(3))
def test_reprojection_equals_reference_shader_build(orc, k):
    import shader_golden as sg
    import marshmallow as mm
    _need(orc.ref_reproject_available())
    case = sg.REPROJECT_CASES[k]
    u = sg.reproject_uniforms(case)
    src = sg.pattern(case[1], case[0], k)
    want = orc.ref_reproject(u, src)
    got, _ = orc.reproject(u, src)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    # and a sweep of camera motions between consecutive frames
    for frame in (1, 6, 13):
        cur = mm.scene.sweep_uniforms(frame, 400, 224)
        prev = mm.scene.sweep_uniforms(frame - 1, 400, 224)
        cur.camera_prev = prev.camera_prev  # the previous frame's camera (set with it)
        src = sg.pattern(224, 400, 100 + frame)
        assert np.array_equal(orc.reproject(cur, src)[0], orc.ref_reproject(cur, src)), frame


@pytest.mark.parametrize("elev,yaw", [(20.0, 0.0), (8.0, 25.0), (45.0, -30.0), (-6.0, 0.0)])
def test_post_passes_match_reference_shader_build(orc, elev, yaw):
    import shader_golden as sg
    import marshmallow as mm
    _need(orc.ref_post_available("god_ray") and orc.ref_post_available("radial_blur")
          and orc.ref_post_available("tonemap"))
    w, h = 320, 180
    u = mm.scene.uniforms(w, h, yaw=yaw, pitch=12.0, sun_elevation=elev)
    src = sg.pattern(h, w, 21)
    g = orc.post_pass("god_rays", u, src)
    rg = orc.ref_post("god_ray", u, src)
    assert np.all(np.abs(g - rg) <= _post_bound(src, [0, 1, 2, 3]))
    b = orc.post_pass("radial_blur", u, g)
    rb = orc.ref_post("radial_blur", u, g)
    assert np.all(np.abs(b - rb) <= 0.5 * _post_bound(g, [0, 1, 2, 3]) + 1e-6 * np.abs(rb))
    t = orc.post_tonemap(src).astype(int)
    rt = orc.unorm8(orc.ref_post("tonemap", None, src)).astype(int)
    d = np.abs(t[..., :3] - rt[..., :3])
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3


@pytest.mark.parametrize("elev,time,yaw", [(30.0, 0.0, 0.0), (15.0, 300.0, 60.0), (60.0, 40.0, 0.0)])
def test_shadow_matches_reference_shader_build(orc, elev, time, yaw):
    import marshmallow as mm
    import marshmallow.lib as L
    _need(orc.ref_model_available())
    w, h = 160, 90
    u = mm.scene.uniforms(w, h, eye=(0.0, 150.0, 0.0), yaw=yaw, pitch=-20.0, sun_elevation=elev, time=time)
    g = mm.scene.terrain_gbuffer(u, w, h)
    tex = {"low_res": orc.noise(L.NOISE_LOWRES, 0, 64, 64, 64, 4),
           "weather": orc.noise(L.NOISE_WEATHER, 0, 256, 256, 1, 4)[0]}
    wp = g.reshape(-1, 4)
    wp = wp[wp[:, 3] != 0]
    got = orc.shadow(u, tex, wp)
    want = orc.ref_model_shadow(u, tex, wp)
    fin = np.isfinite(want)
    assert (got > 0).mean() > 0.2
    assert np.abs(got[fin] - want[fin]).max() <= 1e-6
    assert np.all(got[~fin] >= 0.5 - 1e-6)


def test_oracle_uniforms_match_reference_camera_and_sky(orc):
    # The oracle's own camera/sky set-up (used by the benchmark's reference arm, which must not load
    # the CUDA library) against the reference's Camera and SkyManager compiled unchanged
    # (tests/golden/camera_reference.json, sky_reference.json).
    import math
    recs = json.load(open(os.path.join(GOLDEN, "camera_reference.json")))
    for rec in recs:
        # the reference camera looks along -m_forward: the same camera is (yaw + 180, -pitch) here
        u = np.frombuffer(orc.uniforms(rec["width"], rec["height"], eye=rec["eye"], yaw=rec["yaw"] + 180.0,
                                       pitch=-rec["pitch"], fov=rec["fov"]), np.float32)
        v, rv = u[0:16].astype(np.float64), np.array(rec["view"])
        p, rp = u[16:32].astype(np.float64), np.array(rec["proj"])
        assert np.abs(v - rv).max() <= 1e-6 * max(1.0, np.abs(rv).max()), rec
        assert np.abs(p - rp).max() <= 1e-6 * np.abs(rp).max(), rec
        assert abs(u[36] - rec["aspect"][0]) <= 1e-7 * rec["aspect"][0]
        assert abs(u[37] - rec["tan_half_fov"][0]) <= 1e-7 * rec["tan_half_fov"][0]
    sky = json.load(open(os.path.join(GOLDEN, "sky_reference.json")))
    for r in sky:
        # SkyManager.cpp:47-52 direction from its fractions, then as elevation/azimuth angles
        th, ph = 2.0 * math.pi * (r["elevation"] - 0.5), 2.0 * math.pi * (r["azimuth"] - 0.5)
        d = (math.cos(ph), math.sin(ph) * math.sin(th), math.sin(ph) * math.cos(th))
        el, az = math.degrees(math.asin(max(-1.0, min(1.0, d[1])))), math.degrees(math.atan2(d[2], d[0]))
        u = np.frombuffer(orc.uniforms(64, 64, sun_elevation=el, sun_azimuth=az, time=r["time"]), np.float32)
        sun, sk = u[76:108], u[108:124]
        np.testing.assert_allclose(sun[4:8], r["direction"], rtol=1e-5, atol=1e-6)
        np.testing.assert_allclose(sun[0:4], r["location"], rtol=1e-5, atol=0.05)
        np.testing.assert_allclose(sun[12:28], r["direction_basis"], rtol=1e-5, atol=2e-6)
        np.testing.assert_allclose(sun[8:11], r["color_rgb"], rtol=1e-5)
        np.testing.assert_allclose(sun[28], r["intensity"][0], rtol=1e-5, atol=1e-3)
        np.testing.assert_allclose(sk[0:4], r["beta_r"], rtol=1e-5)
        np.testing.assert_allclose(sk[8:12], r["wind"], rtol=1e-6)
        np.testing.assert_allclose(sk[12], r["mie_directional"][0])


def test_oracle_uniforms_equal_the_library_set_up(orc, mmlib):
    # The same frames built by the library (scene.cpp) and by the oracle: identical bytes.
    import ctypes as C
    import marshmallow as mm
    for k in range(16):
        for w, h in ((3840, 2160), (256, 256)):
            el = (30.0, 5.0, -6.0, 85.0)[k % 4]
            a = np.frombuffer(orc.sweep_uniforms(k, w, h, sun_elevation=el), np.float32)
            u = mm.scene.sweep_uniforms(k, w, h, sun_elevation=el)
            b = np.frombuffer(C.string_at(C.addressof(u), 496), np.float32)
            assert np.array_equal(a, b), (k, w, h)


def test_sphere_intersection_needs_no_fp64():
    # raySphereIntersection (compute-clouds.comp:147-177) in FP32 against FP64 for the camera heights
    # of the scenes and elevations from 1e-4 deg to 90 deg: the shader's `isect.t` for the inner and
    # the outer shell.  The FP32 error is largest for steep rays (sqrt(disc) - B cancels there), not
    # near the horizon, and stays below 0.5 m on a 1000 m / 300 m march grid: no FP64 path is
    # needed on the GPU.
    def isect_t(ro, rd, c, w, T):
        ro = (ro - c) / T(w)
        A = (rd[0] * rd[0] + rd[1] * rd[1]) + rd[2] * rd[2]
        B = T(2) * ((rd[0] * ro[0] + rd[1] * ro[1]) + rd[2] * ro[2])
        C = ((ro[0] * ro[0] + ro[1] * ro[1]) + ro[2] * ro[2]) - T(0.25)
        disc = B * B - T(4) * A * C
        t = (-np.sqrt(disc) - B) / A * T(0.5)
        t = np.where(t < 0, (np.sqrt(disc) - B) / A * T(0.5), t)
        q = (ro + rd * t) * T(w) + c
        d = q - ro
        return np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]).astype(np.float64)

    el = np.radians(np.concatenate([np.geomspace(1e-4, 1.0, 400), np.linspace(1.0, 90.0, 400)]))
    for cam_y in (10.0, 150.0, 1000.0):
        for w in (2000000.0, 2000000.0 * 1.02):
            ts = {}
            for T in (np.float32, np.float64):
                rd = np.array([np.cos(el), np.sin(el), np.zeros_like(el)]).astype(np.float32).astype(T)
                rd = rd / np.sqrt((rd * rd).sum(0))
                ro = np.array([0.0, cam_y, 0.0], T)[:, None]
                c = np.array([0.0, -2000000.0 * 0.5 * 0.995, 0.0], T)[:, None]
                ts[T] = isect_t(ro, rd, c, w, T)
            err = np.abs(ts[np.float32] - ts[np.float64])
            assert (err / ts[np.float64]).max() < 5e-5
            assert err.max() < 0.5
            assert (err / ts[np.float64])[el < np.radians(1.0)].max() < 1e-5


def test_texture_unit_filter_matches_recorded_hardware_fetches(orc, oracle_textures):
    # tests/golden/texture_unit_fetches.npz: fetches of the GB300's texture unit (LINEAR, WRAP,
    # normalized coordinates, UNORM8) recorded by tests/golden/make_texture_unit_golden.py on the
    # seed-0 textures and two random ones (2D 53x37, 3D 24x20x12).  The oracle's texture-unit filter
    # reproduces every channel of every fetch; the exact-weight filter does not.
    g = np.load(os.path.join(GOLDEN, "texture_unit_fetches.npz"))
    for name in ("weather", "curl", "low_res", "hi_res", "random_2d", "random_3d"):
        texels = g[name + "_texels"] if name.startswith("random") else oracle_textures[name]
        coords, want = g[name + "_coords"], g[name + "_fetched"]
        got = orc.sample(texels, coords, filter=orc.FILTER_TEXTURE_UNIT)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name
        exact = orc.sample(texels, coords, filter=orc.FILTER_EXACT)
        assert np.mean(np.any(exact != want, axis=1)) > 0.5, name
