"""The mesh cloud-shadow march (model.frag:52-162, 221-222, 240-276) on the GPU against the CPU restatement."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 640, 360
EYE = (0.0, 150.0, 0.0)


@pytest.fixture(scope="module")
def env(cuda, mmlib):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    yield t, r
    r.close()
    t.close()


def _scene(w, h, **kw):
    import marshmallow as mm
    u = mm.scene.uniforms(w, h, eye=EYE, pitch=kw.pop("pitch", -20.0), **kw)
    return u, mm.scene.terrain_gbuffer(u, w, h)


def _gpu_shadow(cuda, r, tex, u, gbuf, **opts):
    pos = cuda.from_numpy(gbuf).cuda()
    out = cuda.full(gbuf.shape[:2], -1.0, device="cuda")
    r.mesh_shadow(u, tex, pos, shadow=out, **opts)
    cuda.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("elev,time,cov", [(30.0, 0.0, 0.0), (60.0, 40.0, 0.0), (45.0, 5.0, 0.2)])
def test_shadow_exact_matches_oracle_bit_for_bit(cuda, orc, oracle_textures, env, elev, time, cov):
    import marshmallow.lib as L
    tex, r = env
    u, g = _scene(W, H, sun_elevation=elev, time=time)
    got = _gpu_shadow(cuda, r, tex, u, g, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE, coverage_offset=cov)
    want = orc.shadow(u, oracle_textures, g, coverage_offset=cov)
    assert (want > 0).mean() > 0.2  # the scene has cloud shadow to check
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("sampler", ["software", "hardware"])
def test_shadow_fast_within_gates_of_fp64(cuda, orc, oracle_textures, env, sampler):
    # Fast arithmetic (and the texture unit's 8-bit filter weights) against the FP64 restatement.
    # The shadow is a max of densities, so errors do not accumulate; a sample that crosses the
    # 1e-4 early-out or the 0.99 saturation can flip, hence a tail gate on the fraction of pixels.
    import marshmallow.lib as L
    tex, r = env
    s = L.SAMPLER_SOFTWARE if sampler == "software" else L.SAMPLER_HARDWARE
    for elev, time in ((30.0, 0.0), (60.0, 40.0)):
        u, g = _scene(W, H, sun_elevation=elev, time=time)
        got = _gpu_shadow(cuda, r, tex, u, g, math=L.MATH_FAST, sampler=s)
        want = orc.shadow(u, oracle_textures, g, precision=64)
        err = np.abs(got.astype(np.float64) - want)
        print(sampler, elev, time, "mean %.2e p99.9 %.2e max %.2e frac>0.01 %.2e"
              % (err.mean(), np.percentile(err, 99.9), err.max(), (err > 0.01).mean()))
        assert err.mean() <= (2e-5 if s == L.SAMPLER_SOFTWARE else 2e-3)
        assert (err > 0.01).mean() <= (1e-4 if s == L.SAMPLER_SOFTWARE else 5e-3)


def test_shadow_darkens_rgba_and_skips_uncovered_pixels(cuda, env):
    import marshmallow.lib as L
    tex, r = env
    u, g = _scene(320, 180, sun_elevation=40.0, time=10.0)
    assert 0.0 < (g[..., 3] != 0).mean() < 1.0
    rng = np.random.default_rng(7)
    lit = rng.uniform(0.0, 3.0, (180, 320, 4)).astype(np.float32)
    pos = cuda.from_numpy(g).cuda()
    rgba = cuda.from_numpy(lit).cuda()
    sh = cuda.full((180, 320), -1.0, device="cuda")
    r.mesh_shadow(u, tex, pos, shadow=sh, rgba=rgba, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
    cuda.cuda.synchronize()
    s, out = sh.cpu().numpy(), rgba.cpu().numpy()
    cov = g[..., 3] != 0
    assert np.all(s[~cov] == 0.0) and np.array_equal(out[~cov], lit[~cov])
    k = (np.float32(1.0) - s * np.float32(2.0))[..., None]
    want = np.maximum(lit[..., :3] * k, np.float32(0.0))
    assert np.array_equal(out[cov][:, :3], want[cov])
    assert np.all(out[cov][:, 3] == 1.0)
    assert s[cov].max() > 0.0


def test_shadow_argument_errors(cuda, env):
    import marshmallow.lib as L
    tex, r = env
    lib = L.load()
    u, g = _scene(64, 32)
    pos = cuda.from_numpy(g).cuda()
    out = cuda.zeros((32, 64), device="cuda")
    st = tex.scene()
    o = r.options()
    gb = L.GBuffer(pos.data_ptr(), pos.stride(0) * 4, 64, 32)
    # neither output
    assert lib.mm_mesh_shadow(r.ctx, C.byref(u), C.byref(st), C.byref(gb), None, 0, None, 0, C.byref(o), None) \
        == L.MM_ERR_INVALID_ARGUMENT
    # misaligned G-buffer rows
    bad = L.GBuffer(pos.data_ptr() + 4, pos.stride(0) * 4, 64, 32)
    assert lib.mm_mesh_shadow(r.ctx, C.byref(u), C.byref(st), C.byref(bad), C.c_void_p(out.data_ptr()), 256, None, 0,
                              C.byref(o), None) == L.MM_ERR_INVALID_ARGUMENT
    # missing low-res texture
    st2 = tex.scene()
    st2.low_res = None
    assert lib.mm_mesh_shadow(r.ctx, C.byref(u), C.byref(st2), C.byref(gb), C.c_void_p(out.data_ptr()), 256, None, 0,
                              C.byref(o), None) == L.MM_ERR_INVALID_ARGUMENT
    assert b"low_res" in lib.mm_last_error_string()


def test_device_gbuffer_matches_host_gbuffer(cuda, mmlib):
    import marshmallow as mm
    u = mm.scene.uniforms(160, 90, eye=EYE, pitch=-20.0)
    a = mm.scene.terrain_gbuffer(u, 160, 90)
    b = mm.scene.terrain_gbuffer_cuda(u, 160, 90).cpu().numpy()
    assert np.array_equal(a[..., 3], b[..., 3])
    assert np.max(np.abs(a - b)) < 1e-2


@pytest.mark.parametrize("mode", ["exact", "fast_hardware"])
def test_shadow_vs_reference_shader_golden(cuda, env, mode):
    # model.frag itself, compiled as C++ on the CPU, with the shadow recovered from its shaded colour
    # (tests/golden/shader_passes.npz; NaN where the shadow is >= 0.5 and the colour clamps to 0).
    import marshmallow.lib as L
    import shader_golden as sg
    tex, r = env
    z = sg.passes()
    u = L.Uniforms.from_buffer_copy(z["shadow_uniforms"].tobytes())
    g = np.ascontiguousarray(z["shadow_world_pos"])
    opts = dict(math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE) if mode == "exact" else dict(math=L.MATH_FAST,
                                                                                         sampler=L.SAMPLER_HARDWARE)
    got = _gpu_shadow(cuda, r, tex, u, g, **opts)
    want = z["shadow"]
    fin = np.isfinite(want)
    err = np.abs(got[fin].astype(np.float64) - want[fin])
    if mode == "exact":
        assert err.max() <= 1e-6
        assert np.all(got[~fin] >= 0.5 - 1e-6)
    else:
        assert err.mean() <= 2e-3 and (err > 0.01).mean() <= 5e-3
