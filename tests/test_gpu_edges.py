"""Edge cases on the GPU: ragged and degenerate image sizes for every pass (bit-exact against the
oracle in exact arithmetic), the block-row order of the march at every horizon position, and size
limits."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(cuda, mmlib):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    yield t, r
    r.close()
    t.close()


SIZES = [(1, 1), (3, 200), (37, 23), (130, 9)]


@pytest.mark.parametrize("w,h", SIZES)
@pytest.mark.parametrize("mode", [0, 1])
def test_march_ragged_sizes_exact(cuda, orc, oracle_textures, env, w, h, mode):
    # Sizes that are not multiples of the 16x8 block tile or of the 4x4 phase pattern; PHASE16 with a
    # phase whose column/row offset lies outside a 1-pixel image leaves every pixel untouched.
    import marshmallow as mm
    import marshmallow.lib as L
    from gpu_util import render
    tex, r = env
    for phase in ((0, 7, 15) if mode else (0,)):
        u = mm.scene.uniforms(w, h, yaw=15.0, pitch=20.0)
        u.sun.color[3] = float(phase)
        rgba = cuda.full((h, w, 4), -7.0, device="cuda")
        dep = cuda.full((h, w), -7.0, device="cuda")
        r.march(u, tex, rgba, dep, pixel_mode=mode, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
        cuda.cuda.synchronize()
        want, wd, _ = orc.march(u, oracle_textures, w, h, pixel_mode=mode)
        got, gd = rgba.cpu().numpy(), dep.cpu().numpy()
        if mode:
            m = np.zeros((h, w), bool)
            m[phase // 4::4, phase % 4::4] = True
            assert np.all(got[~m] == -7.0) and np.all(gd[~m] == -7.0)
            got, gd, want, wd = got[m], gd[m], want[m], wd[m]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32))


@pytest.mark.parametrize("pitch", [-60.0, -25.0, 5.0, 45.0, 80.0])
def test_block_row_order_every_horizon_position(cuda, orc, oracle_textures, env, pitch):
    # The tiled march launches the block rows above the horizon first (a permutation chosen per
    # camera): horizon above the image, inside it, and below it give the oracle's image.
    import marshmallow as mm
    import marshmallow.lib as L
    from gpu_util import render
    tex, r = env
    w, h = 96, 72
    u = mm.scene.uniforms(w, h, yaw=40.0, pitch=pitch)
    rgba, dep = render(cuda, r, u, tex, w, h, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
    want, wd, _ = orc.march(u, oracle_textures, w, h)
    assert np.array_equal(rgba.view(np.uint32), want.view(np.uint32))
    assert np.array_equal(dep.view(np.uint32), wd.view(np.uint32))


@pytest.mark.parametrize("w,h", SIZES)
def test_reproject_ragged_sizes_exact(cuda, orc, env, w, h):
    import marshmallow as mm
    import marshmallow.lib as L
    _, r = env
    cur = mm.scene.uniforms(w, h, yaw=12.0, pitch=14.0)
    cur.camera_prev = mm.scene.uniforms(w, h, yaw=9.0, pitch=15.0).camera_prev
    rng = np.random.default_rng(w * 1000 + h)
    src = rng.uniform(0, 4, (h, w, 4)).astype(np.float32)
    sd = rng.uniform(1e3, 1e5, (h, w)).astype(np.float32)
    s = (cuda.from_numpy(src).cuda(), cuda.from_numpy(sd).cuda())
    d = (cuda.empty_like(s[0]), cuda.empty_like(s[1]))
    r.reproject(cur, s, d, math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    want, wd = orc.reproject(cur, src, sd)
    assert np.array_equal(d[0].cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(d[1].cpu().numpy(), wd)


@pytest.mark.parametrize("w,h", SIZES)
def test_shadow_ragged_sizes_exact(cuda, orc, oracle_textures, env, w, h):
    import marshmallow as mm
    import marshmallow.lib as L
    tex, r = env
    u = mm.scene.uniforms(w, h, eye=(0.0, 150.0, 0.0), pitch=-35.0, sun_elevation=50.0, time=3.0)
    g = mm.scene.terrain_gbuffer(u, w, h)
    pos = cuda.from_numpy(g).cuda()
    out = cuda.full((h, w), -1.0, device="cuda")
    r.mesh_shadow(u, tex, pos, shadow=out, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE)
    cuda.cuda.synchronize()
    want = orc.shadow(u, oracle_textures, g)
    assert np.array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_shadow_without_covered_pixels(cuda, env):
    # A G-buffer with no mesh fragment: every shadow is 0 and the colour image is untouched.
    import marshmallow as mm
    tex, r = env
    u = mm.scene.uniforms(40, 30)
    pos = cuda.zeros((30, 40, 4), device="cuda")
    rgba = cuda.full((30, 40, 4), 0.25, device="cuda")
    out = cuda.full((30, 40), -1.0, device="cuda")
    r.mesh_shadow(u, tex, pos, shadow=out, rgba=rgba)
    cuda.cuda.synchronize()
    assert bool((out == 0).all()) and bool((rgba == 0.25).all())


@pytest.mark.parametrize("w,h", SIZES)
def test_post_chain_ragged_sizes_exact(cuda, orc, env, w, h):
    import marshmallow as mm
    import marshmallow.lib as L
    _, r = env
    u = mm.scene.uniforms(w, h, yaw=0.0, pitch=12.0, sun_elevation=20.0)
    rng = np.random.default_rng(w + 7 * h)
    img = rng.uniform(0, 3, (h, w, 4)).astype(np.float32)
    clouds = cuda.from_numpy(img).cuda()
    out = cuda.zeros((h, w, 4), dtype=cuda.uint8, device="cuda")
    r.post_chain(u, clouds, out, math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), orc.post_chain(u, img, bgra=1))
    # the production chain on the same ragged sizes: within 1 LSB
    r.post_chain(u, clouds, out)
    cuda.cuda.synchronize()
    d = np.abs(out.cpu().numpy().astype(int) - orc.post_chain(u, img, bgra=1).astype(int))
    assert d.max() <= 1


def test_size_limits(cuda, mmlib, env):
    # Zero and negative sizes and sizes above 32768 are rejected before any launch.
    import marshmallow as mm
    import marshmallow.lib as L
    tex, r = env
    u = mm.scene.uniforms(64, 64)
    buf = cuda.zeros((64, 64, 4), device="cuda")
    st = tex.scene()
    o = r.options()
    for w, h in ((0, 64), (64, 0), (-5, 64), (32769, 1), (1, 32769)):
        img = L.Image(buf.data_ptr(), 1 << 20, None, 0, w, h)
        assert mmlib.mm_clouds_march(r.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None) == \
            L.MM_ERR_INVALID_ARGUMENT, (w, h)
        gb = L.GBuffer(buf.data_ptr(), 1 << 20, w, h)
        assert mmlib.mm_mesh_shadow(r.ctx, C.byref(u), C.byref(st), C.byref(gb), C.c_void_p(buf.data_ptr()),
                                    1 << 20, None, 0, C.byref(o), None) == L.MM_ERR_INVALID_ARGUMENT
    cuda.cuda.synchronize()


def test_half2_coverage_test_needs_fp16_density(cuda, mmlib, env):
    # MM_MATH_FAST_HALF2 reads the density texels as packed FP16: with UNORM8 density, the software
    # sampler or the persistent schedule it is rejected before any launch.
    import marshmallow as mm
    import marshmallow.lib as L
    tex, r = env
    u = mm.scene.uniforms(64, 64)
    buf = cuda.zeros((64, 64, 4), device="cuda")
    img = L.Image(buf.data_ptr(), 64 * 16, None, 0, 64, 64)
    st = tex.scene()
    for kw in (dict(), dict(density_format=L.FORMAT_FP16, sampler=L.SAMPLER_SOFTWARE),
               dict(density_format=L.FORMAT_FP16, schedule=L.SCHEDULE_PERSISTENT)):
        o = r.options(math=L.MATH_FAST_HALF2, **kw)
        assert mmlib.mm_clouds_march(r.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None) == \
            L.MM_ERR_INVALID_ARGUMENT, kw
    cuda.cuda.synchronize()


def test_kernel_variants_exact(cuda, orc, oracle_textures, env):
    # The march picks its kernel per launch (full frames with pooled sun cones, launches of <= 262144
    # rays, larger 1/16-pixel launches); all are the same arithmetic and equal the oracle bit for bit.
    # Full frames at two pixel pitches: 2880x1620 at 60 degrees, 1280x720 at 20 degrees.
    import marshmallow as mm
    import marshmallow.lib as L
    tex, r = env
    for (w, h, mode, fov) in [(2880, 1620, 1, 60.0), (2880, 1620, 0, 60.0), (1280, 720, 0, 20.0), (640, 400, 0, 60.0),
                              (640, 400, 1, 60.0)]:
        u = mm.scene.uniforms(w, h, yaw=30.0, pitch=10.0, fov=fov, time=1.0)
        u.sun.color[3] = 9.0
        rgba = cuda.zeros((h, w, 4), device="cuda")
        dep = cuda.zeros((h, w), device="cuda")
        cnt = cuda.zeros(4, dtype=cuda.int64, device="cuda")
        r.march(u, tex, rgba, dep, pixel_mode=mode, math=L.MATH_EXACT, sampler=L.SAMPLER_SOFTWARE, counters=cnt)
        cuda.cuda.synchronize()
        want, wd, wc = orc.march(u, oracle_textures, w, h, pixel_mode=mode)
        got, gd = rgba.cpu().numpy(), dep.cpu().numpy()
        if mode:
            got, gd, want, wd = got[2::4, 1::4], gd[2::4, 1::4], want[2::4, 1::4], wd[2::4, 1::4]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (w, h, mode)
        assert np.array_equal(gd.view(np.uint32), wd.view(np.uint32)), (w, h, mode)
        # work counts (cloudTest, cloudHiRes, iterations, accumulated samples) equal the oracle's
        assert np.array_equal(cnt.cpu().numpy().astype(np.uint64), wc), (w, h, mode, cnt.cpu().numpy(), wc)
