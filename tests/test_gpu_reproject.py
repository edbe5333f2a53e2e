"""The reprojection pass and the reference's per-frame compute work on the GPU."""
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


@pytest.mark.parametrize("frame", [1, 9])
def test_reproject_bit_exact(cuda, orc, env, frame):
    import marshmallow as mm
    _, r = env
    w, h = 640, 360
    cur = mm.scene.sweep_uniforms(frame, w, h)
    prev = mm.scene.sweep_uniforms(frame - 1, w, h)
    cur.camera_prev = prev.camera_prev
    rng = np.random.default_rng(frame)
    src = rng.uniform(0, 20, (h, w, 4)).astype(np.float32)
    sd = rng.uniform(1e3, 3e5, (h, w)).astype(np.float32)
    s_rgba, s_dep = cuda.from_numpy(src).cuda(), cuda.from_numpy(sd).cuda()
    d_rgba, d_dep = cuda.zeros_like(s_rgba), cuda.zeros_like(s_dep)
    import marshmallow.lib as L
    r.reproject(cur, (s_rgba, s_dep), (d_rgba, d_dep), math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    want, wd = orc.reproject(cur, src, sd)
    assert np.array_equal(d_rgba.cpu().numpy().view(np.uint32), want.view(np.uint32))
    assert np.array_equal(d_dep.cpu().numpy(), wd)


def test_sixteen_phase_frames_rebuild_the_full_frame(cuda, env):
    # Static camera: each frame reprojects the previous one onto itself and marches one pixel in 16;
    # after the 16 phases every pixel has been marched once and the image is the full-frame march.
    import marshmallow as mm
    tex, r = env
    w, h = 320, 180
    full = cuda.zeros((h, w, 4), device="cuda")
    fdep = cuda.zeros((h, w), device="cuda")
    u = mm.scene.uniforms(w, h, yaw=10.0, pitch=18.0)
    r.march(u, tex, full, fdep)
    bufs = [(cuda.zeros((h, w, 4), device="cuda"), cuda.full((h, w), float("inf"), device="cuda")) for _ in range(2)]
    for k in range(16):
        u.sun.color[3] = float(k)
        r.frame(u, tex, bufs[k % 2], bufs[(k + 1) % 2])
    cuda.cuda.synchronize()
    img, dep = bufs[0][0].cpu().numpy(), bufs[0][1].cpu().numpy()
    ref = full.cpu().numpy()
    assert np.allclose(img, ref, rtol=1e-5, atol=1e-7)
    assert np.array_equal(np.isinf(dep), np.isinf(fdep.cpu().numpy()))


def test_reproject_rejects_aliasing(cuda, env):
    import ctypes as C
    import marshmallow as mm
    _, r = env
    a = cuda.zeros((16, 16, 4), device="cuda")
    u = mm.scene.uniforms(16, 16)
    img = r.image(a)
    assert r.lib.mm_clouds_reproject(r.ctx, C.byref(u), C.byref(img), C.byref(img), None, None) == 1


@pytest.mark.parametrize("frame", [1, 9])
def test_reproject_fast_matches_exact(cuda, env, frame):
    # Production arithmetic: the same texels except where a tap lands within rounding of a pixel
    # boundary; colour to float rounding elsewhere (the sum is scaled by 0.1 instead of divided by 10).
    import marshmallow as mm
    import marshmallow.lib as L
    _, r = env
    w, h = 1280, 720
    cur = mm.scene.sweep_uniforms(frame, w, h)
    cur.camera_prev = mm.scene.sweep_uniforms(frame - 1, w, h).camera_prev
    rng = np.random.default_rng(10 + frame)
    src = (cuda.from_numpy(rng.uniform(0, 20, (h, w, 4)).astype(np.float32)).cuda(),
           cuda.from_numpy(rng.uniform(1e3, 3e5, (h, w)).astype(np.float32)).cuda())
    ex = (cuda.empty_like(src[0]), cuda.empty_like(src[1]))
    fa = (cuda.empty_like(src[0]), cuda.empty_like(src[1]))
    r.reproject(cur, src, ex, math=L.MATH_EXACT)
    r.reproject(cur, src, fa, math=L.MATH_FAST)
    cuda.cuda.synchronize()
    e, f = ex[0].cpu().numpy(), fa[0].cpu().numpy()
    close = np.all(np.abs(f - e) <= 1e-5 * np.maximum(np.abs(e), 1.0), axis=-1)
    same_centre = ex[1].cpu().numpy() == fa[1].cpu().numpy()
    print("fast reprojection: %.4f%% of pixels differ, %.4f%% other centre tap"
          % (100 * (1 - close.mean()), 100 * (1 - same_centre.mean())))
    # one tap in ~2000 lands within rounding of a pixel boundary (the centre tap: 0.055% measured);
    # with ten taps per pixel that moves ~0.5% of the pixels
    assert close.mean() >= 0.99 and same_centre.mean() >= 0.999


@pytest.mark.parametrize("math", [0, 1])
def test_frame_equals_sequential_passes(cuda, env, math):
    # mm_clouds_frame runs the reprojection of the other 15 pixels in 16 on a second stream beside
    # the 1/16 march: the result equals reprojecting every pixel and then marching the phase.
    import marshmallow as mm
    tex, r = env
    w, h = 333, 190
    for k, phase in ((3, 0), (4, 6), (5, 15)):
        u = mm.scene.sweep_uniforms(k, w, h)
        u.camera_prev = mm.scene.sweep_uniforms(k - 1, w, h).camera_prev
        u.sun.color[3] = float(phase)
        rng = np.random.default_rng(k)
        prev = (cuda.from_numpy(rng.uniform(0, 3, (h, w, 4)).astype(np.float32)).cuda(),
                cuda.from_numpy(rng.uniform(1e3, 1e5, (h, w)).astype(np.float32)).cuda())
        a = (cuda.full((h, w, 4), -1.0, device="cuda"), cuda.full((h, w), -1.0, device="cuda"))
        b = (cuda.full((h, w, 4), -1.0, device="cuda"), cuda.full((h, w), -1.0, device="cuda"))
        r.frame(u, tex, prev, a, math=math)
        r.reproject(u, prev, b, math=math)
        r.march(u, tex, b[0], b[1], pixel_mode=1, math=math)
        cuda.cuda.synchronize()
        assert cuda.equal(a[0], b[0]) and cuda.equal(a[1], b[1]), (k, phase)


@pytest.mark.parametrize("k", range(3))
def test_reproject_exact_equals_reference_shader_golden(cuda, env, k):
    # reproject.comp itself, compiled as C++ on the CPU (tests/golden/shader_passes.npz): the exact
    # kernel reproduces its image bit for bit (SHA-256 of the rgba).
    import marshmallow.lib as L
    import shader_golden as sg
    _, r = env
    z = sg.passes()
    w, h = sg.REPROJECT_CASES[k][:2]
    u = L.Uniforms.from_buffer_copy(z["reproject_uniforms"][k].tobytes())
    src = cuda.from_numpy(sg.pattern(h, w, k)).cuda()
    dst = cuda.full_like(src, -1.0)
    sd, dd = cuda.zeros((h, w), device="cuda"), cuda.zeros((h, w), device="cuda")
    r.reproject(u, (src, sd), (dst, dd), math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    assert sg.digest(dst.cpu().numpy()) == str(z["reproject_digests"][k])
