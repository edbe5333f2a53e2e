"""The post chain (god-ray.frag, radialBlur.frag, tonemap.frag and the mesh overlay) on the GPU
against the CPU restatement."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

W, H = 640, 360


@pytest.fixture(scope="module")
def env(cuda, mmlib):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    yield t, r
    r.close()
    t.close()


def _clouds(cuda, env, sun_elevation=20.0, yaw=0.0):
    # A cloud frame looking towards the sun: its alpha carries the sun disk the god rays spread.
    import marshmallow as mm
    tex, r = env
    u = mm.scene.uniforms(W, H, yaw=yaw, pitch=12.0, sun_elevation=sun_elevation)
    rgba = cuda.zeros((H, W, 4), device="cuda")
    if sun_elevation > 0:
        r.march(u, tex, rgba)
    else:
        rgba.uniform_(0.0, 2.0)
    cuda.cuda.synchronize()
    return u, rgba


@pytest.mark.parametrize("which", ["god_rays", "radial_blur"])
def test_single_passes_exact(cuda, orc, env, which):
    import marshmallow.lib as L
    _, r = env
    u, src = _clouds(cuda, env)
    if which == "radial_blur":  # feed it a god-ray framebuffer
        g = cuda.empty_like(src)
        r.god_rays(u, src, g, math=L.MATH_EXACT)
        src = g
    dst = cuda.full_like(src, -1.0)
    getattr(r, which)(u, src, dst, math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    want = orc.post_pass(which, u, src.cpu().numpy())
    got = dst.cpu().numpy()
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
    if which == "god_rays":
        assert got[..., 3].max() > 0.1  # the sun is in view


@pytest.mark.parametrize("bgra", [0, 1])
def test_tonemap_exact(cuda, orc, env, bgra):
    import marshmallow.lib as L
    _, r = env
    src = cuda.rand((H, W, 4), device="cuda") * 60.0
    out = cuda.zeros((H, W, 4), dtype=cuda.uint8, device="cuda")
    r.tonemap(src, out, math=L.MATH_EXACT, bgra=bgra)
    cuda.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), orc.post_tonemap(src.cpu().numpy(), bgra=bgra))


@pytest.mark.parametrize("case", ["day", "day+mesh", "night"])
def test_chain_exact(cuda, orc, env, case):
    import marshmallow.lib as L
    _, r = env
    u, clouds = _clouds(cuda, env, sun_elevation=-10.0 if case == "night" else 20.0)
    mesh = None
    if case == "day+mesh":
        mesh = cuda.zeros_like(clouds)
        mesh[H // 2:, :, :3] = cuda.rand((H - H // 2, W, 3), device="cuda")
        mesh[H // 2:, :, 3] = 1.0
    out = cuda.zeros((H, W, 4), dtype=cuda.uint8, device="cuda")
    r.post_chain(u, clouds, out, mesh=mesh, math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    want = orc.post_chain(u, clouds.cpu().numpy(), mesh.cpu().numpy() if mesh is not None else None, bgra=1)
    assert np.array_equal(out.cpu().numpy(), want)


@pytest.mark.parametrize("yaw", [0.0, 25.0])
def test_chain_fast_within_gates(cuda, orc, env, yaw):
    # Production arithmetic: the tap loops run on the texture unit (8-bit fixed-point filter
    # weights) and pow on the SFU; the 8-bit output stays within a few LSB of the exact chain.
    _, r = env
    u, clouds = _clouds(cuda, env, yaw=yaw)
    out = cuda.zeros((H, W, 4), dtype=cuda.uint8, device="cuda")
    r.post_chain(u, clouds, out)
    cuda.cuda.synchronize()
    want = orc.post_chain(u, clouds.cpu().numpy(), bgra=1).astype(int)
    d = np.abs(out.cpu().numpy().astype(int) - want)
    print("fast chain: max %d, frac > 0: %.2e, frac > 1: %.2e" % (d.max(), (d > 0).mean(), (d > 1).mean()))
    assert d.max() <= 4 and (d > 1).mean() <= 1e-3 and (d > 0).mean() <= 0.05


def test_chain_equals_passes_through_framebuffers(cuda, env):
    # mm_post_chain (two kernels, a float plane) == the three single passes through RGBA32F images.
    import marshmallow.lib as L
    _, r = env
    u, clouds = _clouds(cuda, env, yaw=10.0)
    fb1, fb2 = cuda.empty_like(clouds), cuda.empty_like(clouds)
    r.god_rays(u, clouds, fb1, math=L.MATH_EXACT)
    r.radial_blur(u, fb1, fb2, math=L.MATH_EXACT)
    a = cuda.zeros((H, W, 4), dtype=cuda.uint8, device="cuda")
    b = cuda.zeros_like(a)
    r.tonemap(fb2, a, math=L.MATH_EXACT)
    r.post_chain(u, clouds, b, math=L.MATH_EXACT)
    cuda.cuda.synchronize()
    assert cuda.equal(a, b)


def test_post_argument_errors(cuda, env):
    import marshmallow.lib as L
    _, r = env
    lib = L.load()
    u, clouds = _clouds(cuda, env)
    o = r.post_options()
    img = r._rgba_image(clouds)
    # source and destination overlap
    assert lib.mm_post_god_rays(r.ctx, C.byref(u), C.byref(img), C.byref(img), C.byref(o), None) == \
        L.MM_ERR_INVALID_ARGUMENT
    # size mismatch
    small = cuda.zeros((H // 2, W, 4), device="cuda")
    assert lib.mm_post_radial_blur(r.ctx, C.byref(u), C.byref(img), C.byref(r._rgba_image(small)), C.byref(o),
                                   None) == L.MM_ERR_INVALID_ARGUMENT
    # 8-bit pitch too small
    out = cuda.zeros((H, W, 4), dtype=cuda.uint8, device="cuda")
    assert lib.mm_post_tonemap(r.ctx, C.byref(img), out.data_ptr(), W * 2, C.byref(o), None) == \
        L.MM_ERR_INVALID_ARGUMENT
    bad = L.PostOptions(7, 1)
    assert lib.mm_post_chain(r.ctx, C.byref(u), C.byref(img), None, out.data_ptr(), W * 4, C.byref(bad), None) == \
        L.MM_ERR_INVALID_ARGUMENT


def test_exact_passes_vs_reference_shader_golden(cuda, env):
    # god-ray.frag, radialBlur.frag and tonemap.frag themselves, compiled as C++ on the CPU
    # (tests/golden/shader_passes.npz).  The exact kernels equal the CPU restatement, which differs
    # from the compiled shaders only in the centre fetch (the texel itself here; a float-weight filter
    # ~1e-5 of a texel off the centre there): within 3e-5 of each channel's largest input value, and
    # the 8-bit tonemap within one step on at most 0.1% of the bytes.
    import marshmallow.lib as L
    import shader_golden as sg
    _, r = env
    z = sg.passes()
    u = L.Uniforms.from_buffer_copy(z["post_uniforms"].tobytes())
    w, h = sg.POST_SIZE
    src_np = sg.pattern(h, w, 11)
    src = cuda.from_numpy(src_np).cuda()
    g = cuda.full_like(src, -1.0)
    r.god_rays(u, src, g, math=L.MATH_EXACT)
    b = cuda.full_like(src, -1.0)
    r.radial_blur(u, g, b, math=L.MATH_EXACT)
    out8 = cuda.zeros((h, w, 4), dtype=cuda.uint8, device="cuda")
    r.tonemap(src, out8, math=L.MATH_EXACT, bgra=0)
    cuda.cuda.synchronize()
    g_np, b_np, t_np = g.cpu().numpy(), b.cpu().numpy(), out8.cpu().numpy()
    bound_a = 3e-5 * np.abs(src_np[..., 3]).max() + 1e-7
    assert np.abs(g_np[..., 3] - z["god_ray_alpha"]).max() <= bound_a
    bound_rgb = 1.5e-5 * np.abs(g_np[..., :3]).reshape(-1, 3).max(0) + 1e-7
    assert np.all(np.abs(b_np[..., :3] - z["radial_blur_rgb"]) <= bound_rgb)
    d = np.abs(t_np[..., :3].astype(int) - z["tonemap_rgb"].astype(int))
    assert d.max() <= 1 and (d > 0).mean() <= 1e-3
