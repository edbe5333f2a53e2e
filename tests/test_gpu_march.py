"""The CUDA cloud march vs the CPU oracle of compute-clouds.comp.

Gates (colour errors in 1/255 of the reference tonemap, tonemap.frag:10-28):
  - exact arithmetic + software sampler vs the FP32 oracle: identical output and identical work
    counters (bit-exact);
  - vs the FP64 oracle, any arithmetic with the software sampler: RMSE <= 1/255, max <= 4/255 on
    99.9% of pixels (p99.9; at most 0.2% of pixels above 4/255), depth relative error <= 1e-3 on
    99.9% of pixels where both depths are finite.  A pixel where one of the march's thresholds
    (density > 0 at :426, < 1e-4 at :243/:437, accumulated > 0.99 at :476) falls the other way
    takes a different path; the tails above bound how many do.
  - hardware sampler (texture-unit filtering, 8-bit fixed-point weights) vs the FP64 oracle: the
    same colour gates; depth: median relative error <= 1e-4 and at most 3% of pixels above 1e-3.
    The filter-weight quantisation moves densities by up to ~1/256 of a texel step, which shifts
    the first hit of a few rays by one 300 m / 1000 m march step; depth is the march distance of
    that sample, so such a ray's depth moves by one step.
"""
import numpy as np
import pytest

from gpu_util import render, render_counted

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu_textures(cuda, mmlib):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    yield t
    t.close()


@pytest.fixture(scope="module")
def host_textures(gpu_textures):
    return gpu_textures.host_all()


@pytest.fixture(scope="module")
def renderer(cuda, mmlib):
    import marshmallow as mm
    r = mm.render.Renderer()
    yield r
    r.close()


def test_gpu_textures_equal_oracle_textures(host_textures, oracle_textures):
    for k in oracle_textures:
        assert np.array_equal(host_textures[k], oracle_textures[k]), k


@pytest.mark.parametrize("schedule", [0, 1])
def test_exact_software_bit_exact_256(cuda, orc, renderer, gpu_textures, host_textures, schedule):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(256, 256)
    rgba, dep, cnt = render_counted(cuda, renderer, u, gpu_textures, 256, 256, sampler=L.SAMPLER_SOFTWARE,
                                    math=L.MATH_EXACT, schedule=schedule)
    ref, rdep, rcnt = orc.march(u, host_textures, 256, 256, precision=32)
    assert np.array_equal(rgba.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(dep.view(np.uint32), rdep.view(np.uint32))
    assert np.array_equal(cnt, rcnt)


@pytest.mark.parametrize("frame,schedule", [(0, 0), (7, 0), (15, 0), (11, 1)])
def test_exact_software_bit_exact_1080p_rows(cuda, orc, renderer, gpu_textures, host_textures, frame, schedule):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.sweep_uniforms(frame, 1920, 1080)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 1920, 1080, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT,
                       schedule=schedule)
    ref, rdep, _ = orc.march(u, host_textures, 1920, 1080, precision=32, rows=(frame, 1080, 24))
    assert np.array_equal(rgba[frame::24].view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(dep[frame::24].view(np.uint32), rdep.view(np.uint32))


def _gates(e, hardware=False):
    assert e["nan"] == 0
    assert e["rmse_255"] <= 1.0, e
    assert e["p999_255"] <= 4.0, e
    assert e["frac_over_4"] <= 0.002, e
    if hardware:
        assert e.get("depth_rel_median", 0.0) <= 1e-4, e
        assert e.get("depth_frac_over_1e3", 0.0) <= 0.03, e
    else:
        assert e.get("depth_rel_p999", 0.0) <= 1e-3, e


@pytest.mark.parametrize("sampler,schedule", [(0, 0), (1, 0), (0, 1), (1, 1)])
def test_fast_vs_fp64_oracle_256(cuda, orc, renderer, gpu_textures, host_textures, sampler, schedule):
    import marshmallow as mm
    u = mm.scene.uniforms(256, 256)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 256, 256, sampler=sampler, schedule=schedule)
    ref, rdep, _ = orc.march(u, host_textures, 256, 256, precision=64)
    e = mm.metrics.frame_errors(rgba, ref, dep, rdep)
    print("fast sampler=%d vs fp64:" % sampler, e)
    _gates(e, hardware=sampler == 0)


@pytest.mark.parametrize("frame", [0, 5, 10, 15])
def test_fast_vs_fp64_oracle_1080p_sweep(cuda, orc, renderer, gpu_textures, host_textures, frame):
    import marshmallow as mm
    u = mm.scene.sweep_uniforms(frame, 1920, 1080)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 1920, 1080)
    ref, rdep, _ = orc.march(u, host_textures, 1920, 1080, precision=64, rows=(frame % 8, 1080, 8))
    e = mm.metrics.frame_errors(rgba[frame % 8::8], ref, dep[frame % 8::8], rdep)
    print("1080p frame %d fast vs fp64:" % frame, e)
    _gates(e, hardware=True)


@pytest.mark.parametrize("frame", [2, 12])
def test_fast_software_vs_fp64_oracle_1080p(cuda, orc, renderer, gpu_textures, host_textures, frame):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.sweep_uniforms(frame, 1920, 1080)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 1920, 1080, sampler=L.SAMPLER_SOFTWARE)
    ref, rdep, _ = orc.march(u, host_textures, 1920, 1080, precision=64, rows=(frame % 8, 1080, 8))
    e = mm.metrics.frame_errors(rgba[frame % 8::8], ref, dep[frame % 8::8], rdep)
    print("1080p frame %d fast software vs fp64:" % frame, e)
    _gates(e)


def test_persistent_equals_tiled_exact(cuda, renderer, gpu_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.sweep_uniforms(9, 1280, 720)
    for sampler in (L.SAMPLER_SOFTWARE, L.SAMPLER_HARDWARE):
        a, da, ca = render_counted(cuda, renderer, u, gpu_textures, 1280, 720, sampler=sampler, math=L.MATH_EXACT,
                                   schedule=L.SCHEDULE_PERSISTENT)
        b, db, cb = render_counted(cuda, renderer, u, gpu_textures, 1280, 720, sampler=sampler, math=L.MATH_EXACT,
                                   schedule=L.SCHEDULE_TILED)
        assert np.array_equal(a, b) and np.array_equal(da, db) and np.array_equal(ca, cb)


def test_exact_vs_fp64_oracle_1080p(cuda, orc, renderer, gpu_textures, host_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.sweep_uniforms(3, 1920, 1080)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 1920, 1080, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT)
    ref, rdep, _ = orc.march(u, host_textures, 1920, 1080, precision=64, rows=(1, 1080, 8))
    e = mm.metrics.frame_errors(rgba[1::8], ref, dep[1::8], rdep)
    print("1080p exact vs fp64:", e)
    _gates(e)


def test_phase16_updates_one_pixel_in_16(cuda, renderer, gpu_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(200, 120)
    full, dfull = render(cuda, renderer, u, gpu_textures, 200, 120, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT)
    for phase in (0, 6, 15):
        u.sun.color[3] = float(phase)
        for schedule in (L.SCHEDULE_PERSISTENT, L.SCHEDULE_TILED):
            part, dpart = render(cuda, renderer, u, gpu_textures, 200, 120, pixel_mode=L.PIXELS_PHASE16,
                                 sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT, schedule=schedule)
            m = np.zeros((120, 200), bool)
            m[phase // 4::4, phase % 4::4] = True
            assert np.array_equal(part[m], full[m]) and np.all(part[~m] == 0)


def test_reference_uv_mode(cuda, orc, renderer, gpu_textures, host_textures):
    # uv = pixel / (1920, 1080) as the shader hard-codes (compute-clouds.comp:283-285, 305).
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(320, 180)
    rgba, _ = render(cuda, renderer, u, gpu_textures, 320, 180, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT,
                     ref_uv_1080p=1)
    ref, _, _ = orc.march(u, host_textures, 320, 180, precision=32, ref_uv_1080p=1)
    assert np.array_equal(rgba, ref)


@pytest.mark.parametrize("mode", ["exact", "fast_software", "fast"])
def test_vs_reference_shader_golden(cuda, orc, renderer, gpu_textures, mode):
    # compute-clouds.comp itself, compiled as C++ on the CPU (tests/golden/shader_clouds_1080p.npz):
    # the exact kernel within 2e-4 relative on every pixel (it equals the FP32 restatement bit for
    # bit, which the CPU tests hold to that bound); the production kernels within the FP64 gates.
    import marshmallow as mm
    import marshmallow.lib as L
    import shader_golden as sg
    opts = {"exact": dict(sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT), "fast_software": dict(sampler=L.SAMPLER_SOFTWARE),
            "fast": {}}[mode]
    night = mm.render.Textures.from_arrays({"night_sky": sg.night_sky(orc)})
    handles = dict(gpu_textures.handles)
    handles["night_sky"] = night.handles["night_sky"]
    tex = mm.render.Textures(handles=handles)
    for name, u, rows, cols, ref in sg.frames():
        rgba, _ = render(cuda, renderer, u, tex, 1920, 1080, depth=False, pixel_mode=L.PIXELS_PHASE16, ref_uv_1080p=1,
                         **opts)
        got = rgba[rows][:, cols]
        if mode == "exact":
            assert sg.max_rel(got, ref) <= 2e-4, name
        else:
            e = mm.metrics.frame_errors(got, ref)
            print(mode, name, e)
            assert e["nan"] == 0 and e["rmse_255"] <= 1.0 and e["p999_255"] <= 4.0, (name, e)
            assert e["frac_over_4"] <= 0.002, (name, e)
    night.close()


def test_exact_equals_reference_shader_with_the_same_elementary_functions(cuda, orc, renderer, gpu_textures):
    # The reference shader built with mm_math.h's elementary functions, five frames, every 8th pixel of
    # the phase: the exact kernel's rgba has the same SHA-256 (tests/golden/shader_clouds_mm.json).
    import marshmallow as mm
    import marshmallow.lib as L
    import shader_golden as sg
    night = mm.render.Textures.from_arrays({"night_sky": sg.night_sky(orc)})
    handles = dict(gpu_textures.handles)
    handles["night_sky"] = night.handles["night_sky"]
    tex = mm.render.Textures(handles=handles)
    for name, u, rows, cols, sha in sg.mm_frames():
        rgba, _ = render(cuda, renderer, u, tex, 1920, 1080, depth=False, pixel_mode=L.PIXELS_PHASE16, ref_uv_1080p=1,
                         sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT)
        assert sg.digest(np.ascontiguousarray(rgba[rows][:, cols], np.float32)) == sha, name
    night.close()


def test_coverage_offset_and_sun_sweep(cuda, orc, renderer, gpu_textures, host_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    for el, off in ((5.0, -0.2), (60.0, 0.2), (85.0, 0.0)):
        u = mm.scene.uniforms(128, 96, sun_elevation=el)
        rgba, dep = render(cuda, renderer, u, gpu_textures, 128, 96, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT,
                           coverage_offset=off)
        ref, rdep, _ = orc.march(u, host_textures, 128, 96, precision=32, coverage_offset=off)
        assert np.array_equal(rgba, ref) and np.array_equal(dep, rdep)


def test_night_branch(cuda, orc, renderer, gpu_textures, host_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    night = np.random.default_rng(0).integers(0, 256, (90, 160, 4), dtype=np.uint8)
    nt = mm.render.Textures.from_arrays({"night_sky": night})
    handles = dict(gpu_textures.handles)
    handles["night_sky"] = nt.handles["night_sky"]
    tex = mm.render.Textures(handles=handles)
    h = dict(host_textures)
    h["night_sky"] = night
    # 96x64: the team march; 720x400 (288,000 rays): the full-frame kernel with pooled sun cones
    for w, hh in ((96, 64), (720, 400)):
        u = mm.scene.uniforms(w, hh, sun_elevation=-12.0)
        rgba, dep = render(cuda, renderer, u, tex, w, hh, sampler=L.SAMPLER_SOFTWARE, math=L.MATH_EXACT)
        ref, rdep, _ = orc.march(u, h, w, hh, precision=32)
        assert np.array_equal(rgba, ref), (w, hh)
        assert np.array_equal(dep.view(np.uint32), rdep.view(np.uint32)), (w, hh)
    nt.close()


def test_march_rejects_bad_arguments(cuda, mmlib, renderer, gpu_textures):
    import ctypes as C
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(64, 64)
    rgba = cuda.zeros((64, 64, 4), dtype=cuda.float32, device="cuda")
    st = gpu_textures.scene()
    o = mm.render.Renderer.options()
    img = L.Image(rgba.data_ptr(), 8, None, 0, 64, 64)  # pitch too small
    assert mmlib.mm_clouds_march(renderer.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None) == 1
    img = L.Image(rgba.data_ptr(), 64 * 16, None, 0, 64, 64)
    bad = L.SceneTextures(st.weather, None, None, st.low_res, st.hi_res)
    assert mmlib.mm_clouds_march(renderer.ctx, C.byref(u), C.byref(bad), C.byref(img), C.byref(o), None) == 1
    assert b"curl" in mmlib.mm_last_error_string()
    un = mm.scene.uniforms(64, 64, sun_elevation=-5.0)
    assert mmlib.mm_clouds_march(renderer.ctx, C.byref(un), C.byref(st), C.byref(img), C.byref(o), None) == 1
    o.math = 7
    assert mmlib.mm_clouds_march(renderer.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None) == 1
    o = mm.render.Renderer.options(pixel_mode=L.PIXELS_PHASE16)
    u.sun.color[3] = 16.0
    assert mmlib.mm_clouds_march(renderer.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None) == 1
    cuda.cuda.synchronize()


# ------------------------------------------------------------------------------ hardware filtering
#
# The production march reads its textures through the texture unit, whose LINEAR filter uses 8-bit
# fixed-point weights.  The oracle run with the same filter (oracle_frame.filter = 1, pinned fetch
# by fetch against the hardware in test_gpu_sampler.py) is the FP32 march the GPU computes:
#  - exact arithmetic + texture units equals it bit for bit (colour, depth, work counters);
#  - production arithmetic (FMA contraction, SFU square roots, algebraically equal forms) against it:
#    RMSE <= 1/255 as stated; colour within 4/255 and depth within 1e-3 relative on every pixel
#    except those where one of the shader's hard thresholds (density > 0 at :426, < 1e-4 at
#    :243/:437, accumulated > 0.99 at :476) falls the other way.  Such a pixel takes a different
#    path, and the reference's own FP32 arithmetic has the same kind of pixel against FP64: the FP32
#    oracle against the FP64 oracle, both with the texture unit's filter, on the same pixels.  The
#    gate is that production's tail against FP32 is no larger than FP32's own tail against FP64
#    (summed over the frames of a test), and at most 1e-4 of the pixels of any frame.


def _tail(e):
    return e["frac_over_4"], e["depth_frac_over_1e3"] + e["depth_finite_mismatch"]


def _tail_gates(errs_prod, errs_ref):
    """errs_prod: production vs FP32-TU oracle; errs_ref: FP32-TU vs FP64-TU oracle; per frame."""
    for e in errs_prod:
        assert e["nan"] == 0
        assert e["rmse_255"] <= 1.0, e
        assert e["frac_over_4"] <= 1e-4, e
    pc = sum(_tail(e)[0] for e in errs_prod)
    pd = sum(_tail(e)[1] for e in errs_prod)
    rc = sum(_tail(e)[0] for e in errs_ref)
    rd = sum(_tail(e)[1] for e in errs_ref)
    print("colour tail (pixels > 4/255): production vs FP32 %.2e, FP32 vs FP64 %.2e; depth tail (> 1e-3): "
          "production vs FP32 %.2e, FP32 vs FP64 %.2e (sums of per-frame fractions)" % (pc, rc, pd, rd))
    assert pc <= rc, (pc, rc)
    assert pd <= rd, (pd, rd)


@pytest.mark.parametrize("frame", [0, 7, 15])
def test_exact_hardware_bit_exact_vs_oracle_texture_unit(cuda, orc, renderer, gpu_textures, host_textures, frame):
    # Exact arithmetic with the texture units equals the FP32 oracle with the texture unit's filter.
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.sweep_uniforms(frame, 1920, 1080)
    rgba, dep = render(cuda, renderer, u, gpu_textures, 1920, 1080, sampler=L.SAMPLER_HARDWARE, math=L.MATH_EXACT)
    ref, rdep, _ = orc.march(u, host_textures, 1920, 1080, precision=32, rows=(frame, 1080, 24),
                             filter=orc.FILTER_TEXTURE_UNIT)
    assert np.array_equal(rgba[frame::24].view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(dep[frame::24].view(np.uint32), rdep.view(np.uint32))


def test_exact_hardware_counters_vs_oracle_texture_unit_256(cuda, orc, renderer, gpu_textures, host_textures):
    import marshmallow as mm
    import marshmallow.lib as L
    u = mm.scene.uniforms(256, 256)
    rgba, dep, cnt = render_counted(cuda, renderer, u, gpu_textures, 256, 256, sampler=L.SAMPLER_HARDWARE,
                                    math=L.MATH_EXACT)
    ref, rdep, rcnt = orc.march(u, host_textures, 256, 256, precision=32, filter=orc.FILTER_TEXTURE_UNIT)
    assert np.array_equal(rgba.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(dep.view(np.uint32), rdep.view(np.uint32))
    assert np.array_equal(cnt, rcnt)


def _prod_and_ref_errors(cuda, orc, renderer, gpu_textures, host_textures, u, w, h, r0, step, **opts):
    import marshmallow as mm
    rgba, dep = render(cuda, renderer, u, gpu_textures, w, h, **opts)
    off = opts.get("coverage_offset", 0.0)
    kw = dict(coverage_offset=off, rows=(r0, h, step), col_begin=r0, col_step=step, filter=orc.FILTER_TEXTURE_UNIT)
    f32, d32, _ = orc.march(u, host_textures, w, h, precision=32, **kw)
    f64, d64, _ = orc.march(u, host_textures, w, h, precision=64, **kw)
    ep = mm.metrics.frame_errors(rgba[r0::step, r0::step], f32, dep[r0::step, r0::step], d32)
    er = mm.metrics.frame_errors(f32, f64, d32, d64)
    return ep, er


def test_production_vs_oracle_texture_unit_1080p_sweep(cuda, orc, renderer, gpu_textures, host_textures):
    # The benchmark's configuration (fast arithmetic, texture units) over the whole 16-frame sweep,
    # every 2nd row and column.
    import marshmallow as mm
    prod, ref = [], []
    for frame in range(16):
        u = mm.scene.sweep_uniforms(frame, 1920, 1080)
        ep, er = _prod_and_ref_errors(cuda, orc, renderer, gpu_textures, host_textures, u, 1920, 1080, frame % 2, 2)
        prod.append(ep)
        ref.append(er)
        print("frame %2d production vs FP32: rmse %.3f max %.2f >4: %.1e depth>1e-3 %.1e | FP32 vs FP64: rmse %.3f "
              "max %.2f >4: %.1e depth>1e-3 %.1e" % (frame, ep["rmse_255"], ep["max_255"], ep["frac_over_4"],
                                                     ep["depth_frac_over_1e3"], er["rmse_255"], er["max_255"],
                                                     er["frac_over_4"], er["depth_frac_over_1e3"]))
    _tail_gates(prod, ref)


def test_production_vs_oracle_texture_unit_4k_sun_coverage_sweep(cuda, orc, renderer, gpu_textures, host_textures):
    # 3840x2160, sun elevation {5, 30, 60, 85} x coverage offset {-0.2, 0, +0.2}, every 8th row and column.
    import marshmallow as mm
    prod, ref = [], []
    for el in (5.0, 30.0, 60.0, 85.0):
        for off in (-0.2, 0.0, 0.2):
            p = mm.scene.sweep_params(0)
            u = mm.scene.uniforms(3840, 2160, yaw=p["yaw"], pitch=p["pitch"], time=p["time"], sun_elevation=el)
            ep, er = _prod_and_ref_errors(cuda, orc, renderer, gpu_textures, host_textures, u, 3840, 2160, 3, 8,
                                          coverage_offset=off)
            prod.append(ep)
            ref.append(er)
            print("sun %4.1f cov %+.1f production vs FP32: rmse %.3f max %.2f >4: %.1e depth>1e-3 %.1e | FP32 vs "
                  "FP64: rmse %.3f max %.2f >4: %.1e depth>1e-3 %.1e"
                  % (el, off, ep["rmse_255"], ep["max_255"], ep["frac_over_4"], ep["depth_frac_over_1e3"],
                     er["rmse_255"], er["max_255"], er["frac_over_4"], er["depth_frac_over_1e3"]))
    _tail_gates(prod, ref)
