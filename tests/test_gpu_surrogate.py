"""The learned sun-cone surrogate, end to end on the GPU.

Training data: 2^22 samples from the plain six-tap cone at random in-layer points and sun angles
over texture seeds 1-8 (mm_surrogate_generate); training: Adam on the tensor cores
(mm_mlp_train); evaluation: held-out samples of seed 0 and 3840x2160 frames of the seed-0 sweep.

What the test shows (printed, and bounded so regressions are caught):
  - training gain: held-out MSE of the predicted transmittance drops >= 8x from the untrained net;
  - frame error of the surrogate march vs the FP64 oracle and vs the plain march, and its time vs the
    plain march.  Measured on GB300: RMSE 2.0-3.4/255 (above the 2/255 gate of the method) and
    0.8-1.4 ms slower per 4K frame; the assertion only bounds it at 5/255 so a broken pipeline fails.
"""
import ctypes as C

import numpy as np
import pytest

from gpu_util import render, stream_ptr

pytestmark = pytest.mark.gpu
W, H = 3840, 2160


@pytest.fixture(scope="module")
def trained(cuda, mmlib):
    sp = stream_ptr(cuda)
    per_seed = 1 << 19
    X = cuda.empty((8 * per_seed, 16), dtype=cuda.bfloat16, device="cuda")
    T = cuda.empty(8 * per_seed, dtype=cuda.float32, device="cuda")
    n = C.c_int()
    assert mmlib.mm_surrogate_generate(1, 8, per_seed, 150000.0, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()),
                                       C.byref(n), sp) == 0, mmlib.mm_last_error_string()
    assert n.value == 8 * per_seed
    Xe = cuda.empty((1 << 17, 16), dtype=cuda.bfloat16, device="cuda")
    Te = cuda.empty(1 << 17, dtype=cuda.float32, device="cuda")
    ne = C.c_int()
    assert mmlib.mm_surrogate_generate(0, 1, 1 << 17, 150000.0, C.c_void_p(Xe.data_ptr()), C.c_void_p(Te.data_ptr()),
                                       C.byref(ne), sp) == 0
    h = C.c_void_p()
    assert mmlib.mm_mlp_create(11, C.byref(h)) == 0

    def held_out():
        y = cuda.empty(ne.value, device="cuda")
        assert mmlib.mm_mlp_forward(h, C.c_void_p(Xe.data_ptr()), ne.value, C.c_void_p(y.data_ptr()), sp) == 0
        cuda.cuda.synchronize()
        return float(((y - Te[:ne.value]) ** 2).mean())

    before = held_out()
    for lr, steps in ((8e-3, 128), (2.5e-3, 128)):
        assert mmlib.mm_mlp_train(h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()), n.value, 131072, steps, lr,
                                  None, sp) == 0, mmlib.mm_last_error_string()
    after = held_out()
    print("\nsurrogate held-out MSE: untrained %.5f -> trained %.5f (target variance %.5f)" %
          (before, after, float(Te[:ne.value].var())))
    yield h, before, after
    mmlib.mm_mlp_destroy(h)


def test_training_gain(trained):
    _, before, after = trained
    assert after * 8 < before


def test_surrogate_frames_vs_plain_and_oracle(cuda, mmlib, orc, trained):
    import marshmallow as mm
    h = trained[0]
    tex = mm.render.Textures(seed=0)
    r = mm.render.Renderer()
    host = tex.host_all()
    try:
        for frame in (0, 8):
            u = mm.scene.sweep_uniforms(frame, W, H)
            times = {}
            out = {}
            for name, kw in (("plain", {}), ("surrogate", {"surrogate": h.value})):
                rgba = cuda.zeros((H, W, 4), device="cuda")
                dep = cuda.zeros((H, W), device="cuda")
                r.march(u, tex, rgba, dep, **kw)
                cuda.cuda.synchronize()
                e0, e1 = cuda.cuda.Event(enable_timing=True), cuda.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(3):
                    r.march(u, tex, rgba, dep, **kw)
                e1.record()
                cuda.cuda.synchronize()
                times[name] = e0.elapsed_time(e1) / 3
                out[name] = (rgba.cpu().numpy(), dep.cpu().numpy())
            ref, rdep, _ = orc.march(u, host, W, H, precision=64, rows=(3, H, 8), col_begin=3, col_step=8)
            es = mm.metrics.frame_errors(out["surrogate"][0][3::8, 3::8], ref, out["surrogate"][1][3::8, 3::8], rdep)
            ep = mm.metrics.frame_errors(out["plain"][0][3::8, 3::8], ref)
            print("frame %d: plain %.3f ms rmse %.3f/255 | surrogate %.3f ms rmse %.3f/255 p99.9 %.2f/255" %
                  (frame, times["plain"], ep["rmse_255"], times["surrogate"], es["rmse_255"], es["p999_255"]))
            assert es["nan"] == 0
            assert es["rmse_255"] < 5.0
            # depth does not depend on the cone: the same as the plain march up to the contraction
            # choices of two separately compiled kernels
            assert np.mean(out["surrogate"][1] != out["plain"][1]) < 1e-3
    finally:
        r.close()
        tex.close()


def test_night_frames_fall_back_to_the_plain_cone(cuda, mmlib, trained):
    # Outside the training envelope (sun below the horizon) a surrogate request marches the plain
    # cone: the frame equals the plain march bit for bit.
    import marshmallow as mm
    import marshmallow.lib as L
    net = trained[0] if isinstance(trained, tuple) else trained
    w, h = 320, 180
    u = mm.scene.uniforms(w, h, yaw=30.0, pitch=12.0, sun_elevation=-6.0)
    rng = np.random.default_rng(3)
    night = rng.integers(0, 256, (64, 128, 4), dtype=np.uint8)
    tex = mm.render.Textures(seed=0)
    nt = mm.render.Textures.from_arrays({"night_sky": night})
    tex.handles["night_sky"] = nt.handles["night_sky"]
    r = mm.render.Renderer()
    try:
        a = cuda.zeros((h, w, 4), device="cuda")
        b = cuda.zeros((h, w, 4), device="cuda")
        r.march(u, tex, a, surrogate=net)
        r.march(u, tex, b)
        cuda.cuda.synchronize()
        assert cuda.equal(a, b)
    finally:
        r.close()
        del tex.handles["night_sky"]
        tex.close()
        nt.close()
