"""The compute-clouds.comp golden fixture: rgba of the reference's own shader, compiled unchanged as
C++ on the CPU (tests/golden/make_golden.py), at every 32nd pixel of one 1/16 phase of its hard-coded
1920x1080 frame, for five frames on the seed-0 generator textures.  The night frame samples a seeded
night-sky map (weather generator, seed 3, 160x90)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "shader_clouds_1080p.npz")


def night_sky(orc):
    import marshmallow.lib as L
    return orc.noise(L.NOISE_WEATHER, 3, 160, 90, 1, 4)[0]


def frames():
    """[(name, uniforms, rows, cols, rgba (len(rows), len(cols), 4))]"""
    import marshmallow.lib as L
    z = np.load(GOLDEN)
    stride = int(z["stride"])
    out = []
    for name, ub, rgba in zip(z["names"], z["uniforms"], z["rgba"]):
        u = L.Uniforms.from_buffer_copy(ub.tobytes())
        phase = int(u.sun.color[3])
        rows = np.arange(phase // 4, 1080, stride)
        cols = np.arange(phase % 4, 1920, stride)
        assert rgba.shape == (len(rows), len(cols), 4)
        out.append((str(name), u, rows, cols, rgba))
    return out


def oracle_march(orc, u, textures, rows, cols, precision):
    """The CPU restatement at the golden pixels (reference UV mode, 1/16 phase mode)."""
    rgba, _, _ = orc.march(u, textures, 1920, 1080, precision=precision, pixel_mode=1, ref_uv_1080p=1,
                           rows=(int(rows[0]), 1080, int(rows[1] - rows[0])), col_begin=int(cols[0]),
                           col_step=int(cols[1] - cols[0]))
    return rgba


def max_rel(a, ref, floor=1e-3):
    """Largest per-channel error relative to max(|ref|, floor)."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return float((np.abs(a - ref) / np.maximum(np.abs(ref), floor)).max())


# ------------------------------------------------------------------------------------------------
# The other passes: reproject.comp, model.frag's cloud shadow, god-ray.frag, radialBlur.frag and
# tonemap.frag, compiled the same way (tests/golden/shader_passes.npz).

PASSES = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "shader_passes.npz")

# (width, height, yaw step, pitch step, eye offset) of the reprojection cases: the previous frame looks
# from yaw 20, pitch 10 at (0, 10, 0); the current one turns by the steps and moves by the offset.
REPROJECT_CASES = [(1920, 1080, 0.7, -0.4, (0.0, 50.0, 30.0)), (320, 180, -5.0, 2.0, (0.0, 50.0, 30.0)),
                   (333, 127, 10.0, 5.0, (0.0, 0.0, 0.0))]
POST_SIZE = (64, 36)
SHADOW_SIZE = (48, 27)


def pattern(h, w, seed, rgb_scale=20.0):
    """A seeded (h, w, 4) float32 image from an integer hash (the same bits on every machine): rgb in
    [0, rgb_scale), alpha in [0, 1)."""
    i = np.arange(h * w * 4, dtype=np.uint64).reshape(h, w, 4)
    x = (i * np.uint64(2654435761) + np.uint64(seed) * np.uint64(40503)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(2246822519)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(13)
    v = (x >> np.uint64(8)).astype(np.float32) * np.float32(1.0 / (1 << 24))
    return v * np.array([rgb_scale, rgb_scale, rgb_scale, 1.0], np.float32)


def reproject_uniforms(case):
    import ctypes as C
    import marshmallow as mm
    w, h, dyaw, dpitch, move = case
    prev = mm.scene.uniforms(w, h, yaw=20.0, pitch=10.0)
    cur = mm.scene.uniforms(w, h, eye=(move[0], 10.0 + move[1], move[2]), yaw=20.0 + dyaw, pitch=10.0 + dpitch)
    C.memmove(C.addressof(cur.camera_prev), C.addressof(prev.camera), C.sizeof(cur.camera_prev))
    return cur


def post_uniforms():
    import marshmallow as mm
    return mm.scene.uniforms(POST_SIZE[0], POST_SIZE[1], yaw=0.0, pitch=12.0, sun_elevation=20.0)


def digest(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def passes():
    z = np.load(PASSES)
    return {k: z[k] for k in z.files}


# The same frames from the shader built with mm_math.h's elementary functions: SHA-256 digests of the
# rgba of every 8th pixel of the phase (tests/golden/shader_clouds_mm.json), reproduced bit for bit by
# the FP32 restatement and the GPU's exact kernel.
MM_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "shader_clouds_mm.json")


def mm_frames():
    """[(name, uniforms, rows, cols, sha256)]"""
    import json
    import marshmallow.lib as L
    z = json.load(open(MM_GOLDEN))
    stride = int(z["stride"])
    out = []
    for fr in z["frames"]:
        u = L.Uniforms.from_buffer_copy(bytes.fromhex(fr["uniforms"]))
        phase = int(u.sun.color[3])
        out.append((fr["name"], u, np.arange(phase // 4, 1080, stride), np.arange(phase % 4, 1920, stride),
                    fr["sha256"]))
    return out
