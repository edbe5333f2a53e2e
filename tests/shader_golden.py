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
