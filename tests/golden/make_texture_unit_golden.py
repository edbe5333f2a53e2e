"""Records fetches of the GPU's texture unit for the CPU tests of the oracle's filter model.

Runs on a machine with a GB300 (the fixture is the hardware's output, not the oracle's):

    python tests/golden/make_texture_unit_golden.py

writes tests/golden/texture_unit_fetches.npz: for the four seed-0 textures and two random ones
(a 2D texture with sides that are not powers of two and a small 3D one), 2048 normalized
coordinates each (the march's ranges, plus a sweep across texel boundaries at the origin) and the
four filtered channels the texture unit returned for them (LINEAR, WRAP, normalized coordinates,
UNORM8 read as float: the reference samplers).  tests/test_oracle.py checks the oracle's
texture-unit filter against them bit for bit.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (REPO, os.path.join(REPO, "project-marshmallow_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

RANGES = {"weather": 12.0, "curl": 16.0, "low_res": 4.0, "hi_res": 64.0, "random_2d": 8.0, "random_3d": 8.0}


def coords(rng, dims, n, span, size):
    c = rng.uniform(-span, span, (n, dims)).astype(np.float32)
    m = n // 4
    f = np.arange(m) / m * 2.0
    c[:m, 0] = ((np.arange(m) % 2) + f / size).astype(np.float32)
    return c


def main():
    import torch
    import marshmallow as mm
    lib = mm.lib.load()
    rng = np.random.default_rng(2026)
    tex = mm.render.Textures(seed=0)
    textures = {k: tex.host(k) for k in ("weather", "curl", "low_res", "hi_res")}
    handles = dict(tex.handles)
    extra = {"random_2d": rng.integers(0, 256, (37, 53, 4), dtype=np.uint8),
             "random_3d": rng.integers(0, 256, (12, 20, 24, 4), dtype=np.uint8)}
    ex = mm.render.Textures.from_arrays(extra)
    textures.update(extra)
    handles.update(ex.handles)
    out = {}
    for name, texels in textures.items():
        dims = 3 if texels.ndim == 4 else 2
        c = coords(rng, dims, 2048, RANGES[name], texels.shape[-2])
        dc = torch.from_numpy(c).cuda()
        res = torch.empty((len(c), 4), dtype=torch.float32, device="cuda")
        rc = lib.mm_texture_sample(handles[name], C.c_void_p(dc.data_ptr()), len(c), C.c_void_p(res.data_ptr()),
                                   C.c_void_p(torch.cuda.current_stream().cuda_stream))
        assert rc == 0, lib.mm_last_error_string()
        torch.cuda.synchronize()
        out[name + "_coords"] = c
        out[name + "_fetched"] = res.cpu().numpy()
        if name.startswith("random"):
            out[name + "_texels"] = texels
    np.savez_compressed(os.path.join(HERE, "texture_unit_fetches.npz"), **out)
    tex.close()
    ex.close()


if __name__ == "__main__":
    main()
