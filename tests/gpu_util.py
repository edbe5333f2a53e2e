"""Helpers for the GPU tests: device buffers via torch, library calls via ctypes."""
import ctypes as C

import numpy as np


def stream_ptr(torch):
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def noise_fill(torch, lib, kind, seed=0, w=0, h=0, d=0):
    import marshmallow.lib as L
    desc = L.NoiseDesc(kind, seed, w, h, d)
    n = C.c_size_t()
    L.check(lib.mm_noise_texel_bytes(C.byref(desc), C.byref(n)))
    buf = torch.empty(n.value, dtype=torch.uint8, device="cuda")
    L.check(lib.mm_noise_fill(C.byref(desc), C.c_void_p(buf.data_ptr()), n.value, stream_ptr(torch)), "mm_noise_fill")
    torch.cuda.synchronize()
    return buf.cpu().numpy()


def render(torch, renderer, u, textures, w, h, depth=True, **opts):
    rgba = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    dep = torch.zeros((h, w), dtype=torch.float32, device="cuda") if depth else None
    renderer.march(u, textures, rgba, dep, **opts)
    torch.cuda.synchronize()
    return rgba.cpu().numpy(), (dep.cpu().numpy() if depth else None)


def render_counted(torch, renderer, u, textures, w, h, **opts):
    cnt = torch.zeros(4, dtype=torch.int64, device="cuda")
    rgba, dep = render(torch, renderer, u, textures, w, h, counters=cnt, **opts)
    return rgba, dep, cnt.cpu().numpy().astype(np.uint64)
