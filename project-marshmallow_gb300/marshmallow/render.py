"""Textures and frames over CUDA device memory for the library's callers in Python.

Device buffers are torch CUDA tensors (torch is only the allocator and stream provider here); all
work is done by libmm.so's kernels through the C ABI.
"""
import ctypes as C

import numpy as np

from . import lib as L

DEFAULT_SIZES = {
    "low_res": (L.NOISE_LOWRES, 128, 128, 128, 4),
    "hi_res": (L.NOISE_HIRES, 32, 32, 32, 4),
    "curl": (L.NOISE_CURL2D, 128, 128, 1, 2),
    "weather": (L.NOISE_WEATHER, 512, 512, 1, 4),
}


def _stream_ptr(stream):
    if stream is None:
        import torch
        return C.c_void_p(torch.cuda.current_stream().cuda_stream)
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


class Textures:
    """The four seeded cloud textures, generated on the GPU by mm_noise_generate."""

    def __init__(self, seed=0, stream=None, handles=None):
        lib = L.load()
        self.handles = {}
        self.seed = seed
        if handles is not None:
            self.handles = dict(handles)
            return
        s = _stream_ptr(stream)
        for name, (kind, w, h, d, _) in DEFAULT_SIZES.items():
            desc = L.NoiseDesc(kind, seed, w, h, d)
            hnd = C.c_void_p()
            L.check(lib.mm_noise_generate(C.byref(desc), C.byref(hnd), s), "mm_noise_generate(%s)" % name)
            self.handles[name] = hnd

    @classmethod
    def from_arrays(cls, arrays, stream=None, fmt=L.FORMAT_UNORM8):
        """Textures from host UNORM8 arrays: 2D (h, w, c) or 3D (d, h, w, c)."""
        lib = L.load()
        s = _stream_ptr(stream)
        handles = {}
        for name, a in arrays.items():
            if a is None:
                continue
            a = np.ascontiguousarray(a, np.uint8)
            if a.ndim == 3:
                d, (h, w, c) = 1, a.shape
            else:
                d, h, w, c = a.shape
            hnd = C.c_void_p()
            L.check(lib.mm_texture_create(a.ctypes.data, 0, w, h, d, c, fmt, C.byref(hnd), s), "mm_texture_create")
            handles[name] = hnd
        return cls(handles=handles)

    # The files VulkanApplication.cpp:253-262 loads, relative to the reference's Textures/ folder.
    ASSET_FILES = {
        "weather": ("file", "CloudPlacement.png"),
        "night_sky": ("file", "NightSky/nightSky_noOrange.png"),
        "curl": ("file", "CurlNoiseFBM.png"),
        "low_res": ("slices", "3DTextures/lowResCloudShape/lowResCloud", 128),
        "hi_res": ("slices", "3DTextures/hiResCloudShape/hiResClouds ", 32),
    }

    @classmethod
    def from_assets(cls, root, stream=None, fmt=L.FORMAT_UNORM8, files=None):
        """The shipped Nubis texture set (or `files`, same layout) loaded by mm_texture_load_file /
        mm_texture_load_slices from the folder `root`."""
        import os
        lib = L.load()
        s = _stream_ptr(stream)
        handles = {}
        for name, spec in (files or cls.ASSET_FILES).items():
            hnd = C.c_void_p()
            path = os.path.join(root, spec[1]).encode()
            if spec[0] == "file":
                L.check(lib.mm_texture_load_file(path, fmt, C.byref(hnd), s), "mm_texture_load_file(%s)" % name)
            else:
                L.check(lib.mm_texture_load_slices(path, spec[2], fmt, C.byref(hnd), s),
                        "mm_texture_load_slices(%s)" % name)
            handles[name] = hnd
        return cls(handles=handles)

    def host(self, name):
        lib = L.load()
        w, h, d, c, f = (C.c_int() for _ in range(5))
        hnd = self.handles[name]
        L.check(lib.mm_texture_info(hnd, C.byref(w), C.byref(h), C.byref(d), C.byref(c), C.byref(f)))
        shape = (h.value, w.value, c.value) if d.value == 1 else (d.value, h.value, w.value, c.value)
        out = np.zeros(shape, np.uint8)
        L.check(lib.mm_texture_copy_to_host(hnd, out.ctypes.data, out.nbytes), "mm_texture_copy_to_host")
        return out

    def host_all(self):
        return {k: self.host(k) for k in self.handles}

    def set_density_format(self, fmt, stream=None):
        lib = L.load()
        for k in ("low_res", "hi_res"):
            L.check(lib.mm_texture_set_format(self.handles[k], fmt, _stream_ptr(stream)), "mm_texture_set_format")

    def scene(self):
        g = self.handles.get
        return L.SceneTextures(g("weather"), g("night_sky"), g("curl"), g("low_res"), g("hi_res"))

    def close(self):
        lib = L.load()
        for h in self.handles.values():
            lib.mm_texture_destroy(h)
        self.handles = {}


class Renderer:
    """An mm_context plus the march call on torch-allocated frames."""

    def __init__(self):
        self.lib = L.load()
        self.ctx = C.c_void_p()
        L.check(self.lib.mm_context_create(C.byref(self.ctx)), "mm_context_create")

    @staticmethod
    def options(pixel_mode=L.PIXELS_FULL, sampler=L.SAMPLER_HARDWARE, math=L.MATH_FAST, density_format=L.FORMAT_UNORM8,
                coverage_offset=0.0, ref_uv_1080p=0, counters=None, schedule=L.SCHEDULE_TILED, surrogate=None):
        o = L.MarchOptions()
        L.load().mm_march_options_default(C.byref(o))
        o.pixel_mode, o.sampler, o.math, o.density_format = pixel_mode, sampler, math, density_format
        o.coverage_offset, o.ref_uv_1080p = coverage_offset, ref_uv_1080p
        o.d_counters = counters.data_ptr() if counters is not None else None
        o.schedule = schedule
        o.cone = L.CONE_SURROGATE if surrogate is not None else L.CONE_PLAIN
        o.surrogate = surrogate
        return o

    def march(self, u, textures, rgba, depth=None, stream=None, **opts):
        """rgba: (H, W, 4) float32 CUDA tensor; depth: (H, W) float32 CUDA tensor or None."""
        h, w = rgba.shape[0], rgba.shape[1]
        img = L.Image(rgba.data_ptr(), rgba.stride(0) * 4, depth.data_ptr() if depth is not None else None,
                      depth.stride(0) * 4 if depth is not None else 0, w, h)
        o = self.options(**opts)
        st = textures.scene() if isinstance(textures, Textures) else textures
        L.check(self.lib.mm_clouds_march(self.ctx, C.byref(u), C.byref(st), C.byref(img), C.byref(o),
                                         _stream_ptr(stream)), "mm_clouds_march")

    @staticmethod
    def image(rgba, depth=None):
        h, w = rgba.shape[0], rgba.shape[1]
        return L.Image(rgba.data_ptr(), rgba.stride(0) * 4, depth.data_ptr() if depth is not None else None,
                       depth.stride(0) * 4 if depth is not None else 0, w, h)

    def reproject(self, u, src, dst, stream=None, **opts):
        """src, dst: (rgba, depth) tensor pairs of the same size; opts: math=L.MATH_EXACT / MATH_FAST."""
        L.check(self.lib.mm_clouds_reproject(self.ctx, C.byref(u), C.byref(self.image(*src)), C.byref(self.image(*dst)),
                                             C.byref(self.options(**opts)), _stream_ptr(stream)), "mm_clouds_reproject")

    def frame(self, u, textures, prev, out, stream=None, **opts):
        o = self.options(**opts)
        st = textures.scene() if isinstance(textures, Textures) else textures
        L.check(self.lib.mm_clouds_frame(self.ctx, C.byref(u), C.byref(st), C.byref(self.image(*prev)),
                                         C.byref(self.image(*out)), C.byref(o), _stream_ptr(stream)), "mm_clouds_frame")

    def mesh_shadow(self, u, textures, world_pos, shadow=None, rgba=None, stream=None, **opts):
        """model.frag's cloud-shadow march over a G-buffer: world_pos (H, W, 4) float32 CUDA tensor;
        shadow (H, W) float32 and/or rgba (H, W, 4) float32 CUDA tensors receive the result."""
        o = self.options(**opts)
        st = textures.scene() if isinstance(textures, Textures) else textures
        h, w = world_pos.shape[:2]
        g = L.GBuffer(world_pos.data_ptr(), world_pos.stride(0) * 4, w, h)
        L.check(self.lib.mm_mesh_shadow(self.ctx, C.byref(u), C.byref(st), C.byref(g),
                                        shadow.data_ptr() if shadow is not None else None,
                                        shadow.stride(0) * 4 if shadow is not None else 0,
                                        rgba.data_ptr() if rgba is not None else None,
                                        rgba.stride(0) * 4 if rgba is not None else 0, C.byref(o),
                                        _stream_ptr(stream)), "mm_mesh_shadow")

    @staticmethod
    def post_options(math=L.MATH_FAST, bgra=1):
        return L.PostOptions(math, bgra)

    @staticmethod
    def _rgba_image(t):
        return L.Image(t.data_ptr(), t.stride(0) * 4, None, 0, t.shape[1], t.shape[0])

    def god_rays(self, u, src, dst, stream=None, **opts):
        L.check(self.lib.mm_post_god_rays(self.ctx, C.byref(u), C.byref(self._rgba_image(src)),
                                          C.byref(self._rgba_image(dst)), C.byref(self.post_options(**opts)),
                                          _stream_ptr(stream)), "mm_post_god_rays")

    def radial_blur(self, u, src, dst, stream=None, **opts):
        L.check(self.lib.mm_post_radial_blur(self.ctx, C.byref(u), C.byref(self._rgba_image(src)),
                                             C.byref(self._rgba_image(dst)), C.byref(self.post_options(**opts)),
                                             _stream_ptr(stream)), "mm_post_radial_blur")

    def tonemap(self, src, out8, stream=None, **opts):
        """src (H, W, 4) float32, out8 (H, W, 4) uint8 CUDA tensors."""
        L.check(self.lib.mm_post_tonemap(self.ctx, C.byref(self._rgba_image(src)), out8.data_ptr(), out8.stride(0),
                                         C.byref(self.post_options(**opts)), _stream_ptr(stream)), "mm_post_tonemap")

    def post_chain(self, u, clouds, out8, mesh=None, stream=None, **opts):
        m = C.byref(self._rgba_image(mesh)) if mesh is not None else None
        L.check(self.lib.mm_post_chain(self.ctx, C.byref(u), C.byref(self._rgba_image(clouds)), m, out8.data_ptr(),
                                       out8.stride(0), C.byref(self.post_options(**opts)), _stream_ptr(stream)),
                "mm_post_chain")

    def march_batch(self, views, textures, outputs, stream=None, warp_tile_w=8, tiles_per_grab=4, use_graph=1,
                    schedule=L.BATCH_GRAPH, density_format=L.FORMAT_UNORM8, surrogate=None):
        """views: (width, height, uniforms) triples; outputs: matching (rgba, depth) CUDA tensors;
        surrogate: a trained mm_mlp handle for the learned sun cone (graph schedule)."""
        arr = (L.View * len(views))()
        for i, ((w, h, u), (rgba, dep)) in enumerate(zip(views, outputs)):
            arr[i].u = u
            arr[i].out = L.Image(rgba.data_ptr(), rgba.stride(0) * 4, dep.data_ptr() if dep is not None else None,
                                 dep.stride(0) * 4 if dep is not None else 0, w, h)
            arr[i].coverage_offset = 0.0
        o = L.BatchOptions(warp_tile_w, tiles_per_grab, use_graph, schedule, density_format, surrogate)
        st = textures.scene() if isinstance(textures, Textures) else textures
        L.check(self.lib.mm_clouds_march_batch(self.ctx, arr, len(views), C.byref(st), C.byref(o), _stream_ptr(stream)),
                "mm_clouds_march_batch")
        return arr

    def autotune_batch(self, views_arr, n, textures, stream=None):
        st = textures.scene() if isinstance(textures, Textures) else textures
        best = L.BatchOptions()
        table = (C.c_float * 22)()
        L.check(self.lib.mm_batch_autotune(self.ctx, views_arr, n, C.byref(st), C.byref(best), table,
                                           _stream_ptr(stream)), "mm_batch_autotune")
        return best, list(table)

    def close(self):
        if self.ctx:
            self.lib.mm_context_destroy(self.ctx)
            self.ctx = C.c_void_p()
