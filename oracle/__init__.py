"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the CPU-baseline leg of bench.py
use it as the checker.  The library (project-marshmallow_gb300) never imports it.
"""
import ctypes as C
import os
import subprocess

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(ORACLE_DIR, "_build", "liboracle.so")

_lib = None


class OracleTexture(C.Structure):
    _fields_ = [("texels", C.c_void_p), ("width", C.c_int), ("height", C.c_int), ("depth", C.c_int),
                ("channels", C.c_int)]


class OracleTextures(C.Structure):
    _fields_ = [("weather", OracleTexture), ("night_sky", OracleTexture), ("curl", OracleTexture),
                ("low_res", OracleTexture), ("hi_res", OracleTexture)]


class OracleFrame(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("pixel_mode", C.c_int), ("coverage_offset", C.c_float),
                ("ref_uv_1080p", C.c_int), ("row_begin", C.c_int), ("row_end", C.c_int), ("row_step", C.c_int),
                ("col_begin", C.c_int), ("col_step", C.c_int), ("filter", C.c_int)]


def build():
    """Compiles liboracle.so with the committed Makefile (idempotent)."""
    subprocess.run(["make", "-s", "-C", ORACLE_DIR, "_build/liboracle.so"], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        lib.oracle_march_f32.argtypes = [C.c_void_p, C.POINTER(OracleTextures), C.POINTER(OracleFrame), C.c_void_p,
                                         C.c_void_p, C.c_void_p, C.c_int]
        lib.oracle_march_f64.argtypes = lib.oracle_march_f32.argtypes
        lib.oracle_ref_curl.argtypes = [C.c_void_p]
        lib.oracle_ref_curl_hash_index.argtypes = [C.c_float, C.c_float, C.c_float]
        lib.oracle_ref_curl_hash.argtypes = [C.c_float, C.c_float, C.c_float]
        lib.oracle_ref_curl_hash.restype = C.c_float
        lib.oracle_mm_math.argtypes = [C.c_int, C.c_float, C.c_float]
        lib.oracle_mm_math.restype = C.c_float
        lib.oracle_noise_fill.argtypes = [C.c_int, C.c_uint32, C.c_int, C.c_int, C.c_int, C.c_void_p]
        lib.oracle_hash32.argtypes = [C.c_uint32]
        lib.oracle_hash32.restype = C.c_uint32
        lib.oracle_hash3.argtypes = [C.c_int32, C.c_int32, C.c_int32, C.c_uint32]
        lib.oracle_hash3.restype = C.c_uint32
        lib.oracle_tonemap.argtypes = [C.c_void_p, C.c_size_t, C.c_void_p]
        lib.oracle_reproject_f32.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                             C.c_void_p]
        lib.oracle_shadow_f32.argtypes = [C.c_void_p, C.POINTER(OracleTextures), C.c_void_p, C.c_size_t, C.c_float,
                                          C.c_void_p, C.c_int]
        lib.oracle_shadow_f64.argtypes = lib.oracle_shadow_f32.argtypes
        lib.oracle_post_god_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p]
        lib.oracle_post_radial_blur.argtypes = lib.oracle_post_god_rays.argtypes
        lib.oracle_post_tonemap.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_int]
        lib.oracle_post_chain.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                                          C.c_size_t, C.c_int]
        lib.oracle_sample.argtypes = [C.POINTER(OracleTexture), C.c_int, C.c_void_p, C.c_size_t, C.c_int, C.c_void_p]
        lib.oracle_uniforms.argtypes = [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_float,
                                        C.c_float, C.c_float, C.c_int, C.c_void_p]
        _lib = lib
    return _lib


UNIFORM_FLOATS = 124  # the four std140 blocks of descriptor set 2, bindings 0-3 (496 bytes)


def uniforms(width, height, eye=(0.0, 10.0, 0.0), yaw=0.0, pitch=15.0, fov=60.0, sun_elevation=30.0,
             sun_azimuth=0.0, time=0.0, phase=0):
    """The uniform blocks of one frame, built by the oracle's own restatement of the reference's
    Camera and SkyManager (no CUDA library involved): a ctypes array of 124 floats in the std140
    layout the march reads."""
    u = (C.c_float * UNIFORM_FLOATS)()
    e = (C.c_float * 3)(*eye)
    rc = load().oracle_uniforms(e, yaw, pitch, fov, width, height, sun_elevation, sun_azimuth, time, phase,
                                C.addressof(u))
    if rc:
        raise ValueError("oracle_uniforms: invalid arguments")
    return u


def sweep_uniforms(k, width, height, n=16, sun_elevation=30.0, sun_azimuth=0.0):
    """Frame k of the camera sweep (yaw 0 -> 90 deg, pitch 5 -> 25 deg over n frames, t += 0.1 s)."""
    f = k / float(n - 1) if n > 1 else 0.0
    return uniforms(width, height, yaw=90.0 * f, pitch=5.0 + 20.0 * f, time=0.1 * k, sun_elevation=sun_elevation,
                    sun_azimuth=sun_azimuth)


def noise(kind, seed, w, h, d, channels):
    """Texels of a seeded generator as a (d, h, w, channels) uint8 array."""
    out = np.zeros((d, h, w, channels), np.uint8)
    rc = load().oracle_noise_fill(kind, seed, w, h, d, out.ctypes.data)
    if rc:
        raise RuntimeError("oracle_noise_fill failed: %d" % rc)
    return out


def ref_curl():
    out = np.zeros((128, 128, 4), np.uint8)
    rc = load().oracle_ref_curl(out.ctypes.data)
    if rc:
        raise RuntimeError("oracle_ref_curl failed: %d" % rc)
    return out


def _tex(a):
    if a is None:
        return OracleTexture(None, 0, 0, 0, 0)
    a = np.ascontiguousarray(a)
    if a.ndim == 3:  # 2D texture (h, w, c)
        return OracleTexture(a.ctypes.data, a.shape[1], a.shape[0], 1, a.shape[2])
    return OracleTexture(a.ctypes.data, a.shape[2], a.shape[1], a.shape[0], a.shape[3])


FILTER_EXACT, FILTER_TEXTURE_UNIT = 0, 1
# mm_noise_kind values of the seeded generators (include/mm.h)
NOISE_LOWRES, NOISE_HIRES, NOISE_CURL2D, NOISE_WEATHER = 0, 1, 2, 3


def seed_textures(seed=0):
    """The four seeded textures of the benchmark scene from the oracle's own generators."""
    return {"low_res": noise(NOISE_LOWRES, seed, 128, 128, 128, 4), "hi_res": noise(NOISE_HIRES, seed, 32, 32, 32, 4),
            "curl": noise(NOISE_CURL2D, seed, 128, 128, 1, 2)[0], "weather": noise(NOISE_WEATHER, seed, 512, 512, 1, 4)[0]}


def march(uniforms, textures, width, height, precision=32, pixel_mode=0, coverage_offset=0.0, ref_uv_1080p=0,
          rows=None, col_begin=0, col_step=1, nthreads=0, filter=FILTER_EXACT):
    """Runs the oracle march over a pixel sample.

    textures: dict with weather (h,w,4), curl (h,w,2|4), low_res (d,h,w,4), hi_res (d,h,w,4), night_sky (opt).
    rows: (begin, end, step) or None for all rows.  Returns (rgba (n_rows, n_cols, 4), depth (n_rows, n_cols),
    counters [cloudTest, cloudHiRes, iterations, accumulated]).
    """
    lib = load()
    keep = {k: np.ascontiguousarray(v) for k, v in textures.items() if v is not None}
    t = OracleTextures(_tex(keep.get("weather")), _tex(keep.get("night_sky")), _tex(keep.get("curl")),
                       _tex(keep.get("low_res")), _tex(keep.get("hi_res")))
    rb, re_, rs = rows if rows else (0, height, 1)
    f = OracleFrame(width, height, pixel_mode, coverage_offset, ref_uv_1080p, rb, re_, rs, col_begin, col_step,
                    filter)
    n_rows = max(0, (re_ - rb + rs - 1) // rs)
    n_cols = max(0, (width - col_begin + col_step - 1) // col_step)
    rgba = np.zeros((n_rows, n_cols, 4), np.float32)
    depth = np.zeros((n_rows, n_cols), np.float32)
    cnt = np.zeros(4, np.uint64)
    fn = lib.oracle_march_f32 if precision == 32 else lib.oracle_march_f64
    rc = fn(C.addressof(uniforms), C.byref(t), C.byref(f), rgba.ctypes.data, depth.ctypes.data, cnt.ctypes.data,
            nthreads)
    if rc:
        raise RuntimeError("oracle march failed: %d" % rc)
    return rgba, depth, cnt


def sample(texels, coords, filter=FILTER_TEXTURE_UNIT):
    """The oracle's sampler on a UNORM8 texture ((h, w, c) or (d, h, w, c)) at float32 normalized
    coordinates (n, 2) or (n, 3): (n, 4) float32."""
    texels = np.ascontiguousarray(texels, np.uint8)
    coords = np.ascontiguousarray(coords, np.float32)
    out = np.zeros((coords.shape[0], 4), np.float32)
    t = _tex(texels)
    rc = load().oracle_sample(C.byref(t), coords.shape[1], coords.ctypes.data, coords.shape[0], filter,
                              out.ctypes.data)
    if rc:
        raise RuntimeError("oracle_sample failed: %d" % rc)
    return out


def _textures(textures):
    keep = {k: np.ascontiguousarray(v) for k, v in textures.items() if v is not None}
    t = OracleTextures(_tex(keep.get("weather")), _tex(keep.get("night_sky")), _tex(keep.get("curl")),
                       _tex(keep.get("low_res")), _tex(keep.get("hi_res")))
    return keep, t


REF_CLOUDS_LIB = os.path.join(ORACLE_DIR, "_ref", "libref_clouds.so")
_ref_clouds = None


def ref_clouds_available():
    """True where the reference's compute-clouds.comp has been compiled as C++ (`make -C oracle ref`)."""
    return os.path.exists(REF_CLOUDS_LIB)


def ref_clouds_mm_available():
    """True where its build with mm_math.h's elementary functions exists as well."""
    return os.path.exists(REF_CLOUDS_LIB.replace("libref_clouds.so", "libref_clouds_mm.so"))


def ref_clouds_march(uniforms, textures, xs, ys, nthreads=0, mm_math=False):
    """The reference shader itself (compiled from its GLSL on the CPU) at pixels (xs[i], ys[i]) of the
    1920 x 1080 frame it hard-codes; every pixel must be in the phase int(sun.color.a).  Returns rgba (n, 4).
    mm_math: the build whose exp/pow/acos/cos/sin are mm_math.h's (the restatement's), else the C library's."""
    global _ref_clouds
    if _ref_clouds is None:
        _ref_clouds = {}
    key = bool(mm_math)
    if key not in _ref_clouds:
        lib = C.CDLL(REF_CLOUDS_LIB.replace("libref_clouds.so", "libref_clouds_mm.so") if key else REF_CLOUDS_LIB)
        lib.ref_clouds_march.argtypes = [C.c_void_p, C.POINTER(OracleTextures), C.c_void_p, C.c_void_p, C.c_size_t,
                                         C.c_void_p, C.c_int]
        _ref_clouds[key] = lib
    lib = _ref_clouds[key]
    keep, t = _textures(textures)
    xs = np.ascontiguousarray(xs, np.int32)
    ys = np.ascontiguousarray(ys, np.int32)
    out = np.zeros((len(xs), 4), np.float32)
    rc = lib.ref_clouds_march(C.addressof(uniforms), C.byref(t), xs.ctypes.data, ys.ctypes.data, len(xs),
                              out.ctypes.data, nthreads)
    if rc:
        raise RuntimeError("ref_clouds_march failed: %d" % rc)
    return out


_ref_shaders = {}


def _ref_shader(name):
    """oracle/_ref/lib<name>.so: a reference shader compiled as C++ (`make -C oracle ref`), or None."""
    path = os.path.join(ORACLE_DIR, "_ref", "lib%s.so" % name)
    if name not in _ref_shaders:
        _ref_shaders[name] = C.CDLL(path) if os.path.exists(path) else None
    return _ref_shaders[name]


def ref_reproject_available():
    return _ref_shader("ref_reproject") is not None


def ref_reproject(uniforms, src_rgba, nthreads=0):
    """The reference's reproject.comp (compiled from its GLSL on the CPU) over a whole (h, w, 4) image."""
    lib = _ref_shader("ref_reproject")
    lib.ref_reproject.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]
    src = np.ascontiguousarray(src_rgba, np.float32)
    h, w = src.shape[:2]
    dst = np.zeros_like(src)
    rc = lib.ref_reproject(C.addressof(uniforms), src.ctypes.data, w, h, dst.ctypes.data, nthreads)
    if rc:
        raise RuntimeError("ref_reproject failed: %d" % rc)
    return dst


def ref_post_available(which):
    return _ref_shader("ref_" + which) is not None


def ref_post(which, uniforms, src, nthreads=0):
    """The reference's fragment shader (which = "god_ray" | "radial_blur" | "tonemap", compiled from its
    GLSL on the CPU) shading every pixel of a full-screen pass over the (h, w, 4) float32 image src.
    Returns outColor as (h, w, 4) float32 (the 8-bit conversion of the swapchain is left to the caller)."""
    lib = _ref_shader("ref_" + which)
    fn = getattr(lib, "ref_" + which)
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int]
    a = np.ascontiguousarray(src, np.float32)
    out = np.zeros_like(a)
    if fn(C.addressof(uniforms) if uniforms is not None else None, a.ctypes.data, a.shape[1], a.shape[0],
          out.ctypes.data, nthreads):
        raise RuntimeError("ref_%s failed" % which)
    return out


def ref_model_available():
    return _ref_shader("ref_model") is not None


def ref_model_shadow(uniforms, textures, world_pos, nthreads=0):
    """The cloud shadow of the reference's model.frag (compiled from its GLSL on the CPU) at world
    positions (n, 4): shades each fragment with and without clouds and returns accumDensity =
    (1 - shadowed / clear) / 2 from the brightest channel, NaN where the shadowed colour is clamped to 0
    (accumDensity >= 0.5; the shader keeps no more of it)."""
    lib = _ref_shader("ref_model")
    lib.ref_model_shade.argtypes = [C.c_void_p, C.POINTER(OracleTextures), C.c_void_p, C.c_size_t, C.c_void_p,
                                    C.c_void_p, C.c_int]
    keep, t = _textures(textures)
    wp = np.ascontiguousarray(world_pos, np.float32).reshape(-1, 4)
    n = wp.shape[0]
    shadowed = np.zeros((n, 3), np.float32)
    clear = np.zeros((n, 3), np.float32)
    if lib.ref_model_shade(C.addressof(uniforms), C.byref(t), wp.ctypes.data, n, shadowed.ctypes.data,
                           clear.ctypes.data, nthreads):
        raise RuntimeError("ref_model_shade failed")
    k = np.argmax(clear, axis=1)
    c0 = clear[np.arange(n), k].astype(np.float64)
    c = shadowed[np.arange(n), k].astype(np.float64)
    if np.any(c0 <= 0):
        raise RuntimeError("unlit fragment: the shadow cannot be recovered")
    a = (1.0 - c / c0) * 0.5
    a[c <= 0] = np.nan
    return a


def unorm8(x):
    """Float -> UNORM8 as the swapchain stores a colour: clamp to [0, 1], scale by 255 in float, round to
    nearest even."""
    v = np.clip(np.nan_to_num(np.asarray(x, np.float32), nan=0.0), np.float32(0), np.float32(1))
    return np.rint(v * np.float32(255)).astype(np.uint8)


def shadow(uniforms, textures, world_pos, precision=32, coverage_offset=0.0, nthreads=0):
    """model.frag's cloud-shadow march over a G-buffer of world positions (..., 4) -> shadow (...)."""
    lib = load()
    keep, t = _textures(textures)
    pos = np.ascontiguousarray(world_pos, np.float32)
    out = np.zeros(pos.shape[:-1], np.float32)
    nth = nthreads or os.cpu_count() or 1
    fn = lib.oracle_shadow_f32 if precision == 32 else lib.oracle_shadow_f64
    rc = fn(C.addressof(uniforms), C.byref(t), pos.ctypes.data, pos.size // 4, coverage_offset, out.ctypes.data, nth)
    if rc:
        raise RuntimeError("oracle shadow failed: %d" % rc)
    return out


def tonemap(rgba):
    """tonemap.frag's Uncharted-2 operator on an (..., 4) float array -> (..., 3)."""
    a = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros(a.shape[:-1] + (3,), np.float32)
    load().oracle_tonemap(a.ctypes.data, a.size // 4, out.ctypes.data)
    return out


def reproject(uniforms, src_rgba, src_depth=None):
    """reproject.comp over a frame: returns (rgba, depth) from the previous frame's images."""
    h, w = src_rgba.shape[:2]
    src = np.ascontiguousarray(src_rgba, np.float32)
    sd = np.ascontiguousarray(src_depth, np.float32) if src_depth is not None else None
    out = np.zeros_like(src)
    od = np.zeros((h, w), np.float32) if sd is not None else None
    rc = load().oracle_reproject_f32(C.addressof(uniforms), src.ctypes.data, sd.ctypes.data if sd is not None else None,
                                     w, h, out.ctypes.data, od.ctypes.data if od is not None else None)
    if rc:
        raise RuntimeError("oracle reproject failed: %d" % rc)
    return out, od


def post_pass(which, uniforms, src):
    """One post pass on an (h, w, 4) float32 image: which = "god_rays" | "radial_blur"."""
    a = np.ascontiguousarray(src, np.float32)
    out = np.zeros_like(a)
    fn = getattr(load(), "oracle_post_" + which)
    if fn(C.addressof(uniforms), a.ctypes.data, a.shape[1], a.shape[0], out.ctypes.data):
        raise RuntimeError("oracle post pass failed")
    return out


def post_tonemap(src, bgra=0):
    a = np.ascontiguousarray(src, np.float32)
    out = np.zeros(a.shape[:2] + (4,), np.uint8)
    if load().oracle_post_tonemap(a.ctypes.data, a.shape[1], a.shape[0], out.ctypes.data, a.shape[1] * 4, bgra):
        raise RuntimeError("oracle tonemap failed")
    return out


def post_chain(uniforms, clouds, mesh=None, bgra=0):
    """clouds (and the optional mesh layer) (h, w, 4) float32 -> (h, w, 4) uint8."""
    a = np.ascontiguousarray(clouds, np.float32)
    m = np.ascontiguousarray(mesh, np.float32) if mesh is not None else None
    out = np.zeros(a.shape[:2] + (4,), np.uint8)
    if load().oracle_post_chain(C.addressof(uniforms), a.ctypes.data, m.ctypes.data if m is not None else None,
                                a.shape[1], a.shape[0], out.ctypes.data, a.shape[1] * 4, bgra):
        raise RuntimeError("oracle post chain failed")
    return out
