"""ctypes binding of libmm.so (include/mm.h).

The structures mirror the C declarations field for field; `check_layout()` compares their sizes
with the std140 sizes the shader's uniform blocks have (compute-clouds.comp:12-41).  Loading the
library never falls back to anything else: a missing or unbuildable libmm.so raises.
"""
import ctypes as C
import os

from . import build as _build

MM_OK = 0
MM_ERR_INVALID_ARGUMENT = 1
MM_ERR_CUDA = 2
MM_ERR_OUT_OF_MEMORY = 3
MM_ERR_UNSUPPORTED = 4
MM_ERR_TIMEOUT = 5
MM_ERR_NO_DEVICE = 6

NOISE_LOWRES, NOISE_HIRES, NOISE_CURL2D, NOISE_WEATHER, NOISE_REF_CURL = range(5)
FORMAT_UNORM8, FORMAT_FP16, FORMAT_BF16 = range(3)
PIXELS_FULL, PIXELS_PHASE16 = range(2)
SAMPLER_HARDWARE, SAMPLER_SOFTWARE = range(2)
MATH_FAST, MATH_EXACT, MATH_FAST_HALF2 = range(3)
BATCH_PERSISTENT, BATCH_BLOCKS, BATCH_GRAPH = range(3)
SCHEDULE_TILED, SCHEDULE_PERSISTENT = range(2)
CONE_PLAIN, CONE_SURROGATE = range(2)

F16 = C.c_float * 16
F4 = C.c_float * 4
F3 = C.c_float * 3


class CameraUBO(C.Structure):
    _fields_ = [("view", F16), ("proj", F16), ("camera_position", F4), ("camera_params", F4)]


class CameraPrevUBO(C.Structure):
    _fields_ = [("view", F16), ("proj", F16), ("camera_position", F4)]


class SunUBO(C.Structure):
    _fields_ = [("location", F4), ("direction", F4), ("color", F4), ("direction_basis", F16),
                ("intensity", C.c_float), ("pad_", C.c_float * 3)]


class SkyUBO(C.Structure):
    _fields_ = [("beta_r", F4), ("beta_v", F4), ("wind", F4), ("mie_directional", C.c_float),
                ("pad_", C.c_float * 3)]


class Uniforms(C.Structure):
    _fields_ = [("camera", CameraUBO), ("camera_prev", CameraPrevUBO), ("sun", SunUBO), ("sky", SkyUBO)]

    def copy(self):
        u = Uniforms()
        C.memmove(C.byref(u), C.byref(self), C.sizeof(Uniforms))
        return u


class NoiseDesc(C.Structure):
    _fields_ = [("kind", C.c_int), ("seed", C.c_uint32), ("width", C.c_int), ("height", C.c_int),
                ("depth", C.c_int)]


class SceneTextures(C.Structure):
    _fields_ = [("weather", C.c_void_p), ("night_sky", C.c_void_p), ("curl", C.c_void_p),
                ("low_res", C.c_void_p), ("hi_res", C.c_void_p)]


class Image(C.Structure):
    _fields_ = [("rgba", C.c_void_p), ("rgba_pitch_bytes", C.c_size_t), ("depth", C.c_void_p),
                ("depth_pitch_bytes", C.c_size_t), ("width", C.c_int), ("height", C.c_int)]


class MarchOptions(C.Structure):
    _fields_ = [("pixel_mode", C.c_int), ("sampler", C.c_int), ("math", C.c_int),
                ("density_format", C.c_int), ("coverage_offset", C.c_float), ("ref_uv_1080p", C.c_int),
                ("d_counters", C.c_void_p), ("schedule", C.c_int), ("cone", C.c_int), ("surrogate", C.c_void_p)]


class GBuffer(C.Structure):
    _fields_ = [("world_pos", C.c_void_p), ("world_pos_pitch_bytes", C.c_size_t), ("width", C.c_int),
                ("height", C.c_int)]


class PostOptions(C.Structure):
    _fields_ = [("math", C.c_int), ("bgra", C.c_int)]


class View(C.Structure):
    _fields_ = [("u", Uniforms), ("out", Image), ("coverage_offset", C.c_float)]


class BatchOptions(C.Structure):
    _fields_ = [("warp_tile_w", C.c_int), ("tiles_per_grab", C.c_int), ("use_graph", C.c_int), ("schedule", C.c_int),
                ("density_format", C.c_int), ("surrogate", C.c_void_p)]


# Every function include/mm.h declares, with its ctypes signature.
SIGNATURES = {
    "mm_camera_from_angles": (C.c_int, [C.POINTER(C.c_float), C.c_float, C.c_float, C.c_float, C.c_int, C.c_int,
                                        C.POINTER(Uniforms)]),
    "mm_sky_from_sun_angles": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(Uniforms)]),
    "mm_sky_from_reference_fractions": (C.c_int, [C.c_float, C.c_float, C.c_float, C.c_int, C.POINTER(Uniforms)]),
    "mm_noise_generate": (C.c_int, [C.POINTER(NoiseDesc), C.POINTER(C.c_void_p), C.c_void_p]),
    "mm_noise_texel_bytes": (C.c_int, [C.POINTER(NoiseDesc), C.POINTER(C.c_size_t)]),
    "mm_noise_fill": (C.c_int, [C.POINTER(NoiseDesc), C.c_void_p, C.c_size_t, C.c_void_p]),
    "mm_noise_fill_ref_curl_noalloc": (C.c_int, [C.c_int, C.c_int, C.c_void_p, C.c_size_t, C.c_void_p]),
    "mm_noise_hash3": (C.c_int, [C.c_void_p, C.c_uint32, C.c_size_t, C.c_void_p, C.c_void_p]),
    "mm_ref_curl_hash": (C.c_int, [C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "mm_texture_create": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                    C.POINTER(C.c_void_p), C.c_void_p]),
    "mm_image_decode_file": (C.c_int, [C.c_char_p, C.POINTER(C.c_void_p), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "mm_image_free": (C.c_int, [C.c_void_p]),
    "mm_texture_load_file": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_void_p), C.c_void_p]),
    "mm_texture_load_slices": (C.c_int, [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_void_p), C.c_void_p]),
    "mm_texture_info": (C.c_int, [C.c_void_p] + [C.POINTER(C.c_int)] * 5),
    "mm_texture_copy_to_host": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t]),
    "mm_texture_set_format": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    "mm_texture_sample": (C.c_int, [C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_void_p]),
    "mm_texture_destroy": (C.c_int, [C.c_void_p]),
    "mm_march_options_default": (C.c_int, [C.POINTER(MarchOptions)]),
    "mm_context_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "mm_context_destroy": (C.c_int, [C.c_void_p]),
    "mm_clouds_march": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(SceneTextures), C.POINTER(Image),
                                  C.POINTER(MarchOptions), C.c_void_p]),
    "mm_clouds_reproject": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(Image), C.POINTER(Image),
                                      C.POINTER(MarchOptions), C.c_void_p]),
    "mm_clouds_frame": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(SceneTextures), C.POINTER(Image),
                                  C.POINTER(Image), C.POINTER(MarchOptions), C.c_void_p]),
    "mm_mesh_shadow": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(SceneTextures), C.POINTER(GBuffer),
                                 C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t, C.POINTER(MarchOptions),
                                 C.c_void_p]),
    "mm_post_options_default": (C.c_int, [C.POINTER(PostOptions)]),
    "mm_post_god_rays": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(Image), C.POINTER(Image),
                                   C.POINTER(PostOptions), C.c_void_p]),
    "mm_post_radial_blur": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(Image), C.POINTER(Image),
                                      C.POINTER(PostOptions), C.c_void_p]),
    "mm_post_tonemap": (C.c_int, [C.c_void_p, C.POINTER(Image), C.c_void_p, C.c_size_t, C.POINTER(PostOptions),
                                  C.c_void_p]),
    "mm_post_chain": (C.c_int, [C.c_void_p, C.POINTER(Uniforms), C.POINTER(Image), C.POINTER(Image), C.c_void_p,
                                C.c_size_t, C.POINTER(PostOptions), C.c_void_p]),
    "mm_batch_options_default": (C.c_int, [C.POINTER(BatchOptions)]),
    "mm_clouds_march_batch": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int, C.POINTER(SceneTextures),
                                        C.POINTER(BatchOptions), C.c_void_p]),
    "mm_batch_autotune": (C.c_int, [C.c_void_p, C.POINTER(View), C.c_int, C.POINTER(SceneTextures),
                                    C.POINTER(BatchOptions), C.c_void_p, C.c_void_p]),
    "mm_mlp_param_count": (C.c_int, []),
    "mm_mlp_create": (C.c_int, [C.c_uint32, C.POINTER(C.c_void_p)]),
    "mm_mlp_destroy": (C.c_int, [C.c_void_p]),
    "mm_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "mm_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    "mm_mlp_forward": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "mm_mlp_gradients": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_float),
                                   C.c_void_p]),
    "mm_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_float, C.c_void_p,
                               C.c_void_p]),
    "mm_surrogate_generate": (C.c_int, [C.c_uint32, C.c_int, C.c_int, C.c_float, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_int), C.c_void_p]),
    "mm_mlp_save": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mm_mlp_load": (C.c_int, [C.c_void_p, C.c_char_p]),
    "mm_last_error_string": (C.c_char_p, []),
    "mm_abi_version": (C.c_int, []),
    "mm_kernel_launch_count": (C.c_uint64, []),
    "mm_tc_gemm_check": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                   C.c_void_p]),
    "mm_tc_gemm_mn_check": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_void_p]),
    "mm_measure_peaks": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_double), C.c_void_p]),
    "mm_tc_wait_check": (C.c_int, [C.c_int, C.c_uint, C.c_void_p, C.c_void_p]),
}

_lib = None


class MMError(RuntimeError):
    def __init__(self, code, fn, msg):
        super().__init__("%s failed with status %d: %s" % (fn, code, msg))
        self.code = code


def load(build_if_missing=True):
    """Returns the loaded libmm.so (building it first if needed); raises if it cannot be had."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libmm.so is not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc, fn="mm call"):
    if rc != MM_OK:
        msg = load().mm_last_error_string()
        raise MMError(rc, fn, msg.decode() if msg else "")
    return rc


def check_layout():
    """Sizes of the uniform blocks: std140 sizes of compute-clouds.comp:12-41 (padded)."""
    return {"camera": C.sizeof(CameraUBO), "camera_prev": C.sizeof(CameraPrevUBO), "sun": C.sizeof(SunUBO),
            "sky": C.sizeof(SkyUBO), "uniforms": C.sizeof(Uniforms)}
