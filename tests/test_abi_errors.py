"""Every C ABI entry point rejects null or invalid arguments with a status code and a message, on a
machine without a GPU: no crash, no exception, nothing launched.  (The reference reports such
errors by throwing std::runtime_error; the library returns MM_ERR_* and keeps the message in
mm_last_error_string.)"""
import ctypes as C

import pytest

INV = 1  # MM_ERR_INVALID_ARGUMENT


@pytest.fixture(scope="module")
def lib(mmlib):
    return mmlib


def _calls(L):
    """(name, args) pairs that must each return MM_ERR_INVALID_ARGUMENT."""
    u = L.Uniforms()
    img = L.Image()
    st = L.SceneTextures()
    nd = L.NoiseDesc(99, 0, 0, 0, 0)  # unknown kind
    h = C.c_void_p()
    o = L.MarchOptions()
    po = L.PostOptions()
    bo = L.BatchOptions()
    g = L.GBuffer()
    f = C.c_float()
    n = C.c_size_t()
    i = C.c_int()
    return [
        ("mm_camera_from_angles", (None, 0.0, 15.0, 60.0, 64, 64, C.byref(u))),
        ("mm_camera_from_angles", ((C.c_float * 3)(0, 10, 0), 0.0, 15.0, 60.0, 0, 64, C.byref(u))),
        ("mm_sky_from_sun_angles", (30.0, 0.0, 0.0, 0, None)),
        ("mm_sky_from_reference_fractions", (0.1, 0.25, 0.0, 0, None)),
        ("mm_noise_generate", (None, C.byref(h), None)),
        ("mm_noise_generate", (C.byref(nd), C.byref(h), None)),
        ("mm_noise_texel_bytes", (C.byref(nd), C.byref(n))),
        ("mm_noise_texel_bytes", (None, C.byref(n))),
        ("mm_noise_fill", (None, None, 0, None)),
        ("mm_noise_fill_ref_curl_noalloc", (128, 128, None, 0, None)),
        ("mm_texture_create", (None, 0, 4, 4, 1, 4, 0, C.byref(h), None)),
        ("mm_image_decode_file", (b"/nonexistent/x.png", C.byref(C.c_void_p()), C.byref(i), C.byref(i))),
        ("mm_image_decode_file", (b"x", None, C.byref(i), C.byref(i))),
        ("mm_texture_load_file", (b"/nonexistent/x.tga", 0, C.byref(h), None)),
        ("mm_texture_load_slices", (b"/nonexistent/s", 0, 0, C.byref(h), None)),
        ("mm_texture_info", (None, C.byref(i), C.byref(i), C.byref(i), C.byref(i), C.byref(i))),
        ("mm_texture_copy_to_host", (None, None, 0)),
        ("mm_texture_set_format", (None, 0, None)),
        ("mm_texture_sample", (None, None, 4, None, None)),
        ("mm_texture_destroy", (None,)),
        ("mm_march_options_default", (None,)),
        ("mm_context_create", (None,)),
        ("mm_context_destroy", (None,)),
        ("mm_clouds_march", (None, C.byref(u), C.byref(st), C.byref(img), C.byref(o), None)),
        ("mm_clouds_reproject", (None, C.byref(u), C.byref(img), C.byref(img), None, None)),
        ("mm_clouds_frame", (None, C.byref(u), C.byref(st), C.byref(img), C.byref(img), None, None)),
        ("mm_mesh_shadow", (None, C.byref(u), C.byref(st), C.byref(g), None, 0, None, 0, None, None)),
        ("mm_post_options_default", (None,)),
        ("mm_post_god_rays", (None, C.byref(u), C.byref(img), C.byref(img), C.byref(po), None)),
        ("mm_post_radial_blur", (None, C.byref(u), C.byref(img), C.byref(img), C.byref(po), None)),
        ("mm_post_tonemap", (None, C.byref(img), None, 0, C.byref(po), None)),
        ("mm_post_chain", (None, C.byref(u), C.byref(img), None, None, 0, C.byref(po), None)),
        ("mm_batch_options_default", (None,)),
        ("mm_clouds_march_batch", (None, None, 0, C.byref(st), C.byref(bo), None)),
        ("mm_batch_autotune", (None, None, 0, C.byref(st), None, None, None)),
        ("mm_mlp_create", (0, None)),
        ("mm_mlp_destroy", (None,)),
        ("mm_mlp_get_params", (None, None, 0)),
        ("mm_mlp_set_params", (None, None, 0)),
        ("mm_noise_hash3", (None, 0, 4, None, None)),
        ("mm_ref_curl_hash", (None, 4, None, None)),
        ("mm_measure_peaks", (None, None, None, None)),
        ("mm_mlp_forward", (None, None, 0, None, None)),
        ("mm_mlp_gradients", (None, None, None, 0, None, None, None)),
        ("mm_mlp_train", (None, None, None, 0, 0, 0, 0.0, C.byref(f), None)),
        ("mm_surrogate_generate", (1, 0, 0, 0.0, None, None, None, None)),
        ("mm_mlp_save", (None, b"/tmp/x")),
        ("mm_mlp_load", (None, b"/tmp/x")),
        ("mm_tc_wait_check", (0, 1024, None, None)),
        ("mm_tc_gemm_mn_check", (None, None, 128, 64, 1, 1, 1, None, None, None)),
        ("mm_tc_wait_check", (0, 0, C.byref(i), None)),
    ]


def test_invalid_arguments_are_rejected(lib):
    import marshmallow.lib as L
    seen = set()
    for name, args in _calls(L):
        rc = getattr(lib, name)(*args)
        assert rc == INV, (name, rc, lib.mm_last_error_string())
        assert lib.mm_last_error_string(), name
        seen.add(name)
    # every entry point that takes caller pointers is covered (the rest take none or only scalars)
    declared = set(L.SIGNATURES)
    scalar_only = {"mm_last_error_string", "mm_abi_version", "mm_kernel_launch_count", "mm_mlp_param_count",
                   "mm_image_free", "mm_tc_gemm_check"}
    assert declared - scalar_only - seen == set()


def test_no_launch_happened(lib):
    assert lib.mm_kernel_launch_count() >= 0
    before = lib.mm_kernel_launch_count()
    import marshmallow.lib as L
    for name, args in _calls(L):
        getattr(lib, name)(*args)
    assert lib.mm_kernel_launch_count() == before


def test_context_needs_a_device(lib):
    # Without a CUDA device the library says so instead of falling back to anything.
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_void_p()
    rc = lib.mm_context_create(C.byref(h))
    assert rc in (2, 6) and not h.value  # MM_ERR_CUDA or MM_ERR_NO_DEVICE
    assert lib.mm_last_error_string()
