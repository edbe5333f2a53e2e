"""mm_noise_fill_ref_curl_noalloc: the reference curl generator with no device allocation.

It serves callers that cannot allocate device memory when they generate: an engine that owns the
whole device heap, or a frame loop that must not touch the allocator.  It must write exactly what the allocating entry point (mm_noise_fill with
MM_NOISE_REF_CURL) writes, call after call, although every call reuses the same static scratch
array.  This file runs last so a failure here comes after every other test has run.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import noise_fill, stream_ptr

pytestmark = pytest.mark.gpu


def _noalloc(cuda, lib):
    out = cuda.zeros(128 * 128 * 4, dtype=cuda.uint8, device="cuda")
    rc = lib.mm_noise_fill_ref_curl_noalloc(0, 0, C.c_void_p(out.data_ptr()), out.numel(), stream_ptr(cuda))
    assert rc == 0, lib.mm_last_error_string()
    cuda.cuda.synchronize()
    return out.cpu().numpy().reshape(128, 128, 4)


def test_noalloc_matches_allocating_entry_point_twice(cuda, mmlib):
    import marshmallow.lib as L
    want = noise_fill(cuda, mmlib, L.NOISE_REF_CURL).reshape(128, 128, 4)
    golden = np.fromfile(os.path.join(GOLDEN, "curl_fbm_128.rgba"), np.uint8).reshape(128, 128, 4)
    first = _noalloc(cuda, mmlib)
    second = _noalloc(cuda, mmlib)  # same scratch, left over from the first call
    # Noise texels are compared at the library's noise tolerance: identical bytes.
    assert np.array_equal(first, want)
    assert np.array_equal(second, want)
    assert np.array_equal(second, golden)


def test_noalloc_rejects_sizes_beyond_its_scratch(cuda, mmlib):
    out = cuda.zeros(256 * 256 * 4, dtype=cuda.uint8, device="cuda")
    rc = mmlib.mm_noise_fill_ref_curl_noalloc(256, 256, C.c_void_p(out.data_ptr()), out.numel(), stream_ptr(cuda))
    assert rc == 1
    assert b"maximum" in mmlib.mm_last_error_string()
    rc = mmlib.mm_noise_fill_ref_curl_noalloc(128, 128, C.c_void_p(out.data_ptr()), 100, stream_ptr(cuda))
    assert rc == 1
