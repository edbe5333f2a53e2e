"""GPU noise generators vs the CPU oracle: hash/index stage bit-exact, texels bit-exact (the gate
is <= 1 LSB), and the reference-compatible curl equal to the shipped CurlNoiseFBM.tga."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN
from gpu_util import noise_fill, stream_ptr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,seed,size,ch", [
    (0, 0, (128, 128, 128), 4), (1, 0, (32, 32, 32), 4), (2, 0, (128, 128, 1), 2), (3, 0, (512, 512, 1), 4),
    (0, 7, (64, 64, 64), 4), (1, 3, (48, 48, 48), 4), (2, 11, (96, 64, 1), 2), (3, 5, (256, 128, 1), 4)])
def test_noise_matches_oracle(cuda, mmlib, orc, kind, seed, size, ch):
    w, h, d = size
    got = noise_fill(cuda, mmlib, kind, seed, w, h, d).reshape(d, h, w, ch)
    want = orc.noise(kind, seed, w, h, d, ch)
    diff = np.abs(got.astype(int) - want.astype(int))
    assert diff.max() <= 1  # gate: 8-bit texels within 1 LSB
    assert np.array_equal(got, want)  # measured identical


def test_ref_curl_matches_shipped_texture(cuda, mmlib):
    got = noise_fill(cuda, mmlib, 4).reshape(128, 128, 4)
    golden = np.fromfile(os.path.join(GOLDEN, "curl_fbm_128.rgba"), np.uint8).reshape(128, 128, 4)
    assert np.array_equal(got, golden)


def test_hash_stage_bit_exact(cuda, mmlib, orc):
    lib = orc.load()
    rng = np.random.default_rng(1)
    xyz = rng.integers(-1 << 20, 1 << 20, (4096, 3)).astype(np.int32)
    seed = 0x9E3779B9
    d_in = cuda.from_numpy(xyz).cuda()
    d_out = cuda.zeros(4096, dtype=cuda.int32, device="cuda")
    assert mmlib.mm_noise_hash3(C.c_void_p(d_in.data_ptr()), seed, 4096, C.c_void_p(d_out.data_ptr()),
                                stream_ptr(cuda)) == 0
    got = d_out.cpu().numpy().view(np.uint32)
    want = np.array([lib.oracle_hash3(int(a), int(b), int(c), seed) for a, b, c in xyz], np.uint32)
    assert np.array_equal(got, want)
    # Reference curl hash (ImageUtils.cpp:25) on the lattice points its generator visits.
    pts = np.array([(x, y, z) for x in range(-1, 26) for y in range(-1, 26) for z in range(-1, 26, 2)], np.float32)
    d_p = cuda.from_numpy(pts).cuda()
    d_h = cuda.zeros(len(pts), dtype=cuda.float32, device="cuda")
    assert mmlib.mm_ref_curl_hash(C.c_void_p(d_p.data_ptr()), len(pts), C.c_void_p(d_h.data_ptr()),
                                  stream_ptr(cuda)) == 0
    got = d_h.cpu().numpy()
    want = np.array([lib.oracle_ref_curl_hash(*map(float, p)) for p in pts], np.float32)
    assert np.array_equal(got, want)


def test_generate_handles(cuda, mmlib, orc):
    import marshmallow as mm
    t = mm.render.Textures(seed=0)
    try:
        assert np.array_equal(t.host("hi_res"), orc.noise(1, 0, 32, 32, 32, 4))
        assert np.array_equal(t.host("curl"), orc.noise(2, 0, 128, 128, 1, 2)[0])
    finally:
        t.close()


def test_noise_rejects_bad_requests(cuda, mmlib):
    import marshmallow.lib as L
    buf = cuda.empty(16, dtype=cuda.uint8, device="cuda")
    desc = L.NoiseDesc(L.NOISE_LOWRES, 0, 0, 0, 0)
    assert mmlib.mm_noise_fill(C.byref(desc), C.c_void_p(buf.data_ptr()), 16, stream_ptr(cuda)) == 1
    desc = L.NoiseDesc(L.NOISE_HIRES, 0, 1024, 1024, 1024)
    assert mmlib.mm_noise_fill(C.byref(desc), C.c_void_p(buf.data_ptr()), 1 << 32, stream_ptr(cuda)) == 1
