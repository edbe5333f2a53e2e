"""Tensor-core MLP kernels vs the CPU reference (tests/mlp_ref.py): forward outputs, parameter
gradients (the gradient check), training, checkpoints."""
import ctypes as C
import os

import numpy as np
import pytest

import mlp_ref
from gpu_util import stream_ptr

pytestmark = pytest.mark.gpu


def _mlp(lib, seed=1):
    h = C.c_void_p()
    assert lib.mm_mlp_create(seed, C.byref(h)) == 0, lib.mm_last_error_string()
    return h


def _params(lib, h):
    n = lib.mm_mlp_param_count()
    p = np.zeros(n, np.float32)
    assert lib.mm_mlp_get_params(h, p.ctypes.data, n) == 0
    return p


def _bf16_tensor(cuda, x):
    return cuda.from_numpy(np.ascontiguousarray(x, np.float32)).to(cuda.bfloat16).cuda()


def test_tc_gemm_layout(cuda, mmlib):
    cuda.manual_seed(0)
    for K, N in ((16, 64), (64, 64), (128, 80), (128, 32)):
        A = (cuda.randn(128, K) * 0.5).to(cuda.bfloat16)
        B = (cuda.randn(N, K) * 0.5).to(cuda.bfloat16)
        out = cuda.zeros(128, N, device="cuda")
        st = cuda.zeros(1, dtype=cuda.int32, device="cuda")
        dA, dB = A.cuda(), B.cuda()
        assert mmlib.mm_tc_gemm_check(C.c_void_p(dA.data_ptr()), C.c_void_p(dB.data_ptr()), K, N, 0,
                                      C.c_void_p(out.data_ptr()), C.c_void_p(st.data_ptr()), None) == 0
        cuda.cuda.synchronize()
        ref = A.float() @ B.float().T
        assert st.item() == 0
        assert (out.cpu() - ref).abs().max().item() < 1e-4


@pytest.mark.parametrize("a_mn,b_mn,K,N", [(1, 0, 128, 80), (0, 1, 128, 80), (1, 1, 128, 32), (0, 1, 64, 64),
                                            (1, 1, 128, 128)])
def test_tensor_core_gemm_mn_major_operands(cuda, mmlib, a_mn, b_mn, K, N):
    # Operands read MN-major from a [K][MN] tile (the training kernel's in-place transposes), with
    # the K-group stride in the descriptor's leading-byte-offset field.
    torch = cuda
    A = (torch.randn(128, K) * 0.5).to(torch.bfloat16)
    B = (torch.randn(N, K) * 0.5).to(torch.bfloat16)
    dA = (A.T.contiguous() if a_mn else A).cuda()
    dB = (B.T.contiguous() if b_mn else B).cuda()
    ref = A.float() @ B.float().T
    errs = {}
    for lbo_k in (1, 0):
        out = torch.zeros(128, N, device="cuda")
        st = torch.zeros(1, dtype=torch.int32, device="cuda")
        assert mmlib.mm_tc_gemm_mn_check(C.c_void_p(dA.data_ptr()), C.c_void_p(dB.data_ptr()), K, N, a_mn, b_mn,
                                         lbo_k, C.c_void_p(out.data_ptr()), C.c_void_p(st.data_ptr()), None) == 0
        torch.cuda.synchronize()
        assert st.item() == 0
        errs[lbo_k] = (out.cpu() - ref).abs().max().item()
    print("MN-major a=%d b=%d K=%d N=%d: max error, K stride in LBO %.2e, in SBO %.2e" % (a_mn, b_mn, K, N, errs[1],
                                                                                          errs[0]))
    assert errs[1] < 1e-4


def test_forward_matches_reference(cuda, mmlib):
    h = _mlp(mmlib, 3)
    try:
        p = _params(mmlib, h)
        rng = np.random.default_rng(1)
        x = rng.normal(0, 1, (1000, 16)).astype(np.float32)
        dx = _bf16_tensor(cuda, x)
        y = cuda.zeros(1000, device="cuda")
        assert mmlib.mm_mlp_forward(h, C.c_void_p(dx.data_ptr()), 1000, C.c_void_p(y.data_ptr()), stream_ptr(cuda)) == 0
        cuda.cuda.synchronize()
        ref, _ = mlp_ref.forward(p, x)
        assert np.max(np.abs(y.cpu().numpy() - ref)) < 2e-3
    finally:
        mmlib.mm_mlp_destroy(h)


@pytest.mark.parametrize("n", [700, 128 * 400 + 37])
def test_gradients_match_reference(cuda, mmlib, n):
    # n = 700: fewer tiles than CTAs, the last one padded; 51237: every CTA trains on two or more
    # tiles, so the weight gradients are summed in tensor memory across tiles before the flush.
    # Per-layer relative error against the float64 reference with the same BF16 rounding points
    # (measured: 1e-6 .. 3e-4).
    h = _mlp(mmlib, 5)
    try:
        p = _params(mmlib, h)
        rng = np.random.default_rng(2)
        x = rng.normal(0, 1, (n, 16)).astype(np.float32)
        t = rng.uniform(0.05, 0.95, n).astype(np.float32)
        dx, dt = _bf16_tensor(cuda, x), cuda.from_numpy(t).cuda()
        g = cuda.zeros(mmlib.mm_mlp_param_count(), device="cuda")
        loss = C.c_float()
        assert mmlib.mm_mlp_gradients(h, C.c_void_p(dx.data_ptr()), C.c_void_p(dt.data_ptr()), n,
                                      C.c_void_p(g.data_ptr()), C.byref(loss), stream_ptr(cuda)) == 0
        gg = g.cpu().numpy().astype(np.float64)
        ref, ref_loss = mlp_ref.gradients(p, x, t.astype(np.float64))
        assert abs(loss.value - ref_loss) < 1e-3 * ref_loss + 1e-6
        o = 0
        for name, shape in mlp_ref.SIZES:
            k = int(np.prod(shape))
            a, b = gg[o:o + k], ref[o:o + k]
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            print("grad %s rel err %.2e" % (name, rel))
            assert rel < 1e-3, (name, rel)
            o += k
    finally:
        mmlib.mm_mlp_destroy(h)


def test_training_reduces_loss_and_checkpoints(cuda, mmlib, tmp_path):
    h = _mlp(mmlib, 7)
    try:
        rng = np.random.default_rng(3)
        n = 128 * 256
        x = rng.uniform(-1, 1, (n, 16)).astype(np.float32)
        t = (1.0 / (1.0 + np.exp(-(np.sin(3 * x[:, 0]) + x[:, 1] * x[:, 2] - 0.5 * x[:, 3])))).astype(np.float32)
        dx, dt = _bf16_tensor(cuda, x), cuda.from_numpy(t).cuda()
        steps = 400
        hist = np.zeros(steps, np.float32)
        assert mmlib.mm_mlp_train(h, C.c_void_p(dx.data_ptr()), C.c_void_p(dt.data_ptr()), n, 4096, steps, 3e-3,
                                  hist.ctypes.data, stream_ptr(cuda)) == 0, mmlib.mm_last_error_string()
        print("loss %.5f -> %.5f" % (hist[:8].mean(), hist[-8:].mean()))
        assert hist[-8:].mean() < 0.2 * hist[:8].mean()
        path = str(tmp_path / "mlp.ckpt").encode()
        assert mmlib.mm_mlp_save(h, path) == 0
        p1 = _params(mmlib, h)
        h2 = _mlp(mmlib, 99)
        try:
            assert mmlib.mm_mlp_load(h2, path) == 0
            assert np.array_equal(_params(mmlib, h2), p1)
        finally:
            mmlib.mm_mlp_destroy(h2)
        bad = str(tmp_path / "bad.ckpt")
        open(bad, "wb").write(b"nonsense")
        assert mmlib.mm_mlp_load(h, bad.encode()) == 1
    finally:
        mmlib.mm_mlp_destroy(h)


def test_bounded_wait_gives_up_and_reports(cuda, mmlib):
    # The tensor-core kernels wait on mbarriers with a poll limit.  An arrival that never comes (a
    # barrier nothing arrives on) makes the wait give up and report instead of hanging the GPU; the
    # context stays usable afterwards.
    import ctypes as C
    st = cuda.full((2,), -1, dtype=cuda.int32, device="cuda")
    assert mmlib.mm_tc_wait_check(1, 4096, C.c_void_p(st.data_ptr()), None) == 0
    assert mmlib.mm_tc_wait_check(0, 4096, C.c_void_p(st.data_ptr() + 4), None) == 0
    cuda.cuda.synchronize()
    assert st.cpu().tolist() == [0, 1]
    x = cuda.ones(1024, device="cuda")
    assert float((x * 2).sum()) == 2048.0
