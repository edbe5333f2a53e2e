"""The CPU reference of the surrogate network: its analytic gradient agrees with central finite
differences in float64 (this validates the back-propagation formulas the GPU kernels implement)."""
import numpy as np

import mlp_ref


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    n_par = sum(int(np.prod(s)) for _, s in mlp_ref.SIZES)
    assert n_par == 9473
    p = rng.normal(0, 0.3, n_par)
    x = rng.normal(0, 1, (40, 16))
    t = rng.uniform(0, 1, 40)
    g, _ = mlp_ref.gradients(p, x, t, emulate_bf16=False)
    idx = rng.choice(n_par, 200, replace=False)
    idx = np.concatenate([idx, [n_par - 1, 0, 1024, 5200, 9400]])
    h = 1e-6
    for i in idx:
        e = np.zeros(n_par)
        e[i] = h
        fd = (mlp_ref.loss(p + e, x, t) - mlp_ref.loss(p - e, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 + 1e-4 * abs(fd), (i, fd, g[i])


def test_bf16_rounding():
    # bf16 spacing at 1 is 2^-7: 1 + 2^-8 and 1 + 3*2^-8 are ties, rounded to the even neighbour
    v = np.array([1.0, 1.00390625, 1.01171875, 3.14159265, -2.5e-3], np.float32)
    r = mlp_ref.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625
    assert abs(r[3] - 3.140625) < 1e-9
