"""CPU reference of the surrogate network (the checker of the tensor-core kernels).

float64 arithmetic; with `emulate_bf16` the values are rounded to bfloat16 exactly where the GPU
kernels round them (inputs, W1..W3, hidden activations h1, h2, and the back-propagated deltas);
without it the network is a smooth float64 function whose analytic gradient is checked by finite
differences."""
import numpy as np

N_IN, N_HID = 16, 64
SIZES = [("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)),
         ("W3", (N_HID, N_HID)), ("b3", (N_HID,)), ("w4", (N_HID,)), ("b4", (1,))]


def unpack(p):
    out, o = {}, 0
    for name, shape in SIZES:
        n = int(np.prod(shape))
        out[name] = np.asarray(p[o:o + n], np.float64).reshape(shape)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def bf16(x):
    """Round float32 values to bfloat16 (round to nearest even), returned as float64."""
    f = np.asarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(p, x, emulate_bf16=True):
    P = unpack(p)
    q = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    xb = q(x)
    W1, W2, W3 = q(P["W1"]), q(P["W2"]), q(P["W3"])
    z1 = xb @ W1.T + P["b1"]
    h1 = q(np.maximum(z1, 0.0))
    z2 = h1 @ W2.T + P["b2"]
    h2 = q(np.maximum(z2, 0.0))
    z3 = h2 @ W3.T + P["b3"]
    h3 = np.maximum(z3, 0.0)
    z4 = h3 @ P["w4"] + P["b4"][0]
    y = 1.0 / (1.0 + np.exp(-z4))
    return y, dict(xb=xb, W1=W1, W2=W2, W3=W3, h1=h1, h2=h2, h3=h3)


def loss(p, x, t, emulate_bf16=False):
    y, _ = forward(p, x, emulate_bf16)
    return float(np.mean((y - t) ** 2))


def gradients(p, x, t, emulate_bf16=True):
    P = unpack(p)
    q = bf16 if emulate_bf16 else (lambda v: np.asarray(v, np.float64))
    y, c = forward(p, x, emulate_bf16)
    B = len(t)
    dz = 2.0 * (y - t) * y * (1.0 - y) / B
    g = {"w4": c["h3"].T @ dz, "b4": np.array([dz.sum()])}
    d3 = q(dz[:, None] * P["w4"][None, :] * (c["h3"] > 0))
    g["W3"], g["b3"] = d3.T @ c["h2"], d3.sum(0)
    d2 = q((d3 @ c["W3"]) * (c["h2"] > 0))
    g["W2"], g["b2"] = d2.T @ c["h1"], d2.sum(0)
    d1 = q((d2 @ c["W2"]) * (c["h1"] > 0))
    g["W1"], g["b1"] = d1.T @ c["xb"], d1.sum(0)
    return pack(g), float(np.mean((y - t) ** 2))
