"""Error metrics of the parity gates.

Colour error is measured after the reference's own display transform, the Uncharted-2 tonemap of
tonemap.frag:10-28 (exposure 0.7, white point 50.2, gamma 1/2.2, no vignette), scaled to 0..255;
alpha is compared raw x 255; depth by relative error where both depths are finite.
"""
import numpy as np


def _uc2(x):
    return ((x * (0.15 * x + 0.1 * 0.5) + 0.2 * 0.02) / (x * (0.15 * x + 0.5) + 0.2 * 0.3)) - 0.02 / 0.3


def tonemap(rgb):
    x = np.asarray(rgb, np.float64)
    white = 1.0 / _uc2(50.2)
    v = _uc2(0.7 * x) * white
    return np.power(np.maximum(v, 0.0), 1.0 / 2.2)


def frame_errors(rgba, ref_rgba, depth=None, ref_depth=None):
    """RMSE / max colour error in 1/255 units of tonemapped colour, alpha errors, depth errors."""
    a = np.asarray(rgba, np.float64)
    b = np.asarray(ref_rgba, np.float64)
    d = (tonemap(a[..., :3]) - tonemap(b[..., :3])) * 255.0
    out = {
        "rmse_255": float(np.sqrt(np.mean(d * d))),
        "max_255": float(np.max(np.abs(d))) if d.size else 0.0,
        "p999_255": float(np.percentile(np.abs(d).max(-1), 99.9)) if d.size else 0.0,
        "frac_over_4": float(np.mean(np.abs(d).max(-1) > 4.0)) if d.size else 0.0,
        "alpha_max_255": float(np.max(np.abs(a[..., 3] - b[..., 3])) * 255.0) if d.size else 0.0,
        "nan": int(np.isnan(a).sum()),
    }
    if depth is not None and ref_depth is not None:
        x = np.asarray(depth, np.float64)
        y = np.asarray(ref_depth, np.float64)
        both = np.isfinite(x) & np.isfinite(y)
        rel = np.abs(x[both] - y[both]) / np.maximum(np.abs(y[both]), 1e-30)
        out["depth_rel_max"] = float(rel.max()) if rel.size else 0.0
        out["depth_rel_p999"] = float(np.percentile(rel, 99.9)) if rel.size else 0.0
        out["depth_rel_median"] = float(np.median(rel)) if rel.size else 0.0
        out["depth_frac_over_1e3"] = float(np.mean(rel > 1e-3)) if rel.size else 0.0
        out["depth_finite_mismatch"] = float(np.mean(np.isfinite(x) != np.isfinite(y)))
    return out
