"""Lane-utilization model of the GPU march from the oracle's per-iteration trace (analysis only).

Runs the FP32 oracle (texture-unit filter) over one sweep frame with the per-iteration event trace of
`_build/liboracle_trace.so` (oracle_march.cpp, ORACLE_TRACE), groups the rays into the GPU kernel's
8x4 warp tiles, and executes each warp in lockstep: iteration i costs the warp the loop body if any
lane is still marching, cloudHiRes if any lane has a small-step sample with density, and the six-tap
sun cone (compute-clouds.comp:441-453) if any lane accumulates.  Per-lane costs are the rough
instruction weights of the one-thread kernel (ray set-up 250, loop body 70, cloudHiRes 35, cone 450).
It prints each part's share of the warp work and its lane utilization, how many lanes accumulate in
an iteration in which any does, and the cone's utilization when the accumulated samples of a warp are
pooled and computed 32 at a time (the pooled-cone kernel).

    python oracle/lane_model.py [width height frame]      # default 1920 1080 3; 4K needs ~2.7 GB
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import oracle  # noqa: E402

CAP = 320  # events per ray (the longest rays of the sweep take ~310 iterations)
SETUP, BODY, HIRES, CONE = 250.0, 70.0, 35.0, 450.0
TILE_W, TILE_H = 8, 4


def trace(width, height, frame):
    lib_path = os.path.join(oracle.ORACLE_DIR, "_build", "liboracle_trace.so")
    subprocess.run(["make", "-s", "-C", oracle.ORACLE_DIR, "_build/liboracle_trace.so"], check=True)
    saved = oracle.LIB, oracle._lib
    oracle.LIB, oracle._lib = lib_path, None
    try:
        lib = oracle.load()
        lib.oracle_trace_set.argtypes = [C.c_void_p, C.c_size_t]
        ev = np.zeros((height, width, CAP), np.uint8)
        lib.oracle_trace_set(ev.ctypes.data, CAP)
        u = oracle.sweep_uniforms(frame, width, height)
        _, _, counters = oracle.march(u, oracle.seed_textures(0), width, height, filter=oracle.FILTER_TEXTURE_UNIT)
        lib.oracle_trace_set(None, 0)
    finally:
        oracle.LIB, oracle._lib = saved
    return ev, counters


def model(ev):
    h, w, cap = ev.shape
    h, w = h - h % TILE_H, w - w % TILE_W
    tot = dict.fromkeys(["lane", "warp", "lane_b", "warp_b", "lane_h", "warp_h", "lane_c", "warp_c", "pool_c"], 0.0)
    hist = np.zeros(33, np.int64)
    for y0 in range(0, h, TILE_H * 32):
        blk = ev[y0:min(h, y0 + TILE_H * 32), :w]
        rows = blk.shape[0] // TILE_H
        wp = blk[:rows * TILE_H].reshape(rows, TILE_H, w // TILE_W, TILE_W, cap).transpose(0, 2, 1, 3, 4)
        wp = wp.reshape(-1, 32, cap)
        act, hires, acc = wp != 0, (wp == 4) | (wp == 5), wp == 5
        live = act.any(-1)
        tot["lane"] += SETUP * live.sum()
        tot["warp"] += 32 * SETUP * live.any(1).sum()
        tot["lane_b"] += BODY * act.sum()
        tot["warp_b"] += 32 * BODY * act.any(1).sum()
        tot["lane_h"] += HIRES * hires.sum()
        tot["warp_h"] += 32 * HIRES * hires.any(1).sum()
        tot["lane_c"] += CONE * acc.sum()
        tot["warp_c"] += 32 * CONE * acc.any(1).sum()
        tot["pool_c"] += 32 * CONE * np.ceil(acc.sum((1, 2)) / 32.0).sum()
        hist += np.bincount(acc.sum(1).ravel(), minlength=33)[:33]
    lane = tot["lane"] + tot["lane_b"] + tot["lane_h"] + tot["lane_c"]
    warp = tot["warp"] + tot["warp_b"] + tot["warp_h"] + tot["warp_c"]
    k = np.arange(1, 33)
    return {
        "lane_utilization": lane / warp,
        "body": {"share": tot["warp_b"] / warp, "utilization": tot["lane_b"] / tot["warp_b"]},
        "cloud_hires": {"share": tot["warp_h"] / warp, "utilization": tot["lane_h"] / tot["warp_h"]},
        "cone": {"share": tot["warp_c"] / warp, "utilization": tot["lane_c"] / tot["warp_c"]},
        "accumulating_lanes_when_any": float((k * hist[1:]).sum() / max(1, hist[1:].sum())),
        "pooled_cone_utilization": tot["lane_c"] / tot["pool_c"],
        "pooled_warp_work_fraction": (warp - tot["warp_c"] + tot["pool_c"]) / warp,
    }


def main():
    width, height, frame = (int(a) for a in (sys.argv[1:4] if len(sys.argv) >= 4 else (1920, 1080, 3)))
    ev, counters = trace(width, height, frame)
    print("%dx%d sweep frame %d: cloudTest %d, cloudHiRes %d, iterations %d, accumulated %d" %
          ((width, height, frame) + tuple(int(c) for c in counters)))
    for key, val in model(ev).items():
        print("  %-30s %s" % (key, {a: round(float(b), 3) for a, b in val.items()} if isinstance(val, dict)
                              else round(float(val), 3)))


if __name__ == "__main__":
    main()
