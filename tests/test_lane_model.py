"""The lane-utilization model (oracle/lane_model.py) on synthetic traces: lockstep warp costs, the
accumulating-lane histogram and the pooled cone.  CPU only; the traced oracle is not built here."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import lane_model  # noqa: E402


def _frame(events_per_lane):
    # one 8x4 warp tile; events_per_lane: 32 lists of event codes (row-major lanes of the tile)
    cap = max(len(e) for e in events_per_lane)
    ev = np.zeros((4, 8, cap), np.uint8)
    for lane, e in enumerate(events_per_lane):
        ev[lane // 8, lane % 8, :len(e)] = e
    return ev


def test_uniform_warp_is_fully_utilized():
    m = lane_model.model(_frame([[1, 1, 2, 3, 5, 5, 4]] * 32))
    assert abs(m["lane_utilization"] - 1.0) < 1e-12
    assert m["accumulating_lanes_when_any"] == 32
    assert abs(m["pooled_cone_utilization"] - 1.0) < 1e-12


def test_one_accumulating_lane_idles_the_cone():
    lanes = [[1, 3, 3]] * 31 + [[1, 3, 5]]
    m = lane_model.model(_frame(lanes))
    assert abs(m["cone"]["utilization"] - 1.0 / 32) < 1e-12
    assert m["accumulating_lanes_when_any"] == 1
    # the pool computes that one cone in a round of its own: no better, no worse
    assert abs(m["pooled_cone_utilization"] - 1.0 / 32) < 1e-12


def test_pool_gathers_cones_from_different_iterations():
    # lane i accumulates at iteration i % 4: the inline cone runs in 4 iterations with 8 lanes each,
    # the pool in one round of 32
    lanes = [[3] * (i % 4) + [5] + [3] * (3 - i % 4) for i in range(32)]
    m = lane_model.model(_frame(lanes))
    assert abs(m["cone"]["utilization"] - 0.25) < 1e-12
    assert abs(m["pooled_cone_utilization"] - 1.0) < 1e-12
    assert m["pooled_warp_work_fraction"] < 1.0
