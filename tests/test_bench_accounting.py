"""The bench line's accounting on the CPU: the algorithmic FLOP counts per
edge, atom and step follow from the model's layer shapes
(student_model.py:318-322 filter, :440-444 update MLP, :599-605 energy
head), the roofline traffic comes from the committed ncu summary of the same
kernel and workload, and the roofline fraction is achieved over peak."""
import json
import os
import re

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

H, R = 128, 20


def test_flop_counts_follow_from_the_layer_shapes():
    filt = 2 * (R * H + H * 3 * H)                    # Linear(20,128), Linear(128,384)
    update = 2 * (2 * H * H + H * 3 * H)              # Linear(256,128), Linear(128,384)
    head = 2 * (H * 64 + 64 * 32 + 32 * 1)            # Linear(128,64), Linear(64,32), Linear(32,1)
    assert bench.GEMM_FLOP_PER_EDGE == filt == 103_424
    n_atoms, n_edges, layers = 16_858, 859_862, 3
    # forward pass plus the input-gradient pass (the same GEMMs again)
    expect = 2 * (layers * (n_edges * filt + n_atoms * update) + n_atoms * head)
    assert bench.step_gemm_flop(n_atoms, n_edges, layers) == expect
    # per atom-step on the 256-structure batch: ~33 MFLOP
    assert 30e6 < expect / n_atoms < 36e6


@pytest.mark.parametrize("kernel", ["edge_bwd", "edge_fwd"])
def test_roofline_traffic_is_read_from_the_committed_ncu_summary(kernel):
    path = os.path.join(ROOT, "profiles", f"{kernel}_batch256.md")
    text = open(path).read()
    read, write = (float(x) for x in re.search(r"DRAM read \+ write \| ([\d.]+) \+ ([\d.]+) MB", text).groups())
    t = bench.read_traffic(kernel, "batch256")
    assert t is not None
    # the machine-readable figure is the table's read + write (MB rounded to 0.1)
    assert abs(t / 1e6 - (read + write)) < 0.2
    assert bench.read_traffic(kernel, "no_such_workload") is None


def test_roofline_fraction_is_achieved_over_the_measured_peak():
    peak, hbm, src = bench.measured_peaks()
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        assert src == "measured" and peak == d["bf16_tflops"] and hbm == d["hbm_gbs"]
    else:
        assert src == "fallback"
    # the reverse edge kernel on the 256-structure batch: 2 x E x 103,424 FLOP per launch
    # in 0.716 ms is ~248 TFLOP/s, an eighth of the measured bf16 peak
    flop = 2 * 859_862 * bench.GEMM_FLOP_PER_EDGE
    achieved = flop / (0.716e-3) / 1e12
    assert 240 < achieved < 260
    assert 0.10 < achieved / peak < 0.16
