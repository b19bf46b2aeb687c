"""Host-side pieces of bench.py that need no GPU: the DRAM-traffic lookup in
the committed ncu summary (one line per kernel choice), the error metrics of
the parity checks and the peak denominators."""
import json
import os

import numpy as np
import pytest

import bench


def test_profiled_traffic_matches_the_kernel_choice():
    # the summary carries one traffic line per kernel choice the autotuner picks between
    for choice in ({"variant": 3, "fields_per_pass": 128, "unroll": 4, "stages": 0},
                   {"variant": 3, "fields_per_pass": 256, "unroll": 4, "stages": 0}):
        t, src = bench.profiled_traffic(choice)
        assert t is not None and t > 0, src
        # traffic is at least the algorithmic bytes of a 1016-field step and not far above
        alg = 4 * 3538944 * 1016 + 4 * 1036800 * 1016 + 12 * 9253358 + 4 * (1036800 + 1)
        assert alg < t < 1.5 * alg
        assert "ncu" in src and "1016" in src


def test_profiled_traffic_refuses_other_kernel_choices():
    t, src = bench.profiled_traffic({"variant": 1, "fields_per_pass": 128, "unroll": 4, "stages": 2})
    assert t is None
    assert "1,128,4,2" in src


def test_profile_traffic_lines_parse():
    p = os.path.join(bench.ROOT, "profiles", "apply_split_ws_c768_0p25.md")
    lines = [ln for ln in open(p) if ln.startswith("traffic_bytes_per_step[")]
    assert len(lines) >= 1
    for ln in lines:
        key, val = ln[len("traffic_bytes_per_step["):].split("]:", 1)
        assert len(key.split(",")) == 4
        assert int(val.strip()) > 0


def test_rel_errors_and_condition_bound():
    ref = np.array([[1.0, -2.0, 1e-9, 0.0]])
    y = (ref * (1 + 1e-7)).astype(np.float32)
    e = bench.rel_errors(y, ref)
    assert e["max_rel"] < 2e-7 and e["rms_rel"] < 2e-7
    # outputs that cancel: the error over the condition sum stays small when the
    # elementwise relative error does not
    cond = np.array([[1.0, 2.0, 1.0, 1.0]])
    y2 = ref + np.array([[0.0, 0.0, 1e-12, 1e-12]])
    assert bench.cond_errors(y2, ref, cond) <= 1.1e-12
    assert bench.rel_errors(y2, ref)["max_rel"] > 1e-4


def test_peaks_reads_the_measured_file():
    hbm, kind = bench.peaks()
    p = os.path.join(bench.ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        assert kind == "measured"
        assert hbm == pytest.approx(float(json.load(open(p))["hbm_gbs"]))
    else:
        assert kind == "fallback"
