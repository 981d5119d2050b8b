"""bench.py's host-side pieces that need no GPU: the committed DRAM-traffic record it reads for the
roofline line, and its argument defaults."""
import sys

import pytest

import bench


def test_recorded_traffic_names_each_capture():
    t = bench.recorded_traffic(("cull_decide_kernel<5>", "cull_scatter2_kernel"), 4_000_000)
    assert t is not None
    assert 150e6 < t["bytes_per_launch"] < 250e6  # the sweep moves about 200 MB of algorithmic bytes
    assert "cull_decide_kernel<5>: ncu capture at commit" in t["source"]
    assert "cull_scatter2_kernel: ncu capture at commit" in t["source"]
    f = bench.recorded_traffic(("cull_frame_kernel<0,256,2>", "cull_scatter2_kernel"), 4_000_000)
    assert f is not None and f["bytes_per_launch"] > t["bytes_per_launch"] - 10e6


def test_recorded_traffic_refuses_another_scene_size_or_kernel():
    assert bench.recorded_traffic(("cull_decide_kernel<5>",), 1_000_000) is None
    assert bench.recorded_traffic(("no_such_kernel",), 4_000_000) is None


def test_bench_defaults(monkeypatch):
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    a = bench.parse()
    assert (a.gpus, a.impl, a.objects) == (1, "ours", 4_000_000)
    assert a.warmup >= 3 and a.steps > 0
