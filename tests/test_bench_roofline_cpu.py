"""The roofline arithmetic of bench.py's JSON line, on the CPU with synthetic figures.

The issued basis counts 2 DFMA + DADD + DMUL thread instructions per cell (from the committed ncu capture)
over the launch time against the DFMA probe's peak; the FP64-issue fraction counts the same instructions
against the probe's FMA instruction rate (peak / 2); workloads of the same mechanism without a capture of
their own are estimated from their reference-operation count with the captured workload's issued /
reference ratio.
"""
import pytest

import bench


def test_issued_basis_and_fp64_issue():
    issued = {"cells": 1000, "dfma": 3.0e9, "dadd": 1.0e9, "dmul": 2.0e9, "flop_per_cell": (2 * 3.0e9 + 3.0e9) / 1000,
              "command": "ncu ..."}
    n, kernel_ms, peak = 10000, 2000.0, 1.25
    r = bench.roofline_fp64(issued, n, kernel_ms, peak, 4.0e13, 1.0e9, [1, 2, 3, 4, 5, 6])
    flops = issued["flop_per_cell"] * n                      # 9e10
    assert r["issued_flops_per_launch"] == pytest.approx(flops)
    assert r["achieved"] == pytest.approx(flops / 2.0 / 1e12)
    assert r["frac"] == pytest.approx(flops / 2.0 / 1e12 / peak)
    inst = (3.0e9 + 1.0e9 + 2.0e9) / 1000 * n                # thread instructions per launch
    assert r["fp64_issue"]["frac"] == pytest.approx(inst / 2.0 / (peak * 1e12 / 2.0))
    ref = r["reference_operation_count"]
    assert ref["frac"] == pytest.approx(4.0e13 / 2.0 / 1e12 / peak)
    # an all-FMA mix at the probe's rate reaches 1 on both bases
    fma = {"cells": 1, "dfma": 1.0, "dadd": 0.0, "dmul": 0.0, "flop_per_cell": 2.0, "command": ""}
    r = bench.roofline_fp64(fma, 1, 1e3 * 2.0 / (peak * 1e12), peak, None, None, None)
    assert r["frac"] == pytest.approx(1.0) and r["fp64_issue"]["frac"] == pytest.approx(1.0)


def test_estimated_issued_basis_uses_the_captured_ratio(monkeypatch):
    rec = {"flop_per_cell": 1.0e6, "reference_flop_per_cell": 2.5e6}
    monkeypatch.setattr(bench, "profile_record", lambda name, workload: rec)
    r = bench.roofline_fp64_estimated(5.0e12, 4.0, 1.25, {"kernel": "x"})
    ref = 5.0e12 / 4.0 / 1e12
    assert r["reference_operation_count"]["achieved"] == pytest.approx(ref)
    assert r["achieved"] == pytest.approx(ref * 0.4)
    assert r["frac"] == pytest.approx(ref * 0.4 / 1.25)
    assert r["kernel"] == "x" and "estimated" in r["basis"]
    monkeypatch.setattr(bench, "profile_record", lambda name, workload: None)
    r = bench.roofline_fp64_estimated(5.0e12, 4.0, 1.25)
    assert r["frac"] is None and r["reference_operation_count"]["frac"] == pytest.approx(ref / 1.25)


def test_committed_capture_records_are_consistent():
    for w in ("h2air-1M", "c2h2-262144", "air2t-262144"):
        rec = bench.profile_record("fp64_issued.json", w)
        assert rec is not None, w
        flop = (2 * rec["dfma"] + rec["dadd"] + rec["dmul"]) / rec["cells"]
        assert rec["flop_per_cell"] == pytest.approx(flop), w
        assert "--clock-control none" in rec["command"], w
    t = bench.profile_record("traffic.json", "h2air-1M")
    assert t["bytes_per_cell"] == pytest.approx((t["dram_read_bytes"] + t["dram_write_bytes"]) / t["cells"])
