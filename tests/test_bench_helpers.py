"""bench.py's host-side arithmetic on the CPU: the clock-record summary
(median SM clock, throttle reasons), the per-workload summary (quantiles,
rates) and the two roofline figures, on made-up inputs."""
import os
import sys
from types import SimpleNamespace

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def _clock_line(sm, mx, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return "0, %s, %s, 900.5, 0x0, %s, %s, %s, %s" % (sm, mx, hw, hwt, swt, cap)


def test_clock_summary_median_and_reasons():
    c = bench.ClockSampler(0)
    c.lines = [_clock_line(2070, 2070), _clock_line(1900, 2070, cap="Active"),
               _clock_line(2000, 2070), "garbage", _clock_line("[N/A]", 2070)]
    s = c.summary()
    assert s["samples"] == 3
    assert s["sm_mhz"] == 2000 and s["sm_max_mhz"] == 2070
    assert s["reasons"] == ["sw_power_cap"]
    c.lines = [_clock_line(1500, 2070, hwt="Active", hw="Active")]
    assert c.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"]
    c.lines = []
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_workload_summary_rates_and_quantiles():
    res = [SimpleNamespace(nodes_total=100 * (i + 1), len=40 + i, seconds=0.01 * (i + 1), status=0)
           for i in range(100)]
    st = {"kernel_ms": 12.5, "rounds": 7, "kernel_launches": 9, "tasks_donated": 11, "frontier_ms": 0.5,
          "dev_lane_steps": 3, "dev_lane_slots": 4, "dev_idle_cycles": 1, "dev_warp_cycles": 10}
    d = bench._summary("w", 2.0, res, st, {"heuristic": "x"})
    assert d["nodes"] == sum(100 * (i + 1) for i in range(100))
    assert d["nodes_per_s"] == pytest.approx(d["nodes"] / 2.0)
    assert d["instances_per_s"] == pytest.approx(50.0)
    assert d["optimal_len"] == {"min": 40, "p50": 90, "max": 139}
    assert d["latency_s"]["p50"] == pytest.approx(0.51)
    assert d["latency_s"]["p99"] == pytest.approx(1.0) and d["latency_s"]["max"] == pytest.approx(1.0)
    assert d["lane_step_fraction"] == pytest.approx(0.75)
    assert d["idle_fraction"] == pytest.approx(0.1)
    assert d["heuristic"] == "x"


def test_int_roofline_arithmetic():
    import slide
    r = bench._int_roofline(nodes=2e9, kernel_ms=1000.0, peak_ops=64e9)
    assert r["bound"] == "int-issue" and r["ops_per_node"] == slide.MD_OPS_PER_NODE == 16
    assert r["achieved"] == pytest.approx(32.0)
    assert r["peak"] == pytest.approx(64.0)
    assert r["frac"] == pytest.approx(0.5)


def test_hbm_peak_is_the_measured_copy_bandwidth():
    peak, how = bench.load_peaks()
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        import json
        assert how == "measured"
        assert peak == float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"])
    else:
        assert (peak, how) == (6800.0, "fallback")


def test_sector_roofline_arithmetic():
    r = bench._sector_roofline(nodes=1e9, kernel_ms=100.0, reads_per_s=100e9, bound="l2-random",
                               working_set=3 << 20)
    # 1e9 nodes x 64 B in 0.1 s = 640 GB/s against 100e9 reads x 32 B = 3200 GB/s
    assert r["bound"] == "l2-random" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(640.0)
    assert r["peak"] == pytest.approx(3200.0)
    assert r["frac"] == pytest.approx(0.2)
    assert r["lookups_per_s"] == pytest.approx(2e10)


def test_length_histogram_is_sorted_by_length():
    assert bench._hist([60, 58, 60, 102, 9]) == {"9": 1, "58": 1, "60": 2, "102": 1}
