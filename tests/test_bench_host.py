"""Host helpers of bench.py without a GPU: the clock-sample summary that
marks throttled runs, and the lookup of the committed DRAM traffic."""
from types import SimpleNamespace

import bench


def test_clock_summary_reports_median_and_throttle_reasons():
    c = bench.Clocks(0)
    c.proc = SimpleNamespace(terminate=lambda: None, wait=lambda timeout=None: 0, kill=lambda: None)
    c.samples = [["1980", "2070", "0x0", "Not Active", "Not Active", "Not Active", "Active"],
                 ["2070", "2070", "0x0", "Not Active", "Active", "Not Active", "Not Active"],
                 ["2040", "2070", "0x0", "Not Active", "Not Active", "Not Active", "Not Active"],
                 ["[N/A]", "[N/A]"]]
    r = c.stop()
    assert r["sm_mhz"] == 2040.0 and r["sm_max_mhz"] == 2070.0 and r["samples"] == 4
    assert r["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]


def test_clock_summary_without_nvidia_smi():
    r = bench.Clocks(0).stop()
    assert r["sm_mhz"] is None and r["reasons"] == ["nvidia-smi unavailable"]


def test_captured_traffic_lookup():
    """The committed stage-2 capture applies to its own workload and
    precision only."""
    name = "hubbard-cylinder-4x32-phi0.25-U8-Ne112-m2000-midchain"
    assert bench.captured_traffic(name, "bf16x3") == 584870000.0
    assert bench.captured_traffic(name, "bf16x6") is None
    assert bench.captured_traffic("other", "bf16x3") is None
    peaks = bench.measured_peaks()
    assert peaks["hbm_gbs"] > 1000 and peaks["bf16_tflops"] > 100
