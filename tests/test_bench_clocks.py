"""The bench's clock sampler, against a fake nvidia-smi on PATH (no GPU):
samples are kept only inside the marked timed region (plus one polling
interval), and throttle reasons are read from the query's columns."""
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

IDLE = "2070, 2070, 900.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
SLOW = "1500, 2070, 1400.00, 0x0000000000000008, Active, Not Active, Not Active, Active"


def _fake_smi(tmp_path, monkeypatch, script):
    f = tmp_path / "nvidia-smi"
    f.write_text("#!/bin/bash\n" + script)
    f.chmod(0o755)
    monkeypatch.setenv("PATH", f"{tmp_path}:{os.environ['PATH']}")
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    import bench
    return bench


def test_samples_inside_the_timed_region(tmp_path, monkeypatch):
    # start-up slower than the region; then one sample every 20 ms
    bench = _fake_smi(tmp_path, monkeypatch, f"sleep 0.3\nwhile true; do echo '{IDLE}'; sleep 0.02; done\n")
    with bench.ClockSampler(0) as clk:
        assert clk.lines, "the first line arrives before the region starts"
        time.sleep(0.1)                     # warm-up: its samples are not kept
        n_before = len(clk.lines)
        clk.start()
        time.sleep(0.08)
        clk.stop()
    s = clk.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["reasons"] == []
    assert 2 <= s["samples"] <= len(clk.lines) - n_before
    assert s["interval_ms"] == 20 and 70 <= s["region_ms"] <= 200


def test_throttle_reasons_are_reported(tmp_path, monkeypatch):
    bench = _fake_smi(tmp_path, monkeypatch, f"while true; do echo '{SLOW}'; sleep 0.02; done\n")
    with bench.ClockSampler(0) as clk:
        clk.start()
        time.sleep(0.06)
        clk.stop()
    s = clk.summary()
    assert s["sm_mhz"] == 1500.0
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap"]


def test_no_sampler_reads_unsampled(tmp_path, monkeypatch):
    bench = _fake_smi(tmp_path, monkeypatch, "exit 1\n")
    with bench.ClockSampler(0) as clk:
        clk.start()
        clk.stop()
    assert clk.summary()["reasons"] == ["unsampled"]
