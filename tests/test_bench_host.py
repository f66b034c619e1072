"""CPU: the benchmark's host-side pieces -- the clock record it attaches to
every line (nvidia-smi samples with throttle reasons), the peak it divides
by, and the whole-job aggregation."""
import json

import bench


def _line(sm, mx, slow="Not Active", thermal="Not Active", sw_thermal="Not Active", power="Not Active"):
    return f"0, {sm}, {mx}, 950.12, 0x0000000000000000, {slow}, {thermal}, {sw_thermal}, {power}"


def test_clock_summary_median_and_reasons():
    c = bench.Clocks(0)
    c.lines = [_line(2070, 2070), _line(1980, 2070, power="Active"), _line(2070, 2070),
               "0, [N/A], [N/A], [N/A], x, x, x, x, x"]
    s = c.summary()
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"], "samples": 3}
    c.lines = [_line(1200, 2070, thermal="Active"), _line(1300, 2070, slow="Active")]
    s = c.summary()
    assert s["reasons"] == ["hw_slowdown", "hw_thermal_slowdown"] and s["sm_mhz"] == 1250.0


def test_clock_summary_without_samples():
    assert bench.Clocks(0).summary() is None


def test_peak_from_measured_file_or_fallback(tmp_path, monkeypatch):
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6787.6}))
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    assert bench.load_peaks() == (6787.6, "measured")
    monkeypatch.setattr(bench, "ROOT", str(tmp_path / "absent"))
    assert bench.load_peaks() == (6800.0, "fallback")


def test_aggregate_one_rank():
    """numbers per second over the step time (several ranks: test_dist_cpu.py)"""
    ms, mnum = bench.aggregate(2.0, 1 << 19, 1)
    assert ms == 2.0 and abs(mnum - (1 << 19) / 2e-3 / 1e6) < 1e-9
