"""Host logic of bench.py that needs no GPU: the clock record summary, the
workload name and config, and the peak lookup."""
import json

import bench


def _row(sm, mx, hw="Not Active", hwt="Not Active", swt="Not Active", pc="Not Active", t=1.0):
    # (time, [index, clocks.sm, clocks.max.sm, power.draw, reasons.active, hw, hw_thermal, sw_thermal, sw_power_cap])
    return (t, ["0", str(sm), str(mx), "900.0", "0x0", hw, hwt, swt, pc])


def test_clock_summary_median_max_and_no_reasons():
    c = bench.ClockSampler(0)
    c.rows = [_row(2070, 2070), _row(2055, 2070), _row(2070, 2070)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == [] and s["samples"] == 3


def test_clock_summary_collects_active_reasons():
    c = bench.ClockSampler(0)
    c.rows = [_row(1800, 2070, pc="Active"), _row(1700, 2070, hwt="Active"), _row(2070, 2070)]
    s = c.summary()
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert s["sm_mhz"] == 1800.0


def test_clock_summary_without_samples_says_unavailable():
    s = bench.ClockSampler(0).summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["unavailable"]


def test_clock_summary_skips_unreadable_fields():
    c = bench.ClockSampler(0)
    c.rows = [_row("[N/A]", "[N/A]"), _row(2070, 2070)]
    s = c.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0


def test_workload_name_marks_scaled_runs():
    assert bench.workload_name(2448, 2048) == bench.WORKLOAD
    scaled = bench.workload_name(1224, 1024)
    assert scaled.startswith("1224x1024 pair (5 MP workload scaled)") and scaled != bench.WORKLOAD


def test_peaks_reads_measured_file_or_falls_back(tmp_path, monkeypatch):
    monkeypatch.setattr(bench, "ROOT", tmp_path)
    assert bench.peaks() == (6800.0, "fallback")
    (tmp_path / "MEASURED_PEAKS.json").write_text(json.dumps({"hbm_gbs": 6786.9}))
    assert bench.peaks() == (6786.9, "measured")


def test_clock_summary_keeps_the_timed_windows():
    c = bench.ClockSampler(0)
    c.rows = [_row(1000, 2070, t=0.5), _row(2070, 2070, t=1.5, pc="Active"), _row(2055, 2070, t=1.6),
              _row(900, 2070, t=3.0, hwt="Active")]
    c.mark(1.0, 2.0)
    s = c.summary()
    assert s["samples"] == 2 and s["samples_total"] == 4
    assert s["sm_mhz"] == 2062.5 and s["reasons"] == ["sw_power_cap"]


def test_both_arms_share_one_config():
    a = bench.workload_config(2448, 2048, 12, 2501, 2092, 2 * 12 * 2448 * 2048 * 2)
    b = bench.workload_config(2448, 2048, 12, 2501, 2092, 240648192)
    assert a == b and a["workload"] == bench.WORKLOAD and "> 129 MB L2" in a["l2"]


def test_measured_figures_name_committed_profiles():
    """Every ncu figure the bench line quotes names a summary under profiles/
    that exists, and the instruction figure is a plausible warp count."""
    import bench
    for table in (bench.MEASURED_TRAFFIC, bench.MEASURED_ISSUE):
        for key, val in table.items():
            src = val[-1]
            assert (bench.ROOT / src).is_file(), (key, src)
    for (_, W, H), (inst, fma, _) in bench.MEASURED_ISSUE.items():
        assert inst > W * H / 32 and 0.0 < fma < 1.0
