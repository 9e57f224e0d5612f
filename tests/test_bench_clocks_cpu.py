"""The clock record of bench.py: nvidia-smi samples taken during the timed
region become `{"sm_mhz": median, "sm_max_mhz", "reasons": [...]}`, with every
throttle reason seen active in any sample listed (a run that saw a hardware or
thermal slowdown is rejected on that field).  Checked on synthetic samples."""
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

import bench  # noqa: E402


def _sampler(lines):
    s = bench.ClockSampler(None)
    s.lines = lines
    return s


def _line(sm, smax, hw="Not Active", hwt="Not Active", swt="Not Active", cap="Not Active"):
    return f"0, {sm}, {smax}, 900.0, 0x0, {hw}, {hwt}, {swt}, {cap}"


def test_median_clock_and_no_reason():
    s = _sampler([_line(2070, 2070), _line(2055, 2070), _line(2070, 2070)])
    out = s.summary()
    assert out["sm_mhz"] == 2070 and out["sm_max_mhz"] == 2070
    assert out["reasons"] == [] and out["samples"] == 3


def test_reasons_seen_in_any_sample_are_reported():
    s = _sampler([_line(2070, 2070), _line(1900, 2070, cap="Active"), _line(1500, 2070, hwt="Active")])
    out = s.summary()
    assert out["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert out["sm_mhz"] == 1900


def test_malformed_and_missing_samples():
    s = _sampler(["garbage", "0, N/A, N/A, x, y, z, a, b, c"])
    assert s.summary()["reasons"] == ["unsampled"]
    assert _sampler([]).summary()["sm_mhz"] is None
