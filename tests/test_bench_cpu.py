"""Host-side helpers of bench.py, on CPU: the DRAM traffic figure the bench
line carries (profiles/traffic.json, scaled from an ncu capture and tied to
the summary it came from), the parsing of nvidia-smi clock samples (median
SM clock and the throttle reasons that reject a run), and the roofline
denominator."""
from __future__ import annotations

import json
import re
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def _traffic():
    return json.loads((ROOT / "profiles" / "traffic.json").read_text())


@pytest.mark.parametrize("kernel", ["radix_pass_kernel", "persistent_sort_kernel"])
def test_traffic_entry_is_the_scaled_capture(kernel):
    e = _traffic()[kernel]
    # the capture ran the same passes on fewer keys: bytes scale with keys
    assert e["bytes_per_launch"] == e["captured_bytes_per_launch"] * e["bench_n"] // e["captured_n"]
    summary = ROOT / e["summary"]
    assert summary.is_file() and summary.parent.name == "profiles"
    # the summary states the captured read + write bytes (MB, one decimal)
    text = summary.read_text()
    nums = [float(x) for x in re.findall(r"([0-9]+\.[0-9]) MB", text)]
    mb = e["captured_bytes_per_launch"] / 1e6
    assert any(abs(x - mb) < 0.06 for x in nums) or (
        len(nums) >= 2 and abs(nums[0] + nums[1] - mb) < 0.11), (kernel, nums[:4], mb)


def test_profile_traffic_only_for_the_bench_size():
    e = _traffic()["radix_pass_kernel"]
    got, src = bench.profile_traffic(e["bench_n"], "radix_pass_kernel")
    assert got == float(e["bytes_per_launch"]) and src == e["summary"]
    assert bench.profile_traffic(e["bench_n"] // 2, "radix_pass_kernel") == (None, None)
    assert bench.profile_traffic(e["bench_n"], "no_such_kernel") == (None, None)


def _sampler(text):
    c = bench.ClockSampler(None)
    c.proc = object()  # samples were taken
    c.text = text
    return c


def test_clock_summary_median_and_reasons():
    rows = [
        "0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1350.0, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1390.2, 0x0, Not Active, Not Active, Not Active, Not Active",
        "1, 900, 2070, 100.0, 0x40, Active, Active, Active, Not Active",  # another GPU
        "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active",  # unreadable
        "garbage line",
    ]
    s = _sampler("\n".join(rows)).summary(0)
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0
    assert s["reasons"] == ["sw_power_cap"]  # kept and noted, not a rejection
    assert s["samples"] == 3
    s1 = _sampler("\n".join(rows)).summary(1)
    assert s1["sm_mhz"] == 900.0
    assert s1["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown"]


def test_clock_summary_without_samples():
    c = bench.ClockSampler(None)
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    assert _sampler("").summary()["samples"] == 0


def test_peak_source():
    peak, src = bench.peaks()
    assert peak > 0 and src in ("measured", "fallback")
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        assert src == "measured" and peak == float(json.loads(p.read_text())["hbm_gbs"])
