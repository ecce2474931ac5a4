"""Host helpers of bench.py (no GPU): the DRAM traffic per sweep read from the
committed ncu summary, and the clock record's summary (median SM clock, the
throttle reasons seen)."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_profile_traffic_reads_the_sweep_summary():
    per_sweep, note = bench.profile_traffic("tfce_sweep")
    assert per_sweep is not None and 5.24e6 < per_sweep < 1e8  # above the algorithmic bytes
    assert "profiles/tfce_sweep" in note
    assert bench.profile_traffic("no_such_kernel") == (None, None)


def test_clock_summary():
    c = bench.ClockSampler()
    c.lines = [
        "0, 2070 MHz, 2070 MHz, 900 W, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2055, 2070, 1300, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2070, 2070, 1100, 0x0, Not Active, Not Active, Not Active, Not Active",
        "index, clocks.sm [MHz], ...",  # a header line is skipped
    ]
    c.lines[0] = c.lines[0].replace(" MHz", "")
    s = c.summary()
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    empty = bench.ClockSampler()
    assert empty.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
