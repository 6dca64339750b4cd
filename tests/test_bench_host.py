"""Host-side logic of bench.py that decides whether a timed run is kept: the summary of
the nvidia-smi clock samples taken during the timed region."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _line(sm, smax=2070, reasons=("Not Active",) * 4, power=900.5, mask="0x0000000000000000"):
    return ", ".join(["0", str(sm), str(smax), str(power), mask] + list(reasons)) + "\n"


def test_clean_samples():
    s = bench.clock_summary([_line(2070), _line(2055), _line(2070)])
    assert s == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": [], "samples": 3}


def test_reasons_are_collected_and_not_active_ignored():
    lines = [_line(1980, reasons=("Not Active", "Not Active", "Not Active", "Active")),
             _line(1700, reasons=("Active", "Not Active", "Active", "Not Active")),
             _line(2070)]
    s = bench.clock_summary(lines)
    assert s["reasons"] == ["hw_slowdown", "sw_power_cap", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1980.0 and s["samples"] == 3


def test_non_sample_lines_are_skipped():
    lines = ["\n", "No devices were found\n", "0, [N/A], 2070, 1.0, 0x0, a, b, c, d\n",
             _line(2000)]
    s = bench.clock_summary(lines)
    assert s["samples"] == 1 and s["sm_mhz"] == 2000.0


def test_no_samples():
    assert bench.clock_summary([]) == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                                       "samples": 0}
