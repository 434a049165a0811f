"""Host-side pieces of bench.py's measurement, without a GPU: the summary of
the clock record (median SM clock, throttle reasons), the per-launch DRAM
traffic read from the committed ncu summaries, and the HBM peak."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), ".."))
import bench  # noqa: E402


def test_clock_summary_reports_median_and_reasons(tmp_path):
    s = bench.ClockSampler(0, "test")
    s.path = str(tmp_path / "clocks.csv")
    rows = ["0, 2070, 2070, 900.0, 0x0, Not Active, Not Active, Not Active, Not Active",
            "0, 2040, 2070, 1300.0, 0x4, Not Active, Not Active, Not Active, Active",
            "0, 2070, 2070, 1200.0, 0x0, Not Active, Not Active, Not Active, Not Active",
            "a line that is not a sample"]
    with open(s.path, "w") as f:
        f.write("\n".join(rows) + "\n")
    s.proc = object()      # as if nvidia-smi had been sampling
    assert s.summary() == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "samples": 3, "reasons": ["sw_power_cap"]}
    assert not os.path.exists(s.path)


def test_clock_summary_without_a_sampler_is_none():
    assert bench.ClockSampler(0, "unused").summary() is None


def test_profiled_traffic_reads_the_committed_summaries():
    assert bench.profiled_traffic("bp_fdk_walk_kernel", "dd_pair") == 3.66e9
    assert bench.profiled_traffic("dd_forward_tma_kernel", "dd_pair") == 2.38e9
    assert bench.profiled_traffic("bp_fdk_integ_kernel", "dd384") == 7.63e9
    # another workload's capture is not borrowed
    assert bench.profiled_traffic("bp_fdk_walk_kernel", "fdk128") is None
    assert bench.profiled_traffic("no_such_kernel", "dd_pair") is None


def test_measured_peak():
    peak, kind = bench.measured_peaks()
    assert peak > 0 and kind in ("measured", "fallback")
