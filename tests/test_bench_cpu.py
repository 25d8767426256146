"""Host-side helpers of bench.py that shape its JSON line: the clock summary
of the timed region, the roofline traffic figure and the peak source.  No
GPU: the clock sampler is fed recorded samples, as `nvidia-smi` would."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _sampler(samples):
    clk = bench.ClockSampler()
    clk.samples = list(samples)
    return clk


def test_clock_summary_skips_idle_samples_and_names_reasons():
    # (sm MHz, max sm MHz, power W, reasons bit mask)
    clk = _sampler([
        (345.0, 2070.0, 120.0, 0x1),    # idle before the timed region
        (2070.0, 2070.0, 900.0, 0x0),
        (2055.0, 2070.0, 1290.0, 0x4),  # power cap under load
        (1980.0, 2070.0, 1300.0, 0x4),
        (2070.0, 2070.0, 950.0, 0x0),
    ])
    s = clk.summary()
    assert s["samples"] == 4
    assert s["sm_mhz"] == (2055.0 + 2070.0) / 2  # the median of the four busy samples
    assert s["sm_max_mhz"] == 2070.0
    assert s["power_w_max"] == 1300.0
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_slowdowns():
    clk = _sampler([(1500.0, 2070.0, 1000.0, 0x8 | 0x40), (1600.0, 2070.0, 1000.0, 0x20)])
    assert clk.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown",
                                        "sw_thermal_slowdown"]


def test_clock_summary_all_idle_keeps_the_samples():
    s = _sampler([(345.0, 2070.0, 100.0, 0x1)] * 3).summary()
    assert s["samples"] == 3 and s["reasons"] == ["gpu_idle"]


def test_clock_summary_without_samples_says_unavailable():
    s = _sampler([]).summary()
    assert s["sm_mhz"] is None and s["reasons"] == ["unavailable"]


def test_roofline_traffic_comes_from_the_committed_capture():
    # profiles/traffic.txt: per-launch DRAM bytes of each tensor-core kernel,
    # close to the 2 x 2^30 x 8 B = 17.18 GB a 30-qubit block pass moves
    for cls in ("block_tc7", "block_tc"):
        t = bench.ncu_traffic(cls)
        assert t is not None and 0.9 * 17.18e9 < t < 1.05 * 17.18e9, (cls, t)
    assert bench.ncu_traffic("no_such_kernel") is None


def test_peak_source_is_named():
    p = bench.measured_peaks()
    assert p["source"] in ("measured", "fallback") and p["hbm_gbs"] > 0
