"""bench.py's host-side pieces on the CPU: the profiled DRAM traffic it reads
from profiles/ for the roofline, the clock-sample summary that flags a run
(slowdown reasons, median SM clock), the HBM roofline arithmetic and the
workload's config keys."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_profiled_traffic_of_the_bench_shapes():
    """The bench workload's committed ncu traffic lines exist for the shapes
    the autotuner picks among, and are read as bytes per launch."""
    wl = "zeldovich128_z50_nd128_monopole"
    t16 = bench.profiled_traffic(wl, {"kernel": "batched", "group": 16, "leaf_threads": 128})
    t32 = bench.profiled_traffic(wl, {"kernel": "batched", "group": 32, "leaf_threads": 128})
    tpl = bench.profiled_traffic(wl, {"kernel": "plain", "group": 32, "leaf_threads": 128})
    for t in (t16, t32, tpl):
        assert isinstance(t, int) and 1e8 < t < 1e9, t
    assert bench.profiled_traffic("no_such_workload", {"kernel": "batched", "group": 16,
                                                       "leaf_threads": 128}) is None


def _sampler(lines):
    s = bench.ClockSampler(0)
    s.out = "\n".join(lines)
    return s.summary()


def test_clock_summary_median_and_reasons():
    ok = "2070, 2070, 900.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"
    capped = "1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    hot = "1500, 2070, 1300.0, 0x0000000000000020, Not Active, Not Active, Active, Not Active"
    s = _sampler([ok, ok, capped])
    assert s["sm_mhz"] == 2070 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]
    s = _sampler([ok, hot, "garbage line", "N/A, N/A, 1, 2, 3, 4, 5, 6"])
    assert s["samples"] == 2 and "sw_thermal_slowdown" in s["reasons"]
    assert _sampler([])["reasons"] == ["unsampled"]


def test_hbm_roofline_arithmetic(tmp_path, monkeypatch):
    r = bench.hbm_roofline(228523264, 0.9)
    assert r["bound"] == "hbm" and r["unit"] == "GB/s"
    assert r["achieved"] == pytest.approx(228523264 / 0.9e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / r["peak"])
    assert bench.hbm_roofline(None, 0.9) is None
    # without the measured peaks file: the stated fallback
    monkeypatch.setattr(bench, "ROOT", str(tmp_path))
    r = bench.hbm_roofline(1e9, 1.0)
    assert r["peak"] == 6800.0 and r["peak_source"].startswith("fallback")


def test_workload_config_names_the_workload():
    p, kp, cfg = bench.workload(16, 32)
    assert cfg["workload"] == "zeldovich16_z50_nd32_monopole"
    assert cfg["n_particles"] == p.n and cfg["nd"] == 32 and cfg["tdpts"] == 1
    assert cfg["law"] == "poly6" and "l2" in cfg
    assert bench.METRIC == "pair interactions/s" and bench.UNIT == "pairs/s"
