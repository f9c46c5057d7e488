"""The benchmark's host logic on CPU: workload names and the clock record
(timestamped nvidia-smi samples kept only inside the timed region)."""
import datetime
import os
import sys
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_dam_mix_workloads_take_any_scene_count():
    import bench
    _, two, scaling = bench.workload("dam_mix2")
    assert len(two) == 2 and all(len(s["positions"]) == 1_000_000 for s in two) and scaling == "weak"
    _, r0, _ = bench.workload("dam_mix2", rank=0, world=2)
    _, r1, _ = bench.workload("dam_mix2", rank=1, world=2)  # the job's four seeds, two per rank
    assert len(r0) == len(r1) == 2
    seen = [s["positions"][:4].tobytes() for s in r0 + r1]
    assert len(set(seen)) == 4
    for bad in ("dam_mix0", "dam_mix", "dam_mixx", "nope"):
        with pytest.raises(SystemExit):
            bench.workload(bad)


def test_reached_fraction_needs_both_residuals():
    import bench
    assert bench.reached_fraction([1e-5, 1e-5], [0.01, 0.03], 2e-5, 0.02) == 0.5
    assert bench.reached_fraction([3e-5, 1e-5], [0.01, 0.01], 2e-5, 0.02) == 0.5
    assert bench.reached_fraction([1e-5], [0.0], 2e-5, 0.02) == 1.0


def _line(t, sm, slowdown="Not Active", power_cap="Not Active"):
    ts = datetime.datetime.fromtimestamp(t).strftime("%Y/%m/%d %H:%M:%S.%f")[:-3]
    return f"{ts}, 0, {sm}, 2070, 1200.00, 0x0000000000000000, {slowdown}, Not Active, Not Active, {power_cap}"


def test_clock_samples_outside_the_timed_region_are_dropped():
    import bench
    t0 = time.time()
    out = "\n".join([
        _line(t0 - 1.0, 345, slowdown="Active"),  # idle, before the region
        _line(t0 + 0.10, 2070),
        _line(t0 + 0.15, 2062, power_cap="Active"),
        _line(t0 + 0.20, 2070),
        _line(t0 + 2.0, 900),                     # after the region
        "garbage line",
    ])
    c = bench.Clocks.summarise(out, t0, t0 + 0.3)
    assert c["samples_in_region"] == 3 and c["samples"] == 3
    assert c["sm_mhz"] == 2070 and c["sm_max_mhz"] == 2070
    assert c["reasons"] == ["sw_power_cap"]  # the slowdown before the region is not counted


def test_clock_record_without_samples_in_the_region_keeps_all():
    import bench
    t0 = time.time()
    c = bench.Clocks.summarise(_line(t0 - 5, 2070), t0, t0 + 0.01)
    assert c["samples_in_region"] == 0 and c["samples"] == 1 and c["sm_mhz"] == 2070
