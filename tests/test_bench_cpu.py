"""bench.py's host-side pieces without a GPU: the clock record, the per-class roofline table,
the workload sharding and the JSON contract of the reference arm.

The clock record decides whether a run is kept: a sample with hw_slowdown, hw_thermal_slowdown or
sw_thermal_slowdown active must show up in `reasons`, and the SM clock reported is the median
under load.  The class table turns the library's per-class algorithmic bytes and event times
into GB/s, a fraction of the HBM peak and a share of kernel time.
"""
import importlib.util
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _clock_rows(rows):
    # index, sm, sm max, power, active, hw_slowdown, hw_thermal, sw_thermal, sw_power_cap
    return "\n".join(", ".join(str(v) for v in r) for r in rows) + "\n"


def test_clock_summary_median_and_reasons(bench, tmp_path):
    cs = bench.ClockSampler(0)
    cs.path = str(tmp_path / "clocks.csv")
    with open(cs.path, "w") as f:
        f.write(_clock_rows([
            (0, 2070, 2070, 900.0, "0x0", "Not Active", "Not Active", "Not Active", "Not Active"),
            (0, 1980, 2070, 1400.0, "0x4", "Not Active", "Not Active", "Not Active", "Active"),
            (0, 2070, 2070, 1100.0, "0x0", "Not Active", "Not Active", "Not Active", "Not Active"),
            (0, "[N/A]", 2070, 0.0, "0x0", "Not Active", "Not Active", "Not Active", "Not Active"),
        ]))
    s = cs.summary()
    assert s["sm_mhz"] == 2070.0 and s["sm_max_mhz"] == 2070.0 and s["samples"] == 3
    assert s["reasons"] == ["sw_power_cap"]


def test_clock_summary_flags_thermal_slowdown(bench, tmp_path):
    cs = bench.ClockSampler(0)
    cs.path = str(tmp_path / "clocks.csv")
    with open(cs.path, "w") as f:
        f.write(_clock_rows([
            (0, 1500, 2070, 1000.0, "0x40", "Not Active", "Active", "Not Active", "Not Active"),
            (0, 1600, 2070, 1000.0, "0x20", "Not Active", "Not Active", "Active", "Not Active"),
        ]))
    s = cs.summary()
    assert s["reasons"] == ["hw_thermal_slowdown", "sw_thermal_slowdown"]
    assert s["sm_mhz"] == 1550.0


def test_clock_summary_without_nvidia_smi(bench):
    cs = bench.ClockSampler(0)
    assert cs.summary()["reasons"] == ["nvidia-smi unavailable"]


def test_class_table_rates_fractions_shares(bench):
    prof = {"update": {"bytes": 6e9, "ms": 1.0, "launches": 3},
            "projection": {"bytes": 3e9, "ms": 1.0, "launches": 2},
            "svd": {"bytes": 0.0, "ms": 2.0, "launches": 1},
            "unused": {"bytes": 0.0, "ms": 0.0, "launches": 0}}
    t = bench.class_table(prof, 6000.0)
    assert set(t) == {"update", "projection", "svd"}
    assert t["update"]["GB/s"] == pytest.approx(6000.0) and t["update"]["frac"] == pytest.approx(1.0)
    assert t["projection"]["frac"] == pytest.approx(0.5)
    assert t["svd"]["GB/s"] == 0.0 and t["svd"]["frac"] is None
    assert sum(v["share"] for v in t.values()) == pytest.approx(1.0)
    assert t["svd"]["share"] == pytest.approx(0.5)


def test_ranks_solve_disjoint_right_hand_sides(bench):
    import problems
    seeds = [set(problems.shard_seeds(4, r)) for r in range(3)]
    assert all(len(s) == 4 for s in seeds)
    assert not (seeds[0] & seeds[1]) and not (seeds[1] & seeds[2]) and not (seeds[0] & seeds[2])


def test_reference_arm_prints_one_json_line():
    # the reference arm (the oracle port on the host cores) on the same workload at a 24^3 grid:
    # a full calibration solve, then one step of two deflated cycles; one JSON line with the
    # contract's keys, e2e equal to its own value, no host-device traffic
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--ref-cycles", "2", "--grid", "24"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "solves/s" and d["value"] > 0
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert np.isfinite(d["ms_per_step"])
    # solves/s = 1 / (seconds per deflated cycle x the calibration solve's cycle count)
    cal = d["calibration"]
    assert cal["status"] == 0 and cal["relative_residual"] <= 1e-10 and cal["cycles"] > 1
    assert d["config"]["grid"] == [24, 24, 24] and d["config"]["n"] == 24 ** 3
