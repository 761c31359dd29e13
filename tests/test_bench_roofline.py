"""The benchmark's roofline arithmetic (host only): integrand points counted
per timed step from the branch each step took, the FP32 operation rate
against the measured peak, and the instruction-issue ceiling; and the
reference arm's JSON line, run on the CPU."""
from types import SimpleNamespace

import pytest

import bench


def _wl():
    return SimpleNamespace(integration={"xbins": 100, "zbins": 100})


def test_integrand_points_follow_each_steps_branch():
    run = SimpleNamespace(branch_log={25: False, 26: False, 35: True, 36: True})
    per = 100 * 100
    assert bench.integrand_points(_wl(), run, [25]) == 4 * per
    assert bench.integrand_points(_wl(), run, [35]) == 5 * per
    assert bench.integrand_points(_wl(), run, [25, 26, 35, 36]) == (4 + 4 + 5 + 5) * per


def test_roofline_mixed_fields():
    npts, launches = 4096, 2
    per_obs_total = 2 * 5 * 100 * 100                 # two 4-region steps
    r = bench.roofline("wake_mixed_integral", 1.7, launches, per_obs_total, npts,
                       {"fp32_tflops": 75.0, "fp64_tflops": 1.0}, 6786.2, "mixed", 2070.0, 152)
    pts = npts * per_obs_total / launches
    assert r["integrand_points_per_launch"] == pytest.approx(2.048e8)
    assert r["achieved"] == pytest.approx(bench.INTEGRAL_FLOPS_PER_POINT * pts / 1.7e-3 / 1e12)
    assert r["frac"] == pytest.approx(r["achieved"] / 75.0)
    assert r["traffic"] == pytest.approx(bench.INTEGRAL_DRAM_BYTES_PER_POINT * pts)
    ideal_ms = bench.INTEGRAL_WARP_INSTR_PER_POINT * pts / (152 * 4 * 2070e6) * 1e3
    assert r["issue"]["ideal_ms"] == pytest.approx(ideal_ms)
    assert r["issue"]["frac"] == pytest.approx(ideal_ms / 1.7)
    assert 0.0 < r["issue"]["frac"] < 1.0
    assert r["bound"] == "fp32" and r["unit"] == "TFLOP/s"


def test_issue_bound_needs_a_clock():
    assert bench.issue_bound(1e6, 1.0, None, 152) is None


def test_reference_arm_line_on_cpu():
    """`bench.py --impl reference` (the reference's CPU algorithm, the
    oracle here, on the host cores) prints one JSON line with the GPU arm's
    metric, unit and direction, impl "reference", its cpu_baseline and an
    e2e object without host<->device bytes.  A small beam keeps it short."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1", "--particles", "20000"],
                       capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]
