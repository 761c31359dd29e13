"""The bounds-checked build (libdfcsr_gb300_checked.so: every kernel tests
its computed global-memory indices and records the first failure in a
device status word instead of accessing out of range; compute-sanitizer is
not available here).

* The mechanism: dfcsr_bounds_probe tests an index against a size through
  the same check without touching memory; an index past the end is reported
  with its site and value, one inside is not, and a reset clears it.
* The wake path's kernels, run through the checked library on the cases of
  tests/checked_build_workload.py (the kick loop in both precisions, the
  4-region branch with the near band, observers past the lattice end,
  off-grid deposits, interpolation queries outside their grids), record no
  failure, and give the release library's results (<= 1e-12 of each
  result's peak; NaN exactly where the release library gives NaN).
"""
import os
import subprocess
import sys

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROBE = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
from pydfcsr_gb300 import _lib
lib = _lib.load()
assert lib.dfcsr_bounds_checked() == 1
assert _lib.bounds_status(reset=True) is None
_lib.call("dfcsr_bounds_probe", 2, 3, 77, None)
assert _lib.bounds_status() is None
_lib.call("dfcsr_bounds_probe", 5, 3, 77, None)
_lib.call("dfcsr_bounds_probe", -4, 3, 78, None)      # the first failure is kept
assert _lib.bounds_status(reset=True) == (77, 5), _lib.bounds_status()
assert _lib.bounds_status() is None
_lib.call("dfcsr_bounds_probe", -4, 3, 78, None)
assert _lib.bounds_status(reset=True) == (78, -4)
print("probe ok")
"""


def _env(checked):
    env = dict(os.environ)
    env.pop("DFCSR_GB300_CHECKED", None)
    if checked:
        env["DFCSR_GB300_CHECKED"] = "1"
    return env


@cuda
def test_checked_build_probe_reports_site_and_index():
    from pydfcsr_gb300 import build
    build.build(checked=True)
    r = subprocess.run([sys.executable, "-c", PROBE, ROOT], env=_env(True), capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "probe ok" in r.stdout


@cuda
def test_checked_build_wake_path_in_bounds_and_equal(tmp_path):
    from pydfcsr_gb300 import build
    build.build_all()
    res = {}
    for checked in (False, True):
        f = tmp_path / f"out_{int(checked)}.npz"
        r = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "checked_build_workload.py"),
                            str(f)], env=_env(checked), capture_output=True, text=True, timeout=1200)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
        res[checked] = dict(np.load(f))
    assert int(res[True]["checked"]) == 1 and int(res[False]["checked"]) == 0
    assert tuple(res[True]["bounds"]) == (-1, -1), res[True]["bounds"]
    for key, ref in res[False].items():
        if key in ("checked", "bounds"):
            continue
        got = res[True][key]
        assert got.shape == ref.shape, key
        assert np.array_equal(np.isnan(got), np.isnan(ref)), key
        ok = ~np.isnan(ref)
        scale = float(np.max(np.abs(ref[ok]))) if ok.any() else 0.0
        err = float(np.max(np.abs(got[ok] - ref[ok]))) if ok.any() else 0.0
        assert err <= 1e-12 * max(scale, 1e-300), (key, err, scale)
