"""r_gen6 (host FP64 transfer matrices that carry the synthetic beams between
wake steps) against the reference's r_gen6 (pyDFCSR_2D/r_gen6.py:4-122).

* tests/golden/r_gen6.npz holds the reference's matrices for drifts, sector
  and rectangular bends with pole-face edges and a fringe-field half gap,
  quadrupoles of both signs, combined-function magnets, rolls and the pure
  rotation, generated by running the reference (make_golden.py).
* The reference's BmadX tracking notebook (test/test_BmadX_tracking.ipynb)
  records R @ (1e-3 * ones(6)) for a drift (L = 1), a sector bend (L = 0.1,
  angle = 0.05, E2 = 0.1) and a quadrupole (L = 0.1, k1 = 10), printed to
  eight significant digits; those printed vectors are the known answers.
"""
import numpy as np
import pytest

from pydfcsr_gb300.r_gen6 import r_gen6
from tests.helpers import golden

# the notebook's printed outputs (np.matmul(r6, coords), coords = 1e-3 * ones(6))
# and half a unit of the last printed digit: numpy prints the drift's values
# in their shortest exact form, the bend's with 8 decimals, the quad's in
# scientific notation with 8 decimals in the mantissa
NOTEBOOK = [
    ((1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0), [0.002, 0.001, 0.002, 0.001, 0.001, 0.001], "exact"),
    ((0.1, 0.05, 0.0, 0.0, 0.0, 0.1, 0.0),
     [0.00110121, 0.00107898, 0.0011, 0.00094482, 0.00094748, 0.001], "fixed"),
    ((0.1, 0.0, 10.0, 0.0, 0.0, 0.0, 0.0),
     [1.04875693e-03, -3.30011883e-05, 1.15209308e-03, 2.06716826e-03, 1.0e-03, 1.0e-03],
     "scientific"),
]


def _mat(c):
    L, angle, k1, roll, E1, E2, hgap = (float(v) for v in c)
    return r_gen6(L, angle=angle, k1=k1, roll=roll, E1=E1, E2=E2, hgap=hgap)


@pytest.mark.parametrize("case, want, fmt", NOTEBOOK)
def test_notebook_known_answers(case, want, fmt):
    got = _mat(case) @ (np.ones(6) * 1e-3)
    want = np.array(want)
    if fmt == "exact":
        tol = np.full(6, 1e-18)
    elif fmt == "fixed":
        tol = np.full(6, 0.5e-8)
    else:
        tol = 0.5e-8 * 10.0 ** np.floor(np.log10(np.abs(want)))
    assert np.all(np.abs(got - want) <= tol), (got, want)


def test_matrices_match_reference():
    g = golden("r_gen6.npz")
    for c, ref in zip(g["cases"], g["mats"]):
        got = _mat(c)
        scale = max(1.0, float(np.abs(ref).max()))
        assert np.max(np.abs(got - ref)) <= 4e-16 * scale, (c, np.max(np.abs(got - ref)))


def test_tracked_vectors_match_reference():
    g = golden("r_gen6.npz")
    for c, ref in zip(g["cases"][:3], g["tracked"]):
        got = _mat(c) @ (np.ones(6) * 1e-3)
        assert np.max(np.abs(got - ref)) <= 1e-18, (c, got, ref)
