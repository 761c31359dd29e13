"""pydfcsr_gb300.interfaces against the reference's interfaces.py.

tests/golden/interfaces.npz was recorded by running the reference's own
functions (make_golden.py, gen_interfaces): openPMD -> bmadx coordinates and
bmadx -> openPMD data from numpy and torch particles.  Unit conversions
only, so the results must be bitwise equal.
"""
import types

import numpy as np
import pytest
import torch

from pydfcsr_gb300 import interfaces as I
from tests.helpers import golden

KEYS = ("x", "px", "y", "py", "z", "pz", "t", "weight")


def _pmd(g):
    return types.SimpleNamespace(**{k: g[k] for k in ("x", "px", "y", "py", "z", "p")})


def test_openpmd_to_bmadx_matches_reference():
    g = golden("interfaces.npz")
    p0c = float(g["p0c"])
    assert np.array_equal(np.array(I.openpmd_to_bmadx_coords(_pmd(g), p0c)), g["coords"])
    part = I.openpmd_to_bmadx_particles(_pmd(g), p0c, s=float(g["s"]))
    assert part.s == float(g["s"]) and part.p0c == p0c and part.mc2 == float(g["mc2"])
    assert np.array_equal(np.array(part[:6]), g["coords"])


@pytest.mark.parametrize("kind", ["numpy", "torch"])
def test_bmadx_to_openpmd_matches_reference(kind):
    g = golden("interfaces.npz")
    coords = [c.copy() for c in g["coords"]]
    if kind == "torch":
        coords = [torch.from_numpy(c) for c in coords]
    part = I.Particle(*coords, s=float(g["s"]), p0c=float(g["p0c"]), mc2=I.M_ELECTRON)
    dat = I.bmadx_particles_to_openpmd(part, float(g["charge"]))
    assert np.array_equal(np.array([dat[k] for k in KEYS]), g[f"pmd_{kind}"])
    assert dat["species"] == "electron"
    assert dat["status"].dtype.kind == "i" and (dat["status"] == 1).all()


def test_bmadx_to_openpmd_refusals():
    x = np.zeros(3)
    with pytest.raises(ValueError, match="electrons"):
        I.bmadx_particles_to_openpmd(I.Particle(x, x, x, x, x, x, 0.0, 1e9, 938.272e6), 1e-9)
    with pytest.raises(ValueError, match="numpy and torch"):
        lst = [0.0, 0.0]
        I.bmadx_particles_to_openpmd(I.Particle(lst, lst, lst, lst, lst, lst, 0.0, 1e9,
                                                I.M_ELECTRON), 1e-9)
