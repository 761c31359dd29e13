"""Particle steps around the wake on the GPU: linear transport and
Beam.apply_wakes (beams.py:108-131), against the reference's own output
(tests/golden/apply_wakes.npz) and the CPU oracle.

Tolerances: apply_wakes through the C ABI with the reference's polyfit slope
is compared bit for bit with the reference.  Through ``Beam`` the slope comes
from the device moments (not numpy.polyfit), so x_transform moves by a few
ulps; the kicks are then compared at 1e-12 of their largest value.  Transport
is a fused multiply-add chain: 1e-15 relative to each row's scale.
"""
import ctypes

import numpy as np
import pytest

from oracle import oracle as O
from tests.helpers import golden

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _call_apply(coords, g, transverse, slope):
    torch = _torch()
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import ptr, stream_handle
    c = torch.as_tensor(np.ascontiguousarray(coords), device="cuda")
    dE = torch.as_tensor(g["dE_dct"], device="cuda")
    xk = torch.as_tensor(g["x_kick"], device="cuda")
    xr = torch.as_tensor(g["xrange"], device="cuda")
    zr = torch.as_tensor(g["zrange"], device="cuda")
    nx, nz = xr.numel(), zr.numel()
    ws = torch.empty(_lib.query("dfcsr_apply_wakes_workspace_bytes", nx, nz), dtype=torch.uint8,
                     device="cuda")
    _lib.call("dfcsr_apply_wakes", ptr(c), c.shape[1], c.stride(0), ptr(dE), ptr(xk), ptr(xr),
              ptr(zr), nx, nz, float(slope[0]), float(slope[1]), float(g["step_size"]),
              float(g["init_energy"]), 1 if transverse else 0, ptr(ws), ws.numel(),
              stream_handle())
    return c.cpu().numpy()


def test_apply_wakes_capi_matches_reference():
    g = golden("apply_wakes.npz")
    for tag, transverse in (("t", True), ("l", False)):
        out = _call_apply(g["coords"], g, transverse, g["slope"])
        ref = g[f"out_{tag}"]
        np.testing.assert_array_equal(out, ref)


@pytest.mark.parametrize("slope", [(0.0, 0.0), (-0.37, 2.5e-6)])
def test_apply_wakes_capi_bitexact_large(slope):
    """600,000 particles against the oracle bit for bit: random positions
    over and beyond a 64 x 80 mesh, particles exactly on grid lines and on
    the end points (with slope 0, x_transform = x exactly), and x = -0.  The
    kernel's weights come from per-interval reciprocals and one FMA
    correction, which must reproduce the reference's divisions exactly."""
    rng = np.random.default_rng(11)
    nx, nz, n = 64, 80, 600_000
    xr = np.linspace(-3.1e-5, 2.9e-5, nx)
    zr = np.linspace(-1.6e-4, 1.4e-4, nz)
    c = np.zeros((6, n))
    c[0] = rng.uniform(-3.6e-5, 3.4e-5, n)
    c[4] = rng.uniform(-1.8e-4, 1.6e-4, n)
    c[1] = rng.normal(0, 1e-6, n)
    c[5] = rng.normal(0, 1e-4, n)
    k = n // 8
    c[0, :k] = xr[rng.integers(0, nx, k)]
    c[4, k:2 * k] = zr[rng.integers(0, nz, k)]
    c[0, 2 * k:2 * k + 4], c[4, 2 * k:2 * k + 4] = [xr[0], xr[-1], xr[0], xr[-1]], [zr[0], zr[-1], zr[-1], zr[0]]
    c[0, 2 * k + 4] = -0.0
    g = {"dE_dct": rng.normal(0, 3e3, (nx, nz)), "x_kick": rng.normal(0, 1e2, (nx, nz)),
         "xrange": xr, "zrange": zr, "step_size": 0.013, "init_energy": 1e9}
    for transverse in (True, False):
        out = _call_apply(c, g, transverse, slope)
        ref = O.apply_wakes(c, g["dE_dct"], g["x_kick"], xr, zr, g["step_size"], g["init_energy"],
                            transverse, np.array(slope))
        np.testing.assert_array_equal(out, ref)


def test_beam_apply_wakes_vs_oracle():
    from pydfcsr_gb300.beams import Beam
    g = golden("apply_wakes.npz")
    b = Beam(g["coords"], charge=1e-9, energy=float(g["init_energy"]))
    slope = b.slope
    b.apply_wakes(g["dE_dct"], g["x_kick"], g["xrange"], g["zrange"], float(g["step_size"]), True)
    out = b.particle.cpu().numpy()
    ref = O.apply_wakes(g["coords"], g["dE_dct"], g["x_kick"], g["xrange"], g["zrange"],
                        float(g["step_size"]), float(g["init_energy"]), True, slope)
    for row in (1, 5):
        kick = ref[row] - g["coords"][row]
        scale = np.abs(kick).max()
        assert scale > 0
        assert np.abs(out[row] - ref[row]).max() <= 1e-12 * scale
    for row in (0, 2, 3, 4):
        np.testing.assert_array_equal(out[row], g["coords"][row])
    # statistics were refreshed from the kicked particles
    assert b._moments is not None


def test_apply_wakes_empty_and_bad_args():
    torch = _torch()
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import ptr, stream_handle
    c = torch.zeros((6, 0), dtype=torch.float64, device="cuda")
    _lib.call("dfcsr_apply_wakes", ptr(c), 0, 0, None, None, None, None, 4, 4, 0.0, 0.0, 1.0,
              1e9, 0, None, 0, stream_handle())
    with pytest.raises(ValueError):
        _lib.call("dfcsr_apply_wakes", ptr(c), 0, 0, None, None, None, None, 1, 4, 0.0, 0.0, 1.0,
                  1e9, 0, None, 0, stream_handle())


def test_transport_matches_numpy():
    torch = _torch()
    from pydfcsr_gb300.beams import Beam
    from pydfcsr_gb300.synthetic import StepPlan, chicane_lattice, gaussian_beam
    plan = StepPlan(chicane_lattice(0.13))
    coords = gaussian_beam(100_003, 20e-6, 50e-6, 1e-4, 5e-6, -10.0, seed=9)
    dev = torch.as_tensor(coords, device="cuda")
    b = Beam(dev)
    ref = coords.copy()
    for k in (1, 4, 17, 30):
        R = plan.matrix(k)
        b.track(R, 0.13)
        ref = R @ ref
    out = b.particle.cpu().numpy()
    for r in range(6):
        scale = np.abs(ref[r]).max()
        assert np.abs(out[r] - ref[r]).max() <= 1e-15 * 8 * scale, r
    # the caller's tensor is not modified by the in-place updates
    np.testing.assert_array_equal(dev.cpu().numpy(), coords)
    assert b.position == pytest.approx(4 * 0.13)


def test_transport_strided_rows():
    """ld > n: only the first n columns of each row move."""
    torch = _torch()
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import ptr, stream_handle
    rng = np.random.default_rng(3)
    R = rng.normal(size=(6, 6))
    R[0, 3] = R[2, 5] = 0.0
    full = rng.normal(size=(6, 1000))
    t = torch.as_tensor(full, device="cuda")
    Rh = np.ascontiguousarray(R)
    _lib.call("dfcsr_transport6", Rh.ctypes.data_as(ctypes.c_void_p), ptr(t), 700, 1000,
              stream_handle())
    out = t.cpu().numpy()
    ref = R @ full[:, :700]
    assert np.abs(out[:, :700] - ref).max() <= 1e-14 * np.abs(ref).max()
    np.testing.assert_array_equal(out[:, 700:], full[:, 700:])


def test_beam_from_and_to_particle():
    """Beam.from_particle / to_particle: a bmadx-style Particle (numpy or
    torch arrays) in, the same coordinates, energy and position out, ready
    for interfaces.bmadx_particles_to_openpmd."""
    torch = _torch()
    from pydfcsr_gb300 import interfaces as I
    from pydfcsr_gb300.beams import Beam
    rng = np.random.default_rng(9)
    c = rng.normal(0, 1e-4, (6, 1000))
    for arrays in ([r.copy() for r in c], [torch.from_numpy(r.copy()) for r in c]):
        part = I.Particle(*arrays, s=0.25, p0c=1.2e9, mc2=I.M_ELECTRON)
        beam = Beam.from_particle(part, charge=2e-9)
        assert beam.position == 0.25 and beam.init_energy == 1.2e9 and beam.charge == 2e-9
        back = beam.to_particle()
        assert np.array_equal(np.array(back[:6]), c)
        assert back.s == 0.25 and back.p0c == 1.2e9 and back.mc2 == I.M_ELECTRON
        dat = I.bmadx_particles_to_openpmd(back, 2e-9)
        assert np.allclose(dat["weight"].sum(), 2e-9)
