"""Seeded synthetic beams and lattices for the five wake-path workloads.

The reference builds its beams with distgen (Hammersley sequences) and tracks
them with bmadx; neither ships with it.  These seeded numpy generators stand in
for them, and ``r_gen6`` FP64 linear optics carries the beam between wake
steps, so the device path and the CPU oracle always consume identical
particles.

Workloads (names follow the physics, sizes are the defaults used by the tests
and the benchmark):

* ``dipole_c1``  - one 0.3 m dipole of radius 1.5 m (0.2 rad), 1 GeV,
  5e5 Gaussian particles, sigma_z 20 um, sigma_x 10 um, sigma_delta 1e-4,
  zero chirp; 128x128 deposit, SG window 9 order 2, 1 mm steps, 32x32 mesh.
  A 20 mm drift follows the dipole so that the reference-orbit tables cover
  the s' window of observation points at the exit.
* ``chicane_c2`` - four 0.5 m dipoles at +-0.05 rad with 2 m / 0.5 m / 2 m
  drifts; 2e6 particles, sigma_z 50 um, sigma_x 20 um, chirp h = -10 1/m;
  256x256 deposit, 64x64 mesh, 100 steps.
* ``chicane_c3`` - the same chicane, 4e6 particles, double-horn current
  (flat top 100 um with Gaussian horns sigma 5 um at both ends, 3x the flat
  density), x Gaussian 15 um, chirp -10 1/m; 384x384 deposit, 96x96 mesh.
* ``serving_c4`` - request generator: single dipoles with rho ~ U(1, 20) m,
  angle ~ U(0.02, 0.2), N ~ logU(1e5, 4e6), sigma_z ~ U(10, 100) um, grid
  from {64, 128, 256, 512}^2, mesh side from {32, 64, 96, 128}.
* ``chicane_c5`` - 1e7 particles, sigma_z 30 um, sigma_x 10 um, chirp
  -20 1/m, 512x512 deposit, the chicane in 300 steps, 128x128 mesh.
"""
from collections import OrderedDict
from dataclasses import dataclass, field
import math

import numpy as np

from .r_gen6 import r_gen6

__all__ = ["Workload", "workload", "gaussian_beam", "gaussian_beam_device", "double_horn_beam",
           "dipole_lattice", "chicane_lattice", "StepPlan", "serving_requests"]

C_LIGHT = 299792458.0


def dipole_lattice(rho, length, step_size, tail_drift=0.02):
    """Reference-format lattice dict: ``step_size`` first, then elements."""
    lat = OrderedDict()
    lat["step_size"] = step_size
    lat["B1"] = {"type": "dipole", "L": length, "angle": length / rho,
                 "E1": 0.0, "E2": 0.0, "nsep": 1}
    if tail_drift > 0:
        lat["D1"] = {"type": "drift", "L": tail_drift, "nsep": 1}
    return lat


def chicane_lattice(step_size, angle=0.05, lb=0.5, d1=2.0, d2=0.5):
    lat = OrderedDict()
    lat["step_size"] = step_size
    lat["B1"] = {"type": "dipole", "L": lb, "angle": angle, "E1": 0.0, "E2": 0.0, "nsep": 1}
    lat["D1"] = {"type": "drift", "L": d1, "nsep": 1}
    lat["B2"] = {"type": "dipole", "L": lb, "angle": -angle, "E1": 0.0, "E2": 0.0, "nsep": 1}
    lat["D2"] = {"type": "drift", "L": d2, "nsep": 1}
    lat["B3"] = {"type": "dipole", "L": lb, "angle": -angle, "E1": 0.0, "E2": 0.0, "nsep": 1}
    lat["D3"] = {"type": "drift", "L": d1, "nsep": 1}
    lat["B4"] = {"type": "dipole", "L": lb, "angle": angle, "E1": 0.0, "E2": 0.0, "nsep": 1}
    return lat


def gaussian_beam(n, sigma_x, sigma_z, sigma_delta=1e-4, sigma_xp=5e-6,
                  chirp=0.0, seed=1):
    """6D coordinates (x, px, y, py, z, pz) as a (6, n) float64 array.

    z > 0 is the head.  pz = chirp * z + N(0, sigma_delta).
    """
    rng = np.random.default_rng(seed)
    out = np.empty((6, n))
    out[0] = rng.normal(0.0, sigma_x, n)
    out[1] = rng.normal(0.0, sigma_xp, n)
    out[2] = rng.normal(0.0, sigma_x, n)
    out[3] = rng.normal(0.0, sigma_xp, n)
    out[4] = rng.normal(0.0, sigma_z, n)
    out[5] = chirp * out[4] + rng.normal(0.0, sigma_delta, n)
    return out


def gaussian_beam_device(n, sigma_x, sigma_z, sigma_delta=1e-4, sigma_xp=5e-6, chirp=0.0,
                         seed=1, device=None):
    """``gaussian_beam`` drawn on the GPU from a seeded torch CUDA generator
    (same layout; not the same numbers as the numpy generator).  Used by the
    request stream, whose beams are too many to draw on the host."""
    import torch
    dev = device or torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device=dev)
    g.manual_seed(int(seed))
    out = torch.randn((6, n), generator=g, dtype=torch.float64, device=dev)
    scale = torch.tensor([sigma_x, sigma_xp, sigma_x, sigma_xp, sigma_z, sigma_delta],
                         dtype=torch.float64).to(dev, non_blocking=True)
    out.mul_(scale[:, None])
    if chirp:
        out[5].add_(out[4], alpha=chirp)
    return out


def double_horn_z(n, rng, flat=100e-6, horn_sigma=5e-6, horn_ratio=3.0):
    """Mixture sampler for a double-horn current profile.

    Flat top of full width ``flat`` centred on 0 with density 1; at each end a
    Gaussian horn of sigma ``horn_sigma`` whose peak density is ``horn_ratio``
    times the flat density.  Component weights follow from the areas:
    flat area = flat, each horn area = horn_ratio * sqrt(2 pi) * horn_sigma.
    """
    horn_area = horn_ratio * math.sqrt(2 * math.pi) * horn_sigma
    total = flat + 2 * horn_area
    comp = rng.choice(3, size=n, p=[flat / total, horn_area / total, horn_area / total])
    z = np.empty(n)
    m0 = comp == 0
    z[m0] = rng.uniform(-flat / 2, flat / 2, int(m0.sum()))
    m1 = comp == 1
    z[m1] = rng.normal(-flat / 2, horn_sigma, int(m1.sum()))
    m2 = comp == 2
    z[m2] = rng.normal(flat / 2, horn_sigma, int(m2.sum()))
    return z


def double_horn_beam(n, sigma_x=15e-6, sigma_delta=1e-4, sigma_xp=5e-6,
                     chirp=-10.0, seed=3):
    rng = np.random.default_rng(seed)
    out = np.empty((6, n))
    out[0] = rng.normal(0.0, sigma_x, n)
    out[1] = rng.normal(0.0, sigma_xp, n)
    out[2] = rng.normal(0.0, sigma_x, n)
    out[3] = rng.normal(0.0, sigma_xp, n)
    out[4] = double_horn_z(n, rng)
    out[5] = chirp * out[4] + rng.normal(0.0, sigma_delta, n)
    return out


def _element_pieces(lattice):
    """[(name, type, start, end, L, angle, E1, E2)] in lattice order."""
    pieces = []
    s = 0.0
    for name in list(lattice.keys())[1:]:
        e = lattice[name]
        L = float(e["L"])
        pieces.append((name, e["type"], s, s + L, L, float(e.get("angle", 0.0)),
                       float(e.get("E1", 0.0)), float(e.get("E2", 0.0))))
        s += L
    return pieces


class StepPlan:
    """Step positions, per-step transfer matrices and formation lengths.

    Positions follow ``Lattice.get_steps`` (``pyDFCSR_2D/lattice.py:152-173``):
    ``arange(0, L_total + step/2, step)``.  The matrix for step k transports
    from position k-1 to k and is the product of ``r_gen6`` pieces for each
    element the interval crosses; pole-face kicks apply only where the
    interval contains an element's entrance or exit.  Formation lengths follow
    ``CSR2D.run`` (``pyDFCSR_2D/CSR.py:246-270``): in and after a bend
    Lf = (24 R^2 * 5 sigma_z)^(1/3) with R of the latest bend; before the
    first bend Lf accumulates the drift lengths.
    """

    def __init__(self, lattice, n_steps=None):
        self.lattice = lattice
        self.step_size = float(lattice["step_size"])
        self.pieces = _element_pieces(lattice)
        total = self.pieces[-1][3]
        self.positions = np.arange(0, total + self.step_size / 2, self.step_size)
        if n_steps is not None:
            self.positions = self.positions[: n_steps + 1]
        self.total = total

    def element_at(self, s):
        for p in self.pieces:
            if s <= p[3] + 1e-12:
                return p
        return self.pieces[-1]

    def matrix(self, k):
        """Transfer matrix from positions[k-1] to positions[k]."""
        a, b = self.positions[k - 1], self.positions[k]
        m = np.eye(6)
        for (name, typ, s0, s1, L, angle, E1, E2) in self.pieces:
            lo, hi = max(a, s0), min(b, s1)
            if hi - lo <= 1e-12:
                continue
            dl = hi - lo
            if typ == "dipole":
                e1 = E1 if abs(lo - s0) < 1e-12 else 0.0
                e2 = E2 if abs(hi - s1) < 1e-12 else 0.0
                r = r_gen6(dl, angle * dl / L, E1=e1, E2=e2)
            else:
                r = r_gen6(dl, 0.0)
            m = r @ m
        return m

    def formation_length(self, k, sigma_z):
        """Formation length used for the interpolant window at step k."""
        if k == 0:
            return float("inf")
        s = self.positions[k]
        cur = len(self.pieces) - 1
        for i, p in enumerate(self.pieces):
            if s <= p[3] + 1e-12:
                cur = i
                break
        acc = 0.0
        last_R = None
        for (name, typ, s0, s1, L, angle, E1, E2) in self.pieces[:cur + 1]:
            if typ == "dipole":
                last_R = abs(L / angle)
            elif last_R is None:
                acc += L
        if last_R is None:
            return acc
        return (24.0 * last_R ** 2 * 5.0 * sigma_z) ** (1.0 / 3.0)


@dataclass
class Workload:
    name: str
    lattice: OrderedDict
    n_particles: int
    beam_fn: object
    deposit: dict
    integration: dict
    mesh: dict
    n_steps: int
    charge: float = 1e-9
    energy: float = 1e9
    extra: dict = field(default_factory=dict)

    def beam(self, n=None, seed=None):
        return self.beam_fn(n or self.n_particles, seed)


def workload(name, n_particles=None):
    """Return a :class:`Workload` by name (``dipole_c1`` ... ``chicane_c5``)."""
    integ = {"n_formation_length": 1.5, "zbins": 100, "xbins": 100}
    if name == "dipole_c1":
        n = n_particles or 500_000
        return Workload(
            name, dipole_lattice(1.5, 0.3, 0.001), n,
            lambda n, seed: gaussian_beam(n, 10e-6, 20e-6, 1e-4, 5e-6, 0.0, seed or 1),
            {"xbins": 128, "zbins": 128, "xlim": 5, "zlim": 5, "filter_order": 2,
             "filter_window": 9, "velocity_threhold": 1000},
            integ, {"xbins": 32, "zbins": 32, "xlim": 3, "zlim": 3}, 300)
    if name in ("chicane_c2", "chicane_c3", "chicane_c5"):
        if name == "chicane_c2":
            n = n_particles or 2_000_000
            fn = lambda n, seed: gaussian_beam(n, 20e-6, 50e-6, 1e-4, 5e-6, -10.0, seed or 2)
            grid, mesh, steps = 256, 64, 100
        elif name == "chicane_c3":
            n = n_particles or 4_000_000
            fn = lambda n, seed: double_horn_beam(n, 15e-6, 1e-4, 5e-6, -10.0, seed or 3)
            grid, mesh, steps = 384, 96, 100
        else:
            n = n_particles or 10_000_000
            fn = lambda n, seed: gaussian_beam(n, 10e-6, 30e-6, 1e-4, 5e-6, -20.0, seed or 5)
            grid, mesh, steps = 512, 128, 300
        lat = chicane_lattice(6.5 / steps)
        return Workload(
            name, lat, n, fn,
            {"xbins": grid, "zbins": grid, "xlim": 5, "zlim": 5, "filter_order": 2,
             "filter_window": 9, "velocity_threhold": 1000},
            integ, {"xbins": mesh, "zbins": mesh, "xlim": 3, "zlim": 3}, steps)
    raise KeyError(name)


def serving_requests(n_requests=256, rate_hz=200.0, seed=4, n_max=4_000_000,
                     n_min=100_000, steps_per_request=8):
    """Poisson request stream for the serving workload.

    Each request is one beam through one dipole: ``steps_per_request`` DF
    steps (each appended to the request's device history) and one wake
    evaluation on its mesh after the last step.  Returns a list of dicts with
    ``arrival_s``, ``rho``, ``angle``, ``n``, ``sigma_z``, ``grid``, ``mesh``
    and ``seed``.
    """
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, n_requests)
    t = np.cumsum(gaps) - gaps[0]
    out = []
    for i in range(n_requests):
        out.append({
            "id": i,
            "arrival_s": float(t[i]),
            "rho": float(rng.uniform(1.0, 20.0)),
            "angle": float(rng.uniform(0.02, 0.2)),
            "n": int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))),
            "sigma_z": float(rng.uniform(10e-6, 100e-6)),
            "grid": int(rng.choice([64, 128, 256, 512])),
            "mesh": int(rng.choice([32, 64, 96, 128])),
            "seed": int(rng.integers(1, 2**31 - 1)),
            "steps": steps_per_request,
        })
    return out
