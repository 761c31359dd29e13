"""Shared test helpers: fixture loading and the oracle step driver."""
import os

import numpy as np

from oracle import oracle as O
from pydfcsr_gb300.synthetic import StepPlan

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def rel_err(a, b):
    """max |a - b| / max(|b|, 1e-3 max|b|) - pointwise relative error with a
    floor at 1e-3 of the field's peak so zero crossings do not blow it up."""
    a, b = np.asarray(a, float), np.asarray(b, float)
    peak = np.max(np.abs(b)) if b.size else 0.0
    if peak == 0:
        return float(np.max(np.abs(a - b))) if a.size else 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-3 * peak)))


def wake_errors(dE, xk, dE_ref, xk_ref):
    """Error of a wake (dE/dct, x-kick) against a reference wake.

    Both components share the unit (MeV/m); S is the peak of the reference
    wake over the mesh and both components.
      max_rel       max |a - b| / S
      rms_rel       ||a - b||_2 / ||b||_2 over the mesh and both components
      pointwise_dE  max |a - b| / max(|b|, 1e-3 S) for dE/dct  (diagnostic)
      pointwise_xk  the same for the x-kick                     (diagnostic)
    """
    dE, xk, dE_ref, xk_ref = (np.asarray(v, float).ravel() for v in (dE, xk, dE_ref, xk_ref))
    a = np.concatenate([dE, xk])
    b = np.concatenate([dE_ref, xk_ref])
    S = float(np.max(np.abs(b)))
    if S == 0:
        S = 1.0
    nb = float(np.sqrt(np.sum(b * b))) or 1.0
    floor = 1e-3 * S
    return {
        "max_rel": float(np.max(np.abs(a - b)) / S),
        "rms_rel": float(np.sqrt(np.sum((a - b) ** 2)) / nb),
        "pointwise_dE": float(np.max(np.abs(dE - dE_ref) / np.maximum(np.abs(dE_ref), floor))),
        "pointwise_xk": float(np.max(np.abs(xk - xk_ref) / np.maximum(np.abs(xk_ref), floor))),
    }


def rms_rel(a, b):
    a, b = np.asarray(a, float), np.asarray(b, float)
    nb = np.sqrt(np.mean(b * b))
    return float(np.sqrt(np.mean((a - b) ** 2)) / nb) if nb > 0 else 0.0


def dep_from_array(a):
    d = {"xbins": int(a[0]), "zbins": int(a[1]), "xlim": float(a[2]), "zlim": float(a[3]),
         "filter_order": int(a[4]), "filter_window": int(a[5]),
         "velocity_threhold": float(a[6])}
    if len(a) > 7 and a[7] > 0:
        d["upper_limit"] = int(a[7])
    for k in ("xlim", "zlim", "velocity_threhold"):
        if float(d[k]).is_integer():
            d[k] = int(d[k])
    return d


class OracleRun:
    """The oracle over synthetic steps (same call order as CSR2D.run)."""

    def __init__(self, lattice, beam6, dep, integ, grid_rule="reference", charge=1e-9):
        self.plan = StepPlan(lattice)
        self.lattice = lattice
        self.beam6 = np.array(beam6, dtype=float, copy=True)
        self.tracker = O.DFTracker(dep, grid_rule=grid_rule)
        self.integ = integ
        s, rho, dist, nsep, coords, nv, tau = O.reference_trajectory(lattice, 2000)
        self.tables = (s, rho, dist, coords, nv, tau)
        self.position = 0.0
        self.charge = charge
        self.lf = float("inf")

    def stats(self):
        return O.beam_stats(self.beam6[0], self.beam6[4])

    def df_step(self, lf):
        b = self.beam6
        self.tracker.get_DF(b[0], b[4], b[1], self.position)
        self.tracker.append_DF()
        self.tracker.append_interpolant(lf, self.integ["n_formation_length"])

    def init(self):
        self.df_step(float("inf"))

    def step(self, k):
        self.beam6 = self.plan.matrix(k) @ self.beam6
        self.position = self.plan.positions[k]
        st = self.stats()
        self.lf = self.plan.formation_length(k, st["sigma_z"])
        self.df_step(self.lf)
        self.tracker.build_interpolant()
        return self.lf

    def wake_oracle(self):
        st = self.stats()
        return O.WakeOracle(self.tracker, self.tables, self.position, st["sigma_z"],
                            st["sigma_x"], st["slope"][0], st["mean_x"], self.lf,
                            self.integ["n_formation_length"], self.integ["zbins"],
                            self.integ["xbins"], charge=self.charge)


def lattice_from(g):
    """Rebuild a reference-format lattice dict stored in a wake fixture."""
    from collections import OrderedDict
    lat = OrderedDict(step_size=float(g["lattice_step"]))
    for i, (L, angle, is_dip) in enumerate(g["lattice_elements"]):
        if is_dip:
            lat[f"E{i}"] = {"type": "dipole", "L": float(L), "angle": float(angle),
                            "E1": 0.0, "E2": 0.0, "nsep": 1}
        else:
            lat[f"E{i}"] = {"type": "drift", "L": float(L), "nsep": 1}
    return lat


def integ_from(g):
    a = g["integ"]
    return {"n_formation_length": float(a[0]), "zbins": int(a[1]), "xbins": int(a[2])}


def oracle_from_wake_fixture(g, grid_rule="reference"):
    """Run the oracle through the same steps as a wake_*.npz fixture."""
    run = OracleRun(lattice_from(g), g["beam0"], dep_from_array(g["dep"]), integ_from(g),
                    grid_rule=grid_rule)
    run.init()
    for k in range(1, len(g["positions"])):
        run.step(k)
    return run
