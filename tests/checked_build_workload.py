"""Workload of the bounds-checked build test: the wake path's kernels on small
cases, through whichever library the environment selects (the
bounds-checked one with DFCSR_GB300_CHECKED=1).  Saves every result to the
npz file named by the first argument, with the first index-check failure
(site, index; -1, -1 for none) under "bounds".

Covers: the reference's run loop with the kick fed back (transport,
moments, deposit, DF stage, history regrid, mesh, FP64 and mixed wakes,
apply_wakes), a chicane into its 4-region branch with the FP64 near band,
a bend without a tail drift at its last step (observers and columns past
the orbit tables), deposits with particles outside the grid, and
interpolate3D / interpolate1D with queries inside and outside their grids.
"""
import os
import sys

import numpy as np
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main(path):
    import bench
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.deposit import histogram_cic_2d
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.interp1D import interpolate1D
    from pydfcsr_gb300.interp3D import interpolate3D
    from pydfcsr_gb300.synthetic import dipole_lattice, gaussian_beam, workload

    out = {"checked": np.array(_lib.load().dfcsr_bounds_checked())}
    dep = {"xbins": 64, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2, "filter_window": 5,
           "velocity_threhold": 1000}
    integ = {"n_formation_length": 1.5, "zbins": 16, "xbins": 16}
    mesh = {"xbins": 8, "zbins": 8, "xlim": 3, "zlim": 3}
    # the run loop with kicks, both precisions
    lat = dipole_lattice(1.5, 0.05, 0.01)
    beam6 = gaussian_beam(60_000, 10e-6, 20e-6, 1e-4, 5e-6, -5.0, seed=21)
    for prec in ("fp64", "mixed"):
        run = WakeRun(lat, beam6, dep, integ, mesh, precision=prec, grid_rule="configured",
                      host_transport=False)
        bench.tracking_steps(run, 1, 4, prec, float(lat["step_size"]))
        torch.cuda.synchronize()
        out[f"kick_{prec}"] = run.beam.particle.cpu().numpy()
    # chicane into the 4-region branch, FP64 and mixed wakes, the near band
    wl = workload("chicane_c2", n_particles=100_000)
    run = WakeRun(wl.lattice, wl.beam(), wl.deposit, {"n_formation_length": 1.5, "zbins": 40,
                                                      "xbins": 24},
                  mesh, precision="both", grid_rule="configured", host_transport=False)
    for k in range(1, 39):
        run.step(k)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    for prec in ("fp64", "mixed"):
        dE, xk = csr.wake_device(s, x, prec)
        out[f"chicane_{prec}"] = np.stack([dE.cpu().numpy(), xk.cpu().numpy()])
    csr.near_band = 20 * 50e-6
    dE, xk = csr.wake_device(s, x, "mixed")
    out["chicane_band"] = np.stack([dE.cpu().numpy(), xk.cpu().numpy()])
    # a bend without a tail drift, at its last step
    lat = dipole_lattice(1.5, 0.05, 0.01, tail_drift=0.0)
    run = WakeRun(lat, gaussian_beam(60_000, 10e-6, 20e-6, 1e-4, 5e-6, -5.0, seed=22), dep,
                  integ, mesh, precision="both", grid_rule="configured", host_transport=False)
    for k in range(1, len(run.plan.positions)):
        run.step(k)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    for prec in ("fp64", "mixed"):
        dE, xk = csr.wake_device(s, x, prec)
        out[f"end_{prec}"] = np.stack([dE.cpu().numpy(), xk.cpu().numpy()])
    # deposits with particles outside the grid and NaN coordinates
    rng = np.random.default_rng(3)
    q1, q2, w = rng.normal(0, 1.0, 50_000), rng.normal(0, 2.0, 50_000), rng.normal(1, 0.1, 50_000)
    q2[:10] = np.nan
    out["cic"] = histogram_cic_2d(q1, q2, w, 40, -2.0, 2.0, 60, -3.0, 3.0)
    # interpolate3D / interpolate1D inside and outside their grids
    data = rng.normal(size=(7, 9, 11))
    qs = [rng.uniform(-2.0, 13.0, 4000) for _ in range(3)]
    out["interp3d"] = interpolate3D(qs[0], qs[1], qs[2], data, 0.0, 0.5, -1.0, 1.0, 0.8, 1.1)
    tab = rng.normal(size=50)
    out["interp1d"] = interpolate1D(rng.uniform(-5.0, 60.0, 4000), tab, 0.0, 1.0)
    b = _lib.bounds_status()
    out["bounds"] = np.array(b if b is not None else (-1, -1))
    np.savez(path, **out)
    print("bounds", b)


if __name__ == "__main__":
    main(sys.argv[1])
