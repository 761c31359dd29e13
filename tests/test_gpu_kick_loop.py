"""The reference's run loop with the CSR kick applied every step
(CSR.py:297-334: transport, DF and history, mesh, wake, Beam.apply_wakes),
on the GPU with the plain FP64 wake against the oracle doing the same steps
on the host.  The kick feeds back into every later step, so this pins the
whole loop: transport, the moments-sized deposit, DF finalisation, history,
mesh, wake and the kick interpolation.  The same loop with the mixed wake
applies kicks within 1e-4 of the FP64 loop's.

Tolerance: the FP64 wake is bit-exact with the oracle on the same history;
the device DF/history sums are evaluated in fixed orders of their own
(<= 1e-12 of the fields), so after the kicks of several steps every
coordinate row agrees with the oracle's to 1e-9 of that row's largest
kick-induced change (px, pz) or of its spread (the other rows)."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import OracleRun

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


@cuda
def test_kick_loop_fp64_matches_oracle():
    import bench
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import dipole_lattice, gaussian_beam
    lat = dipole_lattice(1.5, 0.05, 0.01)
    beam6 = gaussian_beam(60_000, 10e-6, 20e-6, 1e-4, 5e-6, -5.0, seed=21)
    dep = {"xbins": 64, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 1000}
    integ = {"n_formation_length": 1.5, "zbins": 16, "xbins": 16}
    mesh = {"xbins": 8, "zbins": 8, "xlim": 3, "zlim": 3}
    step = float(lat["step_size"])
    steps = 4
    run = WakeRun(lat, beam6, dep, integ, mesh, precision="fp64", grid_rule="configured",
                  host_transport=False)
    bench.tracking_steps(run, 1, steps, "fp64", step)
    torch.cuda.synchronize()
    gpu = run.beam.particle.cpu().numpy()
    # the same loop with the mixed wake
    runm = WakeRun(lat, beam6, dep, integ, mesh, precision="mixed", grid_rule="configured",
                   host_transport=False)
    bench.tracking_steps(runm, 1, steps, "mixed", step)
    torch.cuda.synchronize()
    gpum = runm.beam.particle.cpu().numpy()

    orc = OracleRun(lat, beam6, dep, integ, grid_rule="configured")
    orc.init()
    for k in range(1, steps + 1):
        orc.step(k)
        st = orc.stats()
        xm, zm, zr, xr = O.csr_mesh(st, mesh["xbins"], mesh["zbins"], mesh["xlim"], mesh["zlim"])
        dE, xk = orc.wake_oracle().points(orc.position + zm, xm)
        shape = (mesh["xbins"], mesh["zbins"])
        orc.beam6 = O.apply_wakes(orc.beam6, dE.reshape(shape), xk.reshape(shape), xr, zr, step,
                                  1e9, True, st["slope"])
    # the beam without kicks, for the size of the kicks
    free = beam6.copy()
    for k in range(1, steps + 1):
        free = run.plan.matrix(k) @ free
    rel = []
    for r in range(6):
        kick = np.abs(orc.beam6[r] - free[r]).max()
        scale = kick if r in (1, 5) else max(kick, np.abs(free[r]).max())
        assert scale > 0, r
        rel.append(float(np.abs(gpu[r] - orc.beam6[r]).max() / scale))
    print("kick loop vs oracle, per row (of the row's scale):", ["%.1e" % v for v in rel])
    assert max(rel) <= 1e-9, rel
    # mixed wake in the loop: the kicks it applies (px, pz changes) within
    # 1e-4 of the FP64 loop's, the other rows at their usual agreement
    for r in (1, 5):
        kick = np.abs(gpu[r] - free[r]).max()
        d = np.abs((gpum[r] - free[r]) - (gpu[r] - free[r])).max()
        print("mixed vs fp64 kick, row", r, "%.1e" % (d / kick))
        assert d <= 1e-4 * kick, (r, d / kick)
    assert np.abs(orc.beam6[5] - free[5]).max() > 0, "the kicks must change pz"


@cuda
@pytest.mark.parametrize("bins", [(16, 16), (100, 100)])
def test_wake_mixed_with_columns_before_the_orbit_start(bins):
    """One step into a dipole (s = 0.01 m) the far region reaches s' < 0,
    more than one orbit-table step before the lattice starts, where the
    reference's interpolate1D gives n' = tau' = 0 (|r - r'| = |R0| for every
    x').  The mixed wake (its distance from the perpendicular foot, which
    divides by |n'|^2) must handle those columns: within 1e-4 of the FP64
    wake, finite everywhere."""
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import dipole_lattice, gaussian_beam
    from tests.helpers import wake_errors
    lat = dipole_lattice(1.5, 0.05, 0.01)
    beam6 = gaussian_beam(60_000, 10e-6, 20e-6, 1e-4, 5e-6, -5.0, seed=21)
    dep = {"xbins": 64, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 1000}
    integ = {"n_formation_length": 1.5, "zbins": bins[1], "xbins": bins[0]}
    mesh = {"xbins": 8, "zbins": 8, "xlim": 3, "zlim": 3}
    run = WakeRun(lat, beam6, dep, integ, mesh, precision="both", grid_rule="configured",
                  host_transport=False)
    run.step(1)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    sh = s.cpu().numpy()
    regions = [csr._regions(v, 0.0)[1] for v in sh]
    assert any(r[0][5] < -csr.lattice.delta_x for r in regions), "no column before the orbit start"
    dE, xk = (t.cpu().numpy() for t in csr.wake_device(s, x, "mixed"))
    d64, x64 = (t.cpu().numpy() for t in csr.wake_device(s, x, "fp64"))
    assert np.isfinite(dE).all() and np.isfinite(xk).all()
    e = wake_errors(dE, xk, d64, x64)
    assert max(e.values()) <= 1e-4, e
    # the same with the mixed kernel's FP64 geometry (jobs without the
    # double-word orbit tables)
    from pydfcsr_gb300.CSR import jobs_to_device
    job = csr._job()
    job.lattice_dw = None
    job.lattice_delta_dw = None
    ip = csr.integration_params
    g = csr.evaluator.mixed(jobs_to_device([job]), s, x, ip.xbins, ip.zbins)
    dEg, xkg = g[0].cpu().numpy(), g[1].cpu().numpy()
    assert np.isfinite(dEg).all() and np.isfinite(xkg).all()
    e = wake_errors(dEg, xkg, d64, x64)
    assert max(e.values()) <= 1e-4, e


@cuda
def test_wake_mixed_with_columns_past_the_orbit_end():
    """At the last step of a lattice without a tail drift (s = 0.05 m, the
    dipole's end) every near region reaches s' = s + 5 sigma_z beyond the
    orbit tables' last sample, where interpolate1D (interp1D.py:14-36) gives
    zero vectors, and the bunch's head half sits beyond it too.  Observers
    with int((s - s_0) / ds) >= Nsample have zero orbit vectors of their own,
    and the reference's wake there is NaN (dE and x_kick; the oracle gives
    NaN at exactly those points).  Both device paths give NaN at the same
    points; everywhere else the mixed wake is finite and within 1e-4 of the
    FP64 wake."""
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import dipole_lattice, gaussian_beam
    from tests.helpers import wake_errors
    lat = dipole_lattice(1.5, 0.05, 0.01, tail_drift=0.0)
    beam6 = gaussian_beam(60_000, 10e-6, 20e-6, 1e-4, 5e-6, -5.0, seed=22)
    dep = {"xbins": 64, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 1000}
    integ = {"n_formation_length": 1.5, "zbins": 32, "xbins": 16}
    mesh = {"xbins": 8, "zbins": 8, "xlim": 3, "zlim": 3}
    run = WakeRun(lat, beam6, dep, integ, mesh, precision="both", grid_rule="configured",
                  host_transport=False)
    last = len(run.plan.positions) - 1
    for k in range(1, last + 1):
        run.step(k)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    sh = s.cpu().numpy()
    lt = csr.lattice
    regions = [csr._regions(v, 0.0)[1] for v in sh]
    assert all(r[-1][5] > lt.max_x + lt.delta_x for r in regions), "near regions must pass the end"
    past = ((sh - lt.min_x) / lt.delta_x).astype(int) >= lt.s.shape[0]
    assert past.any() and not past.all()
    dE, xk = (t.cpu().numpy() for t in csr.wake_device(s, x, "mixed"))
    d64, x64 = (t.cpu().numpy() for t in csr.wake_device(s, x, "fp64"))
    for a in (dE, xk, d64, x64):
        assert (np.isnan(a) == past).all()
    inside = ~past
    assert np.isfinite(dE[inside]).all() and np.isfinite(xk[inside]).all()
    e = wake_errors(dE[inside], xk[inside], d64[inside], x64[inside])
    assert max(e.values()) <= 1e-4, e
