"""The benchmark's pipelined step loop against the plain sequential one.

bench.timed_steps runs the deposit of step k+1 and the moments of step k+2
on a second stream while step k is finalised and its wake computed
(DF_tracker.deposit_DF / get_DF(deposited=...), Beam.status_async /
apply_status).  Every step must see exactly the data of the sequential loop
(update_status -> update_history -> mesh -> wake), so the wakes are equal
bit for bit.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


@cuda
@pytest.mark.parametrize("steps", [1, 2, 9])
def test_pipelined_step_loop_matches_sequential(steps):
    import bench
    from pydfcsr_gb300.synthetic import workload
    wl = workload("chicane_c2", n_particles=200_000)
    lat = bench.lattice_for(wl, steps)
    outs = []
    for mode in ("pipelined", "sequential"):
        run, _ = bench.make_run(wl, lat, "mixed")
        sets = bench.device_step_sets(run, steps)
        csr = run.csr
        if mode == "pipelined":
            bench.timed_steps(run, sets, 1, steps, "mixed", side=torch.cuda.Stream())
            dE, xk = run.last
        else:
            for k in range(1, steps + 1):
                run.beam.particle = sets[k - 1]
                run.beam.update_status()
                run.beam.position = float(run.plan.positions[k])
                run.beam.step = k
                csr.update_history(run.plan.formation_length(k, run.beam.sigma_z))
                csr.get_CSR_mesh()
                s, x = csr.mesh_device()
                dE, xk = csr.wake_device(s, x, "mixed")
        torch.cuda.synchronize()
        outs.append((dE.cpu().numpy(), xk.cpu().numpy(), len(csr.DF_tracker.time_interp)))
    (dE_p, xk_p, n_p), (dE_s, xk_s, n_s) = outs
    assert n_p == n_s
    assert np.isfinite(dE_s).all()
    assert np.array_equal(dE_p, dE_s) and np.array_equal(xk_p, xk_s)


@cuda
def test_kick_loop_early_deposit_matches_sequential():
    """bench.tracking_steps with the deposit enqueued behind the moments (grid
    from the device moments, before the host has them) against the same loop
    with the host grid: wakes and kicked particles equal bit for bit."""
    import bench
    from pydfcsr_gb300.synthetic import workload
    wl = workload("chicane_c2", n_particles=200_000)
    steps = 6
    lat = bench.lattice_for(wl, steps)
    outs = []
    for early in (True, False):
        run, _ = bench.make_run(wl, lat, "mixed")
        bench.tracking_steps(run, 1, steps, "mixed", float(lat["step_size"]), early_deposit=early)
        torch.cuda.synchronize()
        dE, xk = run.last
        outs.append((dE.cpu().numpy(), xk.cpu().numpy(), run.beam.particle.cpu().numpy()))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)
    assert np.isfinite(outs[0][0]).all()


@cuda
def test_deposit_from_device_moments_matches_host_grid():
    """DF_tracker.deposit_DF with the moments as a CUDA tensor (configured
    grid rule) gives the fields of the host-moments deposit bit for bit; a
    beam with zero spread is refused by get_DF as the host path refuses it."""
    from pydfcsr_gb300.deposit import DF_tracker, beam_moments
    from pydfcsr_gb300.synthetic import gaussian_beam
    cfg = {"xbins": 128, "zbins": 160, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 5, "velocity_threhold": 5}
    c = torch.as_tensor(gaussian_beam(300_001, 20e-6, 50e-6, 1e-4, 5e-6, -10.0, seed=4),
                        device="cuda")
    m = beam_moments(c[0], c[4])
    host = m.cpu().numpy()
    fields = []
    for mom in (m, host):
        t = DF_tracker(cfg, precision="mixed", grid_rule="configured")
        dep = t.deposit_DF(c[0], c[4], c[1], mom)
        t.get_DF(c[0], c[4], c[1], 0.0, moments=host, deposited=dep)
        torch.cuda.synchronize()
        fields.append(dep.fields.cpu().numpy())
    # vx is NaN where no particle is (0 / 0, as in the reference)
    assert np.array_equal(fields[0], fields[1], equal_nan=True)
    flat = c.clone()
    flat[0] = 1e-6
    mf = beam_moments(flat[0], flat[4])
    t = DF_tracker(cfg, precision="mixed", grid_rule="configured")
    dep = t.deposit_DF(flat[0], flat[4], flat[1], mf)
    with pytest.raises(ValueError):
        t.get_DF(flat[0], flat[4], flat[1], 0.0, moments=mf.cpu().numpy(), deposited=dep)
    with pytest.raises(ValueError):
        t.deposit_DF(flat[0], flat[4], flat[1], mf.cpu().numpy())
