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
