"""Checkpoint and resume of the wake state between steps.

CSR2D.state_dict() copies the DF tracker's history (logged DFs, ring slices,
logs, interpolant grid) to host data; a fresh CSR2D that loads it and runs
the following steps on the same particles gives the same wakes, bit for bit,
as the run that was never interrupted.  The state goes through pickle, so it
holds no device pointers.
"""
import pickle

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


def _step(run, sets, k, precision):
    csr, beam = run.csr, run.beam
    beam.particle = sets[k - 1]
    beam.update_status()
    beam.position = float(run.plan.positions[k])
    beam.step = k
    csr.update_history(run.plan.formation_length(k, beam.sigma_z))
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    dE, xk = csr.wake_device(s, x, precision)
    return dE.cpu().numpy(), xk.cpu().numpy()


@cuda
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_resume_from_state_dict_is_bitwise(precision):
    import bench
    from pydfcsr_gb300.synthetic import workload
    wl = workload("chicane_c2", n_particles=200_000)
    wl.mesh = dict(wl.mesh, xbins=16, zbins=16)
    total, cut = 8, 5
    lat = bench.lattice_for(wl, total)
    run, _ = bench.make_run(wl, lat, precision)
    sets = bench.device_step_sets(run, total)
    for k in range(1, cut + 1):
        _step(run, sets, k, precision)
    state = pickle.loads(pickle.dumps(run.csr.state_dict()))
    straight = [_step(run, sets, k, precision) for k in range(cut + 1, total + 1)]

    fresh, _ = bench.make_run(wl, lat, precision)
    fresh.csr.load_state_dict(state)
    assert len(fresh.csr.DF_tracker.time_interp) == len(state["DF_tracker"]["logs"]["time_interp"])
    resumed = [_step(fresh, sets, k, precision) for k in range(cut + 1, total + 1)]
    for (dE1, xk1), (dE2, xk2) in zip(straight, resumed):
        assert np.isfinite(dE1).all() and np.abs(dE1).max() > 0
        assert np.array_equal(dE1, dE2) and np.array_equal(xk1, xk2)


@cuda
def test_state_of_other_precision_is_refused():
    import bench
    from pydfcsr_gb300.synthetic import workload
    wl = workload("chicane_c2", n_particles=50_000)
    lat = bench.lattice_for(wl, 2)
    a, _ = bench.make_run(wl, lat, "mixed")
    b, _ = bench.make_run(wl, lat, "fp64")
    with pytest.raises(ValueError, match="precision|tracker"):
        b.csr.load_state_dict(a.csr.state_dict())
