"""Bounded device waits on the GPU: a wait that runs out returns a status
to the host and leaves the CUDA context usable - no fault, no hang.

The DF stage's cooperative launch meets at a grid barrier between its
phases; each CTA's wait there is bounded.  dfcsr_grid_barrier_check runs
that barrier once; asking for one arrival more than the launch has CTAs is
a flag that nothing sets, so every wait runs out after a short spin limit.
"""
import time

import numpy as np
import pytest
import torch

from oracle import oracle as O

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


@cuda
def test_grid_barrier_wait_runs_out_and_reports_timeout():
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.deposit import deposit_cic
    from pydfcsr_gb300.runtime import grid_barrier_check
    grid_barrier_check()                          # one CTA per SM, all arrive
    grid_barrier_check(blocks=1)
    t0 = time.perf_counter()
    with pytest.raises(_lib.DfcsrTimeout, match="gave up"):
        grid_barrier_check(extra_arrivals=1, max_spins=1 << 16)
    assert time.perf_counter() - t0 < 20
    # the barrier, the context and the library keep working
    grid_barrier_check()
    rng = np.random.default_rng(7)
    x, z, w = (rng.normal(0, 1e-5, 50_000) for _ in range(3))
    g = (64, -4e-5, 4e-5, 64, -4e-5, 4e-5)
    o0, o1 = deposit_cic(*(torch.from_numpy(a).cuda() for a in (x, z)), None,
                         torch.from_numpy(w).cuda(), *g)
    torch.cuda.synchronize()
    ref0 = O.histogram_cic_2d(x, z, np.ones_like(x), *g)
    ref1 = O.histogram_cic_2d(x, z, w, *g)
    assert np.max(np.abs(o0.cpu().numpy() - ref0)) <= 1e-12 * np.max(np.abs(ref0))
    assert np.max(np.abs(o1.cpu().numpy() - ref1)) <= 1e-12 * np.max(np.abs(ref1))


@cuda
def test_grid_barrier_check_arguments():
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import grid_barrier_check
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    with pytest.raises(_lib.DfcsrBadArgument, match="blocks"):
        grid_barrier_check(blocks=sms + 1)
    with pytest.raises(_lib.DfcsrBadArgument, match="max_spins"):
        grid_barrier_check(max_spins=0)


@cuda
def test_df_stage_barrier_timeout_reported():
    """The DF stage (one cooperative launch, nine grid barriers) with a short
    spin limit and one arrival more than it has CTAs: every wait runs out, the
    stage's status word says so, DF_tracker.check_status raises DfcsrTimeout,
    and the next normal DF step on the same context reproduces the fields of
    a run without the failure bit for bit."""
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.deposit import DF_tracker
    rng = np.random.default_rng(3)
    n = 50_000
    x, z, px = rng.normal(0, 1e-5, n), rng.normal(0, 2e-5, n), rng.normal(0, 1e-6, n)
    dep = {"xbins": 64, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2,
           "filter_window": 9, "velocity_threhold": 1000}
    xd, zd, pxd = (torch.from_numpy(a).cuda() for a in (x, z, px))
    tr = DF_tracker(dep, grid_rule="configured")
    tr.get_DF(xd, zd, pxd, 0.0)
    tr.check_status()
    good = tr.fields_device.clone()
    tr.barrier_spins, tr.barrier_extra = 1 << 14, 1
    t0 = time.perf_counter()
    tr.get_DF(xd, zd, pxd, 0.0)
    with pytest.raises(_lib.DfcsrTimeout, match="grid-barrier"):
        tr.check_status()
    assert time.perf_counter() - t0 < 20
    assert torch.isnan(tr._cur.scalars[:7]).all() and float(tr._cur.scalars[7]) == 1.0
    tr.barrier_spins, tr.barrier_extra = 0, 0
    tr.get_DF(xd, zd, pxd, 0.0)
    tr.check_status()
    assert float(tr._cur.scalars[7]) == 0.0
    assert torch.equal(tr.fields_device, good)


@cuda
def test_df_stage_barrier_timeout_raised_by_wake_result():
    """Through CSR2D: a DF step whose barrier waits ran out makes the next
    calculate_2D_CSR raise DfcsrTimeout when its result is read."""
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import dipole_lattice, gaussian_beam
    lat = dipole_lattice(1.5, 0.3, 0.02)
    dep = {"xbins": 48, "zbins": 64, "xlim": 5, "zlim": 5, "filter_order": 2, "filter_window": 9,
           "velocity_threhold": 1000, "upper_limit": 64}
    integ = {"n_formation_length": 1.5, "zbins": 24, "xbins": 16}
    mesh = {"xbins": 4, "zbins": 4, "xlim": 3, "zlim": 3}
    run = WakeRun(lat, gaussian_beam(20000, 10e-6, 20e-6, seed=11), dep, integ, mesh,
                  precision="mixed", grid_rule="configured")
    for k in (1, 2):
        run.step(k)
    dE, _ = run.wake()
    assert np.all(np.isfinite(dE))
    tr = run.csr.DF_tracker
    tr.barrier_spins, tr.barrier_extra = 1 << 14, 1
    run.step(3)
    with pytest.raises(_lib.DfcsrTimeout):
        run.wake()
