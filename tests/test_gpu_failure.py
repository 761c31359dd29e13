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
