"""Host side of the wake server: HBM admission and the continuous-batching
scheduler, driven by a fake clock (no GPU)."""
import pytest

from pydfcsr_gb300.serve import Admission, RequestSpec, Scheduler, footprint_bytes
from pydfcsr_gb300.synthetic import serving_requests


def spec(i, t, n=200_000, grid=128, mesh=32, steps=4):
    return RequestSpec(id=i, arrival_s=t, rho=5.0, angle=0.1, n=n, sigma_z=30e-6, grid=grid,
                       mesh=mesh, seed=i + 1, steps=steps)


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


def test_footprint_grows_with_size_and_precision():
    a = footprint_bytes(spec(0, 0.0))
    assert footprint_bytes(spec(0, 0.0, n=400_000)) > a
    assert footprint_bytes(spec(0, 0.0, grid=256)) > a
    assert footprint_bytes(spec(0, 0.0), "fp64") > a
    # a 4e6-particle, 512^2 request stays well under a GB
    big = footprint_bytes(spec(0, 0.0, n=4_000_000, grid=512, mesh=128, steps=8))
    assert 2e8 < big < 1e9


def test_admission_budget_and_slots():
    adm = Admission(1000, max_active=2)
    assert adm.try_admit(600)
    assert not adm.try_admit(500)          # memory
    assert adm.try_admit(400)
    assert not adm.try_admit(1)            # slots
    adm.release(600)
    assert adm.try_admit(500)
    assert adm.used == 900 and adm.active == 2
    assert not adm.can_ever_fit(1001)


def test_scheduler_admits_in_arrival_order_without_overtaking():
    clk = FakeClock()
    small = footprint_bytes(spec(0, 0.0))
    specs = [spec(0, 0.0), spec(1, 0.1, n=3_000_000, grid=512), spec(2, 0.2)]
    big = footprint_bytes(specs[1])
    sched = Scheduler(specs, Admission(small + big - 1, 8), clk)
    assert [s.id for s in sched.admit()] == [0]
    clk.t = 0.3
    # request 1 does not fit beside 0; request 2 would, but must not overtake
    assert sched.admit() == []
    sched.finish(specs[0])
    assert [s.id for s in sched.admit()] == [1]
    assert sched.admit() == []
    sched.finish(specs[1])
    assert [s.id for s in sched.admit()] == [2]


def test_scheduler_refuses_what_never_fits_and_cancels_pending():
    clk = FakeClock()
    specs = [spec(0, 0.0, n=4_000_000, grid=512), spec(1, 0.0), spec(2, 5.0)]
    sched = Scheduler(specs, Admission(footprint_bytes(specs[1]) * 2, 4), clk)
    assert [s.id for s in sched.admit()] == [1]
    assert [s.id for s in sched.refused] == [0]
    assert sched.cancel(2) and not sched.cancel(2)
    sched.finish(specs[1])
    assert sched.finished()


def test_continuous_batching_simulation():
    """Requests join while others run; memory and slot limits hold at every
    tick; every request finishes; the active set really changes mid-stream."""
    clk = FakeClock()
    reqs = serving_requests(n_requests=40, rate_hz=50.0, seed=11, steps_per_request=5)
    specs = [RequestSpec.from_dict(r) for r in reqs]
    budget = 3 * max(footprint_bytes(s) for s in specs)
    adm = Admission(budget, max_active=6)
    sched = Scheduler(specs, adm, clk)
    left = {}
    joined_mid = 0
    ticks = 0
    while not sched.finished():
        new = sched.admit()
        if new and any(left.values()):
            joined_mid += 1
        for s in new:
            left[s.id] = s.steps
        assert adm.used <= budget and adm.active <= 6
        assert adm.active == len(sched.active)
        if not sched.active:
            clk.t = sched.idle_until()
            continue
        for s in list(sched.active):
            left[s.id] -= 1
            if left[s.id] == 0:
                sched.finish(s)
        clk.t += 0.01
        ticks += 1
        assert ticks < 10_000
    assert len(sched.done) == len(specs) and not sched.refused
    assert joined_mid > 0
    assert adm.used == 0 and adm.active == 0


def test_request_spec_from_generator():
    r = serving_requests(n_requests=3, seed=4)[1]
    s = RequestSpec.from_dict(r)
    assert s.id == 1 and s.steps == r["steps"] and s.grid in (64, 128, 256, 512)
    assert 1e5 <= s.n <= 4e6
    with pytest.raises(TypeError):
        RequestSpec.from_dict({"id": 0})


def test_scheduler_fail_releases_memory_and_admits_next():
    clk = FakeClock()
    a, b = spec(0, 0.0), spec(1, 0.0)
    sched = Scheduler([a, b], Admission(footprint_bytes(a), 8), clk)   # room for one
    assert [s.id for s in sched.admit()] == [0]
    assert sched.admit() == []
    sched.fail(a, "DfcsrKernelError: injected")
    assert sched.failed == [(a, "DfcsrKernelError: injected")] and sched.active == []
    assert sched.admission.used == 0
    assert [s.id for s in sched.admit()] == [1]
    sched.finish(b)
    assert sched.finished() and sched.done == [b]


def test_request_errors_leave_cuda_errors_fatal():
    """A library error ends one request; a CUDA error (which can poison the
    context) is not among the per-request errors, so it ends the run."""
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.serve import _request_errors
    errs = _request_errors()
    for cls in (_lib.DfcsrBadArgument, _lib.DfcsrOutOfMemory, _lib.DfcsrTimeout,
                _lib.DfcsrKernelError, _lib.DfcsrAdmissionRefused):
        assert issubclass(cls, errs)
    assert not issubclass(_lib.DfcsrCudaError, errs)
