"""The wake server on the GPU: a result is the same alone and in the mix.

Requests with different particle counts, grids, meshes and lattices arrive
while others are running; each admitted request's DF steps run on its own
stream and all active requests' observation points share one batched wake
launch per tick (replayed from CUDA graphs).  Every point is reduced by one
CTA in a fixed order, so the tolerance for alone-vs-mix is zero: the
results must be bitwise equal.  The mixed results are also compared with the
plain FP64 kernels served on the same stream (max_rel, rms_rel and the
pointwise error with a floor of 1e-3 S all <= 1e-4, S = peak |wake| of that
request's step over both components).
"""
import numpy as np
import pytest

from pydfcsr_gb300.serve import RequestSpec

pytestmark = pytest.mark.gpu


def _stream():
    small = {"n_formation_length": 1.5, "zbins": 40, "xbins": 30}
    out = []
    shapes = [(60_000, 64, 16, 2.0, 0.10, 30e-6), (150_000, 128, 24, 8.0, 0.05, 60e-6),
              (90_000, 64, 16, 1.5, 0.18, 20e-6), (120_000, 128, 32, 15.0, 0.03, 90e-6),
              (70_000, 64, 16, 4.0, 0.12, 45e-6)]
    for i, (n, grid, mesh, rho, angle, sz) in enumerate(shapes):
        out.append(RequestSpec(id=i, arrival_s=0.02 * i, rho=rho, angle=angle, n=n, sigma_z=sz,
                               grid=grid, mesh=mesh, seed=100 + i, steps=4,
                               integration=dict(small), upper_limit=200))
    # smaller integration bins than the rest: alone, its launches are laid
    # out for 24 x 36 bins; in the mix, for 30 x 40
    out[3].integration = {"n_formation_length": 1.5, "zbins": 36, "xbins": 24}
    return out


def _alone(spec, **kw):
    from pydfcsr_gb300.serve import WakeServer
    one = RequestSpec(**{**spec.__dict__, "arrival_s": 0.0})
    srv = WakeServer([one], **kw)
    srv.run()
    return srv.result(spec.id)


def test_alone_equals_mix_bitwise():
    from pydfcsr_gb300.serve import WakeServer
    specs = _stream()
    srv = WakeServer(specs, max_active=3, chunk=256)
    summ = srv.run()
    assert summ["requests"] == len(specs) and summ["refused"] == 0
    assert summ["graphs"] >= 1 and summ["graph_replays"] >= 1
    assert summ["latency_p99_s"] >= summ["latency_p50_s"] > 0
    # some launch carried more than one request's points
    assert max(srv.launch_points) > min(s.mesh ** 2 for s in specs)
    for sp in specs:
        mix = srv.result(sp.id)
        alone = _alone(sp, chunk=256)
        assert [k for k, _, _ in mix] == [k for k, _, _ in alone] == [2, 3, 4]
        for (k, dE_m, xk_m), (_, dE_a, xk_a) in zip(mix, alone):
            assert np.all(np.isfinite(dE_m)) and np.abs(dE_m).max() > 0
            assert np.array_equal(dE_m, dE_a), (sp.id, k)
            assert np.array_equal(xk_m, xk_a), (sp.id, k)


def test_graphs_off_matches_graphs_on():
    from pydfcsr_gb300.serve import WakeServer
    specs = _stream()[:3]
    a = WakeServer(specs, max_active=3, chunk=256, use_graphs=True)
    a.run()
    b = WakeServer(specs, max_active=3, chunk=256, use_graphs=False)
    b.run()
    for sp in specs:
        for (k, dE1, xk1), (_, dE2, xk2) in zip(a.result(sp.id), b.result(sp.id)):
            assert np.array_equal(dE1, dE2) and np.array_equal(xk1, xk2)


def test_mixed_vs_fp64_on_the_same_stream():
    from pydfcsr_gb300.serve import WakeServer
    specs = _stream()
    mixed = WakeServer(specs, max_active=3, chunk=256)
    mixed.run()
    plain = WakeServer(specs, precision="fp64", max_active=3, chunk=256)
    plain.run()
    from tests.helpers import wake_errors
    worst = 0.0
    for sp in specs:
        for (k, dE1, xk1), (k2, dE2, xk2) in zip(mixed.result(sp.id), plain.result(sp.id)):
            assert k == k2
            worst = max(worst, max(wake_errors(dE1, xk1, dE2, xk2).values()))
    assert worst <= 1e-4, worst


def test_admission_refuses_oversize_request():
    from pydfcsr_gb300.serve import WakeServer, footprint_bytes
    specs = _stream()[:2]
    budget = footprint_bytes(specs[0]) + 1
    big = RequestSpec(**{**specs[1].__dict__, "n": 4_000_000, "grid": 512})
    srv = WakeServer([specs[0], big], budget_bytes=budget, chunk=256)
    summ = srv.run()
    assert summ["refused"] == 1 and summ["requests"] == 1


def test_kernel_error_fails_one_request_only(monkeypatch):
    """A kernel error status injected on the host for one request (its DF
    step 3 raises as a failing C-ABI call does): that request fails alone,
    its memory goes back to the budget, and the other requests' results are
    bitwise those of a run without it."""
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.serve import WakeServer, _Live
    specs = _stream()[:3]
    bad = specs[1].id
    real = _Live.advance_finish

    def advance_finish(self):
        if self.spec.id == bad and self.k == 3:
            raise _lib.DfcsrKernelError(4, "dfcsr_df_finalize", "injected kernel error status")
        return real(self)

    monkeypatch.setattr(_Live, "advance_finish", advance_finish)
    srv = WakeServer(specs, max_active=3, chunk=256)
    summ = srv.run()
    monkeypatch.undo()
    assert summ["failed"] == 1 and summ["refused"] == 0
    assert "KERNEL_ERROR" in srv.failed()[bad]
    assert srv.sched.admission.used == 0 and srv.sched.admission.active == 0
    assert [k for k, _, _ in srv.result(bad)] == [2]       # served until it failed
    ref = WakeServer([sp for sp in specs if sp.id != bad], max_active=3, chunk=256)
    ref.run()
    for sp in specs:
        if sp.id == bad:
            continue
        got, want = srv.result(sp.id), ref.result(sp.id)
        assert [k for k, _, _ in got] == [k for k, _, _ in want] == [2, 3, 4]
        for (k, dE1, xk1), (_, dE2, xk2) in zip(got, want):
            assert np.array_equal(dE1, dE2) and np.array_equal(xk1, xk2), (sp.id, k)



def test_df_barrier_timeout_fails_one_request_only(monkeypatch):
    """A DF finalisation whose grid-barrier waits run out (one request's
    step 3 expects an arrival that never comes, with a short spin limit):
    the device reports it in the stage's status word, that request fails
    with a timeout and gets no result for the step, and the other requests'
    results are bitwise those of a run without it."""
    from pydfcsr_gb300.serve import WakeServer, _Live
    specs = _stream()[:3]
    bad = specs[1].id
    real = _Live.advance_finish

    def advance_finish(self):
        if self.spec.id == bad and self.k == 3:
            tr = self.csr.DF_tracker
            tr.barrier_spins, tr.barrier_extra = 1 << 14, 1
        return real(self)

    monkeypatch.setattr(_Live, "advance_finish", advance_finish)
    srv = WakeServer(specs, max_active=3, chunk=256)
    summ = srv.run()
    monkeypatch.undo()
    assert summ["failed"] == 1 and summ["refused"] == 0
    assert "TIMEOUT" in srv.failed()[bad]
    assert srv.sched.admission.used == 0 and srv.sched.admission.active == 0
    assert [k for k, _, _ in srv.result(bad)] == [2]
    ref = WakeServer([sp for sp in specs if sp.id != bad], max_active=3, chunk=256)
    ref.run()
    for sp in specs:
        if sp.id == bad:
            continue
        got, want = srv.result(sp.id), ref.result(sp.id)
        assert [k for k, _, _ in got] == [k for k, _, _ in want] == [2, 3, 4]
        for (k, dE1, xk1), (_, dE2, xk2) in zip(got, want):
            assert np.array_equal(dE1, dE2) and np.array_equal(xk1, xk2), (sp.id, k)
