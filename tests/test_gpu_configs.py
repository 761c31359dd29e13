"""The workloads at their full sizes on the GPU.

* dipole (5e5 particles, 128^2 deposit, SG 9/2, 1 mm steps, 32^2 mesh, the
  plain FP64 method with the reference's grid rule) run to the dipole exit
  and compared with the CPU oracle on the same particles: the history slices
  1e-10, the wake at sampled mesh points 1e-8 (relative, FP64 drop-in).
* chicane with the double-horn beam (4e6 particles, 384^2, 96^2 mesh) and the
  large beam (1e7 particles, 512^2, 128^2 mesh): the mixed-precision wake
  against the plain FP64 kernel on the full mesh, with and without the FP64
  near-source band, and bitwise repeatability; the large beam also in the
  drift after the third bend, where the wake is ~1/300 of its size in the
  bends while the history's terms are not.
* the chicane benchmark beam (2e6 particles, 256^2, 64^2 mesh) over the
  whole 100-step run, every 5th step.
Gates: max_rel, rms_rel and the pointwise error max|a-b| / max(|b|, 1e-3 S)
(S = peak |wake| over both components) all <= 1e-4.  The FP64 kernel itself
is checked against the oracle above and in test_gpu_parity.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.helpers import OracleRun, rel_err, wake_errors

pytestmark = pytest.mark.gpu
cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


class _LazyOracle(OracleRun):
    """OracleRun that stacks the history (build_interpolant) only when asked:
    the dipole's history holds ~260 slices of 500^2 cells."""

    def step(self, k):
        self.beam6 = self.plan.matrix(k) @ self.beam6
        self.position = self.plan.positions[k]
        st = self.stats()
        self.lf = self.plan.formation_length(k, st["sigma_z"])
        self.df_step(self.lf)
        return self.lf


@cuda
def test_dipole_full_size_fp64_vs_oracle():
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import workload
    wl = workload("dipole_c1")
    steps = wl.n_steps
    orc = _LazyOracle(wl.lattice, wl.beam(), wl.deposit, wl.integration, grid_rule="reference")
    run = WakeRun(wl.lattice, wl.beam(), wl.deposit, wl.integration, wl.mesh, precision="fp64",
                  grid_rule="reference")
    orc.init()
    for k in range(1, steps + 1):
        orc.step(k)
        run.step(k)
    orc.tracker.build_interpolant()
    tr = run.csr.DF_tracker
    assert tr.ring.count == len(orc.tracker.time_interp)
    # history: first, middle and last slice of density and density_x
    ring = tr.ring
    for name in ("density", "density_x"):
        ref = getattr(orc.tracker, f"data_{name}_interp")
        for k in (0, ring.count // 2, ring.count - 1):
            dev = ring.slice(k, name)
            assert np.abs(dev - ref[k]).max() <= 1e-10 * np.abs(ref[k]).max(), (name, k)
    st = orc.stats()
    xm, zm, _, _ = O.csr_mesh(st, wl.mesh["xbins"], wl.mesh["zbins"], wl.mesh["xlim"],
                              wl.mesh["zlim"])
    pts = np.linspace(0, xm.size - 1, 16).astype(int)
    ref = orc.wake_oracle().points(orc.position + zm[pts], xm[pts], nthreads=16)
    csr = run.csr
    csr.get_CSR_mesh()
    s, x = csr.mesh_device()
    dE, xk = csr.wake_device(s, x, "fp64")
    dE, xk = dE.cpu().numpy()[pts], xk.cpu().numpy()[pts]
    assert rel_err(dE, ref[0]) < 1e-8
    assert rel_err(xk, ref[1]) < 1e-8


def _mixed_vs_fp64(name, steps, check_at, near_band=0.0):
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import workload
    wl = workload(name)
    run = WakeRun(wl.lattice, wl.beam(), wl.deposit, wl.integration, wl.mesh, precision="both",
                  grid_rule="configured", host_transport=False)
    out = []
    for k in range(1, steps + 1):
        run.step(k)
        if k in check_at:
            csr = run.csr
            csr.get_CSR_mesh()
            s, x = csr.mesh_device()
            dE64, xk64 = (t.cpu().numpy() for t in csr.wake_device(s, x, "fp64"))
            res = {}
            for band in (0.0, near_band) if near_band else (0.0,):
                csr.near_band = band
                dE, xk = (t.cpu().numpy() for t in csr.wake_device(s, x, "mixed"))
                dE2, xk2 = (t.cpu().numpy() for t in csr.wake_device(s, x, "mixed"))
                assert np.array_equal(dE, dE2) and np.array_equal(xk, xk2)   # repeatable
                res[band] = wake_errors(dE, xk, dE64, xk64)
            csr.near_band = 0.0
            out.append((k, abs(run.beam._slope[0]), res))
    return out


@cuda
def test_double_horn_full_size_mixed_vs_fp64():
    """Inside the first bend's drift (3-region branch) and later, once the
    x-z slope exceeds 1 (4-region chirped branch)."""
    out = _mixed_vs_fp64("chicane_c3", 40, (12, 40))
    assert out[0][1] < 1.0 < out[-1][1]
    for k, slope, res in out:
        e = res[0.0]
        assert max(e.values()) <= 1e-4, (k, slope, e)


@cuda
def test_large_beam_full_size_mixed_vs_fp64_with_band():
    from pydfcsr_gb300.synthetic import workload
    sz = 30e-6
    out = _mixed_vs_fp64("chicane_c5", 230, (10, 120, 230), near_band=20 * sz)
    assert workload("chicane_c5").n_particles == 10_000_000
    assert out[0][1] < 1.0 < out[1][1] and out[2][1] > 1.0
    for k, slope, res in out:
        for band, e in res.items():
            assert max(e.values()) <= 1e-4, (k, band, e)


@cuda
def test_chicane_whole_run_mixed_vs_fp64():
    """The benchmark's chicane beam over all 100 steps (both branches of
    get_CSR_wake, the first steps with two or three history slices), every
    5th step and the first two, without and with the FP64 near band
    (20 sigma_z)."""
    steps = (1, 2) + tuple(range(5, 101, 5))
    out = _mixed_vs_fp64("chicane_c2", 100, steps, near_band=20 * 50e-6)
    assert any(slope > 1.0 for _, slope, _ in out) and any(slope < 1.0 for _, slope, _ in out)
    for k, slope, res in out:
        for band, e in res.items():
            assert max(e.values()) <= 1e-4, (k, slope, band, e)
