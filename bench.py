#!/usr/bin/env python
"""Wake-point throughput of the per-step CSR wake path on one GB300.

Workload (the metric's configuration): the four-dipole chicane with a
2e6-particle Gaussian beam (sigma_z 50 um, sigma_x 20 um, chirp h = -10 1/m,
sigma_delta 1e-4, 1 GeV, seeded), 256x256 deposit grid (SG window 9, order 2),
64x64 observation mesh every step, 100 steps over 6.5 m, integration bins
100x100, n_formation_length 1.5, mixed precision (FP32 bulk, FP64 retarded
geometry).  Synthetic data (seeded numpy beam, r_gen6 transport between
steps).

One step = get_DF (device moments, deposit, DF finalisation) + append_DF +
append_interpolant (history ring regrid) + build_interpolant +
get_CSR_mesh + the wake on all 4096 mesh points.

  value        wake points/s with each step's particles already in HBM
  e2e          the same through the public CSR2D calls with HOST buffers:
               pinned-host -> device copy of (x, px, z) every step and the
               (dE_dct, x_kick) result read back every step
  roofline     dominant kernel (wake_mixed_integral), CUDA events on its
               launch stream inside the timed region
  cpu_baseline the CPU oracle (C restatement of the reference, all threads)
               on a bounded sample of the same workload

``--impl reference`` times the CPU oracle (the reference's algorithm restated
in C + numpy; the reference itself is Python/numba and not available on the
GPU host) on the same config and prints the same metric.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "chicane_c2"
METRIC = "wake points/sec (64x64 mesh per step, chicane 2e6 particles, 256x256 grid)"
UNIT = "wake_points/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--particles", type=int, default=None, help="override N (testing only)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain-FP64 comparison leg")
    ap.add_argument("--serve-requests", type=int, default=256,
                    help="requests in the serving stream (0 skips the serving leg)")
    ap.add_argument("--serve-rate", type=float, default=20.0, help="Poisson arrival rate (1/s)")
    ap.add_argument("--serve-fp64-every", type=int, default=16,
                    help="every n-th request of the stream (with its arrival time) is also served "
                         "by the plain FP64 kernels (0 skips)")
    ap.add_argument("--first-step", type=int, default=None,
                    help="first timed step (default: the K timed steps straddle the 3- to "
                         "4-region transition)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the full-run, accuracy and other-workload legs")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(x, world, device):
    """Max of a per-rank float over all ranks (the slowest rank's time sets
    the job's time); ``device`` is where the collective's tensor lives
    ('cuda' under NCCL, 'cpu' under gloo)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(points_per_rank_step, world, step_ms):
    """Whole-job wake points/s: every rank evaluates its own beam's mesh
    (weak scaling), timed by the slowest rank."""
    return world * points_per_rank_step * 1000.0 / step_ms


def beam_seed(rank):
    """Each rank runs an independent beam: the workload's seed offset by rank."""
    return rank


def workload_config(n_particles, precision, first=None, last=None, warmup=None):
    c = {"workload": "chicane_c2: 4 dipoles 0.5 m +-0.05 rad, drifts 2/0.5/2 m, "
                     "1 GeV, N=%d, sigma_z 50um, sigma_x 20um, h=-10/m, grid 256x256, "
                     "SG 9/2, mesh 64x64 every step, 100x100 integration bins" % n_particles,
         "precision": precision,
         "l2": "inputs larger than L2: distinct 96 MB particle set per step; history ring "
               ">= 190 MB"}
    if first is not None:
        c["timed_steps"] = [first, last]
        c["window"] = ("steps 1..%d build the history untimed, %d warm-up steps, then the timed "
                       "steps, which straddle step 35 where |x-z slope| first exceeds 1 "
                       "(3- then 4-region branch of get_CSR_wake)" % (first - warmup - 1, warmup))
    return c


def lattice_for(wl, total_steps):
    """The workload's chicane, extended by a drift if more steps are asked."""
    from pydfcsr_gb300.synthetic import StepPlan
    lat = wl.lattice.copy()
    plan = StepPlan(lat)
    if total_steps + 1 > len(plan.positions):
        extra = (total_steps + 1 - len(plan.positions) + 1) * float(lat["step_size"])
        lat["Dtail"] = {"type": "drift", "L": extra, "nsep": 1}
    return lat


# ------------------------------------------------------------------ clocks
# NVML poller run as a subprocess (no GIL contention with the step loop):
# one line "wall time, SM MHz, max SM MHz, event-reason bits" every 2 ms.
_NVML_POLLER = r"""
import ctypes, sys, time
lib = ctypes.CDLL("libnvidia-ml.so.1")
if lib.nvmlInit_v2() != 0:
    sys.exit(1)
h = ctypes.c_void_p()
if lib.nvmlDeviceGetHandleByIndex_v2(ctypes.c_uint(int(sys.argv[1])), ctypes.byref(h)) != 0:
    sys.exit(1)
clk, mx, rs = ctypes.c_uint(), ctypes.c_uint(), ctypes.c_ulonglong()
lib.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))          # NVML_CLOCK_SM
reasons = (getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None)
           or lib.nvmlDeviceGetCurrentClocksThrottleReasons)
while True:
    lib.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(clk))
    reasons(h, ctypes.byref(rs))
    sys.stdout.write("%.6f,%d,%d,%d\n" % (time.time(), clk.value, mx.value, rs.value))
    sys.stdout.flush()
    time.sleep(0.002)
"""

# NVML clock event reason bits (nvml.h) reported by the benchmark
_REASON_BITS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
                0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}


class ClockSampler:
    """SM clocks and throttle reasons during a region: NVML polled every 2 ms
    by a subprocess (samples inside [mark_start, mark_end] are kept), else
    nvidia-smi every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []
        self.nvml = False
        self.t0 = self.t1 = None

    def _spawn(self, argv):
        self.proc = subprocess.Popen(argv, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                                     text=True)
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def start(self):
        """Start sampling; with NVML, wait (at most 10 s) for the first sample."""
        try:
            self._spawn([sys.executable, "-c", _NVML_POLLER, str(self.index)])
            t_end = time.time() + 10.0
            while not self.lines and self.proc.poll() is None and time.time() < t_end:
                time.sleep(0.005)
            if self.lines:
                self.nvml = True
                return
            self.proc.kill()
        except OSError:
            pass
        self.lines = []
        try:
            self._spawn(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                         "--format=csv,noheader,nounits", "-lms", "200"])
        except OSError:
            self.proc = None

    def mark_start(self):
        self.t0 = time.time()

    def mark_end(self):
        self.t1 = time.time()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        if self.nvml:
            for ln in list(self.lines):
                f = ln.split(",")
                if len(f) != 4:
                    continue
                ts, clk, mxc, bits = float(f[0]), float(f[1]), float(f[2]), int(f[3])
                if self.t0 is not None and not (self.t0 <= ts <= (self.t1 or ts)):
                    continue
                sm.append(clk)
                mx.append(mxc)
                for bit, nm in _REASON_BITS.items():
                    if bits & bit:
                        reasons.add(nm)
            return {"sm_mhz": float(np.median(sm)) if sm else None,
                    "sm_max_mhz": float(max(mx)) if mx else None,
                    "reasons": sorted(reasons), "samples": len(sm),
                    "source": "NVML, every 2 ms, inside the timed region"}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(mx)) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "source": "nvidia-smi, every 200 ms"}


# -------------------------------------------------------------- GPU arm
def make_run(wl, lattice, precision, seed_offset=0):
    from pydfcsr_gb300.harness import WakeRun
    beam = wl.beam(seed=(wl_seed(wl) + seed_offset))
    return WakeRun(lattice, beam, wl.deposit, wl.integration, wl.mesh, precision=precision,
                   grid_rule="configured", host_transport=False), beam


def wl_seed(wl):
    """The workload's own beam seed (chicane_c2 keeps the seed its benchmark
    has always used)."""
    return {"chicane_c2": 2, "chicane_c3": 3, "chicane_c5": 5, "dipole_c1": 1}.get(wl.name, 2)


def device_step_sets(run, steps, first=1):
    """Transport on the device once (before timing, dfcsr_transport6) and keep
    every step's particle set resident: list of (6, N) float64 CUDA tensors
    for steps first..steps (index k - first), starting from the run's current
    particles (those of step first - 1)."""
    import ctypes
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import ptr, stream_handle
    sets = []
    cur = run.beam.particle
    for k in range(first, steps + 1):
        cur = cur.clone()
        R = np.ascontiguousarray(run.plan.matrix(k))
        _lib.call("dfcsr_transport6", R.ctypes.data_as(ctypes.c_void_p), ptr(cur), cur.shape[1],
                  cur.stride(0), stream_handle())
        sets.append(cur)
    return sets


def timed_steps(run, sets, first, count, precision, events=None, wake=True, side=None, set0=1):
    """Run steps first..first+count-1 from device-resident particle sets
    (sets[k - set0] holds step k); ``events`` (list) receives one (start,
    end) CUDA event pair per step.

    Pipelined across steps (the particle sets are resident, and without kicks
    a step's particles do not depend on the previous wake), with ``side`` a
    second stream:
    * the moments of step k+2 are enqueued on ``side`` right after step k's
      wake: their small CTAs run beside the wake's persistent integral CTAs,
      on the FP64 pipe the integral leaves idle;
    * the deposit of step k+1 is enqueued on ``side`` when step k begins
      (its moments are on the host by then): it runs beside step k's DF
      finalisation, regrid, set-up and geometry kernels, which leave SMs
      free;
    * step k's DF finalisation, history and wake go to the main stream."""
    import torch
    csr, beam = run.csr, run.beam
    trk = csr.DF_tracker
    side = side if side is not None else torch.cuda.current_stream()
    stream = torch.cuda.current_stream()
    last = first + count - 1
    if count <= 0:
        return
    # the particle sets (and everything else enqueued so far) are written on
    # the current stream: the side stream's moments and deposits wait for it
    if side is not stream:
        side.wait_stream(stream)

    def status(k):                   # moments of step k (on side)
        beam.particle = sets[k - set0]
        return beam.status_async(side)

    def deposit(k, st):              # deposit of step k (on side)
        p = sets[k - set0]
        return trk.deposit_DF(p[0], p[4], p[1], st.result(), side)

    st = {first: status(first)}
    if first + 1 <= last:
        st[first + 1] = status(first + 1)
    dep = {first: deposit(first, st[first])}
    for k in range(first, last + 1):
        if events is not None:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record(stream)
        if k + 1 <= last:
            dep[k + 1] = deposit(k + 1, st[k + 1])
        beam.particle = sets[k - set0]
        beam.apply_status(st.pop(k))
        beam.position = float(run.plan.positions[k])
        beam.step = k
        lf = run.plan.formation_length(k, beam.sigma_z)
        csr.update_history(lf, deposited=dep.pop(k))
        if wake:
            csr.get_CSR_mesh()
            s, x = csr.mesh_device()
            run.last = csr.wake_device(s, x, precision)
            # get_CSR_wake's branch at this step: 4 regions when |slope| > 1
            run.branch_log = getattr(run, "branch_log", {})
            run.branch_log[k] = abs(float(beam._slope[0])) > 1
        if k + 2 <= last:
            st[k + 2] = status(k + 2)
        if events is not None:
            ev[1].record(stream)
            events.append(ev)


def tracking_steps(run, first, count, precision, step_size, early_deposit=True):
    """The reference's run loop with the CSR kick applied (CSR.py:297-334):
    transport by the step's matrix and beam statistics, the DF step, the wake
    on the mesh, Beam.apply_wakes (pz and px kicks) - every step depends on
    the previous wake, so nothing overlaps across steps.  With
    ``early_deposit`` the deposit is enqueued right behind the moments, on
    the grid taken from the device moments, before the host waits for their
    copy (the GPU deposits while the host sizes the rest of the step)."""
    from pydfcsr_gb300.runtime import as_device_f64
    csr, beam = run.csr, run.beam
    for k in range(first, first + count):
        beam.track(run.plan.matrix(k), 0.0, wait=not early_deposit)
        dep = None
        if early_deposit:
            dep = csr.DF_tracker.deposit_DF(beam.x, beam.z, beam.px, beam.moments_device)
        beam.position = float(run.plan.positions[k])
        csr.update_history(run.plan.formation_length(k, beam.sigma_z), deposited=dep)
        csr.get_CSR_mesh()
        s, x = csr.mesh_device()
        dE, xk = csr.wake_device(s, x, precision)
        xb, zb = int(csr.CSR_params.xbins), int(csr.CSR_params.zbins)
        x0, x1, _, z0, z1, _, _, _, _ = csr._mesh
        xr = as_device_f64(np.linspace(x0, x1, xb))
        zr = as_device_f64(np.linspace(z0, z1, zb))
        beam.apply_wakes(dE.view(xb, zb), xk.view(xb, zb), xr, zr, step_size, True, update=False)
        run.last = (dE, xk)


def e2e_steps(run, host_sets, first, count, precision, dev_bufs, side):
    """Steps through the public API with host buffers: H2D of (x, px, z)
    from pinned memory, CSR2D calls, D2H of (dE_dct, x_kick).

    Pipelined like timed_steps, for a caller that streams beams through
    three device buffers: step k+2's upload goes to a copy stream when step
    k begins (once step k-1's deposit has released that buffer), its moments
    to ``side`` right after step k's wake, step k+1's deposit to ``side``
    when step k begins; step k's results (calculate_2D_CSR with wait=False)
    are read back after step k+1 is enqueued.  host_sets[k - first] holds
    step k."""
    import torch
    csr, beam = run.csr, run.beam
    trk = csr.DF_tracker
    last = first + count - 1
    nb = len(dev_bufs)
    copy = torch.cuda.Stream()
    h2d = d2h = 0
    uploaded = {}                   # step -> event after its upload

    def upload(k, after=None):
        xpz = host_sets[k - first]                  # pinned (3, N): x, px, z
        buf = dev_bufs[k % nb]
        with torch.cuda.stream(copy):
            if after is not None:
                copy.wait_event(after)              # the buffer's previous deposit
            buf[0].copy_(xpz[0], non_blocking=True)
            buf[1].copy_(xpz[1], non_blocking=True)
            buf[4].copy_(xpz[2], non_blocking=True)
            uploaded[k] = copy.record_event()
        return xpz.numel() * 8

    def status(k):
        side.wait_event(uploaded.pop(k))
        beam.particle = dev_bufs[k % nb]
        return beam.status_async(side)

    def deposit(k, st):
        p = dev_bufs[k % nb]
        return trk.deposit_DF(p[0], p[4], p[1], st.result(), side)

    st = {}
    for k in range(first, min(first + 1, last) + 1):
        h2d += upload(k)
        st[k] = status(k)
    dep = {first: deposit(first, st[first])}
    pending = None
    for k in range(first, last + 1):
        if k + 1 <= last:
            dep[k + 1] = deposit(k + 1, st[k + 1])
        if k + 2 <= last:
            # buffer (k + 2) % 3 held step k - 1, whose deposit has been enqueued
            prev = dep.get(k - 1)
            h2d += upload(k + 2, prev.event if prev is not None else None)
        beam.particle = dev_bufs[k % nb]
        beam.apply_status(st.pop(k))
        beam.position = float(run.plan.positions[k])
        lf = run.plan.formation_length(k, beam.sigma_z)
        d = dep.pop(k)
        csr.update_history(lf, deposited=d)
        dep[k - 1] = None
        dep[k] = d                                  # kept until step k + 3's upload
        csr.get_CSR_mesh()
        nxt = csr.calculate_2D_CSR(precision, wait=False)
        if k + 2 <= last:
            st[k + 2] = status(k + 2)
        if pending is not None:
            dE, xk = pending.result()               # step k-1 on the host
            d2h += dE.nbytes + xk.nbytes
        pending = nxt
    dE, xk = pending.result()
    d2h += dE.nbytes + xk.nbytes
    return h2d // count, d2h // count


def timed_window(W, K, transition, n_steps):
    """First timed step: the K timed steps straddle the step where the
    beam's x-z slope first exceeds 1 in magnitude (get_CSR_wake switches
    from its 3-region to its 4-region branch there), so that both branches
    are timed; at least W warm-up steps come before it."""
    first = max(W + 1, transition - K // 2)
    return max(W + 1, min(first, n_steps - K + 1))


# x-z slope first exceeds 1 in magnitude at these steps (chirp h = -10 1/m and
# -20 1/m through the chicane; checked by the accuracy scans below)
TRANSITION = {"chicane_c2": 35, "chicane_c3": 35, "chicane_c5": 57}


def build_history(run, upto):
    """Steps 1..upto on the device without the wake (transport, moments, DF,
    history): the history a timed window starts from."""
    for k in range(1, upto + 1):
        run.step(k)


def time_workload(name, precision, W, K, side, first=None, n_particles=None, points_note="",
                  peaks=None):
    """Time K steps of a workload (DF + history + wake on its whole mesh)
    after W warm-up steps, pipelined like the headline loop.  Returns the
    measurement and the run (its last step's wake in run.last).  With
    ``peaks`` = (HBM GB/s, FMA peaks, SM clock MHz) the measurement also
    carries each stage's roofline and the dominant kernel's."""
    import torch
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.synthetic import workload
    wl = workload(name, n_particles=n_particles)
    if first is None:
        first = timed_window(W, K, TRANSITION.get(name, W + 1), wl.n_steps)
    lattice = lattice_for(wl, first + K - 1)
    run, _ = make_run(wl, lattice, precision)
    f0 = first - W
    build_history(run, f0 - 1)
    sets = device_step_sets(run, first + K - 1, first=f0)
    timed_steps(run, sets, f0, W, precision, side=side, set0=f0)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    _lib.timing_reset()
    _lib.timing_enable(True)
    ev = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    timed_steps(run, sets, first, K, precision, events=ev, side=side, set0=f0)
    e1.record(stream)
    torch.cuda.synchronize()
    kt = {n: _lib.timing_read(n) for n in STAGES}
    _lib.timing_enable(False)
    ms = e0.elapsed_time(e1) / K
    npts = wl.mesh["xbins"] * wl.mesh["zbins"]
    del sets
    out = {"workload": workload_name(wl), "precision": precision, "steps": [first, first + K - 1],
           "warmup": W, "ms_per_step": ms, "wake_points_per_s": npts * 1000.0 / ms,
           "mesh_points": npts, "step_ms_p50": float(np.median([a.elapsed_time(b) for a, b in ev])),
           "kernel_ms_per_step": {n: round(v[0] / K, 4) for n, v in kt.items() if v[1]}}
    if peaks is not None:
        hbm, fma_peaks, clock_mhz = peaks
        kname = "wake_mixed_integral" if precision == "mixed" else "wake_fp64"
        k_ms, k_n = kt[kname]
        if k_n:
            n_sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
            out["roofline"] = roofline(kname, k_ms / k_n, k_n,
                                       integrand_points(wl, run, range(first, first + K)), npts,
                                       fma_peaks, hbm, precision, clock_mhz, n_sms)
        out["stages"] = stage_rooflines(kt, K, wl, run, hbm, fma_peaks)
    return out, run, wl


def workload_name(wl):
    m, d = wl.mesh, wl.deposit
    return (f"{wl.name}: N={wl.n_particles}, grid {d['xbins']}x{d['zbins']}, mesh "
            f"{m['xbins']}x{m['zbins']} every step, {wl.n_steps} steps, integration bins "
            f"{wl.integration['xbins']}x{wl.integration['zbins']}")


def accuracy_scan(name, steps, every, n_particles=None):
    """The mixed wake against the plain FP64 kernel (itself the reference's
    arithmetic, bit-exact on the same history) on the same history, at every
    ``every``-th step of a whole run: per step max_rel, rms_rel and the
    pointwise errors, the x-z slope and the branch (3 or 4 regions)."""
    from pydfcsr_gb300.harness import WakeRun
    from pydfcsr_gb300.synthetic import workload
    wl = workload(name, n_particles=n_particles)
    run = WakeRun(wl.lattice, wl.beam(seed=wl_seed(wl)), wl.deposit, wl.integration, wl.mesh,
                  precision="both", grid_rule="configured", host_transport=False)
    rows = []
    for k in range(1, steps + 1):
        run.step(k)
        if k % every and k != steps:
            continue
        csr = run.csr
        csr.get_CSR_mesh()
        s, x = csr.mesh_device()
        dE64, xk64 = (t.cpu().numpy() for t in csr.wake_device(s, x, "fp64"))
        dE, xk = (t.cpu().numpy() for t in csr.wake_device(s, x, "mixed"))
        e = wake_errors(dE, xk, dE64, xk64)
        slope = float(run.beam._slope[0])
        rows.append({"step": k, "slope": round(slope, 4), "regions": 4 if abs(slope) > 1 else 3,
                     **{kk: float("%.3g" % v) for kk, v in e.items()}})
    worst = {kk: max(r[kk] for r in rows) for kk in ("max_rel", "rms_rel", "pointwise_dE",
                                                     "pointwise_xk")}
    return {"workload": workload_name(wl), "every": every, "steps_checked": len(rows),
            "steps_4_region": sum(r["regions"] == 4 for r in rows), "worst": worst,
            "per_step": rows}


# stages of the step timed with CUDA events (dfcsr_timing_*)
STAGES = ("beam_moments", "deposit_cic2d", "df_finalize", "history_regrid", "wake_fp64",
          "wake_mixed_geometry", "wake_mixed_integral", "wake_mixed_band")


def gpu_arm(a):
    import torch
    import torch.distributed as dist
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.synthetic import workload

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    wl = workload(WORKLOAD, n_particles=a.particles)
    W, K = max(a.warmup, 0), a.steps
    first = a.first_step or timed_window(W, K, TRANSITION[WORKLOAD], wl.n_steps)
    last = first + K - 1
    lattice = lattice_for(wl, last)
    run, beam0 = make_run(wl, lattice, a.precision, seed_offset=beam_seed(rank))
    sets = device_step_sets(run, last)
    npts = wl.mesh["xbins"] * wl.mesh["zbins"]

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    # the history up to the window (untimed), then W warm-up steps; the side
    # stream carries the next step's moments and deposit
    side = torch.cuda.Stream()
    timed_steps(run, sets, 1, first - W - 1, a.precision, wake=False, side=side)
    timed_steps(run, sets, first - W, W, a.precision, side=side)
    barrier()
    fma_peaks = measure_fma_peaks()
    barrier()
    _lib.timing_reset()
    _lib.timing_enable(True)
    clocks = ClockSampler(local)
    clocks.start()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    t0 = time.perf_counter()
    step_events = []
    clocks.mark_start()
    n_launch0 = _lib.kernel_launches()
    e0.record(stream)
    timed_steps(run, sets, first, K, a.precision, events=step_events, side=side)
    e1.record(stream)
    n_launch = _lib.kernel_launches() - n_launch0
    barrier()
    clocks.mark_end()
    wall = time.perf_counter() - t0
    ck = clocks.stop()
    _lib.timing_enable(False)
    dev_ms = e0.elapsed_time(e1)
    kname = "wake_mixed_integral" if a.precision == "mixed" else "wake_fp64"
    kt = {n: _lib.timing_read(n) for n in STAGES}
    k_ms, k_n = kt[kname]
    launches = {n: v[1] for n, v in kt.items()}
    kernel_ms = {n: round(v[0] / K, 4) for n, v in kt.items() if v[1]}
    step_ms = max_over_ranks(dev_ms / K, world, "cuda")
    value = job_value(npts, world, step_ms)

    lat = np.array([ev[0].elapsed_time(ev[1]) for ev in step_events])
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K,
           "warmup": W, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32+f64" if a.precision == "mixed" else "f64",
           "data": "synthetic (seeded numpy Gaussian beam, r_gen6 transport)",
           "config": workload_config(run.beam.n_particle, a.precision, first, last, W),
           "wall_s_timed": wall, "clocks": ck,
           "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                          "definition": "device time of one full step (DF + history + wake)"}}

    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    if k_n:
        n_sms = torch.cuda.get_device_properties(local).multi_processor_count
        out["roofline"] = roofline(kname, k_ms / k_n, k_n,
                                   integrand_points(wl, run, range(first, last + 1)), npts,
                                   fma_peaks, hbm, a.precision, ck.get("sm_mhz"), n_sms)
    out["stages"] = stage_rooflines(kt, K, wl, run, hbm, fma_peaks)
    out["peaks_measured"] = fma_peaks
    out["gpu_launches"] = int(n_launch)   # this library's kernel launches in the timed region
    out["entry_calls_by_name"] = launches
    out["kernel_ms_per_step"] = kernel_ms
    del sets

    # the whole run, all steps timed (both branches in their real proportion)
    if not a.no_extras:
        out["full_run"] = full_run(wl, a.precision, side)

    # plain FP64 leg on the same steps (for the mixed vs FP64 speed-up)
    if not a.no_fp64 and a.precision == "mixed":
        r64, _ = make_run(wl, lattice, "fp64", seed_offset=beam_seed(rank))
        sets = device_step_sets(r64, last)
        K64 = min(K, 3)
        timed_steps(r64, sets, 1, last - K64 - 1, "fp64", wake=False, side=side)
        timed_steps(r64, sets, last - K64, 1, "fp64", side=side)   # warm the FP64 kernel
        torch.cuda.synchronize()
        f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        f0.record(stream)
        timed_steps(r64, sets, last - K64 + 1, K64, "fp64", side=side)
        f1.record(stream)
        torch.cuda.synchronize()
        ms64 = f0.elapsed_time(f1) / K64
        # accuracy of the mixed result vs the FP64 kernel on the last step
        dE32, xk32 = (t.cpu().numpy() for t in run.last)       # last timed step, mixed
        dE64, xk64 = (t.cpu().numpy() for t in r64.last)       # same step, plain FP64
        out["plain_fp64"] = {"ms_per_step": ms64, "value": npts * 1000.0 / ms64, "steps": K64,
                             "mixed_speedup": ms64 / step_ms,
                             "mixed_vs_fp64": wake_errors(dE32, xk32, dE64, xk64),
                             "error_definition": ERROR_DEF + " (last timed step)"}
        del r64, sets
        torch.cuda.empty_cache()

    # end to end through the public API with host buffers
    if not a.no_e2e:
        re2e, _ = make_run(wl, lattice, a.precision, seed_offset=beam_seed(rank))
        sets = device_step_sets(re2e, last)
        timed_steps(re2e, sets, 1, first - W - 1, a.precision, wake=False, side=side)   # history
        host_sets = []
        for t in sets[first - W - 1:last]:
            h = torch.empty((3, t.shape[1]), dtype=torch.float64, pin_memory=True)
            h.copy_(t[[0, 1, 4]])
            host_sets.append(h)
        del sets
        dev_bufs = [torch.zeros_like(re2e.beam.particle) for _ in range(3)]
        e2e_steps(re2e, host_sets[:W], first - W, W, a.precision, dev_bufs, side)
        barrier()
        g0 = time.perf_counter()
        h2d, d2h = e2e_steps(re2e, host_sets[W:], first, K, a.precision, dev_bufs, side)
        barrier()
        e2e_s = time.perf_counter() - g0
        out["e2e"] = {"value": world * npts * K / e2e_s, "unit": UNIT,
                      "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                      "ms_per_step": e2e_s * 1000 / K}
        del re2e, host_sets
        torch.cuda.empty_cache()

    # the full tracking step with the kick fed back (no overlap possible)
    if not a.no_e2e:
        rtr, _ = make_run(wl, lattice, a.precision, seed_offset=beam_seed(rank))
        step = float(lattice["step_size"])
        tracking_steps(rtr, 1, first - 1, a.precision, step)
        barrier()
        q0, q1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        q0.record(stream)
        tracking_steps(rtr, first, K, a.precision, step)
        q1.record(stream)
        barrier()
        ms_tr = max_over_ranks(q0.elapsed_time(q1) / K, world, "cuda")
        out["tracking_with_kicks"] = {
            "value": job_value(npts, world, ms_tr), "unit": UNIT, "ms_per_step": ms_tr,
            "steps": [first, last],
            "definition": "Beam.track (transport kernel + statistics), get_DF / history, mesh, "
                          "wake, Beam.apply_wakes with the wake (pz and px kicks) every step: the "
                          "reference's run loop with apply_CSR; particles stay on the device"}
        del rtr
        torch.cuda.empty_cache()

    if not a.no_extras and a.precision == "mixed":
        out["accuracy"] = {"error_definition": ERROR_DEF,
                           "chicane_c2": accuracy_scan(WORKLOAD, wl.n_steps, 1)}
        rows = [r for r in out["accuracy"]["chicane_c2"]["per_step"] if first <= r["step"] <= last]
        out["timed_window_branches"] = {"steps": [first, last],
                                        "3_region": sum(r["regions"] == 3 for r in rows),
                                        "4_region": sum(r["regions"] == 4 for r in rows)}
        out["workloads"] = other_workloads(W, K, side, out["accuracy"],
                                           peaks=(hbm, fma_peaks, ck.get("sm_mhz")))

    if a.serve_requests > 0 and a.precision == "mixed":
        out["serving"] = serving_leg(a.serve_requests, a.serve_rate, a.serve_fp64_every,
                                     seed=4 + 1000 * rank)

    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(wl, lattice, sample_steps=2, warm_steps=4, n_obs=32)
    if world > 1:
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(out))


ERROR_DEF = ("S = peak |wake| of the FP64 result over the mesh and both components: max_rel = "
             "max|a-b|/S, rms_rel = ||a-b||/||b||, pointwise = max|a-b|/max(|b|, 1e-3 S) per "
             "component; the FP64 kernel is the reference's arithmetic (bit-exact given the "
             "same history)")


def full_run(wl, precision, side):
    """All steps of the workload timed one after another (device-resident
    particle sets, the headline's pipelined loop): ms per step overall and
    per branch of get_CSR_wake."""
    import torch
    lattice = lattice_for(wl, wl.n_steps)
    run, _ = make_run(wl, lattice, precision)
    sets = device_step_sets(run, wl.n_steps)
    timed_steps(run, sets, 1, 3, precision, side=side)          # warm-up on a fresh copy
    run, _ = make_run(wl, lattice, precision)
    ev = []
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    timed_steps(run, sets, 1, wl.n_steps, precision, events=ev, side=side)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in ev]
    total = e0.elapsed_time(e1)
    npts = wl.mesh["xbins"] * wl.mesh["zbins"]
    del sets
    torch.cuda.empty_cache()
    return {"steps": wl.n_steps, "ms_per_step": total / wl.n_steps,
            "wake_points_per_s": npts * wl.n_steps * 1000.0 / total,
            "step_ms": [round(v, 3) for v in ms],
            "definition": "every step of the run timed (history from step 1; the first steps "
                          "have short histories)"}


def other_workloads(W, K, side, accuracy, peaks=None):
    """C1 (the plain FP64 drop-in on the dipole, at its exit), C3 (double-horn
    chicane) and C5 (large beam, 300 steps): a timed window each, and the
    accuracy scans of C3 and C5."""
    import torch
    out = {}
    K1 = min(K, 5)
    # C1: the plain FP64 method, wake on the 32x32 mesh at the last K1 steps
    # up to the dipole exit (step 300), and the mixed form on the same steps
    c1 = {}
    for prec in ("fp64", "mixed"):
        m, run, wl = time_workload("dipole_c1", prec, min(W, 3), K1, side, first=300 - K1 + 1,
                                   peaks=peaks)
        c1[prec] = m
        dE, xk = (t.cpu().numpy() for t in run.last)
        c1[prec + "_last"] = (dE, xk)
        del run
        torch.cuda.empty_cache()
    e = wake_errors(*c1.pop("mixed_last"), *c1.pop("fp64_last"))
    c1["mixed_vs_fp64_at_exit"] = e
    c1["mixed_speedup"] = c1["fp64"]["ms_per_step"] / c1["mixed"]["ms_per_step"]
    out["C1_dipole"] = c1
    for key, name, every in (("C3_double_horn", "chicane_c3", 4), ("C5_large_beam", "chicane_c5", 10)):
        m, run, wl = time_workload(name, "mixed", W, K, side, peaks=peaks)
        del run
        torch.cuda.empty_cache()
        m64, run, _ = time_workload(name, "fp64", 2, 2, side, first=m["steps"][1] - 1)
        del run
        torch.cuda.empty_cache()
        m["plain_fp64_ms_per_step"] = m64["ms_per_step"]
        m["mixed_speedup"] = m64["ms_per_step"] / m["ms_per_step"]
        out[key] = m
        accuracy[name] = accuracy_scan(name, wl.n_steps, every)
        torch.cuda.empty_cache()
    return out


def integrand_points(wl, run, steps):
    """Integrand points of the wake over ``steps`` per observation point:
    4 x xbins x zbins in the 3-region branch of get_CSR_wake, 5 x in the
    4-region one (the branch of each step as timed_steps logged it)."""
    ip = wl.integration
    per = ip["xbins"] * ip["zbins"]
    return sum((5 if run.branch_log[k] else 4) * per for k in steps)


def roofline(kname, launch_ms, launches, per_obs_total, npts, fma_peaks, hbm, precision, clock_mhz,
             n_sms):
    """Roofline object of the dominant kernel: ``per_obs_total`` integrand
    points per observation point summed over the timed steps."""
    pts = npts * per_obs_total / launches        # integrand points per launch
    if precision == "mixed":
        flops = INTEGRAL_FLOPS_PER_POINT * pts
        peak = fma_peaks["fp32_tflops"]
        achieved = flops / (launch_ms * 1e-3) / 1e12
        traffic = INTEGRAL_DRAM_BYTES_PER_POINT * pts
        return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": traffic,
                "dram": {"achieved_gbs": traffic / (launch_ms * 1e-3) / 1e9, "peak_gbs": hbm,
                         "frac": traffic / (launch_ms * 1e-3) / 1e9 / hbm,
                         "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
                "kernel": kname, "launch_ms": launch_ms, "launches": launches,
                "integrand_points_per_launch": pts,
                "algorithmic": f"{INTEGRAL_FLOPS_PER_POINT} FP32 floating-point operations per "
                               "integrand point (FMA = 2; executed thread instructions counted "
                               f"by ncu on this kernel), {pts:.3g} integrand points per launch "
                               "(per timed step: 40,000 per observation point in the 3-region "
                               "branch, 50,000 in the 4-region one)",
                "peak_source": "measured FP32 FMA rate of this GPU (peaks_measured)",
                "binding": INTEGRAL_BINDING,
                "issue": issue_bound(pts, launch_ms, clock_mhz, n_sms)}
    flops = 300 * pts
    peak = fma_peaks["fp64_tflops"]
    achieved = flops / (launch_ms * 1e-3) / 1e12
    return {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "traffic": None, "kernel": kname, "launch_ms": launch_ms,
            "launches": launches, "algorithmic": "~300 FP64 operations per integrand point",
            "peak_source": "measured FP64 FMA rate of this GPU (peaks_measured)"}


# From an ncu capture of wake_mixed_integral on this workload at a 4-region
# step (the ncu --set full capture of step 40's launch, 2.048e8 integrand points):
# FP32 operations per integrand point from the executed (predicated-on)
# thread instructions (23.28e9 FADD + 3.11e9 FMUL + 2 x 5.89e9 FFMA), DRAM
# bytes per integrand point (345.8 + 4.3 MB), warp instructions per
# integrand point (1407.6e6 issued), and the binding unit.
INTEGRAL_FLOPS_PER_POINT = 186
INTEGRAL_DRAM_BYTES_PER_POINT = 1.71
INTEGRAL_WARP_INSTR_PER_POINT = 6.87
INTEGRAL_BINDING = ("instruction issue (68.5 % of issue slots used at 16 warps per SM; stalls per "
                    "issued instruction: long-scoreboard 1.3, not-selected 1.2, wait 1.0, barrier "
                    "0.3); FMA pipe 56 %, L1TEX 63 %, L2 hits 94 %, DRAM 3 %; the FP32 mix is "
                    "mostly FADD (double-word arithmetic: 114 FADD, 29 FFMA, 15 FMUL per "
                    "integrand point), so the FMA-rate peak overstates what the pipe can reach")


def issue_bound(pts, launch_ms, clock_mhz, n_sms):
    """The integral against its instruction-issue ceiling: one warp
    instruction per cycle on each of an SM's four schedulers, at the SM clock
    sampled during the timed region."""
    if not clock_mhz:
        return None
    need = INTEGRAL_WARP_INSTR_PER_POINT * pts
    ideal_ms = need / (n_sms * 4 * clock_mhz * 1e6) * 1e3
    return {"warp_instructions_per_launch": need, "ideal_ms": ideal_ms, "launch_ms": launch_ms,
            "frac": ideal_ms / launch_ms, "clock_mhz": clock_mhz, "sms": n_sms,
            "how": "%.2f warp instructions per integrand point (ncu) / (SMs x 4 schedulers x SM "
                   "clock)" % INTEGRAL_WARP_INSTR_PER_POINT}


def stage_rooflines(kt, K, wl, run, hbm, fma_peaks):
    """Each stage of the step against its roofline: CUDA-event time per
    launch, algorithmic bytes (or operations) per launch, the fraction of the
    bounding peak."""
    n = run.beam.n_particle
    d = wl.deposit
    cells = d["xbins"] * d["zbins"]
    tr = run.csr.DF_tracker
    nxi, nzi = tr.ring.nx, tr.ring.nz
    npts = wl.mesh["xbins"] * wl.mesh["zbins"]
    ip = wl.integration
    rec = (4 * ip["zbins"] * 144 + 5 * ip["xbins"] * 32)   # record bytes written per point (bound)
    # (algorithmic bytes per step, FP64 operations per step or None, what
    # the bytes are, the unit that binds the stage per its ncu profile)
    algo = {
        "beam_moments": (32.0 * n, 15.0 * n, "2 passes x (x, z) FP64 = 32 B per particle; 15 FP64 "
                         "operations per particle (shifted sums)", "FP64 pipe"),
        "deposit_cic2d": (24.0 * n + 16.0 * cells, 20.0 * n,
                          "x, z, px read once (24 B per particle) + 2 grids written; 20 FP64 "
                          "operations per particle (cell keys 6, per-cell moment sums 14)",
                          "FP64 pipe (moment sums) and the latency of the sort passes"),
        "df_finalize": (7 * 8.0 * cells, None, "2 fields read + 5 written, 8 B per cell",
                        "latency of nine dependent phases (grid barriers, FP64 reductions) over "
                        f"a grid of {cells} cells"),
        "history_regrid": (32.0 * nxi * nzi + 40.0 * cells, 40.0 * nxi * nzi,
                           "one FP32 ring slot written (32 B per cell) + 5 source fields read; "
                           "5 fields x 4 corners x 2 FP64 operations per target cell",
                           "FP64 latency"),
        "wake_mixed_geometry": (float(npts * rec), None,
                                "per-point column and row records written (bound)",
                                "issue (double-word FP32 arithmetic)"),
    }
    out = {}
    for name, (work, fp64, how, binding) in algo.items():
        ms, launches = kt.get(name, (0.0, 0))
        if not launches:
            continue
        per_launch_ms = ms / launches
        per_launch_work = work * K / launches
        gbs = per_launch_work / (per_launch_ms * 1e-3) / 1e9
        out[name] = {"ms_per_step": ms / K, "launches_per_step": launches / K,
                     "achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                     "bound": "hbm", "algorithmic": how, "binding": binding}
        if fp64 is not None:
            tf = fp64 * K / launches / (per_launch_ms * 1e-3) / 1e12
            out[name]["fp64"] = {"achieved_tflops": tf, "peak_tflops": fma_peaks["fp64_tflops"],
                                 "frac": tf / fma_peaks["fp64_tflops"]}
    return out


def measure_fma_peaks():
    """FP32 and FP64 fused multiply-add throughput of this GPU (TFLOP/s),
    measured with the library's probe kernel (best of 5, CUDA events)."""
    import ctypes
    import torch
    from pydfcsr_gb300 import _lib
    from pydfcsr_gb300.runtime import ptr, stream_handle
    sink = torch.zeros(2, dtype=torch.float64, device="cuda")
    out = {}
    for name, fp64, iters in (("fp32_tflops", 0, 20000), ("fp64_tflops", 1, 600)):
        flops = ctypes.c_double()
        best = None
        for rep in range(6):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.call("dfcsr_probe_fma", fp64, iters, ptr(sink), ctypes.byref(flops), stream_handle())
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            if rep > 0:
                best = ms if best is None else min(best, ms)
        out[name] = flops.value / (best * 1e-3) / 1e12
    out["how"] = ("dfcsr_probe_fma: 8 independent FMA chains per thread, 4 x 256-thread blocks per "
                  "SM, best of 5 launches timed with CUDA events")
    return out


def serving_leg(n_requests, rate_hz, fp64_every, seed=4):
    """The request stream (single dipoles, rho ~ U(1, 20) m, angle ~
    U(0.02, 0.2), N ~ logU(1e5, 4e6), sigma_z ~ U(10, 100) um, grid from
    {64, 128, 256, 512}^2, mesh side from {32, 64, 96, 128}; 8 DF steps per
    request and a wake on its mesh at steps 2..8) served with continuous
    batching (graphs of every batch size captured before the stream starts),
    with the latency broken down; the same requests all arriving at t = 0
    (capacity); and every ``fp64_every``-th request of the stream, with its
    arrival time, served by the mixed and by the plain FP64 kernels: the
    throughput ratio on the same requests and the error of every served
    result against the FP64 one."""
    import torch
    from pydfcsr_gb300.serve import RequestSpec, WakeServer
    from pydfcsr_gb300.synthetic import serving_requests
    reqs = serving_requests(n_requests=n_requests, rate_hz=rate_hz, seed=seed)
    srv = WakeServer(reqs, precision="mixed", precapture=True)
    full = srv.run()
    del srv
    torch.cuda.empty_cache()
    out = {"stream": f"{n_requests} requests, Poisson arrivals at {rate_hz:g}/s (seed {seed}), "
                     "8 DF steps + 7 wakes each, 100x100 integration bins",
           "mixed": full}
    # capacity: the same requests all waiting at t = 0 (closed loop)
    burst = [RequestSpec.from_dict({**r, "arrival_s": 0.0}) for r in reqs]
    srv = WakeServer(burst, precision="mixed", precapture=True)
    out["capacity"] = srv.run()
    out["capacity"]["definition"] = "the same requests all arriving at t = 0"
    del srv
    torch.cuda.empty_cache()
    if fp64_every > 0:
        sub = [RequestSpec.from_dict(r) for r in reqs[::fp64_every]]
        t0 = sub[0].arrival_s
        sub = [RequestSpec(**{**r.__dict__, "arrival_s": r.arrival_s - t0}) for r in sub]
        m = WakeServer(sub, precision="mixed", precapture=True)
        sm = m.run()
        p = WakeServer(sub, precision="fp64", precapture=True)
        sp = p.run()
        worst = {"max_rel": 0.0, "rms_rel": 0.0, "pointwise_dE": 0.0, "pointwise_xk": 0.0}
        n_res = 0
        for r in sub:
            for (k, dE1, xk1), (_, dE2, xk2) in zip(m.result(r.id), p.result(r.id)):
                e = wake_errors(dE1, xk1, dE2, xk2)
                worst = {kk: max(worst[kk], e[kk]) for kk in worst}
                n_res += 1
        del m, p
        torch.cuda.empty_cache()
        # the same requests all waiting at t = 0: throughput at saturation
        burst = [RequestSpec(**{**r.__dict__, "arrival_s": 0.0}) for r in sub]
        bm = WakeServer(burst, precision="mixed", precapture=True).run()
        bp = WakeServer(burst, precision="fp64", precapture=True).run()
        out["same_stream_fp64"] = {
            "requests": len(sub), "results_compared": n_res,
            "selection": f"every {fp64_every}th request of the stream, arrival times kept",
            "mixed": sm, "fp64": sp,
            "mixed_speedup_throughput_stream": sm["wake_points_per_s"] / sp["wake_points_per_s"],
            "mixed_speedup_wake_time": sp["wake_s"] / sm["wake_s"],
            "saturated": {"mixed": bm, "fp64": bp,
                          "mixed_speedup_throughput": bm["wake_points_per_s"] / bp["wake_points_per_s"],
                          "definition": "the same requests all arriving at t = 0"},
            "notes": "with the stream's arrival times the mixed server keeps up with the arrivals, "
                     "so its throughput is the offered load; the FP64 server falls behind (see "
                     "its latencies); the saturated runs give the throughput ratio",
            "worst_vs_fp64": worst, "error_definition": ERROR_DEF + "; worst over every request "
            "and step"}
        torch.cuda.empty_cache()
    return out


def wake_errors(dE, xk, dE_ref, xk_ref):
    """max_rel / rms_rel / pointwise errors of a wake against a reference
    (S = peak of the reference wake over the mesh and both components)."""
    a = np.concatenate([np.ravel(dE), np.ravel(xk)])
    b = np.concatenate([np.ravel(dE_ref), np.ravel(xk_ref)])
    S = float(np.max(np.abs(b))) or 1.0
    nb = float(np.sqrt(np.sum(b * b))) or 1.0
    fl = 1e-3 * S
    return {"max_rel": float(np.max(np.abs(a - b)) / S),
            "rms_rel": float(np.sqrt(np.sum((a - b) ** 2)) / nb),
            "pointwise_dE": float(np.max(np.abs(np.ravel(dE) - np.ravel(dE_ref)) /
                                         np.maximum(np.abs(np.ravel(dE_ref)), fl))),
            "pointwise_xk": float(np.max(np.abs(np.ravel(xk) - np.ravel(xk_ref)) /
                                         np.maximum(np.abs(np.ravel(xk_ref)), fl)))}


# ------------------------------------------------------------- CPU oracle
def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_oracle_steps(wl, lattice, warm_steps, sample_steps, n_obs, threads):
    """Oracle over steps 1..warm+sample; returns per-step seconds for the
    DF/history part and the wake extrapolated to the full mesh."""
    from oracle import oracle as O
    from pydfcsr_gb300.synthetic import StepPlan
    plan = StepPlan(lattice)
    coords = wl.beam()
    tr = O.DFTracker(wl.deposit, grid_rule="configured")
    tr.get_DF(coords[0], coords[4], coords[1], 0.0)
    tr.append_DF()
    tr.append_interpolant(float("inf"), wl.integration["n_formation_length"])
    s, rho, dist_, nsep, tab, nv, tau = O.reference_trajectory(lattice, 2000)
    npts = wl.mesh["xbins"] * wl.mesh["zbins"]
    per_step = []
    for k in range(1, warm_steps + sample_steps + 1):
        t0 = time.perf_counter()
        coords = plan.matrix(k) @ coords
        pos = plan.positions[k]
        st = O.beam_stats(coords[0], coords[4])
        lf = plan.formation_length(k, st["sigma_z"])
        tr.get_DF(coords[0], coords[4], coords[1], pos)
        tr.append_DF()
        tr.append_interpolant(lf, wl.integration["n_formation_length"])
        tr.build_interpolant()
        t_df = time.perf_counter() - t0
        if k <= warm_steps:
            continue
        xm, zm, _, _ = O.csr_mesh(st, wl.mesh["xbins"], wl.mesh["zbins"], wl.mesh["xlim"],
                                  wl.mesh["zlim"])
        w = O.WakeOracle(tr, (s, rho, dist_, tab, nv, tau), pos, st["sigma_z"], st["sigma_x"],
                         st["slope"][0], st["mean_x"], lf, wl.integration["n_formation_length"],
                         wl.integration["zbins"], wl.integration["xbins"])
        idx = np.linspace(0, npts - 1, n_obs).astype(int)
        t1 = time.perf_counter()
        w.points(pos + zm[idx], xm[idx], nthreads=threads)
        t_w = (time.perf_counter() - t1) * npts / n_obs
        per_step.append(t_df + t_w)
    return float(np.mean(per_step)), npts


def cpu_baseline(wl, lattice, sample_steps, warm_steps, n_obs):
    threads = cpu_threads()
    sec, npts = cpu_oracle_steps(wl, lattice, warm_steps, sample_steps, n_obs, threads)
    return {"value": npts / sec, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"CPU oracle (C restatement of get_CSR_wake/get_CSR_integrand, numpy "
                      f"DF/history) on the same chicane beam: steps 1..{warm_steps + sample_steps} "
                      f"built in full, wake on {n_obs} of {npts} mesh points at each of the last "
                      f"{sample_steps} steps, scaled to the full mesh; {threads} threads"}


def reference_arm(a):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from pydfcsr_gb300.synthetic import workload
    wl = workload(WORKLOAD, n_particles=a.particles)
    W, K = max(a.warmup, 0), a.steps
    lattice = lattice_for(wl, W + K)
    threads = cpu_threads()
    # each timed step: the full DF/history step plus the wake on a sample of
    # the mesh (scaled); warm-up steps build the history (untimed)
    n_obs = 16
    sec, npts = cpu_oracle_steps(wl, lattice, warm_steps=min(W, 4), sample_steps=min(K, 3),
                                 n_obs=n_obs, threads=threads)
    value = npts / sec
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": min(K, 3),
           "warmup": min(W, 4), "ms_per_step": sec * 1000, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded numpy Gaussian beam, r_gen6 transport)",
           "config": workload_config(wl.n_particles, "mixed"),
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"wake on {n_obs} of {npts} mesh points per step, scaled; "
                                      "DF/history steps in full"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    a = parse()
    if a.impl == "reference":
        reference_arm(a)
    else:
        gpu_arm(a)


if __name__ == "__main__":
    main()
