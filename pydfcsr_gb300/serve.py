"""Continuous-batching wake server: many beams, one GPU.

Requests (beams with their own lattice, particle count, deposit grid and
observation mesh) arrive over time.  Each admitted request keeps its history
ring on the device and advances step by step (get_DF + history update on its
own CUDA stream, so the deposits of different beams overlap).  At every tick
the observation points of all active requests are packed into ONE batched
mixed-precision wake launch (one ``dfcsr_wake_job`` per request, a job index
per point), replayed from a CUDA graph captured per shape bucket.  Requests
join and leave between ticks: new ones are admitted as soon as device memory
(estimated footprint against an HBM budget) and a slot are free.

Each point's wake is computed by one CTA in a fixed order, so a request's
result does not depend on which other requests share its launches
(``tests/test_gpu_serving.py`` checks alone == in the mix, bit for bit).

The scheduling core (:class:`Admission`, :class:`Scheduler`) is plain Python
and is tested on the CPU; :class:`WakeServer` drives the GPU.
"""
from dataclasses import dataclass, field
import math
import time

import numpy as np

__all__ = ["RequestSpec", "Admission", "Scheduler", "WakeServer", "footprint_bytes"]


@dataclass
class RequestSpec:
    """One wake-evaluation request: a beam through one dipole."""
    id: int
    arrival_s: float
    rho: float
    angle: float
    n: int
    sigma_z: float
    grid: int
    mesh: int
    seed: int
    steps: int = 8
    sigma_x: float = 20e-6
    integration: dict = field(default_factory=lambda: {"n_formation_length": 1.5,
                                                       "zbins": 100, "xbins": 100})
    upper_limit: int = 600

    @classmethod
    def from_dict(cls, d):
        keys = {k: d[k] for k in ("id", "arrival_s", "rho", "angle", "n", "sigma_z", "grid",
                                  "mesh", "seed") if k in d}
        if "steps" in d:
            keys["steps"] = d["steps"]
        return cls(**keys)


def footprint_bytes(spec, precision="mixed"):
    """Upper estimate of a request's device memory (bytes).

    particles (6 x N doubles), deposit scratch (sort keys/values, per-cell
    partials), DF fields of every step kept for re-interpolation (5 x grid^2
    doubles each), the history ring (up to upper_limit^2 cells per slot, 32 B
    a cell in FP32 or 40 B in FP64, steps + 4 slots), DF scratch, and the
    mesh / result arrays.
    """
    n, g, u = spec.n, spec.grid, spec.upper_limit
    particles = 6 * n * 8
    deposit = 16 * n + (g + 1) ** 2 * (64 + 8) + 256 * ((n + 4095) // 4096) * 4 + (1 << 20)
    df_log = (spec.steps + 1) * 5 * g * g * 8
    ring = (spec.steps + 4) * u * u * (32 if precision == "mixed" else 40)
    df_scratch = 6 * g * g * 8 + (1 << 20)
    mesh = spec.mesh * spec.mesh * 8 * 6
    return int(particles + deposit + df_log + ring + df_scratch + mesh)


class Admission:
    """HBM budget accounting (host side)."""

    def __init__(self, budget_bytes, max_active):
        self.budget = int(budget_bytes)
        self.max_active = int(max_active)
        self.used = 0
        self.active = 0

    def can_ever_fit(self, need):
        return need <= self.budget

    def try_admit(self, need):
        if self.active >= self.max_active or self.used + need > self.budget:
            return False
        self.used += need
        self.active += 1
        return True

    def release(self, need):
        self.used -= need
        self.active -= 1
        assert self.used >= 0 and self.active >= 0


class Scheduler:
    """Arrival queue, admission and the per-tick set of active requests.

    ``clock`` returns the current time in seconds since the start of the
    stream.  Requests are admitted in arrival order (no overtaking: a large
    request at the head waits for memory rather than being skipped).
    """

    def __init__(self, specs, admission, clock, precision="mixed"):
        self.pending = sorted(specs, key=lambda s: (s.arrival_s, s.id))
        self.admission = admission
        self.clock = clock
        self.precision = precision
        self.active = []
        self.refused = []
        self.cancelled = []
        self.failed = []           # (spec, reason)
        self.done = []

    def cancel(self, req_id):
        """Drop a request that has not been admitted yet."""
        for i, s in enumerate(self.pending):
            if s.id == req_id:
                self.cancelled.append(self.pending.pop(i))
                return True
        return False

    def admit(self):
        """Admit arrived requests while they fit; returns the new ones."""
        now = self.clock()
        new = []
        while self.pending and self.pending[0].arrival_s <= now:
            spec = self.pending[0]
            need = footprint_bytes(spec, self.precision)
            if not self.admission.can_ever_fit(need):
                self.refused.append(self.pending.pop(0))
                continue
            if not self.admission.try_admit(need):
                break
            self.pending.pop(0)
            new.append(spec)
        self.active.extend(new)
        return new

    def finish(self, spec):
        self.active.remove(spec)
        self.admission.release(footprint_bytes(spec, self.precision))
        self.done.append(spec)

    def fail(self, spec, reason):
        """End an admitted request whose calls raised: its memory goes back
        to the budget and the queue moves on."""
        self.active.remove(spec)
        self.admission.release(footprint_bytes(spec, self.precision))
        self.failed.append((spec, reason))

    def idle_until(self):
        """Arrival time of the next pending request (None if none)."""
        return self.pending[0].arrival_s if self.pending else None

    def finished(self):
        return not self.pending and not self.active


# ------------------------------------------------------------------ GPU side
def _request_errors():
    """Errors that end one request and leave the CUDA context and the other
    requests usable: a refused argument, a workspace or allocation failure,
    a bounded device wait that gave up, a kernel's error status.  A CUDA
    error (DfcsrCudaError) is not among them: it can poison the context,
    so it ends the whole run."""
    import torch
    from . import _lib
    return (_lib.DfcsrBadArgument, _lib.DfcsrOutOfMemory, _lib.DfcsrTimeout,
            _lib.DfcsrKernelError, _lib.DfcsrAdmissionRefused, torch.cuda.OutOfMemoryError)


class _Live:
    """Device state of one admitted request: its beam, DF history ring,
    workspace and CUDA stream."""

    def __init__(self, spec, admitted_at, precision="mixed", pool=None):
        import torch
        from .beams import Beam
        from .CSR import CSR2D
        from .synthetic import StepPlan, dipole_lattice, gaussian_beam_device

        self.spec = spec
        self.admitted_at = admitted_at
        self.pool = pool if pool is not None else _ResourcePool()
        self.stream, self.ws = self.pool.take()
        L = spec.rho * spec.angle
        self.lattice = dipole_lattice(spec.rho, L, L / spec.steps,
                                      tail_drift=max(0.02, 20 * spec.sigma_z))
        self.plan = StepPlan(self.lattice, n_steps=spec.steps)
        dep = {"xbins": spec.grid, "zbins": spec.grid, "xlim": 5, "zlim": 5, "filter_order": 2,
               "filter_window": 9, "velocity_threhold": 1000, "upper_limit": spec.upper_limit}
        mesh = {"xbins": spec.mesh, "zbins": spec.mesh, "xlim": 3, "zlim": 3}
        with torch.cuda.stream(self.stream):
            coords = gaussian_beam_device(spec.n, spec.sigma_x, spec.sigma_z, 1e-4, 5e-6, 0.0,
                                          spec.seed)
            self.beam = Beam(coords, charge=1e-9, energy=1e9, workspace=self.ws, adopt=True)
            self.csr = CSR2D(beam=self.beam, lattice=self.lattice, particle_deposition=dep,
                             CSR_integration=spec.integration, CSR_computation=mesh,
                             precision=precision, grid_rule="configured", workspace=self.ws)
            self.csr.lattice.device_tables()
        self.k = 0
        self.results = []          # (step, dE_dct [mesh, mesh], x_kick [mesh, mesh])
        self.points = 0
        self.finished_at = None
        self.done_event = None
        self.failed = False
        # latency breakdown (seconds): set-up at admission (beam, first DF
        # step), per-tick host time of its DF steps, its share of the shared
        # wake launches (their whole duration), graph captures in those
        # ticks, ticks taken part in
        self.setup_s = 0.0
        self.df_s = 0.0
        self.wake_s = 0.0
        self.capture_s = 0.0
        self.ticks = 0

    def advance_launch(self):
        """Transport to the next step and enqueue its beam moments on this
        request's stream (no host wait)."""
        import torch
        with torch.cuda.stream(self.stream):
            k = self.k + 1
            self.beam.transport(self.plan.matrix(k))
            self.beam.update_status(wait=False)
            self.beam.position = float(self.plan.positions[k])
            self.beam.step = k
            self.k = k

    def advance_finish(self):
        """Deposit + DF + history update of the step launched by
        advance_launch (the host waits for this request's moments only)."""
        import torch
        with torch.cuda.stream(self.stream):
            self.beam.sync_status()
            self.csr.update_history(self.plan.formation_length(self.k, self.beam.sigma_z))
            self.csr.get_CSR_mesh()
            self.done_event = torch.cuda.Event()
            self.done_event.record(self.stream)

    def check(self):
        """Raise DfcsrTimeout if a DF finalisation of this request reported
        a grid-barrier wait that gave up (waits for this request's DF work)."""
        import torch
        with torch.cuda.stream(self.stream):
            self.csr.DF_tracker.check_status()

    def wants_wake(self):
        return self.k >= 2        # the interpolant needs two history slices

    def last_step(self):
        return self.k >= self.spec.steps

    def release(self):
        """Drop the device state (the stream and workspace go back to the
        pool once this request's work on the stream is done); results stay."""
        if self.stream is not None:
            self.stream.synchronize()
            self.pool.give(self.stream, self.ws)
        self.beam = self.csr = self.ws = self.stream = None


class _ResourcePool:
    """CUDA streams and workspaces reused from one request to the next
    (creating them per request costs host time at every admission).  A
    workspace keeps the buffers of its largest request: the pool holds at
    most ``limit`` of them."""

    def __init__(self, limit=64):
        self.free = []
        self.limit = int(limit)

    def take(self):
        import torch
        from .runtime import Workspace
        if self.free:
            return self.free.pop()
        return torch.cuda.Stream(), Workspace()

    def give(self, stream, ws):
        if len(self.free) < self.limit:
            self.free.append((stream, ws))


class _BatchedWake:
    """Static device buffers for the packed observation points of a tick and
    one CUDA graph per chunk count.

    A tick's points are padded up to a multiple of ``chunk`` (the padding
    repeats the first point; its result is dropped).  The wake over K chunks
    is captured once as a graph on the static buffers and replayed for every
    later tick with the same K, so the number of graphs is bounded by
    ``max_points / chunk`` and a replay costs one launch from the host.
    """

    def __init__(self, max_points, max_jobs, xbins, zbins, precision, chunk, use_graphs):
        import ctypes
        import torch
        from . import _lib
        self.chunk = int(chunk)
        self.cap = int(math.ceil(max_points / self.chunk) * self.chunk)
        self.max_jobs = int(max_jobs)
        self.xbins, self.zbins = int(xbins), int(zbins)
        self.precision = precision
        self.use_graphs = use_graphs
        dev = torch.device("cuda", torch.cuda.current_device())
        f64 = dict(dtype=torch.float64, device=dev)
        self.s = torch.zeros(self.cap, **f64)
        self.x = torch.zeros(self.cap, **f64)
        self.dE = torch.zeros(self.cap, **f64)
        self.xk = torch.zeros(self.cap, **f64)
        self.jop = torch.zeros(self.cap, dtype=torch.int32, device=dev)
        self.job_bytes = ctypes.sizeof(_lib.WakeJob)
        self.jobs = torch.zeros(self.max_jobs * self.job_bytes, dtype=torch.uint8, device=dev)
        self.host = torch.empty(self.cap * 20 + self.max_jobs * self.job_bytes,
                                dtype=torch.uint8).pin_memory()
        self.out_host = torch.empty((2, self.cap), dtype=torch.float64).pin_memory()
        if precision == "mixed":
            need = _lib.query("dfcsr_wake_workspace_bytes", self.xbins, self.zbins, self.cap)
            self.ws = torch.empty(need, dtype=torch.uint8, device=dev)
        else:
            self.ws = None
        self.graphs = {}
        self.warm = False
        self.replays = 0
        self.capture_s = 0.0       # host time of graph captures during the stream
        self.last_capture_s = 0.0

    def _launch(self, n, stream):
        import ctypes
        from . import _lib
        from .runtime import ptr
        h = ctypes.c_void_p(stream.cuda_stream)
        if self.precision == "mixed":
            _lib.call("dfcsr_wake_mixed", ptr(self.jobs), ptr(self.jop), ptr(self.s), ptr(self.x), n,
                      self.xbins, self.zbins, 0, ptr(self.dE), ptr(self.xk), ptr(self.ws),
                      self.ws.numel(), h)
        else:
            _lib.call("dfcsr_wake_fp64", ptr(self.jobs), ptr(self.jop), ptr(self.s), ptr(self.x), n,
                      self.zbins, ptr(self.dE), ptr(self.xk), h)

    def _capture(self, k, stream):
        import torch
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            self._launch(k * self.chunk, stream)
        self.graphs[k] = g
        return g

    def precapture(self, stream):
        """Capture the launch of every chunk count up to the buffers'
        capacity (after one eager launch: the library's one-time set-up),
        so that no capture happens while requests wait."""
        if not self.use_graphs or not self.warm:
            return 0
        for k in range(1, self.cap // self.chunk + 1):
            if k not in self.graphs:
                self._capture(k, stream)
        return len(self.graphs)

    def run(self, jobs_raw, meshes, stream):
        """One tick: the job structs and job index per point go up from
        pinned memory, every request's mesh is built on the device straight
        into the static point buffers (``meshes``: one ``CSR2D._mesh``
        parameter tuple per job), the padding repeats the first point, the
        wake runs (graph replay) and (dE, x_kick) of the real points come
        back.  Returns host arrays."""
        import ctypes
        import torch
        from . import _lib
        from .runtime import ptr
        sizes = [m[2] * m[5] for m in meshes]
        n = int(sum(sizes))
        if n > self.cap or len(jobs_raw) > self.max_jobs * self.job_bytes:
            raise RuntimeError("tick exceeds the static wake buffers")
        padded = int(math.ceil(n / self.chunk) * self.chunk)
        hb = self.host.numpy()
        vj = hb[:padded * 4].view(np.int32)
        off = 0
        for ji, m in enumerate(sizes):
            vj[off:off + m] = ji
            off += m
        vj[n:] = 0
        o = padded * 4
        hb[o:o + len(jobs_raw)] = np.frombuffer(jobs_raw, dtype=np.uint8)
        h = ctypes.c_void_p(stream.cuda_stream)
        with torch.cuda.stream(stream):
            ht = self.host
            self.jop[:padded].copy_(ht[:padded * 4].view(torch.int32), non_blocking=True)
            self.jobs[:len(jobs_raw)].copy_(ht[o:o + len(jobs_raw)], non_blocking=True)
            off = 0
            for m, size in zip(meshes, sizes):
                x0, x1, xb, z0, z1, zb, p0, p1, pos = m
                _lib.call("dfcsr_csr_mesh", x0, x1, xb, z0, z1, zb, p0, p1, pos,
                          ctypes.c_void_p(self.s.data_ptr() + 8 * off),
                          ctypes.c_void_p(self.x.data_ptr() + 8 * off), h)
                off += size
            if padded > n:
                self.s[n:padded].copy_(self.s[:1].expand(padded - n))
                self.x[n:padded].copy_(self.x[:1].expand(padded - n))
            k = padded // self.chunk
            self.last_capture_s = 0.0
            if not self.use_graphs or not self.warm:
                # the first call runs eagerly: one-time library set-up happens
                # outside any capture
                self._launch(padded, stream)
                self.warm = True
            else:
                g = self.graphs.get(k)
                if g is None:
                    t0 = time.perf_counter()
                    g = self._capture(k, stream)
                    self.last_capture_s = time.perf_counter() - t0
                    self.capture_s += self.last_capture_s
                g.replay()
                self.replays += 1
            self.out_host[0, :n].copy_(self.dE[:n], non_blocking=True)
            self.out_host[1, :n].copy_(self.xk[:n], non_blocking=True)
        stream.synchronize()
        out = self.out_host.numpy()
        return out[0, :n].copy(), out[1, :n].copy()


class WakeServer:
    """Runs a request stream through the GPU with continuous batching.

    ``precision``: 'mixed' (FP32 bulk + FP64 geometry, the served form) or
    'fp64' (the plain drop-in kernels on the same stream, for comparison).
    """

    def __init__(self, specs, precision="mixed", budget_bytes=None, max_active=32,
                 use_graphs=True, chunk=2048, precapture=False):
        import torch
        from . import _lib
        from .runtime import require_cuda
        require_cuda()
        if precision not in ("mixed", "fp64"):
            raise ValueError("precision must be 'mixed' or 'fp64'")
        self.precision = precision
        specs = [s if isinstance(s, RequestSpec) else RequestSpec.from_dict(s) for s in specs]
        if budget_bytes is None:
            free, _ = torch.cuda.mem_get_info()
            budget_bytes = int(0.6 * free)
        self.admission = Admission(budget_bytes, max_active)
        self.t0 = None
        self.sched = Scheduler(specs, self.admission, self._clock, precision)
        mesh_max = max((sp.mesh for sp in specs), default=1)
        xb = max((int(sp.integration["xbins"]) for sp in specs), default=1)
        zb = max((int(sp.integration["zbins"]) for sp in specs), default=1)
        self.wake = _BatchedWake(max_active * mesh_max * mesh_max, max_active, xb, zb, precision,
                                 chunk, use_graphs)
        self.stream = torch.cuda.Stream()
        self.pool = _ResourcePool(limit=max_active + 4)
        self.live = {}
        self.ticks = 0
        self.launch_points = []
        self.wake_s = 0.0
        self.precapture_s = 0.0
        _lib.timing_enable(False)    # no event records inside captured graphs
        if precapture and use_graphs:
            self._precapture(specs)

    def _precapture(self, specs):
        """Warm the batched launch with a small request of the stream's
        integration bins, run alone before the stream starts, then capture
        the graphs of all chunk counts."""
        t0 = time.perf_counter()
        base = specs[0] if specs else RequestSpec(0, 0.0, 5.0, 0.1, 20_000, 30e-6, 64, 8, 1)
        warm = RequestSpec(**{**base.__dict__, "id": -1, "arrival_s": 0.0, "n": 20_000,
                              "grid": 64, "mesh": 8, "steps": 2, "seed": 12345})
        lv = _Live(warm, 0.0, self.precision, self.pool)
        lv.advance_launch()
        lv.advance_finish()
        lv.advance_launch()
        lv.advance_finish()
        self._wake_tick([lv], _request_errors())
        lv.release()
        self.wake.precapture(self.stream)
        self.stream.synchronize()
        self.wake_s = 0.0
        self.launch_points = []
        self.precapture_s = time.perf_counter() - t0

    def _clock(self):
        return time.perf_counter() - self.t0

    def _wake_tick(self, reqs, errs):
        """One batched wake launch for every request in `reqs`; a request
        whose DF step failed gets no result and fails alone."""
        from .CSR import wake_job
        if not reqs:
            return
        jobs, meshes = [], []
        for lv in reqs:
            c = lv.csr
            b = c.beam
            ip = c.integration_params
            jobs.append(wake_job(c.DF_tracker, c.lattice, b.position, b._sigma_z, b._sigma_x,
                                 b._slope[0], b._mean_x, c.formation_length, ip.n_formation_length,
                                 c.CSR_scaling, ip.zbins, ip.xbins))
            meshes.append(c._mesh)
        for lv in reqs:
            self.stream.wait_event(lv.done_event)
        t = time.perf_counter()
        dE, xk = self.wake.run(b"".join(bytes(j) for j in jobs), meshes, self.stream)
        dt = time.perf_counter() - t
        self.wake_s += dt
        self.launch_points.append(dE.size)
        for lv in reqs:
            lv.wake_s += dt
            lv.capture_s += self.wake.last_capture_s
        off = 0
        for lv in reqs:
            shape = (lv.csr.CSR_params.xbins, lv.csr.CSR_params.zbins)
            m = shape[0] * shape[1]
            try:
                lv.check()              # a failed DF step: this request's points are invalid
            except errs as e:
                self._fail(lv.spec, e, lv)
                off += m
                continue
            lv.results.append((lv.k, dE[off:off + m].reshape(shape), xk[off:off + m].reshape(shape)))
            lv.points += m
            off += m

    def _fail(self, spec, err, lv=None):
        if lv is not None:
            lv.failed = True
            lv.release()
        self.sched.fail(spec, f"{type(err).__name__}: {err}")

    def _each(self, lives, method, errs):
        """Call ``method`` of every live request; a request that raises one
        of ``errs`` fails alone.  Returns the requests still live."""
        for lv in lives:
            try:
                getattr(lv, method)()
            except errs as e:
                self._fail(lv.spec, e, lv)
        return [lv for lv in lives if not lv.failed]

    def run(self):
        """Serve the whole stream; returns a summary dict.  A request whose
        calls raise a library error (bad argument, out of memory, timeout,
        kernel error status) is marked failed and its memory released; the
        others are served on (``failed()``)."""
        import torch
        errs = _request_errors()
        self.t0 = time.perf_counter()
        sched = self.sched
        while not sched.finished():
            for spec in sched.admit():
                t = time.perf_counter()
                try:
                    self.live[spec.id] = _Live(spec, self._clock(), self.precision, self.pool)
                    self.live[spec.id].setup_s = time.perf_counter() - t
                except errs as e:
                    self._fail(spec, e)
            if not sched.active:
                nxt = sched.idle_until()
                if nxt is not None:
                    time.sleep(max(0.0, nxt - self._clock()))
                continue
            lives = [self.live[s.id] for s in sched.active]
            # every request's transport + moments first, then each request's
            # DF step: the moments of all beams run while the host waits for
            # the first one
            t = time.perf_counter()
            lives = self._each(lives, "advance_launch", errs)
            lives = self._each(lives, "advance_finish", errs)
            dt = time.perf_counter() - t
            for lv in lives:
                lv.df_s += dt
                lv.ticks += 1
            tick = [lv for lv in lives if lv.wants_wake()]
            try:
                self._wake_tick(tick, errs)
            except errs as e:                   # the shared launch: all its requests
                for lv in tick:
                    if not lv.failed:
                        self._fail(lv.spec, e, lv)
            lives = [lv for lv in lives if not lv.failed]
            lives = self._each(lives, "check", errs)   # the DF steps of requests without a wake
            self.ticks += 1
            for lv in lives:
                if lv.last_step():
                    lv.finished_at = self._clock()
                    lv.release()
                    sched.finish(lv.spec)
        torch.cuda.synchronize()
        return self.summary(self._clock())

    def latency_breakdown(self):
        """Per finished request: latency (arrival to last result) and its
        parts - queue (arrival to admission), set-up (beam and first DF step
        at admission), DF steps (host time of the ticks it took part in),
        wake (duration of the shared launches it took part in), graph
        captures within those, other (the remainder: ticks spent on other
        requests' set-up and on the host loop)."""
        out = []
        for lv in self.live.values():
            if lv.finished_at is None:
                continue
            lat = lv.finished_at - lv.spec.arrival_s
            queue = lv.admitted_at - lv.spec.arrival_s
            other = lat - queue - lv.setup_s - lv.df_s - lv.wake_s
            out.append({"id": lv.spec.id, "latency_s": lat, "queue_s": queue, "setup_s": lv.setup_s,
                        "df_s": lv.df_s, "wake_s": lv.wake_s, "capture_s": lv.capture_s,
                        "other_s": other, "ticks": lv.ticks, "points": lv.points,
                        "n": lv.spec.n, "grid": lv.spec.grid, "mesh": lv.spec.mesh})
        return out

    def summary(self, wall):
        br = self.latency_breakdown()
        lat = np.array([b["latency_s"] for b in br])
        pts = sum(lv.points for lv in self.live.values())
        out = {"precision": self.precision, "requests": len(self.live),
               "refused": len(self.sched.refused), "failed": len(self.sched.failed),
               "ticks": self.ticks,
               "wall_s": wall, "wake_points": int(pts),
               "wake_points_per_s": pts / wall if wall > 0 else 0.0,
               "wake_s": self.wake_s,
               "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else None,
               "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else None,
               "mean_points_per_launch": float(np.mean(self.launch_points)) if self.launch_points else 0.0,
               "graphs": len(self.wake.graphs), "graph_replays": self.wake.replays,
               "graph_capture_s_in_stream": self.wake.capture_s,
               "precapture_s": self.precapture_s}
        if lat.size:
            # the parts of the latency at the median and over the slowest 1 %
            # (mean of each part over those requests)
            order = np.argsort(lat)
            tail = [br[i] for i in order[max(0, int(np.floor(0.99 * lat.size)) - 1):]]
            mid = [br[i] for i in order[max(0, lat.size // 2 - 1):lat.size // 2 + 1]]
            keys = ("latency_s", "queue_s", "setup_s", "df_s", "wake_s", "capture_s", "other_s")
            out["breakdown_p50"] = {k: float(np.mean([b[k] for b in mid])) for k in keys}
            out["breakdown_p99"] = {k: float(np.mean([b[k] for b in tail])) for k in keys}
            out["breakdown_p99"]["requests"] = [{k: b[k] for k in ("id", "n", "grid", "mesh", "ticks")}
                                                for b in tail]
        return out

    def result(self, req_id):
        """[(step, dE_dct, x_kick)] of a served request."""
        return self.live[req_id].results

    def failed(self):
        """{request id: reason} of the requests that failed."""
        return {spec.id: reason for spec, reason in self.sched.failed}
