"""CSR wake on the GPU: drop-in for the wake methods of ``pyDFCSR_2D.CSR.CSR2D``.

Kept call surface (pyDFCSR_2D/CSR.py): ``initialization`` (:70-81),
``get_formation_length`` (:140-144), ``get_CSR_mesh`` (:361-394),
``calculate_2D_CSR`` / ``calculate_2D_CSR_parallel`` (:397-451),
``get_CSR_wake(s, x, debug)`` (:454-602) and
``get_CSR_integrand(s, x, t, sp, xp, ignore_vx)`` (:605-782), with the same
attributes afterwards (``dE_dct``, ``x_kick``, ``CSR_xmesh``, ``CSR_zmesh``,
``CSR_zrange``, ``CSR_xrange_transformed``, ``CSR_scaling``).

The reference builds its beam and lattice from YAML + distgen + bmadx; here
they are passed in (a :class:`~pydfcsr_gb300.beams.Beam` and a
:class:`~pydfcsr_gb300.lattice.Lattice` or lattice dict).  The whole
observation mesh is one device call; ``parallel=True`` needs no MPI split on
one GPU and runs the same path.

``precision``: ``'fp64'`` - plain FP64 drop-in (bit-compatible arithmetic
with the reference); ``'mixed'`` - FP32 bulk with the retarded geometry in
double-word FP32 (~48 bits);
``'both'`` keeps both history rings so either can be called.
"""
import ctypes
import datetime
import os

import numpy as np
import torch

from . import _lib
from .deposit import DF_tracker, raise_if_df_failed
from .lattice import Lattice
from .params import CSR_params, Integration_params
from .runtime import as_device_f64, default_workspace, ptr, require_cuda, stream_handle

__all__ = ["CSR2D", "WakeEvaluator", "PendingWake"]


def _isotime():
    """UTC time stamp for file names, local offset, ':' -> '_' (tools.py:16-22)."""
    now = datetime.datetime.now(datetime.timezone.utc).astimezone().replace(microsecond=0)
    return now.isoformat().replace(":", "_")


def wake_job(tracker, lattice, position, sigma_z, sigma_x, slope0, mean_x, formation_length,
             n_formation_length, csr_scaling, zbins, xbins, near_band=0.0):
    """Host ``dfcsr_wake_job`` for one beam."""
    require_cuda()
    tab, rho, dist = lattice.device_tables()
    j = _lib.WakeJob()
    jf = tracker.job_fields()
    if jf["ring32"] is not None and jf["cap"] * jf["nx"] * jf["nz"] * 2 >= 2 ** 32:
        raise ValueError("FP32 history ring too large for 32-bit cell offsets (>= 64 GiB)")
    j.ring64 = jf["ring64"]
    j.ring32 = jf["ring32"]
    for k in ("cap", "head", "nt", "nx", "nz"):
        setattr(j, k, int(jf[k]))
    for k in ("t_min", "x_min", "z_min", "t_delta", "x_delta", "z_delta"):
        setattr(j, k, float(jf[k]))
    j.lattice = tab.data_ptr()
    j.nsample = tab.shape[0]
    j.nelement = rho.numel()
    j.s_min = float(lattice.min_x)
    j.s_delta = float(lattice.delta_x)
    j.rho = rho.data_ptr()
    j.distance = dist.data_ptr()
    j.position = float(position)
    j.sigma_z, j.sigma_x = float(sigma_z), float(sigma_x)
    j.slope0, j.mean_x = float(slope0), float(mean_x)
    j.formation_length = float(formation_length)
    j.n_formation_length = float(n_formation_length)
    j.csr_scaling = float(csr_scaling)
    j.zbins, j.xbins = int(zbins), int(xbins)
    j.near_band = float(near_band)
    j.lattice_delta = lattice.device_deltas().data_ptr()
    tdw, ddw = lattice.device_tables_dw()
    j.lattice_dw, j.lattice_delta_dw = tdw.data_ptr(), ddw.data_ptr()
    return j


def jobs_to_device(jobs, device=None):
    """Copy a list of WakeJob structs into one device buffer."""
    raw = b"".join(bytes(j) for j in jobs)
    host = torch.frombuffer(bytearray(raw), dtype=torch.uint8)
    return host.pin_memory().to(device or torch.device("cuda", torch.cuda.current_device()),
                                non_blocking=True)


class WakeEvaluator:
    """Runs the wake kernels over device observation points."""

    def __init__(self, workspace=None):
        self.ws = workspace or default_workspace()

    def fp64(self, jobs_dev, s, x, zbins_max, job_of_point=None, stream=None):
        n = s.numel()
        dE = torch.empty(n, dtype=torch.float64, device=s.device)
        xk = torch.empty(n, dtype=torch.float64, device=s.device)
        _lib.call("dfcsr_wake_fp64", ptr(jobs_dev), ptr(job_of_point), ptr(s), ptr(x), n,
                  int(zbins_max), ptr(dE), ptr(xk), stream_handle(stream))
        return dE, xk

    def mixed_job(self, job, s, x, xbins_max, zbins_max, use_band=False, stream=None):
        """The mixed wake for one host WakeJob (passed by value: no job copy
        on the stream)."""
        n = s.numel()
        dE = torch.empty(n, dtype=torch.float64, device=s.device)
        xk = torch.empty(n, dtype=torch.float64, device=s.device)
        need = _lib.query("dfcsr_wake_workspace_bytes", int(xbins_max), int(zbins_max), n)
        buf = self.ws.get("wake", need)
        _lib.call("dfcsr_wake_mixed_job", ctypes.byref(job), ptr(s), ptr(x), n, int(xbins_max),
                  int(zbins_max), 1 if use_band else 0, ptr(dE), ptr(xk), ptr(buf), buf.numel(),
                  stream_handle(stream))
        return dE, xk

    def mixed(self, jobs_dev, s, x, xbins_max, zbins_max, job_of_point=None, use_band=False,
              stream=None):
        n = s.numel()
        dE = torch.empty(n, dtype=torch.float64, device=s.device)
        xk = torch.empty(n, dtype=torch.float64, device=s.device)
        need = _lib.query("dfcsr_wake_workspace_bytes", int(xbins_max), int(zbins_max), n)
        buf = self.ws.get("wake", need)
        _lib.call("dfcsr_wake_mixed", ptr(jobs_dev), ptr(job_of_point), ptr(s), ptr(x), n,
                  int(xbins_max), int(zbins_max), 1 if use_band else 0, ptr(dE), ptr(xk), ptr(buf),
                  buf.numel(), stream_handle(stream))
        return dE, xk


class PendingWake:
    """Mesh wake whose device->host copy is in flight: ``result()`` waits for
    it and returns (dE_dct, x_kick) as numpy arrays of ``shape``.

    ``status``: DF finalisations whose status words travel with the copy
    (``DF_tracker.take_unchecked()``); ``result()`` raises DfcsrTimeout if one
    of them reports a grid-barrier wait that gave up."""

    def __init__(self, dE, xk, shape, status=()):
        n = dE.numel()
        cur = torch.cuda.current_stream()
        self._host = torch.empty((2, n), dtype=torch.float64, pin_memory=True)
        self._host[0].copy_(dE, non_blocking=True)
        self._host[1].copy_(xk, non_blocking=True)
        self._flags = torch.zeros(len(status), dtype=torch.float64, pin_memory=True)
        for k, (sc, ev) in enumerate(status):
            cur.wait_event(ev)
            self._flags[k:k + 1].copy_(sc[7:8], non_blocking=True)
        self._event = torch.cuda.Event()
        self._event.record()
        self.shape = shape
        self.nbytes = 2 * n * 8

    def done(self):
        return self._event.query()

    def result(self):
        self._event.synchronize()
        raise_if_df_failed(self._flags.numpy())
        h = self._host.numpy()
        return h[0].reshape(self.shape).copy(), h[1].reshape(self.shape).copy()


class CSR2D:
    """The CSR wake computation of one beam, on the GPU."""

    def __init__(self, input_file=None, parallel=False, *, beam=None, lattice=None,
                 particle_deposition=None, CSR_integration=None, CSR_computation=None,
                 precision="fp64", grid_rule="reference", near_band=0.0, workspace=None):
        if input_file is not None:
            raise NotImplementedError(
                "YAML input files need bmadx/distgen beams; build a Beam and pass beam=, "
                "lattice=, particle_deposition=, CSR_integration=, CSR_computation=")
        if precision not in ("fp64", "mixed", "both"):
            raise ValueError("precision must be 'fp64', 'mixed' or 'both'")
        self.timestamp = _isotime()
        self.precision = precision
        self.near_band = float(near_band)
        self.beam = beam
        self.lattice = lattice if isinstance(lattice, Lattice) or lattice is None else Lattice(lattice)
        self.DF_tracker = DF_tracker(particle_deposition or {}, precision=precision,
                                     grid_rule=grid_rule, workspace=workspace)
        self.integration_params = Integration_params(CSR_integration or {})
        self.CSR_params = CSR_params(CSR_computation or {})
        self.formation_length = None
        self.parallel = False
        self.evaluator = WakeEvaluator(workspace)
        self._jobs_dev = None
        self._mesh = None
        self._mesh_host = None
        self._pending = None
        self._dE_dct = self._x_kick = None
        if beam is not None:
            self.initialization()

    # -------------------------------------------------------------- setup
    def initialization(self):
        """Deposit the initial beam (CSR.py:70-81)."""
        b = self.beam
        self.DF_tracker.get_DF(x=b.x, z=b.z, px=b.px, t=b.position, moments=b._moments)
        self.DF_tracker.append_DF()
        self.DF_tracker.append_interpolant(formation_length=float("inf"),
                                           n_formation_length=self.integration_params.n_formation_length)
        self.CSR_scaling = 8.98755e3 * b.charge

    def get_formation_length(self, R, sigma_z, phi=0.0, inbend=True):
        """(CSR.py:140-144)"""
        if inbend:
            self.formation_length = (24 * (R ** 2) * sigma_z) ** (1 / 3)
        else:
            self.formation_length = (3 * R ** 2 * phi ** 4) / (4 * (-6 * sigma_z + R * phi ** 3))

    def update_history(self, formation_length=None, deposited=None):
        """The per-step DF calls of CSR2D.run (CSR.py:297-307).

        ``deposited`` (extension): a :meth:`DF_tracker.deposit_DF` handle for
        this step's particles, enqueued earlier (e.g. on another stream while
        the previous step ran); the deposit is then not repeated."""
        if formation_length is not None:
            self.formation_length = formation_length
        b = self.beam
        b.sync_status()
        t = self.DF_tracker
        # the beam's moments are of these same (x, z) tensors
        t.get_DF(x=b.x, z=b.z, px=b.px, t=b.position, moments=b._moments, deposited=deposited)
        t.append_DF()
        t.append_interpolant(formation_length=self.formation_length,
                             n_formation_length=self.integration_params.n_formation_length)
        t.build_interpolant()

    # --------------------------------------------------------------- mesh
    def get_CSR_mesh(self):
        """Observation mesh in chirp-removed coordinates (CSR.py:361-394).

        Stores the mesh parameters; the host arrays (``CSR_xmesh``,
        ``CSR_zmesh``, ``CSR_zrange``, ``CSR_xrange_transformed``) are built
        with numpy on first access, and :meth:`mesh_device` builds the same
        points on the GPU (bit for bit: numpy's linspace and polyval
        arithmetic)."""
        b = self.beam
        p = b.slope
        sig_x, mean_x = b.sigma_x_transform, b.mean_x_transform
        sig_z, mean_z = b.sigma_z, b.mean_z
        xlim, zlim = self.CSR_params.xlim, self.CSR_params.zlim
        xbins, zbins = int(self.CSR_params.xbins), int(self.CSR_params.zbins)
        self._mesh = (mean_x - xlim * sig_x, mean_x + xlim * sig_x, xbins,
                      mean_z - zlim * sig_z, mean_z + zlim * sig_z, zbins,
                      float(p[0]), float(p[1]), float(b.position))
        self._mesh_host = None

    def _host_mesh(self):
        if self._mesh_host is None:
            x0, x1, xbins, z0, z1, zbins, p0, p1, _ = self._mesh
            zrange = np.linspace(z0, z1, zbins)
            xrange = np.linspace(x0, x1, xbins)
            xmesh_t, zmesh = np.meshgrid(xrange, zrange, indexing="ij")
            xmesh_t = xmesh_t.flatten()
            zmesh = zmesh.flatten()
            self._mesh_host = (xmesh_t + np.polyval(np.array([p0, p1]), zmesh), zmesh, zrange,
                               xrange)
        return self._mesh_host

    CSR_xmesh = property(lambda self: self._host_mesh()[0])
    CSR_zmesh = property(lambda self: self._host_mesh()[1])
    CSR_zrange = property(lambda self: self._host_mesh()[2])
    CSR_xrange_transformed = property(lambda self: self._host_mesh()[3])

    def mesh_device(self, stream=None):
        """(s, x) of every mesh point as float64 CUDA tensors, point k =
        i * zbins + j like ``position + CSR_zmesh`` and ``CSR_xmesh``."""
        x0, x1, xbins, z0, z1, zbins, p0, p1, _ = self._mesh
        dev = torch.device("cuda", torch.cuda.current_device())
        s = torch.empty(xbins * zbins, dtype=torch.float64, device=dev)
        x = torch.empty(xbins * zbins, dtype=torch.float64, device=dev)
        _lib.call("dfcsr_csr_mesh", x0, x1, xbins, z0, z1, zbins, p0, p1,
                  float(self.beam.position), ptr(s), ptr(x), stream_handle(stream))
        return s, x

    # --------------------------------------------------------------- wake
    def _job(self, position=None):
        b = self.beam
        ip = self.integration_params
        return wake_job(self.DF_tracker, self.lattice,
                        b.position if position is None else position, b._sigma_z, b._sigma_x,
                        b._slope[0], b._mean_x, self.formation_length, ip.n_formation_length,
                        self.CSR_scaling, ip.zbins, ip.xbins, self.near_band)

    def _wake_kind(self, precision):
        p = precision or ("fp64" if self.precision in ("fp64", "both") else "mixed")
        if p == "fp64" and self.DF_tracker.precision == "mixed":
            raise ValueError("the FP64 wake needs the FP64 history (precision 'fp64' or 'both')")
        if p == "mixed" and self.DF_tracker.precision == "fp64":
            raise ValueError("the mixed wake needs the FP32 history (precision 'mixed' or 'both')")
        return p

    def wake_device(self, s, x, precision=None, stream=None):
        """dE/dct and x-kick at device observation points (float64 CUDA
        tensors) - the hot-path call.  Nothing is read back: a caller that
        keeps the results on the device checks the DF finalisations with
        ``DF_tracker.check_status()`` when it next synchronises."""
        kind = self._wake_kind(precision)
        ip = self.integration_params
        if kind == "fp64":
            jobs = jobs_to_device([self._job()])
            self._jobs_dev = jobs
            return self.evaluator.fp64(jobs, s, x, ip.zbins, stream=stream)
        return self.evaluator.mixed_job(self._job(), s, x, ip.xbins, ip.zbins,
                                        use_band=self.near_band > 0, stream=stream)

    def calculate_2D_CSR(self, precision=None, wait=True):
        """Wake on the whole observation mesh (CSR.py:397-418): sets
        ``dE_dct`` and ``x_kick`` (numpy [xbins, zbins]).

        ``wait=False`` (extension) returns at once with a :class:`PendingWake`;
        the results are copied to pinned host memory on the stream and
        ``dE_dct`` / ``x_kick`` wait for that copy when first read.  Reading
        the results raises DfcsrTimeout if a DF finalisation of the history
        since the previous wake reported a barrier wait that gave up."""
        s, x = self.mesh_device()
        dE, xk = self.wake_device(s, x, precision)
        shape = (self.CSR_params.xbins, self.CSR_params.zbins)
        pending = PendingWake(dE, xk, shape, self.DF_tracker.take_unchecked())
        self._pending = pending
        if wait:
            self._resolve()
            return None
        return pending

    def _resolve(self):
        if self._pending is not None:
            self._dE_dct, self._x_kick = self._pending.result()
            self._pending = None

    def _get_dE(self):
        self._resolve()
        return self._dE_dct

    def _set_dE(self, v):
        self._pending = None
        self._dE_dct = v

    def _get_xk(self):
        self._resolve()
        return self._x_kick

    def _set_xk(self, v):
        self._pending = None
        self._x_kick = v

    dE_dct = property(_get_dE, _set_dE)
    x_kick = property(_get_xk, _set_xk)

    def calculate_2D_CSR_parallel(self, precision=None):
        """One GPU evaluates every observation point: same as calculate_2D_CSR
        (the reference splits the mesh over MPI ranks, CSR.py:420-451)."""
        self.calculate_2D_CSR(precision)

    def _regions(self, s, x):
        """Integration regions of get_CSR_wake (CSR.py:478-553) on the host."""
        b = self.beam
        t = b.position
        sigma_z, sigma_x, tt = b._sigma_z, b._sigma_x, b._slope[0]
        x0 = (s - t) * b._slope[0]
        xmean = b._mean_x
        zb, xb = self.integration_params.zbins, self.integration_params.xbins
        nLf = self.integration_params.n_formation_length * self.formation_length
        if np.abs(tt) <= 1:
            s2, s3, s4 = s - 500 * sigma_z, s - 20 * sigma_z, s + 5 * sigma_z
            s1 = np.max((0, s2 - nLf))
            return False, [(2 * xb, zb, x0 - 20 * sigma_x, x0 + 20 * sigma_x, s1, s2),
                           (xb, zb, x0 - 10 * sigma_x, x0 + 10 * sigma_x, s2, s3),
                           (xb, zb, x0 - 10 * sigma_x, x0 + 10 * sigma_x, s3, s4)]
        if tt > 0:
            tan_alpha = -2 * tt / (1 - tt ** 2)
            d = (10 * sigma_x + xmean - x) / tan_alpha
            s4 = s + 3 * sigma_z
            s3 = np.max((0, s - d))
            s2 = s3 - 200 * sigma_z
            x1l, x1r = x + 0.1 * sigma_x, x + 10 * sigma_x
            x2l, x2r = x - 3 * sigma_x, x + 0.1 * sigma_x
        else:
            tan_alpha = 2 * tt / (1 - tt ** 2)
            d = -(xmean - x - 10 * sigma_x) / tan_alpha
            s4 = s + 3 * sigma_z
            s3 = np.max((0, s - d))
            s2 = s3 - 200 * sigma_z
            x1l, x1r = x - 10 * sigma_x, x - 1 * sigma_x
            x2l, x2r = x - 1 * sigma_x, x + 3 * sigma_x
        s1 = np.max((0, s2 - nLf))
        return True, [(2 * xb, zb, x0 - 20 * sigma_x, x0 + 20 * sigma_x, s1, s2),
                      (xb, zb, x0 - 5 * sigma_x, x0 + 5 * sigma_x, s2, s3),
                      (xb, zb, x1l, x1r, s3, s4),
                      (xb, zb, x2l, x2r, s3, s4)]

    def get_CSR_wake(self, s, x, debug=False):
        """Wake at one observation point (CSR.py:454-602).  ``debug=True``
        returns the reference's tuple of region grids and integrand arrays."""
        if not debug:
            dE, xk = self.wake_device(as_device_f64([s]), as_device_f64([x]))
            dE, xk = dE.cpu().numpy(), xk.cpu().numpy()
            return float(dE[0]), float(xk[0])
        chirp, regs = self._regions(s, x)
        xps, sps, ints = [], [], []
        for (nxp, nsp, xl, xr, sl, sr) in regs:
            xp = np.linspace(xl, xr, nxp)
            sp = np.linspace(sl, sr, nsp)
            xpm, spm = np.meshgrid(xp, sp, indexing="ij")
            Iz, Ix = self.get_CSR_integrand(s=s, x=x, t=self.beam.position, sp=spm, xp=xpm)
            xps.append(xp); sps.append(sp); ints += [Iz, Ix]
        if chirp:
            # xp1, xp2, xp3, xp4, sp1, sp2, sp3, then the integrands per region
            return (xps[2], xps[3], xps[1], xps[0], sps[0], sps[1], sps[2], *ints)
        return (xps[0], xps[1], sps[0], sps[1], sps[2], *ints)

    def get_CSR_integrand(self, s, x, t, sp, xp, ignore_vx=False):
        """FP64 integrands at the mesh (sp, xp) (CSR.py:605-782)."""
        spd = as_device_f64(np.asarray(sp)).reshape(-1)
        xpd = as_device_f64(np.asarray(xp)).reshape(-1)
        jobs = jobs_to_device([self._job(position=t)])
        m = spd.numel()
        Iz = torch.empty(m, dtype=torch.float64, device=spd.device)
        Ix = torch.empty(m, dtype=torch.float64, device=spd.device)
        _lib.call("dfcsr_wake_integrand", ptr(jobs), float(s), float(x), ptr(spd), ptr(xpd), m,
                  1 if ignore_vx else 0, ptr(Iz), ptr(Ix), stream_handle())
        shape = np.shape(xp)
        return Iz.cpu().numpy().reshape(shape), Ix.cpu().numpy().reshape(shape)

    # --------------------------------------------------------- checkpoint
    def state_dict(self):
        """(extension) The wake state between steps as host data: the DF
        tracker's history (:meth:`DF_tracker.state_dict`), the formation
        length, the CSR scaling and the output time stamp.  The beam's
        particles are the caller's to save, as in the reference."""
        return {"DF_tracker": self.DF_tracker.state_dict(),
                "formation_length": self.formation_length,
                "CSR_scaling": getattr(self, "CSR_scaling", None),
                "timestamp": self.timestamp}

    def load_state_dict(self, state):
        """(extension) Resume from :meth:`state_dict` (same precision)."""
        self.DF_tracker.load_state_dict(state["DF_tracker"])
        self.formation_length = state["formation_length"]
        if state["CSR_scaling"] is not None:
            self.CSR_scaling = state["CSR_scaling"]
        self.timestamp = state["timestamp"]
        self._pending = None
        self._jobs_dev = None

    # ------------------------------------------------------------- output
    @property
    def prefix(self):
        """Output file prefix ``<write_name>-<timestamp>`` (CSR.py:41)."""
        return f"{self.CSR_params.write_name}-{self.timestamp}"

    def write_wakes(self):
        """Append this step's wakes to ``<workdir>/<prefix>-wakes.h5``
        (CSR.py:799-835), the layout ``postprocessor.py`` reads: group
        ``step_<step>`` (attrs step, position, mean_gamma, beam_energy,
        element, charge) with subgroups ``longitudinal`` (``x_grids``,
        ``z_grids``, ``dE_dct``) and ``transverse`` (``x_grids``,
        ``z_grids``, ``xkicks``), each with attr unit = 'MeV/m'; grids shaped
        like the wake, [xbins, zbins].  Step 1 replaces an existing file.
        Needs h5py; returns the file name."""
        try:
            import h5py
        except ImportError as e:
            raise ImportError("write_wakes writes HDF5 and needs h5py") from e
        b = self.beam
        filename = os.path.join(self.CSR_params.workdir, f"{self.prefix}-wakes.h5")
        if b.step == 1 and os.path.isfile(filename):
            os.remove(filename)
        dE, xk = self.dE_dct, self.x_kick
        x_grids = self.CSR_xmesh.reshape(dE.shape)
        z_grids = self.CSR_zmesh.reshape(dE.shape)
        element = getattr(self.lattice, "current_element", None)
        with h5py.File(filename, "a") as hf:
            g = hf.create_group(f"step_{b.step}")
            g.attrs["step"] = b.step
            g.attrs["position"] = b.position
            g.attrs["mean_gamma"] = b.init_gamma
            g.attrs["beam_energy"] = b.init_energy
            g.attrs["element"] = "" if element is None else element
            g.attrs["charge"] = b.charge
            for name, wake, key in (("longitudinal", dE, "dE_dct"), ("transverse", xk, "xkicks")):
                sub = g.create_group(name)
                sub.attrs["unit"] = "MeV/m"
                sub.create_dataset("x_grids", data=x_grids)
                sub.create_dataset("z_grids", data=z_grids)
                sub.create_dataset(key, data=wake)
        return filename
