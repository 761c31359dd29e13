"""GPU particle beam: the part of ``pyDFCSR_2D.beams.Beam`` the wake path reads.

The reference's Beam wraps bmadx particles (tracking is third-party and out of
scope).  Here the 6D coordinates (x, px, y, py, z, pz) live in one float64
CUDA tensor [6, N]; the statistics the wake needs (beams.py:137-215: means,
standard deviations, the polyfit slope of x on z and the chirp-removed
x_transform) come from one deterministic device moments call per update.
Linear transport by a 6x6 matrix (``track``, one ``dfcsr_transport6`` launch)
stands in for bmadx on linear lattices; ``apply_wakes`` is beams.py:108-131 as
one ``dfcsr_apply_wakes`` call.
"""
import ctypes

import numpy as np
import scipy.constants
import torch

from . import _lib
from .deposit import beam_moments
from .runtime import as_device_f64, default_workspace, ptr, require_cuda, stream_handle

__all__ = ["Beam"]

# electron rest energy in eV, from scipy.constants (physical_constants.py:11)
MC2 = scipy.constants.value("electron mass energy equivalent in MeV") * 1e6


class PendingStatus:
    """Beam moments in flight (see :meth:`Beam.status_async`): the device
    array, its pinned host copy and the event after the copy."""
    __slots__ = ("device", "host", "event")

    def __init__(self, device, host, event):
        self.device, self.host, self.event = device, host, event

    def result(self):
        """The 16 moments as a numpy array (waits for the copy)."""
        self.event.synchronize()
        return self.host.numpy().copy()


class Beam:
    def __init__(self, coords, charge=1e-9, energy=1e9, position=0.0, workspace=None,
                 adopt=False):
        require_cuda()
        self.ws = workspace
        self._charge = float(charge)
        self._init_energy = float(energy)
        self.position = float(position)
        self.step = 0
        self.set_coords(coords, adopt)

    @classmethod
    def from_particle(cls, particle, charge=1e-9, **kw):
        """A beam from a bmadx-style ``Particle`` (fields x..pz, s, p0c; numpy
        or torch arrays), as the reference's Beam holds one (beams.py:33):
        energy = p0c, position = s."""
        coords = [getattr(particle, k) for k in ("x", "px", "y", "py", "z", "pz")]
        if isinstance(coords[0], torch.Tensor):
            coords = torch.stack([c.to(torch.float64) for c in coords])
        else:
            coords = np.stack([np.asarray(c, dtype=np.float64) for c in coords])
        return cls(coords, charge=charge, energy=float(particle.p0c), position=float(particle.s),
                   **kw)

    def to_particle(self):
        """The particles as a bmadx-style ``Particle`` of host numpy arrays
        (s = position, p0c = the initial energy, mc2 = the electron's), for
        :func:`pydfcsr_gb300.interfaces.bmadx_particles_to_openpmd`."""
        from .interfaces import M_ELECTRON, Particle
        h = self.particle.cpu().numpy()
        return Particle(*[h[k].copy() for k in range(6)], s=self.position,
                        p0c=self._init_energy, mc2=M_ELECTRON)

    def set_coords(self, coords, adopt=False):
        """Replace the particle coordinates (array-like [6, N]).

        A CUDA float64 tensor passed in is used as is.  Unless ``adopt`` is
        true it is copied before the first in-place update (track,
        apply_wakes), so the caller's tensor keeps its values."""
        c = as_device_f64(coords)
        if c.dim() != 2 or c.shape[0] != 6:
            raise ValueError("coords must have shape (6, N)")
        self.particle = c
        shared = (isinstance(coords, torch.Tensor) and coords.is_cuda
                  and c.untyped_storage().data_ptr() == coords.untyped_storage().data_ptr())
        self._owned = adopt or not shared
        self.update_status()

    def _own(self):
        if not self._owned:
            self.particle = self.particle.clone()
            self._owned = True

    def status_async(self, stream=None):
        """(extension) Enqueue the moments of the current particles and their
        copy to pinned host memory on ``stream`` (default: the current one);
        returns a :class:`PendingStatus`.  The beam's statistics change only
        when the handle is applied (:meth:`apply_status`), so the moments of
        later particle sets can be in flight while these are in use."""
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            m = beam_moments(self.particle[0], self.particle[4], ws=self.ws)
            host = torch.empty(m.numel(), dtype=torch.float64, pin_memory=True)
            host.copy_(m, non_blocking=True)
            ev = torch.cuda.Event()
            ev.record(s)
        return PendingStatus(m, host, ev)

    def apply_status(self, pending):
        """Set the statistics from a :meth:`status_async` handle (waits for
        its copy)."""
        st = pending.result()
        self._moments_dev = pending.device
        self._moments = st
        self._mean_x, self._mean_z = float(st[1]), float(st[2])
        self._sigma_x, self._sigma_z = float(st[3]), float(st[4])
        self._slope = np.array([st[5], st[6]])

    def update_status(self, stream=None, wait=True):
        """Beam statistics from one device moments call; waits for it (and
        for whatever precedes it on ``stream``, default the current one).

        ``wait=False`` only enqueues the moments and their copy to pinned host
        memory; :meth:`sync_status` (or the next update) completes them."""
        self._pending_status = self.status_async(stream)
        if wait:
            self.sync_status()

    def sync_status(self):
        """Wait for the moments enqueued by ``update_status(wait=False)`` and
        set the statistics from them."""
        pending = getattr(self, "_pending_status", None)
        if pending is None:
            return
        self._pending_status = None
        self.apply_status(pending)

    def transport(self, R):
        """coords <- R coords in place (6x6 FP64 matrix, e.g. from r_gen6)."""
        self._own()
        Rh = np.ascontiguousarray(np.asarray(R, dtype=np.float64))
        if Rh.shape != (6, 6):
            raise ValueError("R must be 6x6")
        n = self.particle.shape[1]
        _lib.call("dfcsr_transport6", Rh.ctypes.data_as(ctypes.c_void_p), ptr(self.particle), n,
                  self.particle.stride(0), stream_handle())

    def track(self, R, step_size, update_step=True, wait=True):
        """Apply a 6x6 transfer matrix and advance (beams.py:101-106 with a
        linear matrix in place of bmadx's track_element).  ``wait=False``
        (extension) enqueues the statistics without waiting for them (see
        :meth:`update_status`); :attr:`moments_device` is then usable at
        once, e.g. to enqueue the step's deposit before the host has them."""
        self.transport(R)
        self.position += step_size
        if update_step:
            self.step += 1
        self.update_status(wait=wait)

    @property
    def moments_device(self):
        """(extension) The latest beam moments (dfcsr_beam_moments) as a CUDA
        float64 tensor, including those still being copied to the host."""
        pending = getattr(self, "_pending_status", None)
        return pending.device if pending is not None else self._moments_dev

    def apply_wakes(self, dE_dct, x_kick, xrange, zrange, step_size, transverse_on, update=True):
        """Kick pz (and px when ``transverse_on``) by the wake interpolated at
        (x_transform, z) (beams.py:108-131); updates the statistics
        (``update=False``, an extension: skip that when the caller tracks the
        beam next, which updates them anyway)."""
        self._own()
        dE = as_device_f64(dE_dct)
        xk = as_device_f64(x_kick) if transverse_on else None
        xr, zr = as_device_f64(xrange), as_device_f64(zrange)
        nx, nz = xr.numel(), zr.numel()
        if tuple(dE.shape) != (nx, nz) or (xk is not None and tuple(xk.shape) != (nx, nz)):
            raise ValueError("wake tables must have shape (len(xrange), len(zrange))")
        ws = (self.ws or default_workspace()).get(
            "apply_wakes", _lib.query("dfcsr_apply_wakes_workspace_bytes", nx, nz))
        n = self.particle.shape[1]
        _lib.call("dfcsr_apply_wakes", ptr(self.particle), n, self.particle.stride(0), ptr(dE),
                  ptr(xk), ptr(xr), ptr(zr), nx, nz, float(self._slope[0]), float(self._slope[1]),
                  float(step_size), self._init_energy, 1 if transverse_on else 0, ptr(ws),
                  ws.numel(), stream_handle())
        if update:
            self.update_status()

    @property
    def n_particle(self):
        return self.particle.shape[1]

    x = property(lambda self: self.particle[0])
    px = property(lambda self: self.particle[1])
    y = property(lambda self: self.particle[2])
    py = property(lambda self: self.particle[3])
    z = property(lambda self: self.particle[4])
    pz = property(lambda self: self.particle[5])
    def _stat(name):
        def get(self):
            self.sync_status()
            return getattr(self, name)
        return property(get)

    mean_x = _stat("_mean_x")
    mean_z = _stat("_mean_z")
    sigma_x = _stat("_sigma_x")
    sigma_z = _stat("_sigma_z")
    slope = property(lambda self: (self.sync_status(), self._slope.copy())[1])
    charge = property(lambda self: self._charge)
    init_energy = property(lambda self: self._init_energy)
    init_gamma = property(lambda self: self._init_energy / MC2)

    @property
    def x_transform(self):
        """x with the linear x-z chirp removed (device tensor)."""
        return self.x - (float(self._slope[0]) * self.z + float(self._slope[1]))

    @property
    def sigma_x_transform(self):
        self.sync_status()
        return float(self._moments[10])

    @property
    def mean_x_transform(self):
        self.sync_status()
        return float(self._moments[9])
