"""GPU particle beam: the part of ``pyDFCSR_2D.beams.Beam`` the wake path reads.

The reference's Beam wraps bmadx particles (tracking is third-party and out of
scope).  Here the 6D coordinates (x, px, y, py, z, pz) live in one float64
CUDA tensor [6, N]; the statistics the wake needs (beams.py:137-215: means,
standard deviations, the polyfit slope of x on z and the chirp-removed
x_transform) come from one deterministic device moments call per update.
Linear transport by a 6x6 matrix (``track``) stands in for bmadx on linear
lattices.
"""
import numpy as np
import torch

from .deposit import beam_moments
from .runtime import as_device_f64, require_cuda

__all__ = ["Beam"]


class Beam:
    def __init__(self, coords, charge=1e-9, energy=1e9, position=0.0):
        require_cuda()
        self._charge = float(charge)
        self._init_energy = float(energy)
        self.position = float(position)
        self.step = 0
        self.set_coords(coords)

    def set_coords(self, coords):
        """Replace the particle coordinates (array-like [6, N])."""
        c = as_device_f64(coords)
        if c.dim() != 2 or c.shape[0] != 6:
            raise ValueError("coords must have shape (6, N)")
        self.particle = c
        self.update_status()

    def update_status(self):
        m = beam_moments(self.particle[0], self.particle[4])
        self._moments_dev = m
        st = m.cpu().numpy()
        self._moments = st
        self._mean_x, self._mean_z = float(st[1]), float(st[2])
        self._sigma_x, self._sigma_z = float(st[3]), float(st[4])
        self._slope = np.array([st[5], st[6]])

    def track(self, R, step_size, update_step=True):
        """Apply a 6x6 transfer matrix (e.g. from r_gen6) and advance."""
        Rt = torch.as_tensor(np.asarray(R, dtype=np.float64), device=self.particle.device)
        self.particle = (Rt @ self.particle).contiguous()
        self.position += step_size
        if update_step:
            self.step += 1
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
    mean_x = property(lambda self: self._mean_x)
    mean_z = property(lambda self: self._mean_z)
    sigma_x = property(lambda self: self._sigma_x)
    sigma_z = property(lambda self: self._sigma_z)
    slope = property(lambda self: self._slope.copy())
    charge = property(lambda self: self._charge)
    init_energy = property(lambda self: self._init_energy)

    @property
    def x_transform(self):
        """x with the linear x-z chirp removed (device tensor)."""
        return self.x - (float(self._slope[0]) * self.z + float(self._slope[1]))

    @property
    def sigma_x_transform(self):
        return float(self._moments[10])

    @property
    def mean_x_transform(self):
        return float(self._moments[9])
