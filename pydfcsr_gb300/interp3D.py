"""Trilinear interpolation on a (t, x, z) grid: drop-in for
pyDFCSR_2D/interp3D.py:18-66, evaluated on the GPU.

``int()`` truncation semantics are kept: a query whose index coordinate u is
in (-1, 0) extrapolates linearly from the first cell, u <= -1 or u >= n gives
0, and the last cell is clamped (i1 = i0 when i0 = n - 1).
"""
import numpy as np
import torch

from . import _lib
from .runtime import as_device_f64, ptr, require_cuda, stream_handle

__all__ = ["interpolate3D", "TrilinearInterpolator"]


def interpolate3D(xval, yval, zval, data, min_x, min_y, min_z, delta_x, delta_y, delta_z):
    """Values of ``data[x, y, z]`` at the query points (numpy in -> numpy out,
    torch in -> CUDA tensor out)."""
    require_cuda()
    as_numpy = not isinstance(xval, torch.Tensor)
    qx = as_device_f64(xval).reshape(-1)
    qy = as_device_f64(yval).reshape(-1)
    qz = as_device_f64(zval).reshape(-1)
    d = as_device_f64(data)
    if d.dim() != 3:
        raise ValueError("data must be a 3D array")
    out = torch.empty_like(qx)
    _lib.call("dfcsr_interp3d", ptr(qx), ptr(qy), ptr(qz), qx.numel(), ptr(d), d.shape[0],
              d.shape[1], d.shape[2], float(min_x), float(min_y), float(min_z), float(delta_x),
              float(delta_y), float(delta_z), ptr(out), stream_handle())
    return out.cpu().numpy() if as_numpy else out


class TrilinearInterpolator:
    """Wrapper holding the grid (pyDFCSR_2D/interp3D.py:144-158)."""

    def __init__(self, data, x, y, z):
        self.data = as_device_f64(data)
        self.min_x, self.max_x = x[0], x[-1]
        self.min_y, self.max_y = y[0], y[-1]
        self.min_z, self.max_z = z[0], z[-1]
        self.delta_x = (self.max_x - self.min_x) / (np.shape(x)[0] - 1)
        self.delta_y = (self.max_y - self.min_y) / (np.shape(y)[0] - 1)
        self.delta_z = (self.max_z - self.min_z) / (np.shape(z)[0] - 1)

    def interp(self, xval, yval, zval):
        return interpolate3D(xval, yval, zval, self.data, self.min_x, self.min_y, self.min_z,
                             self.delta_x, self.delta_y, self.delta_z)
