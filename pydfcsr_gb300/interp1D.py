"""Linear interpolation of a uniformly sampled table: drop-in for
pyDFCSR_2D/interp1D.py:13-36, evaluated on the GPU (same truncation rule as
interpolate3D)."""
import numpy as np
import torch

from . import _lib
from .runtime import as_device_f64, ptr, require_cuda, stream_handle

__all__ = ["interpolate1D", "LinearInterpolator"]


def interpolate1D(xval, data, min_x, delta_x):
    require_cuda()
    as_numpy = not isinstance(xval, torch.Tensor)
    q = as_device_f64(xval).reshape(-1)
    tab = as_device_f64(data).reshape(-1)
    out = torch.empty_like(q)
    _lib.call("dfcsr_interp1d", ptr(q), q.numel(), ptr(tab), tab.numel(), float(min_x),
              float(delta_x), ptr(out), stream_handle())
    return out.cpu().numpy() if as_numpy else out


class LinearInterpolator:
    """Wrapper holding the table (pyDFCSR_2D/interp1D.py:39-48)."""

    def __init__(self, data, x):
        self.data = as_device_f64(data)
        self.min_x, self.max_x = x[0], x[-1]
        self.delta_x = (self.max_x - self.min_x) / (np.shape(x)[0] - 1)

    def interp(self, xval):
        return interpolate1D(xval, self.data, self.min_x, self.delta_x)
