"""Host-side coefficient tables for the device stencils (FP64, numpy).

These are the small per-grid constants the kernels apply; computing them on
the host keeps the kernels' arithmetic identical to the library routines the
reference calls:

* Savitzky-Golay (``scipy.signal.savgol_filter``, mode 'interp', deriv 0):
  smoothing coefficients of the centred least-squares polynomial fit and the
  two edge maps (values of the polynomial fitted to the first / last window).
* ``numpy.gradient(f, grid)`` (edge_order 1): the non-uniform three-point
  weights per interior index, the end spacings, and whether numpy takes its
  uniform-spacing branch (all spacings exactly equal).
* ``scipy.interpolate.RegularGridInterpolator`` (linear, bounds_error False)
  on a tensor-product target: interval index, normalised distance and the
  out-of-bounds flag per target coordinate.
"""
from functools import lru_cache

import numpy as np


@lru_cache(maxsize=64)
def savgol_tables(window, order):
    """(coeff[w], lo[m, w], hi[m, w]) for window w (odd), polynomial order."""
    if window % 2 != 1 or window < 1:
        raise ValueError("window_length must be a positive odd integer")
    if order >= window:
        raise ValueError("polyorder must be less than window_length.")
    m = window // 2
    k = np.arange(window, dtype=float) - m
    A = np.vstack([k ** p for p in range(order + 1)])
    e0 = np.zeros(order + 1)
    e0[0] = 1.0
    coeff = A.T @ np.linalg.solve(A @ A.T, e0)
    pos = np.arange(window, dtype=float)
    V = np.vstack([pos ** p for p in range(order + 1)]).T
    P = np.linalg.solve(V.T @ V, V.T)
    lo = np.vstack([np.arange(m, dtype=float) ** p for p in range(order + 1)]).T @ P
    hi = np.vstack([np.arange(window - m, window, dtype=float) ** p
                    for p in range(order + 1)]).T @ P
    return (np.ascontiguousarray(coeff), np.ascontiguousarray(lo.reshape(m, window)),
            np.ascontiguousarray(hi.reshape(m, window)))


def gradient_table(grid):
    """Coefficients of numpy.gradient along a coordinate array.

    Returns (g[4, n], uniform, dx): rows 0..2 hold a, b, c for interior index
    i (out = a f[i-1] + b f[i] + c f[i+1]); row 3 holds the first and last
    spacing at [3, 0] and [3, 1].
    """
    grid = np.asarray(grid, dtype=float)
    n = grid.size
    d = np.diff(grid)
    g = np.zeros((4, n))
    uniform = bool(np.all(d == d[0]))
    if n > 2:
        d1, d2 = d[:-1], d[1:]
        g[0, 1:-1] = -(d2) / (d1 * (d1 + d2))
        g[1, 1:-1] = (d2 - d1) / (d1 * d2)
        g[2, 1:-1] = d1 / (d2 * (d1 + d2))
    if uniform:
        g[3, 0] = g[3, 1] = d[0]
    else:
        g[3, 0], g[3, 1] = d[0], d[-1]
    return g, uniform, float(d[0])


def rgi_axis(src_grid, targets):
    """Interval index, normalised distance and out-of-bounds flag per target."""
    src = np.asarray(src_grid, dtype=float)
    t = np.asarray(targets, dtype=float)
    i = np.clip(np.searchsorted(src, t, side="right") - 1, 0, src.size - 2)
    w = (t - src[i]) / (src[i + 1] - src[i])
    oob = (t < src[0]) | (t > src[-1])
    return i.astype(np.int32), w, oob.astype(np.uint8)
