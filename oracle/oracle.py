"""CPU oracle for the pyDFCSR_2D per-step wake path - TEST INFRASTRUCTURE ONLY.

This module is the checker, never the product.  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The GPU package ``pydfcsr_gb300`` never imports it and has no CPU
fallback.

It restates the reference's algorithm on the host, function by function:

=========================  ==========================================
oracle function            reference (pyDFCSR_2D/...)
=========================  ==========================================
histogram_cic_2d           deposit.py:43-87      (C: csr_oracle.c)
interpolate3D              interp3D.py:18-66     (C)
interpolate1D              interp1D.py:13-36     (C)
DFTracker.get_DF           deposit.py:145-245
DFTracker.append_DF        deposit.py:247-256
DFTracker.pop_left_DF      deposit.py:258-280
DFTracker.DF_interp        deposit.py:296-309
DFTracker.append_interp... deposit.py:312-392
DFTracker.build_interp...  deposit.py:395-426
reference_trajectory       lattice.py:4-110, 136-150
csr_mesh                   CSR.py:361-394
WakeOracle.wake / points   CSR.py:397-418, 454-782  (C)
apply_wakes                beams.py:108-131
=========================  ==========================================

Third-party arithmetic the reference calls, restated from the published
algorithms (versions in this image: scipy 1.18.1, numpy 2.5.4; the reference
pins neither):

* ``scipy.signal.savgol_filter(x, w, p, axis)`` with the default
  ``mode='interp'``: interior points are the least-squares polynomial
  smoothing coefficients applied as a correlation; the first and last
  ``w // 2`` points are the values of the degree-``p`` least-squares
  polynomial fitted to the first / last ``w`` samples.
* ``scipy.interpolate.RegularGridInterpolator(method='linear',
  bounds_error=False, fill_value=f)``: interval l with g[l] <= v < g[l+1]
  (last interval for the right end point), normalised distance
  (v - g[l]) / (g[l+1] - g[l]), bilinear weights; any coordinate outside
  [g[0], g[-1]] gives ``f``.
* ``numpy.gradient(f, xg, zg)`` (edge_order 1): second-order non-uniform
  central differences inside, first-order one-sided differences at the ends;
  spacings that are all exactly equal use the uniform formula.
* ``numpy.trapz`` / ``trapezoid``: sum of d_i * (y_{i+1} + y_i) / 2.

Parity pin: the fixtures in ``tests/golden`` were produced by running the
reference itself; ``tests/test_oracle_golden.py`` checks this module against
them.
"""
import ctypes
import math
import os
import subprocess
from collections import deque

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(HERE, "csr_oracle.c")

__all__ = ["build", "histogram_cic_2d", "interpolate3D", "interpolate1D",
           "savgol_filter", "gradient2d", "DFTracker", "reference_trajectory",
           "csr_mesh", "beam_stats", "WakeOracle", "apply_wakes"]


def build(force=False):
    """Compile the C restatement with gcc (no FMA contraction, no fast-math)."""
    os.makedirs(_BUILD, exist_ok=True)
    if not force and os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(_SRC):
        return _SO
    tmp = _SO + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                           "-fno-fast-math", "-o", tmp, _SRC, "-lpthread", "-lm"])
    os.replace(tmp, _SO)
    return _SO


_lib = None


class _Ctx(ctypes.Structure):
    _fields_ = [
        ("density", ctypes.c_void_p), ("density_x", ctypes.c_void_p),
        ("density_z", ctypes.c_void_p), ("vx", ctypes.c_void_p), ("vx_x", ctypes.c_void_p),
        ("nt", ctypes.c_int), ("nx", ctypes.c_int), ("nz", ctypes.c_int),
        ("t_min", ctypes.c_double), ("x_min", ctypes.c_double), ("z_min", ctypes.c_double),
        ("t_delta", ctypes.c_double), ("x_delta", ctypes.c_double), ("z_delta", ctypes.c_double),
        ("X0", ctypes.c_void_p), ("Y0", ctypes.c_void_p), ("nX", ctypes.c_void_p),
        ("nY", ctypes.c_void_p), ("tX", ctypes.c_void_p), ("tY", ctypes.c_void_p),
        ("nsample", ctypes.c_int), ("s_min", ctypes.c_double), ("s_delta", ctypes.c_double),
        ("rho", ctypes.c_void_p), ("distance", ctypes.c_void_p), ("nelement", ctypes.c_int),
        ("position", ctypes.c_double), ("sigma_z", ctypes.c_double),
        ("sigma_x", ctypes.c_double), ("slope0", ctypes.c_double), ("mean_x", ctypes.c_double),
        ("formation_length", ctypes.c_double), ("n_formation_length", ctypes.c_double),
        ("csr_scaling", ctypes.c_double), ("zbins", ctypes.c_int), ("xbins", ctypes.c_int),
    ]


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        d = ctypes.c_double
        p = ctypes.c_void_p
        _lib.oracle_cic2d.argtypes = [p, p, p, ctypes.c_long, ctypes.c_int, d, d,
                                      ctypes.c_int, d, d, p]
        _lib.oracle_interp3d.argtypes = [p, p, p, ctypes.c_long, p, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int, d, d, d, d, d, d, p]
        _lib.oracle_interp1d.argtypes = [p, ctypes.c_long, p, ctypes.c_int, d, d, p]
        _lib.oracle_wake_point.argtypes = [ctypes.POINTER(_Ctx), d, d, p, p, p]
        _lib.oracle_wake_point.restype = ctypes.c_long
        _lib.oracle_wake_points.argtypes = [ctypes.POINTER(_Ctx), ctypes.c_long, p, p, p, p,
                                            ctypes.c_int]
        _lib.oracle_ctx_size.restype = ctypes.c_long
        assert _lib.oracle_ctx_size() == ctypes.sizeof(_Ctx), "oracle ctx layout mismatch"
    return _lib


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


# --------------------------------------------------------------- numba loops
def histogram_cic_2d(q1, q2, w, nbins_1, bins_start_1, bins_end_1,
                     nbins_2, bins_start_2, bins_end_2):
    """Restates ``histogram_cic_2d`` (pyDFCSR_2D/deposit.py:43-87)."""
    q1, q2, w = _f64(q1).ravel(), _f64(q2).ravel(), _f64(w).ravel()
    out = np.empty((int(nbins_1), int(nbins_2)))
    lib().oracle_cic2d(_ptr(q1), _ptr(q2), _ptr(w), q1.size, int(nbins_1),
                       float(bins_start_1), float(bins_end_1), int(nbins_2),
                       float(bins_start_2), float(bins_end_2), _ptr(out))
    return out


def interpolate3D(xval, yval, zval, data, min_x, min_y, min_z, delta_x, delta_y, delta_z):
    """Restates ``interpolate3D`` (pyDFCSR_2D/interp3D.py:18-66)."""
    xv, yv, zv = _f64(xval).ravel(), _f64(yval).ravel(), _f64(zval).ravel()
    data = _f64(data)
    out = np.empty(xv.size)
    lib().oracle_interp3d(_ptr(xv), _ptr(yv), _ptr(zv), xv.size, _ptr(data), data.shape[0],
                          data.shape[1], data.shape[2], float(min_x), float(min_y),
                          float(min_z), float(delta_x), float(delta_y), float(delta_z),
                          _ptr(out))
    return out


def interpolate1D(xval, data, min_x, delta_x):
    """Restates ``interpolate1D`` (pyDFCSR_2D/interp1D.py:13-36)."""
    xv, data = _f64(xval).ravel(), _f64(data).ravel()
    out = np.empty(xv.size)
    lib().oracle_interp1d(_ptr(xv), xv.size, _ptr(data), data.size, float(min_x),
                          float(delta_x), _ptr(out))
    return out


# ------------------------------------------------------------ scipy / numpy
def savgol_coeffs(window, order):
    """Least-squares smoothing coefficients (deriv 0), centre at w // 2."""
    m = window // 2
    k = np.arange(window, dtype=float) - m
    A = np.vstack([k ** p for p in range(order + 1)])           # (order+1, w)
    gram = A @ A.T
    e0 = np.zeros(order + 1)
    e0[0] = 1.0
    return A.T @ np.linalg.solve(gram, e0)


def savgol_edges(window, order):
    """Linear maps giving the 'interp' edge values from the first / last window."""
    m = window // 2
    k = np.arange(window, dtype=float)
    V = np.vstack([k ** p for p in range(order + 1)]).T          # (w, order+1)
    P = np.linalg.solve(V.T @ V, V.T)                            # (order+1, w)
    lo = np.vstack([np.arange(m, dtype=float) ** p for p in range(order + 1)]).T
    hi = np.vstack([np.arange(window - m, window, dtype=float) ** p
                    for p in range(order + 1)]).T
    return lo @ P, hi @ P


def savgol_filter(x, window, order, axis):
    """``scipy.signal.savgol_filter(x, window, order, axis=axis)`` (mode 'interp')."""
    x = np.moveaxis(_f64(x), axis, 0)
    n = x.shape[0]
    if window > n:
        raise ValueError("If mode is 'interp', window_length must be less than or equal "
                         "to the size of x.")
    if order >= window:
        raise ValueError("polyorder must be less than window_length.")
    c = savgol_coeffs(window, order)
    m = window // 2
    y = np.zeros_like(x)
    for i in range(m, n - m):
        acc = x[i - m] * c[0]
        for k in range(1, window):
            acc = acc + x[i - m + k] * c[k]
        y[i] = acc
    lo, hi = savgol_edges(window, order)
    for i in range(m):
        acc = x[0] * lo[i, 0]
        for k in range(1, window):
            acc = acc + x[k] * lo[i, k]
        y[i] = acc
        acc = x[n - window] * hi[i, 0]
        for k in range(1, window):
            acc = acc + x[n - window + k] * hi[i, k]
        y[n - m + i] = acc
    return np.moveaxis(y, 0, axis)


def _gradient_axis(f, g):
    f = np.moveaxis(f, 0, 0)
    dxs = np.diff(g)
    out = np.empty_like(f)
    if np.all(dxs == dxs[0]):
        out[1:-1] = (f[2:] - f[:-2]) / (2.0 * dxs[0])
        out[0] = (f[1] - f[0]) / dxs[0]
        out[-1] = (f[-1] - f[-2]) / dxs[0]
        return out
    d1, d2 = dxs[:-1], dxs[1:]
    a = -(d2) / (d1 * (d1 + d2))
    b = (d2 - d1) / (d1 * d2)
    c = d1 / (d2 * (d1 + d2))
    shp = (-1,) + (1,) * (f.ndim - 1)
    out[1:-1] = a.reshape(shp) * f[:-2] + b.reshape(shp) * f[1:-1] + c.reshape(shp) * f[2:]
    out[0] = (f[1] - f[0]) / dxs[0]
    out[-1] = (f[-1] - f[-2]) / dxs[-1]
    return out


def gradient2d(f, xg, zg):
    """``numpy.gradient(f, xg, zg)`` for a 2D array (edge_order 1)."""
    fx = _gradient_axis(f, xg)
    fz = np.moveaxis(_gradient_axis(np.moveaxis(f, 1, 0), zg), 0, 1)
    return fx, fz


def trapz(y, x, axis=-1):
    y = np.moveaxis(np.asarray(y, dtype=float), axis, 0)
    d = np.diff(x).reshape((-1,) + (1,) * (y.ndim - 1))
    terms = d * (y[1:] + y[:-1]) / 2.0
    return terms.sum(0)


def rgi_linear_2d(xg, zg, values, X, Z, fill_value):
    """Bilinear ``RegularGridInterpolator`` with ``bounds_error=False``."""
    X = np.asarray(X, float)
    Z = np.asarray(Z, float)
    i = np.clip(np.searchsorted(xg, X, side="right") - 1, 0, xg.size - 2)
    j = np.clip(np.searchsorted(zg, Z, side="right") - 1, 0, zg.size - 2)
    y0 = (X - xg[i]) / (xg[i + 1] - xg[i])
    y1 = (Z - zg[j]) / (zg[j + 1] - zg[j])
    out = 0.0
    out = out + values[i, j] * (1 - y0) * (1 - y1)
    out = out + values[i, j + 1] * (1 - y0) * y1
    out = out + values[i + 1, j] * y0 * (1 - y1)
    out = out + values[i + 1, j + 1] * y0 * y1
    oob = (X < xg[0]) | (X > xg[-1]) | (Z < zg[0]) | (Z > zg[-1])
    out = np.where(oob, fill_value, out)
    return out


def apply_wakes(coords, dE_dct, x_kick, xrange, zrange, step_size, init_energy,
                transverse_on, slope):
    """Beam.apply_wakes (beams.py:108-131) on a (6, N) array; returns the
    kicked copy.  ``slope`` is the polyfit of x on z that the reference's
    x_transform property computes (beams.py:201-211)."""
    c = np.array(coords, dtype=float, copy=True)
    xt = c[0] - np.polyval(slope, c[4])
    dE_E1 = step_size * np.asarray(dE_dct, float) * 1e6 / init_energy
    c[5] = c[5] + rgi_linear_2d(np.asarray(xrange, float), np.asarray(zrange, float), dE_E1,
                                xt, c[4], 0.0)
    if transverse_on:
        dxp = step_size * np.asarray(x_kick, float) * 1e6 / init_energy
        c[1] = c[1] + rgi_linear_2d(np.asarray(xrange, float), np.asarray(zrange, float), dxp,
                                    xt, c[4], 0.0)
    return c


# ------------------------------------------------------------------ DF_tracker
class DFTracker:
    """Restates ``DF_tracker`` (pyDFCSR_2D/deposit.py:90-426)."""

    def __init__(self, input_dic=None, grid_rule="reference"):
        p = dict(xbins=100, zbins=100, xlim=5, zlim=5, filter_order=0, filter_window=0,
                 velocity_threhold=5, upper_limit=None)
        p.update(input_dic or {})
        for k, v in p.items():
            setattr(self, k, v)
        self.grid_rule = grid_rule
        self.start_time = 0.0
        self.t = 0.0
        self.DF_log, self.time_log = deque(), deque()
        self.sigma_x_log, self.sigma_z_log = deque(), deque()
        self.sigma_x_interp = self.sigma_z_interp = None
        self.time_interp = deque()
        self.density_interp, self.density_x_interp = deque(), deque()
        self.density_z_interp, self.vx_interp, self.vx_x_interp = deque(), deque(), deque()
        self.interp_start = 0
        self.x_grid_interp = self.z_grid_interp = None

    def _sg2(self, a, w):
        return savgol_filter(savgol_filter(a, w, self.filter_order, 0), w, self.filter_order, 1)

    def get_DF(self, x, z, px, t):
        x, z, px = _f64(x), _f64(z), _f64(px)
        sigma_x, sigma_z = np.std(x), np.std(z)
        self.sigma_x, self.sigma_z = sigma_x, sigma_z
        self.xmean, self.zmean = np.mean(x), np.mean(z)
        sel = x[np.abs(z) < 0.1 * sigma_z]
        with np.errstate(all="ignore"):
            slice_sig = np.std(sel) if sel.size else np.nan
            frac = sigma_x / slice_sig
        if frac > 5 or self.grid_rule == "configured":
            xb, zb, win = self.xbins, self.zbins, self.filter_window
        else:
            xb, zb, win = 100, 100, 5
        x0, x1 = self.xmean - self.xlim * sigma_x, self.xmean + self.xlim * sigma_x
        z0, z1 = self.zmean - self.zlim * sigma_z, self.zmean + self.zlim * sigma_z
        xg, zg = np.linspace(x0, x1, xb), np.linspace(z0, z1, zb)
        density = histogram_cic_2d(x, z, np.ones(x.shape), xb, x0, x1, zb, z0, z1)
        vx = histogram_cic_2d(x, z, px, xb, x0, x1, zb, z0, z1)
        thr = np.max(density) / self.velocity_threhold
        m = density > thr
        vx[m] /= density[m]
        density = self._sg2(density, win)
        vx = self._sg2(vx, win)
        dsum = trapz(trapz(density, xg, axis=0), zg)
        density /= dsum
        vx[density <= thr] = 0
        dx_, dz_ = gradient2d(density, xg, zg)
        vxx, _ = gradient2d(vx, xg, zg)
        dx_, dz_, vxx = self._sg2(dx_, win), self._sg2(dz_, win), self._sg2(vxx, win)
        thr2 = np.max(density) / self.velocity_threhold * 8
        with np.errstate(all="ignore"):
            sel = vxx[density > thr2]
            fill = np.mean(sel) if sel.size else np.nan
        vxx[density < thr2] = fill
        self.x_grids, self.z_grids = xg, zg
        self.density, self.vx = density, vx
        self.density_x, self.density_z, self.vx_x = dx_, dz_, vxx
        self.t = t
        self.bins = (xb, zb, win)

    def append_DF(self):
        self.DF_log.append((self.x_grids, self.z_grids, self.density, self.vx,
                            self.density_x, self.density_z, self.vx_x))
        self.time_log.append(self.t)
        self.sigma_x_log.append(self.sigma_x)
        self.sigma_z_log.append(self.sigma_z)
        self.end_time = self.t

    def pop_left_DF(self, new_start_time):
        while self.start_time < new_start_time:
            self.DF_log.popleft(); self.time_log.popleft()
            self.sigma_x_log.popleft(); self.sigma_z_log.popleft()
            self.start_time = self.time_log[0]
        while self.interp_start < new_start_time:
            for d in (self.density_interp, self.density_x_interp, self.density_z_interp,
                      self.vx_interp, self.vx_x_interp, self.time_interp):
                d.popleft()
            self.interp_start = self.time_interp[0]

    def DF_interp(self, DF, x_grids=None, z_grids=None, fill_value=0.0):
        xg = self.x_grids if x_grids is None else x_grids
        zg = self.z_grids if z_grids is None else z_grids
        X, Z = np.meshgrid(self.x_grid_interp, self.z_grid_interp, indexing="ij")
        return rgi_linear_2d(xg, zg, DF, X, Z, fill_value)

    def append_interpolant(self, formation_length, n_formation_length):
        start_point = np.amax((0, self.end_time - n_formation_length * formation_length))
        self.pop_left_DF(start_point)
        if (self.sigma_x_interp and self.sigma_z_interp
                and 2 > self.sigma_x / self.sigma_x_interp > 1 / 2
                and 2 > self.sigma_z / self.sigma_z_interp > 1 / 2):
            self.time_interp.append(self.t)
            self.density_interp.append(self.DF_interp(self.density))
            self.density_x_interp.append(self.DF_interp(self.density_x))
            self.density_z_interp.append(self.DF_interp(self.density_z))
            self.vx_interp.append(self.DF_interp(self.vx))
            self.vx_x_interp.append(self.DF_interp(self.vx_x, fill_value=np.mean(self.vx_x)))
            self.reinterpolated = False
            return
        t_x = np.max(self.sigma_x_log) / np.min(self.sigma_x_log)
        t_z = np.max(self.sigma_z_log) / np.min(self.sigma_z_log)
        xb, zb = int(500 * t_x), int(500 * t_z)
        if isinstance(self.upper_limit, int):
            xb, zb = min(xb, self.upper_limit), min(zb, self.upper_limit)
        self.sigma_x_interp = np.max(self.sigma_x_log)
        self.sigma_z_interp = np.max(self.sigma_z_log)
        self.x_grid_interp = np.linspace(self.xmean - 5 * self.sigma_x_interp,
                                         self.xmean + 5 * self.sigma_x_interp, xb)
        self.z_grid_interp = np.linspace(self.zmean - 5 * self.sigma_z_interp,
                                         self.zmean + 5 * self.sigma_z_interp, zb)
        self.density_interp, self.density_x_interp = deque(), deque()
        self.density_z_interp, self.vx_interp, self.vx_x_interp = deque(), deque(), deque()
        self.time_interp = self.time_log.copy()
        for xg, zg, den, vx, den_x, den_z, vxx in self.DF_log:
            self.density_interp.append(self.DF_interp(den, xg, zg))
            self.density_x_interp.append(self.DF_interp(den_x, xg, zg))
            self.density_z_interp.append(self.DF_interp(den_z, xg, zg))
            self.vx_interp.append(self.DF_interp(vx, xg, zg))
            self.vx_x_interp.append(self.DF_interp(vxx, xg, zg, fill_value=np.mean(vxx)))
        self.reinterpolated = True

    def build_interpolant(self):
        self.min_x, self.max_x = self.time_interp[0], self.time_interp[-1]
        self.min_y, self.max_y = self.x_grid_interp[0], self.x_grid_interp[-1]
        self.min_z, self.max_z = self.z_grid_interp[0], self.z_grid_interp[-1]
        self.delta_x = (self.max_x - self.min_x) / (len(self.time_interp) - 1)
        self.delta_y = (self.max_y - self.min_y) / (self.x_grid_interp.shape[0] - 1)
        self.delta_z = (self.max_z - self.min_z) / (self.z_grid_interp.shape[0] - 1)
        self.data_density_interp = np.array(self.density_interp)
        self.data_density_z_interp = np.array(self.density_z_interp)
        self.data_density_x_interp = np.array(self.density_x_interp)
        self.data_vx_interp = np.array(self.vx_interp)
        self.data_vx_x_interp = np.array(self.vx_x_interp)


# -------------------------------------------------------------------- lattice
def reference_trajectory(lattice, Nsample=2000):
    """Restates ``get_referece_traj`` (pyDFCSR_2D/lattice.py:4-110).

    Returns s, rho (per element angle/L), distance (cumulative element ends),
    nsep, coords (x, y), n_vec = (sin th, -cos th), tau_vec = (cos th, sin th).
    """
    names = list(lattice.keys())[1:]
    ne = len(names)
    distance, rho, nsep = np.zeros(ne), np.zeros(ne), np.zeros(ne)
    for i, nm in enumerate(names):
        e = lattice[nm]
        nsep[i] = e["nsep"]
        if e["type"] == "dipole":
            rho[i] = e["angle"] / e["L"]
        distance[i] = e["L"] if i == 0 else e["L"] + distance[i - 1]
    s = np.linspace(0, distance[-1], Nsample)
    coords, tau, nv = np.zeros((Nsample, 2)), np.zeros((Nsample, 2)), np.zeros((Nsample, 2))
    theta = 0
    tau[0] = (np.cos(theta), np.sin(theta))
    nv[0] = (np.sin(theta), -1 * np.cos(theta))
    e_idx = 0
    for k in range(1, Nsample):
        if s[k] > distance[e_idx]:
            e_idx += 1
        ds = s[k] - s[k - 1]
        e = lattice[names[e_idx]]
        if e["type"] == "dipole":
            phi = ds / e["L"] * e["angle"]
            r = e["L"] / e["angle"]
            cx = coords[k - 1, 0] - r * np.sin(theta)
            cy = coords[k - 1, 1] + r * np.cos(theta)
            coords[k, 0] = cx + r * np.sin(phi + theta)
            coords[k, 1] = cy - r * np.cos(phi + theta)
        else:
            phi = 0
            coords[k, 0] = coords[k - 1, 0] + ds * np.cos(theta)
            coords[k, 1] = coords[k - 1, 1] + ds * np.sin(theta)
        theta += phi
        tau[k] = (np.cos(theta), np.sin(theta))
        nv[k] = (np.sin(theta), -1 * np.cos(theta))
    return s, rho, distance, nsep, coords, nv, tau


# ----------------------------------------------------------------------- mesh
def beam_stats(x, z):
    """Beam statistics used by the wake (pyDFCSR_2D/beams.py:137-215)."""
    x, z = _f64(x), _f64(z)
    slope = np.polyfit(z, x, deg=1)
    return dict(sigma_x=np.std(x), sigma_z=np.std(z), mean_x=np.mean(x), mean_z=np.mean(z),
                slope=slope, x_transform=x - np.polyval(slope, z))


def csr_mesh(stats, xbins, zbins, xlim, zlim):
    """Restates ``get_CSR_mesh`` (pyDFCSR_2D/CSR.py:361-394)."""
    xt = stats["x_transform"]
    sig_x, mean_x = np.std(xt), np.mean(xt)
    sig_z, mean_z = stats["sigma_z"], stats["mean_z"]
    zr = np.linspace(mean_z - zlim * sig_z, mean_z + zlim * sig_z, zbins)
    xr = np.linspace(mean_x - xlim * sig_x, mean_x + xlim * sig_x, xbins)
    xm, zm = np.meshgrid(xr, zr, indexing="ij")
    xm, zm = xm.flatten(), zm.flatten()
    xm = xm + np.polyval(stats["slope"], zm)
    return xm, zm, zr, xr


# ----------------------------------------------------------------------- wake
class WakeOracle:
    """FP64 oracle of ``get_CSR_wake`` / ``calculate_2D_CSR`` over a history.

    ``tracker`` is any object with the attributes ``build_interpolant`` sets
    (``data_*_interp``, ``min_*``, ``delta_*``).
    """

    def __init__(self, tracker, lattice_tables, position, sigma_z, sigma_x, slope0, mean_x,
                 formation_length, n_formation_length, zbins, xbins, charge=1e-9,
                 csr_scaling=None):
        s, rho, distance, coords, nv, tau = lattice_tables
        self._keep = [_f64(tracker.data_density_interp), _f64(tracker.data_density_x_interp),
                      _f64(tracker.data_density_z_interp), _f64(tracker.data_vx_interp),
                      _f64(tracker.data_vx_x_interp)]
        tabs = [_f64(coords[:, 0]), _f64(coords[:, 1]), _f64(nv[:, 0]), _f64(nv[:, 1]),
                _f64(tau[:, 0]), _f64(tau[:, 1])]
        self._keep += tabs + [_f64(rho), _f64(distance)]
        nt, nx, nz = self._keep[0].shape
        c = _Ctx()
        (c.density, c.density_x, c.density_z, c.vx, c.vx_x) = [a.ctypes.data for a in self._keep[:5]]
        c.nt, c.nx, c.nz = nt, nx, nz
        c.t_min, c.x_min, c.z_min = tracker.min_x, tracker.min_y, tracker.min_z
        c.t_delta, c.x_delta, c.z_delta = tracker.delta_x, tracker.delta_y, tracker.delta_z
        (c.X0, c.Y0, c.nX, c.nY, c.tX, c.tY) = [a.ctypes.data for a in tabs]
        c.nsample = tabs[0].size
        c.s_min = s[0]
        c.s_delta = (s[-1] - s[0]) / (s.shape[0] - 1)
        c.rho, c.distance = self._keep[-2].ctypes.data, self._keep[-1].ctypes.data
        c.nelement = self._keep[-1].size
        c.position, c.sigma_z, c.sigma_x = position, sigma_z, sigma_x
        c.slope0, c.mean_x = slope0, mean_x
        c.formation_length, c.n_formation_length = formation_length, n_formation_length
        c.csr_scaling = 8.98755e3 * charge if csr_scaling is None else csr_scaling
        c.zbins, c.xbins = int(zbins), int(xbins)
        self.ctx = c

    def wake(self, s, x, debug=False):
        dE, xk = ctypes.c_double(), ctypes.c_double()
        if not debug:
            lib().oracle_wake_point(ctypes.byref(self.ctx), float(s), float(x),
                                    ctypes.byref(dE), ctypes.byref(xk), None)
            return dE.value, xk.value
        n = 4 * (2 * self.ctx.xbins + self.ctx.zbins + 2 * self.ctx.xbins * self.ctx.zbins * 2)
        buf = np.empty(n)
        lib().oracle_wake_point(ctypes.byref(self.ctx), float(s), float(x), ctypes.byref(dE),
                                ctypes.byref(xk), _ptr(buf))
        return dE.value, xk.value, buf

    def points(self, s, x, nthreads=1):
        s, x = _f64(s), _f64(x)
        dE, xk = np.empty(s.size), np.empty(s.size)
        lib().oracle_wake_points(ctypes.byref(self.ctx), s.size, _ptr(s), _ptr(x), _ptr(dE),
                                 _ptr(xk), int(nthreads))
        return dE, xk
