"""Deposition, distribution functions and the device history ring.

Drop-in for ``pyDFCSR_2D/deposit.py``: ``histogram_cic_2d`` and ``DF_tracker``
keep the reference's names, argument meaning and attributes; the arrays live
on the GPU and every computation runs in the sm_103a library:

* ``histogram_cic_2d`` (deposit.py:43-87) -> sort-by-cell deposit,
  deterministic, both weight channels from one sort;
* ``DF_tracker.get_DF`` (deposit.py:145-245) -> device moments, deposit and
  the fused finalisation (threshold, Savitzky-Golay stencils, trapz
  normalisation, gradients, vx_x fill);
* ``append_DF`` / ``pop_left_DF`` / ``append_interpolant`` /
  ``build_interpolant`` (deposit.py:247-426) -> a device ring of
  (slot, x, z) grids with the five fields interleaved per cell; no per-step
  copy of the history (the reference re-stacks it every step).

Host numpy attributes of the reference (``density``, ``data_density_interp``
...) are still available as lazily copied views for compatibility; hot callers
use the ``*_device`` tensors and the ring directly.
"""
import ctypes
from collections import deque

import numpy as np
import torch

from . import _lib
from .coeffs import savgol_tables
from .runtime import as_device_f64, default_workspace, ptr, require_cuda, stream_handle

__all__ = ["histogram_cic_2d", "deposit_cic", "beam_moments", "DF_tracker", "HistoryRing",
           "FIELDS"]

# field order of the ring and of DF_tracker's device field stack
FIELDS = ("density", "density_x", "density_z", "vx", "vx_x")


def beam_moments(x, z, stream=None, ws=None):
    """Device moments of (x, z): returns a float64 CUDA tensor of 16 values
    (see dfcsr_beam_moments in include/dfcsr_gb300.h)."""
    require_cuda()
    n = x.numel()
    ws = ws or default_workspace()
    out = torch.empty(16, dtype=torch.float64, device=x.device)
    nb = _lib.query("dfcsr_moments_workspace_bytes", n)
    buf = ws.get("moments", nb)
    _lib.call("dfcsr_beam_moments", ptr(x), ptr(z), n, ptr(out), ptr(buf), buf.numel(),
              stream_handle(stream))
    return out


def deposit_cic(q1, q2, w0, w1, nbins_1, bins_start_1, bins_end_1, nbins_2, bins_start_2,
                bins_end_2, stream=None, ws=None, out0=None, out1=None):
    """Deterministic CIC deposit of up to two weight channels (device tensors).

    ``w0 = None`` deposits unit weights.  Returns (out0, out1 or None), each a
    float64 CUDA tensor of shape (nbins_1, nbins_2) (written into ``out0`` /
    ``out1`` when given: contiguous float64 of that many elements).
    """
    require_cuda()
    n = q1.numel()
    ws = ws or default_workspace()
    nb1, nb2 = int(nbins_1), int(nbins_2)
    if out0 is None:
        out0 = torch.empty((nb1, nb2), dtype=torch.float64, device=q1.device)
    if out1 is None and w1 is not None:
        out1 = torch.empty((nb1, nb2), dtype=torch.float64, device=q1.device)
    need = _lib.query("dfcsr_deposit_workspace_bytes", n, nb1, nb2)
    buf = ws.get("deposit", need)
    _lib.call("dfcsr_deposit_cic2d", ptr(q1), ptr(q2), ptr(w0), ptr(w1), n, nb1,
              float(bins_start_1), float(bins_end_1), nb2, float(bins_start_2), float(bins_end_2),
              ptr(out0), ptr(out1), ptr(buf), buf.numel(), stream_handle(stream))
    return out0, out1


def deposit_cic_from_moments(q1, q2, w0, w1, nbins_1, nbins_2, moments, lim_1, lim_2, stream=None,
                             ws=None, out0=None, out1=None):
    """(extension) :func:`deposit_cic` on the grid mean -+ lim sigma per axis
    taken from ``moments`` (a CUDA float64 tensor of dfcsr_beam_moments) on
    the device: nothing waits for the host."""
    require_cuda()
    n = q1.numel()
    ws = ws or default_workspace()
    nb1, nb2 = int(nbins_1), int(nbins_2)
    if moments.dtype != torch.float64 or not moments.is_cuda or moments.numel() < 5:
        raise ValueError("moments must be a CUDA float64 tensor of dfcsr_beam_moments")
    if out0 is None:
        out0 = torch.empty((nb1, nb2), dtype=torch.float64, device=q1.device)
    if out1 is None and w1 is not None:
        out1 = torch.empty((nb1, nb2), dtype=torch.float64, device=q1.device)
    need = _lib.query("dfcsr_deposit_workspace_bytes", n, nb1, nb2)
    buf = ws.get("deposit", need)
    m = moments.contiguous()
    # the deposit's first kernel reads the moments on `stream`: keep their
    # memory from being reused by the allocator before it has run
    m.record_stream(stream if stream is not None else torch.cuda.current_stream())
    _lib.call("dfcsr_deposit_cic2d_moments", ptr(q1), ptr(q2), ptr(w0), ptr(w1), n, nb1, nb2,
              ptr(m), float(lim_1), float(lim_2), ptr(out0), ptr(out1),
              ptr(buf), buf.numel(), stream_handle(stream))
    return out0, out1


def histogram_cic_2d(q1, q2, w, nbins_1, bins_start_1, bins_end_1, nbins_2, bins_start_2,
                     bins_end_2):
    """2D cloud-in-cell histogram of ``q1``, ``q2`` weighted by ``w``.

    Same contract as pyDFCSR_2D/deposit.py:43-87: ``nbins_1`` bins from
    ``bins_start_1`` to ``bins_end_1`` in the first dimension (spacing
    (end - start) / nbins), linear (CIC) weights, contributions outside the
    grid dropped.  numpy inputs give a numpy result; torch inputs give a
    CUDA tensor.
    """
    as_numpy = not isinstance(q1, torch.Tensor)
    a, b, c = as_device_f64(q1).reshape(-1), as_device_f64(q2).reshape(-1), as_device_f64(w).reshape(-1)
    if not (a.numel() == b.numel() == c.numel()):
        raise ValueError("q1, q2 and w must have the same length")
    out, _ = deposit_cic(a, b, c, None, nbins_1, bins_start_1, bins_end_1, nbins_2, bins_start_2,
                         bins_end_2)
    return out.cpu().numpy() if as_numpy else out


class HistoryRing:
    """Device ring of (slot, x, z) grids holding the five DF fields per cell.

    ``ring64`` is float64 [cap, nx, nz, 5] (plain FP64 wake); ``ring32`` is
    float32 [cap, nx, nz, 8] (mixed-precision wake): fields 0..4, the low part
    of density_x in slot 5 (density_x is carried as a float-float pair), 32-byte
    cells so a corner loads as two aligned float4.  Logical
    slice k (0 = oldest) lives in physical slot (head + k) % cap.
    """

    def __init__(self, nx, nz, store64=True, store32=False, cap=8, device=None):
        self.nx, self.nz = int(nx), int(nz)
        self.store64, self.store32 = store64, store32
        self.device = device or torch.device("cuda", torch.cuda.current_device())
        self.cap = 0
        self.head = 0
        self.count = 0
        self.ring64 = self.ring32 = None
        self._grow(max(int(cap), 2))

    def _alloc(self, cap):
        r64 = torch.empty((cap, self.nx, self.nz, 5), dtype=torch.float64,
                          device=self.device) if self.store64 else None
        # no fill: the regrid writes all eight words of every cell of a slot
        # (the two pad words as zeros) before the slot is read
        r32 = torch.empty((cap, self.nx, self.nz, 8), dtype=torch.float32,
                          device=self.device) if self.store32 else None
        return r64, r32

    def _grow(self, cap):
        r64, r32 = self._alloc(cap)
        for k in range(self.count):
            src = (self.head + k) % self.cap
            if r64 is not None:
                r64[k].copy_(self.ring64[src])
            if r32 is not None:
                r32[k].copy_(self.ring32[src])
        self.ring64, self.ring32 = r64, r32
        self.cap, self.head = cap, 0

    def nbytes(self):
        return sum(t.numel() * t.element_size() for t in (self.ring64, self.ring32) if t is not None)

    def push(self):
        """Reserve the next slot; returns (slot64 view or None, slot32 view or None)."""
        if self.count == self.cap:
            self._grow(2 * self.cap)
        slot = (self.head + self.count) % self.cap
        self.count += 1
        return (self.ring64[slot] if self.ring64 is not None else None,
                self.ring32[slot] if self.ring32 is not None else None)

    def pop_left(self):
        if self.count == 0:
            raise IndexError("pop from an empty history ring")
        self.head = (self.head + 1) % self.cap
        self.count -= 1

    def clear(self, nx=None, nz=None):
        if (nx is not None and int(nx) != self.nx) or (nz is not None and int(nz) != self.nz):
            self.nx, self.nz = int(nx), int(nz)
            self.ring64, self.ring32 = self._alloc(self.cap)
        self.head = 0
        self.count = 0

    def slice(self, k, field):
        """Host copy of one field of logical slice k (0 = oldest)."""
        f = FIELDS.index(field)
        slot = (self.head + k) % self.cap
        if self.ring64 is not None:
            return self.ring64[slot][..., f].cpu().numpy()
        return self.ring32[slot][..., f].double().cpu().numpy()

    def stacked(self, field):
        """Host copy [count, nx, nz] of one field in time order (compatibility)."""
        f = FIELDS.index(field)
        idx = [(self.head + k) % self.cap for k in range(self.count)]
        if self.ring64 is not None:
            return self.ring64[idx][..., f].cpu().numpy()
        return self.ring32[idx][..., f].double().cpu().numpy()


_SG_DEVICE = {}


def _sg_tables_device(window, order):
    """Savitzky-Golay tables (coeff, lo, hi of coeffs.savgol_tables) in device
    memory, one copy per device and (window, order), uploaded once with a
    blocking copy (so any stream may read them).  Returns (tensor, (coeff,
    lo, hi) device addresses)."""
    dev = torch.cuda.current_device()
    key = (dev, window, order)
    hit = _SG_DEVICE.get(key)
    if hit is None:
        coeff, lo, hi = savgol_tables(window, order)
        parts = [coeff, lo.ravel(), hi.ravel()]
        t = torch.from_numpy(np.concatenate(parts)).to(torch.device("cuda", dev))
        offs = np.concatenate([[0], np.cumsum([p.size for p in parts])])
        hit = (t, tuple(t.data_ptr() + 8 * int(o) for o in offs[:3]))
        _SG_DEVICE[key] = hit
    return hit


class PendingDeposit:
    """A deposit enqueued by :meth:`DF_tracker.deposit_DF`: the host moments
    it was sized from (None when the grid came from the device moments), the
    field array [5, nx, nz] (channels 0 and 3 written by the deposit) and the
    event recorded after it."""
    __slots__ = ("moments", "fields", "event")

    def __init__(self, moments, fields, event):
        self.moments, self.fields, self.event = moments, fields, event


def raise_if_df_failed(flags):
    """Raise DfcsrTimeout if any DF finalisation status word in ``flags``
    (host values of scalars[7]) is set."""
    bad = int(np.count_nonzero(np.asarray(flags) != 0.0))
    if bad:
        raise _lib.DfcsrTimeout(3, "dfcsr_df_finalize",
                                f"a grid-barrier wait gave up in {bad} DF finalisation(s); "
                                "their fields are invalid")


class _DFEntry:
    """One logged DF: grids (numpy linspaces and their (start, stop, n)),
    the five fields on the device, the finalisation scalars, t and sigmas."""
    __slots__ = ("x_grids", "z_grids", "x_lin", "z_lin", "fields", "scalars", "t", "sigma_x",
                 "sigma_z")

    def __init__(self, x_grids, z_grids, fields, scalars, t, sigma_x, sigma_z, x_lin, z_lin):
        self.x_grids, self.z_grids = x_grids, z_grids
        self.x_lin, self.z_lin = x_lin, z_lin
        self.fields, self.scalars = fields, scalars
        self.t, self.sigma_x, self.sigma_z = t, sigma_x, sigma_z


class DF_tracker:
    """Distribution functions of the beam and their history, on the GPU.

    Mirrors ``pyDFCSR_2D.deposit.DF_tracker`` (deposit.py:90-426).  Extra
    keyword arguments (not in the reference):

    * ``precision``: ``'fp64'`` keeps the FP64 ring for the plain wake,
      ``'mixed'`` the FP32 ring for the mixed-precision wake, ``'both'`` both.
    * ``grid_rule``: ``'reference'`` reproduces get_DF's fallback to a 100x100
      grid and window 5 when sigma_x / sigma_x(slice) <= 5
      (deposit.py:157-168); ``'configured'`` always uses the configured bins
      and window.
    """

    def __init__(self, input_dic={}, precision="fp64", grid_rule="reference", workspace=None):
        self.configure_params(**input_dic)
        if precision not in ("fp64", "mixed", "both"):
            raise ValueError("precision must be 'fp64', 'mixed' or 'both'")
        if grid_rule not in ("reference", "configured"):
            raise ValueError("grid_rule must be 'reference' or 'configured'")
        self.precision = precision
        self.grid_rule = grid_rule
        self.ws = workspace
        self.sigma_x = self.sigma_z = None
        self.x_grids = self.z_grids = None
        self.start_time = 0.0
        self.t = 0.0
        self.slope_log = deque([])
        self.DF_log = deque([])
        self.sigma_x_log = deque([])
        self.sigma_z_log = deque([])
        self.time_log = deque([])
        self.sigma_x_interp = self.sigma_z_interp = None
        self.time_interp = deque([])
        self.interp_start = 0
        self.end_time = 0.0
        self.x_grid_interp = self.z_grid_interp = None
        self.ring = None
        self._cur = None
        self.stats = None
        self.reinterpolated = False
        # finalisation scalars not yet checked for a barrier timeout:
        # [(scalars, event after the finalisation)]
        self._unchecked = []
        # (extension) test hooks of the DF stage's bounded grid-barrier waits:
        # polls before a wait gives up (0: the library's default, about a
        # second) and 1 to expect an arrival that never comes, so that the
        # waits run out and the timeout path is exercised
        self.barrier_spins = 0
        self.barrier_extra = 0

    def configure_params(self, xbins=100, zbins=100, xlim=5, zlim=5, filter_order=0,
                         filter_window=0, velocity_threhold=5, upper_limit=None):
        self.xbins = xbins
        self.zbins = zbins
        self.xlim = xlim
        self.zlim = zlim
        self.velocity_threhold = velocity_threhold
        self.filter_order = filter_order
        self.filter_window = filter_window
        self.upper_limit = upper_limit

    # ------------------------------------------------------------- get_DF
    def _workspace(self):
        return self.ws or default_workspace()

    def _grid(self, st):
        """Grid and smoothing window of get_DF (deposit.py:157-170) from the
        beam moments ``st`` (host array of dfcsr_beam_moments)."""
        sigma_x, sigma_z = float(st[3]), float(st[4])
        xmean, zmean = float(st[1]), float(st[2])
        with np.errstate(all="ignore"):
            frac = np.float64(sigma_x) / np.float64(st[8])
        if frac > 5 or self.grid_rule == "configured":
            xb, zb, win = int(self.xbins), int(self.zbins), int(self.filter_window)
        else:
            xb, zb, win = 100, 100, 5
        x0 = xmean - self.xlim * sigma_x
        x1 = xmean + self.xlim * sigma_x
        z0 = zmean - self.zlim * sigma_z
        z1 = zmean + self.zlim * sigma_z
        return xb, zb, win, x0, x1, z0, z1

    def deposit_DF(self, x, z, px, moments, stream=None):
        """(extension) The deposit half of get_DF: the grid from ``moments``,
        both CIC channels into a new field array, enqueued on ``stream``
        (default: the current stream).  Returns a :class:`PendingDeposit` to
        hand to ``get_DF(..., deposited=...)``; the tracker's state is not
        touched, so the deposit of a later step can run while this step is
        finalised.  ``x``, ``z``, ``px`` must stay unchanged until the
        deposit has run.  Deposits of one tracker share its deposit scratch:
        two of them must not be in flight on different streams at once.

        ``moments`` is the host array of dfcsr_beam_moments, or the CUDA
        tensor itself (e.g. ``beam.moments_device`` while its copy to the
        host is in flight): with the configured grid rule the deposit then
        takes its grid from the device moments and nothing waits for the
        host; get_DF receives the host copy later through its ``moments``
        argument (``CSR2D.update_history`` passes the beam's)."""
        require_cuda()
        s = stream if stream is not None else torch.cuda.current_stream()
        if isinstance(moments, torch.Tensor):
            if self.grid_rule == "configured":
                # the grid from the device moments, by the deposit's first kernel
                xb, zb = int(self.xbins), int(self.zbins)
                with torch.cuda.stream(s):
                    xd, zd, pxd = (as_device_f64(a).reshape(-1) for a in (x, z, px))
                    fields = torch.empty((5, xb, zb), dtype=torch.float64, device=xd.device)
                    deposit_cic_from_moments(xd, zd, None, pxd, xb, zb, moments, self.xlim,
                                             self.zlim, s, self._workspace(), out0=fields[0],
                                             out1=fields[3])
                    ev = torch.cuda.Event()
                    ev.record(s)
                return PendingDeposit(None, fields, ev)
            # the reference's rule picks the bins from the moments: host copy
            moments = moments.cpu().numpy()
        st = np.asarray(moments, dtype=np.float64)
        xb, zb, win, x0, x1, z0, z1 = self._grid(st)
        with torch.cuda.stream(s):
            xd, zd, pxd = (as_device_f64(a).reshape(-1) for a in (x, z, px))
            fields = torch.empty((5, xb, zb), dtype=torch.float64, device=xd.device)
            deposit_cic(xd, zd, None, pxd, xb, x0, x1, zb, z0, z1, s, self._workspace(),
                        out0=fields[0], out1=fields[3])
            ev = torch.cuda.Event()
            ev.record(s)
        return PendingDeposit(st, fields, ev)

    def get_DF(self, x, z, px, t, stream=None, moments=None, deposited=None):
        """Deposit and finalise the current DF (deposit.py:145-245).

        ``moments`` (extension): the host copy of ``beam_moments(x, z)`` when
        the caller already has it for these exact arrays (saves a pass and a
        device synchronisation).  ``deposited`` (extension): the handle of an
        earlier :meth:`deposit_DF` of these particles; the deposit is then
        not repeated (x, z, px are not read) and ``stream`` waits for it."""
        require_cuda()
        ws = self._workspace()
        if deposited is None:
            if moments is None:
                xd, zd = (as_device_f64(a).reshape(-1) for a in (x, z))
                moments = beam_moments(xd, zd, stream, ws).cpu().numpy()
            deposited = self.deposit_DF(x, z, px, moments, stream)
        s = stream if stream is not None else torch.cuda.current_stream()
        s.wait_event(deposited.event)
        fields = deposited.fields
        fields.record_stream(s)
        st = deposited.moments
        if st is None:      # sized on the device from the moments: their host copy
            if moments is None:
                raise ValueError("get_DF: a deposit sized from device moments needs the host "
                                 "moments (the 'moments' argument)")
            st = np.asarray(moments, dtype=np.float64)
            _, _, _, x0, x1, z0, z1 = self._grid(st)
            if x1 == x0 or z1 == z0:
                raise ValueError("dfcsr_deposit_cic2d_moments: empty bin range")
        self.stats = st
        sigma_x, sigma_z = float(st[3]), float(st[4])
        self.sigma_x, self.sigma_z = sigma_x, sigma_z
        self.xmean, self.zmean = float(st[1]), float(st[2])
        xb, zb, win, x0, x1, z0, z1 = self._grid(st)
        xg = np.linspace(x0, x1, xb)
        zg = np.linspace(z0, z1, zb)
        sc = torch.empty(8, dtype=torch.float64, device=fields.device)   # written by df_finalize
        self._finalize(fields, sc, (x0, x1, xb), (z0, z1, zb), xg, zg, win, stream, ws)
        self.x_grids, self.z_grids = xg, zg
        self._cur = _DFEntry(xg, zg, fields, sc, t, sigma_x, sigma_z, (x0, x1, xb), (z0, z1, zb))
        self.t = t
        self.bins = (xb, zb, win)

    def _finalize(self, fields, sc, xlin, zlin, xg, zg, win, stream, ws):
        """The DF stage on the deposited fields.  The Savitzky-Golay tables
        come from a per-device cache; the grid tables (numpy.gradient
        coefficients and diff of each grid) are computed on the device from
        the two linspaces (``dfcsr_df_axis_tables``), equal to the host's
        ``coeffs.gradient_table`` bit for bit; the host only decides numpy's
        uniform-spacing branch from ``xg`` and ``zg``."""
        xb, zb = xg.size, zg.size
        sg = _sg_tables_device(int(win), int(self.filter_order))
        dxh, dzh = np.diff(xg), np.diff(zg)
        gxu, gzu = bool(np.all(dxh == dxh[0])), bool(np.all(dzh == dzh[0]))
        sizes = [4 * xb, 4 * zb, xb - 1, zb - 1]
        offs = np.concatenate([[0], np.cumsum([(v + 31) // 32 * 32 for v in sizes])])
        tab = ws.get("df_axes", 8 * int(offs[-1]))
        base = tab.data_ptr()
        gx, gz, dxg, dzg = [base + 8 * int(o) for o in offs[:4]]
        _lib.call("dfcsr_df_axis_tables", float(xlin[0]), float(xlin[1]), xb, float(zlin[0]),
                  float(zlin[1]), zb, int(gxu), int(gzu), ctypes.c_void_p(gx), ctypes.c_void_p(gz),
                  ctypes.c_void_p(dxg), ctypes.c_void_p(dzg), stream_handle(stream))
        P = _lib.DFParams()
        P.nx, P.nz, P.window, P.order = xb, zb, int(win), int(self.filter_order)
        P.velocity_threshold = float(self.velocity_threhold)
        P.sg_coeff, P.sg_lo, P.sg_hi = sg[1]
        P.gx, P.gz, P.dxg, P.dzg = gx, gz, dxg, dzg
        P.gx_uniform, P.gz_uniform = int(gxu), int(gzu)
        P.gx_dx, P.gz_dx = float(dxh[0]), float(dzh[0])
        P.barrier_spins, P.barrier_extra = int(self.barrier_spins), int(self.barrier_extra)
        need = _lib.query("dfcsr_df_workspace_bytes", xb, zb)
        buf = ws.get("df", need)
        _lib.call("dfcsr_df_finalize", ctypes.byref(P), ptr(fields[0]), ptr(fields[3]),
                  ptr(fields[1]), ptr(fields[2]), ptr(fields[4]), ptr(sc), ptr(buf), buf.numel(),
                  stream_handle(stream))
        ev = torch.cuda.Event()
        ev.record(stream if stream is not None else torch.cuda.current_stream())
        self._unchecked.append((sc, ev))
        if len(self._unchecked) > 256:   # a caller that never checks: bound the list
            self.check_status()

    def take_unchecked(self):
        """(extension) The finalisation scalars not yet checked, as
        [(scalars, event)], handed over to the caller (who checks their
        status word, scalars[7], once the events have passed)."""
        out, self._unchecked = self._unchecked, []
        return out

    def check_status(self):
        """(extension) Raise :class:`DfcsrTimeout` if a DF finalisation since
        the last check reported that one of its grid-barrier waits gave up
        (status word scalars[7] = 1: that step's fields are invalid).  Waits
        for those finalisations."""
        pend = self.take_unchecked()
        if not pend:
            return
        for _, ev in pend:
            ev.synchronize()
        flags = torch.stack([sc[7] for sc, _ in pend]).cpu().numpy()
        raise_if_df_failed(flags)

    # compatibility views of the current DF (host copies)
    def _field(self, name):
        return None if self._cur is None else self._cur.fields[FIELDS.index(name)].cpu().numpy()

    density = property(lambda self: self._field("density"))
    density_x = property(lambda self: self._field("density_x"))
    density_z = property(lambda self: self._field("density_z"))
    vx = property(lambda self: self._field("vx"))
    vx_x = property(lambda self: self._field("vx_x"))

    @property
    def fields_device(self):
        """Current DF as a float64 CUDA tensor [5, nx, nz] in FIELDS order."""
        return None if self._cur is None else self._cur.fields

    # ----------------------------------------------------------- history
    def append_DF(self):
        """append current DF to the log (deposit.py:247-256)"""
        self.DF_log.append(self._cur)
        self.time_log.append(self.t)
        self.sigma_x_log.append(self.sigma_x)
        self.sigma_z_log.append(self.sigma_z)
        self.end_time = self.t

    def pop_left_DF(self, new_start_time):
        """pop history until new_start_time (deposit.py:258-280)"""
        while self.start_time < new_start_time:
            self.DF_log.popleft()
            self.time_log.popleft()
            self.sigma_x_log.popleft()
            self.sigma_z_log.popleft()
            self.start_time = self.time_log[0]
        while self.interp_start < new_start_time:
            self.ring.pop_left()
            self.time_interp.popleft()
            self.interp_start = self.time_interp[0]

    def pop_right_DF(self):
        """pop the newest DF from the log (deposit.py:283-292)"""
        self.DF_log.pop()
        self.time_log.pop()
        self.sigma_x_log.pop()
        self.sigma_z_log.pop()
        self.end_time = self.time_log[-1]

    def _regrid_into_ring(self, entry, stream=None):
        """Regrid one logged DF into a new ring slot: axis tables on the
        device (both grids are linspaces), then the five-field regrid."""
        (xs0, xs1, xsn), (zs0, zs1, zsn) = entry.x_lin, entry.z_lin
        (xt0, xt1, nxi), (zt0, zt1, nzi) = self.x_interp_lin, self.z_interp_lin
        pad = lambda b: (b + 255) // 256 * 256
        sizes = [pad(8 * nxi), pad(8 * nzi), pad(4 * nxi), pad(4 * nzi), pad(nxi), pad(nzi)]
        buf = self._workspace().get("rgi", sum(sizes))
        key = (buf.data_ptr(), nxi, nzi)
        if getattr(self, "_rgi_ptrs", (None,))[0] != key:   # table pointers, once per buffer
            offs = np.concatenate([[0], np.cumsum(sizes)])
            self._rgi_ptrs = (key, tuple(ctypes.c_void_p(buf.data_ptr() + int(o)) for o in offs[:6]))
        wx, wz, ix, iz, ox, oz = self._rgi_ptrs[1]
        h = stream_handle(stream)
        _lib.call("dfcsr_rgi_axis_linspace", xs0, xs1, xsn, xt0, xt1, nxi, ix, wx, ox, h)
        _lib.call("dfcsr_rgi_axis_linspace", zs0, zs1, zsn, zt0, zt1, nzi, iz, wz, oz, h)
        s64, s32 = self.ring.push()
        f = entry.fields
        _lib.call("dfcsr_history_regrid", ptr(f[0]), ptr(f[1]), ptr(f[2]), ptr(f[3]), ptr(f[4]),
                  f.shape[1], f.shape[2], ix, wx, ox, nxi, iz, wz, oz, nzi,
                  ctypes.c_void_p(entry.scalars.data_ptr() + 8 * 4),
                  ptr(s64), ptr(s32), h)

    def _new_ring(self, nxi, nzi):
        store64 = self.precision in ("fp64", "both")
        store32 = self.precision in ("mixed", "both")
        if self.ring is None:
            self.ring = HistoryRing(nxi, nzi, store64, store32, cap=max(8, len(self.DF_log) + 4))
        else:
            self.ring.clear(nxi, nzi)

    def append_interpolant(self, formation_length, n_formation_length, stream=None):
        """Trim the window and append the current DF to the interpolant
        (deposit.py:312-392)."""
        start_point = np.amax((0, self.end_time - n_formation_length * formation_length))
        self.pop_left_DF(new_start_time=start_point)
        if self.sigma_x_interp and self.sigma_z_interp and \
                2 > self.sigma_x / self.sigma_x_interp > 1 / 2 and \
                2 > self.sigma_z / self.sigma_z_interp > 1 / 2:
            self.time_interp.append(self.t)
            self._regrid_into_ring(self._cur, stream)
            self.reinterpolated = False
            return
        max_sigma_x, min_sigma_x = np.max(self.sigma_x_log), np.min(self.sigma_x_log)
        max_sigma_z, min_sigma_z = np.max(self.sigma_z_log), np.min(self.sigma_z_log)
        xbins = int(500 * (max_sigma_x / min_sigma_x))
        zbins = int(500 * (max_sigma_z / min_sigma_z))
        if isinstance(self.upper_limit, int):
            xbins = min(xbins, self.upper_limit)
            zbins = min(zbins, self.upper_limit)
        self.sigma_x_interp = max_sigma_x
        self.sigma_z_interp = max_sigma_z
        self.x_interp_lin = (self.xmean - 5 * self.sigma_x_interp,
                             self.xmean + 5 * self.sigma_x_interp, xbins)
        self.z_interp_lin = (self.zmean - 5 * self.sigma_z_interp,
                             self.zmean + 5 * self.sigma_z_interp, zbins)
        self.x_grid_interp = np.linspace(*self.x_interp_lin)
        self.z_grid_interp = np.linspace(*self.z_interp_lin)
        self._new_ring(xbins, zbins)
        self.time_interp = self.time_log.copy()
        for entry in self.DF_log:
            self._regrid_into_ring(entry, stream)
        self.reinterpolated = True

    def build_interpolant(self):
        """Interpolant parameters over the ring (deposit.py:395-426); the
        history itself is not copied."""
        self.min_x, self.max_x = self.time_interp[0], self.time_interp[-1]
        self.min_y, self.max_y = self.x_grid_interp[0], self.x_grid_interp[-1]
        self.min_z, self.max_z = self.z_grid_interp[0], self.z_grid_interp[-1]
        self.delta_x = (self.max_x - self.min_x) / (len(self.time_interp) - 1)
        self.delta_y = (self.max_y - self.min_y) / (self.x_grid_interp.shape[0] - 1)
        self.delta_z = (self.max_z - self.min_z) / (self.z_grid_interp.shape[0] - 1)

    # -------------------------------------------------------- checkpoint
    _STATE_SCALARS = ("sigma_x", "sigma_z", "xmean", "zmean", "start_time", "t", "end_time",
                      "interp_start", "sigma_x_interp", "sigma_z_interp", "x_interp_lin",
                      "z_interp_lin", "x_grids", "z_grids", "x_grid_interp", "z_grid_interp",
                      "bins", "reinterpolated", "min_x", "max_x", "min_y", "max_y", "min_z",
                      "max_z", "delta_x", "delta_y", "delta_z")
    _STATE_LOGS = ("slope_log", "sigma_x_log", "sigma_z_log", "time_log", "time_interp")

    def state_dict(self):
        """(extension) The tracker's state as host data (numpy arrays, floats,
        tuples; picklable): configuration, logs, every logged DF (fields and
        finalisation scalars) and the history ring's slices in time order.
        Waits for the device.  :meth:`load_state_dict` on a tracker of the
        same precision resumes it: the steps that follow give the same
        results bit for bit.  (The reference keeps its history in memory
        only; its particle dumps, CSR.py:784-797, hold the beam.)"""
        torch.cuda.synchronize()

        def entry(e):
            return {"x_grids": e.x_grids, "z_grids": e.z_grids, "x_lin": e.x_lin,
                    "z_lin": e.z_lin, "fields": e.fields.cpu().numpy(),
                    "scalars": e.scalars.cpu().numpy(), "t": e.t, "sigma_x": e.sigma_x,
                    "sigma_z": e.sigma_z}

        log = list(self.DF_log)
        cur = next((i for i, e in enumerate(log) if e is self._cur), None)
        ring = None
        if self.ring is not None:
            r = self.ring
            idx = [(r.head + k) % r.cap for k in range(r.count)]
            ring = {"nx": r.nx, "nz": r.nz, "count": r.count,
                    "ring64": r.ring64[idx].cpu().numpy() if r.ring64 is not None else None,
                    "ring32": r.ring32[idx].cpu().numpy() if r.ring32 is not None else None}
        return {
            "precision": self.precision, "grid_rule": self.grid_rule,
            "config": {k: getattr(self, k) for k in ("xbins", "zbins", "xlim", "zlim",
                                                     "filter_order", "filter_window",
                                                     "velocity_threhold", "upper_limit")},
            "scalars": {k: getattr(self, k) for k in self._STATE_SCALARS if hasattr(self, k)},
            "stats": None if self.stats is None else np.array(self.stats, dtype=np.float64),
            "logs": {k: list(getattr(self, k)) for k in self._STATE_LOGS},
            "DF_log": [entry(e) for e in log],
            "cur": cur if cur is not None else (None if self._cur is None else entry(self._cur)),
            "ring": ring,
        }

    def load_state_dict(self, state):
        """(extension) Restore a :meth:`state_dict` onto the current device."""
        require_cuda()
        if state["precision"] != self.precision:
            raise ValueError(f"state of a '{state['precision']}' tracker, this one is "
                             f"'{self.precision}'")
        self.configure_params(**state["config"])
        self.grid_rule = state["grid_rule"]
        for k, v in state["scalars"].items():
            setattr(self, k, v)
        self.stats = None if state["stats"] is None else np.array(state["stats"])
        for k in self._STATE_LOGS:
            setattr(self, k, deque(state["logs"][k]))
        dev = torch.device("cuda", torch.cuda.current_device())

        def entry(e):
            return _DFEntry(e["x_grids"], e["z_grids"], torch.from_numpy(e["fields"]).to(dev),
                            torch.from_numpy(e["scalars"]).to(dev), e["t"], e["sigma_x"],
                            e["sigma_z"], tuple(e["x_lin"]), tuple(e["z_lin"]))

        self.DF_log = deque(entry(e) for e in state["DF_log"])
        cur = state["cur"]
        self._cur = self.DF_log[cur] if isinstance(cur, int) else (None if cur is None else entry(cur))
        r = state["ring"]
        self.ring = None
        if r is not None:
            ring = HistoryRing(r["nx"], r["nz"], r["ring64"] is not None, r["ring32"] is not None,
                               cap=max(8, r["count"] + 4), device=dev)
            for k in range(r["count"]):
                s64, s32 = ring.push()
                if s64 is not None:
                    s64.copy_(torch.from_numpy(r["ring64"][k]))
                if s32 is not None:
                    s32.copy_(torch.from_numpy(r["ring32"][k]))
            self.ring = ring
        torch.cuda.synchronize()

    # stacked host copies, like the reference's data_*_interp arrays
    data_density_interp = property(lambda self: self.ring.stacked("density"))
    data_density_x_interp = property(lambda self: self.ring.stacked("density_x"))
    data_density_z_interp = property(lambda self: self.ring.stacked("density_z"))
    data_vx_interp = property(lambda self: self.ring.stacked("vx"))
    data_vx_x_interp = property(lambda self: self.ring.stacked("vx_x"))

    def job_fields(self):
        """Ring pointers and interpolant parameters for a dfcsr_wake_job."""
        r = self.ring
        return dict(ring64=r.ring64.data_ptr() if r.ring64 is not None else None,
                    ring32=r.ring32.data_ptr() if r.ring32 is not None else None,
                    cap=r.cap, head=r.head, nt=r.count, nx=r.nx, nz=r.nz,
                    t_min=float(self.min_x), x_min=float(self.min_y), z_min=float(self.min_z),
                    t_delta=float(self.delta_x), x_delta=float(self.delta_y),
                    z_delta=float(self.delta_z))
