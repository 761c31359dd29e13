"""Device plumbing for the host API: CUDA checks, streams, workspaces, copies.

PyTorch provides device memory and streams; every computation on the wake
path runs in the sm_103a library through ``_lib``.  There is no CPU path: a
call without a CUDA device raises.
"""
import numpy as np
import torch

from . import _lib


class NoCudaDevice(RuntimeError):
    pass


def require_cuda():
    if not torch.cuda.is_available():
        raise NoCudaDevice("pydfcsr_gb300 runs on a CUDA GPU (built for sm_103a); "
                           "no CUDA device is visible and there is no CPU path")
    _lib.load()


def stream_handle(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes_void(s.cuda_stream)


def ctypes_void(v):
    import ctypes
    return ctypes.c_void_p(int(v)) if v else None


def ptr(t):
    """Device pointer of a tensor (None for None)."""
    if t is None:
        return None
    import ctypes
    return ctypes.c_void_p(t.data_ptr())


def as_device_f64(a, device=None):
    """numpy array / torch tensor -> contiguous float64 CUDA tensor."""
    dev = device or torch.device("cuda", torch.cuda.current_device())
    if isinstance(a, torch.Tensor):
        t = a.detach()
        if t.device.type != "cuda":
            t = t.to(dev, non_blocking=False)
        if t.dtype != torch.float64:
            t = t.to(torch.float64)
        return t.contiguous()
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
    return _async_upload(arr, dev)


def _async_upload(a, dev):
    """Stage through torch's caching pinned-host allocator and copy without
    blocking the host; the allocator keeps the staging block alive until the
    copy has run on the current stream.  (A ring of reusable pinned buffers
    with an event per slot measured slower on the host: 43 vs 21 us per
    small upload.)"""
    t = torch.from_numpy(a)
    if t.numel() == 0:
        return t.to(dev)
    return t.pin_memory().to(dev, non_blocking=True)


def host_to_device(arr, dtype=None, device=None):
    dev = device or torch.device("cuda", torch.cuda.current_device())
    a = np.ascontiguousarray(arr if dtype is None else np.asarray(arr, dtype=dtype))
    return _async_upload(a, dev)


class Workspace:
    """Grow-only device scratch buffers keyed by name."""

    def __init__(self):
        self._bufs = {}

    def get(self, name, nbytes):
        nbytes = max(int(nbytes), 256)
        b = self._bufs.get(name)
        if b is None or b.numel() < nbytes:
            b = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
            self._bufs[name] = b
        return b

    def nbytes(self):
        return sum(b.numel() for b in self._bufs.values())


_default_ws = {}


def default_workspace():
    dev = torch.cuda.current_device()
    ws = _default_ws.get(dev)
    if ws is None:
        ws = Workspace()
        _default_ws[dev] = ws
    return ws


def grid_barrier_check(blocks=None, extra_arrivals=0, max_spins=1 << 24, stream=None):
    """Meet once at the DF stage's bounded grid barrier
    (``dfcsr_grid_barrier_check``) with ``blocks`` CTAs (default: one per SM).
    Returns when every CTA arrived; raises ``_lib.DfcsrTimeout`` when the
    wait gave up - ``extra_arrivals=1`` expects one CTA more than the launch
    has, so every wait gives up after ``max_spins`` polls and the CUDA
    context stays usable."""
    require_cuda()
    if blocks is None:
        blocks = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    bar = torch.zeros(4, dtype=torch.int32, device="cuda")
    _lib.call("dfcsr_grid_barrier_check", int(blocks), int(extra_arrivals), int(max_spins),
              ptr(bar), bar.numel() * 4, stream_handle(stream))
