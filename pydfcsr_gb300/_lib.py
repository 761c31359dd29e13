"""ctypes binding of ``libdfcsr_gb300.so`` (the C ABI in include/dfcsr_gb300.h).

Loading never falls back to anything: if the shared library is missing and
cannot be built, importing a compute entry point raises.  Status codes become
Python exceptions with the library's thread-local message.
"""
import ctypes
import os
import threading

from . import build as _build

_c_double = ctypes.c_double
_c_int = ctypes.c_int
_c_i64 = ctypes.c_int64
_c_size = ctypes.c_size_t
_p = ctypes.c_void_p


class DfcsrError(RuntimeError):
    """A dfcsr_gb300 C-ABI call failed."""

    def __init__(self, status, name, message):
        super().__init__(f"{name}: [{status_name(status)}] {message}")
        self.status = status


class DfcsrBadArgument(DfcsrError, ValueError):
    pass


class DfcsrOutOfMemory(DfcsrError, MemoryError):
    pass


class DfcsrTimeout(DfcsrError, TimeoutError):
    pass


class DfcsrKernelError(DfcsrError):
    pass


class DfcsrCudaError(DfcsrError):
    pass


class DfcsrAdmissionRefused(DfcsrError):
    pass


_EXC = {1: DfcsrBadArgument, 2: DfcsrOutOfMemory, 3: DfcsrTimeout, 4: DfcsrKernelError,
        5: DfcsrCudaError, 6: DfcsrAdmissionRefused}

_NAMES = {0: "OK", 1: "BAD_ARG", 2: "OOM", 3: "TIMEOUT", 4: "KERNEL_ERROR", 5: "CUDA_ERROR",
          6: "ADMISSION_REFUSED"}


def status_name(status):
    return _NAMES.get(status, "UNKNOWN")


class DFParams(ctypes.Structure):
    """``dfcsr_df_params``."""
    _fields_ = [
        ("nx", _c_int), ("nz", _c_int), ("window", _c_int), ("order", _c_int),
        ("velocity_threshold", _c_double),
        ("sg_coeff", _p), ("sg_lo", _p), ("sg_hi", _p), ("gx", _p), ("gz", _p),
        ("dxg", _p), ("dzg", _p),
        ("gx_uniform", _c_int), ("gz_uniform", _c_int),
        ("gx_dx", _c_double), ("gz_dx", _c_double),
        ("barrier_spins", ctypes.c_uint), ("barrier_extra", _c_int),
    ]


class WakeJob(ctypes.Structure):
    """``dfcsr_wake_job``."""
    _fields_ = [
        ("ring64", _p), ("ring32", _p),
        ("cap", _c_int), ("head", _c_int), ("nt", _c_int), ("nx", _c_int), ("nz", _c_int),
        ("pad0", _c_int),
        ("t_min", _c_double), ("x_min", _c_double), ("z_min", _c_double),
        ("t_delta", _c_double), ("x_delta", _c_double), ("z_delta", _c_double),
        ("lattice", _p), ("nsample", _c_int), ("nelement", _c_int),
        ("s_min", _c_double), ("s_delta", _c_double),
        ("rho", _p), ("distance", _p),
        ("position", _c_double), ("sigma_z", _c_double), ("sigma_x", _c_double),
        ("slope0", _c_double), ("mean_x", _c_double),
        ("formation_length", _c_double), ("n_formation_length", _c_double),
        ("csr_scaling", _c_double),
        ("zbins", _c_int), ("xbins", _c_int),
        ("near_band", _c_double),
        ("lattice_delta", _p),
        ("lattice_dw", _p), ("lattice_delta_dw", _p),
    ]


# (name, restype, argtypes)
_SIGS = [
    ("dfcsr_version", _c_int, []),
    ("dfcsr_kernel_launches", ctypes.c_longlong, []),
    ("dfcsr_last_error", ctypes.c_char_p, []),
    ("dfcsr_status_name", ctypes.c_char_p, [_c_int]),
    ("dfcsr_abi_sizeof", _c_size, [_c_int]),
    ("dfcsr_bounds_checked", _c_int, []),
    ("dfcsr_bounds_status", _c_int, [ctypes.POINTER(ctypes.c_ulonglong), _c_int]),
    ("dfcsr_bounds_probe", _c_int, [ctypes.c_longlong, ctypes.c_longlong, _c_int, _p]),
    ("dfcsr_timing_enable", None, [_c_int]),
    ("dfcsr_timing_collect", _c_int, []),
    ("dfcsr_timing_get", _c_int, [ctypes.c_char_p, ctypes.POINTER(_c_double),
                                  ctypes.POINTER(ctypes.c_longlong)]),
    ("dfcsr_timing_reset", None, []),
    ("dfcsr_moments_workspace_bytes", _c_size, [_c_i64]),
    ("dfcsr_beam_moments", _c_int, [_p, _p, _c_i64, _p, _p, _c_size, _p]),
    ("dfcsr_deposit_workspace_bytes", _c_size, [_c_i64, _c_int, _c_int]),
    ("dfcsr_deposit_cic2d", _c_int, [_p, _p, _p, _p, _c_i64, _c_int, _c_double, _c_double,
                                      _c_int, _c_double, _c_double, _p, _p, _p, _c_size, _p]),
    ("dfcsr_deposit_cic2d_moments", _c_int, [_p, _p, _p, _p, _c_i64, _c_int, _c_int, _p,
                                              _c_double, _c_double, _p, _p, _p, _c_size, _p]),
    ("dfcsr_deposit_noalloc_max_bytes", _c_size, []),
    ("dfcsr_deposit_cic2d_noalloc", _c_int, [_p, _p, _p, _p, _c_i64, _c_int, _c_double, _c_double,
                                              _c_int, _c_double, _c_double, _p, _p, _p]),
    ("dfcsr_df_workspace_bytes", _c_size, [_c_int, _c_int]),
    ("dfcsr_df_axis_tables", _c_int, [_c_double, _c_double, _c_int, _c_double, _c_double, _c_int,
                                       _c_int, _c_int, _p, _p, _p, _p, _p]),
    ("dfcsr_df_finalize", _c_int, [ctypes.POINTER(DFParams), _p, _p, _p, _p, _p, _p, _p,
                                    _c_size, _p]),
    ("dfcsr_grid_barrier_check", _c_int, [_c_int, _c_int, ctypes.c_uint, _p, _c_size, _p]),
    ("dfcsr_history_regrid", _c_int, [_p, _p, _p, _p, _p, _c_int, _c_int, _p, _p, _p, _c_int,
                                       _p, _p, _p, _c_int, _p, _p, _p, _p]),
    ("dfcsr_rgi_axis_linspace", _c_int, [_c_double, _c_double, _c_int, _c_double, _c_double,
                                          _c_int, _p, _p, _p, _p]),
    ("dfcsr_interp3d", _c_int, [_p, _p, _p, _c_i64, _p, _c_int, _c_int, _c_int, _c_double,
                                 _c_double, _c_double, _c_double, _c_double, _c_double, _p, _p]),
    ("dfcsr_interp1d", _c_int, [_p, _c_i64, _p, _c_int, _c_double, _c_double, _p, _p]),
    ("dfcsr_wake_fp64", _c_int, [_p, _p, _p, _p, _c_i64, _c_int, _p, _p, _p]),
    ("dfcsr_wake_integrand", _c_int, [_p, _c_double, _c_double, _p, _p, _c_i64, _c_int, _p, _p,
                                       _p]),
    ("dfcsr_wake_workspace_bytes", _c_size, [_c_int, _c_int, _c_i64]),
    ("dfcsr_wake_mixed", _c_int, [_p, _p, _p, _p, _c_i64, _c_int, _c_int, _c_int, _p, _p, _p,
                                   _c_size, _p]),
    ("dfcsr_wake_mixed_job", _c_int, [ctypes.POINTER(WakeJob), _p, _p, _c_i64, _c_int, _c_int,
                                       _c_int, _p, _p, _p, _c_size, _p]),
    ("dfcsr_csr_mesh", _c_int, [_c_double, _c_double, _c_int, _c_double, _c_double, _c_int,
                                 _c_double, _c_double, _c_double, _p, _p, _p]),
    ("dfcsr_transport6", _c_int, [_p, _p, _c_i64, _c_i64, _p]),
    ("dfcsr_probe_fma", _c_int, [_c_int, _c_i64, _p, ctypes.POINTER(_c_double), _p]),
    ("dfcsr_apply_wakes_workspace_bytes", _c_size, [_c_int, _c_int]),
    ("dfcsr_apply_wakes", _c_int, [_p, _c_i64, _c_i64, _p, _p, _p, _p, _c_int, _c_int, _c_double,
                                    _c_double, _c_double, _c_double, _c_int, _p, _c_size, _p]),
]

EXPORTS = [n for n, _, _ in _SIGS]

_lib = None
_lock = threading.Lock()


def checked_requested():
    """Whether this process loads the bounds-checked library
    (DFCSR_GB300_CHECKED=1 in the environment)."""
    return os.environ.get("DFCSR_GB300_CHECKED", "") == "1"


def library_path():
    return _build.lib_path(checked_requested())


def load(build_if_needed=True):
    """Load (building first if the sources are newer) and return the CDLL:
    the release library, or the bounds-checked one when
    DFCSR_GB300_CHECKED=1."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        checked = checked_requested()
        path = _build.lib_path(checked)
        if build_if_needed and not _build.up_to_date(checked):
            _build.build(checked=checked)
        if not os.path.exists(path):
            raise ImportError(f"dfcsr_gb300 native library not found at {path}; run "
                              "`python -m pydfcsr_gb300.build` (needs nvcc for sm_103a)")
        lib = ctypes.CDLL(path)
        for name, res, args in _SIGS:
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.dfcsr_abi_sizeof(0) != ctypes.sizeof(DFParams):
            raise ImportError("dfcsr_df_params layout mismatch between binding and library")
        if lib.dfcsr_abi_sizeof(1) != ctypes.sizeof(WakeJob):
            raise ImportError("dfcsr_wake_job layout mismatch between binding and library")
        _lib = lib
        return lib


def call(name, *args):
    """Call an entry point and raise the matching exception on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        msg = lib.dfcsr_last_error().decode(errors="replace")
        raise _EXC.get(st, DfcsrError)(st, name, msg)
    return st


def query(name, *args):
    """Call a size / info function (no status)."""
    return getattr(load(), name)(*args)


def bounds_status(reset=False):
    """First index-check failure recorded by the bounds-checked library, as
    (site, index), or None (always None in the release library).  Waits for
    the device in the checked library."""
    v = ctypes.c_ulonglong(0)
    call("dfcsr_bounds_status", ctypes.byref(v), 1 if reset else 0)
    if not v.value:
        return None
    idx = v.value & 0xFFFFFFFFFFFF
    if idx >= 1 << 47:
        idx -= 1 << 48
    return (v.value >> 48) & 0x7FFF, idx


def kernel_launches():
    """Kernel launches issued by the library so far in this process."""
    return int(load().dfcsr_kernel_launches())


def timing_enable(on=True):
    load().dfcsr_timing_enable(1 if on else 0)


def timing_reset():
    load().dfcsr_timing_reset()


def timing_read(name):
    """(total_ms, launches) of a kernel since the last reset (collects first)."""
    lib = load()
    lib.dfcsr_timing_collect()
    ms, n = ctypes.c_double(), ctypes.c_longlong()
    lib.dfcsr_timing_get(name.encode(), ctypes.byref(ms), ctypes.byref(n))
    return ms.value, n.value
