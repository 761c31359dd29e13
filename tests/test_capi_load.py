"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
header declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

from pydfcsr_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "dfcsr_gb300.h")


def header_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(dfcsr_[a-z0-9_]+)\s*\(", src)))


def test_library_builds_and_loads():
    path = build.build()
    assert os.path.exists(path)
    lib = _lib.load()
    assert lib.dfcsr_version() >= 100


def test_every_header_symbol_exported():
    lib = ctypes.CDLL(build.build())
    names = header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), f"{n} declared in the header but not exported"
    # the binding covers every declared entry point
    assert set(names) <= set(_lib.EXPORTS), set(names) - set(_lib.EXPORTS)


def test_bounds_checked_library_builds_and_exports():
    """The bounds-checked variant builds from the same sources and exports
    the same symbols; it reports itself as checked, the release library not.
    In the release library the status query answers without a device."""
    path = build.build(checked=True)
    assert path != build.build() and os.path.exists(path)
    chk = ctypes.CDLL(path)
    for n in header_functions():
        assert hasattr(chk, n), f"{n} missing from the checked library"
    assert chk.dfcsr_bounds_checked() == 1
    lib = _lib.load()
    assert lib.dfcsr_bounds_checked() == (1 if _lib.checked_requested() else 0)
    if not _lib.checked_requested():
        assert _lib.bounds_status(reset=True) is None   # no device needed
    assert "bounds_status" in dir(_lib)
    with pytest.raises(_lib.DfcsrBadArgument, match="site"):
        _lib.call("dfcsr_bounds_probe", 0, 1, 0, None)


def test_launch_counter_without_gpu():
    """The launch counter is host-side: readable without a device, and an
    argument error launches nothing."""
    n0 = _lib.kernel_launches()
    with pytest.raises(_lib.DfcsrBadArgument):
        _lib.call("dfcsr_csr_mesh", 0.0, 1.0, 0, 0.0, 1.0, 4, 0.0, 0.0, 0.0, None, None, None)
    assert _lib.kernel_launches() == n0


def test_struct_layouts_match():
    lib = _lib.load()
    assert lib.dfcsr_abi_sizeof(0) == ctypes.sizeof(_lib.DFParams)
    assert lib.dfcsr_abi_sizeof(1) == ctypes.sizeof(_lib.WakeJob)
    assert lib.dfcsr_abi_sizeof(7) == 0


def test_status_names_and_sizes():
    lib = _lib.load()
    assert lib.dfcsr_status_name(0) == b"OK"
    assert lib.dfcsr_status_name(6) == b"ADMISSION_REFUSED"
    assert lib.dfcsr_deposit_workspace_bytes(1000, 64, 64) > 4 * 1000
    assert lib.dfcsr_deposit_workspace_bytes(-1, 64, 64) == 0
    assert lib.dfcsr_df_workspace_bytes(64, 64) >= 3 * 64 * 64 * 8   # three scratch fields
    assert lib.dfcsr_wake_workspace_bytes(100, 100, 4096) > 0


def test_noalloc_limits_fit_its_array():
    """The no-alloc deposit's stated maximum (2^20 particles, 256 x 256 grid)
    needs no more scratch than its fixed array holds; grids whose key count
    overflows int are refused, not wrapped."""
    lib = _lib.load()
    assert 0 < lib.dfcsr_deposit_workspace_bytes(1 << 20, 256, 256) <= \
        lib.dfcsr_deposit_noalloc_max_bytes()
    assert lib.dfcsr_deposit_workspace_bytes(1000, 2 ** 31 - 1, 4) == 0
    with pytest.raises(_lib.DfcsrBadArgument, match="no-alloc maximum"):
        _lib.call("dfcsr_deposit_cic2d_noalloc", None, None, None, None, 10, 2 ** 31 - 1, 0.0,
                  1.0, 4, 0.0, 1.0, None, None, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="too large"):
        _lib.call("dfcsr_deposit_cic2d", None, None, None, None, 10, 2 ** 31 - 1, 0.0, 1.0, 4,
                  0.0, 1.0, ctypes.c_void_p(16), None, None, 0, None)


def test_bad_arguments_fail_without_gpu():
    """Argument checks run before any device work, so they are testable here."""
    with pytest.raises(_lib.DfcsrBadArgument):
        _lib.call("dfcsr_deposit_cic2d", None, None, None, None, 10, 0, 0.0, 1.0, 4, 0.0, 1.0,
                  None, None, None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="window_length"):
        p = _lib.DFParams()
        p.nx, p.nz, p.window, p.order = 8, 8, 4, 2
        dummy = ctypes.c_void_p(16)
        _lib.call("dfcsr_df_finalize", ctypes.byref(p), dummy, dummy, dummy, dummy, dummy, dummy,
                  None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument):
        _lib.call("dfcsr_wake_mixed", ctypes.c_void_p(16), None, ctypes.c_void_p(16),
                  ctypes.c_void_p(16), 5, 2000, 100, 0, ctypes.c_void_p(16), ctypes.c_void_p(16),
                  None, 0, None)
    assert "xbins" in _lib.load().dfcsr_last_error().decode()
    job = _lib.WakeJob()
    with pytest.raises(_lib.DfcsrBadArgument, match="xbins"):
        _lib.call("dfcsr_wake_mixed_job", ctypes.byref(job), ctypes.c_void_p(16),
                  ctypes.c_void_p(16), 5, 2000, 100, 0, ctypes.c_void_p(16), ctypes.c_void_p(16),
                  None, 0, None)
    big = _lib.WakeJob()
    big.cap, big.nx, big.nz = 5000, 1000, 1000        # 1e10 float4 of FP32 ring
    with pytest.raises(_lib.DfcsrBadArgument, match="64 GiB"):
        _lib.call("dfcsr_wake_mixed_job", ctypes.byref(big), ctypes.c_void_p(16),
                  ctypes.c_void_p(16), 5, 100, 100, 0, ctypes.c_void_p(16), ctypes.c_void_p(16),
                  None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="null job"):
        _lib.call("dfcsr_wake_mixed_job", None, ctypes.c_void_p(16), ctypes.c_void_p(16), 5, 100,
                  100, 0, ctypes.c_void_p(16), ctypes.c_void_p(16), None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="grids need"):
        _lib.call("dfcsr_df_axis_tables", 0.0, 1.0, 1, 0.0, 1.0, 8, 0, 0, ctypes.c_void_p(16),
                  ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    with pytest.raises(_lib.DfcsrBadArgument, match="longer than"):
        _lib.call("dfcsr_df_axis_tables", 0.0, 1.0, (1 << 24) + 1, 0.0, 1.0, 2**31 - 1, 0, 0,
                  ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16),
                  ctypes.c_void_p(16), None)
    with pytest.raises(_lib.DfcsrBadArgument, match="longer than"):
        _lib.call("dfcsr_rgi_axis_linspace", 0.0, 1.0, 8, 0.0, 1.0, 2**31 - 1,
                  ctypes.c_void_p(16), ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    with pytest.raises(_lib.DfcsrBadArgument, match="moments is null"):
        _lib.call("dfcsr_deposit_cic2d_moments", ctypes.c_void_p(16), ctypes.c_void_p(16), None,
                  None, 10, 8, 8, None, 5.0, 5.0, ctypes.c_void_p(16), None, None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="limits"):
        _lib.call("dfcsr_deposit_cic2d_moments", ctypes.c_void_p(16), ctypes.c_void_p(16), None,
                  None, 10, 8, 8, ctypes.c_void_p(16), 0.0, 5.0, ctypes.c_void_p(16), None, None,
                  0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="zbins"):
        _lib.call("dfcsr_wake_fp64", ctypes.c_void_p(16), None, ctypes.c_void_p(16),
                  ctypes.c_void_p(16), 5, 7000, ctypes.c_void_p(16), ctypes.c_void_p(16), None)
    # an empty wake is a no-op, with or without a job
    _lib.call("dfcsr_wake_mixed_job", None, None, None, 0, 100, 100, 0, None, None, None, 0, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="extra_arrivals"):
        _lib.call("dfcsr_grid_barrier_check", 1, 2, 100, ctypes.c_void_p(16), 16, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="workspace"):
        _lib.call("dfcsr_grid_barrier_check", 1, 0, 100, ctypes.c_void_p(16), 8, None)
