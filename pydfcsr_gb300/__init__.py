"""pydfcsr_gb300 - the pyDFCSR_2D per-step CSR wake path on GB300 (sm_103a).

Host code is Python + PyTorch (device memory and streams); every computation
on the path runs in hand-written CUDA kernels of ``libdfcsr_gb300.so`` through
a plain C ABI (``include/dfcsr_gb300.h``).  There is no CPU fallback.

Reference-compatible modules: ``deposit`` (histogram_cic_2d, DF_tracker),
``interp3D`` (interpolate3D), ``interp1D`` (interpolate1D), ``lattice``
(get_referece_traj, Lattice), ``params``, ``CSR`` (CSR2D), ``r_gen6``.
Additions: ``beams`` (GPU beam), ``serve`` (continuous-batching wake server),
``harness`` and ``synthetic`` (seeded workloads).
"""
__version__ = "0.1.0"


def library_path():
    from . import _lib
    return _lib.library_path()
