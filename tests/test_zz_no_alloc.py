"""The no-allocation deposit entry point, called through the C ABI.

dfcsr_deposit_cic2d_noalloc serves callers that cannot allocate device memory
when they deposit (host codes that plan every device buffer up front and
forbid allocation in their step loop, plugin hosts whose memory is owned by
their own pool): its scratch is a fixed file-scope device array.  These tests
check it against the workspace-taking entry point, dfcsr_deposit_cic2d, on two
calls in a row with different sizes (the second call must not see the first
call's scratch), and that oversize requests are refused.  The file is named
so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

from pydfcsr_gb300 import _lib
from pydfcsr_gb300.deposit import deposit_cic

pytestmark = pytest.mark.gpu

cuda = pytest.mark.skipif(not torch.cuda.is_available(), reason="needs a CUDA GPU")


def _noalloc(x, z, w0, w1, nb1, s1, e1, nb2, s2, e2):
    out0 = torch.empty((nb1, nb2), dtype=torch.float64, device="cuda")
    out1 = torch.empty((nb1, nb2), dtype=torch.float64, device="cuda")
    p = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None
    _lib.call("dfcsr_deposit_cic2d_noalloc", p(x), p(z), p(w0), p(w1), x.numel(), nb1, s1, e1, nb2,
              s2, e2, p(out0), p(out1), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    return out0, out1


def _case(n, nb1, nb2, seed):
    rng = np.random.default_rng(seed)
    x = torch.from_numpy(rng.normal(0, 1e-5, n)).cuda()
    z = torch.from_numpy(rng.normal(0, 2e-5, n)).cuda()
    w = torch.from_numpy(rng.normal(0, 1e-5, n)).cuda()
    return x, z, w, (nb1, -5e-5, 5e-5, nb2, -1e-4, 1e-4)


def _maxrel(a, b):
    a, b = a.cpu().numpy(), b.cpu().numpy()
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / s) if s > 0 else float(np.max(np.abs(a - b)))


@cuda
def test_noalloc_matches_workspace_entry_two_calls():
    # the stated maximum (2^20 particles on a 256 x 256 grid) fits the array
    lib = _lib.load()
    assert lib.dfcsr_deposit_workspace_bytes(1 << 20, 256, 256) <= lib.dfcsr_deposit_noalloc_max_bytes()
    # first call: the maximum; second call: fewer particles on a different grid
    for n, nb1, nb2, seed in ((1 << 20, 256, 256, 1), (70_000, 40, 200, 2)):
        x, z, w, g = _case(n, nb1, nb2, seed)
        a0, a1 = _noalloc(x, z, None, w, *g)
        b0, b1 = deposit_cic(x, z, None, w, *g)
        torch.cuda.synchronize()
        assert _maxrel(a0, b0) < 1e-12
        assert _maxrel(a1, b1) < 1e-12
        assert float(a0.sum()) > 0.5 * n


@cuda
def test_noalloc_refuses_oversize():
    x, z, w, g = _case(16, 8, 8, 3)
    with pytest.raises(_lib.DfcsrBadArgument, match="no-alloc maximum"):
        _lib.call("dfcsr_deposit_cic2d_noalloc", None, None, None, None, (1 << 20) + 1, 8, 0.0,
                  1.0, 8, 0.0, 1.0, None, None, None)
    with pytest.raises(_lib.DfcsrBadArgument, match="no-alloc maximum"):
        _noalloc(x, z, None, w, 300, g[1], g[2], 300, g[4], g[5])
