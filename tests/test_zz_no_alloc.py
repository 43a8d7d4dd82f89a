"""GPU: the allocation-free free-energy reduction against xpfc_FE_calc.

xpfc_FE_calc_noalloc serves callers that cannot allocate device memory; it
keeps its partial sums in a fixed array inside the library.  This file is
collected last so that a run stopping at its first failure has already run
every other test; it passes alone in a fresh process as well (the first call
on the device sets the array's address up).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fields(rng, n):
    psi = 0.05 + 0.1 * rng.standard_normal(n)
    return [psi, psi ** 2, psi ** 3, psi ** 4, 0.3 * rng.standard_normal(n)]


def test_fe_noalloc_matches_fe_calc_twice():
    import torch

    import xpfc_cuda_gb300 as X
    L = X.load()
    Mx = My = Mz = 48
    n = Mx * My * Mz
    a, b, ff = 1.0, 1.0 / 3.0, 0.125 ** 3
    p = X.default_params(Mx=Mx, My=My, Mz=Mz, a=a, b=b, ff_factor=ff, precision=X._lib.FP64)
    rng = np.random.default_rng(17)
    bufs = [X._lib.BUF_PSI, X._lib.BUF_PSI2, X._lib.BUF_PSI3, X._lib.BUF_PSI4, X._lib.BUF_CONVL]
    with X.Xpfc(p) as x:
        for call in range(2):
            host = _fields(rng, n)
            for bid, h in zip(bufs, host):
                x.upload(bid, h)
            F_ref = x.FE_calc_wrapper(0, *bufs)
            dev = [torch.tensor(h, dtype=torch.float64, device="cuda") for h in host]
            torch.cuda.synchronize()
            F = C.c_double(float("nan"))
            rc = L.xpfc_FE_calc_noalloc(*[d.data_ptr() for d in dev], n, a, b, ff, C.byref(F),
                                        torch.cuda.current_stream().cuda_stream)
            assert rc == X._lib.OK, L.xpfc_last_error(None)
            assert abs(F.value - F_ref) <= 1e-12 * abs(F_ref), (call, F.value, F_ref)


def test_fe_noalloc_rejects_oversize_and_null():
    """Sizes beyond the fixed scratch and null arrays are refused before any
    launch (the arrays here are real, small device buffers)."""
    import torch

    import xpfc_cuda_gb300 as X
    L = X.load()
    F = C.c_double()
    small = torch.zeros(16, dtype=torch.float64, device="cuda")
    one = C.c_void_p(small.data_ptr())
    rc = L.xpfc_FE_calc_noalloc(one, one, one, one, one, (1 << 28) + 1, 1.0, 1.0, 1.0, C.byref(F), None)
    assert rc == X._lib.EINVAL and b"exceed the maximum" in L.xpfc_last_error(None)
    rc = L.xpfc_FE_calc_noalloc(None, one, one, one, one, 10, 1.0, 1.0, 1.0, C.byref(F), None)
    assert rc == X._lib.EINVAL
    # a valid call on the same buffers still works: 16 zeros sum to zero
    rc = L.xpfc_FE_calc_noalloc(one, one, one, one, one, 16, 1.0, 1.0, 1.0, C.byref(F),
                                torch.cuda.current_stream().cuda_stream)
    assert rc == X._lib.OK and F.value == 0.0
