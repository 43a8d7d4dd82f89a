"""Checkpoint/resume of the fused state and the asynchronous field read-back.

The reference restarts only from its 6-digit VTK field (iconfig = 10,
read_input.cu:124-241) and copies the field back synchronously after the loop
(copy_to_cpu.cu:3-18, main.cu:453).  A full-precision snapshot must resume bit
for bit; a read-back started between step calls must return the field of the
iteration it was requested at while later steps run."""
import math

import numpy as np
import pytest

from helpers import FCC_PEAKS

pytestmark = pytest.mark.gpu
DX = 0.125


def _params(X, N, precision, two_d=False):
    L = N * DX
    if two_d:
        return X.default_params(Mx=N, My=N, Mz=1, Lx=L, Ly=L, Lz=1.0, precision=precision, t_sample=10,
                                ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=4, psi0=0.04, sigma=0.22,
                                peaks=FCC_PEAKS, envelope=X._lib.ENVELOPE_MAX, ff_factor=DX ** 2, noise_amp=0.01,
                                noise_seed=9)
    return X.default_params(Mx=N, My=N, Mz=N, Lx=L, Ly=L, Lz=L, precision=precision, t_sample=10,
                            ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=4, psi0=0.04, sigma=0.22, peaks=FCC_PEAKS,
                            envelope=X._lib.ENVELOPE_MAX, ff_factor=DX ** 3, noise_amp=0.01, noise_seed=9)


# 256^3 mixed keeps the pencil-axis spectrum of S, a third array in the snapshot
@pytest.mark.parametrize("N,prec,two_d", [(64, "MIXED", False), (32, "FP64", False), (128, "MIXED", True),
                                          (256, "MIXED", False)])
def test_snapshot_resumes_bit_for_bit(tmp_path, N, prec, two_d):
    import xpfc_cuda_gb300 as X
    p = _params(X, N, getattr(X._lib, prec), two_d)
    with X.Xpfc(p) as x:
        x.initialize(None)
        x.step(17)
        x.save_state(tmp_path / "s.snap")
        r_cont = x.step(23)
        f_cont = x.copy2cpu()
    with X.Xpfc(p) as y:
        y.load_state(tmp_path / "s.snap")
        assert y.iteration == 17
        r_res = y.step(23)
        f_res = y.copy2cpu()
    assert np.array_equal(f_cont, f_res)
    assert r_cont == r_res


def test_snapshot_rejects_another_grid(tmp_path):
    import xpfc_cuda_gb300 as X
    with X.Xpfc(_params(X, 32, X._lib.MIXED)) as x:
        x.initialize(None)
        x.save_state(tmp_path / "s.snap")
    with X.Xpfc(_params(X, 64, X._lib.MIXED)) as y:
        with pytest.raises(X.XpfcError, match="EINVAL"):
            y.load_state(tmp_path / "s.snap")
    (tmp_path / "junk").write_bytes(b"not a snapshot at all" * 4)
    with X.Xpfc(_params(X, 32, X._lib.MIXED)) as z:
        with pytest.raises(X.XpfcError, match="EIO"):
            z.load_state(tmp_path / "junk")


def test_async_readback_overlaps_later_steps():
    import xpfc_cuda_gb300 as X
    p = _params(X, 128, X._lib.MIXED)
    with X.Xpfc(p) as x:
        x.initialize(None)
        x.step(9)
        ref9 = x.copy2cpu()
        x.copy2cpu_async()
        x.step_async(30)           # runs while the copy of iteration 9 proceeds
        f9, it = x.copy2cpu_wait()
        x.collect()
        ref39 = x.copy2cpu()
        x.copy2cpu_async()
        f39, it39 = x.copy2cpu_wait()
    assert it == 9 and np.array_equal(f9, ref9)
    assert it39 == 39 and np.array_equal(f39, ref39)
    assert not np.array_equal(f9, f39)
