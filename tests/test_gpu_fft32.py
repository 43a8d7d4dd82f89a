"""GPU: the FP32 transforms of the mixed-precision step, directly.

The fused step keeps its state as spectra (packed real format: each row of
n0 reals is n0/2 complex values, slot 0 holding X[0] + i X[n0/2]): S is the
row (x) and, in 3-D, column (y) transform of the field, W the same transform
of the nonlinear term N(psi) = -a psi^2 + b psi^3, and at 256-point pencils
Shat is S transformed along the pencil axis as well.  A full-precision
snapshot (xpfc_save_state) holds them as the kernels wrote them, so the
forward transforms are checked against numpy.fft here; the inverse
transforms are checked by round trips: the field read back after
initialisation (inverse xy transforms), and after steps whose update is the
identity (dt = 1e-30 rounds the semi-implicit factors to 1 and 0 in FP32), so
that every pass of the step -- the pencil's forward and inverse transforms,
the inverse column, row and forward column transforms -- runs and must give
the field back.
"""
import math
import struct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# FP32 transforms of length up to 4096: max error relative to the largest
# coefficient (log2 N rounding steps of 6e-8)
TOL = 2e-6
SHAPES_3D = [(48, 48, 48), (64, 64, 64), (96, 96, 96), (128, 128, 128), (192, 64, 128), (256, 256, 256)]
SHAPES_2D = [(512, 512), (1024, 1024), (4096, 4096), (256, 1024)]


def _params(X, Mx, My, Mz, dt=1.0):
    L = (Mx * 0.125, My * 0.125, Mz * 0.125)
    return X.default_params(Mx=Mx, My=My, Mz=Mz, Lx=L[0], Ly=L[1], Lz=L[2], dt=dt, nsteps=1, t_sample=1000,
                            precision=X._lib.MIXED, psi0=0.05, sigma=0.25,
                            peaks=((2 * math.pi, 1.0, 1.0, 8.0),), envelope=X._lib.ENVELOPE_MAX,
                            ff_factor=0.125 ** 3, noise_amp=0.0)


def _read_snapshot(path):
    raw = open(path, "rb").read()
    magic = raw[:8]
    esz, nb, Mx, My, Mz, narr = struct.unpack_from("<6i", raw, 8)
    it, nbytes = struct.unpack_from("<2q", raw, 32)
    assert magic == b"XPFCSNP1" and esz == 4 and nb == 1
    arrs = [np.frombuffer(raw, dtype=np.complex64, count=nbytes // 8, offset=56 + k * nbytes) for k in range(narr)]
    return (Mx, My, Mz), arrs


def _packed(x):
    """numpy's real transform along the last axis in the library's packed
    format: slot 0 = X[0] + i X[n0/2], slots 1 .. n0/2-1 as they are."""
    r = np.fft.rfft(x, axis=-1)
    h = x.shape[-1] // 2
    out = r[..., :h].copy()
    out[..., 0] = r[..., 0] + 1j * r[..., h]
    return out


def _close(got, ref):
    err = np.abs(got.astype(np.complex128) - ref).max() / np.abs(ref).max()
    assert err < TOL, err


@pytest.mark.parametrize("shape", SHAPES_3D + [s + (1,) for s in SHAPES_2D])
def test_fp32_forward_transforms_match_numpy(shape, tmp_path):
    import xpfc_cuda_gb300 as X
    Mx, My, Mz = shape
    p = _params(X, Mx, My, Mz)
    rng = np.random.default_rng(Mx + 3 * My + 7 * Mz)
    psi = 0.05 + 0.1 * rng.standard_normal(Mx * My * Mz)
    psi -= psi.mean() - 0.05
    with X.Xpfc(p) as x:
        x.initialize(psi)
        x.save_state(str(tmp_path / "s.snap"))
        back = x.copy2cpu().reshape(-1)
    (_, _, _), arrs = _read_snapshot(str(tmp_path / "s.snap"))
    # the library works on the field as FP32 ([Mx][My][Mz], last index the
    # real axis; in 2-D [Mx][My])
    f = psi.astype(np.float32).astype(np.float64)
    grid = f.reshape(Mx, My, Mz) if Mz > 1 else f.reshape(Mx, My)
    nl = -p.a * f ** 2 + p.b * f ** 3
    nlg = nl.reshape(grid.shape)
    if Mz > 1:
        S_ref = np.fft.fft(_packed(grid), axis=1)
        W_ref = np.fft.fft(_packed(nlg), axis=1)
    else:
        S_ref = _packed(grid)
        W_ref = _packed(nlg)
    _close(arrs[0].reshape(S_ref.shape), S_ref)
    _close(arrs[1].reshape(W_ref.shape), W_ref)
    if len(arrs) == 3:
        # the kept pencil-axis spectrum (256-point pencils)
        _close(arrs[2].reshape(S_ref.shape), np.fft.fft(S_ref, axis=0))
    # inverse transforms: the read-back is the field itself
    assert np.abs(back - f).max() < 1e-6 * np.abs(f).max() * 10


@pytest.mark.parametrize("shape", [(64, 64, 64), (96, 96, 96), (128, 128, 128), (256, 256, 256), (512, 512, 1),
                                   (4096, 4096, 1)])
def test_fp32_step_transforms_round_trip(shape):
    import xpfc_cuda_gb300 as X
    Mx, My, Mz = shape
    p = _params(X, Mx, My, Mz, dt=1e-30)
    rng = np.random.default_rng(11 + Mx + Mz)
    psi = 0.05 + 0.1 * rng.standard_normal(Mx * My * Mz)
    psi -= psi.mean() - 0.05
    with X.Xpfc(p) as x:
        x.initialize(psi)
        x.step(3)
        back = x.copy2cpu().reshape(-1)
    f = psi.astype(np.float32).astype(np.float64)
    # three round trips through every pass of the step, FP32 rounding only
    assert np.abs(back - f).max() < 3e-6 * np.abs(f).max(), np.abs(back - f).max()
