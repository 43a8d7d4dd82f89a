"""Why the 512^2 reference decks cannot be matched to rounding in float-power
semantics (CPU, oracle only).

The reference takes its powers as powf((float)psi, p) (power_functions.cu:47):
psi is rounded to float first, so the step is discontinuous at every float
rounding boundary.  Two FP64 implementations whose transforms round
differently (about 1e-16) compute the same float power almost everywhere,
but wherever the difference carries a value of psi across a float rounding
boundary their powers differ by a float ulp (about 4e-9 at psi = 0.05); the
next steps spread that difference and it triggers more jumps until the two
trajectories are apart by the float-rounding level.  With exact powers the
same transform differences stay at rounding level.

The test runs the reference's loop (main.cu:306-435: forward transforms of
psi^2 and psi^3, euler_step.cu:50-59, inverse transform, scaling) twice on
the 512^2 noise deck of the GPU fixtures: once in the oracle (its own
transforms) and once with numpy's transforms and the oracle's powers and
tables, so that only the transforms' rounding differs.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as O

N = 512
L = 64.0
SEED = 20261204   # the 512^2 decks' initial field (tests/golden/make_golden_gpu.py)
PEAKS = ((2 * math.pi, 1.0, 1.0, 4.0), (2 * math.pi * math.sqrt(2.0), 1.0, 1.0 / math.sqrt(2.0), 4.0))


def _params(ref_compat):
    # initialize.cu:10-17 (the two-peak sum kernel), s = 0.2, a_in 1, b_in 3
    return O.make_params(N, N, 1, L=(L, L, 1.0), a=1.0, b=1.0 / 3.0, eps=0.0, Mo=1.0, dt=1.0, sigma=0.2,
                         peaks=PEAKS, envelope=0, ref_compat=ref_compat, ff_factor=L * L / (N - 1.0) ** 2)


def _numpy_loop(p, psi0, steps):
    """The reference's step with numpy's real transforms in place of the
    oracle's; powers (ox_power) and k-space tables (ox_k2_c2) from the
    oracle."""
    k2, c2 = O.k2_c2(p)
    h = N // 2 + 1
    k2 = k2.reshape(N, N)[:, :h]
    c2 = c2.reshape(N, N)[:, :h]
    den = 1.0 + k2 * p.dt * p.Mo * (1.0 - p.eps) - k2 * p.Mo * p.dt * c2

    def power(x, pw):
        x = np.ascontiguousarray(x.reshape(-1))
        out = np.empty_like(x)
        O.lib().ox_power(C.byref(p), O._dp(x), O._dp(out), pw, x.size)
        return out.reshape(N, N)

    psi = psi0.reshape(N, N).copy()
    nh = np.fft.rfft2(psi)
    for _ in range(steps):
        p2 = np.fft.rfft2(power(psi, 2))
        p3 = np.fft.rfft2(power(psi, 3))
        nn = (nh + p.a * k2 * p.Mo * p.dt * p2 - p.b * k2 * p.dt * p.Mo * p3) / den
        psi = np.fft.irfft2(nn, s=(N, N))
        nh = np.fft.rfft2(psi)
    return psi.reshape(-1)


def _gap(ref_compat, steps):
    p = _params(ref_compat)
    psi0 = O.pin_mean(0.05 + 0.1 * np.random.default_rng(SEED).standard_normal(N * N), 0.05)
    ours, _, _, _ = O.run(p, psi0, steps, steps)
    other = _numpy_loop(p, psi0, steps)
    return np.linalg.norm(other - ours) / np.linalg.norm(ours)


@pytest.mark.timeout(300)
def test_float_powers_amplify_transform_rounding_at_512():
    # float powers: the two transforms' trajectories end far apart
    # (measured 5.4e-10 after 400 iterations, the size of the library's
    # difference from the reference's GPU run at 512^2)
    assert _gap(1, 400) > 1e-11
    # exact powers: the same transforms stay at rounding level
    assert _gap(0, 400) < 1e-14
