"""Known-answer tests of the oracle (CPU): its FFT against numpy, Philox
against the published Random123 vectors, and identities of the step."""
import math

import numpy as np
import pytest


@pytest.mark.parametrize("shape", [(8,), (6,), (1, 16, 16), (4, 6, 10), (3, 5, 7), (12, 48, 96), (2, 3, 256)])
def test_fft_matches_numpy(oracle_mod, shape):
    rng = np.random.default_rng(len(shape) + sum(shape))
    x = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    f = oracle_mod.fft3(x, -1)
    assert np.abs(f - np.fft.fftn(x)).max() <= 1e-14 * np.abs(f).max()
    b = oracle_mod.fft3(x, +1)
    assert np.abs(b - np.fft.ifftn(x) * x.size).max() <= 1e-14 * np.abs(b).max()


def test_philox_known_answers(oracle_mod):
    # Random123 kat_vectors, philox4x32 with 10 rounds
    P = oracle_mod.philox
    assert P([0, 0, 0, 0], [0, 0]) == [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]
    assert P([0xffffffff] * 4, [0xffffffff] * 2) == [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]
    assert P([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0]) == \
        [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]


def _field(O, n, nz, seed=2):
    psi = O.ic_noise(n, n, nz, 0.05, 0.1, seed)
    return O.pin_mean(psi, 0.05)


def test_parseval_free_energy(oracle_mod):
    """The nonlocal term 1/2 sum n (C2*n) equals 1/2 (1/N) sum_k c2 |n_k|^2."""
    O = oracle_mod
    n = 16
    p = O.make_params(n, n, n, L=(2.0, 2.0, 2.0), sigma=0.2)
    psi = _field(O, n, n)
    k2, c2 = O.k2_c2(p)
    nk = O.fft3(psi.reshape(n, n, n), -1).reshape(-1)
    conv = O.fft3((c2 * nk).reshape(n, n, n), +1).reshape(-1).real / psi.size
    real_space = 0.5 * np.sum(psi * conv)
    k_space = 0.5 * np.sum(c2 * np.abs(nk) ** 2) / psi.size
    assert abs(real_space - k_space) <= 1e-13 * abs(k_space)


def test_uniform_field_is_a_fixed_point(oracle_mod):
    O = oracle_mod
    p = O.make_params(8, 8, 8, L=(1.0, 1.0, 1.0), sigma=0.2)
    psi = np.full(512, 0.07)
    out, F, mean, rms = O.run(p, psi, 10, 5)
    assert np.ptp(out) < 1e-16 and abs(out.mean() - 0.07) < 1e-16
    assert np.nanmax(F) - np.nanmin(F) < 1e-15
    assert np.nanmax(rms) < 1e-14


def test_linear_growth_of_one_mode(oracle_mod):
    """n = n0 + eps cos(k x): after one step the mode is multiplied by
    (1 - dt Mo k^2 N'(n0)) / (1 + dt Mo k^2 (1 - eps_r - c2(k))),
    N'(n) = -2 a n + 3 b n^2 (euler_step.cu:50-54 linearised)."""
    O = oracle_mod
    n, L, n0, e = 32, 4.0, 0.05, 1e-7
    a, b, dt, Mo, eps_r = 1.0, 1.0 / 3.0, 0.5, 1.0, 0.02
    p = O.make_params(n, n, 1, L=(L, L, 1.0), a=a, b=b, dt=dt, Mo=Mo, eps=eps_r, sigma=0.2)
    m = 5
    x = np.arange(n) * L / n
    psi = (n0 + e * np.cos(2 * math.pi * m * x / L))[None, :].repeat(n, 0).reshape(-1).copy()
    out, F, mean, rms = O.run(p, psi, 1, 0)
    amp = 2 * np.fft.fft2(out.reshape(n, n))[0, m].real / n ** 2
    k = 2 * math.pi * m / L
    c2 = O.lib().ox_c2(p, k)
    Np = -2 * a * n0 + 3 * b * n0 ** 2
    g = (1 - dt * Mo * k * k * Np) / (1 + dt * Mo * k * k * (1 - eps_r - c2))
    assert abs(amp / e - g) < 1e-6 * abs(g)


def test_conserved_noise_is_hermitian_and_mean_free(oracle_mod):
    O = oracle_mod
    n, nz = 16, 12
    p = O.make_params(n, n, nz, L=(2.0, 2.0, 1.5), noise_amp=0.01, noise_seed=9)
    xi = O.noise_k(p, 3).reshape(nz, n, n)
    assert xi[0, 0, 0] == 0
    r = O.fft3(xi, +1)
    assert np.abs(r.imag).max() <= 1e-14 * np.abs(r.real).max()
    k2, _ = O.k2_c2(p)
    var = np.abs(xi.reshape(-1)) ** 2 / (0.01 ** 2 * xi.size * np.maximum(k2, 1e-30))
    assert abs(var[k2 > 0].mean() - 1.0) < 0.05
    assert np.array_equal(O.noise_k(p, 3), O.noise_k(p, 3)) and not np.array_equal(O.noise_k(p, 3), O.noise_k(p, 4))
