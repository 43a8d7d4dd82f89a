"""ctypes view of the CPU oracle (test infrastructure, not product code).

Only tests/, __graft_entry__.smoke() and bench.py's CPU legs import this.
"""
import ctypes as C
import math
import os

import numpy as np

from . import build_oracle

MAXPEAKS = 8


class OxParams(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("Lx", C.c_double), ("Ly", C.c_double), ("Lz", C.c_double),
        ("a", C.c_double), ("b", C.c_double),
        ("eps", C.c_double), ("Mo", C.c_double), ("dt", C.c_double),
        ("sigma", C.c_double),
        ("npeaks", C.c_int),
        ("pk_k", C.c_double * MAXPEAKS), ("pk_alpha", C.c_double * MAXPEAKS),
        ("pk_rho", C.c_double * MAXPEAKS), ("pk_beta", C.c_double * MAXPEAKS),
        ("envelope", C.c_int),
        ("ref_compat", C.c_int),
        ("ff_factor", C.c_double),
        ("noise_amp", C.c_double),
        ("noise_seed", C.c_uint64),
    ]


class OxDiag(C.Structure):
    _fields_ = [("F", C.c_double), ("mean", C.c_double), ("rms", C.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        dp = C.POINTER(C.c_double)
        L.ox_fft3.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int]
        L.ox_fft_freq.argtypes = [C.c_int, C.c_double, dp]
        L.ox_c2.argtypes = [C.POINTER(OxParams), C.c_double]
        L.ox_c2.restype = C.c_double
        L.ox_k2_c2.argtypes = [C.POINTER(OxParams), dp, dp]
        L.ox_power.argtypes = [C.POINTER(OxParams), dp, dp, C.c_int, C.c_long]
        L.ox_euler_step.argtypes = [C.POINTER(OxParams), dp, dp, dp, dp, dp, dp]
        L.ox_convolve_fields.argtypes = [C.POINTER(OxParams), dp, dp, dp]
        L.ox_FE_calc.argtypes = [C.POINTER(OxParams), dp, dp, dp, dp, dp]
        L.ox_FE_calc.restype = C.c_double
        L.ox_sse_calculation.argtypes = [C.POINTER(OxParams), dp, dp, dp, dp, dp, dp]
        L.ox_sse_calculation.restype = C.c_double
        L.ox_mean.argtypes = [dp, C.c_long]
        L.ox_mean.restype = C.c_double
        L.ox_pin_mean.argtypes = [dp, C.c_long, C.c_double]
        L.ox_noise_k.argtypes = [C.POINTER(OxParams), C.c_long, dp]
        L.ox_run.argtypes = [C.POINTER(OxParams), dp, C.c_long, C.c_int, C.POINTER(OxDiag)]
        L.ox_run.restype = C.c_int
        L.ox_bench.argtypes = [C.POINTER(OxParams), dp, C.c_long, dp]
        L.ox_bench.restype = C.c_int
        L.ox_threads.restype = C.c_int
        L.ox_philox4x32.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.ox_gauss_pair.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, dp, dp]
        L.ox_ic_noise.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_uint64]
        L.ox_ic_fcc_seed.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_double]
        L.ox_ic_reference.argtypes = [dp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int,
                                      C.c_double, C.c_double, C.c_double, C.c_int, C.c_int,
                                      C.c_double, C.c_double, C.c_double]
        L.ox_ic_reference.restype = C.c_double
        _lib = L
    return _lib


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def make_params(nx, ny, nz=1, L=(8.0, 8.0, 8.0), a=1.0, b=1.0 / 3.0, eps=0.0, Mo=1.0, dt=1.0,
                sigma=0.1, peaks=((2 * math.pi, 1.0, 1.0, 8.0),), envelope=1, ref_compat=0,
                ff_factor=None, noise_amp=0.0, noise_seed=0):
    p = OxParams()
    p.nx, p.ny, p.nz = nx, ny, nz
    p.Lx, p.Ly, p.Lz = L
    p.a, p.b, p.eps, p.Mo, p.dt, p.sigma = a, b, eps, Mo, dt, sigma
    p.npeaks = len(peaks)
    for i, (k, al, rho, beta) in enumerate(peaks):
        p.pk_k[i], p.pk_alpha[i], p.pk_rho[i], p.pk_beta[i] = k, al, rho, beta
    p.envelope = envelope
    p.ref_compat = ref_compat
    if ff_factor is None:
        ff_factor = (L[0] / nx) * (L[1] / ny) * ((L[2] / nz) if nz > 1 else 1.0)
    p.ff_factor = ff_factor
    p.noise_amp = noise_amp
    p.noise_seed = noise_seed
    return p


def fft3(x, sign):
    """Unnormalised complex FFT over all axes of a C-order [nz][ny][nx] array."""
    a = np.ascontiguousarray(x, dtype=np.complex128).copy()
    shp = a.shape
    while len(shp) < 3:
        shp = (1,) + shp
    v = a.view(np.float64)
    lib().ox_fft3(_dp(v), shp[2], shp[1], shp[0], sign)
    return a


def k2_c2(p):
    n = p.nx * p.ny * p.nz
    k2 = np.empty(n)
    c2 = np.empty(n)
    lib().ox_k2_c2(C.byref(p), _dp(k2), _dp(c2))
    return k2, c2


def run(p, psi, nsteps, t_sample):
    psi = np.ascontiguousarray(psi, dtype=np.float64).copy()
    diag = (OxDiag * (nsteps + 1))()
    rc = lib().ox_run(C.byref(p), _dp(psi.reshape(-1)), nsteps, t_sample, diag)
    if rc != 0:
        raise RuntimeError("ox_run failed")
    F = np.array([d.F for d in diag])
    mean = np.array([d.mean for d in diag])
    rms = np.array([d.rms for d in diag])
    return psi, F, mean, rms


def bench(p, psi, nsteps):
    """Wall-clock seconds of nsteps oracle steps (no diagnostics)."""
    psi = np.ascontiguousarray(psi, dtype=np.float64).copy()
    sec = C.c_double()
    if lib().ox_bench(C.byref(p), _dp(psi.reshape(-1)), nsteps, C.byref(sec)) != 0:
        raise RuntimeError("ox_bench failed")
    return sec.value, psi


def threads():
    return lib().ox_threads()


def ic_noise(nx, ny, nz, n0, amp, seed):
    psi = np.empty(nx * ny * nz)
    lib().ox_ic_noise(_dp(psi), nx, ny, nz, n0, amp, seed)
    return psi


def ic_fcc_seed(psi, nx, ny, nz, L, n0, amp, radius):
    lib().ox_ic_fcc_seed(_dp(psi), nx, ny, nz, L[0], L[1], L[2], n0, amp, radius)
    return psi


def pin_mean(psi, psi0):
    lib().ox_pin_mean(_dp(psi), psi.size, psi0)
    return psi


def mean(psi):
    return lib().ox_mean(_dp(psi), psi.size)


def ic_reference(Mx, My, Lx, Ly, psi0, iconfig, A_10=0.0, A_11=0.0, A_tri=0.0, iseed=0, ishape=0,
                 h=0.0, k=0.0, roa=0.0):
    psi = np.empty(Mx * My)
    lib().ox_ic_reference(_dp(psi), Mx, My, Lx, Ly, psi0, iconfig, A_10, A_11, A_tri, iseed, ishape,
                          h, k, roa)
    return psi


def noise_k(p, step):
    out = np.empty(2 * p.nx * p.ny * p.nz)
    lib().ox_noise_k(C.byref(p), step, _dp(out))
    return out.view(np.complex128)


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().ox_philox4x32(c, k, o)
    return list(o)


def stage(name):
    return getattr(lib(), name)
