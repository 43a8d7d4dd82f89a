"""Shared test helpers: map library parameters onto the oracle's."""
import math

import numpy as np


def oracle_params(O, p):
    """Oracle parameters for library params p (same memory layout: the
    library's fastest axis is the oracle's x)."""
    if p.Mz > 1:
        nx, ny, nz, L = p.Mz, p.My, p.Mx, (p.Lz, p.Ly, p.Lx)
    else:
        nx, ny, nz, L = p.My, p.Mx, 1, (p.Ly, p.Lx, 1.0)
    peaks = [(p.pk_k[i], p.pk_alpha[i], p.pk_rho[i], p.pk_beta[i]) for i in range(p.npeaks)]
    return O.make_params(nx, ny, nz, L=L, a=p.a, b=p.b, eps=p.eps, Mo=p.Mo, dt=p.dt, sigma=p.sigma,
                         peaks=peaks, envelope=p.envelope, ref_compat=p.ref_compat, ff_factor=p.ff_factor,
                         noise_amp=p.noise_amp, noise_seed=p.noise_seed)


SINGLE_PEAK = ((2 * math.pi, 1.0, 1.0, 8.0),)
FCC_PEAKS = ((2 * math.pi, 1.0, 1.0, 8.0), (2 * math.pi * 2 / math.sqrt(3), 1.0, 1.0, 6.0))


def rel_l2(a, b):
    a = np.asarray(a).reshape(-1)
    b = np.asarray(b).reshape(-1)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
