"""Parameter sweeps: many independent solves through one xpfc_batch.

The sweep workload: n instances with grid N drawn from {48, 64, 96, 128}
(cubes, dx = 0.125), mean density n0 from U[0, 0.08], Debye-Waller width sigma
from U[0.28, 0.35], the single-peak or the two-peak fcc kernel with
probability 1/2 each, eta = 2, chi = 1, dt = 1, diagnostics every 100 steps,
FP32 bulk with FP64 k = 0 and sums; instance i has initial-field seed i.
Draws come from numpy's PCG64 seeded with `seed`, so a sweep is reproducible.

sigma starts at 0.28 because with dt = 1 at dx = 0.125 the explicit nonlinear
term of the scheme (euler_step.cu:50-59) diverges once the liquid at n0 = 0.08
crystallises, which it does for sigma below about 0.27.
"""
import math
import time

import numpy as np

from . import _lib
from .api import Batch, Xpfc, build_initial_field, default_params

SIZES = (48, 64, 96, 128)
DX = 0.125
SINGLE = ((2 * math.pi, 1.0, 1.0, 8.0),)
FCC = ((2 * math.pi, 1.0, 1.0, 8.0), (2 * math.pi * 2 / math.sqrt(3), 1.0, 1.0, 6.0))


def sweep_params(n=64, seed=0, sizes=SIZES, precision=_lib.MIXED, sigma=(0.28, 0.35), n0=(0.0, 0.08),
                 t_sample=100, device=0):
    """The n instance parameter sets of a sweep (list of xpfc_params)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        N = int(sizes[rng.integers(len(sizes))])
        psi0 = float(rng.uniform(*n0))
        sg = float(rng.uniform(*sigma))
        peaks = FCC if rng.random() < 0.5 else SINGLE
        L = N * DX
        out.append(default_params(Mx=N, My=N, Mz=N, Lx=L, Ly=L, Lz=L, psi0=psi0, sigma=sg, peaks=peaks,
                                  envelope=_lib.ENVELOPE_MAX, a=1.0, b=1.0 / 3.0, eps=0.0, Mo=1.0, dt=1.0,
                                  t_sample=t_sample, precision=precision, ic_kind=_lib.IC_NOISE, ic_amp=0.1,
                                  ic_seed=i, noise_amp=0.0, ff_factor=DX ** 3, ref_compat=0, device=device))
    return out


def points(params):
    return sum(p.Mx * p.My * p.Mz for p in params)


def solve_batch(params, fields, steps):
    """create -> initialize(host fields) -> step -> diagnostics -> fields ->
    destroy, all instances together.  Returns (fields, diagnostics, groups)."""
    with Batch(params) as b:
        b.initialize(fields)
        b.step(steps)
        diags = [b.collect(i) for i in range(len(params))]
        outs = [b.get_field(i) for i in range(len(params))]
        return outs, diags, b.groups


def solve_sequential(params, fields, steps):
    """The same solves one after another, one xpfc_ctx each."""
    outs, diags = [], []
    for p, f in zip(params, fields):
        with Xpfc(p) as x:
            x.initialize(f)
            diags.append(x.step(steps))
            outs.append(x.copy2cpu())
    return outs, diags


def timed(fn, *a):
    t0 = time.perf_counter()
    r = fn(*a)
    return time.perf_counter() - t0, r


def initial_fields(params):
    return [build_initial_field(p) for p in params]
