"""GPU parity: the staged entry points and the fused step against the oracle
and the reference's golden vectors."""
import json
import math
import os

import numpy as np
import pytest

from helpers import FCC_PEAKS, SINGLE_PEAK, oracle_params, rel_l2

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _golden_params(X, name, tmp_path):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    (tmp_path / "pfc.input").write_text(bytes(z["deck"]).decode())
    if "vtk_in" in z.files:
        from tests_vtk import write_restart
        write_restart(tmp_path / "initial_density_field.vtk", z["vtk_in"], 64, 64, 0.125)
    p = X.read_input(str(tmp_path / "pfc.input"))
    return z, p


@pytest.mark.parametrize("name", ["tri32_gauss", "sq32_circle", "vtk64_restart"])
def test_staged_loop_matches_reference_golden(name, tmp_path):
    """main.cu's loop through the per-stage entry points, reference semantics
    (float powf powers), against the reference's own kernels."""
    import xpfc_cuda_gb300 as X
    z, p = _golden_params(X, name, tmp_path)
    meta = json.loads(bytes(z["params"]).decode())
    assert p.nsteps == math.ceil(meta["N_t_steps"])
    assert abs(p.ff_factor - meta["ff_factor"]) < 1e-15
    with X.Xpfc(p) as x:
        x.initialize(z["psi0"])
        F, R = X.run_reference_loop(x, p.nsteps, p.t_sample)
        final = x.download(X._lib.BUF_PSI_NP1_R)
    # Reference semantics compute n^2, n^3, n^4 with float powf
    # (power_functions.cu:47).  The golden run used the host's powf, this run
    # the device's; they differ by an ulp on some points, which moves F by up
    # to ~1e-5 relative where F cancels strongly (sq32_circle: F drops from 0.61
    # to 0.011) and the residual RMS (which cancels to ~1e-7 of the field) by
    # up to ~1e-2.  The reference prints F with 10 decimals and the RMS with 6
    # digits (sum_reduction.cu:64,77).  Exact-power parity is tested below.
    # sq32_circle is the strongly nonlinear square-lattice deck: F swings
    # between 0.6 and -0.6 and the amplitude reaches ~3, so the ulp-level
    # differences grow with the iterations; it is compared over its first
    # 25 iterations only.
    horizon = 25 if name == "sq32_circle" else p.nsteps
    ftol = 2e-4 if name == "sq32_circle" else 2e-5
    for it, v in z["F"]:
        if it <= horizon:
            assert abs(F[int(it)] - v) <= ftol * abs(v), (it, F[int(it)], v)
    for it, v in z["RMS"]:
        if it <= horizon:
            assert abs(R[int(it)] - v) <= 2e-2 * abs(v), (it, R[int(it)], v)
    if horizon == p.nsteps:
        assert abs(F[p.nsteps] - z["FINAL"][0][1]) <= ftol * abs(z["FINAL"][0][1])
        assert rel_l2(final, z["psi_final"]) < 10 * ftol


# The parameter sets of the 64^3/128^3/256^3 cases as written (sigma 0.1/0.12)
# diverge under the reference's own scheme (the oracle, bit-exact with the
# reference kernels, blows up within 20 steps at any dt down to 0.01): the
# explicit nonlinear term makes the high-k map unstable once the growing
# crystal drives n below about -0.41.  The tests keep dx = 0.125, the kernels,
# the noise and dt, and use sigma above that threshold: 0.25 (single peak:
# relaxation of the initial noise) and 0.22 (fcc: noise-driven liquid).
DX = 0.125


def _setup(X, O, shape, L, steps, ts, precision, peaks=SINGLE_PEAK, noise=0.0, psi0=0.05, amp=0.1, sigma=0.25,
           seed=1):
    Mx, My, Mz = shape
    Lx, Ly, Lz = Mx * DX, My * DX, (Mz * DX if Mz > 1 else 1.0)
    vol = DX ** 3 if Mz > 1 else DX ** 2
    p = X.default_params(Mx=Mx, My=My, Mz=Mz, Lx=Lx, Ly=Ly, Lz=Lz, nsteps=steps, t_sample=ts, precision=precision,
                         ic_kind=X._lib.IC_NOISE, ic_amp=amp, ic_seed=seed, psi0=psi0, sigma=sigma, peaks=peaks,
                         envelope=X._lib.ENVELOPE_MAX, ff_factor=vol, noise_amp=noise, noise_seed=7)
    return p, X.build_initial_field(p)


@pytest.mark.parametrize("shape,steps", [((32, 32, 1), 200), ((64, 64, 1), 100), ((16, 16, 16), 100),
                                         ((32, 32, 32), 60), ((24, 48, 32), 40)])
def test_fused_fp64_matches_oracle(oracle_mod, shape, steps):
    import xpfc_cuda_gb300 as X
    p, psi0 = _setup(X, oracle_mod, shape, 8.0, steps, 20, X._lib.FP64)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(steps)
        field = x.copy2cpu()
    ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, steps, 20)
    assert rel_l2(field, ref) < 1e-10
    for r in recs:
        i = r["iteration"]
        if r["F"] is not None:
            assert abs(r["F"] - F[i]) <= 1e-12 * abs(F[i]), (i, r["F"], F[i])
            assert abs(r["mean"] - mean[i]) <= 1e-13
        if r["rms"] is not None:
            assert abs(r["rms"] - rms[i]) <= 1e-8 * abs(rms[i]) + 1e-14, (i, r["rms"], rms[i])


@pytest.mark.parametrize("shape,steps", [((4096, 4096, 1), 3), ((2048, 512, 1), 6), ((512, 16, 16), 10),
                                         ((16, 512, 32), 10)])
def test_fused_fp64_large_2d_matches_oracle(oracle_mod, shape, steps):
    """Large 2-D FP64 grids, whose pencils are one column wide in shared
    memory (4096) or two (2048)."""
    import xpfc_cuda_gb300 as X
    p, psi0 = _setup(X, oracle_mod, shape, 8.0, steps, 3, X._lib.FP64, noise=0.01)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(steps)
        field = x.copy2cpu()
    ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, steps, 3)
    assert rel_l2(field, ref) < 1e-10
    for r in recs:
        if r["F"] is not None:
            assert abs(r["F"] - F[r["iteration"]]) <= 1e-12 * abs(F[r["iteration"]])


def test_staged_fp64_matches_oracle(oracle_mod):
    import xpfc_cuda_gb300 as X
    p, psi0 = _setup(X, oracle_mod, (32, 32, 1), 8.0, 50, 10, X._lib.FP64)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        F, R = X.run_reference_loop(x, 50, 10)
        final = x.download(X._lib.BUF_PSI_NP1_R)
    ref, Fo, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, 50, 10)
    assert rel_l2(final, ref) < 1e-11
    for i, v in F.items():
        assert abs(v - Fo[i]) <= 1e-12 * abs(Fo[i])
    for i, v in R.items():
        assert abs(v - rms[i]) <= 1e-9 * abs(rms[i])


@pytest.mark.parametrize("shape,steps,fcc", [((64, 64, 64), 300, False), ((128, 128, 1), 300, False),
                                             ((64, 64, 64), 200, True)])
def test_fused_mixed_within_tolerance(oracle_mod, shape, steps, fcc):
    """FP32 bulk, FP64 k = 0 and sums: F rel <= 1e-6, field rel-L2 <= 1e-5."""
    import xpfc_cuda_gb300 as X
    if fcc:
        p, psi0 = _setup(X, oracle_mod, shape, 8.0, steps, 100, X._lib.MIXED, peaks=FCC_PEAKS, noise=0.01,
                         psi0=0.04, amp=0.05, sigma=0.22)
    else:
        p, psi0 = _setup(X, oracle_mod, shape, 8.0, steps, 100, X._lib.MIXED)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(steps)
        field = x.copy2cpu()
    ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, steps, 100)
    assert rel_l2(field, ref) <= 1e-5
    for r in recs:
        i = r["iteration"]
        if r["F"] is not None:
            assert abs(r["F"] - F[i]) <= 1e-6 * abs(F[i]), (i, r["F"], F[i])
            assert abs(r["mean"] - mean[i]) <= 1e-9


@pytest.mark.parametrize("shape,steps", [((48, 48, 48), 60), ((96, 96, 96), 30), ((192, 192, 1), 60),
                                         ((48, 96, 192), 20), ((512, 512, 1), 30), ((1024, 1024, 1), 20),
                                         ((256, 2048, 1), 10), ((512, 16, 16), 20), ((16, 512, 32), 20),
                                         ((512, 64, 1), 30), ((4096, 4096, 1), 3)])
def test_fused_mixed_radix3_sizes(oracle_mod, shape, steps):
    """The 12- and 24-point register plans (48, 96, 192) and the large 2-D
    grids on the mixed path, with conserved noise, against the FP64 oracle."""
    import xpfc_cuda_gb300 as X
    p, psi0 = _setup(X, oracle_mod, shape, 8.0, steps, 10, X._lib.MIXED, peaks=FCC_PEAKS, noise=0.01, psi0=0.04,
                     amp=0.05, sigma=0.22)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(steps)
        field = x.copy2cpu()
    ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, steps, 10)
    assert rel_l2(field, ref) <= 1e-5
    for r in recs:
        i = r["iteration"]
        if r["F"] is not None:
            assert abs(r["F"] - F[i]) <= 1e-6 * abs(F[i]), (i, r["F"], F[i])


def test_fused_noise_fp64_matches_oracle(oracle_mod):
    import xpfc_cuda_gb300 as X
    p, psi0 = _setup(X, oracle_mod, (32, 32, 32), 8.0, 20, 10, X._lib.FP64, peaks=FCC_PEAKS, noise=0.01,
                     psi0=0.04, amp=0.05, sigma=0.22)
    with X.Xpfc(p) as x:
        x.initialize(psi0)
        recs = x.step(20)
        field = x.copy2cpu()
    ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), psi0, 20, 10)
    assert rel_l2(field, ref) < 1e-9
    assert abs(np.mean(field) - 0.04) < 1e-12


def test_uniform_field_stays_uniform():
    import xpfc_cuda_gb300 as X
    for prec in (X._lib.FP64, X._lib.MIXED):
        p = X.default_params(Mx=32, My=32, Mz=32, precision=prec, psi0=0.07, t_sample=10)
        with X.Xpfc(p) as x:
            x.initialize(np.full(32 ** 3, 0.07))
            recs = x.step(30)
            f = x.copy2cpu()
        assert np.ptp(f) < (1e-15 if prec == X._lib.FP64 else 1e-7)
        Fs = [r["F"] for r in recs if r["F"] is not None]
        assert max(Fs) - min(Fs) <= 1e-12 * abs(Fs[0])
