"""Batched sweeps (xpfc_batch_*): every instance of a batch gets the result it
gets alone, bit for bit, whatever group it lands in; FP64 instances match the
oracle; a diverging instance leaves the others untouched."""
import numpy as np
import pytest

from helpers import FCC_PEAKS, SINGLE_PEAK, oracle_params, rel_l2

pytestmark = pytest.mark.gpu
DX = 0.125


def _params(X, shape, precision, psi0=0.05, sigma=0.25, peaks=SINGLE_PEAK, noise=0.0, seed=1, envelope=None,
            ts=10):
    Mx, My, Mz = shape
    three = Mz > 1
    return X.default_params(Mx=Mx, My=My, Mz=Mz, Lx=Mx * DX, Ly=My * DX, Lz=Mz * DX if three else 1.0,
                            precision=precision, t_sample=ts, ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=seed,
                            psi0=psi0, sigma=sigma, peaks=peaks,
                            envelope=X._lib.ENVELOPE_MAX if envelope is None else envelope,
                            ff_factor=DX ** (3 if three else 2), noise_amp=noise, noise_seed=100 + seed)


def _alone(X, p, field, steps):
    with X.Xpfc(p) as x:
        x.initialize(field)
        recs = x.step(steps)
        return x.copy2cpu(), recs


def test_batch_matches_single_runs_bitwise():
    import xpfc_cuda_gb300 as X
    M, D = X._lib.MIXED, X._lib.FP64
    ps = [
        _params(X, (32, 32, 32), M, 0.04, 0.22, FCC_PEAKS, 0.01, 3),
        _params(X, (48, 48, 48), D, 0.05, 0.25, SINGLE_PEAK, 0.0, 4),
        _params(X, (32, 32, 32), M, 0.06, 0.25, SINGLE_PEAK, 0.01, 5),
        _params(X, (128, 128, 1), M, 0.03, 0.25, SINGLE_PEAK, 0.01, 6),
        _params(X, (128, 128, 128), M, 0.04, 0.22, FCC_PEAKS, 0.01, 7),
        _params(X, (32, 32, 32), M, 0.02, 0.27, SINGLE_PEAK, 0.01, 8, X._lib.ENVELOPE_SUM),
        _params(X, (48, 48, 48), D, 0.03, 0.22, FCC_PEAKS, 0.0, 9),
        _params(X, (128, 128, 1), M, 0.05, 0.22, FCC_PEAKS, 0.01, 10),
        _params(X, (128, 128, 128), M, 0.06, 0.25, SINGLE_PEAK, 0.01, 11),
    ]
    fields = [X.build_initial_field(p) for p in ps]
    steps = 30
    with X.Batch(ps) as b:
        assert b.groups == 4
        assert [b.group_of(i) for i in range(len(ps))] == [0, 1, 0, 2, 3, 0, 1, 2, 3]
        b.initialize(fields)
        b.step(steps)
        got = [(b.get_field(i), b.collect(i)) for i in range(len(ps))]
    for i, p in enumerate(ps):
        f1, r1 = _alone(X, p, fields[i], steps)
        fb, rb = got[i]
        assert np.array_equal(fb, f1), (i, rel_l2(fb, f1))
        assert rb == r1, i


def test_batch_fp64_matches_oracle(oracle_mod):
    import xpfc_cuda_gb300 as X
    ps = [_params(X, (16, 16, 16), X._lib.FP64, 0.04, 0.22, FCC_PEAKS, 0.01, 1),
          _params(X, (16, 16, 16), X._lib.FP64, 0.06, 0.25, SINGLE_PEAK, 0.01, 2),
          _params(X, (16, 16, 16), X._lib.FP64, 0.05, 0.27, SINGLE_PEAK, 0.01, 3, X._lib.ENVELOPE_SUM)]
    fields = [X.build_initial_field(p) for p in ps]
    with X.Batch(ps) as b:
        assert b.groups == 1
        b.initialize(fields)
        b.step(20)
        for i, p in enumerate(ps):
            ref, F, mean, rms = oracle_mod.run(oracle_params(oracle_mod, p), fields[i], 20, 10)
            assert rel_l2(b.get_field(i), ref) < 1e-10, i
            for r in b.collect(i):
                it = r["iteration"]
                if r["F"] is not None:
                    assert abs(r["F"] - F[it]) <= 1e-12 * abs(F[it]), (i, it)
                if r["rms"] is not None:
                    assert abs(r["rms"] - rms[it]) <= 1e-8 * abs(rms[it]) + 1e-14, (i, it)


def test_batch_generated_fields_and_continuation():
    """NULL fields use each instance's generator; two step calls equal one."""
    import xpfc_cuda_gb300 as X
    ps = [_params(X, (32, 32, 32), X._lib.MIXED, 0.03 + 0.01 * k, 0.22 + 0.01 * k, FCC_PEAKS, 0.01, 20 + k)
          for k in range(3)]
    with X.Batch(ps) as b:
        b.initialize(None)
        b.step(12)
        b.step(18)
        got = [b.get_field(i) for i in range(3)]
        last = [b.collect(i) for i in range(3)]
    for i, p in enumerate(ps):
        f1, _ = _alone(X, p, X.build_initial_field(p), 12)
        with X.Xpfc(p) as x:
            x.initialize(None)
            x.step(12)
            r2 = x.step(18)
            f2 = x.copy2cpu()
        assert np.array_equal(got[i], f2), i
        assert last[i] == r2, i


def test_batch_nonfinite_instance_is_isolated():
    import xpfc_cuda_gb300 as X
    ps = [_params(X, (32, 32, 32), X._lib.FP64, 0.05, 0.25, SINGLE_PEAK, 0.0, 1),
          _params(X, (32, 32, 32), X._lib.FP64, 0.05, 0.25, SINGLE_PEAK, 0.0, 2)]
    good = X.build_initial_field(ps[0])
    bad = np.full(32 ** 3, np.nan)
    with X.Batch(ps) as b:
        b.initialize([good, bad])
        b.step(10)
        recs = b.collect(0)
        with pytest.raises(X.XpfcError, match="ENONFINITE"):
            b.collect(1)
        fb = b.get_field(0)
    f1, r1 = _alone(X, ps[0], good, 10)
    assert np.array_equal(fb, f1)
    assert recs == r1
