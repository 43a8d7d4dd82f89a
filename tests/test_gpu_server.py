"""The serving loop (xpfc_server_*): every request's field and diagnostics are
bit for bit those of the same solve alone, whatever else runs beside it;
admission keeps the device memory under the budget; failures stay with their
request."""
import numpy as np
import pytest

from helpers import FCC_PEAKS, SINGLE_PEAK

pytestmark = pytest.mark.gpu
DX = 0.125


def _params(X, N, precision, psi0, sigma, peaks, noise, seed, two_d=False, ts=10):
    if two_d:
        return X.default_params(Mx=N, My=N, Mz=1, Lx=N * DX, Ly=N * DX, Lz=1.0, precision=precision, t_sample=ts,
                                ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=seed, psi0=psi0, sigma=sigma,
                                peaks=peaks, envelope=X._lib.ENVELOPE_MAX, ff_factor=DX ** 2, noise_amp=noise,
                                noise_seed=50 + seed)
    return X.default_params(Mx=N, My=N, Mz=N, Lx=N * DX, Ly=N * DX, Lz=N * DX, precision=precision, t_sample=ts,
                            ic_kind=X._lib.IC_NOISE, ic_amp=0.05, ic_seed=seed, psi0=psi0, sigma=sigma, peaks=peaks,
                            envelope=X._lib.ENVELOPE_MAX, ff_factor=DX ** 3, noise_amp=noise, noise_seed=50 + seed)


def _alone(X, p, steps, field=None):
    with X.Xpfc(p) as x:
        x.initialize(field)
        recs = x.step(steps)
        return x.copy2cpu(), recs


def _mix(X):
    M, D = X._lib.MIXED, X._lib.FP64
    return [
        (_params(X, 32, M, 0.04, 0.22, FCC_PEAKS, 0.01, 1), 37),
        (_params(X, 64, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 2), 25),
        (_params(X, 32, D, 0.03, 0.25, SINGLE_PEAK, 0.0, 3), 51),
        (_params(X, 128, M, 0.04, 0.22, FCC_PEAKS, 0.01, 4, two_d=True), 44),
        (_params(X, 48, M, 0.06, 0.28, FCC_PEAKS, 0.0, 5), 30),
        (_params(X, 32, M, 0.02, 0.3, SINGLE_PEAK, 0.01, 6), 19),
        (_params(X, 64, M, 0.04, 0.22, FCC_PEAKS, 0.01, 7), 33),
        (_params(X, 32, D, 0.05, 0.22, FCC_PEAKS, 0.01, 8), 8),
    ]


def test_server_results_equal_single_runs():
    import xpfc_cuda_gb300 as X
    mix = _mix(X)
    given = X.build_initial_field(mix[2][0])
    with X.Server(max_running=4, chunk_steps=5) as s:
        ids = []
        for k, (p, n) in enumerate(mix):
            ids.append(s.submit(p, n, field=given if k == 2 else None, keep_field=True))
        got = []
        for rid, (p, n) in zip(ids, mix):
            s.wait(rid, timeout=120.0)
            got.append(s.result(rid, shape=(p.Mx, p.My, p.Mz)))
            info = s.info(rid)
            assert info["state"] == X._lib.REQ_DONE and info["t_submit"] <= info["t_admit"] <= info["t_done"]
        st = s.stats()
        assert st["done"] == len(mix) and st["failed"] == 0
    for k, ((p, n), (f, recs)) in enumerate(zip(mix, got)):
        f1, r1 = _alone(X, p, n, given if k == 2 else None)
        if not np.array_equal(f, f1):
            # say which side moved: a second solve alone, and where they differ
            f2, _ = _alone(X, p, n, given if k == 2 else None)
            d = np.abs(f - f1).reshape(-1)
            idx = np.flatnonzero(d)
            pytest.fail("request %d: %d of %d values differ (max %.3e, first %s); non-finite: served %d, alone %d; "
                        "a second solve alone equals the first: %s, equals the served one: %s" % (
                            k, idx.size, d.size, float(np.nanmax(d)), idx[:4].tolist(), int((~np.isfinite(f)).sum()),
                            int((~np.isfinite(f1)).sum()), bool(np.array_equal(f1, f2)), bool(np.array_equal(f, f2))))
        assert recs == r1, k


def test_server_budget_and_failures():
    import xpfc_cuda_gb300 as X
    M = X._lib.MIXED
    p64 = _params(X, 64, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 1)
    one = 3 * 4 * 64 ** 3 + 8 * 64 ** 3 + (4 << 20)
    budget = 2 * one + one // 2          # room for two 64^3 solves at a time
    with X.Server(hbm_budget_bytes=budget, max_running=8, chunk_steps=8) as s:
        ids = [s.submit(_params(X, 64, M, 0.05, 0.25, SINGLE_PEAK, 0.01, k), 40) for k in range(6)]
        big = s.submit(_params(X, 128, M, 0.05, 0.25, SINGLE_PEAK, 0.0, 9), 10)
        bad = s.submit(p64, 10, field=np.full(64 ** 3, np.nan))
        for rid in ids:
            s.wait(rid, timeout=120.0)
            assert s.info(rid)["state"] == X._lib.REQ_DONE
        s.wait(big, timeout=120.0)
        with pytest.raises(X.XpfcError, match="ENOMEM"):
            s.result(big)
        s.wait(bad, timeout=120.0)
        with pytest.raises(X.XpfcError, match="ENONFINITE"):
            s.result(bad)
        st = s.stats()
        assert st["peak_bytes_in_use"] <= budget
        assert st["done"] == 7 and st["failed"] == 1
        assert st["contexts_created"] == 2 and st["contexts_reused"] == 5
        f0, r0 = s.result(ids[0])
        assert f0 is None and r0
        s.release(ids[0])
        with pytest.raises(X.XpfcError):
            s.info(ids[0])


def test_server_stop_fails_queued_requests():
    import xpfc_cuda_gb300 as X
    s = X.Server(max_running=1, chunk_steps=4)
    p = _params(X, 64, X._lib.MIXED, 0.05, 0.25, SINGLE_PEAK, 0.01, 1)
    ids = [s.submit(p, 200) for _ in range(4)]
    s.wait(ids[0], timeout=120.0)
    s.close()
