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


def _solve_bytes(N, esz, two_d=False):
    """Device bytes the server books for one solve (S, W, read-back, the FP64
    initial field while it is prepared, tables): grids without a kept
    spectrum."""
    cells = N ** 2 if two_d else N ** 3
    return 3 * esz * cells + 8 * cells + (4 << 20)


def _serve_behind_blocker(X, reqs, merge_max, extra_budget=0):
    """Runs reqs [(params, steps, field)] on a server whose budget holds a
    128^3 FP64 blocker alone: the blocker is admitted first and the requests
    queue behind it, so that the groups they can form are formed when it
    finishes.  Returns ([(field, records)], stats)."""
    D = X._lib.FP64
    blocker = _params(X, 128, D, 0.05, 0.25, SINGLE_PEAK, 0.0, 99)
    smallest = min(_solve_bytes(p.Mx, 4 if p.precision == X._lib.MIXED else 8, p.Mz == 1) for p, _, _ in reqs)
    budget = _solve_bytes(128, 8) + smallest - 1 + extra_budget
    with X.Server(hbm_budget_bytes=budget, max_running=16, chunk_steps=5, merge_max=merge_max) as s:
        b = s.submit(blocker, 300)
        ids = [s.submit(p, n, field=f, keep_field=True) for p, n, f in reqs]
        s.wait(b, timeout=120.0)
        out = []
        for rid, (p, n, f) in zip(ids, reqs):
            s.wait(rid, timeout=120.0)
            try:
                out.append(s.result(rid, shape=(p.Mx, p.My, p.Mz)))
            except X.XpfcError as e:
                out.append(e)
        st = s.stats()
    assert st["peak_bytes_in_use"] <= budget
    return out, st


def test_server_merged_groups_equal_single_runs():
    """Queued requests of one grid with step counts within 25 % run as merged
    groups (one launch per pass for all of them); each result is bit for bit
    the solve alone, including solves that end before their group's last
    iteration (final free energy and field taken there) and a caller's field."""
    import xpfc_cuda_gb300 as X
    M, D = X._lib.MIXED, X._lib.FP64
    given = X.build_initial_field(_params(X, 64, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 13))
    reqs = [
        (_params(X, 64, M, 0.04, 0.22, FCC_PEAKS, 0.01, 11), 40, None),
        (_params(X, 64, M, 0.06, 0.28, SINGLE_PEAK, 0.01, 12), 37, None),
        (_params(X, 64, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 13), 34, given),
        (_params(X, 64, M, 0.03, 0.3, FCC_PEAKS, 0.01, 14), 42, None),
        (_params(X, 128, M, 0.04, 0.22, FCC_PEAKS, 0.01, 15, two_d=True), 30, None),
        (_params(X, 128, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 16, two_d=True), 28, None),
        (_params(X, 128, M, 0.02, 0.3, FCC_PEAKS, 0.01, 17, two_d=True), 25, None),
        (_params(X, 32, D, 0.03, 0.25, SINGLE_PEAK, 0.0, 18), 20, None),
        (_params(X, 32, D, 0.05, 0.22, FCC_PEAKS, 0.0, 19), 24, None),
        # step count outside the 64^3 group's band: runs alone
        (_params(X, 64, M, 0.04, 0.25, SINGLE_PEAK, 0.01, 20), 100, None),
    ]
    got, st = _serve_behind_blocker(X, reqs, merge_max=4)
    assert st["merged_groups"] == 3 and st["merged_solves"] == 9, st
    assert st["done"] == len(reqs) + 1 and st["failed"] == 0, st
    for k, ((p, n, f), res) in enumerate(zip(reqs, got)):
        assert not isinstance(res, Exception), (k, res)
        field, recs = res
        f1, r1 = _alone(X, p, n, f)
        assert np.array_equal(field, f1), (k, float(np.nanmax(np.abs(field - f1))))
        assert recs == r1, k
        assert recs[-1]["iteration"] == n and recs[-1]["F"] is not None and recs[-1]["rms"] is None, k


def test_server_merged_group_keeps_failures_local():
    """A non-finite solve in a merged group fails alone (ENONFINITE); its
    group's other solves are the solves alone."""
    import xpfc_cuda_gb300 as X
    M = X._lib.MIXED
    reqs = [
        (_params(X, 32, M, 0.04, 0.22, FCC_PEAKS, 0.01, 21), 30, None),
        (_params(X, 32, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 22), 27, np.full(32 ** 3, np.nan)),
        (_params(X, 32, M, 0.03, 0.3, FCC_PEAKS, 0.01, 23), 33, None),
    ]
    got, st = _serve_behind_blocker(X, reqs, merge_max=8)
    assert st["merged_groups"] == 1 and st["merged_solves"] == 3, st
    assert isinstance(got[1], X.XpfcError) and "ENONFINITE" in str(got[1])
    for k in (0, 2):
        p, n, f = reqs[k]
        f1, r1 = _alone(X, p, n, f)
        assert np.array_equal(got[k][0], f1), k
        assert got[k][1] == r1, k


def test_server_merged_group_context_reused():
    """A finished merged group's context goes to the pool; the next group of
    the same grid and size takes it with new params (box, tables, pinned
    means, seeds) and still gives every solve's results alone."""
    import xpfc_cuda_gb300 as X
    M, D = X._lib.MIXED, X._lib.FP64
    blocker = _params(X, 128, D, 0.05, 0.25, SINGLE_PEAK, 0.0, 99)
    waves = [[(_params(X, 32, M, 0.04, 0.22, FCC_PEAKS, 0.01, 31), 30),
              (_params(X, 32, M, 0.05, 0.25, SINGLE_PEAK, 0.01, 32), 27)],
             [(_params(X, 32, M, 0.02, 0.3, SINGLE_PEAK, 0.01, 33), 26),
              (_params(X, 32, M, 0.06, 0.28, FCC_PEAKS, 0.01, 34), 31)]]
    # the second wave's box differs (dx 0.15): the pooled context keys on the
    # grid, so it must take the new box's k-grid
    for p, _ in waves[1]:
        X.set_params(p, Lx=32 * 0.15, Ly=32 * 0.15, Lz=32 * 0.15, ff_factor=0.15 ** 3)
    # one context in flight (a merged group counts once): each wave queues
    # behind its blocker and forms its group when the blocker finishes
    with X.Server(max_running=1, chunk_steps=5, merge_max=8) as s:
        got = []
        for wave in waves:
            b = s.submit(blocker, 200)
            ids = [s.submit(p, n, keep_field=True) for p, n in wave]
            s.wait(b, timeout=120.0)
            for rid, (p, n) in zip(ids, wave):
                s.wait(rid, timeout=120.0)
                got.append(s.result(rid, shape=(p.Mx, p.My, p.Mz)))
        st = s.stats()
    assert st["merged_groups"] == 2 and st["merged_solves"] == 4, st
    # the blocker's context and the first group's are reused by the second wave
    assert st["contexts_created"] == 2 and st["contexts_reused"] == 2, st
    for (p, n), (f, recs) in zip(waves[0] + waves[1], got):
        f1, r1 = _alone(X, p, n)
        assert np.array_equal(f, f1)
        assert recs == r1
