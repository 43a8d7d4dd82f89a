"""Host-side workload generators of the sweep and the serving stream: seeded,
reproducible, inside the stated ranges, and the shapes the library accepts."""
import numpy as np


def test_sweep_params_are_reproducible_and_in_range():
    from xpfc_cuda_gb300 import sweep as SW
    a, b = SW.sweep_params(64, seed=3), SW.sweep_params(64, seed=3)
    assert [(p.Mx, p.psi0, p.sigma, p.npeaks) for p in a] == [(p.Mx, p.psi0, p.sigma, p.npeaks) for p in b]
    assert {p.Mx for p in a} <= set(SW.SIZES)
    for i, p in enumerate(a):
        assert p.Mx == p.My == p.Mz and abs(p.Lx - p.Mx * SW.DX) < 1e-12
        assert 0.0 <= p.psi0 <= 0.08 and 0.28 <= p.sigma <= 0.35 and p.npeaks in (1, 2)
        assert p.ic_seed == i and p.t_sample == 100
    assert SW.points(a) == sum(p.Mx ** 3 for p in a)
    assert [p.Mx for p in SW.sweep_params(64, seed=4)] != [p.Mx for p in a]


def test_request_stream_is_poisson_like_and_in_range():
    from xpfc_cuda_gb300 import serving as SV
    st = SV.request_stream(2000, rate=20.0, seed=1)
    t = np.array([a for a, _, _ in st])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 20.0) < 0.005
    sizes = np.array([p.Mx for _, p, _ in st])
    for n, w in zip(SV.SIZES, SV.WEIGHTS):
        assert abs((sizes == n).mean() - w) < 0.04, n
    steps = np.array([k for _, _, k in st])
    assert steps.min() >= 200 and steps.max() <= 5000
    assert [p.Mx for _, p, _ in SV.request_stream(50, seed=1)] == list(sizes[:50])


def test_summary_percentiles():
    from xpfc_cuda_gb300 import serving as SV
    recs = [{"t_submit": 0.0, "t_admit": float(i), "t_done": float(2 * i + 1), "cells": 8, "steps": 10,
             "state": 2} for i in range(100)]
    s = SV.summarise(recs, 200.0, 20.0)
    assert s["requests"] == 100 and s["done"] == 100
    assert abs(s["latency_p50_s"] - np.percentile([2 * i + 1 for i in range(100)], 50)) < 1e-12
    assert abs(s["queue_p99_s"] - np.percentile(range(100), 99)) < 1e-12
    assert abs(s["served_gpt_steps_per_s"] - 100 * 80 / 199.0 / 1e9) < 1e-18
