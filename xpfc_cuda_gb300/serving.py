"""Request streams for the serving loop (xpfc_server) and a driver that plays
one against a server.

The stream: Poisson arrivals at `rate` per second; grid N^3 with N drawn from
(64, 96, 128, 192, 256) with weights (0.3, 0.25, 0.2, 0.15, 0.1); steps from
U[200, 5000]; the physics of the sweep workload (dx = 0.125, n0 in U[0, 0.08],
sigma in U[0.28, 0.35], single-peak or fcc kernel, diagnostics every 100 steps,
FP32 bulk); initial fields from each request's generator on the device.
Draws come from numpy's PCG64 seeded with `seed`.
"""
import math
import threading
import time

import numpy as np

from . import _lib
from .api import default_params

SIZES = (64, 96, 128, 192, 256)
WEIGHTS = (0.3, 0.25, 0.2, 0.15, 0.1)
DX = 0.125
SINGLE = ((2 * math.pi, 1.0, 1.0, 8.0),)
FCC = ((2 * math.pi, 1.0, 1.0, 8.0), (2 * math.pi * 2 / math.sqrt(3), 1.0, 1.0, 6.0))


def request_stream(n, rate=20.0, seed=0, steps=(200, 5000), sizes=SIZES, weights=WEIGHTS, device=0,
                   precision=_lib.MIXED):
    """[(arrival time in s, params, nsteps)] of n requests."""
    rng = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += float(rng.exponential(1.0 / rate))
        N = int(rng.choice(sizes, p=np.asarray(weights) / np.sum(weights)))
        k = int(rng.integers(steps[0], steps[1] + 1))
        psi0 = float(rng.uniform(0.0, 0.08))
        sg = float(rng.uniform(0.28, 0.35))
        peaks = FCC if rng.random() < 0.5 else SINGLE
        L = N * DX
        p = default_params(Mx=N, My=N, Mz=N, Lx=L, Ly=L, Lz=L, psi0=psi0, sigma=sg, peaks=peaks,
                           envelope=_lib.ENVELOPE_MAX, a=1.0, b=1.0 / 3.0, eps=0.0, Mo=1.0, dt=1.0, t_sample=100,
                           precision=precision, ic_kind=_lib.IC_NOISE, ic_amp=0.1, ic_seed=1000 + i,
                           noise_amp=0.0, ff_factor=DX ** 3, ref_compat=0, device=device)
        out.append((t, p, k))
    return out


def play(server, stream, keep=()):
    """Submits each request at its arrival time (from a thread of its own) and
    waits for all; returns per-request dicts with the server's timestamps and
    the makespan (first arrival to last completion, wall clock)."""
    ids = [None] * len(stream)
    t0 = time.perf_counter()

    def submitter():
        for i, (t, p, k) in enumerate(stream):
            d = t - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            ids[i] = server.submit(p, k, keep_field=i in keep)

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    out = []
    for i, (t, p, k) in enumerate(stream):
        server.wait(ids[i])
        info = server.info(ids[i])
        info.update(cells=p.Mx * p.My * p.Mz, steps=k, N=p.Mx)
        out.append(info)
    makespan = time.perf_counter() - t0
    return ids, out, makespan


def summarise(recs, makespan, rate):
    lat = np.array([r["t_done"] - r["t_submit"] for r in recs])
    wait = np.array([r["t_admit"] - r["t_submit"] for r in recs])
    serv = np.array([r["t_done"] - r["t_admit"] for r in recs])
    work = float(sum(r["cells"] * r["steps"] for r in recs))
    span = max(r["t_done"] for r in recs) - min(r["t_submit"] for r in recs)
    q = lambda a, x: float(np.percentile(a, x))   # noqa: E731
    return {"requests": len(recs), "done": int(sum(r["state"] == _lib.REQ_DONE for r in recs)),
            "latency_p50_s": q(lat, 50), "latency_p99_s": q(lat, 99),
            "queue_p50_s": q(wait, 50), "queue_p99_s": q(wait, 99),
            "service_p50_s": q(serv, 50), "service_p99_s": q(serv, 99),
            "served_gpt_steps_per_s": work / span / 1e9, "makespan_s": makespan,
            "offered_gpt_steps_per_s": rate * work / len(recs) / 1e9}


def sequential_estimate(stream, precision, k_short=20, k_long=60):
    """Solves of `stream` run one after another in one process, each alone in
    its own xpfc_ctx at `precision` (the plain sequential baseline of the
    serving loop), estimated from two timed solves per grid size: a solve of
    N^3 and k steps takes a_N + b_N k seconds (create, device initial field,
    step with its diagnostics, read-back of the diagnostics, destroy).
    Returns solves/s over the stream, and the latency percentiles of a FIFO
    queue served that way under the stream's own arrival times."""
    from .api import Xpfc
    import ctypes as C
    cost = {}
    for N in sorted({p.Mx for _, p, _ in stream}):
        p = [q for _, q, _ in stream if q.Mx == N][0]
        q = type(p)()
        C.pointer(q)[0] = p
        q.precision = precision
        t = {}
        for k in (k_short, k_long):
            best = None
            for _ in range(2):
                t0 = time.perf_counter()
                with Xpfc(q) as x:
                    x.initialize(None)
                    x.step(k)
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            t[k] = best
        b = max((t[k_long] - t[k_short]) / (k_long - k_short), 0.0)
        cost[N] = (max(t[k_short] - b * k_short, 0.0), b)
    service = [cost[p.Mx][0] + cost[p.Mx][1] * k for _, p, k in stream]
    free = 0.0
    lat = []
    for (t_arr, _, _), s in zip(stream, service):
        start = max(free, t_arr)
        free = start + s
        lat.append(free - t_arr)
    lat = np.array(lat)
    return {"value": len(stream) / sum(service), "unit": "solves/s",
            "latency_p50_s": float(np.percentile(lat, 50)), "latency_p99_s": float(np.percentile(lat, 99)),
            "total_service_s": float(sum(service)),
            "per_size": {"%d^3" % N: {"per_solve_s": a, "per_step_ms": 1e3 * b} for N, (a, b) in cost.items()},
            "how": "per grid size, solves of %d and %d steps timed alone (best of 2); service time = a_N + b_N steps "
                   "summed over the stream's requests; latencies from a FIFO queue under the stream's arrivals"
                   % (k_short, k_long)}
