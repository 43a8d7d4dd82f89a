#!/usr/bin/env python3
"""Throughput of the fused XPFC step on GB300: grid-point-steps/s.

Workload (one "step" = one semi-implicit time step of the whole field):
256^3 periodic grid, dx = 0.125 (L = 32), two-peak fcc correlation kernel
(k = 2 pi, 4 pi/sqrt 3; alpha = 1, 1; rho = 1, 1; beta = 8, 6; max envelope),
eta = 2, chi = 1, n0 = 0.04, initial n = n0 + N(0, 0.05^2) (seeded Philox),
conserved noise of amplitude 0.01 every step, dt = 1, diagnostics every 100
steps; FP32 bulk with FP64 k = 0 and sums.  sigma = 0.22: at sigma = 0.12 this
parameter set diverges under the reference's own scheme within 20 steps (the
explicit nonlinear term), while the work per step does not depend on sigma.
All inputs are synthetic and seeded.

Default arm: libxpfc through its C ABI on one GPU per rank (replicas: every
rank advances its own independent solve; no collective on the data path).
--impl reference: the CPU implementation of the same step (the FP64 oracle
restating the reference's loop, OpenMP on the host cores), rank 0 only.

Three more legs ride on the same line: "sweep" (64 independent solves of
1000 steps through one xpfc_batch: solves/s, against the same solves one
context at a time), "serve" (a Poisson stream of solve requests through
xpfc_server: latency percentiles and served grid-point-steps/s, every solve
in a context of its own, then with merged groups, and a saturating burst
of 64^3 requests both ways) and "two_d"
(the 2-D step at 4096^2, the reference's own benchmark size, both
precisions).

Prints one JSON line on rank 0.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "Gpt-steps/s @256^3 mixed vs FP64 on 1 GB300 (F rel<=1e-6); sweep solves/s, p99"
UNIT = "Gpt-steps/s"
DX = 0.125
FCC = ((2 * math.pi, 1.0, 1.0, 8.0), (2 * math.pi * 2 / math.sqrt(3), 1.0, 1.0, 6.0))
# the step's passes (algorithmic bytes per launch from xpfc_pass_bytes)
PASS_NAMES = {0: "pencil_kernel", 1: "col_kernel(inverse)", 2: "row_kernel(fused)", 3: "col_kernel(forward)"}
FLOOR_BYTES_PER_POINT = 16.125   # two read+write sweeps of the FP32 state at 256^3
SIGMA = 0.22


def workload_params(X, n, precision, rank):
    L = n * DX
    return X.default_params(Mx=n, My=n, Mz=n, Lx=L, Ly=L, Lz=L, psi0=0.04, sigma=SIGMA, peaks=FCC,
                            envelope=X._lib.ENVELOPE_MAX, a=1.0, b=1.0 / 3.0, eps=0.0, Mo=1.0, dt=1.0,
                            nsteps=2001, t_sample=100, precision=precision, ic_kind=X._lib.IC_NOISE,
                            ic_amp=0.05, ic_seed=1 + rank, noise_amp=0.01, noise_seed=11 + rank,
                            ff_factor=DX ** 3, ref_compat=0)


def config(n, precision):
    return {"workload": "XPFC step %d^3, fcc kernel, conserved noise 0.01/step, %s" % (
        n, "FP32 bulk + FP64 k=0 and sums" if precision == "mixed" else "FP64"),
        "grid": n, "dx": DX, "sigma": SIGMA, "precision": precision, "diag_every": 100,
        "l2": "flushed between timed steps (256 MB write outside the timed events)",
        "parallelism": "replicas (one independent solve per GPU)"}


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(dev)], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        sm, smax, reasons, power = [], None, set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            c = [x.strip() for x in line.split(",")]
            if len(c) < 9:
                continue
            try:
                sm.append(float(c[1]))
                smax = float(c[2])
                power.append(float(c[3]))
            except ValueError:
                continue
            for nm, v in zip(names, c[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.f.name)
        load = [v for v in sm if smax and v > 0.5 * smax] or sm
        return {"sm_mhz": statistics.median(load) if load else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm),
                "power_w_max": max(power) if power else None}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cpu_baseline(n, steps=None, target_s=15.0):
    """The FP64 oracle on the host cores over a bounded sample of the workload."""
    import numpy as np  # noqa: F401
    from oracle import oracle as O
    L = n * DX
    p = O.make_params(n, n, n, L=(L, L, L), a=1.0, b=1.0 / 3.0, sigma=SIGMA, peaks=FCC, envelope=1,
                      ff_factor=DX ** 3, noise_amp=0.01, noise_seed=11)
    psi = O.ic_noise(n, n, n, 0.04, 0.05, 1)
    O.pin_mean(psi, 0.04)
    if steps is None:
        t1, _ = O.bench(p, psi, 1)
        steps = max(1, min(40, int(target_s / max(t1, 1e-3))))
    sec, _ = O.bench(p, psi, steps)
    return {"value": n ** 3 * steps / sec / 1e9, "unit": UNIT, "cores": O.threads(), "host_cpus": os.cpu_count(),
            "kind": "port",
            "sample": "%d full steps of the %d^3 workload (FP64 oracle, OpenMP, %d threads), %.1f s" % (
                steps, n, O.threads(), sec)}


def accuracy(X, n, rank, local, host_psi, k):
    """The mixed-precision step against the FP64 oracle on the benchmark's own
    workload: k steps of the n^3 case from the same initial field (the oracle
    runs them on the host cores), free energy and field compared."""
    import numpy as np
    from oracle import oracle as O
    L = n * DX
    q = workload_params(X, n, X._lib.MIXED, rank)
    q.device = local
    q.t_sample = k
    with X.Xpfc(q) as x:
        x.initialize(host_psi)
        recs = x.step(k)
        field = x.copy2cpu().reshape(-1)
    P = O.make_params(n, n, n, L=(L, L, L), a=q.a, b=q.b, sigma=q.sigma, peaks=FCC, envelope=1, ff_factor=DX ** 3,
                      noise_amp=q.noise_amp, noise_seed=q.noise_seed)
    ref, F, mean, rms = O.run(P, host_psi, k, k)
    fin = [r for r in recs if r["iteration"] == k][0]
    dev = field - field.mean()
    return {"steps": k, "F_rel": abs(fin["F"] - F[k]) / abs(F[k]),
            "field_rel_l2": float(np.linalg.norm(field - ref) / np.linalg.norm(ref)),
            "deviation_rel_l2": float(np.linalg.norm(dev - (ref - ref.mean())) / np.linalg.norm(ref - ref.mean())),
            "mean_abs_err": abs(fin["mean"] - mean[k]),
            "against": "FP64 oracle on the host cores, same initial field and noise stream",
            "bar": "F rel <= 1e-6, field rel-L2 <= 1e-5"}


def reference_gpu_program(n, steps=101):
    """LC2500/XPFC_CUDA's own program (baseline/ref_gpu.py, built for sm_103a
    on this machine from its staged sources) at n^2, timed by its own TIMING
    line over `steps` loop iterations with t_sample larger than the run (no
    sampling inside the loop), as the reference times itself."""
    try:
        from baseline import ref_gpu
    except ImportError as e:
        return {"unavailable": "baseline/ref_gpu.py not importable: %s" % e}
    prog = ref_gpu.programs()["xpfc_ref"]
    if not os.path.exists(prog):
        return {"unavailable": "the reference program is not built here (its sources are not staged)"}
    import math as _m
    dt = 0.25
    t = (steps - 1) * dt
    text = ("1 no_val\n0.05 0.25 psi_0 s\n1 3 0.1 1 a b eps Mo\n\n%d %d Lx Ly\n%d %d Mx My\n\n%g t\n%g dt\n"
            "%d t_sample\n\n0 iconfig\n0.2 0.1 A_10 A_11\n0.3 A_tri\n\n1 iseed\n1 ishape\n4.0 4.0 6.0 h k roa\n"
            % (n // 8, n // 8, n, n, t, dt, 10 ** 7))
    r = ref_gpu.run(prog, text, 10 ** 7, keep_field=False, timeout=600)
    ms = r["timing"].get("Full iteration time.")
    iters = int(_m.ceil(t / dt + 1))
    if r["returncode"] != 0 or not ms:
        return {"unavailable": "the reference program failed (rc %d)" % r["returncode"]}
    return {"value": n * n * iters / (ms / 1e3) / 1e9, "unit": UNIT, "loop_ms": ms, "loop_iterations": iters,
            "what": "the reference's own main.cu loop (cuFFT Z2Z, FP64), its TIMING line, one GB300, "
                    "cuFFT's multi-GPU descriptor calls served on one GPU (cufftXtSetGPUs refuses one GPU)"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    n = args.size
    L = n * DX
    p = O.make_params(n, n, n, L=(L, L, L), a=1.0, b=1.0 / 3.0, sigma=SIGMA, peaks=FCC, envelope=1,
                      ff_factor=DX ** 3, noise_amp=0.01, noise_seed=11)
    psi = O.ic_noise(n, n, n, 0.04, 0.05, 1)
    O.pin_mean(psi, 0.04)
    # bounded sample: at most REF_MAX_STEPS timed steps of the full-size
    # workload (one 256^3 FP64 step takes ~0.25 s on 16 cores), after the same
    # number of warm-up steps as the library's arm
    REF_MAX_STEPS = 40
    k = max(1, min(args.steps, REF_MAX_STEPS))
    _, psi = O.bench(p, psi, args.warmup)
    sec, _ = O.bench(p, psi, k)
    v = n ** 3 * k / sec / 1e9
    cb = {"value": v, "unit": UNIT, "cores": O.threads(), "host_cpus": os.cpu_count(), "kind": "port",
          "sample": "%d timed steps (+%d warm-up) of the %d^3 workload (of the %d requested), FP64 oracle "
                    "restating the reference loop (main.cu:306-435); the reference itself is CUDA-only"
                    % (k, args.warmup, n, args.steps)}
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": k, "warmup": args.warmup, "ms_per_step": 1e3 * sec / k,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded Philox initial field and noise)", "config": config(n, "mixed"),
            "cpu_baseline": cb, "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def load_traffic(kernel, n):
    """DRAM bytes per launch from the committed ncu summary, or None."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        e = t[kernel]
        return e["bytes_per_launch_at"][str(n)]
    except (OSError, KeyError, ValueError):
        return None


def measured_peak():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def sweep_cpu_estimate(params, steps, per_size_steps=3):
    """Host-core time of the sweep, estimated from a few oracle steps per grid size."""
    from oracle import oracle as O
    t_step = {}
    for N in sorted({p.Mx for p in params}):
        L = N * DX
        q = O.make_params(N, N, N, L=(L, L, L), a=1.0, b=1.0 / 3.0, sigma=0.3, peaks=FCC, envelope=1,
                          ff_factor=DX ** 3)
        psi = O.ic_noise(N, N, N, 0.04, 0.1, 1)
        sec, _ = O.bench(q, psi, per_size_steps)
        t_step[N] = sec / per_size_steps
    total = sum(t_step[p.Mx] * steps for p in params)
    return {"value": len(params) / total, "unit": "solves/s", "cores": O.threads(), "kind": "port",
            "sample": "%d oracle steps per grid size (%s), scaled to %d instances x %d steps" % (
                per_size_steps, ", ".join("%d^3: %.3f s/step" % (k, v) for k, v in sorted(t_step.items())),
                len(params), steps)}


def run_two_d(args, local, group, barrier):
    """The 2-D step at the reference's own benchmark size (4096^2, dx = 0.125,
    single-peak kernel, conserved noise 0.01, diagnostics every 100): device
    time per step with CUDA events, both precisions."""
    import torch

    import xpfc_cuda_gb300 as X
    n = args.two_d_size
    out = {"grid": "%d^2" % n, "unit": UNIT}
    for prec, name, k in ((X._lib.MIXED, "mixed", 400), (X._lib.FP64, "fp64", 40)):
        L = n * DX
        p = X.default_params(Mx=n, My=n, Mz=1, Lx=L, Ly=L, Lz=1.0, psi0=0.04, sigma=0.25,
                             peaks=((2 * math.pi, 1.0, 1.0, 8.0),), envelope=X._lib.ENVELOPE_MAX, precision=prec,
                             t_sample=100, ic_kind=X._lib.IC_NOISE, ic_amp=0.05, noise_amp=0.01, noise_seed=5,
                             ff_factor=DX ** 2, device=local)
        stream = torch.cuda.Stream()
        with X.Xpfc(p, stream=stream.cuda_stream) as x:
            x.initialize(None)
            x.step_async(5)
            x.collect()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            e0.record(stream)
            x.step_async(k)
            e1.record(stream)
            x.collect()
            barrier()
            ms = group.max(e0.elapsed_time(e1))
        out[name] = {"value": group.sum(n * n * k) / (ms / 1e3) / 1e9, "ms_per_step": ms / k, "steps": k}
    if not args.no_ref_gpu and group.rank == 0:
        out["reference_program"] = reference_gpu_program(n)
    return out


def run_sweep(args, rank, local, group, barrier):
    """Batched parameter sweep (xpfc_batch): solves/s through the C ABI."""
    import numpy as np

    from xpfc_cuda_gb300 import sweep as SW
    ps = SW.sweep_params(args.sweep_n, seed=rank, device=local)
    fields = SW.initial_fields(ps)
    SW.solve_batch(ps, fields, 3)                    # warm-up: every kernel instance the sweep uses
    barrier()
    tb, (outs, diags, groups) = SW.timed(SW.solve_batch, ps, fields, args.sweep_steps)
    barrier()
    tb_max = group.max(tb)
    solves = group.sum(len(ps)) / tb_max
    out = {"value": solves, "unit": "solves/s", "instances": len(ps), "steps": args.sweep_steps,
           "seconds": tb_max, "groups": groups,
           "gpt_steps_per_s": group.sum(SW.points(ps) * args.sweep_steps) / tb_max / 1e9,
           "finite": bool(all(np.isfinite(f).all() for f in outs)),
           "workload": "N in U{48,64,96,128}^3, n0 in U[0,0.08], sigma in U[0.28,0.35], single-peak or fcc "
                       "(p=0.5), dt=1, diagnostics every 100, FP32 bulk; seed i for instance i",
           "timed": "xpfc_batch_create + initialize(host FP64 fields) + step + collect + get_field(host) + destroy"}
    if not args.no_sweep_seq:
        barrier()
        ts, (outs_s, diags_s) = SW.timed(SW.solve_sequential, ps, fields, args.sweep_steps)
        barrier()
        out["sequential"] = {"value": group.sum(len(ps)) / group.max(ts), "unit": "solves/s", "seconds": ts,
                             "what": "the same solves one xpfc_ctx after another"}
        out["identical_to_sequential"] = bool(all(np.array_equal(a, b) for a, b in zip(outs, outs_s)) and
                                             diags == diags_s)
    if rank == 0 and group.world == 1 and not args.no_cpu:
        out["cpu_baseline"] = sweep_cpu_estimate(ps, args.sweep_steps)
    return out


def run_serve(args, rank, local, group, barrier):
    """Serving loop (xpfc_server) on a Poisson request stream: latency
    percentiles and served throughput."""
    import numpy as np

    import xpfc_cuda_gb300 as X
    from xpfc_cuda_gb300 import serving as SV
    rate = 20.0
    stream = SV.request_stream(args.serve_requests, rate=rate, seed=rank, device=local)
    # a few of the smaller requests keep their fields for the same-as-alone check
    keep = [i for i, (_, p, k) in enumerate(stream) if p.Mx <= 96 and k <= 2000][:3]
    budget = 150 << 30

    def play(strm, merge_max, keep_ids=()):
        with X.Server(hbm_budget_bytes=budget, max_running=args.serve_running, chunk_steps=16, device=local,
                      merge_max=merge_max) as srv:
            # warm server: one short solve of every size (kernel modules loaded,
            # one pooled context per size)
            warm = [srv.submit(p, 3) for p in {p.Mx: p for _, p, _ in strm}.values()]
            for w in warm:
                srv.wait(w)
            barrier()
            ids, recs, span = SV.play(srv, strm, set(keep_ids))
            barrier()
            stats = srv.stats()
            same = True
            for i in keep_ids:
                _, p, k = strm[i]
                f, r = srv.result(ids[i], shape=(p.Mx, p.My, p.Mz))
                with X.Xpfc(p) as x:
                    x.initialize(None)
                    r1 = x.step(k)
                    f1 = x.copy2cpu()
                same &= bool(np.array_equal(f, f1) and r == r1)
        return recs, span, stats, same

    def brief(recs, span, stats, same, r):
        o = SV.summarise(recs, span, r)
        return {"solves_per_s": len(recs) / span, "latency_p50_s": o["latency_p50_s"],
                "latency_p99_s": o["latency_p99_s"], "served_gpt_steps_per_s": o["served_gpt_steps_per_s"],
                "merged_groups": stats["merged_groups"], "merged_solves": stats["merged_solves"],
                "same_as_alone": same}

    recs, span, stats, same = play(stream, 0, keep)
    out = SV.summarise(recs, span, rate)
    out["solves_per_s"] = len(recs) / span
    if args.serve_merge > 1:
        # the same stream with merged groups (queued requests of one grid with
        # step counts within 25 % share every launch)
        m = brief(*play(stream, args.serve_merge, keep), rate)
        m["merge_max"] = args.serve_merge
        out["with_merging"] = m
        same &= m["same_as_alone"]
        # a burst of 64^3 requests (passes bound by launch latency) that
        # saturates the server, without and with merging: its capacity
        srate = 1000.0
        small = SV.request_stream(200, rate=srate, seed=100 + rank, sizes=(64,), weights=(1.0,), device=local)
        s0 = brief(*play(small, 0), srate)
        s1 = brief(*play(small, args.serve_merge), srate)
        out["small_grid_stream"] = {"workload": "200 requests of 64^3, Poisson 1000/s (a burst that saturates the "
                                                "server), steps U[200,5000], sweep physics",
                                    "without_merging": s0, "with_merging": s1,
                                    "solves_per_s_ratio": s1["solves_per_s"] / s0["solves_per_s"]}
    if not args.no_serve_seq:
        # the plain sequential baselines: the same requests one at a time, each
        # alone, in FP64 and in mixed precision (estimated per grid size)
        seq64 = SV.sequential_estimate(stream, X._lib.FP64)
        seq32 = SV.sequential_estimate(stream, X._lib.MIXED)
        out["sequential_fp64"] = seq64
        out["sequential_mixed"] = seq32
        out["solves_per_s_vs_sequential_fp64"] = out["solves_per_s"] / seq64["value"]
        out["solves_per_s_vs_sequential_mixed"] = out["solves_per_s"] / seq32["value"]
    out.update({"unit": "s", "rate_per_s": rate, "max_running": args.serve_running, "chunk_steps": 16,
                "hbm_budget_gb": budget / 2 ** 30, "peak_device_gb": stats["peak_bytes_in_use"] / 2 ** 30,
                "contexts_created": stats["contexts_created"], "contexts_reused": stats["contexts_reused"],
                "same_as_alone_checked": len(keep), "same_as_alone": same,
                "workload": "%d requests, Poisson 20/s, N^3 with N in (64,96,128,192,256) w=(.3,.25,.2,.15,.1), "
                            "steps U[200,5000], sweep physics, FP32 bulk, device initial fields" % len(stream),
                "timed": "wall clock from the first arrival to the last completion; per-request times from the "
                         "server's clock (submit, admit, done)"})
    return out


def run_ours(args):
    import torch
    import numpy as np

    import xpfc_cuda_gb300 as X

    from xpfc_cuda_gb300.replicas import Group
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    group = Group("nccl", device="cuda")

    def barrier():
        group.barrier()
        torch.cuda.synchronize()

    allmax = group.max

    n = args.size
    prec = X._lib.MIXED if args.precision == "mixed" else X._lib.FP64
    p = workload_params(X, n, prec, rank)
    p.device = local
    # a dedicated stream: the legacy default stream has handle 0, which the
    # library would read as "make your own stream"
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    host_psi = X.build_initial_field(p)
    x = X.Xpfc(p, stream=stream.cuda_stream)
    x.initialize(host_psi)
    x.step_async(args.warmup)
    x.collect()
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    launches0 = x.launch_count
    barrier()
    clk = Clocks(local)
    for k in range(args.steps):
        flush.zero_()
        starts[k].record(stream)
        x.step_async(1)
        ends[k].record(stream)
    x.collect()
    barrier()
    clocks = clk.stop()
    launches = x.launch_count - launches0
    ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
    ms_max = allmax(ms)
    # per-pass durations for the roofline: a second run of the same steps with
    # an event pair around every launch (kept out of the timed loop above,
    # whose passes run back to back)
    x.set_profiling(True)
    for k in range(min(args.steps, 500)):
        flush.zero_()
        x.step_async(1)
    x.collect()
    prof = x.profile()
    x.set_profiling(False)
    from xpfc_cuda_gb300.replicas import throughput
    value = throughput(n ** 3 * args.steps, ms / 1e3, group) / 1e9

    # FP64 plain path on the same workload (the "vs FP64" half of the metric)
    fp64 = None
    if not args.no_fp64 and args.precision == "mixed":
        p64 = workload_params(X, n, X._lib.FP64, rank)
        p64.device = local
        with X.Xpfc(p64, stream=stream.cuda_stream) as y:
            y.initialize(host_psi)
            y.step_async(2)
            y.collect()
            k64 = max(3, args.steps // 4)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            barrier()
            e0.record(stream)
            y.step_async(k64)
            e1.record(stream)
            y.collect()
            barrier()
            t64 = allmax(e0.elapsed_time(e1))
        fp64 = {"value": ws * n ** 3 * k64 / (t64 / 1e3) / 1e9, "unit": UNIT, "ms_per_step": t64 / k64,
                "steps": k64, "l2": "not flushed (state 2 x 134 MB > L2)"}

    # end to end through the C ABI with host buffers: upload the initial
    # field, run the solve segment with its diagnostics, download the field
    e2e = None
    if not args.no_e2e:
        ke = args.e2e_steps
        out = np.empty(n ** 3)
        barrier()
        t0 = time.perf_counter()
        x.initialize(host_psi)
        recs = x.step(ke)
        out[:] = x.copy2cpu().reshape(-1)
        torch.cuda.synchronize()
        te = allmax(time.perf_counter() - t0)
        diag_bytes = 8 * 8 * max(1, len(recs))
        e2e = {"value": ws * n ** 3 * ke / te / 1e9, "unit": UNIT,
               "h2d_bytes_per_step": int(8 * n ** 3 / ke),
               "d2h_bytes_per_step": int((4 * n ** 3 if prec == X._lib.MIXED else 8 * n ** 3) / ke + diag_bytes / ke),
               "steps": ke, "seconds": te,
               "what": "xpfc_initialize(host FP64 field) + xpfc_step(%d, diagnostics every 100) + "
                       "xpfc_get_field(host)" % ke}

    # roofline of the dominant pass
    peak, peak_kind = measured_peak()
    passes = {k: v for k, v in prof.items() if k in PASS_NAMES and v[1] > 0}
    dom = max(passes, key=lambda k: passes[k][0]) if passes else None
    roof = None
    if dom is not None:
        avg_ms = passes[dom][0] / passes[dom][1]
        alg = x.pass_bytes(dom)
        achieved = alg / (avg_ms / 1e3) / 1e9
        traffic = load_traffic(PASS_NAMES[dom], n)
        roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "kernel": PASS_NAMES[dom], "algorithmic_bytes": alg,
                "avg_launch_ms": avg_ms, "peak_source": peak_kind,
                "passes": {PASS_NAMES[k]: {"avg_ms": v[0] / v[1], "launches": v[1],
                                           "algorithmic_bytes": x.pass_bytes(k),
                                           "GB/s": x.pass_bytes(k) / (v[0] / v[1] / 1e3) / 1e9}
                           for k, v in passes.items()},
                "step_frac_of_two_sweep_floor": (value * 1e9 / ws) * FLOOR_BYTES_PER_POINT / (peak * 1e9)}

    cpu = None
    acc = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(n)
        if args.precision == "mixed":
            acc = accuracy(X, n, rank, local, host_psi, args.accuracy_steps)

    sweep = None
    if not args.no_sweep:
        torch.cuda.set_stream(torch.cuda.default_stream())
        sweep = run_sweep(args, rank, local, group, barrier)

    serve = None
    if not args.no_serve:
        serve = run_serve(args, rank, local, group, barrier)

    two_d = None
    if not args.no_two_d:
        two_d = run_two_d(args, local, group, barrier)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec == X._lib.MIXED else "f64",
                "data": "synthetic (seeded Philox initial field and noise)", "config": config(n, args.precision),
                "clocks": clocks, "e2e": e2e, "gpu_launches": launches, "roofline": roof, "cpu_baseline": cpu,
                "accuracy": acc,
                "fp64": fp64, "sweep": sweep, "serve": serve, "two_d": two_d}
        print(json.dumps(line), flush=True)
    x.close()
    group.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="xpfc", choices=["xpfc", "reference"])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-sweep-seq", action="store_true")
    ap.add_argument("--sweep-n", type=int, default=64)
    ap.add_argument("--sweep-steps", type=int, default=1000)
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-running", type=int, default=16)
    ap.add_argument("--serve-merge", type=int, default=8,
                    help="solves per merged group in the serving leg's merged runs (0: no merged runs)")
    ap.add_argument("--no-serve-seq", action="store_true", help="skip the sequential baselines of the serve leg")
    ap.add_argument("--no-two-d", action="store_true")
    ap.add_argument("--two-d-size", type=int, default=4096)
    ap.add_argument("--no-ref-gpu", action="store_true", help="skip the reference program's 2-D timing")
    ap.add_argument("--accuracy-steps", type=int, default=40)
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
