"""Generate golden vectors from LC2500/XPFC_CUDA's own program run on a GPU.

Runs on the GPU machine.  Builds the reference program from its staged sources
(baseline/ref_gpu.py: the reference's own CUDA code for sm_103a, cuFFT for its
transforms; the output-precision build prints F and the residual with 17
digits and writes the VTK field with 17 digits) and runs it on the decks of
make_golden.py plus two 512^2 decks (the 64^3-point 2-D analogue: dx = 0.125,
a seeded noise liquid read through the iconfig = 10 restart, 61 and 2001
loop iterations).  Each deck gives tests/golden/gpu_<name>.npz with the
full-precision F and residual series and final field, the same series from the
unmodified-output build, and the run's metadata.  With --exact-powers it runs
the 512^2 decks and a 4096^2 triangle-lattice deck on the build whose
apply_power takes its powers in double precision (power_functions.cu:47,
powf -> pow; nothing else changed) and writes tests/golden/gpu_xp_<name>.npz
(the 4096^2 field as every 16th point in each direction).  Also probes the build linked
against cuFFT as shipped (whose cufftXtSetGPUs is given one GPU) and times the
reference loop (its TIMING line, main.cu:305,437) at 512^2 and 4096^2.

Usage (GPU machine, sources staged):
    python tests/golden/make_golden_gpu.py [--out DIR] [--no-timing]
    python tests/golden/make_golden_gpu.py --exact-powers [--out DIR]
    python tests/golden/make_golden_gpu.py --float-4096 [--out DIR]
"""
import argparse
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, HERE)

from baseline import ref_gpu  # noqa: E402
from make_golden import cases, deck, vtk_text  # noqa: E402


NOISE512_SEED = 20261204


def noise512(amp=0.1):
    """The 512^2 decks' initial field (a seeded noise liquid of standard
    deviation amp; regenerated by the tests from the same seed instead of
    being stored)."""
    return 0.05 + amp * np.random.default_rng(NOISE512_SEED).standard_normal(512 * 512)


def gpu_cases():
    out = [(name, text, vtk_in) for name, text, vtk_in, _ in cases()]
    out.append(("noise512_t60", deck(0.05, 0.2, 1, 3, 0, 1, 64, 64, 512, 512, 60, 1, 20, 10), noise512()))
    out.append(("noise512_t2000", deck(0.05, 0.2, 1, 3, 0, 1, 64, 64, 512, 512, 2000, 1, 100, 10), noise512()))
    # the same liquid with half the noise: its minimum stays far from the
    # explicit scheme's stability edge (n = -0.41)
    out.append(("noise512q_t2000", deck(0.05, 0.2, 1, 3, 0, 1, 64, 64, 512, 512, 2000, 1, 100, 10),
                noise512(0.05)))
    return out


def t_sample_of(text):
    return int(text.split("\n")[9].split()[0])


def dims_of(vtk_in):
    return int(round(np.sqrt(vtk_in.size)))


def meta():
    m = {}
    try:
        m["gpu"] = subprocess.run(["nvidia-smi", "--query-gpu=name,driver_version", "--format=csv,noheader"],
                                  capture_output=True, text=True).stdout.strip()
    except OSError:
        m["gpu"] = None
    try:
        m["nvcc"] = subprocess.run([ref_gpu._nvcc(), "--version"], capture_output=True, text=True).stdout.strip()
    except OSError:
        m["nvcc"] = None
    try:
        with open(os.path.join(ref_gpu.BIN, "BUILD.json")) as f:
            b = json.load(f)
        m["build"] = {"nccl": b["nccl"].split(" (")[0], "programs": b["programs"]}
    except (OSError, KeyError):
        m["build"] = None
    return m


def _vtk_extra(name, vtk_in):
    # small restart fields are stored; the 512^2 one is regenerated from its seed
    if vtk_in is None:
        return {}
    if vtk_in.size <= 4096:
        return {"vtk_in": vtk_in}
    return {"vtk_seed": np.array([NOISE512_SEED]),
            "vtk_amp": np.array([0.05 if name.startswith("noise512q") else 0.1])}


# the 2-D benchmark size (4096^2, as many points as 256^3): the reference's
# triangle lattice with a Gaussian seed, 101 iterations; its final field is
# stored as every SAMPLE-th point in each direction
TRI4096 = ("tri4096_t25", deck(0.05, 0.25, 1, 3, 0.1, 1, 512, 512, 4096, 4096, 25, 0.25, 20, 0,
                               iseed=1, ishape=1, h=4.0, k=4.0, roa=6.0))
SAMPLE = 16


def exact_powers(progs, info, out, only=None):
    """The 512^2 decks and the 4096^2 deck on the double-precision-power build
    (gpu_xp_*.npz)."""
    info = dict(info, variant="power_functions.cu:47 powf -> pow (double-precision powers), 17-digit output")
    runs = [(name, text, vtk_in) for name, text, vtk_in in gpu_cases() if name.startswith("noise512")]
    runs.append(TRI4096 + (None,))
    for name, text, vtk_in in runs:
        if only and name not in only.split(","):
            continue
        ts = t_sample_of(text)
        vtk = vtk_text(vtk_in, dims_of(vtk_in), dims_of(vtk_in), 0.125) if vtk_in is not None else None
        xp = ref_gpu.run(progs["xpfc_ref_xp"], text, ts, vtk_in=vtk, timeout=1800)
        if xp["returncode"] != 0 or "psi_final" not in xp:
            print(name, "FAILED", xp["returncode"], xp["stdout_tail"][-1500:], xp["stderr_tail"][-1500:], flush=True)
            continue
        field = {"psi_final": xp["psi_final"]}
        if xp["psi_final"].size > 512 * 512:
            nx, ny = xp["dims"][0], xp["dims"][1]
            field = {"psi_sample": xp["psi_final"].reshape(nx, ny)[::SAMPLE, ::SAMPLE].copy(),
                     "sample_stride": np.array([SAMPLE])}
        np.savez_compressed(
            os.path.join(out, "gpu_xp_%s.npz" % name),
            deck=np.frombuffer(text.encode(), dtype=np.uint8),
            F=np.array(xp["F"], dtype=np.float64).reshape(-1, 2),
            RMS=np.array(xp["RMS"], dtype=np.float64).reshape(-1, 2),
            final_iteration=np.array([xp["final_iteration"]]),
            meta=np.frombuffer(json.dumps(dict(info, timing=xp["timing"])).encode(), dtype=np.uint8),
            **field, **_vtk_extra(name, vtk_in))
        print("xp", name, "F", xp["F"][:2], "...", xp["F"][-1:], "timing", xp["timing"], flush=True)


def float_4096(progs, info, out):
    """The 4096^2 deck on the full-precision-output build in the reference's
    own semantics (float powers): gpu_tri4096_t25.npz."""
    name, text = TRI4096
    hp = ref_gpu.run(progs["xpfc_ref_hp"], text, t_sample_of(text), timeout=1800)
    if hp["returncode"] != 0 or "psi_final" not in hp:
        print(name, "FAILED", hp["returncode"], hp["stdout_tail"][-1500:], hp["stderr_tail"][-1500:], flush=True)
        return
    nx, ny = hp["dims"][0], hp["dims"][1]
    np.savez_compressed(
        os.path.join(out, "gpu_%s.npz" % name),
        deck=np.frombuffer(text.encode(), dtype=np.uint8),
        F=np.array(hp["F"], dtype=np.float64).reshape(-1, 2),
        RMS=np.array(hp["RMS"], dtype=np.float64).reshape(-1, 2),
        final_iteration=np.array([hp["final_iteration"]]),
        psi_sample=hp["psi_final"].reshape(nx, ny)[::SAMPLE, ::SAMPLE].copy(),
        sample_stride=np.array([SAMPLE]),
        meta=np.frombuffer(json.dumps(dict(info, timing=hp["timing"])).encode(), dtype=np.uint8))
    print(name, "F", hp["F"][:2], "...", hp["F"][-1:], "timing", hp["timing"], flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--no-timing", action="store_true")
    ap.add_argument("--only", default=None, help="comma-separated deck names")
    ap.add_argument("--exact-powers", action="store_true")
    ap.add_argument("--float-4096", action="store_true", help="the 4096^2 deck in the reference's float powers")
    a = ap.parse_args()
    os.makedirs(a.out, exist_ok=True)
    progs = ref_gpu.build()
    info = meta()
    if a.exact_powers:
        exact_powers(progs, info, a.out, a.only)
        return
    if a.float_4096:
        float_4096(progs, info, a.out)
        return

    # the program linked against cuFFT as shipped, on the smallest deck
    name, text, vtk_in = gpu_cases()[2]
    stock = ref_gpu.run(progs["xpfc_ref_stock"], text, t_sample_of(text), keep_field=False, timeout=300)
    lines = [ln for ln in (stock["stdout_tail"] + stock["stderr_tail"]).splitlines() if "cufftXtSetGpus" in ln]
    info["stock_cufft_xt_one_gpu"] = {"deck": name, "returncode": stock["returncode"], "lines": lines}
    print("stock build:", info["stock_cufft_xt_one_gpu"], flush=True)

    for name, text, vtk_in in gpu_cases():
        if a.only and name not in a.only.split(","):
            continue
        ts = t_sample_of(text)
        vtk = vtk_text(vtk_in, dims_of(vtk_in), dims_of(vtk_in), 0.125) if vtk_in is not None else None
        hp = ref_gpu.run(progs["xpfc_ref_hp"], text, ts, vtk_in=vtk, timeout=900)
        lo = ref_gpu.run(progs["xpfc_ref"], text, ts, vtk_in=vtk, keep_field=False, timeout=900)
        if hp["returncode"] != 0 or lo["returncode"] != 0 or "psi_final" not in hp:
            print(name, "FAILED", hp["returncode"], lo["returncode"], hp["stdout_tail"][-1500:],
                  hp["stderr_tail"][-1500:], flush=True)
            continue
        extra = _vtk_extra(name, vtk_in)
        np.savez_compressed(
            os.path.join(a.out, "gpu_%s.npz" % name),
            deck=np.frombuffer(text.encode(), dtype=np.uint8),
            F=np.array(hp["F"], dtype=np.float64).reshape(-1, 2),
            RMS=np.array(hp["RMS"], dtype=np.float64).reshape(-1, 2),
            psi_final=hp["psi_final"],
            final_iteration=np.array([hp["final_iteration"]]),
            F_stock_output=np.array(lo["F"], dtype=np.float64).reshape(-1, 2),
            RMS_stock_output=np.array(lo["RMS"], dtype=np.float64).reshape(-1, 2),
            meta=np.frombuffer(json.dumps(dict(info, timing=hp["timing"])).encode(), dtype=np.uint8),
            **extra)
        print(name, "F", hp["F"][:2], "...", hp["F"][-1:], "RMS", hp["RMS"][:1], "timing", hp["timing"], flush=True)

    if not a.no_timing:
        timing = {"meta": info, "runs": []}
        for M, t, dt in ((512, 100, 1.0), (4096, 25, 0.25)):
            for ts in (1000000, 100):
                text = deck(0.05, 0.25, 1, 3, 0.1, 1, M // 8, M // 8, M, M, t, dt, ts, 0, iseed=1, ishape=1,
                            h=4.0, k=4.0, roa=6.0)
                r = ref_gpu.run(progs["xpfc_ref"], text, ts, keep_field=False, timeout=900)
                steps = int(t / dt + 1)
                ms = r["timing"].get("Full iteration time.")
                rec = {"grid": "%d^2" % M, "loop_iterations": steps, "t_sample": ts, "loop_ms": ms,
                       "returncode": r["returncode"],
                       "gpt_steps_per_s": (M * M * steps / (ms / 1e3) / 1e9) if ms else None}
                timing["runs"].append(rec)
                print("timing", rec, flush=True)
        with open(os.path.join(a.out, "reference_gpu_timing.json"), "w") as f:
            json.dump(timing, f, indent=1)


if __name__ == "__main__":
    main()
