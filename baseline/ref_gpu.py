"""Build and run LC2500/XPFC_CUDA's own CUDA program on one GPU (sm_103a).

The reference is a single CUDA program (main.cu plus its stage files) with no
library API.  This recipe builds it, for the parity fixtures and the timing
the step is compared with, in three steps:

stage(ref)   copies the reference's sources from its tree (the build
             container's checkout, given by path or XPFC_REFERENCE) into
             baseline/_ref/src, unmodified, and into baseline/_ref/src_hp with
             the output precision raised and nothing else changed: the free
             energy and residual printf formats (sum_reduction.cu:64,77, %0.10f
             and %0.5e -> %.17e) and the VTK writer's stream precision
             (write_vtk.cu:8, 6 -> 17 significant digits), and into
             baseline/_ref/src_xp: src_hp with one more edit, the powers of
             apply_power taken in double precision (power_functions.cu:47,
             powf -> pow), for the comparison with the library's exact-power
             path.  baseline/_ref is git-ignored: no reference source enters
             the repository.
build()      on a machine with nvcc (the GPU machine; it is aarch64 there),
             compiles those sources for sm_103a as Makefile_Example:12-37 does
             (same file list, -O3; host flags without -march=native) and links:
               xpfc_ref_stock  the sources against cuFFT as shipped;
               xpfc_ref        the same with baseline/xt_one_gpu.cu, which
                               serves cuFFT's multi-GPU descriptor calls on
                               one GPU (cufftXtSetGPUs refuses a single GPU);
               xpfc_ref_hp     src_hp with xt_one_gpu.cu (full-precision output);
               xpfc_ref_xp     src_xp with xt_one_gpu.cu (full-precision output,
                               double-precision powers).
             NCCL: the system's (or the CUDA Python wheel's) header and
             library when present, else the one-rank stand-in in
             baseline/nccl_one_rank (a sum reduce to root 0 over one rank is a
             copy).
run(...)     runs a program in a scratch directory on a pfc.input deck (and an
             initial_density_field.vtk for iconfig = 10) and parses what it
             prints: "iteration: n F = ..." (sum_reduction.cu:64),
             "SSE_gpu = ..." (sum_reduction.cu:77, one per n % t_sample == 0,
             main.cu:326), "TIMING: ... ms (Full iteration time.)"
             (helpers_header.cuh:46, main.cu:437) and the final
             density_data<n>.vtk (main.cu:455).

Usage:  python baseline/ref_gpu.py stage [--ref DIR]   (build container)
        python baseline/ref_gpu.py build                 (GPU machine)
"""
import argparse
import concurrent.futures as cf
import glob
import hashlib
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SRC = os.path.join(OUT, "src")
SRC_HP = os.path.join(OUT, "src_hp")
SRC_XP = os.path.join(OUT, "src_xp")
BIN = os.path.join(OUT, "gpu")
# Makefile_Example:29 (randn.cu is not in it and does not compile)
UNITS = ["main", "initialize", "FFT_freq", "Avg_calc", "linspace", "read_input", "write_vtk", "convolve_fields",
         "FE_calc", "euler_step", "scaling_step", "power_functions", "sum_reduction", "copy_to_cpu",
         "permute_matrices", "copy_matrix", "sse_calculation"]
HEADERS = ["globals.cuh", "helpers_header.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# output-precision edits of src_hp: (file, exact text, replacement)
HP_EDITS = [
    ("sum_reduction.cu", 'printf("iteration: %d F = %0.10f", it, sum*ff_factor);',
     'printf("iteration: %d F = %.17e", it, sum*ff_factor);'),
    ("sum_reduction.cu", 'printf( " SSE_gpu = %0.5e \\n", sqrt(sum/M2) );',
     'printf( " SSE_gpu = %.17e \\n", sqrt(sum/M2) );'),
    ("write_vtk.cu", "    ofstream vtkFile(vtkFilename);\n",
     "    ofstream vtkFile(vtkFilename);\n    vtkFile.precision(17);\n"),
]
# src_xp: src_hp's edits plus the powers in double precision (the reference
# rounds psi to float and takes powf, which makes its trajectory jump by a
# float ulp wherever a double-rounding difference moves psi across a float
# rounding boundary)
XP_EDITS = HP_EDITS + [
    ("power_functions.cu", "double a = powf(psi[i + j*Mx].x, pow_i);",
     "double a = pow(psi[i + j*Mx].x, pow_i);"),
]


def _sha(path):
    with open(path, "rb") as f:
        return hashlib.sha256(f.read()).hexdigest()


def stage(ref):
    """Copies the reference's sources (and the output-precision variant)."""
    if not ref or not os.path.isfile(os.path.join(ref, "main.cu")):
        raise SystemExit("stage: no reference tree at %r (give --ref or XPFC_REFERENCE)" % (ref,))
    for d in (SRC, SRC_HP, SRC_XP):
        os.makedirs(d, exist_ok=True)
    manifest = {"reference": os.path.abspath(ref), "files": {}, "hp_edits": [], "xp_edits": []}
    for name in [u + ".cu" for u in UNITS] + HEADERS:
        for d in (SRC, SRC_HP, SRC_XP):
            shutil.copyfile(os.path.join(ref, name), os.path.join(d, name))
        manifest["files"][name] = _sha(os.path.join(SRC, name))
    for tree, edits, key in ((SRC_HP, HP_EDITS, "hp_edits"), (SRC_XP, XP_EDITS, "xp_edits")):
        for name, old, new in edits:
            path = os.path.join(tree, name)
            text = open(path).read()
            if text.count(old) != 1:
                raise SystemExit("stage: the edit of %s for %s does not apply" % (name, os.path.basename(tree)))
            with open(path, "w") as f:
                f.write(text.replace(old, new))
            manifest[key].append({"file": name, "from": old, "to": new})
    with open(os.path.join(OUT, "MANIFEST.json"), "w") as f:
        json.dump(manifest, f, indent=1)
    return OUT


def staged():
    return all(os.path.isfile(os.path.join(d, "main.cu")) for d in (SRC, SRC_HP, SRC_XP))


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _find_nccl():
    """(include dir, library dir) of an NCCL installation, or None."""
    inc_dirs = ["/usr/include", "/usr/local/include", "/usr/local/cuda/include"]
    lib_dirs = ["/usr/lib/aarch64-linux-gnu", "/usr/lib/x86_64-linux-gnu", "/usr/lib64", "/usr/local/lib",
                "/usr/local/cuda/lib64"]
    try:
        import nvidia  # the CUDA Python wheels (nvidia-nccl-cu*) that PyTorch installs
        for p in nvidia.__path__:
            inc_dirs.append(os.path.join(p, "nccl", "include"))
            lib_dirs.append(os.path.join(p, "nccl", "lib"))
    except ImportError:
        pass
    inc = next((d for d in inc_dirs if os.path.isfile(os.path.join(d, "nccl.h"))), None)
    lib = next((d for d in lib_dirs if glob.glob(os.path.join(d, "libnccl.so*"))), None)
    if inc and lib:
        return inc, lib
    return None


def programs():
    return {k: os.path.join(BIN, k) for k in ("xpfc_ref_stock", "xpfc_ref", "xpfc_ref_hp", "xpfc_ref_xp")}


def build(force=False, log=print):
    """Compiles the staged sources for sm_103a; returns the built programs."""
    if not staged():
        raise RuntimeError("the reference sources are not staged (python baseline/ref_gpu.py stage)")
    os.makedirs(BIN, exist_ok=True)
    progs = programs()
    if not force and all(os.path.exists(p) for p in progs.values()):
        return progs
    nccl = _find_nccl()
    inc = ["-I", os.path.join(HERE, "shim")]
    link_nccl = []
    extra = []
    if nccl:
        inc += ["-I", nccl[0]]
        link_nccl = ["-L", nccl[1], "-Xlinker", "-rpath=" + nccl[1], "-lnccl"]
        nccl_kind = "system NCCL (%s)" % nccl[1]
    else:
        inc += ["-I", os.path.join(HERE, "nccl_one_rank")]
        extra.append(("nccl_one_rank.o", os.path.join(HERE, "nccl_one_rank", "nccl_one_rank.cu")))
        nccl_kind = "one-rank stand-in (no NCCL found)"
    flags = ["-O3", "-std=c++17", "-w"] + ARCH + ["-Xcompiler", "-fopenmp"] + inc

    jobs = []
    for tag, src in (("src", SRC), ("src_hp", SRC_HP), ("src_xp", SRC_XP)):
        d = os.path.join(BIN, tag)
        os.makedirs(d, exist_ok=True)
        for u in UNITS:
            jobs.append((os.path.join(d, u + ".o"), os.path.join(src, u + ".cu"), ["-I", src]))
    for obj, src in extra + [("xt_one_gpu.o", os.path.join(HERE, "xt_one_gpu.cu"))]:
        jobs.append((os.path.join(BIN, obj), src, []))

    def compile_one(job):
        obj, src, more = job
        cmd = [_nvcc()] + flags + more + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        list(ex.map(compile_one, jobs))
    objs = {tag: [os.path.join(BIN, tag, u + ".o") for u in UNITS] for tag in ("src", "src_hp", "src_xp")}
    shim = [os.path.join(BIN, "xt_one_gpu.o")]
    nccl_obj = [os.path.join(BIN, "nccl_one_rank.o")] if not nccl else []
    libs = ["-lcufft", "-lcudart", "-ldl", "-Xcompiler", "-fopenmp"] + link_nccl
    for name, ob in (("xpfc_ref_stock", objs["src"]), ("xpfc_ref", objs["src"] + shim),
                     ("xpfc_ref_hp", objs["src_hp"] + shim), ("xpfc_ref_xp", objs["src_xp"] + shim)):
        cmd = [_nvcc()] + ARCH + ob + nccl_obj + ["-o", progs[name] + ".tmp"] + libs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        os.replace(progs[name] + ".tmp", progs[name])
    with open(os.path.join(BIN, "BUILD.json"), "w") as f:
        json.dump({"nccl": nccl_kind, "flags": flags, "programs": list(progs)}, f, indent=1)
    log("reference program built (%s)" % nccl_kind)
    return progs


_F = re.compile(r"iteration: (-?\d+) F = ([-+0-9.eEnaif]+)")
_SSE = re.compile(r"SSE_gpu = ([-+0-9.eEnaif]+)")
_TIMING = re.compile(r"TIMING: ([-+0-9.eE]+) ms \(([^)]*)\)")


def read_vtk(path):
    """(values in the reference's [Mx][My] host layout, (nx, ny))."""
    with open(path) as f:
        lines = f.read().split("\n")
    dims = None
    start = None
    for i, ln in enumerate(lines[:20]):
        if ln.startswith("DIMENSIONS"):
            dims = [int(v) for v in ln.split()[1:4]]
        if ln.startswith("LOOKUP_TABLE"):
            start = i + 1
            break
    nx, ny = dims[0], dims[1]
    vals = np.array([float(v) for v in lines[start:start + nx * ny]])
    # write_vtk.cu:25-29 writes densityData[j*ny + i] in file order i*nx + j
    return vals.reshape(ny, nx).T.reshape(-1), (nx, ny)


def parse(stdout, t_sample):
    F = [(int(m.group(1)), float(m.group(2))) for m in _F.finditer(stdout)]
    sse = [float(m.group(1)) for m in _SSE.finditer(stdout)]
    # one residual per loop iteration n with n % t_sample == 0 (main.cu:326)
    R = [(k * t_sample, v) for k, v in enumerate(sse)]
    timing = {m.group(2): float(m.group(1)) for m in _TIMING.finditer(stdout)}
    return F, R, timing


def run(prog, deck, t_sample, vtk_in=None, timeout=600, keep_field=True, workdir=None):
    """Runs a reference program on a deck; returns its parsed output."""
    own = workdir is None
    d = tempfile.mkdtemp(prefix="xpfc_ref_") if own else workdir
    try:
        with open(os.path.join(d, "pfc.input"), "w") as f:
            f.write(deck)
        if vtk_in is not None:
            with open(os.path.join(d, "initial_density_field.vtk"), "w") as f:
                f.write(vtk_in)
        r = subprocess.run([prog], cwd=d, capture_output=True, text=True, timeout=timeout)
        F, R, timing = parse(r.stdout, t_sample)
        out = {"returncode": r.returncode, "F": F, "RMS": R, "timing": timing,
               "stdout_tail": r.stdout[-3000:], "stderr_tail": r.stderr[-3000:]}
        vt = sorted(glob.glob(os.path.join(d, "density_data*.vtk")),
                    key=lambda p: int(re.findall(r"(\d+)\.vtk$", p)[0]))
        if keep_field and vt:
            out["final_iteration"] = int(re.findall(r"(\d+)\.vtk$", vt[-1])[0])
            out["psi_final"], out["dims"] = read_vtk(vt[-1])
        return out
    finally:
        if own:
            shutil.rmtree(d, ignore_errors=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["stage", "build"])
    ap.add_argument("--ref", default=os.environ.get("XPFC_REFERENCE"))
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    if a.what == "stage":
        print(stage(a.ref))
    else:
        print(json.dumps(build(force=a.force)))


if __name__ == "__main__":
    sys.exit(main())
