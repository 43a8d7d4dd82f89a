"""Build recipe of libxpfc.so (the CUDA kernels + the C ABI), in-tree.

nvcc cross-compiles for sm_103a only; translation units compile in parallel
and are rebuilt when a source or header is newer than the library.  Output:
xpfc_cuda_gb300/_lib/libxpfc.so (git-ignored).
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libxpfc.so")
# XPFC_BUILD_CHECKED=1 builds the self-checking diagnostics library instead
# (every step-kernel access checked against the registered buffers), into
# its own objects and libxpfc_checked.so
CHECKED = os.environ.get("XPFC_BUILD_CHECKED") == "1"
if CHECKED:
    OUT = os.path.join(OUT, "checked")
    LIB = os.path.join(HERE, "_lib", "libxpfc_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def _units():
    cu = ["-std=c++17", "-O3", "-lineinfo", "-DNDEBUG", "-Xcompiler", "-fPIC,-ffp-contract=off"] + ARCH
    if CHECKED:
        cu = cu + ["-DXPFC_CHECKED"]
    return [
        ("launch_f32_p1.o", [nvcc()] + cu + ["-DXPFC_PART=1", "-c", os.path.join(CSRC, "xpfc_launch_f32.cu")]),
        ("launch_f32_p2.o", [nvcc()] + cu + ["-DXPFC_PART=2", "-c", os.path.join(CSRC, "xpfc_launch_f32.cu")]),
        ("launch_f64_p1.o", [nvcc()] + cu + ["-DXPFC_PART=1", "-c", os.path.join(CSRC, "xpfc_launch_f64.cu")]),
        ("launch_f64_p2.o", [nvcc()] + cu + ["-DXPFC_PART=2", "-c", os.path.join(CSRC, "xpfc_launch_f64.cu")]),
        ("capi.o", [nvcc()] + cu + ["-c", os.path.join(CSRC, "xpfc_capi.cu")]),
        ("noalloc.o", [nvcc()] + cu + ["-c", os.path.join(CSRC, "xpfc_noalloc.cu")]),
        ("host.o", ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall",
                    "-c", os.path.join(CSRC, "xpfc_host.cpp")]),
    ]


def _newest_source():
    files = glob.glob(os.path.join(CSRC, "*")) + glob.glob(os.path.join(REPO, "include", "*.h"))
    return max(os.path.getmtime(f) for f in files)


def build(force=False, verbose=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_source():
        return LIB
    units = _units()
    newest = _newest_source()

    def run(unit):
        obj, cmd = unit
        path = os.path.join(OUT, obj)
        if not force and os.path.exists(path) and os.path.getmtime(path) >= newest:
            return path
        full = cmd + ["-o", path + ".tmp"]
        r = subprocess.run(full, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(full), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        os.replace(path + ".tmp", path)
        return path

    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(run, units))
    link = [nvcc(), "-shared"] + ARCH + ["-Xcompiler", "-fPIC"] + objs + ["-o", LIB + ".tmp"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s%s" % (" ".join(link), r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
