"""Generate the golden vectors in tests/golden/ from LC2500/XPFC_CUDA itself.

Builds oracle/_ref/ref_harness (oracle/ref/Makefile: the reference's own host
code and kernel bodies compiled with g++ from the reference tree) and runs it on
the pfc.input decks below, each in a scratch directory.  The outputs are stored
as small .npz fixtures that the CPU tests compare the oracle against, so the
oracle is pinned to the reference's behaviour (2-D, square grids, the
reference's hard-coded two-peak sum DCF).

Usage:  python tests/golden/make_golden.py [--ref /path/to/reference]
The reference tree is only needed here; the fixtures are committed.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REFDIR = os.path.join(REPO, "oracle", "ref")
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")


def deck(psi0, s, a_in, b_in, eps, Mo, Lx, Ly, Mx, My, t, dt, t_sample, iconfig,
         A10=0.2, A11=0.1, Atri=0.3, iseed=0, ishape=0, h=4.0, k=4.0, roa=2.0):
    # pfc.input line layout of read_input.cu:19-115 (text after each value is ignored)
    return (f"1 no_val\n{psi0} {s} psi_0 s\n{a_in} {b_in} {eps} {Mo} a b eps Mo\n\n"
            f"{Lx} {Ly} Lx Ly\n{Mx} {My} Mx My\n\n{t} t\n{dt} dt\n{t_sample} t_sample\n\n"
            f"{iconfig} iconfig\n{A10} {A11} A_10 A_11\n{Atri} A_tri\n\n{iseed} iseed\n{ishape} ishape\n"
            f"{h} {k} {roa} h k roa\n")


def vtk_text(values, nx, ny, spacing):
    # legacy ASCII STRUCTURED_POINTS as write_vtk.cu:12-29 lays it out, full precision
    head = ("# vtk DataFile Version 3.0\nDensity Data\nASCII\nDATASET STRUCTURED_POINTS\n"
            f"DIMENSIONS {nx} {ny} 1\nORIGIN 0 0 0\nSPACING {spacing} {spacing} 1\n"
            f"POINT_DATA {nx * ny}\nSCALARS DensityData float\nLOOKUP_TABLE default\n")
    return head + "".join(f"{v:.17g}\n" for v in values)


def cases():
    rng = np.random.default_rng(20251203)
    vtk64 = 0.05 + 0.1 * rng.standard_normal(64 * 64)
    return [
        ("tri32_gauss", deck(0.05, 0.25, 1, 3, 0.1, 1, 8, 8, 32, 32, 20, 0.25, 5, 0,
                             iseed=1, ishape=1, h=4.0, k=4.0, roa=6.0), None, True),
        ("sq32_circle", deck(0.1, 0.22, 1.2, 3, 0, 1, 8, 8, 32, 32, 20, 0.3, 5, 1,
                             iseed=1, ishape=0, h=4.0, k=4.0, roa=2.5), None, False),
        ("liq16", deck(0.07, 0.2, 1, 3, 0, 1, 4, 4, 16, 16, 10, 1, 5, 2), None, True),
        ("vtk64_restart", deck(-0.05, 0.22, 1, 3, 0.05, 1.5, 8, 8, 64, 64, 15, 0.5, 5, 10),
         vtk64, False),
    ]


def parse_kv(path):
    out = {}
    for line in open(path):
        k, v = line.split()
        out[k] = float(v)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("XPFC_REFERENCE"),
                    help="the reference tree (or XPFC_REFERENCE)")
    args = ap.parse_args()
    if not args.ref:
        ap.error("give --ref or set XPFC_REFERENCE")
    subprocess.run(["make", "-s", "-C", REFDIR, f"REF={args.ref}"], check=True)
    for name, text, vtk_in, keep_vtk in cases():
        with tempfile.TemporaryDirectory() as d:
            with open(os.path.join(d, "pfc.input"), "w") as f:
                f.write(text)
            if vtk_in is not None:
                with open(os.path.join(d, "initial_density_field.vtk"), "w") as f:
                    f.write(vtk_text(vtk_in, 64, 64, 0.125))
            r = subprocess.run([HARNESS], cwd=d, capture_output=True, text=True)
            if r.returncode != 0:
                print(r.stdout[-2000:], r.stderr[-2000:])
                sys.exit(f"harness failed for {name}")
            p = parse_kv(os.path.join(d, "ref_params.txt"))
            M2 = int(p["Mx"] * p["My"])
            rd = lambda n: np.fromfile(os.path.join(d, n), dtype=np.float64, count=M2)
            F, RMS, FINAL = [], [], []
            for line in open(os.path.join(d, "ref_diag.txt")):
                tag, it, val = line.split()
                (F if tag == "F" else RMS if tag == "RMS" else FINAL).append((int(it), float(val)))
            extra = {}
            if keep_vtk:
                extra["vtk0"] = np.frombuffer(open(os.path.join(d, "density_data0.vtk"), "rb").read(),
                                              dtype=np.uint8)
            if vtk_in is not None:
                extra["vtk_in"] = vtk_in
            np.savez_compressed(
                os.path.join(HERE, f"{name}.npz"),
                deck=np.frombuffer(text.encode(), dtype=np.uint8),
                params=np.frombuffer(json.dumps(p).encode(), dtype=np.uint8),
                k2=rd("ref_k2.bin"), c2=rd("ref_c2.bin"), psi0=rd("ref_psi0.bin"),
                psi_final=rd("ref_psi_final.bin"),
                F=np.array(F, dtype=np.float64).reshape(-1, 2),
                RMS=np.array(RMS, dtype=np.float64).reshape(-1, 2),
                FINAL=np.array(FINAL, dtype=np.float64).reshape(-1, 2),
                **extra)
            print(name, "steps", p["N_t_steps"], "F", F[:2], "...", FINAL)


if __name__ == "__main__":
    main()
