"""Build recipe for the CPU oracle (test infrastructure, not product code).

Compiles oracle/xpfc_oracle.c into oracle/_build/liboracle.so with gcc.
-ffp-contract=off keeps x86 and aarch64 results identical (no FMA contraction).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False):
    src = os.path.join(HERE, "xpfc_oracle.c")
    hdr = os.path.join(HERE, "xpfc_oracle.h")
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-ffp-contract=off",
           "-std=c11", "-D_GNU_SOURCE", "-Wall", "-Wno-unused-variable",
           src, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True))
