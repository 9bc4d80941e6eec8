"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/hss_oracle.cpp into oracle/_build/libhss_oracle.so with g++ and
OpenMP.  `-ffp-contract=off` keeps every multiply and add separately rounded,
as the Fortran reference build (`-fp-model precise`) does.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libhss_oracle.so")
SRC = [os.path.join(HERE, "hss_oracle.cpp")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    newest = max(os.path.getmtime(p) for p in SRC + [os.path.join(HERE, "hss_oracle.h")])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-o", LIB] + SRC + ["-ldl"]
    if verbose:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
