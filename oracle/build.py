"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/gvom_oracle.c into oracle/_build/libgvom_oracle.so with
gcc, without contraction of multiply-adds (-ffp-contract=off), with OpenMP for
the timed multi-thread mode.  Portable C11: builds the same on x86_64 and
aarch64.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "gvom_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgvom_oracle.so")

CFLAGS = ["-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
          "-shared", "-Wall", "-Wextra"]


def build_oracle(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(__file__)):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose=True))
