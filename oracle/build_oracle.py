"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/rfmm_oracle.c`` into ``oracle/_build/librfmm_oracle.so`` with
IEEE single-precision semantics (no FMA contraction, no fast-math) and OpenMP.
The product library never links or loads this file.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "rfmm_oracle.c")
# The contract's transcendental functions, shared with the kernels.
MATH_DIR = os.path.join(os.path.dirname(HERE), "fmm-rainbow_gb300", "csrc")
MATH_H = os.path.join(MATH_DIR, "rfmm_math.h")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "librfmm_oracle.so")

CFLAGS = [
    "-O2",
    "-std=c11",
    "-fPIC",
    "-shared",
    "-fopenmp",
    "-ffp-contract=off",
    "-fno-fast-math",
    "-fno-finite-math-only",
    "-Wall",
    "-Wextra",
    "-Wno-unused-parameter",
]


def build(force: bool = False, quiet: bool = True) -> str:
    """Compile the oracle if it is missing or older than its source."""
    os.makedirs(OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)
            and os.path.getmtime(LIB) >= os.path.getmtime(MATH_H)
            and os.path.getmtime(LIB) >= os.path.getmtime(__file__)):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = ["gcc", *CFLAGS, "-I", MATH_DIR, SRC, "-o", tmp, "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    if res.stderr and not quiet:
        sys.stderr.write(res.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, quiet=False))
