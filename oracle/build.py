"""Build the CPU oracle shared library (test infrastructure only).

``python oracle/build.py`` compiles ``oracle/pairs_oracle.c``,
``oracle/dmat_oracle.c`` and ``oracle/wick_oracle.c`` into ``oracle/_build/liboracle.so`` with FMA
contraction disabled, so the FP64 operation order is the one of picca's numba
kernels.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liboracle.so")


def build(force=False, quiet=True):
    """Compile the oracle if it is missing or older than its source."""
    srcs = [os.path.join(HERE, name) for name in ("pairs_oracle.c", "dmat_oracle.c", "wick_oracle.c")]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(src) for src in srcs)):
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-fno-fast-math", "-o", tmp] + srcs + ["-lm"]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, quiet=False))
