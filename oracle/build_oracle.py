"""Build recipe for the CPU oracle library (oracle/_build/libtg_oracle.so).

Plain gcc, no FMA contraction and no fast-math, so the C restatement rounds like the Python source
it restates. OpenMP parallelises the walk and brute force over groups/targets for the timed CPU
baseline; results do not depend on the thread count.
"""

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtg_oracle.so")
SRCS = [os.path.join(HERE, f) for f in ("tg_oracle.c", "tg_oracle_corr.c", "tg_oracle.h")]


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(f) for f in SRCS):
        return LIB
    cmd = [
        "gcc", "-O2", "-fno-fast-math", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
        "-Wall", "-o", LIB + ".tmp", *[f for f in SRCS if f.endswith(".c")], "-lm",
    ]
    if verbose:
        print(" ".join(cmd), file=sys.stderr)
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
