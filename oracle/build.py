"""Build recipe for the CPU oracle (test infrastructure only).

    g++ -O2 -std=c++17 -fopenmp -ffp-contract=off -shared oracle.cpp -> _build/liboracle.so

-ffp-contract=off keeps every a*b+c a separately rounded multiply and add, as
in the reference's x86 builds, so the oracle gives the same bits on x86 and Arm.
The reference library itself is not built here: it needs Kokkos, which is not
installed, so there is nothing to put under oracle/_ref.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "oracle.cpp")
OUT_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "liboracle.so")
FLAGS = ["-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]


def build_oracle(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC):
        return LIB_PATH
    tmp = LIB_PATH + ".tmp"
    cmd = [os.environ.get("CXX", "g++")] + FLAGS + [SRC, "-o", tmp]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv, verbose="-v" in sys.argv))
