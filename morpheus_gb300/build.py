"""Build recipe for the morpheus-gb300 CUDA library (sm_103a only).

Compiles every ``csrc/*.cu`` translation unit in parallel with nvcc and links
them into ``morpheus_gb300/libmorpheus_gb300.so`` (a plain C-ABI shared library,
CUDA runtime linked statically, no PyTorch dependency).  Objects are rebuilt
only when a source, a header or the flags change.

    python -m morpheus_gb300.build          # build (incremental)
    python -m morpheus_gb300.build --force  # rebuild everything
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD_DIR = os.path.join(HERE, "_build")
LIB_NAME = "libmorpheus_gb300.so"
LIB_PATH = os.path.join(HERE, LIB_NAME)

NVCC = os.environ.get("MGB_NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC",
    "-I",
    INCLUDE,
]


def _flags_digest() -> str:
    return hashlib.sha1(" ".join([NVCC] + NVCC_FLAGS).encode()).hexdigest()[:12]


def _newest(paths) -> float:
    return max((os.path.getmtime(p) for p in paths), default=0.0)


def _compile(src: str, obj: str, verbose: bool) -> None:
    cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{res.stdout}\n{res.stderr}")


def build_library(force: bool = False, verbose: bool = False) -> str:
    """Compile and link the library; return the path of the shared object."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    digest = _flags_digest()
    stamp = os.path.join(BUILD_DIR, "flags.txt")
    old = open(stamp).read().strip() if os.path.exists(stamp) else ""
    if old != digest:
        force = True
    newest_header = _newest(headers)
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD_DIR, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if force or not os.path.exists(obj) or os.path.getmtime(obj) < max(
            os.path.getmtime(src), newest_header
        ):
            jobs.append((src, obj))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 4))
        with cf.ThreadPoolExecutor(workers) as ex:
            list(ex.map(lambda j: _compile(j[0], j[1], verbose), jobs))
    if force or jobs or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < _newest(objs):
        tmp = LIB_PATH + ".tmp"
        cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB_PATH


if __name__ == "__main__":
    print(build_library(force="--force" in sys.argv, verbose="-v" in sys.argv))
