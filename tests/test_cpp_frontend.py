"""The C++17 front end (include/Morpheus_GB300.hpp): tests/cpp/test_frontend.cpp
is compiled against the library and the oracle on CPU (the header and the C ABI
agree, the program links), and run on the GPU, where it checks multiply,
convert, activate, sort, dot, reduce and waxpby against the oracle."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_frontend.cpp")


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.isdir(os.path.join(c, "include")):
            return c
    pytest.skip("CUDA toolkit headers not found")


def _build(out, lib_built, oracle_built):
    cuda = _cuda_home()
    libdir = os.path.dirname(os.path.abspath(lib_built))
    orcdir = os.path.dirname(os.path.abspath(oracle_built))
    cudalib = next((d for d in (os.path.join(cuda, "lib64"), os.path.join(cuda, "lib"),
                                os.path.join(cuda, "targets", "sbsa-linux", "lib"))
                    if os.path.isdir(d)), os.path.join(cuda, "lib64"))
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda, "include"), SRC, "-o", out,
           "-L", libdir, "-lmorpheus_gb300", "-L", orcdir, "-loracle", "-L", cudalib, "-lcudart",
           f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{orcdir}", f"-Wl,-rpath,{cudalib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    return out


def test_frontend_compiles_and_links(lib_built, oracle_built, tmp_path):
    _build(str(tmp_path / "test_frontend"), lib_built, oracle_built)


@pytest.mark.gpu
def test_frontend_on_gpu(cuda, oracle_built, lib_built, tmp_path):
    exe = _build(str(tmp_path / "test_frontend"), lib_built, oracle_built)
    weights = os.path.join(ROOT, "morpheus_gb300", "selector_weights.bin")
    r = subprocess.run([exe, str(tmp_path), weights], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert ", 0 failed" in r.stdout
