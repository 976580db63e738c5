"""CPU: the C-ABI library builds for sm_103a, loads without a GPU, exports every
symbol include/mgb.h declares, and rejects bad arguments before touching CUDA."""
import ctypes as C
import os
import re

import pytest

from morpheus_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mgb.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mgb_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(lib_built):
    lib = C.CDLL(lib_built)
    missing = [s for s in header_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_bindings_cover_header(lib_built):
    assert set(_lib.declared_symbols()) == set(header_symbols())


def test_status_strings_and_version(lib_built):
    lib = _lib.load()
    assert lib.mgb_version() >= 100
    assert b"FormatConversionException" in lib.mgb_status_string(2)
    assert lib.mgb_status_string(0) == b"MGB_SUCCESS"


@pytest.mark.parametrize("fmt", ["csr", "coo", "dia", "ell", "hyb", "hdc"])
@pytest.mark.parametrize("dt", ["f64", "f32"])
def test_null_descriptor_is_rejected(lib_built, fmt, dt):
    lib = _lib.load()
    fn = getattr(lib, f"mgb_spmv_{fmt}_{dt}")
    assert fn(None, None, None, 1, None) == 8  # MGB_ERR_BAD_ARGUMENT


def test_negative_sizes_rejected(lib_built):
    lib = _lib.load()
    d = _lib.Csr(-1, 4, 0, None, None, None)
    assert lib.mgb_spmv_csr_f64(C.byref(d), None, None, 1, None) == 8
    assert lib.mgb_waxpby_f64(-5, 1.0, None, 1.0, None, None, None) == 8
    out = C.c_double()
    assert lib.mgb_dot_f64(10, None, None, C.byref(out), None) != 0


def test_empty_matrix_is_a_noop_without_gpu(lib_built):
    lib = _lib.load()
    d = _lib.Csr(0, 0, 0, None, None, None)
    assert lib.mgb_spmv_csr_f64(C.byref(d), None, None, 1, None) == 0


def test_size_limits_rejected_before_any_device_work(lib_built):
    """int32 indices: matrices past the limits are refused up front
    (MGB_ERR_INVALID_INPUT) instead of overflowing inside a kernel."""
    lib = _lib.load()
    fake = C.c_void_p(16)  # never dereferenced: the size checks come first
    big = _lib.Csr(10, 10, (1 << 31) - 100, fake, fake, fake)
    assert lib.mgb_spmv_csr_f64(C.byref(big), fake, fake, 1, None) == 3
    assert lib.mgb_spmv_csr_variant_f64(C.byref(big), fake, fake, 1, 2, None) == 3
    coo = _lib.Coo(1 << 31, 10, 5, fake, fake, fake)
    assert lib.mgb_spmv_coo_f64(C.byref(coo), fake, fake, 1, None) == 3
    bad_variant = _lib.Csr(10, 10, 5, fake, fake, fake)
    assert lib.mgb_spmv_csr_variant_f64(C.byref(bad_variant), fake, fake, 1, 7, None) == 8
    out = C.c_int64()
    assert lib.mgb_spmv_csr_host_workspace_bytes(C.byref(bad_variant), 3, C.byref(out)) == 8
    assert lib.mgb_spmv_csr_host_workspace_bytes(C.byref(bad_variant), 8, C.byref(out)) == 0 and out.value > 0


def test_null_pointers_with_nonempty_sizes_rejected(lib_built):
    lib = _lib.load()
    d = _lib.Csr(10, 10, 5, None, None, None)
    assert lib.mgb_spmv_csr_f64(C.byref(d), None, None, 1, None) == 8
    assert lib.mgb_spmv_dot_csr_f64(C.byref(d), None, None, 1, 1, None, None) == 8
    coo = _lib.Coo(10, 10, 5, None, None, None)
    assert lib.mgb_spmv_coo_f64(C.byref(coo), None, None, 1, None) == 8


def test_chunk_plan_sizes_and_arguments_without_gpu(lib_built):
    """The chunk plan's size depends on the GPU's SM count: without a device
    the size query is MGB_ERR_CUDA (no guessed SM count); a missing plan, a
    plan of the wrong size, or a plan for another kernel is refused before
    any device work.  (The sizes themselves are checked on the GPU.)"""
    import torch
    lib = _lib.load()
    n = C.c_int64()
    d = _lib.Csr(2_000_000, 2_000_000, 30_000_000, None, None, None)
    if not torch.cuda.is_available():
        assert lib.mgb_csr_plan_entries(C.byref(d), C.byref(n)) == 6  # MGB_ERR_CUDA
        assert "cuda" in lib.mgb_last_cuda_error_string().decode().lower()
    n.value = 30_000_000 // 2048 + 2
    bad = _lib.Csr(-1, 4, 0, None, None, None)
    assert lib.mgb_csr_plan_entries(C.byref(bad), C.byref(n)) == 8
    assert lib.mgb_csr_plan_entries(None, C.byref(n)) == 8
    fake = C.c_void_p(256)  # never dereferenced: the size checks come first
    df = _lib.Csr(2_000_000, 2_000_000, 30_000_000, fake, fake, fake)
    assert lib.mgb_csr_plan(C.byref(df), None, n.value, None) == 8
    assert lib.mgb_csr_plan(C.byref(df), fake, 10, None) == 8
    assert lib.mgb_spmv_csr_planned_f64(C.byref(df), None, 10, fake, fake, 1, None) == 8
    assert lib.mgb_spmv_csr_planned_f32(C.byref(df), fake, 10, fake, fake, 1, None) == 8
