"""GPU: the allocation-free COO SpMV entry point (mgb_spmv_coo_f64_noalloc).

Some callers cannot allocate device memory while they run -- real-time loops
of a host that forbids allocation once running, hosts that reserve all device
memory up front, plugins whose host process owns the allocator.  For
them the library offers one COO SpMV whose carry buffer is a fixed 4 MiB
device array compiled into the library instead of stream-ordered scratch.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  It calls the entry point
through the C ABI (ctypes) and compares it with the allocating entry point
mgb_spmv_coo_f64 and with the oracle's Serial COO multiply on two calls in a
row; the second call reuses the array with the first call's carries still in
it.  One matrix has a row that spans several 2048-entry chunks, so carries of
one row come from several chunks.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import rel_err
from morpheus_gb300 import _lib
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MAX_NNZ = 357_892_096  # the documented capacity of the fixed scratch array


def _spmv(name, A, x, y, init):
    lib = _lib.load()
    d = A._desc()
    st = getattr(lib, name)(C.byref(d), C.c_void_p(x.data_ptr()), C.c_void_p(y.data_ptr()), init,
                            C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.mgb_status_string(st)


def _long_row_case():
    """Short rows around one row of 9,000 entries (spans several chunks)."""
    lens = np.where(np.arange(3000) % 4 == 0, 3, 0)
    lens[1234] = 9000
    return gen.random_lengths_csr(3000, 20000, lens, seed=23)


def test_noalloc_matches_allocating_entry_point_and_oracle(cuda):
    cases = [gen.power_law(200_000, seed=21), _long_row_case(),
             gen.random_csr(5000, 7000, 0.002, seed=22, empty_row_frac=0.3)]
    for call, hm in enumerate(cases):  # calls in a row, different matrices
        coo = gen.csr_to_coo_host(hm)
        A = mgb.matrix_from_host(coo, device="cuda")
        x_np = gen.x_vector(hm["ncols"], seed=call)
        y0_np = gen.x_vector(hm["nrows"], seed=call + 7)
        x = torch.from_numpy(x_np).cuda()
        y0 = torch.from_numpy(y0_np).cuda()
        om = O.OracleMatrix.from_host(coo)
        for init in (1, 0):
            y_ref, y_new = y0.clone(), y0.clone()
            _spmv("mgb_spmv_coo_f64", A, x, y_ref, init)
            _spmv("mgb_spmv_coo_f64_noalloc", A, x, y_new, init)
            torch.cuda.synchronize()
            got = y_new.cpu().numpy()
            assert rel_err(got, y_ref.cpu().numpy()) <= 1e-12
            want = om.multiply(x_np, y0_np.copy(), init=bool(init))
            assert rel_err(got, want) <= 1e-12


def test_noalloc_rejects_matrices_beyond_capacity(cuda):
    lib = _lib.load()
    # sizes only: the capacity check runs before any pointer is used
    d = _lib.Coo(10, 10, MAX_NNZ + 1, None, None, None)
    assert lib.mgb_spmv_coo_f64_noalloc(C.byref(d), None, None, 1, None) == 3  # MGB_ERR_INVALID_INPUT
    # exactly at the capacity the size check passes (no rows: nothing runs)
    d_max = _lib.Coo(0, 10, MAX_NNZ, None, None, None)
    assert lib.mgb_spmv_coo_f64_noalloc(C.byref(d_max), None, None, 1, None) == 0
    d_ok = _lib.Coo(10, 10, 0, None, None, None)
    y = torch.ones(10, dtype=torch.float64, device="cuda")
    assert lib.mgb_spmv_coo_f64_noalloc(C.byref(d_ok), None, C.c_void_p(y.data_ptr()), 1, None) == 0
    torch.cuda.synchronize()
    assert torch.count_nonzero(y).item() == 0
