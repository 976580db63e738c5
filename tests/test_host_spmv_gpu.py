"""CSR SpMV on host-resident data (mgb_spmv_csr_host_*, multiply_host):
block-pipelined copies and kernels give the oracle's result for every block
count, both kernels, init / accumulate, pinned and pageable buffers."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import golden, rel_err
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _host_csr(hm, pin):
    A = mgb.matrix_from_host(hm, device="cpu")
    if pin:
        A._ro, A._ci, A._v = A._ro.pin_memory(), A._ci.pin_memory(), A._v.pin_memory()
    return A


def _check(hm, dtype, init, nblocks, pin, variant=None):
    A = _host_csr(hm, pin)
    if variant is not None:
        A._variant = variant
    x = torch.from_numpy(gen.x_vector(hm["ncols"], seed=1, dtype=dtype))
    y0 = gen.x_vector(hm["nrows"], seed=2, dtype=dtype)
    y = torch.from_numpy(y0.copy())
    if pin:
        x, y = x.pin_memory(), y.pin_memory()
    mgb.multiply_host(A, x, y, init=init, nblocks=nblocks)
    h64 = {k: (v.astype(np.float64) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v) for k, v in hm.items()}
    ref = O.OracleMatrix.from_host(h64).multiply(x.numpy().astype(np.float64), y0.astype(np.float64), init=init)
    if dtype == np.float64:
        assert rel_err(y.numpy(), ref) <= 1e-12
    else:
        habs = {k: (np.abs(v) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v) for k, v in h64.items()}
        scale = O.OracleMatrix.from_host(habs).multiply(np.abs(x.numpy().astype(np.float64)),
                                                        np.abs(y0.astype(np.float64)), init=init)
        assert np.linalg.norm(y.numpy().astype(np.float64) - ref) <= 1e-5 * max(np.linalg.norm(scale), 1e-300)


CASES = {
    "golden": lambda dt: {k: (v.astype(dt) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v)
                          for k, v in golden()["CSR"].items()},
    "power_law": lambda dt: gen.power_law(40000, seed=51, dtype=dt),
    "stencil": lambda dt: gen.stencil_27pt(22, seed=52, dtype=dt),
    "empty_rows": lambda dt: gen.random_csr(5000, 4000, 0.002, seed=53, dtype=dt, empty_row_frac=0.5),
    "long_rows": lambda dt: gen.random_lengths_csr(300, 60000, np.where(np.arange(300) % 37 == 0, 20000, 3),
                                                   seed=54, dtype=dt),
    "all_empty": lambda dt: gen.random_lengths_csr(100, 100, np.zeros(100, dtype=np.int64), seed=55, dtype=dt),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("nblocks", [0, 1, 3, 8])
def test_host_spmv_matches_oracle(cuda, case, dtype, nblocks):
    hm = CASES[case](dtype)
    for init in (True, False):
        _check(hm, dtype, init, nblocks, pin=True)


@pytest.mark.parametrize("variant", [mgb.CSR_SEGMENTS, mgb.CSR_ROWS, mgb.CSR_SPLIT, mgb.CSR_ROWS_GATHER])
def test_host_spmv_every_kernel_and_pageable(cuda, variant):
    hm = gen.power_law(20000, seed=56)
    _check(hm, np.float64, True, 4, pin=False, variant=variant)
    _check(gen.laplacian_2d(70), np.float64, False, 5, pin=True, variant=variant)


def test_host_spmv_rejects_device_data(cuda):
    A = mgb.matrix_from_host(golden()["CSR"], device="cuda")
    with pytest.raises(mgb.InvalidInputException):
        mgb.multiply_host(A, torch.zeros(10, dtype=torch.float64), torch.zeros(10, dtype=torch.float64))
    H = mgb.matrix_from_host(golden()["CSR"], device="cpu")
    with pytest.raises(mgb.InvalidInputException):
        mgb.multiply_host(H, torch.zeros(10, dtype=torch.float64, device="cuda"), torch.zeros(10, dtype=torch.float64))
