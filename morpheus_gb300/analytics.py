"""Matrix analytics with the reference's names (core/src/Morpheus_MatrixAnalytics.hpp:85-261),
computed on the GPU in one pass (analytics.cu).  std_nnnz is returned as a
float (the reference truncates it to an integer)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from .algorithms import _stream_handle
from .containers import CSR_FORMAT, CsrMatrix, DynamicMatrix, _Matrix

NFEATURES = 12
FEATURE_NAMES = ["log2_nrows", "log2_nnz", "mean_row", "cv_row", "log2_max_row", "min_row", "log2_ndiags",
                 "log2_dia_fill", "true_diag_share", "log2_ell_fill", "hyb_coo_share", "rel_bandwidth"]


def _as_csr(A: _Matrix) -> CsrMatrix:
    if isinstance(A, DynamicMatrix):
        A = A.active()
    if A.FORMAT == CSR_FORMAT:
        return A
    from .convert import from_coo, to_coo
    return from_coo(to_coo(A), CSR_FORMAT)


def analyze(A: _Matrix, stream=None) -> dict:
    M = _as_csr(A)
    out = (C.c_double * 14)()
    d = M._desc()
    _lib.call("mgb_analytics_csr", C.byref(d), out, _stream_handle(stream))
    keys = ["average_nnnz", "density", "max_nnnz", "min_nnnz", "std_nnnz", "count_diagonals",
            "count_true_diagonals", "true_diagonal_nnz", "bandwidth", "hyb_coo_nnz",
            "dia_feasible", "ell_feasible", "hyb_feasible", "hdc_feasible"]
    return dict(zip(keys, list(out)))


def features(A: _Matrix, stream=None) -> tuple[np.ndarray, np.ndarray]:
    """(12 float32 selector features, 6-byte feasibility mask in formats_e order)."""
    M = _as_csr(A)
    f = (C.c_float * NFEATURES)()
    m = (C.c_uint8 * 6)()
    d = M._desc()
    _lib.call("mgb_features_csr", C.byref(d), f, m, _stream_handle(stream))
    return np.array(list(f), dtype=np.float32), np.array(list(m), dtype=np.uint8)


def average_nnnz(A) -> float: return analyze(A)["average_nnnz"]
def density(A) -> float: return analyze(A)["density"]
def max_nnnz(A) -> int: return int(analyze(A)["max_nnnz"])
def min_nnnz(A) -> int: return int(analyze(A)["min_nnnz"])
def std_nnnz(A) -> float: return analyze(A)["std_nnnz"]
def count_diagonals(A) -> int: return int(analyze(A)["count_diagonals"])
def count_true_diagonals(A) -> int: return int(analyze(A)["count_true_diagonals"])
