"""Matrix analytics with the reference's names (core/src/Morpheus_MatrixAnalytics.hpp:85-261),
computed on the GPU in one pass (analytics.cu, analytics_counts.cu) over the
active container, whatever its format: nothing is converted.  The statistics
and selector features describe the entries of the matrix's COO form, so they
do not depend on the active format; count_nnz_per_row / count_nnz_per_diagonal
keep the reference's per-format semantics (a DIA row counts its in-range
diagonal slots, for instance).  std_nnnz is returned as a float (the
reference truncates it to an integer)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .algorithms import _stream_handle
from .containers import (COO_FORMAT, CSR_FORMAT, DIA_FORMAT, ELL_FORMAT, HDC_FORMAT, HYB_FORMAT, DynamicMatrix,
                         _Matrix)
from .exceptions import InvalidInputException, NotImplementedException

NFEATURES = 12
FEATURE_NAMES = ["log2_nrows", "log2_nnz", "mean_row", "cv_row", "log2_max_row", "min_row", "log2_ndiags",
                 "log2_dia_fill", "true_diag_share", "log2_ell_fill", "hyb_coo_share", "rel_bandwidth"]
_NAME = {COO_FORMAT: "coo", CSR_FORMAT: "csr", DIA_FORMAT: "dia", ELL_FORMAT: "ell", HYB_FORMAT: "hyb",
         HDC_FORMAT: "hdc"}


def _active(A: _Matrix) -> _Matrix:
    M = A.active() if isinstance(A, DynamicMatrix) else A
    if M.device.type != "cuda":
        raise NotImplementedException("analytics run on the device; copy the matrix to a CUDA device first")
    return M


def _typed(M: _Matrix) -> str:
    from .algorithms import _suffix
    return "_" + _suffix(M.dtype)


def _entry(base: str, M: _Matrix, typed_formats) -> str:
    return f"{base}_{_NAME[M.FORMAT]}" + (_typed(M) if M.FORMAT in typed_formats else "")


def analyze(A: _Matrix, stream=None) -> dict:
    M = _active(A)
    out = (C.c_double * 14)()
    d = M._desc()
    _lib.call(_entry("mgb_analytics", M, (DIA_FORMAT, HDC_FORMAT)), C.byref(d), out, _stream_handle(stream))
    keys = ["average_nnnz", "density", "max_nnnz", "min_nnnz", "std_nnnz", "count_diagonals",
            "count_true_diagonals", "true_diagonal_nnz", "bandwidth", "hyb_coo_nnz",
            "dia_feasible", "ell_feasible", "hyb_feasible", "hdc_feasible"]
    return dict(zip(keys, list(out)))


def features(A: _Matrix, stream=None) -> tuple[np.ndarray, np.ndarray]:
    """(12 float32 selector features, 6-byte feasibility mask in formats_e order),
    computed from the active container in place."""
    M = _active(A)
    f = (C.c_float * NFEATURES)()
    m = (C.c_uint8 * 6)()
    d = M._desc()
    _lib.call(_entry("mgb_features", M, (DIA_FORMAT, HDC_FORMAT)), C.byref(d), f, m, _stream_handle(stream))
    return np.array(list(f), dtype=np.float32), np.array(list(m), dtype=np.uint8)


def average_nnnz(A) -> float: return analyze(A)["average_nnnz"]
def density(A) -> float: return analyze(A)["density"]
def max_nnnz(A) -> int: return int(analyze(A)["max_nnnz"])
def min_nnnz(A) -> int: return int(analyze(A)["min_nnnz"])
def std_nnnz(A) -> float: return analyze(A)["std_nnnz"]


def _counts(A: _Matrix, what: str, n: int, out, init: bool, stream) -> torch.Tensor:
    M = _active(A)
    if out is None:
        out = torch.zeros(n, dtype=torch.int32, device=M.device)
        init = True
    if out.dtype != torch.int32 or out.numel() < n or not out.is_contiguous() or out.device.type != "cuda":
        raise InvalidInputException(f"{what}: out must be a contiguous CUDA int32 vector of {n} entries")
    typed = (DIA_FORMAT, ELL_FORMAT, HYB_FORMAT, HDC_FORMAT) if what == "diagonal" else ()
    d = M._desc()
    _lib.call(_entry(f"mgb_count_nnz_per_{what}", M, typed), C.byref(d), C.c_void_p(out.data_ptr()),
              1 if init else 0, _stream_handle(stream))
    return out


def count_nnz_per_row(A: _Matrix, out: torch.Tensor | None = None, init: bool = True, stream=None) -> torch.Tensor:
    """core/src/Morpheus_MatrixAnalytics.hpp:112-124: out[i] (+)= entries of row i."""
    return _counts(A, "row", A.nrows(), out, init, stream)


def count_nnz_per_diagonal(A: _Matrix, out: torch.Tensor | None = None, init: bool = True,
                           stream=None) -> torch.Tensor:
    """core/src/Morpheus_MatrixAnalytics.hpp:206-218: out[c - r + nrows - 1] (+)= 1."""
    return _counts(A, "diagonal", A.nrows() + A.ncols() - 1, out, init, stream)


def count_nnz(vec: torch.Tensor, threshold: int = 0, stream=None) -> int:
    """core/src/Morpheus_VectorAnalytics.hpp:124: entries > threshold and != 0."""
    if vec.dtype != torch.int32 or not vec.is_contiguous() or vec.device.type != "cuda":
        raise InvalidInputException("count_nnz: a contiguous CUDA int32 vector is required")
    out = C.c_int64()
    _lib.call("mgb_count_nnz_vector", C.c_void_p(vec.data_ptr()), vec.numel(), int(threshold), C.byref(out),
              _stream_handle(stream))
    return out.value


def count_diagonals(A: _Matrix) -> int:
    """core/src/Morpheus_MatrixAnalytics.hpp:220-243"""
    return count_nnz(count_nnz_per_diagonal(A), 0)


def count_true_diagonals(A: _Matrix, threshold: int) -> int:
    """core/src/Morpheus_MatrixAnalytics.hpp:245-261: diagonals with more than
    `threshold` entries."""
    return count_nnz(count_nnz_per_diagonal(A), threshold)
