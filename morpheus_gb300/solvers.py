"""Fused solver steps and conjugate gradients on the device (no reference
counterpart; built on the reference's multiply / dot / waxpby semantics,
core/src/Morpheus_Multiply.hpp:57-78, Morpheus_Dot.hpp:50-58,
Morpheus_WAXPBY.hpp:52-64).

    multiply_dot(A, x, y, init=True) -> device scalar   y = A*x and x.y in one pass
    waxpby_dot(n, alpha, x, beta, y, w) -> device scalar  w = alpha*x + beta*y and w.w
    cg(A, b, x, max_iters, rtol) -> (iterations, relative residual)

A must be a CsrMatrix (or a DynamicMatrix holding one) on the device; the CSR
kernel is the matrix's cached choice (CsrMatrix.kernel_variant()).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .algorithms import _stream_handle, _suffix, _vec
from .containers import CSR_FORMAT, DynamicMatrix
from .exceptions import InvalidInputException, NotImplementedException


def _csr(A):
    if isinstance(A, DynamicMatrix):
        A = A.active()
    if A.FORMAT != CSR_FORMAT:
        raise NotImplementedException("fused solver steps take a CsrMatrix")
    if A.device.type != "cuda":
        raise NotImplementedException("matrix lives in host memory (the library has no host path)")
    return A


def multiply_dot(A, x, y, init: bool = True, out: torch.Tensor | None = None, stream=None) -> torch.Tensor:
    """y = A*x (or y += A*x) and x[:nrows] . y, returned as a 1-element device tensor."""
    A = _csr(A)
    xt, yt = _vec(x), _vec(y)
    if xt.dtype != A.dtype or yt.dtype != A.dtype:
        raise InvalidInputException("x, y and A must share the value type")
    if xt.numel() < A.ncols() or yt.numel() < A.nrows():
        raise InvalidInputException("x or y too short for A")
    out = torch.empty(1, dtype=A.dtype, device=yt.device) if out is None else out
    d = A._desc()
    _lib.call(f"mgb_spmv_dot_csr_{_suffix(A.dtype)}", C.byref(d), C.c_void_p(xt.data_ptr()),
              C.c_void_p(yt.data_ptr()), 1 if init else 0, A.kernel_variant(), C.c_void_p(out.data_ptr()),
              _stream_handle(stream))
    return out


def waxpby_dot(n: int, alpha: float, x, beta: float, y, w, out: torch.Tensor | None = None,
               stream=None) -> torch.Tensor:
    """w = alpha*x + beta*y and w.w (1-element device tensor)."""
    xt, yt, wt = _vec(x), _vec(y), _vec(w)
    out = torch.empty(1, dtype=xt.dtype, device=xt.device) if out is None else out
    _lib.call(f"mgb_waxpby_dot_{_suffix(xt.dtype)}", int(n), alpha, C.c_void_p(xt.data_ptr()), beta,
              C.c_void_p(yt.data_ptr()), C.c_void_p(wt.data_ptr()), C.c_void_p(out.data_ptr()),
              _stream_handle(stream))
    return out


def cg(A, b, x, max_iters: int = 1000, rtol: float = 1e-10, stream=None) -> tuple[int, float]:
    """Conjugate gradients for an SPD CSR matrix; x holds the initial guess
    and receives the solution.  Returns (iterations, sqrt(r.r / b.b))."""
    A = _csr(A)
    bt, xt = _vec(b), _vec(x)
    if bt.dtype != A.dtype or xt.dtype != A.dtype:
        raise InvalidInputException("b, x and A must share the value type")
    if A.nrows() != A.ncols() or bt.numel() < A.nrows() or xt.numel() < A.nrows():
        raise InvalidInputException("cg needs a square matrix and vectors of its size")
    it, res = C.c_int64(), C.c_double()
    d = A._desc()
    _lib.call(f"mgb_cg_csr_{_suffix(A.dtype)}", C.byref(d), A.kernel_variant(), C.c_void_p(bt.data_ptr()),
              C.c_void_p(xt.data_ptr()), int(max_iters), float(rtol), C.byref(it), C.byref(res),
              _stream_handle(stream))
    return it.value, res.value
