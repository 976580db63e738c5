"""Algorithm front-ends with the reference's names and argument meaning:

    multiply(A, x, y, init=True)       core/src/Morpheus_Multiply.hpp:57-78
    dot(n, x, y) -> scalar             core/src/Morpheus_Dot.hpp:50-58
    reduce(in, size) -> scalar         core/src/Morpheus_Reduction.hpp:46-52
    waxpby(n, alpha, x, beta, y, w)    core/src/Morpheus_WAXPBY.hpp:52-64

Every call goes to the sm_103a kernels through the C ABI.  Containers and
vectors must live on a CUDA device: host containers raise
NotImplementedException (the library has no CPU path).  Calls are issued on
torch's current CUDA stream unless `stream` is given; multiply and waxpby are
asynchronous, dot and reduce return a Python float (synchronising).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .containers import (COO_FORMAT, CSR_FORMAT, CSR_ROWS, CSR_SEGMENTS, CSR_SPLIT, DIA_FORMAT, ELL_FORMAT, HDC_FORMAT,
                         HYB_FORMAT, DynamicMatrix, _Matrix)
from .exceptions import InvalidInputException, NotImplementedException

_FMT_NAME = {COO_FORMAT: "coo", CSR_FORMAT: "csr", DIA_FORMAT: "dia", ELL_FORMAT: "ell",
             HYB_FORMAT: "hyb", HDC_FORMAT: "hdc"}


def _suffix(dtype) -> str:
    if dtype == torch.float64:
        return "f64"
    if dtype == torch.float32:
        return "f32"
    raise InvalidInputException(f"unsupported value type {dtype}")


def _stream_handle(stream) -> C.c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    if isinstance(stream, torch.cuda.Stream):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


def _vec(v) -> torch.Tensor:
    t = v.data if hasattr(v, "data") and not isinstance(v, torch.Tensor) else v
    if not isinstance(t, torch.Tensor):
        raise InvalidInputException("vectors must be torch tensors or DenseVector")
    if t.device.type != "cuda":
        raise NotImplementedException("vector is not on a CUDA device (no host path)")
    if not t.is_contiguous():
        raise InvalidInputException("vectors must be contiguous")
    return t


def _check_device(A: _Matrix) -> None:
    if A.device.type != "cuda":
        raise NotImplementedException(
            "matrix lives in host memory; copy it to the device first (the library has no host path)")


def multiply(A: _Matrix, x, y, init: bool = True, stream=None) -> None:
    """y = A*x (init) or y += A*x (not init), on the device."""
    if isinstance(A, DynamicMatrix):
        A = A.active()
    _check_device(A)
    xt, yt = _vec(x), _vec(y)
    if xt.dtype != A.dtype or yt.dtype != A.dtype:
        raise InvalidInputException("x, y and A must share the value type")
    if xt.numel() < A.ncols() or yt.numel() < A.nrows():
        raise InvalidInputException("x or y too short for A")
    desc = A._desc()
    if A.FORMAT == CSR_FORMAT:  # cached per matrix: kernel choice, and the chunk plan of the lane-segment kernel
        variant, sh = A.kernel_variant(), _stream_handle(stream)
        if variant == CSR_SEGMENTS:
            plan, entries = A.chunk_plan(sh)
            _lib.call(f"mgb_spmv_csr_planned_{_suffix(A.dtype)}", C.byref(desc), C.c_void_p(plan.data_ptr()),
                      entries, C.c_void_p(xt.data_ptr()), C.c_void_p(yt.data_ptr()), 1 if init else 0, sh)
        else:
            _lib.call(f"mgb_spmv_csr_variant_{_suffix(A.dtype)}", C.byref(desc), C.c_void_p(xt.data_ptr()),
                      C.c_void_p(yt.data_ptr()), 1 if init else 0, variant, sh)
        return
    name = f"mgb_spmv_{_FMT_NAME[A.FORMAT]}_{_suffix(A.dtype)}"
    _lib.call(name, C.byref(desc), C.c_void_p(xt.data_ptr()), C.c_void_p(yt.data_ptr()),
              1 if init else 0, _stream_handle(stream))


def host_kernel_variant(A) -> int:
    """CSR kernel choice for a host-resident CsrMatrix, by the rule of
    mgb_csr_choose_kernel (row-tile kernel when the longest row is <= 28 and
    <= 1.5 x mean + 2; split kernel when a row is longer than 8192 or rows
    average >= 512),
    computed once on the host and cached."""
    v = getattr(A, "_variant", None)
    if v is None:
        lens = (A.row_offsets()[1:] - A.row_offsets()[:-1]) if A.nrows() else None
        if lens is None or A.nnnz() == 0:
            v = CSR_SEGMENTS
        else:
            mx = int(lens.max().item())
            mean = A.nnnz() / A.nrows()
            v = CSR_ROWS if (32 * mx <= 896 and mx <= 1.5 * mean + 2.0) else CSR_SEGMENTS
            if mx > 8192 or mean >= 512:
                v = CSR_SPLIT
        A._variant = v
    return v


def multiply_host(A, x, y, init: bool = True, nblocks: int = 0, stream=None) -> None:
    """y = A*x (or y += A*x) for a CsrMatrix, x and y in HOST memory (pin them
    for overlap): the matrix goes to the GPU in row blocks that are
    multiplied while the next block is copied.  Synchronous."""
    if isinstance(A, DynamicMatrix):
        A = A.active()
    if A.FORMAT != CSR_FORMAT:
        raise NotImplementedException("multiply_host takes a CsrMatrix")
    if A.device.type != "cpu":
        raise InvalidInputException("multiply_host takes a host-resident matrix (use multiply for device data)")
    for t in (x, y):
        if not isinstance(t, torch.Tensor) or t.device.type != "cpu" or not t.is_contiguous():
            raise InvalidInputException("x and y must be contiguous host tensors")
    if x.dtype != A.dtype or y.dtype != A.dtype:
        raise InvalidInputException("x, y and A must share the value type")
    if x.numel() < A.ncols() or y.numel() < A.nrows():
        raise InvalidInputException("x or y too short for A")
    desc = A._desc()
    # the device workspace is kept with the matrix (no allocation per call)
    dev = torch.cuda.current_device()
    ws = getattr(A, "_host_ws", None)
    if ws is None or ws.device.index != dev:
        nb = C.c_int64()
        _lib.call("mgb_spmv_csr_host_workspace_bytes", C.byref(desc), A.dtype.itemsize, C.byref(nb))
        ws = A._host_ws = torch.empty(max(nb.value, 1), dtype=torch.uint8, device=f"cuda:{dev}")
    _lib.call(f"mgb_spmv_csr_host_{_suffix(A.dtype)}", C.byref(desc), C.c_void_p(x.data_ptr()),
              C.c_void_p(y.data_ptr()), 1 if init else 0, host_kernel_variant(A), int(nblocks),
              C.c_void_p(ws.data_ptr()), ws.numel(), _stream_handle(stream))


def dot(n: int, x, y, stream=None) -> float:
    xt, yt = _vec(x), _vec(y)
    sfx = _suffix(xt.dtype)
    out = C.c_double() if sfx == "f64" else C.c_float()
    yp = xt.data_ptr() if yt.data_ptr() == xt.data_ptr() else yt.data_ptr()
    _lib.call(f"mgb_dot_{sfx}", int(n), C.c_void_p(xt.data_ptr()), C.c_void_p(yp), C.byref(out),
              _stream_handle(stream))
    return out.value


def dot_async(n: int, x, y, result: torch.Tensor, stream=None) -> None:
    xt, yt, rt = _vec(x), _vec(y), _vec(result)
    _lib.call(f"mgb_dot_{_suffix(xt.dtype)}_async", int(n), C.c_void_p(xt.data_ptr()),
              C.c_void_p(yt.data_ptr()), C.c_void_p(rt.data_ptr()), _stream_handle(stream))


def reduce(x, size: int, stream=None) -> float:
    xt = _vec(x)
    sfx = _suffix(xt.dtype)
    out = C.c_double() if sfx == "f64" else C.c_float()
    _lib.call(f"mgb_reduce_{sfx}", C.c_void_p(xt.data_ptr()), int(size), C.byref(out),
              _stream_handle(stream))
    return out.value


def waxpby(n: int, alpha: float, x, beta: float, y, w, stream=None) -> None:
    xt, yt, wt = _vec(x), _vec(y), _vec(w)
    sfx = _suffix(xt.dtype)
    _lib.call(f"mgb_waxpby_{sfx}", int(n), alpha, C.c_void_p(xt.data_ptr()), beta,
              C.c_void_p(yt.data_ptr()), C.c_void_p(wt.data_ptr()), _stream_handle(stream))
