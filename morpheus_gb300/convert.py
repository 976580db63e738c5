"""Format conversion on the device, with the reference's API:

    convert(src, dst)          Morpheus::convert<ExecSpace>(src, dst)
                               (core/src/Morpheus_Convert.hpp:53-57): dst's
                               format is the target; dst is resized and filled.
    convert(dyn, fmt) -> conversion_error_e
                               in-place switch of a DynamicMatrix through a
                               temporary COO (core/src/Morpheus_Convert.hpp:88-141);
                               on failure the matrix keeps its format and data.
    sort_by_row_and_column(coo), is_sorted(coo)
                               impl/Coo/Serial/Morpheus_Sort_Impl.hpp:109-186

All work runs in the CUDA kernels of convert.cu; results are bit-identical to
the reference's Serial conversions (including its tie-breaks and quirks).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .algorithms import _stream_handle, _suffix
from .containers import (COO_FORMAT, CSR_FORMAT, DIA_FORMAT, ELL_FORMAT, HDC_FORMAT, HYB_FORMAT, NFORMATS,
                         CooMatrix, CsrMatrix, DiaMatrix, DynamicMatrix, EllMatrix, HdcMatrix, HybMatrix,
                         _Matrix, conversion_error_e, formats_e)
from .exceptions import MorpheusException, NotImplementedException

_NAME = {COO_FORMAT: "coo", CSR_FORMAT: "csr", DIA_FORMAT: "dia", ELL_FORMAT: "ell", HYB_FORMAT: "hyb",
         HDC_FORMAT: "hdc"}


def _dev_check(A: _Matrix) -> None:
    if A.device.type != "cuda":
        raise NotImplementedException("convert: containers must live on a CUDA device")


def _call(name, *args):
    _lib.call(name, *args)


def _i64():
    return C.c_int64()


def to_coo(A: _Matrix, stream=None) -> CooMatrix:
    """Any container -> a new COO container (the reference's X -> COO)."""
    if isinstance(A, DynamicMatrix):
        A = A.active()
    _dev_check(A)
    sfx = _suffix(A.dtype)
    if A.FORMAT == COO_FORMAT:
        return CooMatrix(A.nrows(), A.ncols(), A.nnnz(), A.row_indices().clone(), A.column_indices().clone(),
                         A.values().clone(), A.dtype, A.device)
    out = CooMatrix(A.nrows(), A.ncols(), A.nnnz(), dtype=A.dtype, device=A.device)
    sd, dd = A._desc(), out._desc()
    _call(f"mgb_convert_{_NAME[A.FORMAT]}_to_coo_{sfx}", C.byref(sd), C.byref(dd), _stream_handle(stream))
    return out


def from_coo(coo: CooMatrix, fmt: int, hyb_width: int = 0, stream=None) -> _Matrix:
    """COO -> a new container of format `fmt` (the reference's COO -> Y)."""
    _dev_check(coo)
    sfx = _suffix(coo.dtype)
    sh = _stream_handle(stream)
    sd = coo._desc()
    n, m, z, dt, dev = coo.nrows(), coo.ncols(), coo.nnnz(), coo.dtype, coo.device
    fmt = int(fmt)
    if fmt == COO_FORMAT:
        return to_coo(coo)
    if fmt == CSR_FORMAT:
        out = CsrMatrix(n, m, z, dtype=dt, device=dev)
    elif fmt == DIA_FORMAT:
        nd = _i64()
        _call("mgb_convert_coo_to_dia_plan", C.byref(sd), C.byref(nd), sh)
        out = DiaMatrix(n, m, z, nd.value, dtype=dt, device=dev)
    elif fmt == ELL_FORMAT:
        w = _i64()
        _call("mgb_convert_coo_to_ell_plan", C.byref(sd), C.byref(w), sh)
        out = EllMatrix(n, m, z, w.value, dtype=dt, device=dev)
    elif fmt == HYB_FORMAT:
        w, en, cn = _i64(), _i64(), _i64()
        _call("mgb_convert_coo_to_hyb_plan", C.byref(sd), int(hyb_width), C.byref(w), C.byref(en), C.byref(cn), sh)
        out = HybMatrix(EllMatrix(n, m, en.value, w.value, dtype=dt, device=dev),
                        CooMatrix(n, m, cn.value, dtype=dt, device=dev), dt, dev)
    elif fmt == HDC_FORMAT:
        nd, dn, cn = _i64(), _i64(), _i64()
        _call("mgb_convert_coo_to_hdc_plan", C.byref(sd), C.byref(nd), C.byref(dn), C.byref(cn), sh)
        out = HdcMatrix(DiaMatrix(n, m, dn.value, nd.value, dtype=dt, device=dev),
                        CsrMatrix(n, m, cn.value, dtype=dt, device=dev), dt, dev)
    else:
        raise NotImplementedException(f"format {fmt}")
    dd = out._desc()
    _call(f"mgb_convert_coo_to_{_NAME[fmt]}_{sfx}", C.byref(sd), C.byref(dd), sh)
    return out


def convert(src, dst, stream=None, hyb_width: int = 0):
    """convert(src, dst) fills container dst; convert(dyn, fmt) converts in place."""
    if isinstance(dst, (int, formats_e)) and not isinstance(dst, bool):
        return convert_inplace(src, dst, stream=stream, hyb_width=hyb_width)
    if isinstance(src, DynamicMatrix):
        src = src.active()
    target = dst.active_index() if isinstance(dst, DynamicMatrix) else dst.FORMAT
    if src.FORMAT == target:
        out = from_coo(to_coo(src), target, hyb_width=hyb_width) if target == COO_FORMAT else _deep_copy(src)
    else:
        tmp = src if src.FORMAT == COO_FORMAT else to_coo(src, stream)
        out = from_coo(tmp, target, hyb_width=hyb_width, stream=stream)
    if isinstance(dst, DynamicMatrix):
        dst.assign(out)
    else:
        dst.__dict__.update(out.__dict__)
    return dst


def _deep_copy(A: _Matrix) -> _Matrix:
    from .containers import matrix_from_host, matrix_to_host
    return matrix_from_host(matrix_to_host(A), device=A.device, dtype=A.dtype)


def convert_inplace(dyn: DynamicMatrix, fmt, stream=None, hyb_width: int = 0) -> conversion_error_e:
    """core/src/Morpheus_Convert.hpp:88-124.  fmt = AUTO_FORMAT (-1) asks the
    learned selector for the target format."""
    fmt = int(fmt)
    if fmt == -1:
        from .selector import select_format
        fmt = select_format(dyn)
    if fmt < 0 or fmt >= NFORMATS:
        return conversion_error_e.PROXY_TO_DYNAMIC
    if dyn.active_index() == fmt:
        return conversion_error_e.CONV_SUCCESS
    try:
        temp = to_coo(dyn.active(), stream)
    except MorpheusException:
        return conversion_error_e.DYNAMIC_TO_PROXY
    try:
        out = from_coo(temp, fmt, hyb_width=hyb_width, stream=stream)
    except MorpheusException:
        return conversion_error_e.PROXY_TO_DYNAMIC
    dyn.assign(out)
    return conversion_error_e.CONV_SUCCESS


def sort_by_row_and_column(A: CooMatrix, stream=None) -> None:
    _dev_check(A)
    d = A._desc()
    _call(f"mgb_coo_sort_by_row_and_column_{_suffix(A.dtype)}", C.byref(d), _stream_handle(stream))


def is_sorted(A: CooMatrix, stream=None) -> bool:
    _dev_check(A)
    d = A._desc()
    out = C.c_int()
    _call("mgb_coo_is_sorted", C.byref(d), C.byref(out), _stream_handle(stream))
    return bool(out.value)


__all__ = ["convert", "convert_inplace", "to_coo", "from_coo", "sort_by_row_and_column", "is_sorted"]
_ = torch
