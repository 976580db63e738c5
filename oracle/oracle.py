"""ctypes wrapper of the CPU oracle (oracle.cpp).  TEST INFRASTRUCTURE ONLY.

The oracle restates the Morpheus reference's Serial/OpenMP algorithms on the
SpMV hot path.  Only tests/, __graft_entry__.smoke() and bench.py's CPU
baseline import this module; the product never does.

Matrices cross this boundary as plain dicts of numpy arrays ("host matrices"):

    COO: format, nrows, ncols, nnz, row_indices, column_indices, values
    CSR: format, nrows, ncols, nnz, row_offsets, column_indices, values
    DIA: ... ndiags, pitch, alignment, diagonal_offsets, values (pitch*ndiags,
         column-major: entry (i, n) at [i + pitch*n])
    ELL: ... entries_per_row, width, pitch, alignment, column_indices, values
         (pitch*width, column-major)
    HYB: format, nrows, ncols, nnz, alignment, ell: <ELL dict>, coo: <COO dict>
    HDC: format, nrows, ncols, nnz, alignment, dia: <DIA dict>, csr: <CSR dict>
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
COO, CSR, DIA, ELL, HYB, HDC = range(6)
FORMAT_NAMES = ["COO", "CSR", "DIA", "ELL", "HYB", "HDC"]

STATUS_OK = 0
STATUS_NOT_IMPLEMENTED = 1
STATUS_FORMAT_CONVERSION = 2
STATUS_INVALID_INPUT = 3
STATUS_RUNTIME = 4
STATUS_BAD_ARGUMENT = 8

_lib = None


class OracleError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"oracle {what} failed with status {status}")
        self.status = status


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liboracle.so")
        if not os.path.exists(path):
            from oracle.build import build_oracle  # noqa: WPS433

            build_oracle()
        _lib = C.CDLL(path)
        L = _lib
        L.orc_new.restype = C.c_void_p
        L.orc_new.argtypes = [C.c_int, C.c_int]
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_clone.restype = C.c_void_p
        L.orc_clone.argtypes = [C.c_void_p]
        L.orc_format.argtypes = [C.c_void_p]
        L.orc_activate.argtypes = [C.c_void_p, C.c_int]
        L.orc_shape.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.orc_resize.argtypes = [C.c_void_p, C.POINTER(C.c_int64)]
        L.orc_array.restype = C.c_int64
        L.orc_array.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_void_p)]
        L.orc_convert.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_coo_to_hyb_width.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        L.orc_convert_inplace.argtypes = [C.c_void_p, C.c_int]
        L.orc_sort_by_row_and_column.argtypes = [C.c_void_p]
        L.orc_is_sorted.argtypes = [C.c_void_p]
        L.orc_count_nnz_per_diagonal.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.orc_count_nnz_per_row.argtypes = [C.c_void_p, C.c_void_p, C.c_int]
        L.orc_multiply.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.orc_dot_f64.restype = C.c_double
        L.orc_dot_f64.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
        L.orc_dot_f32.restype = C.c_float
        L.orc_dot_f32.argtypes = [C.c_int64, C.c_void_p, C.c_void_p]
        L.orc_reduce_f64.restype = C.c_double
        L.orc_reduce_f64.argtypes = [C.c_void_p, C.c_int64]
        L.orc_reduce_f32.restype = C.c_float
        L.orc_reduce_f32.argtypes = [C.c_void_p, C.c_int64]
        L.orc_waxpby_f64.argtypes = [C.c_int64, C.c_double, C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]
        L.orc_waxpby_f32.argtypes = [C.c_int64, C.c_float, C.c_void_p, C.c_float, C.c_void_p, C.c_void_p]
        L.orc_exceeds_tolerance.argtypes = [C.c_int64, C.c_int64, C.c_int64]
        L.orc_max_threads.restype = C.c_int
    return _lib


def _dt_code(dtype) -> int:
    dt = np.dtype(dtype)
    if dt == np.float64:
        return 0
    if dt == np.float32:
        return 1
    raise ValueError(f"unsupported value type {dt}")


def _np_dtype(code: int):
    return np.float64 if code == 0 else np.float32


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


_PREFIX = {HYB: ("ell", "coo"), HDC: ("dia", "csr")}
_IDX_NAMES = {
    COO: ["row_indices", "column_indices"],
    CSR: ["row_offsets", "column_indices"],
    DIA: ["diagonal_offsets"],
    ELL: ["column_indices"],
}


class OracleMatrix:
    """One oracle container (any of the six formats), FP64 or FP32."""

    def __init__(self, fmt: int, dtype=np.float64, _handle=None):
        self.dtype = np.dtype(dtype)
        self._code = _dt_code(dtype)
        self.h = _handle if _handle is not None else lib().orc_new(fmt, self._code)
        if not self.h:
            raise ValueError("bad format/dtype")

    def __del__(self):
        h = getattr(self, "h", None)
        if h and _lib is not None:
            _lib.orc_free(h)
            self.h = None

    # -- shape / arrays --------------------------------------------------
    @property
    def format(self) -> int:
        return lib().orc_format(self.h)

    def shape(self) -> list[int]:
        s = (C.c_int64 * 10)()
        lib().orc_shape(self.h, s)
        return list(s)

    def _array(self, name: str, dtype) -> np.ndarray:
        p = C.c_void_p()
        n = lib().orc_array(self.h, name.encode(), C.byref(p))
        if n < 0:
            raise KeyError(name)
        if n == 0:
            return np.zeros(0, dtype=dtype)
        buf = (C.c_char * (n * np.dtype(dtype).itemsize)).from_address(p.value)
        return np.frombuffer(buf, dtype=dtype).copy()

    def _set_array(self, name: str, arr: np.ndarray, dtype) -> None:
        arr = np.ascontiguousarray(arr, dtype=dtype)
        p = C.c_void_p()
        n = lib().orc_array(self.h, name.encode(), C.byref(p))
        if n != arr.size:
            raise ValueError(f"{name}: expected {n} elements, got {arr.size}")
        if n:
            C.memmove(p.value, arr.ctypes.data, arr.nbytes)

    # -- host-dict conversion ------------------------------------------
    @classmethod
    def from_host(cls, hm: dict) -> "OracleMatrix":
        fmt = hm["format"]
        dt = _values_dtype(hm)
        m = cls(fmt, dt)
        s = (C.c_int64 * 10)(*([0] * 10))
        s[0], s[1], s[2], s[3] = fmt, hm["nrows"], hm["ncols"], hm["nnz"]
        if fmt == DIA:
            s[4], s[6] = hm["ndiags"], hm.get("alignment", 32)
        elif fmt == ELL:
            s[4], s[7] = hm["entries_per_row"], hm.get("alignment", 32)
        elif fmt == HYB:
            s[4], s[7], s[8], s[9] = (hm["ell"]["entries_per_row"], hm["ell"]["nnz"],
                                      hm["coo"]["nnz"], hm.get("alignment", 32))
        elif fmt == HDC:
            s[4], s[6], s[7], s[8] = (hm["dia"]["ndiags"], hm["dia"]["nnz"], hm["csr"]["nnz"],
                                      hm.get("alignment", 32))
        st = lib().orc_resize(m.h, s)
        if st != STATUS_OK:
            raise OracleError(st, "resize")
        for name, arr, is_idx in _iter_arrays(hm):
            m._set_array(name, arr, np.int32 if is_idx else m.dtype)
        return m

    def to_host(self) -> dict:
        s = self.shape()
        fmt = s[0]
        vt = self.dtype
        hm = {"format": fmt, "nrows": s[1], "ncols": s[2], "nnz": s[3]}
        if fmt in (COO, CSR):
            for n in _IDX_NAMES[fmt]:
                hm[n] = self._array(n, np.int32)
            hm["values"] = self._array("values", vt)
        elif fmt == DIA:
            hm.update(ndiags=s[4], pitch=s[5], alignment=s[6])
            hm["diagonal_offsets"] = self._array("diagonal_offsets", np.int32)
            hm["values"] = self._array("values", vt)
        elif fmt == ELL:
            hm.update(entries_per_row=s[4], width=s[5], pitch=s[6], alignment=s[7])
            hm["column_indices"] = self._array("column_indices", np.int32)
            hm["values"] = self._array("values", vt)
        elif fmt == HYB:
            hm["alignment"] = s[9]
            hm["ell"] = {"format": ELL, "nrows": s[1], "ncols": s[2], "nnz": s[7],
                         "entries_per_row": s[4], "width": s[5], "pitch": s[6], "alignment": s[9],
                         "column_indices": self._array("ell.column_indices", np.int32),
                         "values": self._array("ell.values", vt)}
            hm["coo"] = {"format": COO, "nrows": s[1], "ncols": s[2], "nnz": s[8],
                         "row_indices": self._array("coo.row_indices", np.int32),
                         "column_indices": self._array("coo.column_indices", np.int32),
                         "values": self._array("coo.values", vt)}
        elif fmt == HDC:
            hm["alignment"] = s[8]
            hm["dia"] = {"format": DIA, "nrows": s[1], "ncols": s[2], "nnz": s[6],
                         "ndiags": s[4], "pitch": s[5], "alignment": s[8],
                         "diagonal_offsets": self._array("dia.diagonal_offsets", np.int32),
                         "values": self._array("dia.values", vt)}
            hm["csr"] = {"format": CSR, "nrows": s[1], "ncols": s[2], "nnz": s[7],
                         "row_offsets": self._array("csr.row_offsets", np.int32),
                         "column_indices": self._array("csr.column_indices", np.int32),
                         "values": self._array("csr.values", vt)}
        return hm

    # -- algorithms ----------------------------------------------------
    def convert(self, fmt: int) -> "OracleMatrix":
        """Morpheus::convert<Serial>(src, dst) with dst an empty `fmt` container."""
        dst = OracleMatrix(fmt, self.dtype)
        st = lib().orc_convert(self.h, dst.h)
        if st != STATUS_OK:
            raise OracleError(st, f"convert to {FORMAT_NAMES[fmt]}")
        return dst

    def coo_to_hyb(self, width: int) -> "OracleMatrix":
        dst = OracleMatrix(HYB, self.dtype)
        st = lib().orc_coo_to_hyb_width(self.h, dst.h, int(width))
        if st != STATUS_OK:
            raise OracleError(st, "coo_to_hyb")
        return dst

    def convert_inplace(self, fmt: int) -> int:
        """Morpheus::convert<Serial>(dyn, fmt) -> conversion_error_e."""
        return lib().orc_convert_inplace(self.h, int(fmt))

    def activate(self, fmt: int) -> None:
        lib().orc_activate(self.h, int(fmt))

    def clone(self) -> "OracleMatrix":
        return OracleMatrix(self.format, self.dtype, _handle=lib().orc_clone(self.h))

    def sort_by_row_and_column(self) -> None:
        st = lib().orc_sort_by_row_and_column(self.h)
        if st != STATUS_OK:
            raise OracleError(st, "sort")

    def is_sorted(self) -> bool:
        return bool(lib().orc_is_sorted(self.h))

    def count_nnz_per_diagonal(self, out: np.ndarray | None = None, init: bool = True) -> np.ndarray:
        """The reference's count_nnz_per_diagonal of this container's format."""
        s = self.shape()
        out = np.zeros(s[1] + s[2] - 1, dtype=np.int32) if out is None else out
        assert out.dtype == np.int32 and out.size == s[1] + s[2] - 1 and out.flags.c_contiguous
        st = lib().orc_count_nnz_per_diagonal(self.h, _ptr(out), 1 if init else 0)
        if st != STATUS_OK:
            raise OracleError(st, "count_nnz_per_diagonal")
        return out

    def count_nnz_per_row(self, out: np.ndarray | None = None, init: bool = True) -> np.ndarray:
        """The reference's count_nnz_per_row of this container's format."""
        s = self.shape()
        out = np.zeros(s[1], dtype=np.int32) if out is None else out
        assert out.dtype == np.int32 and out.size == s[1] and out.flags.c_contiguous
        st = lib().orc_count_nnz_per_row(self.h, _ptr(out), 1 if init else 0)
        if st != STATUS_OK:
            raise OracleError(st, "count_nnz_per_row")
        return out

    def multiply(self, x: np.ndarray, y: np.ndarray | None = None, init: bool = True,
                 threads: int = 0) -> np.ndarray:
        """Serial (threads=0) or OpenMP (threads>0) multiply; returns y."""
        s = self.shape()
        x = np.ascontiguousarray(x, dtype=self.dtype)
        if y is None:
            y = np.zeros(s[1], dtype=self.dtype)
        assert y.dtype == self.dtype and y.flags.c_contiguous
        st = lib().orc_multiply(self.h, _ptr(x), _ptr(y), 1 if init else 0, int(threads))
        if st != STATUS_OK:
            raise OracleError(st, "multiply")
        return y


def _values_dtype(hm: dict):
    if "values" in hm:
        return hm["values"].dtype
    sub = hm["ell"] if hm["format"] == HYB else hm["dia"]
    return sub["values"].dtype


def _iter_arrays(hm: dict):
    fmt = hm["format"]
    if fmt in _PREFIX:
        for part in _PREFIX[fmt]:
            sub = hm[part]
            for name in _IDX_NAMES[sub["format"]]:
                yield f"{part}.{name}", sub[name], True
            yield f"{part}.values", sub["values"], False
    else:
        for name in _IDX_NAMES[fmt]:
            yield name, hm[name], True
        yield "values", hm["values"], False


# -- dense vector ops ------------------------------------------------------

def dot(n: int, x: np.ndarray, y: np.ndarray):
    if x.dtype == np.float64:
        return lib().orc_dot_f64(n, _ptr(x), _ptr(y) if y is not x else _ptr(x))
    return lib().orc_dot_f32(n, _ptr(x), _ptr(y) if y is not x else _ptr(x))


def reduce(x: np.ndarray, n: int):
    if x.dtype == np.float64:
        return lib().orc_reduce_f64(_ptr(x), n)
    return lib().orc_reduce_f32(_ptr(x), n)


def waxpby(n: int, alpha, x: np.ndarray, beta, y: np.ndarray, w: np.ndarray) -> np.ndarray:
    f = lib().orc_waxpby_f64 if x.dtype == np.float64 else lib().orc_waxpby_f32
    f(n, alpha, _ptr(x), beta, _ptr(y), _ptr(w))
    return w


def exceeds_tolerance(nrows: int, nnz: int, ncols: int) -> bool:
    return bool(lib().orc_exceeds_tolerance(nrows, nnz, ncols))


def max_threads() -> int:
    return lib().orc_max_threads()
