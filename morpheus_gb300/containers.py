"""Device containers mirroring the Morpheus containers (core/src/Morpheus_*Matrix.hpp).

Each container owns its arrays as torch tensors (device memory on "cuda", or a
host mirror on "cpu") and produces the plain C descriptor the C ABI takes.
Accessors keep the reference names: nrows(), ncols(), nnnz(), row_offsets(),
column_indices(), values(), diagonal_offsets(), ell(), coo(), dia(), csr(),
format_enum(), format_index(), resize(...).

Slabs are column-major with an explicit pitch, the layout the reference uses on
CUDA (LayoutLeft): DIA values(i, n) at [i + pitch*n] with pitch = pad(nrows, 32)
(core/src/impl/Dia/Morpheus_Utils_Impl.hpp:33-36); ELL slot (i, n) at
[i + pitch*n] with pitch = nrows and width = pad(entries_per_row, 32)
(core/src/Morpheus_EllMatrix.hpp:189-202).
"""
from __future__ import annotations

import ctypes as C
import enum

import numpy as np
import torch

from . import _lib
from .exceptions import InvalidInputException


class formats_e(enum.IntEnum):
    """core/src/Morpheus_FormatsRegistry.hpp:56-64"""
    COO_FORMAT = 0
    CSR_FORMAT = 1
    DIA_FORMAT = 2
    ELL_FORMAT = 3
    HYB_FORMAT = 4
    HDC_FORMAT = 5
    NFORMATS = 6


class conversion_error_e(enum.IntEnum):
    """core/src/Morpheus_Convert.hpp:63-67"""
    DYNAMIC_TO_PROXY = 0
    PROXY_TO_DYNAMIC = 1
    CONV_SUCCESS = 2


COO_FORMAT, CSR_FORMAT, DIA_FORMAT, ELL_FORMAT, HYB_FORMAT, HDC_FORMAT, NFORMATS = range(7)
INVALID_INDEX = -1
# CSR SpMV kernels (MGB_CSR_SEGMENTS / MGB_CSR_ROWS / MGB_CSR_SPLIT /
# MGB_CSR_ROWS_GATHER of include/mgb.h)
CSR_SEGMENTS, CSR_ROWS, CSR_SPLIT, CSR_ROWS_GATHER = 1, 2, 3, 4


def get_pad_size(length: int, alignment: int) -> int:
    """core/src/impl/Dia/Morpheus_Utils_Impl.hpp:33-36"""
    return alignment * ((length + alignment - 1) // alignment)


def _dev(device) -> torch.device:
    return torch.device(device)


def _idx(n: int, device) -> torch.Tensor:
    return torch.zeros(int(n), dtype=torch.int32, device=device)


def _val(n: int, dtype, device) -> torch.Tensor:
    return torch.zeros(int(n), dtype=dtype, device=device)


def _as(t, dtype, device) -> torch.Tensor:
    if isinstance(t, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(t))
    return t.to(device=device, dtype=dtype).contiguous().reshape(-1)


def _ptr(t: torch.Tensor | None):
    return C.c_void_p(t.data_ptr() if t is not None and t.numel() else 0)


class _Matrix:
    FORMAT: int = -1

    def __init__(self, nrows=0, ncols=0, nnz=0, dtype=torch.float64, device="cuda"):
        self._nrows, self._ncols, self._nnz = int(nrows), int(ncols), int(nnz)
        self.dtype = dtype
        self.device = _dev(device)

    def nrows(self) -> int:
        return self._nrows

    def ncols(self) -> int:
        return self._ncols

    def nnnz(self) -> int:
        return self._nnz

    def format_enum(self) -> formats_e:
        return formats_e(self.FORMAT)

    def format_index(self) -> int:
        return self.FORMAT

    def set_nrows(self, n): self._nrows = int(n)
    def set_ncols(self, n): self._ncols = int(n)
    def set_nnnz(self, n): self._nnz = int(n)

    def _tensors(self) -> dict:
        raise NotImplementedError

    def to(self, device) -> "_Matrix":
        """Deep copy into another space (Morpheus::copy + create_mirror)."""
        return matrix_from_host(matrix_to_host(self), device=device, dtype=self.dtype)

    def is_device(self) -> bool:
        return self.device.type == "cuda"


class CooMatrix(_Matrix):
    """core/src/Morpheus_CooMatrix.hpp"""
    FORMAT = COO_FORMAT

    def __init__(self, nrows=0, ncols=0, nnz=0, row_indices=None, column_indices=None, values=None,
                 dtype=torch.float64, device="cuda"):
        super().__init__(nrows, ncols, nnz, dtype, device)
        self._ri = _as(row_indices, torch.int32, self.device) if row_indices is not None else _idx(nnz, self.device)
        self._ci = _as(column_indices, torch.int32, self.device) if column_indices is not None else _idx(nnz, self.device)
        self._v = _as(values, dtype, self.device) if values is not None else _val(nnz, dtype, self.device)
        if not (self._ri.numel() == self._ci.numel() == self._v.numel() == self._nnz):
            raise InvalidInputException("COO arrays must all hold nnz entries")

    def row_indices(self): return self._ri
    def column_indices(self): return self._ci
    def values(self): return self._v
    crow_indices = row_indices
    ccolumn_indices = column_indices
    cvalues = values

    def resize(self, nrows, ncols, nnz):
        self.__init__(nrows, ncols, nnz, dtype=self.dtype, device=self.device)

    def _desc(self) -> _lib.Coo:
        return _lib.Coo(self._nrows, self._ncols, self._nnz, _ptr(self._ri), _ptr(self._ci), _ptr(self._v))


class CsrMatrix(_Matrix):
    """core/src/Morpheus_CsrMatrix.hpp:533-537"""
    FORMAT = CSR_FORMAT

    def __init__(self, nrows=0, ncols=0, nnz=0, row_offsets=None, column_indices=None, values=None,
                 dtype=torch.float64, device="cuda"):
        super().__init__(nrows, ncols, nnz, dtype, device)
        self._ro = _as(row_offsets, torch.int32, self.device) if row_offsets is not None else _idx(nrows + 1, self.device)
        self._ci = _as(column_indices, torch.int32, self.device) if column_indices is not None else _idx(nnz, self.device)
        self._v = _as(values, dtype, self.device) if values is not None else _val(nnz, dtype, self.device)
        if self._ro.numel() != self._nrows + 1 or self._ci.numel() != self._nnz or self._v.numel() != self._nnz:
            raise InvalidInputException("CSR arrays have the wrong sizes")
        self._variant = None
        self._plan = None

    def row_offsets(self): return self._ro
    def column_indices(self): return self._ci
    def values(self): return self._v
    crow_offsets = row_offsets
    ccolumn_indices = column_indices
    cvalues = values

    def kernel_variant(self) -> int:
        """SpMV kernel for this matrix (CSR_ROWS / CSR_ROWS_GATHER for short
        rows of nearly equal length with neighbouring / scattered columns,
        CSR_SPLIT for very long rows, else CSR_SEGMENTS), measured once on the device and
        cached.  Values may change in place; after writing new row offsets in
        place, call forget_kernel_variant()."""
        if self._variant is None:
            out = C.c_int()
            d = self._desc()
            _lib.call("mgb_csr_choose_kernel", C.byref(d), C.byref(out), None)
            self._variant = out.value
        return self._variant

    def chunk_plan(self, stream=None) -> tuple[torch.Tensor, int]:
        """(plan, entries): the first row of every warp chunk of the
        lane-segment kernel (mgb_csr_plan), made once on `stream` (a raw
        CUDA stream handle or None) and cached, so that multiplies skip the
        row-offset searches.  Cleared with the kernel choice."""
        if self._plan is None:
            d = self._desc()
            n = C.c_int64()
            _lib.call("mgb_csr_plan_entries", C.byref(d), C.byref(n))
            plan = torch.empty(n.value, dtype=torch.int32, device=self.device)
            _lib.call("mgb_csr_plan", C.byref(d), C.c_void_p(plan.data_ptr()), n.value, stream)
            self._plan = (plan, n.value)
        return self._plan

    def forget_kernel_variant(self) -> None:
        """Drops the cached kernel choice and chunk plan (call after writing
        new row offsets in place)."""
        self._variant = None
        self._plan = None

    def resize(self, nrows, ncols, nnz):
        self.__init__(nrows, ncols, nnz, dtype=self.dtype, device=self.device)

    def _desc(self) -> _lib.Csr:
        return _lib.Csr(self._nrows, self._ncols, self._nnz, _ptr(self._ro), _ptr(self._ci), _ptr(self._v))


class DiaMatrix(_Matrix):
    """core/src/Morpheus_DiaMatrix.hpp:192-201"""
    FORMAT = DIA_FORMAT

    def __init__(self, nrows=0, ncols=0, nnz=0, ndiags=0, alignment=32, diagonal_offsets=None,
                 values=None, dtype=torch.float64, device="cuda"):
        super().__init__(nrows, ncols, nnz, dtype, device)
        self._ndiags, self._alignment = int(ndiags), int(alignment)
        self._pitch = get_pad_size(self._nrows, self._alignment)
        self._off = _as(diagonal_offsets, torch.int32, self.device) if diagonal_offsets is not None \
            else _idx(ndiags, self.device)
        if values is not None:
            if isinstance(values, torch.Tensor) and values.dim() == 2:
                values = values.t()  # (pitch, ndiags) -> column-major flat
            self._v = _as(values, dtype, self.device)
        else:
            self._v = _val(self._pitch * self._ndiags, dtype, self.device)
        if self._off.numel() != self._ndiags or self._v.numel() != self._pitch * self._ndiags:
            raise InvalidInputException("DIA arrays have the wrong sizes")

    def ndiags(self): return self._ndiags
    def alignment(self): return self._alignment
    def pitch(self): return self._pitch
    def diagonal_offsets(self): return self._off
    cdiagonal_offsets = diagonal_offsets

    def values(self) -> torch.Tensor:
        """(pitch x ndiags) view; element (i, n) of the slab."""
        return self._v.view(self._ndiags, self._pitch).t() if self._ndiags else self._v.view(self._pitch, 0)
    cvalues = values

    def values_flat(self): return self._v

    def resize(self, nrows, ncols, nnz, ndiags, alignment=32):
        self.__init__(nrows, ncols, nnz, ndiags, alignment, dtype=self.dtype, device=self.device)

    def _desc(self) -> _lib.Dia:
        return _lib.Dia(self._nrows, self._ncols, self._nnz, self._ndiags, self._pitch,
                        _ptr(self._off), _ptr(self._v))


class EllMatrix(_Matrix):
    """core/src/Morpheus_EllMatrix.hpp:189-202, 563"""
    FORMAT = ELL_FORMAT

    def __init__(self, nrows=0, ncols=0, nnz=0, entries_per_row=0, alignment=32, column_indices=None,
                 values=None, dtype=torch.float64, device="cuda"):
        super().__init__(nrows, ncols, nnz, dtype, device)
        self._epr, self._alignment = int(entries_per_row), int(alignment)
        self._width = get_pad_size(self._epr, self._alignment)
        self._pitch = self._nrows
        n = self._pitch * self._width
        self._ci = _as(column_indices, torch.int32, self.device) if column_indices is not None \
            else torch.full((n,), INVALID_INDEX, dtype=torch.int32, device=self.device)
        self._v = _as(values, dtype, self.device) if values is not None else _val(n, dtype, self.device)
        if self._ci.numel() != n or self._v.numel() != n:
            raise InvalidInputException("ELL arrays have the wrong sizes")

    def entries_per_row(self): return self._epr
    def alignment(self): return self._alignment
    def width(self): return self._width
    def pitch(self): return self._pitch

    @staticmethod
    def invalid_index() -> int:
        return INVALID_INDEX

    def column_indices(self): return self._ci.view(self._width, self._pitch).t()
    def values(self): return self._v.view(self._width, self._pitch).t()
    ccolumn_indices = column_indices
    cvalues = values

    def resize(self, nrows, ncols, nnz, entries_per_row, alignment=32):
        self.__init__(nrows, ncols, nnz, entries_per_row, alignment, dtype=self.dtype, device=self.device)

    def _desc(self) -> _lib.Ell:
        return _lib.Ell(self._nrows, self._ncols, self._nnz, self._epr, self._width, self._pitch,
                        _ptr(self._ci), _ptr(self._v))


class HybMatrix(_Matrix):
    """core/src/Morpheus_HybMatrix.hpp:359-376, 473-476"""
    FORMAT = HYB_FORMAT

    def __init__(self, ell: EllMatrix | None = None, coo: CooMatrix | None = None, dtype=torch.float64,
                 device="cuda", alignment=32):
        ell = ell if ell is not None else EllMatrix(dtype=dtype, device=device)
        coo = coo if coo is not None else CooMatrix(dtype=dtype, device=device)
        super().__init__(ell.nrows(), ell.ncols(), ell.nnnz() + coo.nnnz(), ell.dtype, ell.device)
        self._ell, self._coo, self._alignment = ell, coo, int(alignment)

    def ell(self): return self._ell
    def coo(self): return self._coo
    cell = ell
    ccoo = coo

    def alignment(self): return self._alignment

    def _desc(self) -> _lib.Hyb:
        return _lib.Hyb(self._ell._desc(), self._coo._desc())


class HdcMatrix(_Matrix):
    """core/src/Morpheus_HdcMatrix.hpp:148, 356-367, 464-467"""
    FORMAT = HDC_FORMAT
    true_diagonal_ratio = 0.2

    def __init__(self, dia: DiaMatrix | None = None, csr: CsrMatrix | None = None, dtype=torch.float64,
                 device="cuda", alignment=32):
        dia = dia if dia is not None else DiaMatrix(dtype=dtype, device=device)
        csr = csr if csr is not None else CsrMatrix(dtype=dtype, device=device)
        super().__init__(dia.nrows(), dia.ncols(), dia.nnnz() + csr.nnnz(), dia.dtype, dia.device)
        self._dia, self._csr, self._alignment = dia, csr, int(alignment)

    def dia(self): return self._dia
    def csr(self): return self._csr
    cdia = dia
    ccsr = csr

    def alignment(self): return self._alignment

    def _desc(self) -> _lib.Hdc:
        return _lib.Hdc(self._dia._desc(), self._csr._desc())


_CLASSES = [CooMatrix, CsrMatrix, DiaMatrix, EllMatrix, HybMatrix, HdcMatrix]


class DynamicMatrix(_Matrix):
    """core/src/Morpheus_DynamicMatrix.hpp:102-462: one active container of any format."""
    FORMAT = -1

    def __init__(self, src: _Matrix | None = None, dtype=torch.float64, device="cuda"):
        if src is None:
            src = CooMatrix(dtype=dtype, device=device)
        self._set(src)

    def _set(self, src: _Matrix) -> None:
        if isinstance(src, DynamicMatrix):
            src = src.active()
        self._active = src
        super().__init__(src.nrows(), src.ncols(), src.nnnz(), src.dtype, src.device)

    def active(self) -> _Matrix:
        return self._active

    def active_index(self) -> int:
        return self._active.FORMAT

    def active_enum(self) -> formats_e:
        return formats_e(self._active.FORMAT)

    def format_enum(self) -> formats_e:
        return self.active_enum()

    def format_index(self) -> int:
        return self.active_index()

    def activate(self, fmt) -> None:
        """core/src/Morpheus_DynamicMatrix.hpp:409-442: switch to an EMPTY
        container of the new format (no data is converted).  Activating the
        format that is already active, or an index past the last format,
        leaves the matrix unchanged."""
        fmt = int(fmt)
        if fmt < 0 or fmt >= NFORMATS or fmt == self.active_index():
            return
        self._set(_CLASSES[fmt](dtype=self.dtype, device=self.device))

    def assign(self, src: _Matrix) -> "DynamicMatrix":
        self._set(src)
        return self

    def _desc(self):
        return self._active._desc()


# ---------------------------------------------------------------------------
# host-dict interchange (the same schema the oracle and the generators use)
# ---------------------------------------------------------------------------

def _np(t: torch.Tensor) -> np.ndarray:
    return t.detach().to("cpu").contiguous().numpy().copy()


def matrix_to_host(A: _Matrix) -> dict:
    if isinstance(A, DynamicMatrix):
        A = A.active()
    f = A.FORMAT
    hm = {"format": f, "nrows": A.nrows(), "ncols": A.ncols(), "nnz": A.nnnz()}
    if f == COO_FORMAT:
        hm.update(row_indices=_np(A._ri), column_indices=_np(A._ci), values=_np(A._v))
    elif f == CSR_FORMAT:
        hm.update(row_offsets=_np(A._ro), column_indices=_np(A._ci), values=_np(A._v))
    elif f == DIA_FORMAT:
        hm.update(ndiags=A.ndiags(), pitch=A.pitch(), alignment=A.alignment(),
                  diagonal_offsets=_np(A._off), values=_np(A._v))
    elif f == ELL_FORMAT:
        hm.update(entries_per_row=A.entries_per_row(), width=A.width(), pitch=A.pitch(),
                  alignment=A.alignment(), column_indices=_np(A._ci), values=_np(A._v))
    elif f == HYB_FORMAT:
        hm.update(alignment=A.alignment(), ell=matrix_to_host(A.ell()), coo=matrix_to_host(A.coo()))
    elif f == HDC_FORMAT:
        hm.update(alignment=A.alignment(), dia=matrix_to_host(A.dia()), csr=matrix_to_host(A.csr()))
    return hm


def matrix_from_host(hm: dict, device="cuda", dtype=None) -> _Matrix:
    f = hm["format"]
    if dtype is None:
        vals = hm["values"] if "values" in hm else (hm["ell"] if f == HYB_FORMAT else hm["dia"])["values"]
        dtype = torch.float64 if vals.dtype == np.float64 else torch.float32
    n, m, z = hm["nrows"], hm["ncols"], hm["nnz"]
    if f == COO_FORMAT:
        return CooMatrix(n, m, z, hm["row_indices"], hm["column_indices"], hm["values"], dtype, device)
    if f == CSR_FORMAT:
        return CsrMatrix(n, m, z, hm["row_offsets"], hm["column_indices"], hm["values"], dtype, device)
    if f == DIA_FORMAT:
        return DiaMatrix(n, m, z, hm["ndiags"], hm.get("alignment", 32), hm["diagonal_offsets"],
                         hm["values"], dtype, device)
    if f == ELL_FORMAT:
        return EllMatrix(n, m, z, hm["entries_per_row"], hm.get("alignment", 32), hm["column_indices"],
                         hm["values"], dtype, device)
    if f == HYB_FORMAT:
        return HybMatrix(matrix_from_host(hm["ell"], device, dtype), matrix_from_host(hm["coo"], device, dtype),
                         dtype, device, hm.get("alignment", 32))
    if f == HDC_FORMAT:
        return HdcMatrix(matrix_from_host(hm["dia"], device, dtype), matrix_from_host(hm["csr"], device, dtype),
                         dtype, device, hm.get("alignment", 32))
    raise InvalidInputException(f"unknown format {f}")
