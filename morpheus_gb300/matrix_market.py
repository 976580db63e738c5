"""Matrix Market I/O with the reference's behaviour
(core/src/Morpheus_MatrixMarket.hpp:62-190, core/src/impl/Morpheus_MatrixMarket_Impl.hpp).

    read_matrix_market_file(A, filename)   A: CooMatrix, DynamicMatrix (COO active) or a 1-D tensor
    write_matrix_market_file(A, filename)  A: CooMatrix, DynamicMatrix (COO active) or a 1-D tensor

Reading parses on the host, converts indices to base 0, expands symmetric
matrices (each off-diagonal entry mirrored right after itself), and sorts by
(row, column) with a stable host sort, as the reference's Serial sort does,
before the arrays are placed on the container's device.  Errors raise the
reference's exception classes: IOException for malformed files, NotImplementedException for complex,
hermitian and skew-symmetric data, RuntimeException for a DynamicMatrix whose
active format is not COO.

One reference defect is fixed: a banner with symmetry "unsymmetric" is read
as "general" (the reference accepts the word but then replaces the matrix by
an unfilled one of nnz + off-diagonals entries,
core/src/impl/Morpheus_MatrixMarket_Impl.hpp:198-240).
"""
from __future__ import annotations

import numpy as np
import torch

from .containers import COO_FORMAT, CooMatrix, DynamicMatrix
from .exceptions import IOException, NotImplementedException, RuntimeException

_STORAGE = ("array", "coordinate")
_TYPES = ("complex", "real", "integer", "pattern")
_SYMMETRY = ("general", "symmetric", "unsymmetric", "hermitian", "skew-symmetric")


def _banner(line: str) -> tuple[str, str, str]:
    """core/src/impl/Morpheus_MatrixMarket_Impl.hpp:68-100"""
    t = line.split()
    if len(t) != 5 or t[0] != "%%MatrixMarket" or t[1] != "matrix":
        raise IOException("invalid MatrixMarket banner")
    storage, dtype, symmetry = t[2], t[3], t[4]
    if storage not in _STORAGE:
        raise IOException(f"invalid MatrixMarket storage format [{storage}]")
    if dtype not in _TYPES:
        raise IOException(f"invalid MatrixMarket data type [{dtype}]")
    if symmetry not in _SYMMETRY:
        raise IOException(f"invalid MatrixMarket symmetry [{symmetry}]")
    return storage, dtype, symmetry


def _split(text: str) -> tuple[tuple[str, str, str], list[str], list[str]]:
    """(banner, tokens of the size line, every token after it).  Lines that
    start with '%' before the size line are comments."""
    lines = text.split("\n")
    if not lines:
        raise IOException("invalid MatrixMarket banner")
    banner = _banner(lines[0])
    i = 1
    while i < len(lines) and lines[i][:1] == "%":
        i += 1
    if i >= len(lines):
        raise IOException("unexpected EOF while reading MatrixMarket entries")
    return banner, lines[i].split(), "\n".join(lines[i + 1:]).split()


def _parse_int(tok: str) -> int:
    try:
        return int(tok)
    except ValueError:
        raise IOException(f"invalid MatrixMarket integer [{tok}]") from None


def read_coordinate(text: str, dtype=np.float64) -> tuple[int, int, np.ndarray, np.ndarray, np.ndarray]:
    """Host arrays (nrows, ncols, rows, cols, vals) of a coordinate file,
    base 0, symmetric entries expanded, sorted by (row, column)."""
    (storage, kind, symmetry), size, body = _split(text)
    if storage != "coordinate":
        raise IOException("only coordinate storage format is supported for reading a "
                          "MatrixMarket file into CooMatrix container")
    if len(size) != 3:
        raise IOException("invalid MatrixMarket coordinate format")
    nrows, ncols, nnz = (_parse_int(t) for t in size)
    if kind == "complex":
        raise NotImplementedException("Morpheus does not currently support complex matrices")
    per = 2 if kind == "pattern" else 3
    if len(body) < per * nnz:
        raise IOException("unexpected EOF while reading MatrixMarket entries")
    tok = np.array(body[:per * nnz], dtype=object).reshape(nnz, per) if nnz else np.zeros((0, per), object)
    try:
        rows = tok[:, 0].astype(np.int64)
        cols = tok[:, 1].astype(np.int64)
        vals = np.ones(nnz, dtype=dtype) if per == 2 else tok[:, 2].astype(np.float64).astype(dtype)
    except ValueError as e:
        raise IOException(f"invalid MatrixMarket entry ({e})") from None
    if nnz:
        if rows.min() < 1:
            raise IOException("found invalid row index (index < 1)")
        if cols.min() < 1:
            raise IOException("found invalid column index (index < 1)")
        if rows.max() > nrows:
            raise IOException("found invalid row index (index > num_rows)")
        if cols.max() > ncols:
            raise IOException("found invalid column index (index > num_columns)")
    rows -= 1
    cols -= 1
    if symmetry == "hermitian":
        raise NotImplementedException("MatrixMarket I/O does not currently support hermitian matrices")
    if symmetry == "skew-symmetric":
        raise NotImplementedException("MatrixMarket I/O does not currently support skew-symmetric matrices")
    if symmetry == "symmetric":
        off = rows != cols
        # entry n, then its mirror when off-diagonal (reference order)
        reps = 1 + off.astype(np.int64)
        idx = np.repeat(np.arange(nnz), reps)
        mirror = np.zeros(idx.size, dtype=bool)
        mirror[np.cumsum(reps) - 1] = off
        r2, c2 = rows[idx], cols[idx]
        rows = np.where(mirror, c2, r2)
        cols = np.where(mirror, r2, c2)
        vals = vals[idx]
    order = np.lexsort((cols, rows))  # stable: equal (row, col) keep file order
    return nrows, ncols, rows[order].astype(np.int32), cols[order].astype(np.int32), vals[order]


def read_array(text: str, dtype=np.float64) -> np.ndarray:
    """core/src/impl/Morpheus_MatrixMarket_Impl.hpp:251-316 for an n x 1 or
    1 x n array (a vector); entries in file order."""
    (storage, kind, symmetry), size, body = _split(text)
    if storage != "array":
        raise IOException("only coordinate storage format is supported for reading a "
                          "MatrixMarket file into DenseVector container")
    if len(size) != 2:
        raise IOException("invalid MatrixMarket array format")
    nrows, ncols = (_parse_int(t) for t in size)
    if kind == "pattern":
        raise NotImplementedException("pattern array MatrixMarket format is not supported")
    if kind == "complex":
        raise NotImplementedException("complex type is not supported")
    n = nrows * ncols
    if len(body) < n:
        raise IOException("unexpected EOF while reading MatrixMarket entries")
    if symmetry != "general":
        raise NotImplementedException("only general array symmetric MatrixMarket format is supported")
    if nrows != 1 and ncols != 1 and n:
        raise NotImplementedException("a dense array with more than one row and column needs a DenseMatrix")
    try:
        return np.array(body[:n], dtype=np.float64).astype(dtype)
    except ValueError as e:
        raise IOException(f"invalid MatrixMarket entry ({e})") from None


def _read_text(filename: str) -> str:
    try:
        with open(filename, "r") as f:
            return f.read()
    except OSError as e:
        raise IOException(f"failed to open {filename}: {e}") from None


def _np_dtype(torch_dtype):
    return np.float32 if torch_dtype == torch.float32 else np.float64


def read_matrix_market_file(A, filename: str):
    """Fill A (CooMatrix, DynamicMatrix with COO active, or a 1-D torch
    tensor standing for a DenseVector) from a Matrix Market file; returns A."""
    text = _read_text(filename)
    if isinstance(A, DynamicMatrix):
        if A.active_index() != COO_FORMAT:
            raise RuntimeException("read_matrix_market_stream: The active state of a DynamicMatrix must be set "
                                   "to Morpheus::COO_FORMAT before reading a MatrixMarket stream!")
        coo = CooMatrix(dtype=A.dtype, device=A.device)
        _fill_coo(coo, text)
        A.assign(coo)
        return A
    if isinstance(A, CooMatrix):
        _fill_coo(A, text)
        return A
    if isinstance(A, torch.Tensor):
        v = read_array(text, _np_dtype(A.dtype))
        A.resize_(v.size)
        A.copy_(torch.from_numpy(v))
        return A
    raise NotImplementedException(f"Matrix Market reading into {type(A).__name__}")


def _fill_coo(coo: CooMatrix, text: str) -> None:
    n, m, r, c, v = read_coordinate(text, _np_dtype(coo.dtype))
    out = CooMatrix(n, m, r.size, r, c, v, dtype=coo.dtype, device=coo.device)
    coo.__dict__.update(out.__dict__)


def write_matrix_market_file(A, filename: str) -> None:
    """core/src/impl/Morpheus_MatrixMarket_Impl.hpp:415-485: coordinate real
    general (1-based indices, tab-separated size line) or array real general."""
    if isinstance(A, DynamicMatrix):
        if A.active_index() != COO_FORMAT:
            raise RuntimeException("write_matrix_market_stream: The active state of a DynamicMatrix must be set "
                                   "to Morpheus::COO_FORMAT before writing a MatrixMarket stream!")
        A = A.active()
    if isinstance(A, CooMatrix):
        r = A.row_indices().cpu().numpy().astype(np.int64) + 1
        c = A.column_indices().cpu().numpy().astype(np.int64) + 1
        v = A.values().cpu().numpy()
        with open(filename, "w") as f:
            f.write("%%MatrixMarket matrix coordinate real general\n")
            f.write(f"{A.nrows()}\t{A.ncols()}\t{A.nnnz()}\n")
            f.writelines(f"{a} {b} {_fmt(x)}\n" for a, b, x in zip(r.tolist(), c.tolist(), v.tolist()))
        return
    if isinstance(A, torch.Tensor):
        v = A.detach().cpu().numpy().reshape(-1)
        with open(filename, "w") as f:
            f.write("%%MatrixMarket matrix array real general\n")
            f.write(f"{v.size}\t1\n")
            f.writelines(f"{_fmt(x)}\n" for x in v.tolist())
        return
    raise NotImplementedException(f"Matrix Market writing of {type(A).__name__}")


def _fmt(x: float) -> str:
    """Shortest text that reads back to the same value (the reference streams
    with the default 6 significant digits, which does not round-trip)."""
    return repr(float(x))
