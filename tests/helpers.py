"""Shared test helpers: golden fixtures, host-matrix comparison, error norms."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FORMATS = ["COO", "CSR", "DIA", "ELL", "HYB", "HDC"]
INDEX_KEYS = {"row_indices", "column_indices", "row_offsets", "diagonal_offsets"}
# normwise relative error bars for y (FP64 / FP32), against the FP64 oracle
TOL = {np.dtype(np.float64): 1e-12, np.dtype(np.float32): 1e-5}


def golden(dtype=np.float64) -> dict:
    """The reference's 10x10 fixture in all six formats (tests/golden/small_matrix.json)."""
    with open(os.path.join(HERE, "golden", "small_matrix.json")) as f:
        raw = json.load(f)
    return {k: _np(raw[k], dtype) for k in FORMATS}


def _np(d, dtype):
    out = {}
    for k, v in d.items():
        if isinstance(v, dict):
            out[k] = _np(v, dtype)
        elif isinstance(v, list):
            out[k] = np.asarray(v, dtype=np.int32 if k in INDEX_KEYS else dtype)
        else:
            out[k] = v
    return out


def assert_same_matrix(a: dict, b: dict, path: str = "") -> None:
    """Bit-exact equality of two host matrices (structure, indices, values)."""
    assert a["format"] == b["format"], f"{path}format {a['format']} != {b['format']}"
    for k in sorted(set(a) | set(b)):
        if k in ("alignment",):
            continue
        assert k in a and k in b, f"{path}{k} missing"
        va, vb = a[k], b[k]
        if isinstance(va, dict):
            assert_same_matrix(va, vb, f"{path}{k}.")
        elif isinstance(va, np.ndarray):
            assert va.shape == vb.shape, f"{path}{k}: shape {va.shape} != {vb.shape}"
            if va.dtype.kind == "f":
                assert np.array_equal(va.view(np.uint8), np.asarray(vb, va.dtype).view(np.uint8)), \
                    f"{path}{k}: values differ (first at {np.flatnonzero(va != vb)[:5]})"
            else:
                assert np.array_equal(va, vb), f"{path}{k}: differ at {np.flatnonzero(va != vb)[:5]}"
        else:
            assert va == vb, f"{path}{k}: {va} != {vb}"


def rel_err(y: np.ndarray, ref: np.ndarray) -> float:
    y = np.asarray(y, dtype=np.float64)
    ref = np.asarray(ref, dtype=np.float64)
    den = np.linalg.norm(ref)
    num = np.linalg.norm(y - ref)
    return float(num / den) if den > 0 else float(num)


def dense_of(hm: dict) -> np.ndarray:
    """Dense matrix of a COO/CSR host matrix (small cases)."""
    A = np.zeros((hm["nrows"], hm["ncols"]))
    if hm["format"] == 1:
        ro = hm["row_offsets"]
        for i in range(hm["nrows"]):
            for jj in range(ro[i], ro[i + 1]):
                A[i, hm["column_indices"][jj]] += hm["values"][jj]
    else:
        for r, c, v in zip(hm["row_indices"], hm["column_indices"], hm["values"]):
            A[r, c] += v
    return A
