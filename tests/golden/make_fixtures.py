"""Generate tests/golden/small_matrix.json from the reference's own test fixtures.

The Morpheus tests define one hand-written 10x10, 32-entry matrix in all six
formats (core/tests/utils/Macros_Definitions.hpp:29-73 and the
reset_small_container() bodies in Macros_{Coo,Csr,Dia,Ell,Hyb,Hdc}Matrix.hpp).
This script reads those headers as text, extracts every assignment and writes
the six containers in the host-matrix schema used by the tests.  Run it where
the reference tree is available:

    python tests/golden/make_fixtures.py /path/to/morpheus
"""
from __future__ import annotations

import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = r"(-?[0-9.]+)"


def body(text: str, predicate: str) -> str:
    """Body of the reset_small_container() overload selected by `predicate`."""
    i = text.index(predicate)
    start = text.index("{", text.index(")", i))
    depth, j = 0, start
    while True:
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
            if depth == 0:
                return text[start:j]
        j += 1


def pad(n: int, a: int = 32) -> int:
    return a * ((n + a - 1) // a)


def parse_1d(src: str, prefix: str, field: str) -> dict[int, float]:
    out = {}
    for m in re.finditer(rf"{re.escape(prefix)}{field}\((\d+)\)\s*=\s*(?:\(value_type\))?{NUM};", src):
        out[int(m.group(1))] = float(m.group(2))
    return out


def parse_2d(src: str, prefix: str, field: str) -> dict[tuple[int, int], float]:
    out = {}
    for m in re.finditer(rf"{re.escape(prefix)}{field}\((\d+),\s*(\d+)\)\s*=\s*(?:\(value_type\))?{NUM};", src):
        out[(int(m.group(1)), int(m.group(2)))] = float(m.group(3))
    return out


def dense_1d(d: dict, n: int, cast) -> list:
    assert set(d) == set(range(n)), (sorted(d), n)
    return [cast(d[i]) for i in range(n)]


def slab(d: dict, nrows: int, ncols: int, pitch: int, fill, cast) -> list:
    """column-major slab [i + pitch*j] with unspecified entries = fill"""
    out = [fill] * (pitch * ncols)
    for (i, j), v in d.items():
        assert i < nrows and j < ncols
        out[i + pitch * j] = cast(v)
    return out


def main(ref: str) -> None:
    U = os.path.join(ref, "core", "tests", "utils")
    read = lambda f: open(os.path.join(U, f)).read()  # noqa: E731
    defs = read("Macros_Definitions.hpp")
    const = {m.group(1): int(m.group(2)) for m in re.finditer(r"const size_t (\w+)\s*=\s*(\d+);", defs)}
    N, M, NNZ = const["SMALL_MATRIX_NROWS"], const["SMALL_MATRIX_NCOLS"], const["SMALL_MATRIX_NNZ"]
    fx = {"source": "core/tests/utils/Macros_*.hpp reset_small_container()", "constants": const}

    coo = body(read("Macros_CooMatrix.hpp"), "is_coo_matrix_format_container_v")
    fx["COO"] = {"format": 0, "nrows": N, "ncols": M, "nnz": NNZ,
                 "row_indices": dense_1d(parse_1d(coo, "c.", "row_indices"), NNZ, int),
                 "column_indices": dense_1d(parse_1d(coo, "c.", "column_indices"), NNZ, int),
                 "values": dense_1d(parse_1d(coo, "c.", "values"), NNZ, float)}

    csr = body(read("Macros_CsrMatrix.hpp"), "is_csr_matrix_format_container_v")
    fx["CSR"] = {"format": 1, "nrows": N, "ncols": M, "nnz": NNZ,
                 "row_offsets": dense_1d(parse_1d(csr, "c.", "row_offsets"), N + 1, int),
                 "column_indices": dense_1d(parse_1d(csr, "c.", "column_indices"), NNZ, int),
                 "values": dense_1d(parse_1d(csr, "c.", "values"), NNZ, float)}

    nd = const["SMALL_DIA_MATRIX_NDIAGS"]
    dia = body(read("Macros_DiaMatrix.hpp"), "is_dia_matrix_format_container_v")
    fx["DIA"] = {"format": 2, "nrows": N, "ncols": M, "nnz": NNZ, "ndiags": nd, "pitch": pad(N),
                 "alignment": 32,
                 "diagonal_offsets": dense_1d(parse_1d(dia, "c.", "diagonal_offsets"), nd, int),
                 "values": slab(parse_2d(dia, "c.", "values"), N, nd, pad(N), 0.0, float)}

    epr = const["SMALL_ELL_ENTRIES_PER_ROW"]
    ell = body(read("Macros_EllMatrix.hpp"), "is_ell_matrix_format_container_v")
    fx["ELL"] = {"format": 3, "nrows": N, "ncols": M, "nnz": NNZ, "entries_per_row": epr,
                 "width": pad(epr), "pitch": N, "alignment": 32,
                 "column_indices": slab(parse_2d(ell, "c.", "column_indices"), N, pad(epr), N, -1, int),
                 "values": slab(parse_2d(ell, "c.", "values"), N, pad(epr), N, 0.0, float)}

    hepr, hell, hcoo = (const["SMALL_HYB_ENTRIES_PER_ROW"], const["SMALL_HYB_ELL_NNZ"],
                        const["SMALL_HYB_COO_NNZ"])
    hyb = body(read("Macros_HybMatrix.hpp"), "is_hyb_matrix_format_container_v")
    fx["HYB"] = {"format": 4, "nrows": N, "ncols": M, "nnz": NNZ, "alignment": 32,
                 "ell": {"format": 3, "nrows": N, "ncols": M, "nnz": hell, "entries_per_row": hepr,
                         "width": pad(hepr), "pitch": N, "alignment": 32,
                         "column_indices": slab(parse_2d(hyb, "c.ell().", "column_indices"), N, pad(hepr), N, -1, int),
                         "values": slab(parse_2d(hyb, "c.ell().", "values"), N, pad(hepr), N, 0.0, float)},
                 "coo": {"format": 0, "nrows": N, "ncols": M, "nnz": hcoo,
                         "row_indices": dense_1d(parse_1d(hyb, "c.coo().", "row_indices"), hcoo, int),
                         "column_indices": dense_1d(parse_1d(hyb, "c.coo().", "column_indices"), hcoo, int),
                         "values": dense_1d(parse_1d(hyb, "c.coo().", "values"), hcoo, float)}}

    dnnz, cnnz, dnd = const["SMALL_HDC_DIA_NNZ"], const["SMALL_HDC_CSR_NNZ"], const["SMALL_HDC_DIA_NDIAG"]
    hdc = body(read("Macros_HdcMatrix.hpp"), "is_hdc_matrix_format_container_v")
    fx["HDC"] = {"format": 5, "nrows": N, "ncols": M, "nnz": NNZ, "alignment": 32,
                 "dia": {"format": 2, "nrows": N, "ncols": M, "nnz": dnnz, "ndiags": dnd, "pitch": pad(N),
                         "alignment": 32,
                         "diagonal_offsets": dense_1d(parse_1d(hdc, "c.dia().", "diagonal_offsets"), dnd, int),
                         "values": slab(parse_2d(hdc, "c.dia().", "values"), N, dnd, pad(N), 0.0, float)},
                 "csr": {"format": 1, "nrows": N, "ncols": M, "nnz": cnnz,
                         "row_offsets": dense_1d(parse_1d(hdc, "c.csr().", "row_offsets"), N + 1, int),
                         "column_indices": dense_1d(parse_1d(hdc, "c.csr().", "column_indices"), cnnz, int),
                         "values": dense_1d(parse_1d(hdc, "c.csr().", "values"), cnnz, float)}}

    with open(os.path.join(HERE, "small_matrix.json"), "w") as f:
        json.dump(fx, f, indent=1)
    print("wrote", os.path.join(HERE, "small_matrix.json"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path to the Morpheus source tree>")
    main(sys.argv[1])
