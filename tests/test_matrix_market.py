"""Matrix Market reader/writer: the cases of the reference's
core/tests/Test_MatrixMarket.hpp (malformed banners, sizes, indices, EOF,
unsupported types and symmetries; general, symmetric and pattern matrices;
vectors), on fixtures written by this file."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from morpheus_gb300 import matrix_market as mm

GENERAL = """%%MatrixMarket matrix coordinate real general
% a comment
3 4 5
3 4 -1.5
1 1 1.25
2 3 7
1 4 2.5e-3
2 1 -0.5
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def _coo(A):
    return (A.row_indices().cpu().numpy().tolist(), A.column_indices().cpu().numpy().tolist(),
            A.values().cpu().numpy().tolist())


def test_general_real_is_sorted_base0(tmp_path):
    A = mgb.CooMatrix(device="cpu")
    mgb.read_matrix_market_file(A, _write(tmp_path, "g.mtx", GENERAL))
    assert (A.nrows(), A.ncols(), A.nnnz()) == (3, 4, 5)
    r, c, v = _coo(A)
    assert r == [0, 0, 1, 1, 2] and c == [0, 3, 0, 2, 3]
    assert v == [1.25, 2.5e-3, -0.5, 7.0, -1.5]


def test_symmetric_expansion(tmp_path):
    text = """%%MatrixMarket matrix coordinate real symmetric
4 4 4
1 2 2.125
3 3 -1
4 1 0.5
2 2 6
"""
    A = mgb.CooMatrix(device="cpu")
    mgb.read_matrix_market_file(A, _write(tmp_path, "s.mtx", text))
    r, c, v = _coo(A)
    assert A.nnnz() == 6
    assert list(zip(r, c, v)) == [(0, 1, 2.125), (0, 3, 0.5), (1, 0, 2.125), (1, 1, 6.0), (2, 2, -1.0),
                                  (3, 0, 0.5)]


def test_pattern_and_integer(tmp_path):
    A = mgb.CooMatrix(device="cpu")
    mgb.read_matrix_market_file(A, _write(tmp_path, "p.mtx",
                                          "%%MatrixMarket matrix coordinate pattern symmetric\n3 3 2\n2 1\n3 3\n"))
    assert _coo(A) == ([0, 1, 2], [1, 0, 2], [1.0, 1.0, 1.0])
    B = mgb.CooMatrix(device="cpu")
    mgb.read_matrix_market_file(B, _write(tmp_path, "i.mtx",
                                          "%%MatrixMarket matrix coordinate integer general\n2 2 2\n2 2 -3\n1 2 4\n"))
    assert _coo(B) == ([0, 1], [1, 1], [4.0, -3.0])


def test_duplicates_keep_file_order(tmp_path):
    A = mgb.CooMatrix(device="cpu")
    mgb.read_matrix_market_file(A, _write(tmp_path, "d.mtx",
                                          "%%MatrixMarket matrix coordinate real general\n2 2 3\n2 1 1\n1 1 2\n2 1 3\n"))
    assert _coo(A) == ([0, 1, 1], [0, 0, 0], [2.0, 1.0, 3.0])


@pytest.mark.parametrize("text,exc", [
    ("%%MatrixMarket matrix coordinate real general symmetric\n2 2 1\n1 1 1\n", mgb.IOException),
    ("%MatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix sparse real general\n2 2 1\n1 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate double general\n2 2 1\n1 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real upper\n2 2 1\n1 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1 5\n1 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n0 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 0 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 1\n1 3 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 2 4\n1 1 1.11\n2 2 1\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 1 1 0\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix coordinate real hermitian\n2 2 1\n1 1 1\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix coordinate real skew-symmetric\n2 2 1\n2 1 1\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix array real general\n2 1\n1\n2\n", mgb.IOException),  # array into a CooMatrix
])
def test_invalid_files(tmp_path, text, exc):
    with pytest.raises(exc):
        mgb.read_matrix_market_file(mgb.CooMatrix(device="cpu"), _write(tmp_path, "bad.mtx", text))


def test_dynamic_matrix_must_be_coo(tmp_path):
    f = _write(tmp_path, "g.mtx", GENERAL)
    dyn = mgb.DynamicMatrix(mgb.CsrMatrix(device="cpu"), device="cpu")
    with pytest.raises(mgb.RuntimeException):
        mgb.read_matrix_market_file(dyn, f)
    dyn.activate(mgb.COO_FORMAT)
    mgb.read_matrix_market_file(dyn, f)
    assert dyn.active_index() == mgb.COO_FORMAT and dyn.nnnz() == 5


@pytest.mark.parametrize("text,exc", [
    (None, None),
    ("%%MatrixMarket matrix array real general\n4 1 7\n1\n2\n3\n4\n", mgb.IOException),
    ("%%MatrixMarket matrix array real symmetric\n2 1\n1\n2\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix array complex general\n2 1\n1 0\n2 0\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix array pattern general\n2 1\n", mgb.NotImplementedException),
    ("%%MatrixMarket matrix array real general\n4 1\n1\n2\n", mgb.IOException),
    ("%%MatrixMarket matrix coordinate real general\n2 1 1\n1 1 1\n", mgb.IOException),
])
def test_vectors(tmp_path, text, exc):
    v = torch.zeros(0, dtype=torch.float64)
    if text is None:
        mgb.read_matrix_market_file(v, _write(tmp_path, "v.mtx",
                                              "%%MatrixMarket matrix array integer general\n4 1\n1\n-2\n3\n40\n"))
        assert v.tolist() == [1.0, -2.0, 3.0, 40.0]
        return
    with pytest.raises(exc):
        mgb.read_matrix_market_file(v, _write(tmp_path, "v.mtx", text))


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_write_read_roundtrip(tmp_path, dtype):
    from morpheus_gb300 import generators as gen
    hm = gen.power_law(500, seed=5)
    coo = mgb.CooMatrix(hm["nrows"], hm["ncols"], hm["nnz"],
                        np.repeat(np.arange(hm["nrows"]), np.diff(hm["row_offsets"])),
                        hm["column_indices"], hm["values"], dtype=dtype, device="cpu")
    f = str(tmp_path / "w.mtx")
    mgb.write_matrix_market_file(coo, f)
    B = mgb.CooMatrix(dtype=dtype, device="cpu")
    mgb.read_matrix_market_file(B, f)
    for a, b in zip(_coo(coo), _coo(B)):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    v = torch.linspace(-1, 1, 17, dtype=dtype)
    mgb.write_matrix_market_file(v, str(tmp_path / "v.mtx"))
    w = torch.zeros(0, dtype=dtype)
    mgb.read_matrix_market_file(w, str(tmp_path / "v.mtx"))
    assert torch.equal(v, w)


@pytest.mark.gpu
def test_read_to_device_and_multiply(cuda, tmp_path):
    from oracle import oracle as O
    A = mgb.CooMatrix(device="cuda")
    mgb.read_matrix_market_file(A, _write(tmp_path, "g.mtx", GENERAL))
    x = torch.tensor([1.0, -2.0, 0.5, 4.0], dtype=torch.float64, device="cuda")
    y = torch.zeros(3, dtype=torch.float64, device="cuda")
    mgb.multiply(A, x, y)
    ref = O.OracleMatrix.from_host(mgb.matrix_to_host(A)).multiply(x.cpu().numpy())
    assert np.array_equal(y.cpu().numpy(), ref)
