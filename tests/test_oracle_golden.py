"""CPU: pin the oracle against the reference's own golden fixtures and known answers.

Fixtures: the 10x10 matrix of core/tests/utils/Macros_*.hpp in all six formats
(tests/golden/small_matrix.json, made by tests/golden/make_fixtures.py), the
banded multiply fixture shape of core/tests/Test_Multiply.hpp:161-186 with its
dense-product check and 1e-13 absolute tolerance
(core/tests/utils/Macros_DenseVector.hpp:187-223), and the dot / reduce known
answers of core/tests/Test_Dot.hpp:74-87 and core/tests/Test_Reduce.hpp:74-81.
"""
import numpy as np
import pytest

from helpers import FORMATS, assert_same_matrix, dense_of, golden
from morpheus_gb300 import generators as gen
from oracle import oracle as O

DTYPES = [np.float64, np.float32]


@pytest.fixture(autouse=True)
def _built(oracle_built):
    return oracle_built


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("fmt", FORMATS)
def test_golden_to_coo(fmt, dtype):
    """Every golden container converts to the golden COO (Serial X -> COO)."""
    g = golden(dtype)
    m = O.OracleMatrix.from_host(g[fmt])
    assert_same_matrix(m.convert(O.COO).to_host(), g["COO"])


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("fmt", FORMATS)
def test_coo_to_golden(fmt, dtype):
    """The golden COO converts to every golden container (Serial COO -> X),
    pinning the ELL max-width, HYB mean-width and HDC 0.2*N rules."""
    g = golden(dtype)
    out = O.OracleMatrix.from_host(g["COO"]).convert(FORMATS.index(fmt)).to_host()
    assert_same_matrix(out, g[fmt])


@pytest.mark.parametrize("src", FORMATS)
@pytest.mark.parametrize("dst", FORMATS)
def test_any_to_any_via_coo(src, dst):
    g = golden()
    out = O.OracleMatrix.from_host(g[src]).convert(FORMATS.index(dst)).to_host()
    assert_same_matrix(out, g[dst])


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("init", [True, False])
def test_golden_multiply(fmt, dtype, init):
    g = golden(dtype)
    A = dense_of(g["COO"])
    x = np.linspace(-1, 1, 10).astype(dtype)
    y0 = np.arange(10, dtype=dtype) * 0.5
    y = O.OracleMatrix.from_host(g[fmt]).multiply(x, y0.copy(), init=init)
    ref = A @ x.astype(np.float64) + (0 if init else y0.astype(np.float64))
    tol = 1e-13 * 100 if dtype == np.float64 else 1e-4
    assert np.max(np.abs(y - ref)) <= tol


@pytest.mark.parametrize("fmt", FORMATS)
def test_dynamic_inplace_roundtrip(fmt):
    """core/tests/Serial/Test_Convert_Dynamic.hpp:195-213: in-place convert to
    every format succeeds and converts back to the same COO."""
    g = golden()
    dyn = O.OracleMatrix.from_host(g[fmt])
    for target in range(6):
        assert dyn.convert_inplace(target) == 2  # CONV_SUCCESS
        assert dyn.format == target
        assert_same_matrix(dyn.convert(O.COO).to_host(), g["COO"])


@pytest.mark.parametrize("N", [10, 100, 1000])
@pytest.mark.parametrize("dtype", DTYPES)
def test_banded_multiply_all_formats(N, dtype):
    """Test_Multiply.hpp fixture shape: diagonals 0, +-5k; dense O(N^2) check."""
    A = gen.banded(N, diag_freq=5, seed=N, dtype=dtype)
    coo = O.OracleMatrix.from_host(A).convert(O.COO)
    x = gen.x_vector(N, seed=5374857, dtype=dtype)
    dense = dense_of(A).astype(dtype)
    ref = np.zeros(N, dtype=dtype)
    for i in range(N):  # the reference accumulates the dense product in value_type
        for j in np.flatnonzero(dense[i]):
            ref[i] += dense[i, j] * x[j]
    tol = 1e-13 if dtype == np.float64 else 1e-5
    for f in range(6):
        m = coo.convert(f)
        for init in (True, False):
            y = np.ones(N, dtype=dtype)
            m.multiply(x, y, init=init)
            expect = ref + (0 if init else 1)
            assert np.max(np.abs(y.astype(np.float64) - expect)) <= tol * (10 if dtype == np.float64 else 10)


@pytest.mark.parametrize("n", [50, 5000, 50000])
def test_dot_known_answer(n):
    x = np.arange(1, n + 1, dtype=np.float64)
    y = (n - np.arange(n)).astype(np.float64)
    exact = sum((i + 1) * (n - i) for i in range(n))
    assert O.dot(n, x, y) == exact


@pytest.mark.parametrize("vsize,rsize", [(50, 50), (50, 25), (5000, 5000), (5000, 1000), (50000, 50000), (50000, 100)])
def test_reduce_known_answer(vsize, rsize):
    d = np.arange(vsize, dtype=np.float64) + 1.5
    exact = sum(i + 1.5 for i in range(rsize))
    assert O.reduce(d, rsize) == exact


def test_waxpby_matches_formula():
    rng = np.random.default_rng(3)
    for n in (50, 5000, 50000):
        x = rng.uniform(-5, 5, n)
        y = rng.uniform(-2, 2, n)
        w = np.zeros(n)
        O.waxpby(n, 2.15, x, -3.2, y, w)
        assert np.array_equal(w, 2.15 * x + (-3.2) * y)
        O.waxpby(n, 1.0, x, -3.2, y, w)
        assert np.array_equal(w, x + (-3.2) * y)


def test_exceeds_tolerance_rule():
    # core/src/impl/Morpheus_Utils.hpp:91-105: fill > 10 and size > 1e8
    assert O.exceeds_tolerance(2_000_000, 30_000_000, 2974)
    assert not O.exceeds_tolerance(4_096_000, 109_215_352, 27)
    assert not O.exceeds_tolerance(10, 32, 9)


def test_coo_to_ell_throws_on_fill():
    N = 1_000_000
    lens = np.zeros(N, dtype=np.int64)
    lens[::1000] = 1
    lens[7] = 500  # one long row -> W = 500, fill = N*W/nnz >> 10, N*W > 1e8
    A = gen.random_lengths_csr(N, N, lens, seed=1)
    m = O.OracleMatrix.from_host(A)
    with pytest.raises(O.OracleError) as e:
        m.convert(O.ELL)
    assert e.value.status == O.STATUS_FORMAT_CONVERSION
    dyn = O.OracleMatrix.from_host(A)
    assert dyn.convert_inplace(O.ELL) == 1  # PROXY_TO_DYNAMIC, data kept
    assert dyn.format == O.CSR


def test_dia_to_coo_drops_explicit_zeros():
    g = golden()
    d = dict(g["DIA"])
    d["values"] = d["values"].copy()
    d["values"][4 + 32 * 0] = 0.0  # no-op (already padding)
    # zero an existing entry: (3, 0) sits on diagonal -3 (column 3 of the slab)
    d["values"][3 + 32 * 3] = 0.0
    coo = O.OracleMatrix.from_host(d).convert(O.COO).to_host()
    # nnz stays 32; the dropped entry leaves a zero-initialised (0,0,0) tail
    # entry that the stable sort places right after the real (0,0) entry
    assert coo["nnz"] == 32
    assert coo["values"][0] == 1.11
    assert coo["row_indices"][1] == 0 and coo["column_indices"][1] == 0 and coo["values"][1] == 0.0
    assert 11.11 not in coo["values"].tolist()


def test_sort_is_stable_with_duplicates():
    hm = {"format": 0, "nrows": 3, "ncols": 3, "nnz": 6,
          "row_indices": np.array([2, 0, 2, 0, 1, 2], np.int32),
          "column_indices": np.array([1, 2, 1, 0, 1, 0], np.int32),
          "values": np.array([1, 2, 3, 4, 5, 6], np.float64)}
    m = O.OracleMatrix.from_host(hm)
    assert not m.is_sorted()
    m.sort_by_row_and_column()
    out = m.to_host()
    assert out["row_indices"].tolist() == [0, 0, 1, 2, 2, 2]
    assert out["column_indices"].tolist() == [0, 2, 1, 0, 1, 1]
    assert out["values"].tolist() == [4, 2, 5, 6, 1, 3]
    assert m.is_sorted()


def test_unsorted_coo_to_csr_keeps_coo_order():
    hm = {"format": 0, "nrows": 3, "ncols": 4, "nnz": 5,
          "row_indices": np.array([2, 0, 2, 0, 1], np.int32),
          "column_indices": np.array([3, 2, 0, 1, 1], np.int32),
          "values": np.array([1, 2, 3, 4, 5], np.float64)}
    out = O.OracleMatrix.from_host(hm).convert(O.CSR).to_host()
    assert out["row_offsets"].tolist() == [0, 2, 3, 5]
    assert out["column_indices"].tolist() == [2, 1, 1, 3, 0]
    assert out["values"].tolist() == [2, 4, 5, 1, 3]


def test_hdc_nonsquare_midpoint_quirk():
    """COO -> HDC records the midpoint bin as offset 0, exact for square
    matrices only (impl/Hdc/Serial/Morpheus_Convert_Impl.hpp:186-190).  For a
    non-square matrix whose midpoint-bin diagonal is a true diagonal, its
    entries match no stored offset and overflow the CSR part, which was sized
    without them (undefined behaviour in the reference); the oracle raises."""
    N, M = 10, 20
    rows = np.repeat(np.arange(N), 2).astype(np.int32)
    cols = np.stack([np.arange(N) + 5, np.arange(N) + 10], 1).reshape(-1).astype(np.int32)
    hm = {"format": 0, "nrows": N, "ncols": M, "nnz": 2 * N, "row_indices": rows,
          "column_indices": cols, "values": np.arange(1, 2 * N + 1, dtype=np.float64)}
    with pytest.raises(O.OracleError) as e:
        O.OracleMatrix.from_host(hm).convert(O.HDC)
    assert e.value.status == O.STATUS_RUNTIME
    # a non-square matrix whose true diagonals avoid the midpoint bin converts
    cols2 = np.stack([np.arange(N) + 2, np.arange(N) + 10], 1).reshape(-1).astype(np.int32)
    hm2 = dict(hm, column_indices=cols2)
    out = O.OracleMatrix.from_host(hm2).convert(O.HDC).to_host()
    assert out["dia"]["diagonal_offsets"].tolist() == [2, 10]
    assert out["csr"]["nnz"] == 0


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_host_builders_match_oracle_convert(seed):
    """The vectorised builders used for large workloads produce the same
    structures as the oracle's convert (so the large benchmarks run on
    reference-identical containers)."""
    A = gen.power_law(3000, mu=1.5, sigma=1.0, max_len=200, seed=seed)
    m = O.OracleMatrix.from_host(A)
    assert_same_matrix(gen.csr_to_coo_host(A), m.convert(O.COO).to_host())
    assert_same_matrix(gen.csr_to_ell_host(A), m.convert(O.ELL).to_host())
    W = max(1, A["nnz"] // A["nrows"])
    assert_same_matrix(gen.csr_to_hyb_host(A, W), m.convert(O.HYB).to_host())
    coo = m.convert(O.COO)
    assert_same_matrix(gen.csr_to_hyb_host(A, 7), coo.coo_to_hyb(7).to_host())
    S = gen.add_offband(gen.stencil_27pt(12, seed=seed), 0.01, seed=seed + 1)
    s = O.OracleMatrix.from_host(S)
    assert_same_matrix(gen.csr_to_hdc_host(S), s.convert(O.HDC).to_host())
    P = gen.stencil_27pt(10, seed=seed)
    assert_same_matrix(gen.csr_to_dia_host(P), O.OracleMatrix.from_host(P).convert(O.DIA).to_host())


def test_generator_sizes():
    assert gen.laplacian_2d(256)["nnz"] == 326_656
    n = 20
    assert gen.stencil_27pt(n)["nnz"] == (3 * n - 2) ** 3
    A = gen.power_law(20000, seed=0)
    lens = np.diff(A["row_offsets"])
    assert lens.min() >= 1 and lens.max() <= 4096
    # columns strictly increasing within every row
    ro, ci = A["row_offsets"], A["column_indices"]
    d = np.diff(ci.astype(np.int64))
    starts = np.zeros(A["nnz"], bool)
    starts[ro[:-1][lens > 0]] = True
    assert np.all(d[~starts[1:]] > 0)


def _numpy_counts(hm: dict):
    """Independent per-format counts (the reference's rules, in numpy)."""
    f, N, M = hm["format"], hm["nrows"], hm["ncols"]
    rows = np.zeros(N, dtype=np.int64)
    diag = np.zeros(N + M - 1, dtype=np.int64)
    if f == 0:
        np.add.at(rows, hm["row_indices"], 1)
        np.add.at(diag, hm["column_indices"] - hm["row_indices"] + N - 1, 1)
    elif f == 1:
        lens = np.diff(hm["row_offsets"])
        rows += lens
        r = np.repeat(np.arange(N), lens)
        np.add.at(diag, hm["column_indices"] - r + N - 1, 1)
    elif f == 2:
        P, off = hm["pitch"], hm["diagonal_offsets"]
        v = hm["values"].reshape(hm["ndiags"], P)
        for k, o in enumerate(off):
            c = np.arange(N) + o
            rows += (c >= 0) & (c < M)
            diag[o + N - 1] += np.count_nonzero(v[k])
    elif f == 3:
        W, P = hm["width"], hm["pitch"]
        ci = hm["column_indices"].reshape(W, P)[:, :N].T
        v = hm["values"].reshape(W, P)[:, :N].T
        valid = ci != -1
        rows += valid.sum(1)
        good = valid & (v != 0)
        k = good.sum(1)
        for i in range(N):
            for n in range(k[i]):
                if good[i, n]:
                    diag[ci[i, n] - i + N - 1] += 1
    else:
        a, b = (hm["ell"], hm["coo"]) if f == 4 else (hm["dia"], hm["csr"])
        ra, da = _numpy_counts(a)
        rb, db = _numpy_counts(b)
        rows, diag = ra + rb, da + db
    return rows, diag


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("fmt", FORMATS)
def test_counts_per_format_golden(fmt, dtype):
    """count_nnz_per_row / count_nnz_per_diagonal of every golden container
    by the format's own rule (impl/<Fmt>/Serial/Morpheus_NonZeros_Per_Row_Impl.hpp,
    impl/<Fmt>/{Kokkos,Serial}/Morpheus_NonZeros_Per_Diagonal_Impl.hpp),
    against an independent numpy restatement; init=False accumulates."""
    hm = golden(dtype)[fmt]
    om = O.OracleMatrix.from_host(hm)
    rows, diag = _numpy_counts(hm)
    assert np.array_equal(om.count_nnz_per_row(), rows)
    assert np.array_equal(om.count_nnz_per_diagonal(), diag)
    r2 = om.count_nnz_per_row()
    om.count_nnz_per_row(out=r2, init=False)
    assert np.array_equal(r2, 2 * rows)
    d2 = om.count_nnz_per_diagonal()
    om.count_nnz_per_diagonal(out=d2, init=False)
    assert np.array_equal(d2, 2 * diag)
    # the golden matrix stores no explicit zeros: every format counts its 32 entries
    assert diag.sum() == 32 and (fmt == "DIA" or fmt == "HDC" or rows.sum() == 32)


def test_counts_format_quirks():
    """DIA rows count in-range diagonal slots, explicit zeros included; an ELL
    row whose valid nonzero slots do not come first loses the later ones in
    the per-diagonal count (the reference's scan of the first k slots)."""
    dia = {"format": 2, "nrows": 4, "ncols": 4, "nnz": 5, "ndiags": 2, "pitch": 32, "alignment": 32,
           "diagonal_offsets": np.array([0, 1], np.int32), "values": np.zeros(64)}
    dia["values"][[0, 1, 2, 3]] = [1.0, 0.0, 3.0, 4.0]  # main diagonal, an explicit zero in row 1
    dia["values"][32 + 0] = 5.0                        # (0, 1)
    om = O.OracleMatrix.from_host(dia)
    assert om.count_nnz_per_row().tolist() == [2, 2, 2, 1]
    d = om.count_nnz_per_diagonal()
    assert d[3] == 3 and d[4] == 1 and d.sum() == 4
    ell = {"format": 3, "nrows": 2, "ncols": 5, "nnz": 4, "entries_per_row": 3, "width": 32, "pitch": 2,
           "alignment": 32, "column_indices": np.full(64, -1, np.int32), "values": np.zeros(64)}
    ell["column_indices"][[0, 4]] = [0, 3]   # row 0: slot 0 -> col 0, slot 2 -> col 3 (slot 1 a gap)
    ell["values"][[0, 4]] = [1.0, 2.0]
    ell["column_indices"][[1, 3]] = [1, 2]   # row 1: slot 0 -> col 1 holding 0.0, slot 1 -> col 2
    ell["values"][[1, 3]] = [0.0, 7.0]
    om = O.OracleMatrix.from_host(ell)
    assert om.count_nnz_per_row().tolist() == [2, 2]
    d = om.count_nnz_per_diagonal()
    # row 0: k = 2, slots 0..1 -> only (0, 0); row 1: k = 1, slot 0 holds a zero -> nothing
    assert d.tolist() == [0, 1, 0, 0, 0, 0]
