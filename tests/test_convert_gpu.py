"""GPU parity of format conversion: every result must be bit-identical to the
oracle's Serial convert (indices, values, padding, order, tie-breaks, sizes)."""
import numpy as np
import pytest

import morpheus_gb300 as mgb
from helpers import FORMATS, assert_same_matrix, golden
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def gpu_convert(hm, fmt, hyb_width=0):
    A = mgb.matrix_from_host(hm, device="cuda")
    if A.FORMAT == fmt:
        out = A
    else:
        coo = mgb.to_coo(A) if A.FORMAT != 0 else A
        out = mgb.from_coo(coo, fmt, hyb_width=hyb_width)
    return mgb.matrix_to_host(out)


def oracle_convert(hm, fmt, hyb_width=0):
    om = O.OracleMatrix.from_host(hm)
    if fmt == O.HYB and hyb_width:
        return om.convert(O.COO).coo_to_hyb(hyb_width).to_host()
    return om.convert(fmt).to_host()


def both(hm, fmt, hyb_width=0):
    """(gpu, oracle) results, or the exception class both raise."""
    try:
        ref = oracle_convert(hm, fmt, hyb_width)
    except O.OracleError as e:
        ref = e.status
    try:
        got = gpu_convert(hm, fmt, hyb_width)
    except mgb.MorpheusException as e:
        got = e
    return got, ref


def check_all_targets(hm, formats=range(6)):
    for f in formats:
        got, ref = both(hm, f)
        if isinstance(ref, int):
            expect = {O.STATUS_FORMAT_CONVERSION: mgb.FormatConversionException,
                      O.STATUS_RUNTIME: mgb.RuntimeException}[ref]
            assert isinstance(got, expect), f"target {FORMATS[f]}: expected {expect.__name__}, got {got!r}"
        else:
            assert not isinstance(got, Exception), f"target {FORMATS[f]}: {got!r}"
            assert_same_matrix(got, ref, f"{FORMATS[f]}:")


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("src", FORMATS)
@pytest.mark.parametrize("dst", FORMATS)
def test_golden_pairs(cuda, src, dst, dtype):
    g = golden(dtype)
    out = gpu_convert(g[src], FORMATS.index(dst))
    assert_same_matrix(out, g[dst])


@pytest.mark.parametrize("fmt", FORMATS)
def test_dynamic_inplace(cuda, fmt):
    g = golden()
    dyn = mgb.DynamicMatrix(mgb.matrix_from_host(g[fmt]))
    for target in range(6):
        assert mgb.convert(dyn, target) == mgb.conversion_error_e.CONV_SUCCESS
        assert dyn.active_index() == target
        assert_same_matrix(mgb.matrix_to_host(mgb.to_coo(dyn)), g["COO"])


def test_convert_into_container(cuda):
    g = golden()
    src = mgb.matrix_from_host(g["CSR"])
    dst = mgb.DiaMatrix()
    mgb.convert(src, dst)
    assert_same_matrix(mgb.matrix_to_host(dst), g["DIA"])
    hyb = mgb.HybMatrix()
    mgb.convert(dst, hyb)
    assert_same_matrix(mgb.matrix_to_host(hyb), g["HYB"])


@pytest.mark.parametrize("seed", [0, 1])
def test_power_law_all_targets(cuda, seed):
    A = gen.power_law(20000, mu=1.8, sigma=1.1, max_len=600, seed=seed)
    check_all_targets(A)
    p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
    got, ref = both(gen.csr_to_coo_host(A), O.HYB, hyb_width=p90)
    assert_same_matrix(got, ref)


def test_stencil_and_offband(cuda):
    S = gen.stencil_27pt(14, seed=2)
    check_all_targets(S)
    check_all_targets(gen.add_offband(S, 0.01, seed=3))


def test_banded_and_laplacian(cuda):
    check_all_targets(gen.banded(500, seed=4))
    check_all_targets(gen.laplacian_2d(40))


def test_empty_rows_and_nonsquare(cuda):
    check_all_targets(gen.random_csr(3000, 3000, 0.003, seed=5, empty_row_frac=0.4))
    check_all_targets(gen.random_csr(700, 1900, 0.01, seed=6))
    check_all_targets(gen.random_csr(1900, 700, 0.01, seed=7))


def _coo(rows, cols, vals, n, m):
    return {"format": 0, "nrows": n, "ncols": m, "nnz": len(rows),
            "row_indices": np.asarray(rows, np.int32), "column_indices": np.asarray(cols, np.int32),
            "values": np.asarray(vals, np.float64)}


def test_unsorted_and_duplicate_coo(cuda):
    rng = np.random.default_rng(8)
    A = gen.csr_to_coo_host(gen.random_csr(400, 400, 0.02, seed=9))
    perm = rng.permutation(A["nnz"])
    shuffled = dict(A, row_indices=A["row_indices"][perm], column_indices=A["column_indices"][perm],
                    values=A["values"][perm])
    check_all_targets(shuffled)
    # duplicates (same (r, c) several times, with different values)
    dup_idx = rng.integers(0, A["nnz"], 300)
    dup = dict(A, nnz=A["nnz"] + 300,
               row_indices=np.concatenate([A["row_indices"], A["row_indices"][dup_idx]]),
               column_indices=np.concatenate([A["column_indices"], A["column_indices"][dup_idx]]),
               values=np.concatenate([A["values"], rng.standard_normal(300)]))
    check_all_targets(dup)
    perm2 = rng.permutation(dup["nnz"])
    check_all_targets(dict(dup, row_indices=dup["row_indices"][perm2],
                           column_indices=dup["column_indices"][perm2], values=dup["values"][perm2]))


def test_sort_matches_oracle(cuda):
    rng = np.random.default_rng(10)
    n = 5000
    hm = _coo(rng.integers(0, 300, n), rng.integers(0, 50, n), rng.standard_normal(n), 300, 50)
    om = O.OracleMatrix.from_host(hm)
    om.sort_by_row_and_column()
    A = mgb.matrix_from_host(hm)
    assert not mgb.is_sorted(A)
    mgb.sort_by_row_and_column(A)
    assert mgb.is_sorted(A)
    assert_same_matrix(mgb.matrix_to_host(A), om.to_host())


def test_dia_with_explicit_zero_tail(cuda):
    g = golden()
    d = dict(g["DIA"])
    d["values"] = d["values"].copy()
    d["values"][3 + 32 * 3] = 0.0  # drop entry (3, 0)
    got, ref = both(d, O.COO)
    assert_same_matrix(got, ref)
    for f in range(1, 6):
        got, ref = both(ref, f)
        if not isinstance(ref, int):
            assert_same_matrix(got, ref)


def test_ell_with_gaps_and_unsorted_rows(cuda):
    g = golden()
    e = dict(g["ELL"])
    ci, v = e["column_indices"].copy(), e["values"].copy()
    p = e["pitch"]
    # swap slots 0 and 1 of row 0 (columns out of order), put a gap in row 1
    ci[0], ci[p] = ci[p], ci[0]
    v[0], v[p] = v[p], v[0]
    ci[1 + p], v[1 + p] = -1, 0.0
    e.update(column_indices=ci, values=v, nnz=31)
    got, ref = both(e, O.COO)
    assert_same_matrix(got, ref)


def test_hyb_with_unsorted_coo_part(cuda):
    g = golden()
    h = {k: (dict(v) if isinstance(v, dict) else v) for k, v in g["HYB"].items()}
    c = h["coo"]
    c["row_indices"] = c["row_indices"][[0, 2, 1]].copy()
    c["column_indices"] = c["column_indices"][[0, 2, 1]].copy()
    c["values"] = c["values"][[0, 2, 1]].copy()
    got, ref = both(h, O.COO)
    assert_same_matrix(got, ref)


def test_hdc_nonsquare_midpoint_raises(cuda):
    N, M = 10, 20
    rows = np.repeat(np.arange(N), 2)
    cols = np.stack([np.arange(N) + 5, np.arange(N) + 10], 1).reshape(-1)
    got, ref = both(_coo(rows, cols, np.arange(1, 2 * N + 1), N, M), O.HDC)
    assert ref == O.STATUS_RUNTIME and isinstance(got, mgb.RuntimeException)


def test_fill_tolerance_rejections(cuda):
    N = 1_000_000
    lens = np.zeros(N, dtype=np.int64)
    lens[::1000] = 1
    lens[7] = 500
    A = gen.random_lengths_csr(N, N, lens, seed=11)
    for f in (O.ELL,):
        got, ref = both(A, f)
        assert ref == O.STATUS_FORMAT_CONVERSION
        assert isinstance(got, mgb.FormatConversionException)
    dyn = mgb.DynamicMatrix(mgb.matrix_from_host(A))
    assert mgb.convert(dyn, mgb.ELL_FORMAT) == mgb.conversion_error_e.PROXY_TO_DYNAMIC
    assert dyn.active_index() == mgb.CSR_FORMAT


@pytest.mark.slow
def test_power_law_full_size_roundtrip(cuda):
    """Full power-law size: CSR -> COO -> HYB(p90) -> COO -> CSR is the identity
    (size-independent property; the oracle is not needed at this size)."""
    import torch
    A = gen.power_law(2_000_000, seed=0)
    M = mgb.matrix_from_host(A)
    p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
    hyb = mgb.from_coo(mgb.to_coo(M), mgb.HYB_FORMAT, hyb_width=p90)
    back = mgb.from_coo(mgb.to_coo(hyb), mgb.CSR_FORMAT)
    assert torch.equal(back.row_offsets().cpu(), M.row_offsets().cpu())
    assert torch.equal(back.column_indices().cpu(), M.column_indices().cpu())
    assert torch.equal(back.values().cpu(), M.values().cpu())
    with pytest.raises(mgb.FormatConversionException):  # W = max row ~2974: the reference throws too
        mgb.from_coo(mgb.to_coo(M), mgb.ELL_FORMAT)
