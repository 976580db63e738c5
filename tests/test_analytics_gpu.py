"""GPU: analytics of every format read in place.

count_nnz_per_row / count_nnz_per_diagonal of all six formats (FP64 and FP32
containers) must equal the oracle's restatement of the reference's
per-format rules bit for bit, with init and accumulate.  The statistics and
the selector's 12 features describe the matrix's COO form, so for a matrix
without explicit zeros they must be identical in every format -- and no
format may be converted to get them.
"""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import FORMATS, golden
from morpheus_gb300 import analytics, selector
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(name, dtype):
    if name == "golden":
        return golden(dtype)["CSR"]
    if name == "power_law":
        return gen.power_law(20000, seed=41, dtype=dtype)
    if name == "stencil_offband":
        return gen.add_offband(gen.stencil_27pt(16, seed=42, dtype=dtype), 0.01, seed=43)
    if name == "empty_rows":
        return gen.random_csr(3000, 3000, 0.002, seed=44, dtype=dtype, empty_row_frac=0.3)
    if name == "nonsquare":
        return gen.random_csr(300, 1100, 0.02, seed=45, dtype=dtype)
    raise ValueError(name)


def _all_formats(A):
    om = O.OracleMatrix.from_host(A)
    out = {}
    for f, name in enumerate(FORMATS):
        try:
            out[name] = om.convert(f).to_host()
        except O.OracleError:
            pass  # refused by the fill tolerance, as in the reference
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["golden", "power_law", "stencil_offband", "empty_rows", "nonsquare"])
def test_counts_every_format_match_oracle(cuda, case, dtype):
    for name, hm in _all_formats(_case(case, dtype)).items():
        om = O.OracleMatrix.from_host(hm)
        M = mgb.matrix_from_host(hm, device="cuda")
        want_r, want_d = om.count_nnz_per_row(), om.count_nnz_per_diagonal()
        r = analytics.count_nnz_per_row(M)
        d = analytics.count_nnz_per_diagonal(M)
        assert np.array_equal(r.cpu().numpy(), want_r), f"{name}: rows"
        assert np.array_equal(d.cpu().numpy(), want_d), f"{name}: diagonals"
        analytics.count_nnz_per_row(M, out=r, init=False)
        analytics.count_nnz_per_diagonal(M, out=d, init=False)
        assert np.array_equal(r.cpu().numpy(), 2 * want_r), f"{name}: rows accumulated"
        assert np.array_equal(d.cpu().numpy(), 2 * want_d), f"{name}: diagonals accumulated"
        assert analytics.count_diagonals(M) == np.count_nonzero(want_d)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_counts_format_quirks(cuda, dtype):
    """DIA explicit zeros and ELL rows with gaps: the reference's rules, not
    the entry count (oracle pinned in test_oracle_golden.test_counts_format_quirks)."""
    dia = {"format": 2, "nrows": 40, "ncols": 40, "nnz": 70, "ndiags": 3, "pitch": 64, "alignment": 32,
           "diagonal_offsets": np.array([-1, 0, 5], np.int32), "values": np.zeros(192, dtype)}
    rng = np.random.default_rng(7)
    dia["values"][:] = rng.choice([0.0, 1.5, -2.0], 192).astype(dtype)
    ell = {"format": 3, "nrows": 50, "ncols": 60, "nnz": 80, "entries_per_row": 4, "width": 32, "pitch": 50,
           "alignment": 32, "column_indices": np.full(1600, -1, np.int32), "values": np.zeros(1600, dtype)}
    slots = rng.random(1600) < 0.1
    ell["column_indices"][slots] = rng.integers(0, 60, slots.sum())
    ell["values"][slots] = rng.choice([0.0, 3.0], slots.sum()).astype(dtype)
    for hm in (dia, ell):
        om = O.OracleMatrix.from_host(hm)
        M = mgb.matrix_from_host(hm, device="cuda")
        assert np.array_equal(analytics.count_nnz_per_row(M).cpu().numpy(), om.count_nnz_per_row())
        assert np.array_equal(analytics.count_nnz_per_diagonal(M).cpu().numpy(), om.count_nnz_per_diagonal())


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("case", ["golden", "power_law", "stencil_offband", "empty_rows", "nonsquare"])
def test_statistics_and_features_same_in_every_format(cuda, case, dtype, monkeypatch):
    """analyze() and features() read every format in place (a conversion
    would raise here) and agree with the CSR values exactly."""
    A = _case(case, dtype)
    ref_st = analytics.analyze(mgb.matrix_from_host(A, device="cuda"))
    ref_f, ref_m = analytics.features(mgb.matrix_from_host(A, device="cuda"))
    forms = {name: mgb.matrix_from_host(hm, device="cuda") for name, hm in _all_formats(A).items()}
    import sys
    conv = sys.modules["morpheus_gb300.convert"]  # the module (the package re-exports a function of that name)

    def no_conversion(*a, **k):
        raise AssertionError("analytics converted the matrix")
    monkeypatch.setattr(conv, "to_coo", no_conversion)
    monkeypatch.setattr(conv, "from_coo", no_conversion)
    for name, M in forms.items():
        st = analytics.analyze(M)
        assert st == ref_st, f"{name}: {st} != {ref_st}"
        f, m = analytics.features(M)
        assert np.array_equal(f.view(np.uint32), ref_f.view(np.uint32)), name
        assert np.array_equal(m, ref_m), name
        dyn = mgb.DynamicMatrix(M)
        f2, _ = analytics.features(dyn)
        assert np.array_equal(f2.view(np.uint32), ref_f.view(np.uint32)), f"{name} (dynamic)"


def test_selector_choice_independent_of_active_format(cuda):
    A = gen.stencil_27pt(20, seed=46)
    choices = set()
    for name, hm in _all_formats(A).items():
        dyn = mgb.DynamicMatrix(mgb.matrix_from_host(hm, device="cuda"))
        choices.add(selector.select_format(dyn))
    assert len(choices) == 1
    _ = torch
