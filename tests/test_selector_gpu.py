"""GPU: analytics/feature kernel, selector network kernels (forward, gradient
against the FP64 NumPy oracle, Adam training) and the AUTO_FORMAT switch."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import golden
from morpheus_gb300 import analytics, corpus, selector
from morpheus_gb300 import generators as gen
from oracle import mlp_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _host_stats(A):
    ro = A["row_offsets"].astype(np.int64)
    lens = np.diff(ro)
    rows = np.repeat(np.arange(A["nrows"]), lens)
    d = A["column_indices"].astype(np.int64) - rows
    hist = np.bincount(d + A["nrows"] - 1, minlength=A["nrows"] + A["ncols"] - 1)
    min_elem = int(A["nrows"] * 0.2)
    true = (hist >= min_elem) & (hist > 0)
    return lens, hist, true, d


@pytest.mark.parametrize("case", ["golden", "power_law", "stencil", "empty_rows"])
def test_analytics_matches_host(cuda, case):
    if case == "golden":
        A = golden()["CSR"]
    elif case == "power_law":
        A = gen.power_law(20000, seed=1)
    elif case == "stencil":
        A = gen.add_offband(gen.stencil_27pt(14, seed=2), 0.01, seed=3)
    else:
        A = gen.random_csr(3000, 3000, 0.002, seed=4, empty_row_frac=0.3)
    st = analytics.analyze(mgb.matrix_from_host(A))
    lens, hist, true, d = _host_stats(A)
    assert st["average_nnnz"] == pytest.approx(lens.mean(), rel=1e-12)
    assert st["max_nnnz"] == lens.max() and st["min_nnnz"] == lens.min()
    assert st["std_nnnz"] == pytest.approx(lens.std(), rel=1e-9, abs=1e-12)
    assert st["count_diagonals"] == np.count_nonzero(hist)
    assert st["count_true_diagonals"] == np.count_nonzero(true)
    assert st["true_diagonal_nnz"] == hist[true].sum()
    assert st["bandwidth"] == np.abs(d).max()
    W = max(1, A["nnz"] // A["nrows"])
    assert st["hyb_coo_nnz"] == np.maximum(lens - W, 0).sum()
    # feasibility flags agree with the oracle's conversions
    om = O.OracleMatrix.from_host(A)
    for key, fmt in (("dia_feasible", O.DIA), ("ell_feasible", O.ELL), ("hyb_feasible", O.HYB),
                     ("hdc_feasible", O.HDC)):
        try:
            om.convert(fmt)
            ok = 1.0
        except O.OracleError:
            ok = 0.0
        assert st[key] == ok, key


def _random_problem(n, seed):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, 12)).astype(np.float32) * 3 + 1
    mu = X.mean(0).astype(np.float32)
    sigma = X.std(0).astype(np.float32) + 0.1
    feas = (rng.random((n, 6)) < 0.7).astype(np.uint8)
    feas[:, 1] = 1
    labels = np.array([rng.choice(np.flatnonzero(f)) for f in feas], np.int32)
    return X, mu, sigma, feas, labels


@pytest.mark.parametrize("n", [1, 37, 300])
def test_forward_and_gradient_match_fp64_oracle(cuda, n):
    X, mu, sigma, feas, labels = _random_problem(n, seed=n)
    sel = selector.Selector.random(mu, sigma, seed=3)
    p = sel.params.cpu().numpy()
    ref = mlp_oracle.forward(p, mu, sigma, X, feas)
    logp = sel.logp(X, feas)
    ok = feas > 0
    assert np.allclose(np.exp(logp[ok]), ref["p"][ok], rtol=1e-4, atol=1e-6)
    g, loss = sel.grad(X, labels, feas)
    g_ref, loss_ref = mlp_oracle.grad(p, mu, sigma, X, labels, feas)
    assert loss == pytest.approx(loss_ref, rel=1e-4)
    rel = np.linalg.norm(g - g_ref) / np.linalg.norm(g_ref)
    assert rel <= 1e-4, rel
    # deterministic
    g2, _ = sel.grad(X, labels, feas)
    assert np.array_equal(g, g2)


def test_training_learns_a_rule(cuda):
    rng = np.random.default_rng(5)
    n = 2000
    X = rng.normal(size=(n, 12)).astype(np.float32)
    labels = np.where(X[:, 0] > 0.5, 2, np.where(X[:, 1] < -0.3, 4, 1)).astype(np.int32)
    feas = np.ones((n, 6), np.uint8)
    sel = selector.Selector.random(X.mean(0), X.std(0), seed=1)
    hist = sel.train(X, labels, feas, epochs=60, lr=3e-3, batch=128)
    assert hist[-1] < 0.25 * hist[0]
    acc = np.mean(sel.predict(X, feas) == labels)
    assert acc > 0.95
    # infeasible formats are never chosen
    feas2 = feas.copy()
    feas2[:, 2] = 0
    assert not np.any(sel.predict(X, feas2) == 2)


def test_weights_roundtrip(cuda, tmp_path):
    X, mu, sigma, feas, _ = _random_problem(50, seed=9)
    sel = selector.Selector.random(mu, sigma, seed=4)
    path = str(tmp_path / "w.bin")
    sel.save(path, {"note": "test"})
    sel2 = selector.Selector.load(path)
    assert np.array_equal(sel.logp(X, feas), sel2.logp(X, feas))


def test_corpus_generation_and_measurement(cuda):
    for seed in range(6):
        A, desc = corpus.generate(seed)
        assert A.nnnz() <= corpus.NNZ_CAP * 1.06
        f, feas = analytics.features(A)
        assert np.all(np.isfinite(f)) and feas[0] == 1 and feas[1] == 1
    t = corpus.measure(A, reps=2)
    assert np.isfinite(t[0]) and np.isfinite(t[1]) and np.all(t > 0)


def test_auto_format_switch(cuda):
    X, mu, sigma, feas, _ = _random_problem(20, seed=10)
    sel = selector.Selector.random(mu, sigma, seed=5)
    selector._DEFAULT = sel  # any trained or untrained network exercises the path
    try:
        g = golden()
        dyn = mgb.DynamicMatrix(mgb.matrix_from_host(g["CSR"]))
        expect = selector.select_format(dyn)
        assert mgb.convert(dyn, selector.AUTO_FORMAT) == mgb.conversion_error_e.CONV_SUCCESS
        assert dyn.active_index() == expect
        x = torch.linspace(-1, 1, 10, dtype=torch.float64, device="cuda")
        y = torch.zeros(10, dtype=torch.float64, device="cuda")
        mgb.multiply(dyn, x, y)
        ref = O.OracleMatrix.from_host(g["CSR"]).multiply(x.cpu().numpy())
        assert np.allclose(y.cpu().numpy(), ref, rtol=1e-12, atol=1e-12)
    finally:
        selector._DEFAULT = None


@pytest.mark.parametrize("case", ["golden", "power_law", "stencil", "nonsquare"])
@pytest.mark.parametrize("fmt", ["CSR", "COO", "HYB"])
def test_count_nnz_per_row_and_diagonal(cuda, case, fmt):
    """count_nnz_per_row / count_nnz_per_diagonal / count_diagonals /
    count_true_diagonals against the oracle's per-diagonal count and host
    per-row lengths, on CSR, COO and (through COO) HYB containers."""
    if case == "golden":
        A = golden()["CSR"]
    elif case == "power_law":
        A = gen.power_law(20000, seed=31)
    elif case == "stencil":
        A = gen.stencil_27pt(14, seed=32)
    else:
        A = gen.random_csr(300, 1100, 0.02, seed=33)
    om = O.OracleMatrix.from_host(A)
    host = om.convert(FORMATS_IDX[fmt]).to_host()
    M = mgb.matrix_from_host(host, device="cuda")
    lens = np.diff(A["row_offsets"].astype(np.int64))
    diag = om.convert(O.COO).count_nnz_per_diagonal()
    rows = analytics.count_nnz_per_row(M)
    assert np.array_equal(rows.cpu().numpy(), lens)
    d = analytics.count_nnz_per_diagonal(M)
    assert np.array_equal(d.cpu().numpy(), diag)
    # init=False accumulates into the given vector
    analytics.count_nnz_per_diagonal(M, out=d, init=False)
    assert np.array_equal(d.cpu().numpy(), 2 * diag)
    analytics.count_nnz_per_row(M, out=rows, init=False)
    assert np.array_equal(rows.cpu().numpy(), 2 * lens)
    assert analytics.count_diagonals(M) == np.count_nonzero(diag)
    for thr in (0, 1, 5, int(0.2 * A["nrows"])):
        assert analytics.count_true_diagonals(M, thr) == np.count_nonzero(diag > thr)


FORMATS_IDX = {"COO": 0, "CSR": 1, "DIA": 2, "ELL": 3, "HYB": 4, "HDC": 5}
