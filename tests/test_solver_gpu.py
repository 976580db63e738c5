"""Fused solver steps (SpMV + dot, waxpby + dot) and device CG against the
oracle.  The SpMV half of multiply_dot runs the same kernel code as multiply,
so y must be bit-identical to it; dots and CG iterates are compared within
FP64 tolerances; CG's recurrence is checked against the FP64 restatement in
oracle/cg_oracle.py and its solution against the true residual b - A x."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import golden
from morpheus_gb300 import generators as gen
from morpheus_gb300 import solvers
from oracle import cg_oracle
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _spd_banded(n, seed):
    """Symmetric, strictly diagonally dominant (so SPD) banded matrix."""
    rng = np.random.default_rng(seed)
    rows, cols, vals = [], [], []
    for d in (1, 2, 7, 40):
        i = np.arange(n - d)
        v = rng.uniform(-1, 1, n - d)
        rows += [i, i + d]
        cols += [i + d, i]
        vals += [v, v]
    rows, cols, vals = np.concatenate(rows), np.concatenate(cols), np.concatenate(vals)
    off = np.zeros(n)
    np.add.at(off, rows, np.abs(vals))
    rows = np.concatenate([rows, np.arange(n)])
    cols = np.concatenate([cols, np.arange(n)])
    vals = np.concatenate([vals, off + 1.0])
    o = np.lexsort((cols, rows))
    return gen.csr_from_sorted_keys(n, n, rows[o], cols[o], vals[o])


CASES = {
    "golden": lambda dt: {k: (v.astype(dt) if isinstance(v, np.ndarray) and v.dtype.kind == "f" else v)
                          for k, v in golden()["CSR"].items()},
    "laplacian": lambda dt: gen.laplacian_2d(70, dtype=dt),
    "stencil": lambda dt: gen.stencil_27pt(18, seed=3, dtype=dt),
    "power_law": lambda dt: gen.power_law(30000, seed=4, dtype=dt),
    "empty_rows": lambda dt: gen.random_csr(3000, 3000, 0.003, seed=5, dtype=dt, empty_row_frac=0.4),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("variant", [mgb.CSR_SEGMENTS, mgb.CSR_ROWS, mgb.CSR_SPLIT, mgb.CSR_ROWS_GATHER])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_multiply_dot(cuda, case, variant, dtype):
    hm = CASES[case](dtype)
    A = mgb.matrix_from_host(hm, device="cuda")
    A._variant = variant
    x = torch.from_numpy(gen.x_vector(hm["ncols"], seed=1, dtype=dtype)).cuda()
    y0 = torch.from_numpy(gen.x_vector(hm["nrows"], seed=2, dtype=dtype)).cuda()
    for init in (True, False):
        y_ref = y0.clone()
        mgb.multiply(A, x, y_ref, init=init)
        y = y0.clone()
        d = solvers.multiply_dot(A, x, y, init=init)
        assert torch.equal(y, y_ref)  # same SpMV code: bit-identical
        ref = float(np.dot(x[:hm["nrows"]].double().cpu().numpy(), y_ref.double().cpu().numpy()))
        scale = float(np.dot(np.abs(x[:hm["nrows"]].double().cpu().numpy()), np.abs(y_ref.double().cpu().numpy())))
        tol = 1e-13 if dtype == np.float64 else 1e-5
        assert abs(float(d.item()) - ref) <= tol * max(scale, 1e-300)


def test_multiply_dot_deterministic(cuda):
    hm = gen.power_law(50000, seed=6)
    A = mgb.matrix_from_host(hm, device="cuda")
    x = torch.from_numpy(gen.x_vector(hm["ncols"], seed=1)).cuda()
    y = torch.empty(hm["nrows"], dtype=torch.float64, device="cuda")
    a = solvers.multiply_dot(A, x, y).item()
    b = solvers.multiply_dot(A, x, y).item()
    assert a == b


def test_multiply_dot_needs_rows_le_cols(cuda):
    hm = gen.random_csr(50, 20, 0.2, seed=7)
    A = mgb.matrix_from_host(hm, device="cuda")
    with pytest.raises(mgb.InvalidInputException):
        solvers.multiply_dot(A, torch.zeros(20, dtype=torch.float64, device="cuda"),
                             torch.zeros(50, dtype=torch.float64, device="cuda"))


@pytest.mark.parametrize("n", [1, 1000, 1_000_003])
def test_waxpby_dot(cuda, n):
    x = torch.from_numpy(gen.x_vector(n, seed=8)).cuda()
    y = torch.from_numpy(gen.x_vector(n, seed=9)).cuda()
    w = torch.empty_like(x)
    d = solvers.waxpby_dot(n, 0.5, x, -2.0, y, w)
    wr = O.waxpby(n, 0.5, x.cpu().numpy(), -2.0, y.cpu().numpy(), np.zeros(n))
    assert np.allclose(w.cpu().numpy(), wr, rtol=0, atol=4e-16 * (np.abs(wr) + 1))
    assert abs(d.item() - float(wr @ wr)) <= 1e-13 * float(wr @ wr)


@pytest.mark.parametrize("variant", [mgb.CSR_SEGMENTS, mgb.CSR_ROWS, mgb.CSR_SPLIT, mgb.CSR_ROWS_GATHER])
def test_cg_follows_the_recurrence(cuda, variant):
    """25 iterations (rtol 0): the device iterate equals the FP64 restatement
    to rounding (CG amplifies rounding differences slowly on a
    well-conditioned matrix)."""
    hm = _spd_banded(5000, seed=10)
    b = gen.x_vector(5000, seed=11)
    x0 = gen.x_vector(5000, seed=12) * 0.1
    xr, itr, resr = cg_oracle.cg(hm, b, x0, 25, 0.0)
    A = mgb.matrix_from_host(hm, device="cuda")
    A._variant = variant
    x = torch.from_numpy(x0.copy()).cuda()
    it, res = solvers.cg(A, torch.from_numpy(b).cuda(), x, max_iters=25, rtol=0.0)
    assert it == itr == 25
    assert np.linalg.norm(x.cpu().numpy() - xr) <= 1e-10 * np.linalg.norm(xr)
    assert res == pytest.approx(resr, rel=1e-6)


@pytest.mark.parametrize("case", ["laplacian", "spd_banded"])
def test_cg_converges(cuda, case):
    hm = gen.laplacian_2d(100) if case == "laplacian" else _spd_banded(20000, seed=13)
    n = hm["nrows"]
    b = gen.x_vector(n, seed=14)
    A = mgb.matrix_from_host(hm, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, res = solvers.cg(A, torch.from_numpy(b).cuda(), x, max_iters=5000, rtol=1e-10)
    assert 0 < it < 5000 and res <= 1e-10
    true_res = b - O.OracleMatrix.from_host(hm).multiply(x.cpu().numpy())
    assert np.linalg.norm(true_res) <= 1e-8 * np.linalg.norm(b)
    _, itr, _ = cg_oracle.cg(hm, b, np.zeros(n), 5000, 1e-10)
    assert abs(it - itr) <= max(2, itr // 50)  # same recurrence: same iteration count up to rounding


def test_cg_stops_at_max_iters_and_zero_rhs(cuda):
    hm = gen.laplacian_2d(60)
    A = mgb.matrix_from_host(hm, device="cuda")
    b = torch.from_numpy(gen.x_vector(hm["nrows"], seed=15)).cuda()
    x = torch.zeros_like(b)
    it, res = solvers.cg(A, b, x, max_iters=7, rtol=1e-14)
    assert it == 7 and res > 1e-14
    x = torch.zeros_like(b)
    it, res = solvers.cg(A, torch.zeros_like(b), x, max_iters=100, rtol=1e-10)
    assert it == 0 and res == 0.0 and torch.count_nonzero(x) == 0


def test_cg_rejects_non_spd_and_nonsquare(cuda):
    hm = gen.laplacian_2d(20)
    neg = dict(hm, values=-hm["values"])
    A = mgb.matrix_from_host(neg, device="cuda")
    b = torch.from_numpy(gen.x_vector(hm["nrows"], seed=16)).cuda()
    with pytest.raises(mgb.RuntimeException):
        solvers.cg(A, b, torch.zeros_like(b), max_iters=50, rtol=1e-10)
    B = mgb.matrix_from_host(gen.random_csr(30, 40, 0.1, seed=17), device="cuda")
    with pytest.raises(mgb.InvalidInputException):
        solvers.cg(B, torch.zeros(40, dtype=torch.float64, device="cuda"),
                   torch.zeros(40, dtype=torch.float64, device="cuda"))


def test_cg_f32(cuda):
    hm = gen.laplacian_2d(60, dtype=np.float32)
    n = hm["nrows"]
    b = gen.x_vector(n, seed=18, dtype=np.float32)
    A = mgb.matrix_from_host(hm, device="cuda")
    x = torch.zeros(n, dtype=torch.float32, device="cuda")
    it, res = solvers.cg(A, torch.from_numpy(b).cuda(), x, max_iters=2000, rtol=1e-5)
    assert 0 < it < 2000 and res <= 1e-5
    h64 = dict(hm, values=hm["values"].astype(np.float64))
    true = b.astype(np.float64) - O.OracleMatrix.from_host(h64).multiply(x.double().cpu().numpy())
    assert np.linalg.norm(true) <= 1e-4 * np.linalg.norm(b)
