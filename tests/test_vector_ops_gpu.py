"""GPU parity of dot / reduce / waxpby against the oracle and the reference's
known answers (core/tests/Test_Dot.hpp:74-87, Test_Reduce.hpp:74-81,
Test_WAXPBY.hpp:75-120)."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import rel_err
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [50, 5000, 50000])
@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
def test_dot_known_answer(cuda, n, dtype):
    x = torch.arange(1, n + 1, dtype=dtype, device="cuda")
    y = (n - torch.arange(n, device="cuda")).to(dtype)
    exact = sum((i + 1) * (n - i) for i in range(n))
    got = mgb.dot(n, x, y)
    if dtype == torch.float64:
        assert got == exact
    else:
        assert abs(got - exact) <= 4 * np.finfo(np.float32).eps * exact


@pytest.mark.parametrize("vsize,rsize", [(50, 50), (50, 25), (5000, 5000), (5000, 1000), (50000, 50000), (50000, 100)])
def test_reduce_known_answer(cuda, vsize, rsize):
    d = torch.arange(vsize, dtype=torch.float64, device="cuda") + 1.5
    exact = sum(i + 1.5 for i in range(rsize))
    assert mgb.reduce(d, rsize) == exact


@pytest.mark.parametrize("n", [1, 7, 1000, 1 << 20, (1 << 22) + 3])
def test_dot_reduce_random(cuda, n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    y = rng.standard_normal(n)
    xt, yt = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    assert rel_err(np.array([mgb.dot(n, xt, yt)]), np.array([O.dot(n, x, y)])) <= 1e-12 * max(1, np.sqrt(n) / 100)
    assert abs(mgb.dot(n, xt, xt) - O.dot(n, x, x)) <= 1e-12 * O.dot(n, x, x)
    exact = float(np.sum(np.abs(x)))
    assert abs(mgb.reduce(xt, n) - O.reduce(x, n)) <= 1e-12 * exact
    # misaligned views exercise the scalar path
    if n > 3:
        assert abs(mgb.dot(n - 1, xt[1:], yt[1:]) - O.dot(n - 1, x[1:].copy(), y[1:].copy())) <= 1e-11 * n


def test_dot_async_writes_device_scalar(cuda):
    x = torch.ones(1000, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    mgb.dot_async(1000, x, x, out)
    assert out.item() == 1000.0


@pytest.mark.parametrize("alpha,beta", [(2.15, -3.2), (1.0, -3.2), (2.15, 1.0)])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_waxpby(cuda, alpha, beta, dtype):
    rng = np.random.default_rng(0)
    for n in (50, 5000, 50000):
        x = rng.uniform(-5, 5, n).astype(dtype)
        y = rng.uniform(-2, 2, n).astype(dtype)
        w_ref = np.zeros(n, dtype)
        O.waxpby(n, dtype(alpha), x, dtype(beta), y, w_ref)
        w = torch.zeros(n, dtype=torch.from_numpy(x).dtype, device="cuda")
        mgb.waxpby(n, alpha, torch.from_numpy(x).cuda(), beta, torch.from_numpy(y).cuda(), w)
        tol = 1e-13 if dtype == np.float64 else 1e-5
        assert np.max(np.abs(w.cpu().numpy().astype(np.float64) - w_ref)) <= tol * 10


# FP64 reduce splits each large vector between FP64 adds and an exact
# fixed-point accumulation on the integer pipe; the split engages once every
# thread of the grid sees at least one 16-element step (a few million elements).
N_SPLIT = (1 << 22) + 3


def test_reduce_wide_exponent_range(cuda):
    import math
    rng = np.random.default_rng(11)
    x = rng.standard_normal(N_SPLIT) * np.exp2(rng.integers(-600, 600, N_SPLIT))
    got = mgb.reduce(torch.from_numpy(x).cuda(), N_SPLIT)
    exact = math.fsum(x)  # correctly rounded
    assert abs(got - exact) <= 1e-14 * float(np.sum(np.abs(x)))
    # exact cancellation: the result stays within the same bound of zero
    y = np.concatenate([x, -x])
    assert abs(mgb.reduce(torch.from_numpy(y).cuda(), y.size)) <= 1e-14 * float(np.sum(np.abs(y)))


@pytest.mark.parametrize("special", ["inf", "-inf", "nan", "inf-inf"])
def test_reduce_special_values_propagate(cuda, special):
    """Inf and NaN reach the result from either share of the split (the
    positions below fall in both, as in the Serial sum)."""
    rng = np.random.default_rng(12)
    base = torch.from_numpy(rng.uniform(-1, 1, N_SPLIT)).cuda()
    for pos in rng.integers(0, N_SPLIT, 24):
        x = base.clone()
        if special == "inf-inf":
            x[int(pos)] = np.inf
            x[(int(pos) + 7) % N_SPLIT] = -np.inf
        else:
            x[int(pos)] = float(special)
        got = mgb.reduce(x, N_SPLIT)
        if special in ("nan", "inf-inf"):
            assert np.isnan(got), (special, int(pos))
        else:
            assert got == float(special), (special, int(pos), got)
