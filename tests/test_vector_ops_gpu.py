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
