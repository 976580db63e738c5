"""GPU: batched persistent CSR SpMV (every configuration, autotuner, CUDA-graph
replay) against the oracle's Serial multiply of each matrix."""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import rel_err
from morpheus_gb300 import batched
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def make_batch(count, seed, dtype=np.float64, nmax=3000):
    mats = gen.batched_csr(count, nmin=1, nmax=nmax, lam_lo=0.5, lam_hi=60, seed=seed, dtype=dtype)
    # a few awkward items: empty matrix rows, one long row, 1x1
    mats.append(gen.random_lengths_csr(50, 50, np.zeros(50, dtype=np.int64), seed=1, dtype=dtype))
    lens = np.ones(40, dtype=np.int64); lens[3] = 9000
    mats.append(gen.random_lengths_csr(40, 20000, lens, seed=2, dtype=dtype))
    mats.append(gen.random_lengths_csr(1, 1, np.array([1]), seed=3, dtype=dtype))
    tdt = torch.float64 if dtype == np.float64 else torch.float32
    dev = [mgb.matrix_from_host(m) for m in mats]
    xs = [torch.from_numpy(gen.x_vector(m["ncols"], seed=i, dtype=dtype)).cuda() for i, m in enumerate(mats)]
    ys = [torch.from_numpy(gen.x_vector(m["nrows"], seed=i + 1, dtype=dtype)).cuda() for i, m in enumerate(mats)]
    return mats, dev, xs, ys, tdt


def check(mats, xs, ys, y0s, init, tol):
    for m, x, y, y0 in zip(mats, xs, ys, y0s):
        ref = O.OracleMatrix.from_host(m).multiply(x.cpu().numpy(), y0.copy(), init=init)
        assert rel_err(y.cpu().numpy(), ref) <= tol


@pytest.mark.parametrize("config", range(11))
def test_every_config(cuda, config):
    mats, dev, xs, ys, _ = make_batch(60, seed=config)
    y0s = [y.cpu().numpy() for y in ys]
    b = batched.CsrBatch(dev, xs, ys)
    b.plan(config)
    b.multiply(init=False)
    torch.cuda.synchronize()
    assert b.planned_ok()
    check(mats, xs, ys, y0s, False, 1e-12)
    b.multiply(init=True)
    torch.cuda.synchronize()
    check(mats, xs, ys, y0s, True, 1e-12)


def test_autotune_and_graph_replay(cuda):
    mats, dev, xs, ys, _ = make_batch(120, seed=11)
    b = batched.CsrBatch(dev, xs, ys)
    best, times = b.autotune(reps=2, use_cache=False)
    assert 0 <= best < batched.num_configs() and len(times) == batched.num_configs()
    assert min(times) == times[best]
    g = b.capture_graph(init=True)
    for y in ys:
        y.fill_(123.0)
    g.replay()
    torch.cuda.synchronize()
    y0s = [y.cpu().numpy() for y in ys]
    check(mats, xs, ys, y0s, True, 1e-12)
    for x in xs:  # the graph reads x in place
        x.mul_(-2.0)
    g.replay()
    torch.cuda.synchronize()
    check(mats, xs, ys, y0s, True, 1e-12)


@pytest.mark.parametrize("config", [6, 7, 10])
def test_shared_x_configs_f32_and_wide_x(cuda, config):
    """Matrix-per-CTA configurations keep x in shared memory up to 64 KB;
    wider x (here 20,000 and 40,000 columns) is read from global memory."""
    mats, dev, xs, ys, _ = make_batch(40, seed=20 + config, dtype=np.float32)
    extra = gen.random_lengths_csr(300, 40000, np.full(300, 25), seed=9, dtype=np.float32)
    mats.append(extra)
    dev.append(mgb.matrix_from_host(extra))
    xs.append(torch.from_numpy(gen.x_vector(40000, seed=4, dtype=np.float32)).cuda())
    ys.append(torch.zeros(300, dtype=torch.float32, device="cuda"))
    b = batched.CsrBatch(dev, xs, ys)
    b.plan(config)
    b.multiply(init=True)
    torch.cuda.synchronize()
    assert b.planned_ok()
    for m, x, y in zip(mats, xs, ys):
        ref = O.OracleMatrix.from_host({k: (v.astype(np.float64) if isinstance(v, np.ndarray) and v.dtype.kind == "f"
                                            else v) for k, v in m.items()}).multiply(x.double().cpu().numpy())
        scale = O.OracleMatrix.from_host({k: (np.abs(v).astype(np.float64) if isinstance(v, np.ndarray)
                                              and v.dtype.kind == "f" else v) for k, v in m.items()}).multiply(
            np.abs(x.double().cpu().numpy()))
        err = np.linalg.norm(y.double().cpu().numpy() - ref) / max(np.linalg.norm(scale), 1e-300)
        assert err <= 1e-5


@pytest.mark.parametrize("config", [6, 7, 10])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_shared_x_configs_unaligned_x(cuda, config, dtype):
    """x vectors that start one element past a 16-byte boundary are copied
    into shared memory element by element; the result is unchanged."""
    mats, dev, xs, ys, _ = make_batch(50, seed=40 + config, dtype=dtype)
    xs = [torch.cat([torch.zeros(1, dtype=x.dtype, device=x.device), x])[1:] for x in xs]
    assert all(x.data_ptr() % 16 != 0 for x in xs)
    y0s = [y.cpu().numpy() for y in ys]
    b = batched.CsrBatch(dev, xs, ys)
    b.plan(config)
    b.multiply(init=False)
    torch.cuda.synchronize()
    assert b.planned_ok()
    for m, x, y, y0 in zip(mats, xs, ys, y0s):
        m64 = dict(m, values=m["values"].astype(np.float64))
        x64 = x.cpu().numpy().astype(np.float64)
        ref = O.OracleMatrix.from_host(m64).multiply(x64, y0.astype(np.float64).copy(), init=False)
        if dtype == np.float64:
            assert rel_err(y.cpu().numpy(), ref) <= 1e-12
        else:
            scale = O.OracleMatrix.from_host(dict(m64, values=np.abs(m64["values"]))).multiply(
                np.abs(x64), np.abs(y0.astype(np.float64)), init=False)
            err = np.linalg.norm(y.double().cpu().numpy() - ref) / max(np.linalg.norm(scale), 1e-300)
            assert err <= 1e-5


def test_config_mismatch_is_a_noop(cuda):
    mats, dev, xs, ys, _ = make_batch(10, seed=5)
    b = batched.CsrBatch(dev, xs, ys)
    b.plan(1)
    before = [y.clone() for y in ys]
    b.config = 6  # launch a config the workspace was not planned for
    b.multiply()
    torch.cuda.synchronize()
    assert not b.planned_ok()
    assert all(torch.equal(a, c) for a, c in zip(before, ys))


def test_float32(cuda):
    mats, dev, xs, ys, _ = make_batch(40, seed=7, dtype=np.float32)
    b = batched.CsrBatch(dev, xs, ys)
    b.autotune(reps=1, use_cache=False)
    b.multiply()
    torch.cuda.synchronize()
    for m, x, y in zip(mats, xs, ys):
        m64 = dict(m, values=m["values"].astype(np.float64))
        ref = O.OracleMatrix.from_host(m64).multiply(x.cpu().numpy().astype(np.float64))
        scale = O.OracleMatrix.from_host(dict(m64, values=np.abs(m64["values"]))).multiply(
            np.abs(x.cpu().numpy().astype(np.float64)))
        err = np.linalg.norm(y.cpu().numpy() - ref) / max(np.linalg.norm(scale), 1e-300)
        assert err <= 1e-5
