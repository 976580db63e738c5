"""GPU parity at the full sizes of the benchmark configurations.

    C1  5-point Laplacian 256^2 (N = 65,536): CSR, COO, DIA
    C2  power-law N = 2,000,000 (lognormal(2, 1.2) rows, ~3.04e7 nnz):
        CSR, COO, HYB with the ELL width at the 90th-percentile row length,
        and the reference's own HYB rule (width = nnz / N); FP64 and FP32
    C3  27-point stencil 160^3 (N = 4,096,000, 109,215,352 nnz): DIA, CSR,
        FP64 and FP32, and HDC of the stencil plus 1 % random off-band entries
    C5  4,096 CSR matrices (N log-uniform 64..8192, Poisson row lengths):
        every batched configuration, every matrix checked

Every conversion the GPU makes is compared bit for bit with the oracle's
Serial convert of the same matrix (the reference's Serial convert restated,
impl/<Fmt>/Serial/Morpheus_Convert_Impl.hpp), and every round trip back to
CSR must reproduce the generated matrix exactly.  y is compared with the
oracle's multiply of the same container (OpenMP restatement, which sums each
row in the Serial order): normwise relative error <= 1e-12 in FP64; in FP32
<= 1e-5 against the FP64 oracle relative to || |A| |x| + |y0| ||, and
<= 1e-4 against the FP32 oracle on the same scale.  Matrices are built once
per module.
"""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import assert_same_matrix, rel_err
from morpheus_gb300 import batched
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu

THREADS = None


def _threads():
    global THREADS
    if THREADS is None:
        THREADS = O.max_threads()
    return THREADS


def _map_values(hm, fn):
    out = {}
    for k, v in hm.items():
        if isinstance(v, dict):
            out[k] = _map_values(v, fn)
        elif isinstance(v, np.ndarray) and v.dtype.kind == "f":
            out[k] = fn(v)
        else:
            out[k] = v
    return out


def check_multiply(hm, seed=0):
    """Multiply the host container hm on the GPU (init and accumulate) and
    compare with the oracle's multiply of the same container."""
    dtype = O._values_dtype(hm)
    n, m = hm["nrows"], hm["ncols"]
    x = gen.x_vector(m, seed=seed, dtype=dtype)
    y0 = gen.x_vector(n, seed=seed + 1, dtype=dtype)
    A = mgb.matrix_from_host(hm, device="cuda")
    xt = torch.from_numpy(x).cuda()
    om = O.OracleMatrix.from_host(hm)
    if dtype == np.float32:
        hm64 = _map_values(hm, lambda v: v.astype(np.float64))
        om64 = O.OracleMatrix.from_host(hm64)
        oabs = O.OracleMatrix.from_host(_map_values(hm64, np.abs))
    errs = []
    for init in (True, False):
        yt = torch.from_numpy(y0.copy()).cuda()
        mgb.multiply(A, xt, yt, init=init)
        y = yt.cpu().numpy()
        ref = om.multiply(x, y0.copy(), init=init, threads=_threads())
        if dtype == np.float64:
            err = rel_err(y, ref)
            assert err <= 1e-12, f"format {hm['format']} init={init}: rel err {err:.3e}"
        else:
            ref64 = om64.multiply(x.astype(np.float64), y0.astype(np.float64), init=init, threads=_threads())
            scale = np.linalg.norm(oabs.multiply(np.abs(x.astype(np.float64)), np.abs(y0.astype(np.float64)),
                                                 init=init, threads=_threads()))
            err = float(np.linalg.norm(y.astype(np.float64) - ref64) / scale)
            assert err <= 1e-5, f"format {hm['format']} init={init}: FP32 error vs FP64 oracle {err:.3e}"
            e32 = float(np.linalg.norm(y.astype(np.float64) - ref.astype(np.float64)) / scale)
            assert e32 <= 1e-4, f"format {hm['format']} init={init}: FP32 error vs FP32 oracle {e32:.3e}"
        errs.append(err)
    return max(errs)


def gpu_to_coo(hm):
    return mgb.to_coo(mgb.matrix_from_host(hm, device="cuda"))


def gpu_from_coo(coo_dev, fmt, hyb_width=0):
    return mgb.from_coo(coo_dev, fmt, hyb_width=hyb_width)


def assert_round_trip_to_csr(dev_matrix, csr_hm):
    back = mgb.from_coo(mgb.to_coo(dev_matrix), mgb.CSR_FORMAT)
    assert_same_matrix(mgb.matrix_to_host(back), csr_hm, "round trip:")


# --------------------------------------------------------------------------
# C1: 5-point Laplacian 256^2
# --------------------------------------------------------------------------

def test_c1_laplacian_256(cuda):
    A = gen.laplacian_2d(256)
    assert (A["nrows"], A["nnz"]) == (65_536, 326_656)
    coo = gpu_to_coo(A)
    ocoo = O.OracleMatrix.from_host(A).convert(O.COO)
    assert_same_matrix(mgb.matrix_to_host(coo), ocoo.to_host(), "COO:")
    dia = gpu_from_coo(coo, mgb.DIA_FORMAT)
    odia = ocoo.convert(O.DIA).to_host()
    assert odia["ndiags"] == 5
    assert_same_matrix(mgb.matrix_to_host(dia), odia, "DIA:")
    assert_round_trip_to_csr(dia, A)
    for hm in (A, ocoo.to_host(), odia):
        check_multiply(hm, seed=0)


# --------------------------------------------------------------------------
# C2: power-law N = 2e6
# --------------------------------------------------------------------------

@pytest.fixture(scope="module")
def c2():
    A = gen.power_law(2_000_000, seed=0)
    p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
    ocoo = O.OracleMatrix.from_host(A).convert(O.COO)
    return {"csr": A, "p90": p90, "coo": ocoo.to_host(), "hyb_p90": ocoo.coo_to_hyb(p90).to_host(),
            "hyb_ref": ocoo.convert(O.HYB).to_host()}


def test_c2_conversions_bit_exact(cuda, c2):
    A = c2["csr"]
    assert A["nrows"] == 2_000_000 and 2.9e7 < A["nnz"] < 3.2e7
    coo = gpu_to_coo(A)
    assert_same_matrix(mgb.matrix_to_host(coo), c2["coo"], "COO:")
    hyb = gpu_from_coo(coo, mgb.HYB_FORMAT, hyb_width=c2["p90"])
    assert_same_matrix(mgb.matrix_to_host(hyb), c2["hyb_p90"], "HYB(p90):")
    assert_round_trip_to_csr(hyb, A)
    hyb_ref = gpu_from_coo(coo, mgb.HYB_FORMAT)  # the reference's width rule max(1, nnz / N)
    assert c2["hyb_ref"]["ell"]["entries_per_row"] == max(1, A["nnz"] // A["nrows"])
    assert_same_matrix(mgb.matrix_to_host(hyb_ref), c2["hyb_ref"], "HYB(ref):")
    assert_round_trip_to_csr(hyb_ref, A)
    # ELL at the longest row exceeds the fill tolerance, in the reference too
    with pytest.raises(O.OracleError):
        O.OracleMatrix.from_host(c2["coo"]).convert(O.ELL)
    with pytest.raises(mgb.FormatConversionException):
        gpu_from_coo(coo, mgb.ELL_FORMAT)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("fmt", ["csr", "coo", "hyb_p90"])
def test_c2_multiply(cuda, c2, fmt, dtype):
    hm = c2[fmt] if dtype == np.float64 else _map_values(c2[fmt], lambda v: v.astype(np.float32))
    check_multiply(hm, seed=0)


# --------------------------------------------------------------------------
# C3: 27-point stencil 160^3
# --------------------------------------------------------------------------

@pytest.fixture(scope="module")
def c3():
    S = gen.stencil_27pt(160, seed=0)
    ocoo = O.OracleMatrix.from_host(S).convert(O.COO)
    odia = ocoo.convert(O.DIA)
    return {"csr": S, "dia": odia.to_host()}


@pytest.fixture(scope="module")
def c3_offband(c3):
    H = gen.add_offband(c3["csr"], 0.01, seed=1)
    ohdc = O.OracleMatrix.from_host(H).convert(O.COO).convert(O.HDC)
    return {"csr": H, "hdc": ohdc.to_host()}


def test_c3_dia_bit_exact_and_round_trip(cuda, c3):
    S = c3["csr"]
    assert (S["nrows"], S["nnz"]) == (4_096_000, 109_215_352)
    dia = gpu_from_coo(gpu_to_coo(S), mgb.DIA_FORMAT)
    assert c3["dia"]["ndiags"] == 27
    assert_same_matrix(mgb.matrix_to_host(dia), c3["dia"], "DIA:")
    assert_round_trip_to_csr(dia, S)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("fmt", ["dia", "csr"])
def test_c3_multiply(cuda, c3, fmt, dtype):
    hm = c3[fmt] if dtype == np.float64 else _map_values(c3[fmt], lambda v: v.astype(np.float32))
    check_multiply(hm, seed=0)


def test_c3_hdc_offband(cuda, c3_offband):
    H = c3_offband["csr"]
    extra = H["nnz"] - 109_215_352
    assert 1.0e6 < extra < 1.1e6  # ~1 % random off-band entries
    hdc = gpu_from_coo(gpu_to_coo(H), mgb.HDC_FORMAT)
    want = c3_offband["hdc"]
    assert want["dia"]["ndiags"] == 27 and want["csr"]["nnz"] > 1.0e6
    assert_same_matrix(mgb.matrix_to_host(hdc), want, "HDC:")
    assert_round_trip_to_csr(hdc, H)
    check_multiply(want, seed=0)


# --------------------------------------------------------------------------
# C5: 4,096 matrices in one batched launch
# --------------------------------------------------------------------------

def test_c5_full_batch_every_config(cuda):
    mats = gen.batched_csr(4096, seed=0)
    assert len(mats) == 4096
    sizes = [m["nrows"] for m in mats]
    assert min(sizes) >= 64 and max(sizes) <= 8192
    xs_np = [gen.x_vector(m["ncols"], seed=1 + i) for i, m in enumerate(mats)]
    refs = np.concatenate([O.OracleMatrix.from_host(m).multiply(x) for m, x in zip(mats, xs_np)])
    bounds = np.cumsum([0] + sizes)
    dev = [mgb.matrix_from_host(m) for m in mats]
    xs = [torch.from_numpy(x).cuda() for x in xs_np]
    ys = [torch.zeros(m["nrows"], dtype=torch.float64, device="cuda") for m in mats]
    b = batched.CsrBatch(dev, xs, ys)
    for config in range(batched.num_configs()):
        for y in ys:
            y.fill_(7.0)
        b.plan(config)
        b.multiply(init=True)
        torch.cuda.synchronize()
        assert b.planned_ok(), f"config {config}"
        got = torch.cat(ys).cpu().numpy()
        for i in range(len(mats)):  # every matrix
            lo, hi = bounds[i], bounds[i + 1]
            e = rel_err(got[lo:hi], refs[lo:hi])
            assert e <= 1e-12, f"config {config}, matrix {i} (N={sizes[i]}): rel err {e:.3e}"
    best, _ = b.autotune(reps=2, use_cache=False)
    g = b.capture_graph(init=True)
    for y in ys:
        y.fill_(-3.0)
    g.replay()
    torch.cuda.synchronize()
    got = torch.cat(ys).cpu().numpy()
    worst = max(rel_err(got[bounds[i]:bounds[i + 1]], refs[bounds[i]:bounds[i + 1]]) for i in range(len(mats)))
    assert worst <= 1e-12, f"graph replay of config {best}: worst rel err {worst:.3e}"
