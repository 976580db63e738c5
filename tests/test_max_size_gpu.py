"""Maximum sizes: a CSR matrix whose nnz sits just below the int32 limit the
kernels accept (2^31 - 4096), built on the device: every CSR kernel and the
COO kernel give the exact window sums (values 1, column j of row r is
(r + j) mod ncols), checked against an FP64 prefix-sum computation."""
import pytest
import torch

import morpheus_gb300 as mgb

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

L = 1000                       # entries per row
N = (2 ** 31 - 4096) // L - 1  # rows: nnz just under the limit
M = 3_000_001                  # columns


@pytest.fixture(scope="module")
def big(cuda):
    if torch.cuda.get_device_properties(0).total_memory < 80 * 2**30:
        pytest.skip("needs a GPU with >= 80 GB")
    dev = torch.device("cuda")
    nnz = N * L
    ro = (torch.arange(N + 1, device=dev, dtype=torch.int64) * L).to(torch.int32)
    r = torch.arange(N, device=dev, dtype=torch.int64)
    ci = torch.empty(nnz, dtype=torch.int32, device=dev)
    step = 1 << 14  # rows per piece, to bound the int64 temporaries
    j = torch.arange(L, device=dev, dtype=torch.int64)
    for a in range(0, N, step):
        b = min(N, a + step)
        ci[a * L:b * L] = ((r[a:b, None] + j[None, :]) % M).reshape(-1).to(torch.int32)
    va = torch.ones(nnz, dtype=torch.float64, device=dev)
    x = torch.rand(M, dtype=torch.float64, device=dev, generator=torch.Generator(device=dev).manual_seed(5)) - 0.5
    # y_ref[r] = sum_{j<L} x[(r + j) mod M] from an FP64 prefix sum of x repeated
    xx = torch.cat([x, x[:L]])
    cs = torch.cat([torch.zeros(1, dtype=torch.float64, device=dev), torch.cumsum(xx, 0)])
    rm = r % M
    y_ref = cs[rm + L] - cs[rm]
    A = mgb.CsrMatrix(N, M, nnz, ro, ci, va)
    yield A, x, y_ref
    del A, ci, va


@pytest.mark.parametrize("variant", [mgb.CSR_SEGMENTS, mgb.CSR_ROWS, mgb.CSR_SPLIT, mgb.CSR_ROWS_GATHER])
def test_csr_at_int32_limit(big, variant):
    A, x, y_ref = big
    A._variant = variant
    y = torch.empty(N, dtype=torch.float64, device="cuda")
    mgb.multiply(A, x, y)
    torch.cuda.synchronize()
    err = (torch.linalg.norm(y - y_ref) / torch.linalg.norm(y_ref)).item()
    assert err <= 1e-12, err


def test_chooser_and_coo_at_int32_limit(big):
    A, x, y_ref = big
    A.forget_kernel_variant()
    assert A.kernel_variant() == mgb.CSR_SPLIT  # rows of 1000 entries on average
    coo = mgb.to_coo(A)
    y = torch.empty(N, dtype=torch.float64, device="cuda")
    mgb.multiply(coo, x, y)
    torch.cuda.synchronize()
    err = (torch.linalg.norm(y - y_ref) / torch.linalg.norm(y_ref)).item()
    assert err <= 1e-12, err
