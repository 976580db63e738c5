"""CPU checks of the benchmark's byte, FMA and roofline accounting.

The headline and per-config numbers divide algorithmic bytes (or FMAs) by
measured time, so the formulas themselves are pinned here against the
benchmark configurations' known sizes (27-point stencil 160^3: 109,215,352
nonzeros; DIA of it: 27 diagonals) and small hand-computed cases.
"""
import numpy as np
import pytest

import bench
from morpheus_gb300 import generators as gen


def test_csr_and_dia_bytes_of_the_stencil():
    n, nnz = 4_096_000, 109_215_352
    csr = {"format": 1, "nrows": n, "ncols": n, "nnz": nnz}
    dia = {"format": 2, "nrows": n, "ncols": n, "nnz": nnz, "ndiags": 27}
    # nnz (4 + 8) + 4 (N + 1) + 8 (N + M)
    assert bench.algorithmic_bytes(csr, 8) == 1_392_504_228
    # D N 8 + 4 D + 8 (N + M)
    assert bench.algorithmic_bytes(dia, 8) == 950_272_108
    assert bench.fma_count(dia) == 27 * n  # every slot, zeros included
    assert bench.fma_count(csr) == nnz


def test_ell_hyb_bytes_count_real_entries_only():
    A = gen.laplacian_2d(16)
    ell = gen.csr_to_ell_host(A)
    assert (ell["entries_per_row"], ell["width"]) == (5, 32)  # 27 padding slots per row, not counted
    n = A["nrows"]
    assert bench.algorithmic_bytes(ell, 8) == A["nnz"] * 12 + 2 * n * 8
    hyb = gen.csr_to_hyb_host(A, 3)
    e, c = hyb["ell"], hyb["coo"]
    assert bench.ell_stored(e) + c["nnz"] == A["nnz"]
    assert bench.algorithmic_bytes(hyb, 8) == bench.ell_stored(e) * 12 + c["nnz"] * 16 + 2 * n * 8


def test_roofline_names_the_largest_floor():
    hm = {"format": 2, "nrows": 4_096_000, "ncols": 4_096_000, "nnz": 109_215_352, "ndiags": 27}
    peaks = {"hbm_gbs": 6800.0, "fp64_fma_per_s": 5.3e11, "random_sectors_per_s": 3.1e11}
    r = bench.roofline(hm, 8, 200.0, peaks, "banded")
    nbytes = bench.algorithmic_bytes(hm, 8)
    assert r["achieved"] == pytest.approx(nbytes / 200e-6 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6800.0)
    assert r["floors_us"]["hbm"] == pytest.approx(nbytes / 6800e9 * 1e6)
    assert r["floors_us"]["fp64_pipe"] == pytest.approx(27 * 4_096_000 / 5.3e11 * 1e6)
    assert r["binding_unit"] == "fp64_pipe" and "l1tex_random_sectors" not in r["floors_us"]
    assert r["frac_of_binding_unit"] == pytest.approx(r["floors_us"]["fp64_pipe"] / 200.0)
    # scattered x adds the sector floor; FP32 has no FP64 floor
    csr = {"format": 1, "nrows": 2_000_000, "ncols": 2_000_000, "nnz": 30_000_000}
    r2 = bench.roofline(csr, 4, 150.0, peaks, "scattered")
    assert set(r2["floors_us"]) == {"hbm", "l1tex_random_sectors"}
    sectors = 30_000_000 + bench.stream_bytes(csr, 4) / 32.0
    assert r2["floors_us"]["l1tex_random_sectors"] == pytest.approx(sectors / 3.1e11 * 1e6)


def test_profile_traffic_reads_the_committed_summaries():
    got = bench.profile_traffic("c3_stencil27_160_dia_f64")
    assert got is not None
    value, source = got
    assert 0.9e9 < value < 1.1e9 and source.startswith("profiles/spmv_dia_stencil27_f64.md")
    assert bench.profile_traffic("no_such_workload") is None
    # every summary that names a workload carries a usable traffic figure or none
    for key in ("c3_stencil27_160_csr_f64", "c3_stencil27_160_csr_f32", "c3_stencil27_160_ell_f64",
                "c2_power_law_2e6_csr_f64", "vector_reduce_2^26_f64"):
        t = bench.profile_traffic(key)
        assert t is not None and t[0] > 0, key
    assert np.isfinite(bench.profile_traffic("c5_batched_4096_csr_f64")[0])
