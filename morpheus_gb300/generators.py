"""Seeded synthetic matrices for the benchmark workloads and tests.

All generators return host matrices (dicts of numpy arrays in the schema of
containers.matrix_to_host) in CSR with columns sorted ascending in each row,
so that every format derived from them round-trips bit-exactly through COO.
Randomness comes from numpy's PCG64 generator with an explicit seed.

Workloads (sizes of the reference configurations):
  laplacian_2d(256)            5-point Laplacian, N = 65,536, nnz = 326,656
  power_law(2_000_000)         lognormal(2.0, 1.2) row lengths clipped to
                               [1, 4096], uniform distinct columns, N(0,1)
                               values; nnz ~= 3.04e7
  stencil_27pt(160)            27-point stencil on 160^3, N = 4,096,000,
                               nnz = 109,215,352, centre 26 / neighbours -1
                               plus 1e-3 N(0,1) jitter
  add_offband(A, 0.01)         stencil plus 1% random entries off the band
  banded(N, diag_freq=5)       the reference's multiply test fixture shape:
                               diagonals 0 and +-5k (core/tests/Test_Multiply.hpp:161-186)
"""
from __future__ import annotations

import math

import numpy as np

CSR = 1


def _rng(seed):
    return np.random.Generator(np.random.PCG64(seed))


def _nonzero_normal(rng, n, dtype=np.float64):
    v = rng.standard_normal(n).astype(dtype)
    v[v == 0] = 1.0  # exact zeros would be dropped by DIA/HDC -> COO
    return v


def csr_from_sorted_keys(nrows: int, ncols: int, rows: np.ndarray, cols: np.ndarray,
                         vals: np.ndarray) -> dict:
    counts = np.bincount(rows, minlength=nrows).astype(np.int64)
    ro = np.zeros(nrows + 1, dtype=np.int64)
    np.cumsum(counts, out=ro[1:])
    return {"format": CSR, "nrows": int(nrows), "ncols": int(ncols), "nnz": int(rows.size),
            "row_offsets": ro.astype(np.int32), "column_indices": cols.astype(np.int32),
            "values": vals}


def laplacian_2d(n: int = 256, dtype=np.float64) -> dict:
    """5-point Laplacian on an n x n grid (diagonal 4, neighbours -1)."""
    N = n * n
    idx = np.arange(N, dtype=np.int64)
    i, j = idx // n, idx % n
    offs = [(-n, i > 0), (-1, j > 0), (0, np.ones(N, bool)), (1, j < n - 1), (n, i < n - 1)]
    rows, cols, vals = [], [], []
    for o, m in offs:
        r = idx[m]
        rows.append(r)
        cols.append(r + o)
        vals.append(np.full(r.size, 4.0 if o == 0 else -1.0, dtype=dtype))
    rows = np.concatenate(rows); cols = np.concatenate(cols); vals = np.concatenate(vals)
    order = np.lexsort((cols, rows))
    return csr_from_sorted_keys(N, N, rows[order], cols[order], vals[order])


def power_law(N: int = 2_000_000, mu: float = 2.0, sigma: float = 1.2, max_len: int = 4096,
              seed: int = 0, dtype=np.float64, ncols: int | None = None) -> dict:
    """Lognormal row lengths, distinct uniform columns per row (sorted)."""
    M = N if ncols is None else ncols
    rng = _rng(seed)
    lens = np.clip(np.rint(rng.lognormal(mu, sigma, N)), 1, min(max_len, M)).astype(np.int64)
    nnz = int(lens.sum())
    rows = np.repeat(np.arange(N, dtype=np.int64), lens)
    keys = rows * M + rng.integers(0, M, nnz, dtype=np.int64)
    keys.sort()
    while True:  # redraw duplicate (row, col) pairs until every row is distinct
        dup = np.flatnonzero(keys[1:] == keys[:-1]) + 1
        if dup.size == 0:
            break
        r = keys[dup] // M
        keys[dup] = r * M + rng.integers(0, M, dup.size, dtype=np.int64)
        keys.sort()
    rows = keys // M
    cols = keys - rows * M
    vals = _nonzero_normal(rng, nnz, dtype)
    return csr_from_sorted_keys(N, M, rows, cols, vals)


def stencil_offsets_27(n: int) -> list[tuple[int, int, int]]:
    return [(di, dj, dk) for di in (-1, 0, 1) for dj in (-1, 0, 1) for dk in (-1, 0, 1)]


def stencil_27pt(n: int = 160, jitter: float = 1e-3, seed: int = 0, dtype=np.float64) -> dict:
    """27-point stencil on an n^3 grid, rows in (i, j, k) lexicographic order."""
    N = n ** 3
    rng = _rng(seed)
    idx = np.arange(N, dtype=np.int64)
    i, j, k = idx // (n * n), (idx // n) % n, idx % n
    counts = np.zeros(N, dtype=np.int64)
    masks = []
    for di, dj, dk in stencil_offsets_27(n):
        m = ((i + di >= 0) & (i + di < n) & (j + dj >= 0) & (j + dj < n) &
             (k + dk >= 0) & (k + dk < n))
        masks.append(m)
        counts += m
    ro = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(counts, out=ro[1:])
    nnz = int(ro[-1])
    cols = np.empty(nnz, dtype=np.int32)
    vals = np.empty(nnz, dtype=dtype)
    pos = ro[:-1].copy()
    for (di, dj, dk), m in zip(stencil_offsets_27(n), masks):  # offsets ascending
        o = di * n * n + dj * n + dk
        r = idx[m]
        p = pos[m]
        cols[p] = (r + o).astype(np.int32)
        base = 26.0 if o == 0 else -1.0
        vals[p] = base + jitter * rng.standard_normal(r.size)
        pos[m] += 1
    return {"format": CSR, "nrows": N, "ncols": N, "nnz": nnz, "row_offsets": ro.astype(np.int32),
            "column_indices": cols, "values": vals}


def add_offband(A: dict, frac: float = 0.01, seed: int = 1) -> dict:
    """Add round(frac * nnz) random entries at unoccupied (r, c), N(0,1) values."""
    rng = _rng(seed)
    N, M = A["nrows"], A["ncols"]
    ro = A["row_offsets"].astype(np.int64)
    cols0 = A["column_indices"]
    extra = int(round(frac * A["nnz"]))
    new = np.unique(rng.integers(0, N, extra, dtype=np.int64) * M + rng.integers(0, M, extra, dtype=np.int64))
    nr = new // M
    nc = new - nr * M
    # rows are sorted by column: a vectorised binary search in each new
    # entry's row gives its merge position and whether (r, c) is occupied
    lo, hi = ro[nr], ro[nr + 1]
    while True:
        act = lo < hi
        if not act.any():
            break
        mid = (lo + hi) // 2
        go_right = act & (cols0[np.minimum(mid, max(A["nnz"] - 1, 0))] < nc)
        lo = np.where(go_right, mid + 1, lo)
        hi = np.where(act & ~go_right, mid, hi)
    hit = lo < ro[nr + 1]
    hit[hit] = cols0[lo[hit]] == nc[hit]
    keep = ~hit
    nr, nc, at = nr[keep], nc[keep], lo[keep]
    new_vals = _nonzero_normal(rng, nr.size, A["values"].dtype)
    ro_new = ro.copy()
    ro_new[1:] += np.cumsum(np.bincount(nr, minlength=N))
    # at is non-decreasing and np.insert keeps equal positions in the given order
    cols = np.insert(cols0, at, nc.astype(np.int32))
    vals = np.insert(A["values"], at, new_vals)
    return {"format": CSR, "nrows": int(N), "ncols": int(M), "nnz": int(cols.size),
            "row_offsets": ro_new.astype(np.int32), "column_indices": cols, "values": vals}


def banded(N: int, diag_freq: int = 5, seed: int = 0, dtype=np.float64) -> dict:
    """Diagonals 0 and +-k*diag_freq with values U[-2, 2] (the reference's
    DiagonalMatrixGenerator shape, core/tests/utils/MatrixGenerator.hpp:35-78)."""
    rng = _rng(seed)
    offs = [0] + [s * d for d in range(diag_freq, N, diag_freq) for s in (1, -1)]
    rows, cols = [], []
    for o in offs:
        r = np.arange(max(0, -o), min(N, N - o), dtype=np.int64)
        rows.append(r); cols.append(r + o)
    rows = np.concatenate(rows); cols = np.concatenate(cols)
    order = np.lexsort((cols, rows))
    rows, cols = rows[order], cols[order]
    vals = rng.uniform(-2.0, 2.0, rows.size).astype(dtype)
    vals[vals == 0] = 1.0
    return csr_from_sorted_keys(N, N, rows, cols, vals)


def random_csr(N: int, M: int, density: float, seed: int = 0, dtype=np.float64,
               empty_row_frac: float = 0.0) -> dict:
    """Uniform random sparsity (distinct sorted columns), optional empty rows."""
    rng = _rng(seed)
    nnz_target = max(0, int(round(density * N * M)))
    keys = np.unique(rng.integers(0, N, nnz_target, dtype=np.int64) * M +
                     rng.integers(0, M, nnz_target, dtype=np.int64))
    rows = keys // M
    if empty_row_frac > 0:
        dead = rng.random(N) < empty_row_frac
        keep = ~dead[rows]
        keys, rows = keys[keep], rows[keep]
    vals = _nonzero_normal(rng, keys.size, dtype)
    return csr_from_sorted_keys(N, M, rows, keys - rows * M, vals)


def random_lengths_csr(N: int, M: int, lengths: np.ndarray, seed: int = 0, dtype=np.float64) -> dict:
    """CSR with the given row lengths (clipped to M), distinct sorted uniform columns."""
    rng = _rng(seed)
    lens = np.minimum(np.asarray(lengths, dtype=np.int64), M)
    rows = np.repeat(np.arange(N, dtype=np.int64), lens)
    parts = []
    for r, L in zip(np.flatnonzero(lens), lens[lens > 0]):
        parts.append(np.sort(rng.choice(M, size=int(L), replace=False)))
    cols = np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)
    vals = _nonzero_normal(rng, rows.size, dtype)
    return csr_from_sorted_keys(N, M, rows, cols, vals)


def x_vector(n: int, seed: int = 0, dtype=np.float64) -> np.ndarray:
    """x uniform in [-1, 1] (the reference fills x from [-1, 1])."""
    return _rng(seed).uniform(-1.0, 1.0, n).astype(dtype)


def csr_to_dia_host(A: dict, alignment: int = 32) -> dict:
    """DIA of a CSR host matrix by the COO -> DIA rule (offsets = sorted set of
    c - r; entry (r, n) = value), vectorized for large stencils.  Equivalent to
    the reference convert for matrices without duplicate entries."""
    N, M = A["nrows"], A["ncols"]
    ro = A["row_offsets"].astype(np.int64)
    rows = np.repeat(np.arange(N, dtype=np.int64), np.diff(ro))
    d = A["column_indices"].astype(np.int64) - rows
    offs = np.unique(d)
    pitch = alignment * ((N + alignment - 1) // alignment)
    slot = np.searchsorted(offs, d)
    vals = np.zeros(pitch * offs.size, dtype=A["values"].dtype)
    vals[rows + pitch * slot] = A["values"]
    return {"format": 2, "nrows": N, "ncols": M, "nnz": A["nnz"], "ndiags": int(offs.size),
            "pitch": int(pitch), "alignment": alignment, "diagonal_offsets": offs.astype(np.int32),
            "values": vals}


def csr_to_coo_host(A: dict) -> dict:
    ro = A["row_offsets"].astype(np.int64)
    rows = np.repeat(np.arange(A["nrows"], dtype=np.int32), np.diff(ro))
    return {"format": 0, "nrows": A["nrows"], "ncols": A["ncols"], "nnz": A["nnz"],
            "row_indices": rows, "column_indices": A["column_indices"].copy(),
            "values": A["values"].copy()}


def csr_to_ell_host(A: dict, width: int | None = None, alignment: int = 32) -> dict:
    """ELL by the COO -> ELL placement rule (slots fill in order, padding
    (-1, 0)); width defaults to the longest row like the reference."""
    N = A["nrows"]
    ro = A["row_offsets"].astype(np.int64)
    lens = np.diff(ro)
    W = int(lens.max()) if width is None else int(width)
    if lens.size and lens.max() > W:
        raise ValueError("row longer than the ELL width")
    Wp = alignment * ((W + alignment - 1) // alignment)
    rows = np.repeat(np.arange(N, dtype=np.int64), lens)
    slot = np.arange(A["nnz"], dtype=np.int64) - np.repeat(ro[:-1], lens)
    ci = np.full(N * Wp, -1, dtype=np.int32)
    va = np.zeros(N * Wp, dtype=A["values"].dtype)
    ci[rows + N * slot] = A["column_indices"]
    va[rows + N * slot] = A["values"]
    return {"format": 3, "nrows": N, "ncols": A["ncols"], "nnz": A["nnz"], "entries_per_row": W,
            "width": Wp, "pitch": N, "alignment": alignment, "column_indices": ci, "values": va}


def csr_to_hyb_host(A: dict, width: int, alignment: int = 32) -> dict:
    """HYB by the COO -> HYB rule with ELL width `width`: the first `width`
    entries of each row go to ELL, the rest to COO in order."""
    N = A["nrows"]
    ro = A["row_offsets"].astype(np.int64)
    lens = np.diff(ro)
    rows = np.repeat(np.arange(N, dtype=np.int64), lens)
    slot = np.arange(A["nnz"], dtype=np.int64) - np.repeat(ro[:-1], lens)
    in_ell = slot < width
    ell_lens = np.minimum(lens, width)
    ell_ro = np.zeros(N + 1, dtype=np.int64)
    np.cumsum(ell_lens, out=ell_ro[1:])
    ell_csr = {"format": 1, "nrows": N, "ncols": A["ncols"], "nnz": int(in_ell.sum()),
               "row_offsets": ell_ro.astype(np.int32), "column_indices": A["column_indices"][in_ell],
               "values": A["values"][in_ell]}
    ell = csr_to_ell_host(ell_csr, width=width, alignment=alignment)
    coo = {"format": 0, "nrows": N, "ncols": A["ncols"], "nnz": int((~in_ell).sum()),
           "row_indices": rows[~in_ell].astype(np.int32),
           "column_indices": A["column_indices"][~in_ell].copy(), "values": A["values"][~in_ell].copy()}
    return {"format": 4, "nrows": N, "ncols": A["ncols"], "nnz": A["nnz"], "alignment": alignment,
            "ell": ell, "coo": coo}


def csr_to_hdc_host(A: dict, alignment: int = 32, ratio: float = 0.2) -> dict:
    """HDC by the COO -> HDC rule (diagonals with >= floor(ratio * N) entries
    to DIA, the rest to CSR in order); square matrices only."""
    N, M = A["nrows"], A["ncols"]
    assert N == M
    ro = A["row_offsets"].astype(np.int64)
    lens = np.diff(ro)
    rows = np.repeat(np.arange(N, dtype=np.int64), lens)
    d = A["column_indices"].astype(np.int64) - rows
    hist = np.bincount(d + N - 1, minlength=N + M - 1)
    min_elem = int(N * ratio)
    true_d = np.flatnonzero(hist >= min_elem) - (N - 1)
    is_dia = np.isin(d, true_d)
    dia_part = {"format": 1, "nrows": N, "ncols": M, "nnz": int(is_dia.sum()),
                "row_offsets": None, "column_indices": A["column_indices"][is_dia],
                "values": A["values"][is_dia]}
    counts = np.bincount(rows[is_dia], minlength=N)
    dro = np.zeros(N + 1, dtype=np.int64); np.cumsum(counts, out=dro[1:])
    dia_part["row_offsets"] = dro.astype(np.int32)
    dia = csr_to_dia_host(dia_part, alignment)
    # keep every true diagonal (even one without entries here) in sorted order
    if dia["ndiags"] != true_d.size:
        raise ValueError("unexpected diagonal set")
    ccounts = np.bincount(rows[~is_dia], minlength=N)
    cro = np.zeros(N + 1, dtype=np.int64); np.cumsum(ccounts, out=cro[1:])
    csr = {"format": 1, "nrows": N, "ncols": M, "nnz": int((~is_dia).sum()),
           "row_offsets": cro.astype(np.int32), "column_indices": A["column_indices"][~is_dia].copy(),
           "values": A["values"][~is_dia].copy()}
    return {"format": 5, "nrows": N, "ncols": M, "nnz": A["nnz"], "alignment": alignment,
            "dia": dia, "csr": csr}


def batched_csr(count: int = 4096, nmin: int = 64, nmax: int = 8192, lam_lo: float = 3.0, lam_hi: float = 40.0,
                seed: int = 0, dtype=np.float64) -> list[dict]:
    """Independent square CSR matrices: N log-uniform in [nmin, nmax], row
    lengths Poisson(lambda) with lambda ~ U[lam_lo, lam_hi] per matrix, distinct
    uniform columns (sorted), N(0,1) values."""
    rng = _rng(seed)
    out = []
    for _ in range(count):
        N = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)))))
        lam = rng.uniform(lam_lo, lam_hi)
        lens = np.minimum(rng.poisson(lam, N), N).astype(np.int64)
        rows = np.repeat(np.arange(N, dtype=np.int64), lens)
        keys = rows * N + rng.integers(0, N, rows.size, dtype=np.int64)
        keys.sort()
        while True:
            dup = np.flatnonzero(keys[1:] == keys[:-1]) + 1
            if dup.size == 0:
                break
            keys[dup] = (keys[dup] // N) * N + rng.integers(0, N, dup.size, dtype=np.int64)
            keys.sort()
        r = keys // N
        vals = _nonzero_normal(rng, keys.size, dtype)
        out.append(csr_from_sorted_keys(N, N, r, keys - r * N, vals))
    return out
