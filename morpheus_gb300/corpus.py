"""Synthetic training/evaluation corpus for the learned format selector.

Families (each plus 0-5 % random off-pattern entries, exactly 0 % for a
quarter of the matrices): banded (bandwidth
1-64), block-diagonal (block 4-256), uniform random, lognormal-row power law,
2-D (5/9-point) and 3-D (7/27-point) stencils; N log-uniform in
[1e4, 4e6].  Matrices are generated on the GPU (torch ops are used here only
to produce inputs) with at most NNZ_CAP = 120,000,000 entries (a 27-point
stencil on 160^3 has 109 M): without a cap the uniform-density family alone
would reach 1.4e10 entries.  A family's parameters are narrowed where the cap
binds; over the 2,000 training and 400 held-out seeds that is 185 matrices
(71 block-diagonal, 62 uniform, 51 banded, 1 lognormal).
Labels are measured: every format the reference's fill-tolerance rule
admits is built with the GPU conversions and timed with CUDA events; a
format the conversion refuses gets an infinite time.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .analytics import features
from .containers import COO_FORMAT, CSR_FORMAT, CsrMatrix
from .convert import from_coo, to_coo
from .exceptions import MorpheusException

NNZ_CAP = 120_000_000
FAMILIES = ["banded", "block", "uniform", "lognormal", "stencil2d", "stencil3d"]


def _csr_from_keys(keys: torch.Tensor, N: int, M: int, g: torch.Generator) -> CsrMatrix:
    keys = torch.unique(keys)
    rows = torch.div(keys, M, rounding_mode="floor")
    cols = (keys - rows * M).to(torch.int32)
    counts = torch.bincount(rows, minlength=N)
    ro = torch.zeros(N + 1, dtype=torch.int64, device=keys.device)
    ro[1:] = torch.cumsum(counts, 0)
    vals = torch.randn(keys.numel(), generator=g, device=keys.device, dtype=torch.float64)
    vals[vals == 0] = 1.0
    return CsrMatrix(N, M, keys.numel(), ro.to(torch.int32), cols, vals, torch.float64, keys.device)


def _offsets_keys(N: int, offsets, dev) -> torch.Tensor:
    r = torch.arange(N, device=dev, dtype=torch.int64)
    parts = []
    for o in offsets:
        c = r + o
        m = (c >= 0) & (c < N)
        parts.append(r[m] * N + c[m])
    return torch.cat(parts)


def generate(seed: int, device="cuda") -> tuple[CsrMatrix, dict]:
    """One corpus matrix (square, FP64) and its description."""
    rng = np.random.default_rng(seed)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    fam = FAMILIES[int(rng.integers(len(FAMILIES)))]
    N = int(round(math.exp(rng.uniform(math.log(1e4), math.log(4e6)))))
    dev = torch.device(device)
    desc = {"family": fam, "seed": seed}
    cap = int(NNZ_CAP / 1.06)  # room for the off-pattern entries
    if fam == "banded":
        bw = int(rng.integers(1, 65))
        bw = max(1, min(bw, (cap // N - 1) // 2))
        N = min(N, cap // (2 * bw + 1))
        keys = _offsets_keys(N, range(-bw, bw + 1), dev)
        desc["bandwidth"] = bw
    elif fam == "block":
        b = int(rng.integers(4, 257))
        b = max(1, min(b, cap // N))
        N = min(N, cap // b)
        nb = (N + b - 1) // b
        i = torch.arange(b, device=dev, dtype=torch.int64)
        base = torch.arange(nb, device=dev, dtype=torch.int64) * b
        rr = (base[:, None, None] + i[None, :, None]).expand(nb, b, b)
        cc = (base[:, None, None] + i[None, None, :]).expand(nb, b, b)
        m = (rr < N) & (cc < N)
        keys = (rr[m] * N + cc[m])
        desc["block"] = b
    elif fam == "uniform":
        dens = math.exp(rng.uniform(math.log(1e-6), math.log(1e-3)))
        nnz = int(min(cap, max(N, dens * N * N)))
        keys = torch.randint(0, N * N, (nnz,), generator=g, device=dev, dtype=torch.int64)
        desc["density"] = nnz / (N * N)
    elif fam == "lognormal":
        mu, sigma = rng.uniform(0.5, 3.0), rng.uniform(0.5, 1.5)
        lens = np.clip(np.rint(rng.lognormal(mu, sigma, N)), 1, 4096).astype(np.int64)
        N = min(N, cap)
        lens = lens[:N]
        if lens.sum() > cap:  # shrink the part above one entry per row
            extra = lens - 1
            lens = 1 + (extra * ((cap - N) / max(1, int(extra.sum())))).astype(np.int64)
        lt = torch.from_numpy(lens).to(dev)
        rows = torch.repeat_interleave(torch.arange(N, device=dev, dtype=torch.int64), lt)
        keys = rows * N + torch.randint(0, N, (rows.numel(),), generator=g, device=dev, dtype=torch.int64)
        desc.update(mu=mu, sigma=sigma)
    elif fam == "stencil2d":
        n = max(2, int(round(math.sqrt(N))))
        pts = 9 if rng.random() < 0.5 else 5
        n = min(n, int(math.sqrt(cap / pts)))
        N = n * n
        offs = [(a, b) for a in (-1, 0, 1) for b in (-1, 0, 1) if pts == 9 or abs(a) + abs(b) <= 1]
        r = torch.arange(N, device=dev, dtype=torch.int64)
        i, j = r // n, r % n
        parts = []
        for a, b in offs:
            m = (i + a >= 0) & (i + a < n) & (j + b >= 0) & (j + b < n)
            parts.append(r[m] * N + (r[m] + a * n + b))
        keys = torch.cat(parts)
        desc["points"] = pts
    else:
        n = max(2, int(round(N ** (1 / 3))))
        pts = 27 if rng.random() < 0.5 else 7
        if n ** 3 * pts > cap:
            n = int((cap / pts) ** (1 / 3))
        N = n ** 3
        offs = [(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)
                if pts == 27 or abs(a) + abs(b) + abs(c) <= 1]
        r = torch.arange(N, device=dev, dtype=torch.int64)
        i, j, k = r // (n * n), (r // n) % n, r % n
        parts = []
        for a, b, c in offs:
            m = (i + a >= 0) & (i + a < n) & (j + b >= 0) & (j + b < n) & (k + c >= 0) & (k + c < n)
            parts.append(r[m] * N + (r[m] + a * n * n + b * n + c))
        keys = torch.cat(parts)
        desc["points"] = pts
    # a quarter of the matrices keep their pure pattern (0 % off-pattern
    # entries): only those can be DIA matrices, since a few scattered entries
    # add a diagonal each and the DIA fill test then refuses the format
    extra = 0.0 if rng.random() < 0.25 else rng.uniform(0.0, 0.05)
    ne = int(extra * keys.numel())
    if ne:
        keys = torch.cat([keys, torch.randint(0, N * N, (ne,), generator=g, device=dev, dtype=torch.int64)])
    desc.update(nrows=N, extra_frac=extra)
    A = _csr_from_keys(keys, N, N, g)
    desc["nnz"] = A.nnnz()
    return A, desc


def time_spmv(M, x: torch.Tensor, y: torch.Tensor, reps: int = 10, warmup: int = 2, replays: int = 3) -> float:
    """Device time (ms) of one multiply: `reps` calls captured in one CUDA
    graph, replayed `replays` times between CUDA events, so small matrices
    are timed on the GPU rather than by the host's per-call overhead."""
    from .algorithms import multiply
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):  # also caches the CSR kernel choice outside the capture
            multiply(M, x, y)
    torch.cuda.current_stream().wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        for _ in range(reps):
            multiply(M, x, y)
    g.replay()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(replays):
        g.replay()
    e1.record()
    torch.cuda.synchronize()
    del g
    return e0.elapsed_time(e1) / (reps * replays)


def measure(A: CsrMatrix, reps: int = 10) -> np.ndarray:
    """SpMV time (ms) of every format; inf where the conversion is refused."""
    times = np.full(6, np.inf)
    x = torch.rand(A.ncols(), dtype=A.dtype, device=A.device) * 2 - 1
    y = torch.zeros(A.nrows(), dtype=A.dtype, device=A.device)
    coo = to_coo(A)
    times[CSR_FORMAT] = time_spmv(A, x, y, reps)
    times[COO_FORMAT] = time_spmv(coo, x, y, reps)
    for f in (2, 3, 4, 5):
        try:
            M = from_coo(coo, f)
        except MorpheusException:
            continue
        times[f] = time_spmv(M, x, y, reps)
        del M
    return times


def build(n: int, seed0: int, reps: int = 10, log=None) -> dict:
    """n corpus matrices: features, feasibility, per-format times, labels."""
    X = np.zeros((n, 12), np.float32)
    F = np.zeros((n, 6), np.uint8)
    T = np.zeros((n, 6))
    descs = []
    for i in range(n):
        A, d = generate(seed0 + i)
        X[i], F[i] = features(A)
        T[i] = measure(A, reps)
        F[i] &= np.isfinite(T[i]).astype(np.uint8)
        descs.append(d)
        if log and (i + 1) % 100 == 0:
            log(f"corpus {i + 1}/{n}")
        del A
    return {"X": X, "feasible": F, "times": T, "labels": np.argmin(T, axis=1).astype(np.int32), "desc": descs}
