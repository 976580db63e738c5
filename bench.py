"""SpMV throughput benchmark (GB/s of algorithmic bytes, % of HBM peak).

Default workload: FP64 CSR SpMV on the power-law matrix (N = 2,000,000,
lognormal(2.0, 1.2) row lengths clipped to [1, 4096], uniform distinct
columns, N(0,1) values, int32 indices; seeded synthetic data).  One step = one
y = A*x over the whole matrix.  The 0.4 GB working set is larger than L2, so no
flush is needed between steps.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                    [--workload power_law|stencil27|laplacian|uniform|batched|cg]
                    [--format csr|coo|dia|ell|hyb|hdc] [--dtype f64|f32] [--size S]
                    [--csr-kernel auto|segments|rows|gather|split]

`uniform` is N rows of 12 distinct uniform random columns each (short equal
rows with scattered x reads); `--csr-kernel` forces one CSR kernel instead of
the library's per-matrix choice, to compare kernels on one matrix.

Under torchrun (N > 1) every rank runs an independent replica (rows of
different matrices are independent objects; no collective on the data path),
`value` is the sum over ranks and `scaling` is "weak".

--impl reference times the reference's CPU algorithm for the same workload:
the oracle's restatement of Morpheus's OpenMP multiply
(impl/Csr/OpenMP/Morpheus_Multiply_Impl.hpp:37-58), on all host cores, rank 0
only (the reference library itself needs Kokkos and cannot be built here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

FALLBACK_HBM_GBS = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


# --------------------------------------------------------------------------
# workloads
# --------------------------------------------------------------------------

DEFAULT_SIZE = {"power_law": 2_000_000, "stencil27": 160, "laplacian": 256, "uniform": 2_000_000}


UNIFORM_ROW_LEN = 12
CSR_KERNELS = {"auto": None, "segments": 1, "rows": 2, "split": 3, "gather": 4}


def build_workload(name: str, fmt: str, dtype, seed: int, size: int | None = None):
    """size: rows of the power-law matrix, or the grid edge of the stencil /
    Laplacian (defaults: the benchmark configurations; smaller sizes are for
    profiler captures)."""
    from morpheus_gb300 import generators as gen
    n = size or DEFAULT_SIZE.get(name, 0)
    if name == "power_law":
        A = gen.power_law(n, seed=seed, dtype=dtype)
    elif name == "stencil27":
        A = gen.stencil_27pt(n, seed=seed, dtype=dtype)
        if fmt == "hdc":
            A = gen.add_offband(A, 0.01, seed=seed + 1)
    elif name == "laplacian":
        A = gen.laplacian_2d(n, dtype=dtype)
    elif name == "uniform":  # n rows of ROW_LEN distinct uniform random columns (scattered x reads)
        A = gen.random_lengths_csr(n, n, np.full(n, UNIFORM_ROW_LEN), seed=seed, dtype=dtype)
    else:
        raise SystemExit(f"unknown workload {name}")
    if fmt == "csr":
        hm = A
    elif fmt == "coo":
        hm = gen.csr_to_coo_host(A)
    elif fmt == "dia":
        hm = gen.csr_to_dia_host(A)
    elif fmt == "ell":
        p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
        hm = gen.csr_to_hyb_host(A, p90)["ell"] if name == "power_law" else gen.csr_to_ell_host(A)
        if name == "power_law":  # ELL part only: rows longer than p90 are truncated -> use HYB for full
            raise SystemExit("power-law ELL at the p90 width needs the COO remainder: use --format hyb")
    elif fmt == "hyb":
        p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
        hm = gen.csr_to_hyb_host(A, p90 if name == "power_law" else max(1, A["nnz"] // A["nrows"]))
    elif fmt == "hdc":
        hm = gen.csr_to_hdc_host(A)
    else:
        raise SystemExit(f"unknown format {fmt}")
    return A, hm


def algorithmic_bytes(hm: dict, vbytes: int) -> int:
    """Bytes one SpMV must move: every stored index/value once, x once, y once."""
    f = hm["format"]
    n, m = hm["nrows"], hm["ncols"]
    xy = (m + n) * vbytes
    if f == 0:
        return hm["nnz"] * (8 + vbytes) + xy
    if f == 1:
        return hm["nnz"] * (4 + vbytes) + 4 * (n + 1) + xy
    if f == 2:
        return hm["ndiags"] * n * vbytes + 4 * hm["ndiags"] + xy
    if f == 3:
        return n * hm["width"] * (4 + vbytes) + xy
    if f == 4:
        e, c = hm["ell"], hm["coo"]
        return n * e["width"] * (4 + vbytes) + c["nnz"] * (8 + vbytes) + xy
    if f == 5:
        d, c = hm["dia"], hm["csr"]
        return d["ndiags"] * n * vbytes + 4 * d["ndiags"] + c["nnz"] * (4 + vbytes) + 4 * (n + 1) + xy
    raise ValueError(f)


def host_arrays(hm: dict):
    out = []
    for k, v in hm.items():
        if isinstance(v, dict):
            out += host_arrays(v)
        elif isinstance(v, np.ndarray):
            out.append((k, v))
    return out


# --------------------------------------------------------------------------
# clocks
# --------------------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        rows = [r.split(",") for r in out.strip().splitlines() if r.count(",") >= 8]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i]
                          and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# --------------------------------------------------------------------------
# CPU baseline (oracle restatement of the reference OpenMP multiply)
# --------------------------------------------------------------------------

def cpu_multiply_timing(hm: dict, x: np.ndarray, budget_s: float, threads: int, min_reps: int = 3):
    from oracle import oracle as O
    from oracle.build import build_oracle
    build_oracle()
    om = O.OracleMatrix.from_host(hm)
    y = np.zeros(hm["nrows"], dtype=x.dtype)
    om.multiply(x, y, init=True, threads=threads)  # warm
    times = []
    t_end = time.perf_counter() + budget_s
    while len(times) < min_reps or time.perf_counter() < t_end:
        t0 = time.perf_counter()
        om.multiply(x, y, init=True, threads=threads)
        times.append(time.perf_counter() - t0)
        if len(times) >= 10000:
            break
    return times


def run_reference(args, rank: int):
    if rank != 0:
        return
    dtype = np.float64 if args.dtype == "f64" else np.float32
    vbytes = np.dtype(dtype).itemsize
    from oracle import oracle as O
    from oracle.build import build_oracle
    build_oracle()
    threads = O.max_threads()
    if args.workload == "batched":
        from morpheus_gb300 import generators as gen
        mats = gen.batched_csr(args.batch, seed=0, dtype=dtype)
        sample = mats[: min(len(mats), 256)]  # bounded sample per step
        oms = [O.OracleMatrix.from_host(m) for m in sample]
        xs = [np.random.default_rng(1 + i).uniform(-1, 1, m["ncols"]).astype(dtype) for i, m in enumerate(sample)]
        ysb = [np.zeros(m["nrows"], dtype=dtype) for m in sample]
        nbytes = sum(algorithmic_bytes(m, vbytes) for m in sample)

        def step():
            for om, xv, yv in zip(oms, xs, ysb):
                om.multiply(xv, yv, init=True, threads=threads)
        hm = {"nrows": sum(m["nrows"] for m in mats), "ncols": sum(m["ncols"] for m in mats),
              "nnz": sum(m["nnz"] for m in mats)}
        sample_desc = f"first {len(sample)} of {len(mats)} matrices per step, one OpenMP multiply each"
    else:
        A, hm = build_workload(args.workload, args.format, dtype, seed=0, size=args.size)
        nbytes = algorithmic_bytes(hm, vbytes)
        x = np.random.default_rng(1).uniform(-1, 1, hm["ncols"]).astype(dtype)
        om = O.OracleMatrix.from_host(hm)
        y = np.zeros(hm["nrows"], dtype=dtype)

        def step():
            om.multiply(x, y, init=True, threads=threads)
        sample_desc = f"full matrix, {args.steps} timed multiplies"
    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    el = time.perf_counter() - t0
    gbs = nbytes * args.steps / el / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": gbs, "unit": "GB/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (seeded)", "config": config_dict(args, hm),
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{sample_desc} (reference OpenMP algorithm restated in oracle/oracle.cpp)"},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


METRIC = "SpMV GB/s (% HBM peak)"


def config_dict(args, hm):
    name = (f"batched_csr_{args.batch}_{args.dtype}" if args.workload == "batched"
            else f"{args.workload}_{args.format}_{args.dtype}")
    return {"workload": name, "format": args.format.upper(),
            "nrows": hm["nrows"], "ncols": hm["ncols"], "nnz": hm["nnz"],
            "l2": "inputs larger than L2 (no flush needed)" if args.workload != "laplacian"
            else "L2 flushed between steps (256 MB scratch write)",
            "parallelism": f"replicas x{args.gpus}",
            **({"size": args.size} if getattr(args, "size", None) else {}),
            **({"row_len": UNIFORM_ROW_LEN} if args.workload == "uniform" else {}),
            **({"csr_kernel": args.csr_kernel}
               if args.format == "csr" and getattr(args, "csr_kernel", "auto") != "auto" else {})}


# --------------------------------------------------------------------------
# GPU arm
# --------------------------------------------------------------------------

def run_gpu(args, rank: int, world: int, local_rank: int):
    import ctypes as C

    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import _lib

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dtype = np.float64 if args.dtype == "f64" else np.float32
    tdtype = torch.float64 if args.dtype == "f64" else torch.float32
    vbytes = np.dtype(dtype).itemsize
    A, hm = build_workload(args.workload, args.format, dtype, seed=rank, size=args.size)
    nbytes = algorithmic_bytes(hm, vbytes)
    M = mgb.matrix_from_host(hm, device=dev)
    if args.format == "csr" and CSR_KERNELS[args.csr_kernel] is not None:
        M._variant = CSR_KERNELS[args.csr_kernel]  # a forced CSR kernel (profiling comparisons)
    x_np = np.random.default_rng(1 + rank).uniform(-1, 1, hm["ncols"]).astype(dtype)
    x = torch.from_numpy(x_np).to(dev)
    y = torch.zeros(hm["nrows"], dtype=tdtype, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush = None
    if args.workload == "laplacian":  # L2-resident: flush with a >L2 write between steps
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    # correctness gate on this exact input (rank 0): GPU vs oracle OpenMP multiply
    check_err = None
    if rank == 0 and not args.skip_check:
        from oracle import oracle as O
        from oracle.build import build_oracle
        build_oracle()
        ref = O.OracleMatrix.from_host(hm).multiply(x_np, threads=O.max_threads())
        mgb.multiply(M, x, y, init=True)
        torch.cuda.synchronize()
        yy = y.cpu().numpy().astype(np.float64)
        check_err = float(np.linalg.norm(yy - ref) / max(np.linalg.norm(ref), 1e-300))

    for _ in range(args.warmup):
        mgb.multiply(M, x, y, init=True)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    per = []
    torch.cuda.synchronize()
    if flush is None:
        ev0.record(stream)
        for _ in range(args.steps):
            mgb.multiply(M, x, y, init=True)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        kernel_ms = ms / args.steps
    else:
        # flush between steps; time each SpMV separately with events
        ms = 0.0
        for _ in range(args.steps):
            flush.fill_(1)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            mgb.multiply(M, x, y, init=True)
            b.record(stream)
            per.append((a, b))
        torch.cuda.synchronize()
        times = [a.elapsed_time(b) for a, b in per]
        ms = sum(times)
        kernel_ms = ms / args.steps
    clocks = sampler.stop()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        kernel_ms = ms / args.steps
    value = world * nbytes * args.steps / (ms * 1e-3) / 1e9

    # e2e: host buffers through the C ABI, H2D of the step's inputs and D2H of y inside the region
    pinned = {}
    h2d = 0
    for k, arr in host_arrays(hm):
        t = torch.from_numpy(np.ascontiguousarray(arr)).pin_memory()
        pinned[id(arr)] = t
        h2d += t.numel() * t.element_size()
    xh = torch.from_numpy(x_np).pin_memory()
    h2d += xh.numel() * xh.element_size()
    yh = torch.empty(hm["nrows"], dtype=tdtype).pin_memory()
    d2h = yh.numel() * yh.element_size()
    dev_bufs = mgb.matrix_from_host(hm, device=dev)  # destination buffers of the copies

    def dev_tensors(Mx):
        out = []
        for name in ("_ri", "_ro", "_ci", "_off", "_v"):
            if hasattr(Mx, name):
                out.append(getattr(Mx, name))
        for sub in ("_ell", "_coo", "_dia", "_csr"):
            if hasattr(Mx, sub):
                out += dev_tensors(getattr(Mx, sub))
        return out

    host_list = [pinned[id(a)] for _, a in host_arrays(hm)]
    dst_list = dev_tensors(dev_bufs)
    # pair host and device tensors by size and dtype (same traversal order)
    pairs = []
    used = set()
    for h in host_list:
        for i, d in enumerate(dst_list):
            if i not in used and d.numel() == h.numel() and d.dtype == h.dtype:
                pairs.append((h, d))
                used.add(i)
                break
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_api = "torch copies + multiply"
    host_csr = None
    if args.format == "csr":
        # the library's host-data entry point: pipelined block copies + kernels
        host_csr = mgb.matrix_from_host(hm, device="cpu", dtype=tdtype)
        host_csr._ro = pinned[id(hm["row_offsets"])]
        host_csr._ci = pinned[id(hm["column_indices"])]
        host_csr._v = pinned[id(hm["values"])].to(tdtype) if pinned[id(hm["values"])].dtype != tdtype \
            else pinned[id(hm["values"])]
        e2e_api = "multiply_host (mgb_spmv_csr_host, pipelined row blocks)"
        mgb.multiply_host(host_csr, xh, yh, init=True)  # warm-up (pool allocation, kernel choice)
    else:
        for h, d in pairs:  # one untimed end-to-end step (allocator pool, first-touch costs)
            d.copy_(h, non_blocking=True)
        x.copy_(xh, non_blocking=True)
        mgb.multiply(dev_bufs, x, y, init=True)
        yh.copy_(y, non_blocking=True)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(e2e_steps):
        if host_csr is not None:
            mgb.multiply_host(host_csr, xh, yh, init=True)
        else:
            for h, d in pairs:
                d.copy_(h, non_blocking=True)
            x.copy_(xh, non_blocking=True)
            mgb.multiply(dev_bufs, x, y, init=True)
            yh.copy_(y, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / e2e_steps
    e2e_val = world * nbytes / (e2e_ms * 1e-3) / 1e9

    if rank != 0:
        return
    peak, peak_src = peaks()
    achieved = nbytes / (kernel_ms * 1e-3) / 1e9
    traffic = profile_traffic(args)
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (seeded power-law / stencil generators, N(0,1) values)",
        "config": config_dict(args, hm),
        "pct_hbm_peak": 100.0 * achieved / peak,
        "rel_err_vs_oracle": check_err,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                     else "fallback 6.8 TB/s", "algorithmic_bytes_per_launch": nbytes},
        "e2e": {"value": e2e_val, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "api": e2e_api},
        "gflops": 2.0 * hm["nnz"] / (kernel_ms * 1e-3) / 1e9 if hm.get("nnz") else None,
        "gpu_launches": args.steps * launches_per_step(hm),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        from oracle import oracle as O
        threads = O.max_threads()
        times = cpu_multiply_timing(hm, x_np, args.cpu_budget, threads)
        med = statistics.median(times)
        # the Serial algorithm on one core, a bounded sample (about 3 s)
        st = cpu_multiply_timing(hm, x_np, min(3.0, args.cpu_budget), 0, min_reps=1)
        line["cpu_baseline"] = {"value": nbytes / med / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
                                "sample": f"full matrix, {len(times)} multiplies over ~{args.cpu_budget:.0f} s, "
                                          "median (reference OpenMP algorithm restated in oracle/oracle.cpp)",
                                "serial_1_core": {"value": nbytes / statistics.median(st) / 1e9, "unit": "GB/s",
                                                  "sample": f"{len(st)} Serial multiplies, median"}}
    print(json.dumps(line), flush=True)


def run_gpu_cg(args, rank: int, world: int, local_rank: int):
    """Conjugate gradients on a 2-D 5-point Laplacian (SPD, default 2048^2 grid,
    N = 4.19 M, nnz = 21 M, CSR FP64): the device-resident fused CG
    (mgb_cg_csr_f64: SpMV + p.Ap, x/r update + r.r, graph-captured blocks of
    16 iterations) against the same recurrence composed of the library's
    separate calls (multiply, dot, waxpby).  One step = one CG iteration;
    `value` = fused iterations per second; the unfused rate is reported beside it."""
    import torch
    import morpheus_gb300 as mgb
    from morpheus_gb300 import generators as gen
    from morpheus_gb300 import solvers
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    n = args.size or 2048
    hm = gen.laplacian_2d(n)
    A = mgb.matrix_from_host(hm, device=dev)
    N = hm["nrows"]
    b = torch.from_numpy(np.random.default_rng(3 + rank).uniform(-1, 1, N)).to(dev)
    iters = max(args.steps, 16)
    stream = torch.cuda.current_stream(dev)

    def fused():
        x = torch.zeros(N, dtype=torch.float64, device=dev)
        it, _ = solvers.cg(A, b, x, max_iters=iters, rtol=0.0)
        return it

    def unfused():
        # the same recurrence from the separate calls; dot returns a host scalar
        x = torch.zeros(N, dtype=torch.float64, device=dev)
        r = b.clone()
        p = r.clone()
        ap = torch.empty_like(r)
        rr = mgb.dot(N, r, r)
        for _ in range(iters):
            mgb.multiply(A, p, ap)
            alpha = rr / mgb.dot(N, p, ap)
            mgb.waxpby(N, 1.0, x, alpha, p, x)
            mgb.waxpby(N, 1.0, r, -alpha, ap, r)
            rr_new = mgb.dot(N, r, r)
            mgb.waxpby(N, 1.0, r, rr_new / rr, p, p)
            rr = rr_new
        return iters

    for _ in range(max(1, args.warmup)):
        fused()
    unfused()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(stream)
    done = fused()
    e1.record(stream)
    unfused()
    e2.record(stream)
    torch.cuda.synchronize()
    clocks = sampler.stop()
    fused_ms = e0.elapsed_time(e1)
    unfused_ms = e1.elapsed_time(e2)
    spmv_bytes = algorithmic_bytes(hm, 8)
    line = {
        "metric": "CG iterations/s (fused device-resident CG)", "value": done / (fused_ms * 1e-3),
        "unit": "iterations/s", "n_gpus": 1, "steps": done, "warmup": args.warmup,
        "ms_per_step": fused_ms / done, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (2-D 5-point Laplacian, b uniform in [-1, 1])",
        "config": {"workload": f"cg_laplacian_{n}x{n}_f64", "nrows": N, "nnz": hm["nnz"],
                   "kernel_variant": A.kernel_variant()},
        "unfused": {"value": iters / (unfused_ms * 1e-3), "unit": "iterations/s", "ms_per_step": unfused_ms / iters},
        "speedup_of_fused": unfused_ms / fused_ms,
        "spmv_share_bytes_per_iteration": spmv_bytes,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def run_gpu_batched(args, rank: int, world: int, local_rank: int):
    """4,096 independent FP64 CSR SpMVs per step in one autotuned persistent
    launch, replayed as a CUDA graph; baseline: the same SpMVs as separate
    single-matrix calls."""
    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import batched
    from morpheus_gb300 import generators as gen

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dtype = np.float64 if args.dtype == "f64" else np.float32
    vbytes = np.dtype(dtype).itemsize
    mats = gen.batched_csr(args.batch, seed=rank, dtype=dtype)
    nbytes = sum(algorithmic_bytes(m, vbytes) for m in mats)
    dmats = [mgb.matrix_from_host(m, device=dev) for m in mats]
    xs_np = [np.random.default_rng(1 + i).uniform(-1, 1, m["ncols"]).astype(dtype) for i, m in enumerate(mats)]
    xs = [torch.from_numpy(v).to(dev) for v in xs_np]
    ys = [torch.zeros(m["nrows"], dtype=dmats[0].dtype, device=dev) for m in mats]
    b = batched.CsrBatch(dmats, xs, ys)
    if args.batched_config is None:
        best, tune_ms = b.autotune(reps=3, use_cache=False)
    else:  # a fixed configuration (profiling comparisons): no autotuning launches
        best, tune_ms = args.batched_config, None
        b.plan(best)
    check_err = None
    if rank == 0 and not args.skip_check:
        from oracle import oracle as O
        from oracle.build import build_oracle
        build_oracle()
        b.multiply()
        torch.cuda.synchronize()
        errs = []
        for i in range(0, len(mats), max(1, len(mats) // 64)):  # 64 sampled matrices
            ref = O.OracleMatrix.from_host(mats[i]).multiply(xs_np[i])
            errs.append(np.linalg.norm(ys[i].cpu().numpy() - ref) / max(np.linalg.norm(ref), 1e-300))
        check_err = float(max(errs))
    g = b.capture_graph(init=True)
    stream = torch.cuda.current_stream(dev)
    for _ in range(args.warmup):
        g.replay()
    torch.cuda.synchronize()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    kernel_ms = ms / args.steps
    # baseline: one single-matrix call per matrix (the reference's usage)
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for A, x, y in zip(dmats, xs, ys):
        mgb.multiply(A, x, y)
    torch.cuda.synchronize()
    s0.record(stream)
    for A, x, y in zip(dmats, xs, ys):
        mgb.multiply(A, x, y)
    s1.record(stream)
    torch.cuda.synchronize()
    sep_ms = s0.elapsed_time(s1)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * nbytes * args.steps / (ms * 1e-3) / 1e9
    # e2e: host arrays -> device, batched launch, y -> host, every step
    host = []
    for m, xv in zip(mats, xs_np):
        host.append([torch.from_numpy(np.ascontiguousarray(m[k])).pin_memory()
                     for k in ("row_offsets", "column_indices", "values")] + [torch.from_numpy(xv).pin_memory()])
    dsts = [[A.row_offsets(), A.column_indices(), A.values(), x] for A, x in zip(dmats, xs)]
    yh = [torch.empty(y.numel(), dtype=y.dtype).pin_memory() for y in ys]
    h2d = sum(t.numel() * t.element_size() for h in host for t in h)
    d2h = sum(t.numel() * t.element_size() for t in yh)
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    torch.cuda.synchronize()
    a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a0.record(stream)
    for _ in range(e2e_steps):
        for hs, ds in zip(host, dsts):
            for h, d in zip(hs, ds):
                d.copy_(h, non_blocking=True)
        b.multiply()
        for y, h in zip(ys, yh):
            h.copy_(y, non_blocking=True)
    a1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = a0.elapsed_time(a1) / e2e_steps
    if rank != 0:
        return
    peak, peak_src = peaks()
    achieved = nbytes / (kernel_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": args.dtype, "data": "synthetic (seeded batched CSR generator)",
        "config": {"workload": f"batched_csr_{args.batch}_{args.dtype}", "matrices": len(mats),
                   "nnz_total": int(sum(m["nnz"] for m in mats)),
                   "rows_total": int(sum(m["nrows"] for m in mats)),
                   "l2": "inputs larger than L2 (no flush needed)", "parallelism": f"replicas x{world}",
                   ("autotuned_config" if tune_ms is not None else "fixed_config"): best,
                   "config_chunk_seg": batched.config_info(best),
                   **({"autotune_ms_per_config": tune_ms} if tune_ms is not None else {})},
        "pct_hbm_peak": 100.0 * achieved / peak, "rel_err_vs_oracle": check_err,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": batched_traffic(args), "peak_source": peak_src,
                     "algorithmic_bytes_per_launch": nbytes},
        "separate_calls": {"ms": sep_ms, "GB/s": nbytes / (sep_ms * 1e-3) / 1e9, "launches": 2 * len(mats),
                           "speedup_of_batched": sep_ms / kernel_ms},
        "e2e": {"value": world * nbytes / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms},
        "gpu_launches": args.steps * 1, "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        from oracle.build import build_oracle
        build_oracle()
        threads = O.max_threads()
        oms = [O.OracleMatrix.from_host(m) for m in mats]
        ys_h = [np.zeros(m["nrows"], dtype=dtype) for m in mats]
        t0 = time.perf_counter()
        done_bytes = 0
        for om, m, xv, yv in zip(oms, mats, xs_np, ys_h):  # the reference: one multiply per matrix
            om.multiply(xv, yv, init=True, threads=threads)
            done_bytes += algorithmic_bytes(m, vbytes)
            if time.perf_counter() - t0 > args.cpu_budget:
                break
        el = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": done_bytes / el / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
                                "sample": f"one OpenMP multiply per matrix over the batch (reference usage), "
                                          f"{done_bytes} bytes in {el:.2f} s"}
    print(json.dumps(line), flush=True)


def launches_per_step(hm) -> int:
    f = hm["format"]
    if f == 0:
        return 2  # chunk kernel + carry fix-up
    if f == 4:
        return 1 + (2 if hm["coo"]["nnz"] else 0)
    return 1


def batched_traffic(args):
    """DRAM bytes per launch of the batched kernel from its committed ncu
    summary (the default 4,096-matrix FP64 batch only)."""
    if args.batch != 4096 or args.dtype != "f64":
        return None
    p = os.path.join(ROOT, "profiles", "spmv_batched_csr_f64.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def profile_traffic(args):
    """DRAM bytes per launch from the committed ncu summary, if one exists."""
    p = os.path.join(ROOT, "profiles", f"spmv_{args.format}_{args.workload}_{args.dtype}.md")
    if args.size is not None or not os.path.exists(p):  # summaries describe the default sizes
        return None
    for line in open(p):
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="mgb", choices=["mgb", "reference"])
    ap.add_argument("--workload", default="power_law",
                    choices=["power_law", "stencil27", "laplacian", "uniform", "batched", "cg"])
    ap.add_argument("--csr-kernel", default="auto", choices=sorted(CSR_KERNELS),
                    help="force one CSR kernel instead of the per-matrix choice (profiling)")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--batched-config", type=int, default=None,
                    help="batched workload: use this configuration instead of autotuning (profiling)")
    ap.add_argument("--size", type=int, default=None,
                    help="power-law rows / stencil or Laplacian grid edge (default: the benchmark size)")
    ap.add_argument("--format", default="csr", choices=["csr", "coo", "dia", "ell", "hyb", "hdc"])
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=10.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-check", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        if args.workload == "batched":
            run_gpu_batched(args, rank, world, local_rank)
        elif args.workload == "cg":
            run_gpu_cg(args, rank, world, local_rank)
        else:
            run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
