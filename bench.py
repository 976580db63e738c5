"""SpMV benchmark: GB/s of algorithmic bytes (% of HBM peak), the learned
format selector's speed-up over CSR, and relative error against the oracle.

Default (`--workload suite`): one run measures every benchmark configuration.

  headline   27-point stencil on a 160^3 grid (N = 4,096,000, 109,215,352
             nnz), FP64, through the product path: a DynamicMatrix built in
             CSR and switched in place by the learned selector
             (convert(dyn, AUTO_FORMAT)).  `value` = GB/s of that format's
             multiply; `csr_default` = the library's CSR multiply on the same
             matrix; `speedup_vs_csr_default` = t_csr / t_selected.
  per_config C1 Laplacian 256^2 (CSR, COO, DIA; L2 flushed between steps),
             C2 power-law N = 2e6 (CSR, COO, HYB at the 90th-percentile row
             length; FP64 and FP32), C3 stencil (DIA, CSR, FP32 DIA / CSR,
             HDC of the stencil plus 1 % off-band entries), C4 the learned
             selector on 400 held-out corpus matrices (every format timed
             here; regret and speed-up over CSR-only), C5 4,096 CSR matrices
             in one persistent launch.  Every SpMV entry carries rel_err
             against the oracle, a roofline naming its binding unit (HBM,
             FP64 pipe or L1TEX random-sector rate, each ceiling measured in
             this run by the library's peak kernels) and CPU baselines (the
             reference's Serial algorithm on one core and its OpenMP
             algorithm on every host core, both restated in oracle/).

One step = one y = A*x over the whole matrix; inputs are larger than L2
except C1, which is timed with a 256 MB write between steps.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]
                    [--workload suite|peaks|power_law|stencil27|laplacian|uniform|batched|cg|convert]
                    [--format csr|coo|dia|ell|hyb|hdc] [--dtype f64|f32] [--size S]
                    [--csr-kernel auto|segments|rows|gather|split]

The single workloads time one configuration (profiling commands use them);
`peaks` prints the measured ceilings alone.  Under torchrun (N > 1) every rank
runs an independent replica of the headline (rows of different matrices are
independent; no collective on the data path), `value` is the sum over ranks,
`scaling` is "weak", and rank 0 alone adds the per-config entries.

--impl reference times the reference's CPU algorithm on the same workload:
the oracle's restatement of Morpheus's OpenMP multiply
(impl/<Fmt>/OpenMP/Morpheus_Multiply_Impl.hpp) on every host core, rank 0
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
METRIC = "SpMV GB/s (% HBM peak); learned-format vs CSR-default speedup, rel err<=1e-12"
FORMAT_NAMES = ["coo", "csr", "dia", "ell", "hyb", "hdc"]
# The format the learned selector picks for the 27-point stencil (checked by
# the GPU arm, which reports the format it actually switched to); the
# reference arm times its OpenMP multiply in this format.
HEADLINE_FORMAT = "dia"


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
CSR_KERNEL_NAMES = {1: "lane segments", 2: "row tiles", 3: "split chunks", 4: "row tiles (gather carve-out)"}


def build_csr(name: str, dtype, seed: int, size: int | None = None, offband: bool = False) -> dict:
    """Host CSR of a benchmark matrix.  size: rows of the power-law / uniform
    matrix, or the grid edge of the stencil / Laplacian."""
    from morpheus_gb300 import generators as gen
    n = size or DEFAULT_SIZE.get(name, 0)
    if name == "power_law":
        A = gen.power_law(n, seed=seed, dtype=dtype)
    elif name == "stencil27":
        A = gen.stencil_27pt(n, seed=seed, dtype=dtype)
        if offband:
            A = gen.add_offband(A, 0.01, seed=seed + 1)
    elif name == "laplacian":
        A = gen.laplacian_2d(n, dtype=dtype)
    elif name == "uniform":  # n rows of ROW_LEN distinct uniform random columns (scattered x reads)
        A = gen.random_lengths_csr(n, n, np.full(n, UNIFORM_ROW_LEN), seed=seed, dtype=dtype)
    else:
        raise SystemExit(f"unknown workload {name}")
    return A


def build_workload(name: str, fmt: str, dtype, seed: int, size: int | None = None):
    """(host CSR, host matrix in `fmt`), formats built on the host by the
    reference's conversion rules (single-workload mode)."""
    from morpheus_gb300 import generators as gen
    A = build_csr(name, dtype, seed, size, offband=(name == "stencil27" and fmt == "hdc"))
    if fmt == "csr":
        hm = A
    elif fmt == "coo":
        hm = gen.csr_to_coo_host(A)
    elif fmt == "dia":
        hm = gen.csr_to_dia_host(A)
    elif fmt == "ell":
        if name == "power_law":  # rows longer than p90 would be truncated: the COO remainder is HYB's
            raise SystemExit("power-law ELL at the p90 width needs the COO remainder: use --format hyb")
        hm = gen.csr_to_ell_host(A)
    elif fmt == "hyb":
        p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
        hm = gen.csr_to_hyb_host(A, p90 if name == "power_law" else max(1, A["nnz"] // A["nrows"]))
    elif fmt == "hdc":
        hm = gen.csr_to_hdc_host(A)
    else:
        raise SystemExit(f"unknown format {fmt}")
    return A, hm


def ell_stored(e: dict) -> int:
    """Entries an ELL part really holds (its padding slots excluded)."""
    return int(e["nnz"])


def algorithmic_bytes(hm: dict, vbytes: int) -> int:
    """Bytes one SpMV must move: every stored index/value once (ELL padding
    slots not counted), x once, y once."""
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
        return ell_stored(hm) * (4 + vbytes) + xy
    if f == 4:
        e, c = hm["ell"], hm["coo"]
        return ell_stored(e) * (4 + vbytes) + c["nnz"] * (8 + vbytes) + xy
    if f == 5:
        d, c = hm["dia"], hm["csr"]
        return d["ndiags"] * n * vbytes + 4 * d["ndiags"] + c["nnz"] * (4 + vbytes) + 4 * (n + 1) + xy
    raise ValueError(f)


def fma_count(hm: dict) -> int:
    """FMAs one SpMV issues: one per stored slot the kernel multiplies (every
    DIA slot, including the zeros a diagonal holds; every real entry of the
    other formats)."""
    f = hm["format"]
    if f == 2:
        return hm["ndiags"] * hm["nrows"]
    if f == 5:
        return hm["dia"]["ndiags"] * hm["nrows"] + hm["csr"]["nnz"]
    return int(hm["nnz"])


def stream_bytes(hm: dict, vbytes: int) -> int:
    """Matrix bytes (indices and values) one SpMV streams."""
    return algorithmic_bytes(hm, vbytes) - (hm["nrows"] + hm["ncols"]) * vbytes


def launches_per_step(hm) -> int:
    f = hm["format"]
    if f == 0:
        return 2  # chunk kernel + carry fix-up
    if f == 4:
        return 1 + (2 if hm["coo"]["nnz"] else 0)
    return 1


def host_arrays(hm: dict):
    out = []
    for k, v in hm.items():
        if isinstance(v, dict):
            out += host_arrays(v)
        elif isinstance(v, np.ndarray):
            out.append((k, v))
    return out


def cast_values(hm: dict, dtype) -> dict:
    out = {}
    for k, v in hm.items():
        if isinstance(v, dict):
            out[k] = cast_values(v, dtype)
        elif isinstance(v, np.ndarray) and v.dtype.kind == "f":
            out[k] = v.astype(dtype)
        else:
            out[k] = v
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
# ceilings of the binding units, measured on this GPU
# --------------------------------------------------------------------------

def measure_unit_peaks(dev) -> dict:
    """FP64 FMA throughput and random 8-byte gather rate (one 32-byte L1TEX
    sector each) of this GPU, from the library's peak kernels
    (mgb_peak_dfma_f64, mgb_peak_gather_f64) timed with CUDA events; best of
    3 launches after a warm-up."""
    import ctypes as C

    import torch

    from morpheus_gb300 import _lib
    lib = _lib.load()
    tpb = lib.mgb_peak_threads_per_block()
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    stream = torch.cuda.current_stream(dev)
    sh = C.c_void_p(stream.cuda_stream)

    def best_ms(launch, reps=3):
        launch()
        torch.cuda.synchronize(dev)
        out = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            launch()
            b.record(stream)
            b.synchronize()
            out.append(a.elapsed_time(b))
        return min(out)

    blocks = sms * 8
    sink = torch.empty(blocks * tpb, dtype=torch.float64, device=dev)
    iters = 512  # ~2.4 ms per launch
    ms = best_ms(lambda: _lib.call("mgb_peak_dfma_f64", blocks, iters, C.c_void_p(sink.data_ptr()), sh))
    fma_per_s = blocks * tpb * iters * 8 / (ms * 1e-3)
    table_len = 1 << 21  # 16 MB of doubles: L2-resident, like x of the power-law matrix
    table = torch.rand(table_len, dtype=torch.float64, device=dev)
    steps = 128
    ms_g = best_ms(lambda: _lib.call("mgb_peak_gather_f64", C.c_void_p(table.data_ptr()), table_len, blocks, steps,
                                     C.c_void_p(sink.data_ptr()), sh))
    gathers_per_s = blocks * tpb * steps * 8 / (ms_g * 1e-3)
    hbm, src = peaks()
    return {"hbm_gbs": hbm, "hbm_source": f"{src} (MEASURED_PEAKS.json hbm_gbs: copy read+write)"
            if src == "measured" else "fallback 6.8 TB/s",
            "fp64_fma_per_s": fma_per_s, "fp64_tflops": 2 * fma_per_s / 1e12,
            "random_sectors_per_s": gathers_per_s, "sms": sms,
            "how": "mgb_peak_dfma_f64: 8 independent FMA chains per lane, 8 CTAs x 256 threads per SM; "
                   "mgb_peak_gather_f64: 8 random 8-byte loads in flight per lane from a 16 MB table; "
                   "best of 3 launches, CUDA events"}


def roofline(hm: dict, vbytes: int, us: float, unit_peaks: dict, x_access: str, traffic=None,
             nbytes: int | None = None) -> dict:
    """HBM roofline plus the binding unit: the largest of the HBM floor
    (algorithmic bytes / copy peak), the FP64 floor (FMAs / measured FMA
    rate; FP64 only) and, for scattered x reads, the L1TEX floor ((one
    sector per x read + the matrix stream's sectors) / measured sector rate)."""
    nbytes = algorithmic_bytes(hm, vbytes) if nbytes is None else nbytes
    achieved = nbytes / (us * 1e-6) / 1e9
    peak = unit_peaks["hbm_gbs"]
    floors = {"hbm": nbytes / (peak * 1e9) * 1e6}
    if vbytes == 8:
        floors["fp64_pipe"] = fma_count(hm) / unit_peaks["fp64_fma_per_s"] * 1e6
    if x_access == "scattered":
        sectors = int(hm["nnz"]) + stream_bytes(hm, vbytes) / 32.0
        floors["l1tex_random_sectors"] = sectors / unit_peaks["random_sectors_per_s"] * 1e6
    unit = max(floors, key=floors.get)
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "traffic": None if traffic is None else traffic[0],
           "algorithmic_bytes_per_launch": nbytes,
           "binding_unit": unit, "floor_us": floors[unit], "frac_of_binding_unit": floors[unit] / us,
           "floors_us": floors}
    if traffic is not None:
        out["traffic_source"] = traffic[1]
    return out


def profile_traffic(key: str):
    """(DRAM bytes per launch, source) from a committed ncu summary whose
    `workload:` line names this configuration, else None."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return None
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        lines = open(os.path.join(d, fn)).read().splitlines()
        keys = [k for ln in lines if ln.startswith("workload:") for k in ln.split(":", 1)[1].split()]
        if key not in keys:
            continue
        for ln in lines:
            if ln.startswith("dram_bytes_per_launch:"):
                try:
                    v = float(ln.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    return None
                note = ln.split(":", 1)[1].strip().split(None, 1)
                return v, f"profiles/{fn}" + (f" {note[1]}" if len(note) > 1 else "")
    return None


# --------------------------------------------------------------------------
# CPU baselines (oracle restatement of the reference's Serial / OpenMP multiply)
# --------------------------------------------------------------------------

def cpu_multiply_timing(om, x: np.ndarray, budget_s: float, threads: int, min_reps: int = 3):
    y = np.zeros(om.shape()[1], dtype=x.dtype)
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


def cpu_baselines(om, x, nbytes: int, budget_s: float) -> dict:
    from oracle import oracle as O
    threads = O.max_threads()
    omp = cpu_multiply_timing(om, x, budget_s, threads)
    ser = cpu_multiply_timing(om, x, budget_s, 0, min_reps=1)
    return {"value": nbytes / statistics.median(omp) / 1e9, "unit": "GB/s", "cores": threads, "kind": "port",
            "sample": f"full matrix, {len(omp)} OpenMP multiplies over ~{budget_s:.1f} s, median "
                      "(reference OpenMP algorithm restated in oracle/oracle.cpp)",
            "serial_1_core": {"value": nbytes / statistics.median(ser) / 1e9, "unit": "GB/s", "cores": 1,
                              "sample": f"{len(ser)} Serial multiplies, median"}}


def oracle_error(om, hm_dtype, x: np.ndarray, y: np.ndarray) -> float:
    """Normwise relative error of y against the oracle's multiply (FP64 on
    FP64 inputs; an FP32 y against the FP64 oracle of the same FP32 inputs)."""
    from oracle import oracle as O
    if hm_dtype == np.float64:
        ref = om.multiply(x, threads=O.max_threads())
    else:
        ref = om.multiply(x, threads=O.max_threads())  # om holds FP64 values of the FP32 inputs
    ref = ref.astype(np.float64)
    y = y.astype(np.float64)
    den = np.linalg.norm(ref)
    return float(np.linalg.norm(y - ref) / den) if den > 0 else float(np.linalg.norm(y))


# --------------------------------------------------------------------------
# GPU timing helpers
# --------------------------------------------------------------------------

def time_multiply(M, x, y, steps: int, warmup: int, stream, flush=None) -> float:
    """Mean device time (ms) of one multiply over `steps` calls, CUDA events
    on the launching stream.  With `flush`, a >L2 write precedes every call
    and each call is timed alone."""
    import torch

    import morpheus_gb300 as mgb
    for _ in range(max(1, warmup)):
        mgb.multiply(M, x, y, init=True)
    torch.cuda.synchronize()
    if flush is None:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            mgb.multiply(M, x, y, init=True)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps
    per = []
    for _ in range(steps):
        flush.fill_(1)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        mgb.multiply(M, x, y, init=True)
        b.record(stream)
        per.append((a, b))
    torch.cuda.synchronize()
    return sum(a.elapsed_time(b) for a, b in per) / steps


def device_format(A_csr, fmt: str, hyb_width: int = 0):
    """The device matrix in `fmt`, made from the device CSR by the library's
    GPU conversions (the product path)."""
    import morpheus_gb300 as mgb
    if fmt == "csr":
        return A_csr
    coo = mgb.to_coo(A_csr)
    if fmt == "coo":
        return coo
    return mgb.from_coo(coo, FORMAT_NAMES.index(fmt), hyb_width=hyb_width)


def e2e_multiply(M, hm_dev, x_np, y, stream, steps: int, dev):
    """End to end through the public API with host buffers: every step
    copies the container's arrays and x from pinned host memory, multiplies,
    and copies y back (ms per step, H2D bytes, D2H bytes)."""
    import torch

    import morpheus_gb300 as mgb

    def dev_tensors(Mx):
        out = []
        for name in ("_ri", "_ro", "_ci", "_off", "_v"):
            if hasattr(Mx, name):
                out.append(getattr(Mx, name))
        for sub in ("_ell", "_coo", "_dia", "_csr"):
            if hasattr(Mx, sub):
                out += dev_tensors(getattr(Mx, sub))
        return out

    dst = dev_tensors(M)
    src = [t.detach().cpu().pin_memory() for t in dst]  # the same arrays in host memory
    xh = torch.from_numpy(x_np).pin_memory()
    x = torch.empty_like(xh, device=dev)
    yh = torch.empty(y.numel(), dtype=y.dtype).pin_memory()
    h2d = sum(t.numel() * t.element_size() for t in src) + xh.numel() * xh.element_size()
    d2h = yh.numel() * yh.element_size()

    def step():
        for h, d in zip(src, dst):
            d.copy_(h, non_blocking=True)
        x.copy_(xh, non_blocking=True)
        mgb.multiply(M, x, y, init=True)
        yh.copy_(y, non_blocking=True)
    step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps, h2d, d2h


# --------------------------------------------------------------------------
# the suite
# --------------------------------------------------------------------------

def spmv_entry(key, M, x_np, xt, steps, warmup, stream, unit_peaks, x_access, cpu_budget, flush=None,
               hm=None, om=None, extra=None):
    """One per-config SpMV measurement: time, GB/s, rel_err, roofline, CPU."""
    import torch

    import morpheus_gb300 as mgb
    from oracle import oracle as O
    hm = hm if hm is not None else mgb.matrix_to_host(M)
    dtype = np.float64 if M.dtype == torch.float64 else np.float32
    vbytes = 8 if dtype == np.float64 else 4
    nbytes = algorithmic_bytes(hm, vbytes)
    y = torch.zeros(M.nrows(), dtype=M.dtype, device=xt.device)
    mgb.multiply(M, xt, y, init=True)
    torch.cuda.synchronize()
    if om is None:
        om = O.OracleMatrix.from_host(hm if dtype == np.float64 else cast_values(hm, np.float64))
    err = oracle_error(om, dtype, x_np.astype(np.float64), y.cpu().numpy())
    ms = time_multiply(M, xt, y, steps, warmup, stream, flush)
    us = ms * 1e3
    out = {"config": key, "format": FORMAT_NAMES[hm["format"]].upper(), "dtype": "f64" if vbytes == 8 else "f32",
           "nrows": hm["nrows"], "nnz": int(hm["nnz"]), "us_per_spmv": us, "GB/s": nbytes / (ms * 1e-3) / 1e9,
           "rel_err_vs_oracle": err, "rel_err_bar": 1e-12 if vbytes == 8 else 1e-5,
           "roofline": roofline(hm, vbytes, us, unit_peaks, x_access, profile_traffic(key)),
           "l2": "flushed between steps (256 MB write)" if flush is not None else "inputs larger than L2"}
    if M.FORMAT == mgb.CSR_FORMAT:
        out["csr_kernel"] = CSR_KERNEL_NAMES.get(M.kernel_variant(), str(M.kernel_variant()))
    if extra:
        out.update(extra)
    if cpu_budget > 0:
        om_t = om if dtype == np.float64 else O.OracleMatrix.from_host(hm)
        out["cpu_baseline"] = cpu_baselines(om_t, x_np, nbytes, cpu_budget)
    return out


def run_suite(args, rank: int, world: int, local_rank: int):
    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import generators as gen
    from morpheus_gb300.selector import AUTO_FORMAT
    from oracle import oracle as O
    from oracle.build import build_oracle

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.current_stream(dev)
    t_start = time.time()
    if rank == 0:
        build_oracle()
    unit_peaks = measure_unit_peaks(dev)

    # ---- headline: the 27-point stencil through DynamicMatrix + selector --
    S = build_csr("stencil27", np.float64, seed=rank, size=args.size)
    A_csr = mgb.matrix_from_host(S, device=dev)
    dyn = mgb.DynamicMatrix(mgb.matrix_from_host(S, device=dev))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    status = mgb.convert(dyn, AUTO_FORMAT)
    torch.cuda.synchronize()
    switch_ms = (time.perf_counter() - t0) * 1e3
    if status != mgb.conversion_error_e.CONV_SUCCESS:
        raise SystemExit(f"selector switch failed: {status}")
    # the same switch again on a second DynamicMatrix over the CSR container
    # (the first call also pays one-time costs: allocator pool growth, the
    # selector's weights)
    dyn2 = mgb.DynamicMatrix(A_csr)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mgb.convert(dyn2, AUTO_FORMAT)
    torch.cuda.synchronize()
    switch_warm_ms = (time.perf_counter() - t0) * 1e3
    del dyn2
    sel_fmt = FORMAT_NAMES[dyn.active_index()]
    M_sel = dyn.active()
    hm_sel = mgb.matrix_to_host(M_sel)
    x_np = gen.x_vector(S["ncols"], seed=rank, dtype=np.float64)
    xt = torch.from_numpy(x_np).to(dev)
    y = torch.zeros(S["nrows"], dtype=torch.float64, device=dev)
    sel_bytes = algorithmic_bytes(hm_sel, 8)
    csr_bytes = algorithmic_bytes(S, 8)
    check = {}
    om_sel = om_csr = None
    if rank == 0 and not args.skip_check:
        om_sel = O.OracleMatrix.from_host(hm_sel)
        om_csr = O.OracleMatrix.from_host(S)
        mgb.multiply(dyn, xt, y, init=True)
        torch.cuda.synchronize()
        check["selected"] = oracle_error(om_sel, np.float64, x_np, y.cpu().numpy())
        mgb.multiply(A_csr, xt, y, init=True)
        torch.cuda.synchronize()
        check["csr"] = oracle_error(om_csr, np.float64, x_np, y.cpu().numpy())
    for _ in range(args.warmup):
        mgb.multiply(dyn, xt, y, init=True)
        mgb.multiply(A_csr, xt, y, init=True)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        mgb.multiply(dyn, xt, y, init=True)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    csr_ms = time_multiply(A_csr, xt, y, args.steps, 0, stream)
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    kernel_ms = ms / args.steps
    value = world * sel_bytes * args.steps / (ms * 1e-3) / 1e9
    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_ms, h2d, d2h = e2e_multiply(M_sel, hm_sel, x_np, y, stream, e2e_steps, dev)
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        return
    us = kernel_ms * 1e3
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generators with the benchmark configurations' shapes; N(0,1) / stencil values)",
        "config": headline_config(S, HEADLINE_FORMAT, world),
        "selected_format": sel_fmt.upper(),
        "selected_format_matches_reference_arm": sel_fmt == HEADLINE_FORMAT,
        "pct_hbm_peak": 100.0 * (sel_bytes / (kernel_ms * 1e-3) / 1e9) / unit_peaks["hbm_gbs"],
        "rel_err_vs_oracle": check.get("selected"),
        "csr_default": {"us_per_spmv": csr_ms * 1e3, "GB/s": csr_bytes / (csr_ms * 1e-3) / 1e9,
                        "kernel": CSR_KERNEL_NAMES.get(A_csr.kernel_variant()),
                        "rel_err_vs_oracle": check.get("csr"),
                        "roofline": roofline(S, 8, csr_ms * 1e3, unit_peaks, "banded",
                                             profile_traffic("c3_stencil27_160_csr_f64"))},
        "speedup_vs_csr_default": csr_ms / kernel_ms,
        "selector_switch_ms": switch_warm_ms, "selector_switch_first_call_ms": switch_ms,
        "roofline": roofline(hm_sel, 8, us, unit_peaks, "banded",
                             profile_traffic(f"c3_stencil27_160_{sel_fmt}_f64")),
        "unit_peaks": unit_peaks,
        "e2e": {"value": world * sel_bytes / (e2e_ms * 1e-3) / 1e9, "unit": "GB/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
                "api": "pinned host arrays -> device containers (torch copies), morpheus_gb300.multiply, y -> host"},
        "gpu_launches": args.steps * launches_per_step(hm_sel),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baselines(om_sel or O.OracleMatrix.from_host(hm_sel), x_np, sel_bytes,
                                             args.cpu_budget)
    per = []
    if not args.headline_only:
        ck = 0 if args.no_cpu_baseline else args.cfg_cpu_budget
        steps = args.steps
        wu = max(3, args.warmup)
        # C3: the selected format and CSR at full size, from the headline run
        key_sel = f"c3_stencil27_160_{sel_fmt}_f64"
        per.append(spmv_entry(key_sel, M_sel, x_np, xt, steps, wu, stream, unit_peaks, "banded", ck,
                              hm=hm_sel, om=om_sel, extra={"note": "the headline's selected format"}))
        per.append(spmv_entry("c3_stencil27_160_csr_f64", A_csr, x_np, xt, steps, wu, stream, unit_peaks, "banded",
                              ck, hm=S, om=om_csr, extra={"note": "the headline's CSR default"}))
        if sel_fmt != "dia":
            per.append(spmv_entry("c3_stencil27_160_dia_f64", device_format(A_csr, "dia"), x_np, xt, steps, wu,
                                  stream, unit_peaks, "banded", ck))
        del dyn, M_sel, om_sel, om_csr
        # C3 FP32: DIA and CSR
        S32 = cast_values(S, np.float32)
        A32 = mgb.matrix_from_host(S32, device=dev)
        x32 = x_np.astype(np.float32)
        xt32 = torch.from_numpy(x32).to(dev)
        per.append(spmv_entry("c3_stencil27_160_dia_f32", device_format(A32, "dia"), x32, xt32, steps, wu,
                              stream, unit_peaks, "banded", ck))
        per.append(spmv_entry("c3_stencil27_160_csr_f32", A32, x32, xt32, steps, wu, stream, unit_peaks, "banded",
                              ck, hm=S32))
        del A32, xt32
        # C3 + 1 % off-band entries in HDC
        H = gen.add_offband(S, 0.01, seed=rank + 1)
        AH = mgb.matrix_from_host(H, device=dev)
        xh_np = gen.x_vector(H["ncols"], seed=rank, dtype=np.float64)
        per.append(spmv_entry("c3_stencil27_160_offband_hdc_f64", device_format(AH, "hdc"), xh_np,
                              torch.from_numpy(xh_np).to(dev), steps, wu, stream, unit_peaks, "banded", ck))
        del AH, H
        # ELL of the stencil (width = longest row, 27 -> 32 padded slots)
        per.append(spmv_entry("c3_stencil27_160_ell_f64", device_format(A_csr, "ell"), x_np, xt, steps, wu, stream,
                              unit_peaks, "banded", ck))
        del A_csr, S
        torch.cuda.empty_cache()
        # C2: power law, CSR / COO / HYB(p90), FP64 and FP32
        P = build_csr("power_law", np.float64, seed=rank)
        p90 = int(np.percentile(np.diff(P["row_offsets"]), 90))
        for dt, sfx in ((np.float64, "f64"), (np.float32, "f32")):
            Pd = P if dt == np.float64 else cast_values(P, np.float32)
            AP = mgb.matrix_from_host(Pd, device=dev)
            xp = gen.x_vector(P["ncols"], seed=rank, dtype=dt)
            xpt = torch.from_numpy(xp).to(dev)
            for fmt in ("csr", "coo", "hyb"):
                M = device_format(AP, fmt, hyb_width=p90 if fmt == "hyb" else 0)
                per.append(spmv_entry(f"c2_power_law_2e6_{fmt}_{sfx}", M, xp, xpt, steps, wu, stream, unit_peaks,
                                      "scattered", ck, hm=Pd if fmt == "csr" else None,
                                      extra={"hyb_ell_width": p90} if fmt == "hyb" else None))
                del M
            del AP
        del P
        torch.cuda.empty_cache()
        # C1: Laplacian 256^2, L2 flushed between steps
        L = build_csr("laplacian", np.float64, seed=0)
        AL = mgb.matrix_from_host(L, device=dev)
        xl = gen.x_vector(L["ncols"], seed=0)
        xlt = torch.from_numpy(xl).to(dev)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
        for fmt in ("csr", "coo", "dia", "ell"):
            per.append(spmv_entry(f"c1_laplacian_256_{fmt}_f64", device_format(AL, fmt), xl, xlt, steps, wu,
                                  stream, unit_peaks, "banded", ck, flush=flush, hm=L if fmt == "csr" else None))
        del flush
        # C5: batched
        per.append(batched_entry(args, dev, stream, unit_peaks, ck))
        torch.cuda.empty_cache()
        # C4: selector on held-out corpus matrices
        if args.selector_test > 0:
            per.append(selector_entry(args.selector_test))
        # conversions at the benchmark sizes against the Serial convert
        per.append(convert_entry(dev, ck))
        # dot / reduce / waxpby on 512 MB vectors
        per.extend(vector_entry(dev, stream, unit_peaks, ck))
    line["per_config"] = per
    line["suite_seconds"] = time.time() - t_start
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def headline_config(S: dict, fmt: str, world: int) -> dict:
    return {"workload": "stencil27_160_f64_learned_format", "matrix": "27-point stencil, 160^3 grid",
            "format": fmt.upper(), "format_choice": "learned selector (convert(dyn, AUTO_FORMAT))",
            "nrows": S["nrows"], "ncols": S["ncols"], "nnz": int(S["nnz"]),
            "l2": "inputs larger than L2 (no flush needed)", "parallelism": f"replicas x{world}"}


def vector_entry(dev, stream, unit_peaks, cpu_budget: float, n: int = 1 << 26) -> list:
    """dot / reduce / waxpby on 2^26-element FP64 vectors (512 MB each, larger
    than L2), device-resident, timed with CUDA events over 20 launches after a
    warm-up.  Each names its binding unit: HBM (algorithmic bytes / copy
    peak) or the FP64 pipe (FP64 operations / measured FMA rate; an FP64 add
    costs the same as an FMA).  The reduce splits its elements between FP64
    adds and exact integer-pipe accumulation, so its FP64 floor is that of the
    FP64 share (9 of 16).  CPU: the oracle's Serial restatement, one core."""
    import ctypes as C

    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import _lib
    from oracle import oracle as O
    lib = _lib.load()
    rng = np.random.default_rng(21)
    x_np, y_np = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    x, y = torch.from_numpy(x_np).to(dev), torch.from_numpy(y_np).to(dev)
    w = torch.empty_like(x)
    out = torch.zeros(1, dtype=torch.float64, device=dev)
    sh = C.c_void_p(stream.cuda_stream)
    X, Y, W, R = (C.c_void_p(t.data_ptr()) for t in (x, y, w, out))

    def timed_us(launch, k=20):
        for _ in range(3):
            launch()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(k):
            launch()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / k * 1e3

    def cpu_us(fn):
        t0 = time.perf_counter()
        reps = 0
        while reps < 1 or (time.perf_counter() - t0 < min(cpu_budget, 2.0) and reps < 5):
            fn()
            reps += 1
        return (time.perf_counter() - t0) / reps * 1e6

    def check(name, code):
        if code != 0:
            raise SystemExit(f"{name} failed with status {code}")

    ops = [
        ("dot_xy", lambda: check("dot", lib.mgb_dot_f64_async(n, X, Y, R, sh)), 16 * n, n,
         lambda: O.dot(n, x_np, y_np), lambda: float(out.item())),
        ("dot_xx", lambda: check("dot", lib.mgb_dot_f64_async(n, X, X, R, sh)), 8 * n, n,
         lambda: O.dot(n, x_np, x_np), lambda: float(out.item())),
        ("reduce", lambda: check("reduce", lib.mgb_reduce_f64_async(X, n, R, sh)), 8 * n, n * 9 // 16,
         lambda: O.reduce(x_np, n), lambda: float(out.item())),
        ("waxpby_alpha_beta", lambda: check("waxpby", lib.mgb_waxpby_f64(n, 2.15, X, -3.2, Y, W, sh)), 24 * n, 2 * n,
         None, None),
        ("waxpby_alpha_1", lambda: check("waxpby", lib.mgb_waxpby_f64(n, 2.15, X, 1.0, Y, W, sh)), 24 * n, n,
         None, None),
    ]
    res = []
    for name, launch, nbytes, fp64_ops, cpu_fn, gpu_val in ops:
        us = timed_us(launch)
        floors = {"hbm": nbytes / (unit_peaks["hbm_gbs"] * 1e9) * 1e6,
                  "fp64_pipe": fp64_ops / unit_peaks["fp64_fma_per_s"] * 1e6}
        unit = max(floors, key=floors.get)
        e = {"config": f"vector_{name}_2^26_f64", "us": us, "GB/s": nbytes / (us * 1e-6) / 1e9,
             "roofline": {"bound": "hbm", "achieved": nbytes / (us * 1e-6) / 1e9, "peak": unit_peaks["hbm_gbs"],
                          "unit": "GB/s", "frac": nbytes / (us * 1e-6) / 1e9 / unit_peaks["hbm_gbs"],
                          "algorithmic_bytes_per_launch": nbytes, "fp64_ops_per_launch": fp64_ops,
                          "binding_unit": unit, "floor_us": floors[unit], "frac_of_binding_unit": floors[unit] / us,
                          "floors_us": floors},
             "l2": "inputs larger than L2"}
        tr = profile_traffic(f"vector_{name}_2^26_f64")
        e["roofline"]["traffic"] = None if tr is None else tr[0]
        if tr is not None:
            e["roofline"]["traffic_source"] = tr[1]
        if cpu_fn is not None:
            import math
            launch()
            torch.cuda.synchronize(dev)
            got = gpu_val()
            want = cpu_fn()
            terms = x_np if name == "reduce" else x_np * (y_np if name == "dot_xy" else x_np)
            exact = math.fsum(terms)  # correctly rounded sum of the (rounded) terms
            scale = float(np.sum(np.abs(terms)))
            # errors relative to sum |terms|, against the correctly rounded sum:
            # the GPU's and the oracle's (the Serial restatement, one long
            # recursive sum)
            e["rel_err_vs_fsum"] = abs(got - exact) / scale
            e["oracle_rel_err_vs_fsum"] = abs(want - exact) / scale
            if cpu_budget > 0:
                cu = cpu_us(cpu_fn)
                e["cpu_baseline"] = {"value": nbytes / (cu * 1e-6) / 1e9, "unit": "GB/s", "cores": 1, "kind": "port",
                                     "sample": "full vectors, Serial restatement in oracle/oracle.cpp"}
        else:
            w_ref = np.empty(n)
            a, b = (2.15, -3.2) if name == "waxpby_alpha_beta" else (2.15, 1.0)
            O.waxpby(n, a, x_np, b, y_np, w_ref)
            e["max_abs_err_vs_oracle"] = float(np.max(np.abs(w.cpu().numpy() - w_ref)))
        res.append(e)
    del x, y, w
    return res


def batched_entry(args, dev, stream, unit_peaks, cpu_budget) -> dict:
    """C5: 4,096 CSR matrices, one autotuned persistent launch replayed as a
    CUDA graph, every matrix checked against the oracle; baselines: the same
    multiplies as 4,096 separate library calls, and the reference's OpenMP
    / Serial multiply per matrix on the host."""
    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import batched
    from morpheus_gb300 import generators as gen
    from oracle import oracle as O
    mats = gen.batched_csr(4096, seed=0)
    nbytes = sum(algorithmic_bytes(m, 8) for m in mats)
    dmats = [mgb.matrix_from_host(m, device=dev) for m in mats]
    xs_np = [gen.x_vector(m["ncols"], seed=1 + i) for i, m in enumerate(mats)]
    xs = [torch.from_numpy(v).to(dev) for v in xs_np]
    ys = [torch.zeros(m["nrows"], dtype=torch.float64, device=dev) for m in mats]
    b = batched.CsrBatch(dmats, xs, ys)
    best, tune_ms = b.autotune(reps=3, use_cache=False)
    g = b.capture_graph(init=True)
    g.replay()
    torch.cuda.synchronize()
    oms = [O.OracleMatrix.from_host(m) for m in mats]
    got = [y.cpu().numpy() for y in ys]
    errs = []
    for om, xv, yv in zip(oms, xs_np, got):
        ref = om.multiply(xv)
        den = np.linalg.norm(ref)
        errs.append(float(np.linalg.norm(yv - ref) / den) if den > 0 else float(np.linalg.norm(yv)))
    for _ in range(max(3, args.warmup)):
        g.replay()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        g.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    for A, x, y in zip(dmats, xs, ys):
        mgb.multiply(A, x, y)
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for A, x, y in zip(dmats, xs, ys):
        mgb.multiply(A, x, y)
    s1.record(stream)
    torch.cuda.synchronize()
    sep_ms = s0.elapsed_time(s1)
    nnz = int(sum(m["nnz"] for m in mats))
    fake = {"format": 1, "nrows": sum(m["nrows"] for m in mats), "ncols": sum(m["ncols"] for m in mats),
            "nnz": nnz}
    rl = roofline(fake, 8, ms * 1e3, unit_peaks, "scattered", profile_traffic("c5_batched_4096_csr_f64"),
                  nbytes=nbytes)
    out = {"config": "c5_batched_4096_csr_f64", "format": "CSR (batched)", "dtype": "f64", "matrices": len(mats),
           "nnz": nnz, "us_per_batch": ms * 1e3, "GB/s": nbytes / (ms * 1e-3) / 1e9,
           "rel_err_vs_oracle": max(errs), "rel_err_bar": 1e-12, "matrices_checked": len(errs),
           "autotuned_config": best, "config_info": batched.config_info(best), "autotune_ms_per_config": tune_ms,
           "roofline": rl,
           "separate_calls": {"ms": sep_ms, "speedup_of_batched": sep_ms / ms,
                              "note": "4,096 morpheus_gb300.multiply calls (Python call overhead included)"}}
    if cpu_budget > 0:
        threads = O.max_threads()
        res = {}
        for label, th in (("openmp", threads), ("serial", 0)):
            t0 = time.perf_counter()
            done = 0
            k = 0
            while k < len(mats) and time.perf_counter() - t0 < cpu_budget:
                oms[k].multiply(xs_np[k], threads=th)
                done += algorithmic_bytes(mats[k], 8)
                k += 1
            res[label] = (done / (time.perf_counter() - t0) / 1e9, k)
        out["cpu_baseline"] = {"value": res["openmp"][0], "unit": "GB/s", "cores": threads, "kind": "port",
                               "sample": f"one OpenMP multiply per matrix, first {res['openmp'][1]} matrices",
                               "serial_1_core": {"value": res["serial"][0], "unit": "GB/s", "cores": 1,
                                                 "sample": f"first {res['serial'][1]} matrices"}}
    del g, b
    return out


def convert_entry(dev, cpu_budget: float) -> dict:
    """GPU conversions through the public API (to_coo / from_coo, each with
    its size plan and validation) at the benchmark sizes, against the
    reference's Serial convert (oracle restatement) of the same pair on one
    host core.  GB/s = (source + destination bytes) / time."""
    import torch

    import morpheus_gb300 as mgb
    from morpheus_gb300 import generators as gen
    from oracle import oracle as O

    def mat_bytes(hm):
        return sum(a.nbytes for _, a in host_arrays(hm))

    def gpu_ms(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            fn()
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        return best * 1e3

    S = build_csr("stencil27", np.float64, seed=0)
    P = build_csr("power_law", np.float64, seed=0)
    p90 = int(np.percentile(np.diff(P["row_offsets"]), 90))
    H = gen.add_offband(S, 0.01, seed=1)
    out = []
    cases = [("c3_stencil27_160", S, "coo", None), ("c3_stencil27_160", S, "dia", None),
             ("c3_stencil27_160_offband", H, "hdc", None), ("c2_power_law_2e6", P, "hyb", p90),
             ("c2_power_law_2e6", P, "csr", None)]
    for name, A, fmt, width in cases:
        dA = mgb.matrix_from_host(A, device=dev)
        coo = mgb.to_coo(dA)
        f = FORMAT_NAMES.index(fmt)
        if fmt == "coo":
            run = lambda: mgb.to_coo(dA)
            src_hm, label = A, "CSR -> COO"
        else:
            run = lambda: mgb.from_coo(coo, f, hyb_width=width or 0)
            src_hm, label = mgb.matrix_to_host(coo), f"COO -> {fmt.upper()}"
        res = run()
        dst_hm = mgb.matrix_to_host(res)
        nbytes = mat_bytes(src_hm) + mat_bytes(dst_hm)
        ms = gpu_ms(run)
        e = {"config": f"convert_{name}_{'csr_to_coo' if fmt == 'coo' else 'coo_to_' + fmt}", "pair": label,
             "nnz": int(A["nnz"]), "ms": ms, "GB/s": nbytes / (ms * 1e-3) / 1e9, "bytes": nbytes,
             "timing": "wall clock around the public call (plan, validation and conversion kernels), best of 3"}
        if width:
            e["hyb_ell_width"] = width
        if cpu_budget > 0:
            om = O.OracleMatrix.from_host(src_hm)
            t0 = time.perf_counter()
            if fmt == "hyb":
                om.coo_to_hyb(width)
            else:
                om.convert(f)
            el = time.perf_counter() - t0
            e["cpu_serial"] = {"ms": el * 1e3, "GB/s": nbytes / el / 1e9, "cores": 1, "kind": "port",
                               "sample": "one Serial convert of the same pair (oracle/oracle.cpp)",
                               "speedup_of_gpu": el * 1e3 / ms}
        out.append(e)
        del dA, coo, res
        torch.cuda.empty_cache()
    return {"config": "convert", "pairs": out}


def selector_entry(n_test: int) -> dict:
    """C4: the committed selector on held-out corpus matrices (seeds from
    1,000,000, never trained on), every format timed here on the GPU."""
    from morpheus_gb300 import corpus, selector
    t0 = time.time()
    te = corpus.build(n_test, seed0=1_000_000)
    sel = selector.default_selector()
    pred = sel.predict(te["X"], te["feasible"])
    ev = selector.evaluate(te["times"], pred)
    names = ["COO", "CSR", "DIA", "ELL", "HYB", "HDC"]
    labels = np.argmin(te["times"], axis=1)
    return {"config": "c4_selector_heldout", "matrices": n_test, "nnz_cap": corpus.NNZ_CAP,
            "max_nnz": int(max(d["nnz"] for d in te["desc"])),
            "learned": ev,
            "label_counts": {names[k]: int((labels == k).sum()) for k in range(6) if (labels == k).any()},
            "seconds": time.time() - t0,
            "targets": {"mean_regret": "<= 0.10", "geomean_speedup_vs_csr": ">= 1.5"}}


# --------------------------------------------------------------------------
# reference arm
# --------------------------------------------------------------------------

def run_reference(args, rank: int):
    if rank != 0:
        return
    from morpheus_gb300 import generators as gen
    from oracle import oracle as O
    from oracle.build import build_oracle
    build_oracle()
    threads = O.max_threads()
    if args.workload == "suite":
        S = build_csr("stencil27", np.float64, seed=0, size=args.size)
        hm = gen.csr_to_dia_host(S) if HEADLINE_FORMAT == "dia" else S
        nbytes = algorithmic_bytes(hm, 8)
        x = gen.x_vector(S["ncols"], seed=0)
        om = O.OracleMatrix.from_host(hm)
        y = np.zeros(S["nrows"])
        cfg = headline_config(S, HEADLINE_FORMAT, args.gpus)

        def step():
            om.multiply(x, y, init=True, threads=threads)
        sample_desc = f"full matrix in {HEADLINE_FORMAT.upper()}, {args.steps} timed multiplies"
        dtype_name = "f64"
    elif args.workload == "batched":
        dtype = np.float64 if args.dtype == "f64" else np.float32
        mats = gen.batched_csr(args.batch, seed=0, dtype=dtype)
        sample = mats[: min(len(mats), 256)]  # bounded sample per step
        oms = [O.OracleMatrix.from_host(m) for m in sample]
        xs = [np.random.default_rng(1 + i).uniform(-1, 1, m["ncols"]).astype(dtype) for i, m in enumerate(sample)]
        ysb = [np.zeros(m["nrows"], dtype=dtype) for m in sample]
        nbytes = sum(algorithmic_bytes(m, np.dtype(dtype).itemsize) for m in sample)

        def step():
            for om, xv, yv in zip(oms, xs, ysb):
                om.multiply(xv, yv, init=True, threads=threads)
        hm = {"nrows": sum(m["nrows"] for m in mats), "ncols": sum(m["ncols"] for m in mats),
              "nnz": sum(m["nnz"] for m in mats)}
        cfg = config_dict(args, hm)
        sample_desc = f"first {len(sample)} of {len(mats)} matrices per step, one OpenMP multiply each"
        dtype_name = args.dtype
    else:
        dtype = np.float64 if args.dtype == "f64" else np.float32
        A, hm = build_workload(args.workload, args.format, dtype, seed=0, size=args.size)
        nbytes = algorithmic_bytes(hm, np.dtype(dtype).itemsize)
        x = np.random.default_rng(1).uniform(-1, 1, hm["ncols"]).astype(dtype)
        om = O.OracleMatrix.from_host(hm)
        y = np.zeros(hm["nrows"], dtype=dtype)

        def step():
            om.multiply(x, y, init=True, threads=threads)
        cfg = config_dict(args, hm)
        sample_desc = f"full matrix, {args.steps} timed multiplies"
        dtype_name = args.dtype
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
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype_name,
        "data": "synthetic (seeded)", "config": cfg,
        "cpu_baseline": {"value": gbs, "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"{sample_desc} (reference OpenMP algorithm restated in oracle/oracle.cpp)"},
        "e2e": {"value": gbs, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


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
# single-configuration GPU arm (profiling commands)
# --------------------------------------------------------------------------

def run_gpu(args, rank: int, world: int, local_rank: int):
    import torch

    import morpheus_gb300 as mgb

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

    check_err = None
    om = None
    if rank == 0 and not args.skip_check:
        from oracle import oracle as O
        from oracle.build import build_oracle
        build_oracle()
        om = O.OracleMatrix.from_host(hm)
        mgb.multiply(M, x, y, init=True)
        torch.cuda.synchronize()
        check_err = oracle_error(om, dtype, x_np, y.cpu().numpy())

    for _ in range(args.warmup):
        mgb.multiply(M, x, y, init=True)
    torch.cuda.synchronize()
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    sampler = ClockSampler(local_rank)
    sampler.start()
    time.sleep(0.3)
    ms = time_multiply(M, x, y, args.steps, 0, stream, flush) * args.steps
    clocks = sampler.stop()
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    kernel_ms = ms / args.steps
    value = world * nbytes * args.steps / (ms * 1e-3) / 1e9

    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_api = "pinned host arrays -> device containers (torch copies), morpheus_gb300.multiply, y -> host"
    if args.format == "csr":
        # the library's host-data entry point: pipelined block copies + kernels
        host_csr = mgb.matrix_from_host(hm, device="cpu", dtype=tdtype)
        host_csr._ro, host_csr._ci, host_csr._v = (host_csr._ro.pin_memory(), host_csr._ci.pin_memory(),
                                                   host_csr._v.pin_memory())
        xh = torch.from_numpy(x_np).pin_memory()
        yh = torch.empty(hm["nrows"], dtype=tdtype).pin_memory()
        mgb.multiply_host(host_csr, xh, yh, init=True)  # warm-up (workspace, kernel choice)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(e2e_steps):
            mgb.multiply_host(host_csr, xh, yh, init=True)
        e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1) / e2e_steps
        h2d = sum(a.nbytes for _, a in host_arrays(hm)) + xh.numel() * xh.element_size()
        d2h = yh.numel() * yh.element_size()
        e2e_api = "multiply_host (mgb_spmv_csr_host, pipelined row blocks)"
    else:
        e2e_ms, h2d, d2h = e2e_multiply(M, hm, x_np, y, stream, e2e_steps, dev)
    e2e_val = world * nbytes / (e2e_ms * 1e-3) / 1e9

    if rank != 0:
        return
    unit_peaks = measure_unit_peaks(dev)
    x_access = "scattered" if args.workload in ("power_law", "uniform") else "banded"
    key = f"{args.workload}_{args.format}_{args.dtype}" + (f"_size{args.size}" if args.size else "")
    rl = roofline(hm, vbytes, kernel_ms * 1e3, unit_peaks, x_access, profile_traffic(key))
    line = {
        "metric": METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kernel_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (seeded power-law / stencil generators, N(0,1) values)",
        "config": config_dict(args, hm),
        "pct_hbm_peak": 100.0 * rl["frac"],
        "rel_err_vs_oracle": check_err,
        "roofline": rl, "unit_peaks": unit_peaks,
        "e2e": {"value": e2e_val, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_ms, "api": e2e_api},
        "gflops": 2.0 * hm["nnz"] / (kernel_ms * 1e-3) / 1e9 if hm.get("nnz") else None,
        "gpu_launches": args.steps * launches_per_step(hm),
        "clocks": clocks,
    }
    if args.format == "csr":
        line["csr_kernel"] = CSR_KERNEL_NAMES.get(M.kernel_variant())
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        om = om or O.OracleMatrix.from_host(hm)
        line["cpu_baseline"] = cpu_baselines(om, x_np, nbytes, args.cpu_budget)
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
    """4,096 independent CSR SpMVs per step in one autotuned (or fixed)
    persistent launch, replayed as a CUDA graph (profiling commands)."""
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
    xs = [torch.from_numpy(np.random.default_rng(1 + i).uniform(-1, 1, m["ncols"]).astype(dtype)).to(dev)
          for i, m in enumerate(mats)]
    ys = [torch.zeros(m["nrows"], dtype=dmats[0].dtype, device=dev) for m in mats]
    b = batched.CsrBatch(dmats, xs, ys)
    if args.batched_config is None:
        best, tune_ms = b.autotune(reps=3, use_cache=False)
    else:  # a fixed configuration (profiling comparisons): no autotuning launches
        best, tune_ms = args.batched_config, None
        b.plan(best)
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
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    if rank != 0:
        return
    kernel_ms = ms / args.steps
    peak, _ = peaks()
    achieved = nbytes / (kernel_ms * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": world * nbytes * args.steps / (ms * 1e-3) / 1e9, "unit": "GB/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": kernel_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": args.dtype,
        "data": "synthetic (seeded batched CSR generator)",
        "config": {"workload": f"batched_csr_{args.batch}_{args.dtype}", "matrices": len(mats),
                   ("autotuned_config" if tune_ms is not None else "fixed_config"): best,
                   "config_chunk_seg": batched.config_info(best)},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "algorithmic_bytes_per_launch": nbytes},
        "gpu_launches": args.steps, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_gpu_convert(args, rank: int, world: int, local_rank: int):
    """One conversion, repeated: CSR -> COO -> --format of the --workload
    matrix (profiling commands; the suite reports every pair at full size)."""
    import torch

    import morpheus_gb300 as mgb
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    dtype = np.float64 if args.dtype == "f64" else np.float32
    A = build_csr(args.workload_matrix, dtype, seed=rank, size=args.size)
    dA = mgb.matrix_from_host(A, device=dev)
    fmt = FORMAT_NAMES.index(args.format)
    p90 = int(np.percentile(np.diff(A["row_offsets"]), 90))
    width = p90 if args.format == "hyb" and args.workload_matrix == "power_law" else 0

    def step():
        coo = mgb.to_coo(dA)
        return coo if fmt == 0 else mgb.from_coo(coo, fmt, hyb_width=width)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        out = step()
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / args.steps
    if rank == 0:
        print(json.dumps({"workload": f"convert_{args.workload_matrix}_csr_to_{args.format}", "ms_per_step": ms,
                          "nnz": int(A["nnz"]), "steps": args.steps, "out_nnz": out.nnnz()}), flush=True)


def run_peaks(args, local_rank: int):
    import torch
    torch.cuda.set_device(local_rank)
    p = measure_unit_peaks(torch.device("cuda", local_rank))
    print(json.dumps({"workload": "peaks", **p}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mgb", choices=["mgb", "reference"])
    ap.add_argument("--workload", default="suite",
                    choices=["suite", "peaks", "power_law", "stencil27", "laplacian", "uniform", "batched", "cg",
                             "convert"])
    ap.add_argument("--workload-matrix", default="stencil27", choices=["stencil27", "power_law", "laplacian"],
                    help="convert workload: the matrix converted")
    ap.add_argument("--csr-kernel", default="auto", choices=sorted(CSR_KERNELS),
                    help="force one CSR kernel instead of the per-matrix choice (profiling)")
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--batched-config", type=int, default=None,
                    help="batched workload: use this configuration instead of autotuning (profiling)")
    ap.add_argument("--size", type=int, default=None,
                    help="power-law rows / stencil or Laplacian grid edge (default: the benchmark size)")
    ap.add_argument("--format", default="csr", choices=FORMAT_NAMES)
    ap.add_argument("--dtype", default="f64", choices=["f64", "f32"])
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-budget", type=float, default=5.0, help="seconds per CPU baseline of the headline")
    ap.add_argument("--cfg-cpu-budget", type=float, default=1.0, help="seconds per CPU baseline of a per-config entry")
    ap.add_argument("--selector-test", type=int, default=400, help="held-out corpus matrices for the C4 entry")
    ap.add_argument("--headline-only", action="store_true", help="suite: skip the per-config entries")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--skip-check", action="store_true")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "peaks":
        if rank == 0:
            run_peaks(args, local_rank)
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    try:
        if args.workload == "suite":
            run_suite(args, rank, world, local_rank)
        elif args.workload == "batched":
            run_gpu_batched(args, rank, world, local_rank)
        elif args.workload == "cg":
            run_gpu_cg(args, rank, world, local_rank)
        elif args.workload == "convert":
            run_gpu_convert(args, rank, world, local_rank)
        else:
            run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
