"""Batched CSR SpMV: many independent y_i = A_i x_i in one persistent launch.

    batch = CsrBatch(matrices, xs, ys)        # device CsrMatrix list + vectors
    batch.autotune()                          # project autotuner (CUDA events)
    batch.multiply()                          # memset + one persistent kernel
    g = batch.capture_graph(); g.replay()     # the same launch as a CUDA graph

The reference has no batched path: its equivalent is one Morpheus::multiply
call per matrix.  Autotune results are cached per batch shape class
(value type, number of matrices, log2 mean rows, log2 mean row length).
"""
from __future__ import annotations

import ctypes as C
import math

import torch

from . import _lib
from .algorithms import _stream_handle, _suffix
from .containers import CsrMatrix
from .exceptions import InvalidInputException

_TUNE_CACHE: dict[tuple, int] = {}


def num_configs() -> int:
    return _lib.load().mgb_spmv_batched_csr_num_configs()


def config_info(cfg: int) -> tuple[int, int]:
    ch, sg = C.c_int64(), C.c_int()
    _lib.call("mgb_spmv_batched_csr_config_info", int(cfg), C.byref(ch), C.byref(sg))
    return ch.value, sg.value


class CsrBatch:
    def __init__(self, matrices: list[CsrMatrix], xs: list[torch.Tensor], ys: list[torch.Tensor]):
        if not matrices or len(matrices) != len(xs) or len(xs) != len(ys):
            raise InvalidInputException("CsrBatch needs equally many matrices, xs and ys")
        dt = matrices[0].dtype
        dev = matrices[0].device
        for A, x, y in zip(matrices, xs, ys):
            if A.dtype != dt or x.dtype != dt or y.dtype != dt:
                raise InvalidInputException("CsrBatch: one value type for all items")
            if A.device.type != "cuda" or x.device.type != "cuda" or y.device.type != "cuda":
                raise InvalidInputException("CsrBatch: device containers only")
            if x.numel() < A.ncols() or y.numel() < A.nrows():
                raise InvalidInputException("CsrBatch: vector too short")
        self.matrices, self.xs, self.ys = matrices, xs, ys
        self.dtype, self.device = dt, dev
        n = len(matrices)
        items = (_lib.BatchItem * n)()
        for i, (A, x, y) in enumerate(zip(matrices, xs, ys)):
            items[i] = _lib.BatchItem(A.nrows(), A.ncols(), A.nnnz(), A.row_offsets().data_ptr(),
                                      A.column_indices().data_ptr(), A.values().data_ptr(),
                                      x.data_ptr(), y.data_ptr())
        raw = torch.frombuffer(bytearray(bytes(items)), dtype=torch.uint8)
        self._items = raw.to(dev)
        nb = C.c_int64()
        _lib.call("mgb_spmv_batched_csr_workspace_bytes", n, C.byref(nb))
        self._ws = torch.zeros(nb.value, dtype=torch.uint8, device=dev)
        self.nitems = n
        self.config = None

    def key(self) -> tuple:
        rows = sum(A.nrows() for A in self.matrices) / self.nitems
        nnz = sum(A.nnnz() for A in self.matrices)
        mean_len = nnz / max(1, sum(A.nrows() for A in self.matrices))
        return (str(self.dtype), int(math.log2(self.nitems + 1)), int(math.log2(rows + 1)),
                int(math.log2(mean_len + 1)))

    def plan(self, config: int, stream=None) -> None:
        _lib.call("mgb_spmv_batched_csr_plan", C.c_void_p(self._items.data_ptr()), self.nitems, int(config),
                  C.c_void_p(self._ws.data_ptr()), self._ws.numel(), _stream_handle(stream))
        self.config = int(config)

    def autotune(self, reps: int = 5, stream=None, use_cache: bool = True) -> tuple[int, list[float]]:
        k = self.key()
        if use_cache and k in _TUNE_CACHE:
            self.plan(_TUNE_CACHE[k], stream)
            return self.config, []
        nc = num_configs()
        ms = (C.c_float * nc)()
        best = C.c_int()
        _lib.call(f"mgb_spmv_batched_csr_autotune_{_suffix(self.dtype)}", C.c_void_p(self._items.data_ptr()),
                  self.nitems, C.c_void_p(self._ws.data_ptr()), self._ws.numel(), int(reps), C.byref(best), ms,
                  _stream_handle(stream))
        self.config = best.value
        _TUNE_CACHE[k] = best.value
        return best.value, list(ms)

    def multiply(self, init: bool = True, stream=None) -> None:
        if self.config is None:
            self.plan(2, stream)
        _lib.call(f"mgb_spmv_batched_csr_{_suffix(self.dtype)}", C.c_void_p(self._items.data_ptr()), self.nitems,
                  self.config, C.c_void_p(self._ws.data_ptr()), 1 if init else 0, _stream_handle(stream))

    def planned_ok(self) -> bool:
        """False if the last launch found the workspace planned for another
        config (or for none: a chunk total beyond 2^31 - 1), or skipped an
        item too large for 32-bit indices (nnz >= 2^31 - 4096)."""
        return int(self._ws[12:16].view(torch.int32).item()) == 0

    def capture_graph(self, init: bool = True) -> torch.cuda.CUDAGraph:
        """The batched launch (two memsets + kernel) captured as a CUDA graph."""
        if self.config is None:
            self.plan(2)
        s = torch.cuda.Stream(device=self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.multiply(init, stream=s)  # warm the launch outside capture
        torch.cuda.current_stream(self.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            self.multiply(init, stream=s)
        return g
