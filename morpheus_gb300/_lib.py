"""ctypes binding of libmorpheus_gb300.so (the C ABI declared in include/mgb.h).

The library is built in-tree by morpheus_gb300.build.  There is no CPU
fallback: if the shared object is missing or cannot be loaded, every compute
call raises instead of silently running elsewhere.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from .exceptions import raise_for_status

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmorpheus_gb300.so")

_lock = threading.Lock()
_lib = None

i64 = C.c_int64
i32p = C.POINTER(C.c_int32)
vp = C.c_void_p


class Coo(C.Structure):
    _fields_ = [("nrows", i64), ("ncols", i64), ("nnz", i64),
                ("row_indices", vp), ("column_indices", vp), ("values", vp)]


class Csr(C.Structure):
    _fields_ = [("nrows", i64), ("ncols", i64), ("nnz", i64),
                ("row_offsets", vp), ("column_indices", vp), ("values", vp)]


class Dia(C.Structure):
    _fields_ = [("nrows", i64), ("ncols", i64), ("nnz", i64), ("ndiags", i64), ("pitch", i64),
                ("diagonal_offsets", vp), ("values", vp)]


class Ell(C.Structure):
    _fields_ = [("nrows", i64), ("ncols", i64), ("nnz", i64), ("entries_per_row", i64),
                ("width", i64), ("pitch", i64), ("column_indices", vp), ("values", vp)]


class BatchItem(C.Structure):
    _fields_ = [("nrows", i64), ("ncols", i64), ("nnz", i64), ("row_offsets", vp), ("column_indices", vp),
                ("values", vp), ("x", vp), ("y", vp)]


class Hyb(C.Structure):
    _fields_ = [("ell", Ell), ("coo", Coo)]


class Hdc(C.Structure):
    _fields_ = [("dia", Dia), ("csr", Csr)]


# name -> (restype, argtypes)
_SIGS: dict[str, tuple] = {
    "mgb_status_string": (C.c_char_p, [C.c_int]),
    "mgb_version": (C.c_int, []),
    "mgb_last_cuda_error_string": (C.c_char_p, []),
}
for _fmt, _st in (("csr", Csr), ("coo", Coo), ("dia", Dia), ("ell", Ell), ("hyb", Hyb), ("hdc", Hdc)):
    for _dt in ("f64", "f32"):
        _SIGS[f"mgb_spmv_{_fmt}_{_dt}"] = (C.c_int, [C.POINTER(_st), vp, vp, C.c_int, vp])
for _dt, _ct in (("f64", C.c_double), ("f32", C.c_float)):
    _SIGS[f"mgb_dot_{_dt}"] = (C.c_int, [i64, vp, vp, C.POINTER(_ct), vp])
    _SIGS[f"mgb_dot_{_dt}_async"] = (C.c_int, [i64, vp, vp, vp, vp])
    _SIGS[f"mgb_reduce_{_dt}"] = (C.c_int, [vp, i64, C.POINTER(_ct), vp])
    _SIGS[f"mgb_reduce_{_dt}_async"] = (C.c_int, [vp, i64, vp, vp])
    _SIGS[f"mgb_waxpby_{_dt}"] = (C.c_int, [i64, _ct, vp, _ct, vp, vp, vp])
_SIGS["mgb_csr_choose_kernel"] = (C.c_int, [C.POINTER(Csr), C.POINTER(C.c_int), vp])
for _dt in ("f64", "f32"):
    _SIGS[f"mgb_spmv_csr_variant_{_dt}"] = (C.c_int, [C.POINTER(Csr), vp, vp, C.c_int, C.c_int, vp])
    _SIGS[f"mgb_spmv_csr_planned_{_dt}"] = (C.c_int, [C.POINTER(Csr), vp, i64, vp, vp, C.c_int, vp])
_SIGS["mgb_csr_plan_entries"] = (C.c_int, [C.POINTER(Csr), C.POINTER(i64)])
_SIGS["mgb_csr_plan"] = (C.c_int, [C.POINTER(Csr), vp, i64, vp])
_SIGS["mgb_analytics_csr"] = (C.c_int, [C.POINTER(Csr), C.POINTER(C.c_double), vp])
_SIGS["mgb_count_nnz_per_row_csr"] = (C.c_int, [C.POINTER(Csr), vp, C.c_int, vp])
_SIGS["mgb_count_nnz_per_row_coo"] = (C.c_int, [C.POINTER(Coo), vp, C.c_int, vp])
_SIGS["mgb_count_nnz_per_diagonal_csr"] = (C.c_int, [C.POINTER(Csr), vp, C.c_int, vp])
_SIGS["mgb_count_nnz_per_diagonal_coo"] = (C.c_int, [C.POINTER(Coo), vp, C.c_int, vp])
_SIGS["mgb_count_nnz_vector"] = (C.c_int, [vp, i64, C.c_int32, C.POINTER(i64), vp])
_SIGS["mgb_features_csr"] = (C.c_int, [C.POINTER(Csr), C.POINTER(C.c_float), C.POINTER(C.c_uint8), vp])
for _fmt, _st in (("dia", Dia), ("ell", Ell), ("hyb", Hyb), ("hdc", Hdc)):
    _SIGS[f"mgb_count_nnz_per_row_{_fmt}"] = (C.c_int, [C.POINTER(_st), vp, C.c_int, vp])
    for _dt in ("f64", "f32"):
        _SIGS[f"mgb_count_nnz_per_diagonal_{_fmt}_{_dt}"] = (C.c_int, [C.POINTER(_st), vp, C.c_int, vp])
for _name, _st in (("coo", Coo), ("dia_f64", Dia), ("dia_f32", Dia), ("ell", Ell), ("hyb", Hyb),
                   ("hdc_f64", Hdc), ("hdc_f32", Hdc)):
    _SIGS[f"mgb_analytics_{_name}"] = (C.c_int, [C.POINTER(_st), C.POINTER(C.c_double), vp])
    _SIGS[f"mgb_features_{_name}"] = (C.c_int, [C.POINTER(_st), C.POINTER(C.c_float), C.POINTER(C.c_uint8), vp])
_SIGS["mgb_mlp_num_params"] = (C.c_int, [])
_SIGS["mgb_mlp_forward_f32"] = (C.c_int, [vp, vp, vp, vp, vp, i64, vp, vp])
_SIGS["mgb_mlp_grad_f32"] = (C.c_int, [vp, vp, vp, vp, vp, vp, i64, vp, vp, vp])
_SIGS["mgb_mlp_adam_f32"] = (C.c_int, [vp, vp, vp, vp, i64, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int,
                                       vp])
_SIGS["mgb_spmv_batched_csr_num_configs"] = (C.c_int, [])
_SIGS["mgb_spmv_batched_csr_config_info"] = (C.c_int, [C.c_int, C.POINTER(i64), C.POINTER(C.c_int)])
_SIGS["mgb_spmv_batched_csr_workspace_bytes"] = (C.c_int, [i64, C.POINTER(i64)])
_SIGS["mgb_spmv_batched_csr_plan"] = (C.c_int, [vp, i64, C.c_int, vp, i64, vp])
for _dt in ("f64", "f32"):
    _SIGS[f"mgb_spmv_batched_csr_{_dt}"] = (C.c_int, [vp, i64, C.c_int, vp, C.c_int, vp])
    _SIGS[f"mgb_spmv_batched_csr_autotune_{_dt}"] = (C.c_int, [vp, i64, vp, i64, C.c_int, C.POINTER(C.c_int),
                                                               C.POINTER(C.c_float), vp])
for _dt, _ct in (("f64", C.c_double), ("f32", C.c_float)):
    _SIGS[f"mgb_spmv_dot_csr_{_dt}"] = (C.c_int, [C.POINTER(Csr), vp, vp, C.c_int, C.c_int, vp, vp])
    _SIGS[f"mgb_waxpby_dot_{_dt}"] = (C.c_int, [i64, _ct, vp, _ct, vp, vp, vp, vp])
    _SIGS[f"mgb_cg_csr_{_dt}"] = (C.c_int, [C.POINTER(Csr), C.c_int, vp, vp, i64, C.c_double, C.POINTER(i64),
                                            C.POINTER(C.c_double), vp])
for _dt in ("f64", "f32"):
    _SIGS[f"mgb_spmv_csr_host_{_dt}"] = (C.c_int, [C.POINTER(Csr), vp, vp, C.c_int, C.c_int, i64, vp, i64, vp])
_SIGS["mgb_spmv_csr_host_workspace_bytes"] = (C.c_int, [C.POINTER(Csr), C.c_int, C.POINTER(i64)])
_SIGS["mgb_spmv_coo_f64_noalloc"] = (C.c_int, [C.POINTER(Coo), vp, vp, C.c_int, vp])
_P = C.POINTER
for _name, _s, _d in (("csr_to_coo", Csr, Coo), ("coo_to_csr", Coo, Csr), ("dia_to_coo", Dia, Coo),
                      ("coo_to_dia", Coo, Dia), ("ell_to_coo", Ell, Coo), ("coo_to_ell", Coo, Ell),
                      ("hyb_to_coo", Hyb, Coo), ("coo_to_hyb", Coo, Hyb), ("hdc_to_coo", Hdc, Coo),
                      ("coo_to_hdc", Coo, Hdc)):
    for _dt in ("f64", "f32"):
        _SIGS[f"mgb_convert_{_name}_{_dt}"] = (C.c_int, [_P(_s), _P(_d), vp])
_SIGS["mgb_convert_coo_to_dia_plan"] = (C.c_int, [_P(Coo), _P(i64), vp])
_SIGS["mgb_convert_coo_to_ell_plan"] = (C.c_int, [_P(Coo), _P(i64), vp])
_SIGS["mgb_convert_coo_to_hyb_plan"] = (C.c_int, [_P(Coo), i64, _P(i64), _P(i64), _P(i64), vp])
_SIGS["mgb_convert_coo_to_hdc_plan"] = (C.c_int, [_P(Coo), _P(i64), _P(i64), _P(i64), vp])
for _dt in ("f64", "f32"):
    _SIGS[f"mgb_coo_sort_by_row_and_column_{_dt}"] = (C.c_int, [_P(Coo), vp])
_SIGS["mgb_coo_is_sorted"] = (C.c_int, [_P(Coo), _P(C.c_int), vp])
_SIGS["mgb_peak_dfma_f64"] = (C.c_int, [i64, i64, vp, vp])
_SIGS["mgb_peak_gather_f64"] = (C.c_int, [vp, i64, i64, i64, vp, vp])
_SIGS["mgb_peak_threads_per_block"] = (C.c_int, [])


def load(path: str | None = None):
    """Load (once) and return the CDLL with prototypes attached."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise ImportError(
                f"{p} is missing: build it with `python -m morpheus_gb300.build` "
                "(there is no CPU fallback)")
        lib = C.CDLL(p)
        for name, (res, args) in _SIGS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def call(name: str, *args) -> None:
    """Call an mgb_* entry point and raise the mapped exception on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        raise_for_status(st, name, lib.mgb_last_cuda_error_string().decode())


def declared_symbols() -> list[str]:
    return sorted(_SIGS)
