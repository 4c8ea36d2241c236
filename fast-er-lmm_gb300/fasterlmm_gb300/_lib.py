"""
ctypes binding of the C ABI in include/fasterlmm_gb300.h.

The library is loaded once per process.  There is no fallback: if ``libfasterlmm_gb300.so`` has not been built,
every call raises.  Status codes other than FLMM_OK raise :class:`FlmmError` carrying the library's message.
ctypes releases the GIL for the duration of each call.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libfasterlmm_gb300.so"

_i, _i64, _d, _p, _sz, _s = C.c_int, C.c_int64, C.c_double, C.c_void_p, C.c_size_t, C.c_char_p
_pi32 = C.POINTER(C.c_int32)
_psz = C.POINTER(C.c_size_t)

# name -> argument types (all return int status unless listed in _RESTYPE)
SIGNATURES: dict[str, list] = {
    "flmm_version": [],
    "flmm_status_string": [_i],
    "flmm_last_error": [],
    "flmm_kernel_launches": [],
    "flmm_context_create": [_i, C.POINTER(_p)],
    "flmm_context_destroy": [_p],
    "flmm_standardise_f64": [_p, _i64, _i, _i, _p, _i64, _p],
    "flmm_standardise_dosage": [_p, _i64, _i, _i, _p, _i64, _p],
    "flmm_transpose_f64": [_p, _i64, _i, _i, _p, _i64, _p],
    "flmm_gram_f64": [_p, _i64, _i, _i, _d, _p, _i64, _p],
    "flmm_loco_kinship": [_p, _p, _i64, _i, _d, _p, _p],
    "flmm_covariate_basis_workspace_bytes": [_p, _i, _i, _psz],
    "flmm_covariate_basis": [_p, _p, _i, _i, _p, _p, _p, _p, _sz, _p],
    "flmm_project_kinship_workspace_bytes": [_i, _i, _psz],
    "flmm_project_kinship": [_p, _i64, _p, _i, _i, _p, _i64, _p, _sz, _p],
    "flmm_eigh_workspace_bytes": [_p, _i, _psz],
    "flmm_eigh": [_p, _p, _i, _p, _p, _sz, _p],
    "flmm_eigh_batched_workspace_bytes": [_p, _i, _i, _i, _psz],
    "flmm_eigh_batched": [_p, _p, _i, _i, _p, _i, _i, _p, _sz, _p],
    "flmm_eigh_batched_f32_workspace_bytes": [_p, _i, _i, _psz],
    "flmm_eigh_batched_f32": [_p, _p, _i, _i, _p, _p, _sz, _p],
    "flmm_eigh_refine_workspace_bytes": [_i, _i, _psz],
    "flmm_eigh_refine_f32": [_p, _p, _p, _p, _i, _i, _p, _sz, _p],
    "flmm_refine_product_workspace_bytes": [_i, _i, _psz],
    "flmm_refine_product": [_p, _p, _i, _i, _i, _p, _p, _p, _sz, _p],
    "flmm_compat_spectrum": [_p, _i, _i, _p, _p],
    "flmm_compat_spectrum_f32": [_p, _i, _i, _p, _p],
    "flmm_regress_out": [_p, _i64, _i, _i, _p, _i, _p, _p, _i64, _p],
    "flmm_gemm_nt_f64": [_p, _i64, _p, _i64, _p, _i64, _i, _i, _i, _d, _p],
    "flmm_delta_grid_nodes": [_d, _d, _i, _p, _p],
    "flmm_fit_delta_f64_workspace_bytes": [_i, _i, _psz],
    "flmm_fit_delta_f64": [_p, _i, _p, _i64, _i, _i, _d, _d, _i, _p, _p, _p, _sz, _p],
    "flmm_wald_f64_workspace_bytes": [_i, _i, _psz],
    "flmm_wald_f64": [_p, _i, _p, _i64, _p, _i, _i, _p, _i64, _i, _p, _p, _p, _p, _p, _i64, _p, _p, _sz, _p],
    "flmm_axpy_f64": [_i64, _d, _p, _p, _p],
    "flmm_perm_orders": [_p, _i, C.c_uint64, _i, _i, _p, _p],
    "flmm_pack_perm_columns": [_p, _i64, _i, _i, _p, _i, _p, _i64, _p],
    "flmm_fill_nullh2": [_p, _i, _p, _i, _p, _i64, _p],
    "flmm_fill_f64": [_p, _i64, _d, _p],
    "flmm_neglog10_pvalue": [_p, _i64, _i, _p, _p],
    "flmm_bed_decode": [_p, _i64, _i, _i, _p, _i, _i, _p, _i64, _p],
    "flmm_delta_features_f32": [_p, _i, _p, _i64, _i, _p, _p],
    "flmm_delta_mlp_f32": [_p, _i, _p, _p, _p, _p, _p, C.c_float, _d, _d, _p, _p],
    "flmm_fit_delta_learned_workspace_bytes": [_i, _i, _i, _psz],
    "flmm_fit_delta_learned": [_p, _i, _p, _i64, _i, _i, _d, _d, _i, _p, _p, _p, _p, _p, C.c_float, _i, _i, _p, _p, _p,
                               _p, _sz, _p],
    "flmm_mlp_grad_workspace_bytes": [_i, _psz],
    "flmm_mlp_grad": [_p, _p, _i64, _i, _p, _p, _i, C.c_float, _i, _p, _p, _p, _sz, _p],
    "flmm_mlp_adamw": [_p, _p, _p, _p, _i, C.c_float, C.c_float, C.c_float, C.c_float, C.c_float, _p],
    "flmm_fit_delta_lowrank_f64": [_p, _i, _p, _i64, _p, _i, _i, _i, _d, _d, _i, _p, _p, _p, _sz, _p],
    "flmm_wald_lowrank_f64_workspace_bytes": [_i, _i, _i, _i, _psz],
    "flmm_wald_lowrank_f64": [_p, _i, _p, _i64, _p, _i64, _i, _i, _p, _i, _i, _p, _i64, _p, _i64, _i, _p, _p, _p, _p,
                              _p, _i64, _p, _p, _sz, _p],
    "flmm_row_sumsq_f64": [_p, _i64, _i, _i, _p, _p],
    "flmm_shift_diagonal_f64": [_p, _i, _i64, _d, _p],
    "flmm_clamp_nonneg_f64": [_p, _i64, _p, _p],
    "flmm_gls_loss_workspace_bytes": [_i, _i, _i, _i, _psz],
    "flmm_gls_loss_f64": [_p, _i, _p, _i64, _i, _p, _i64, _i, _p, _i, _i, _i, _p, _p, _sz, _p],
    "flmm_fit_delta_gls_workspace_bytes": [_i, _i, _i, _i, _psz],
    "flmm_fit_delta_gls_f64": [_p, _i, _p, _i64, _i, _p, _i64, _i, _i, _d, _d, _i, _i, _p, _p, _p, _sz, _p],
    "flmm_wald_gls_workspace_bytes": [_i, _i, _i, _psz],
    "flmm_wald_gls_f64": [_p, _i, _p, _i64, _i, _p, _i64, _p, _i, _i, _p, _i64, _i, _p, _p, _p, _p, _p, _i64, _p,
                          _p, _sz, _p],
    "flmm_chisq1_from_f": [_p, _i64, _i, _p, _p],
    "flmm_perm_threshold_p": [_p, _i, _i, _i, _d, _p, _p],
    "flmm_f_pvalue": [_p, _i64, _i, _p, _p],
    "flmm_epi_setup_f64": [_p, _i, _p, _i64, _i, _p, _i64, _p, _i, _p, _p, _p, _p, _p, _p],
    "flmm_epi_wald_f32": [_p, _i64, _p, _i64, _p, _i, _i, _i, _i, _i, _i, _d, _d, _p, _p, _p, _i64, _p, _p, _p],
    "flmm_format_f64": [_p, _i64, _p, _i64, _p],
    "flmm_write_gwas_tsv": [_s, _i64, _p, _p, _p, _p, _p, _d, _p, _p, _p, _p, _p, _i64, _p, _i64, _s, _i64],
    "flmm_write_column_tsv": [_s, _s, _p, _i64],
    "flmm_fill_rows_host_f64": [_p, _i64, _i64, _p, _i64, _i],
    "flmm_host_alloc_mapped": [_sz, C.POINTER(_p), C.POINTER(_p)],
    "flmm_host_free_mapped": [_p],
    "flmm_context_check": [_p, _p],
    "flmm_split_rows_f16": [_p, _i, _i64, _i, _i, _p, _p, _i64, _p, _p],
    "flmm_gemm_split_f16": [_p, _p, _p, _p, _i64, _i, _p, _p, _p, _i64, _i, _i, _p, _i64, _i, _p],
    "flmm_tc_config": [_i, _i, _i],
    "flmm_autotune_report": [_p, _sz, C.POINTER(C.c_int)],
    "flmm_fit_delta_fast_workspace_bytes": [_i, _i, _psz],
    "flmm_fit_delta_fast": [_p, _i, _p, _i64, _i, _i, _d, _d, _i, _p, _p, _p, _sz, _p],
    "flmm_fit_delta_fast_noalloc": [_p, _i, _p, _i64, _i, _i, _d, _d, _i, _p, _p, _p],
    "flmm_mean_f32": [_p, _i, _p, _p],
    "flmm_wald_interp_nodes": [_p, _i, _p, _d, _d, _i, _p, _p],
    "flmm_wald_split_prep_columns": [_p, _i, _p, _i64, _p, _i, _p, _d, _d, _i, _p, _p, _i64, _p, _p, _i64, _p, _p,
                                     _p, _p, _p],
    "flmm_wald_split_prep_variants": [_p, _i64, _i, _i, _p, _p, _p, _p, _i64, _p, _p, _p],
    "flmm_wald_split_f16": [_p, _p, _p, _i64, _p, _p, _p, _i64, _p, _p, _p, _i, _i, _p, _p, _i64, _p, _p, _p, _i64, _p,
                            _i, _i, _i, _p, _p, _p, _p, _p, _i64, _p, C.c_float, _p, _p, _i, _p],
    "flmm_wald_split_f16_df": [_p, _p, _p, _i64, _p, _p, _p, _i64, _p, _p, _p, _i, _i, _p, _p, _i64, _p, _p, _p,
                               _i64, _p, _i, _i, _i, _p, _p, _p, _p, _p, _i64, _p, C.c_float, _p, _p, _i, _i, _p],
    "flmm_lr_prep_columns": [_p, _i, _p, _i64, _p, _i64, _i, _p, _p, _i, _p, C.c_double, C.c_double, _i, _p, _p,
                             _i64, _p, _p, _i64, _p, _p, _p, _p, _p],
    "flmm_lr_prep_variants": [_p, _i64, _p, _i64, _p, _i64, _i, _i, _i, _p, _i64, _i, _p, _p, _i64, _p, _p, _p, _i64,
                              _p, _p],
    "flmm_lr_residual": [_p, _i64, _p, _i64, _i, _i, _p, _i64, _p, _p],
    "flmm_lr_wald_refine": [_p, _p, _i, C.c_float, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _i64, _p, _p, _i, _i,
                            _i, _i, _i, _p, _p, _p, _p, _p, _i64, _p, _p],
    "flmm_lr_interp_nodes": [_p, _i, _p, C.c_double, C.c_double, _i, _p, _i64, _p],
    "flmm_wald_refine_f32": [_p, _p, _p, _i, C.c_float, _p, _i64, _p, _i64, _p, _p, _i, _i, _i, _p, _p, _p, _p, _p,
                             _i64, _p, _p],
    "flmm_scan_opts_default": [_p],
    "flmm_scan_create": [_i, _i, _i, _p, C.POINTER(_p)],
    "flmm_scan_destroy": [_p],
    "flmm_scan_group_prepare": [_p, _p, _p, _i64, _i, _p, _p, _i, _p],
    "flmm_scan_rotate_phenos": [_p, _p, _i64, _i, _p],
    "flmm_scan_fit_delta": [_p, _i, _p, _p],
    "flmm_scan_wald": [_p, _i, _p, _i64, _i, _p, _i, _p, _p, _p, _p, _p, _i64, _p, _p],
    "flmm_scan_run": [_p, _p, _i64, _i, _p, _i, _p, _p, _p, _p, _p, _i64, _p, _p, _p],
    "flmm_convert_f64_f32": [_i64, _p, _p, _p],
    "flmm_accumulate_f32_f64": [_i64, _p, _p, _p],
    "flmm_loco_kinship_f32": [_p, _p, _i, _d, _p, _p],
}
_RESTYPE = {"flmm_status_string": C.c_char_p, "flmm_last_error": C.c_char_p, "flmm_kernel_launches": C.c_uint64}


class ScanOpts(C.Structure):
    """flmm_scan_opts of include/fasterlmm_gb300.h."""
    _fields_ = [("n_grid", C.c_int), ("log_delta_min", C.c_double), ("log_delta_max", C.c_double),
                ("refine", C.c_int), ("eigh_refine_steps", C.c_int), ("f_refine", C.c_double), ("pipeline", C.c_int)]


class FlmmError(RuntimeError):
    def __init__(self, fn: str, status: int, message: str):
        super().__init__(f"{fn} failed: {message} (status {status})")
        self.status = status


_lock = threading.RLock()
_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises if it is missing (build it with ``fasterlmm_gb300.build()``)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(f"fasterlmm_gb300 CUDA library not built ({LIB_PATH} missing); "
                                   "run fasterlmm_gb300.build() -- there is no CPU fallback")
            h = C.CDLL(str(LIB_PATH))
            for name, argtypes in SIGNATURES.items():
                fn = getattr(h, name)
                fn.argtypes = argtypes
                fn.restype = _RESTYPE.get(name, C.c_int)
            _lib = h
    return _lib


def call(name: str, *args) -> None:
    """Call an int-status entry point; raise FlmmError on failure."""
    h = lib()
    rc = getattr(h, name)(*args)
    if rc != 0:
        msg = h.flmm_last_error().decode(errors="replace") or h.flmm_status_string(rc).decode()
        raise FlmmError(name, rc, msg)


def query_bytes(name: str, *args) -> int:
    out = C.c_size_t(0)
    call(name, *args, C.byref(out))
    return int(out.value)


_contexts: dict[int, C.c_void_p] = {}


def context(device: int) -> C.c_void_p:
    """Per-device library context (cuSOLVER handle), created on first use and kept for the process."""
    with _lock:
        ctx = _contexts.get(device)
        if ctx is None:
            ctx = C.c_void_p()
            h = lib()
            rc = h.flmm_context_create(device, C.byref(ctx))
            if rc != 0:
                raise FlmmError("flmm_context_create", rc, h.flmm_last_error().decode(errors="replace"))
            _contexts[device] = ctx
        return ctx


def tc_config(mode: int, pair: int = 1, group: int = 1) -> None:
    """Kernel form / tile order of the split products: 0 defaults, 1 autotune, 2 forced (pair, group)."""
    call("flmm_tc_config", int(mode), int(pair), int(group))


def autotune_report() -> list[dict]:
    """Shapes tuned so far in this process, with the chosen kernel form and tile order and their times."""
    buf = C.create_string_buffer(1 << 16)
    n = C.c_int(0)
    call("flmm_autotune_report", C.cast(buf, C.c_void_p), len(buf), C.byref(n))
    out = []
    for line in buf.value.decode().splitlines():
        ng, mr, nr, k, k2, pair, group, ms, dms = line.split()
        out.append({"kernel": "wald" if ng == "2" else "gemm", "rows": int(mr), "cols": int(nr), "K": int(k),
                    "K2": int(k2), "pair": bool(int(pair)), "group": int(group), "ms": float(ms),
                    "default_ms": float(dms)})
    return out


def kernel_launches() -> int:
    """Kernels launched by the library so far in this process."""
    return int(lib().flmm_kernel_launches())
