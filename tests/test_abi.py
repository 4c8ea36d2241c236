"""
CPU checks of the C ABI: the library builds for sm_103a, loads without a GPU, and exports every entry point that
include/*.h declares; the Python binding declares exactly those entry points.  No compute call is made here.
"""
from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]


def _declared() -> set[str]:
    names = set()
    for h in (REPO / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(flmm_\w+)\s*\(", text, flags=re.M))
    return names


@pytest.fixture(scope="module")
def built():
    from fasterlmm_gb300 import build
    return build()


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(str(built))
    declared = _declared()
    assert len(declared) >= 20
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, f"declared in include/ but not exported: {missing}"


def test_binding_matches_header(built):
    from fasterlmm_gb300 import _lib
    assert set(_lib.SIGNATURES) == _declared()
    h = _lib.lib()
    assert h.flmm_version() >= 100
    assert h.flmm_status_string(0).decode() == "ok"
    assert "workspace" in h.flmm_status_string(4).decode()


def test_argument_errors_without_gpu(built):
    """Argument validation happens on the host before any CUDA call, so it is testable without a device."""
    from fasterlmm_gb300 import _lib
    with pytest.raises(_lib.FlmmError) as e:
        _lib.call("flmm_fill_f64", None, 10, 0.0, None)
    assert e.value.status == 1
    with pytest.raises(_lib.FlmmError):
        _lib.call("flmm_neglog10_pvalue", None, 5, 0, None, None)
    size = ctypes.c_size_t(0)
    _lib.call("flmm_wald_f64_workspace_bytes", 100, 50, ctypes.byref(size))
    assert size.value >= 8 * (2 * 100 * 50 + 100)


def test_no_cpu_fallback_without_cuda():
    """The product path refuses to run without a CUDA device instead of computing on the CPU."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from fasterlmm_gb300 import core
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        core.grm(torch.zeros(4, 4, dtype=torch.float64))


def test_host_row_fill(built):
    """flmm_fill_rows_host_f64 (host code: the streamed nullh2 rows) fills exactly the rows and columns asked for."""
    import numpy as np
    from fasterlmm_gb300 import _lib
    for rows, threads in ((2000, 8), (100, 8), (1, 1), (5000, 3)):
        dst = np.zeros((rows + 20, 70))
        vec = np.random.default_rng(rows).standard_normal(64)
        _lib.call("flmm_fill_rows_host_f64", dst.ctypes.data + 8 * 70 * 10, 70, rows, vec.ctypes.data, 64, threads)
        assert (dst[10:10 + rows, :64] == vec).all()
        assert not dst[:10].any() and not dst[10 + rows:].any() and not dst[:, 64:].any()
    with pytest.raises(_lib.FlmmError):
        _lib.call("flmm_fill_rows_host_f64", None, 70, 10, None, 64, 1)


def test_new_entry_points_validate_arguments_without_gpu(built):
    """The training, learned-fit and autotuner entry points reject bad arguments on the host."""
    from fasterlmm_gb300 import _lib
    size = ctypes.c_size_t(0)
    _lib.call("flmm_mlp_grad_workspace_bytes", 2048, ctypes.byref(size))
    assert size.value == 4 * 25092 * 128  # one padded partial gradient per 16-row CTA
    with pytest.raises(_lib.FlmmError) as e:  # no parameters / features
        _lib.call("flmm_mlp_grad", None, None, 65, 10, None, None, 16, 0.1, 1, None, None, None, 0, None)
    assert e.value.status == 1
    with pytest.raises(_lib.FlmmError):  # AdamW steps count from 1
        _lib.call("flmm_mlp_adamw", 8, 8, 8, 8, 0, 1e-3, 0.9, 0.999, 1e-8, 0.0, None)
    with pytest.raises(_lib.FlmmError, match="Neff must be >= 32"):
        p = 256
        _lib.call("flmm_fit_delta_learned", p, 16, p, 16, 10, 64, -10.0, 10.0, 1, p, p, p, p, p, 0.0, 3, 64, p, p, p,
                  p, 1 << 20, None)
    _lib.call("flmm_fit_delta_learned_workspace_bytes", 995, 64, 71324, ctypes.byref(size))
    assert size.value >= 4 * 71324 * 65 + 8 * 71324 + 4 * 71324
    with pytest.raises(_lib.FlmmError):
        _lib.call("flmm_tc_config", 3, 1, 1)
    with pytest.raises(_lib.FlmmError):
        _lib.call("flmm_tc_config", 2, 1, 0)  # a forced tile order needs group >= 1
    _lib.tc_config(1)
    assert isinstance(_lib.autotune_report(), list)


def test_dropin_raises_the_references_value_error_before_any_device_work():
    """A lone Z_kin or chrom_kin is a ValueError, as in the reference (fasterlmm/core.py:694-695), with or without GPU."""
    import numpy as np
    import torch
    from fasterlmm_gb300 import core, gls
    Z, X, Y = torch.zeros(6, 4, dtype=torch.float64), torch.ones(6, 1, dtype=torch.float64), torch.zeros(6, 2,
                                                                                                        dtype=torch.float64)
    chrom = np.array([1, 1, 2, 2])
    for fn in (core.loco_scan_compat, gls.loco_scan):
        with pytest.raises(ValueError, match="go together"):
            fn(Z, X, Y, chrom, Z_kin=Z)
        with pytest.raises(ValueError, match="go together"):
            fn(Z, X, Y, chrom, chrom_kin=chrom)
