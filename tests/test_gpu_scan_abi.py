"""
GPU tests of the scan-level C ABI (flmm_scan_*): a whole LOCO permutation scan driven through ctypes on the
library's entry points alone -- standardisation, permutation orders and column packing, then flmm_scan_create /
group_prepare / rotate_phenos / run (or fit_delta + wald per chromosome) -- with torch used only to hold device
memory.  Checked against the reference's golden outputs at its parity tolerance (rtol 1e-5, atol 1e-6; F 1e-5), and
bit for bit against the Python driver of the same fast form, which issues the same kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import z_float
from parity import DETAIL, assert_scan_close

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from fasterlmm_gb300 import _lib, build
    build()
    return _lib


def _p(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def _dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def _inputs(lib, G, X, Y, n_perm, seed=19930909, seed_cols=None):
    """Device inputs through the library: standardised variant-major Zt, X, packed scan columns Yt_all."""
    Z = _dev(z_float(G))
    N, M = Z.shape
    Zt = torch.empty((M, N), dtype=torch.float64, device="cuda")
    lib.call("flmm_standardise_f64", _p(Z), M, N, M, _p(Zt), N, None)
    B = Y.shape[1]
    Yt_real = _dev(np.asarray(Y).T)
    cols = torch.tensor(list(range(B)) if seed_cols is None else list(seed_cols), dtype=torch.int64, device="cuda")
    orders = torch.empty((B, n_perm, N), dtype=torch.int32, device="cuda")
    if n_perm:
        lib.call("flmm_perm_orders", _p(cols), B, seed, n_perm, N, _p(orders), None)
    Yt = torch.empty((B * (1 + n_perm), N), dtype=torch.float64, device="cuda")
    lib.call("flmm_pack_perm_columns", _p(Yt_real), N, B, N, _p(orders) if n_perm else None, n_perm, _p(Yt), N, None)
    return Zt, _dev(X), Yt


def _scan(lib, G, X, Y, chrom, n_perm, *, kin=None, loco=True, per_chrom=False, opts=None):
    """Run the scan through the C ABI; returns numpy outputs (M, B) and max_F (P,)."""
    Zt, Xd, Yt = _inputs(lib, G, X, Y, n_perm)
    M, N = Zt.shape
    D = Xd.shape[1]
    B = Y.shape[1]
    P = Yt.shape[0]
    o = lib.ScanOpts()
    lib.call("flmm_scan_opts_default", C.byref(o))
    for k, v in (opts or {}).items():
        setattr(o, k, v)
    scan = C.c_void_p()
    lib.call("flmm_scan_create", 0, N, D, C.byref(o), C.byref(scan))
    try:
        chrom = np.ascontiguousarray(np.asarray(chrom, dtype=np.int32))
        if kin is None:
            Zk, ck = Zt, chrom
        else:
            Gk, ck = kin
            Zk, _, _ = _inputs(lib, Gk, X, Y[:, :1], 0)
            ck = np.ascontiguousarray(np.asarray(ck, dtype=np.int32))
        units = np.unique(chrom).astype(np.int32) if loco else np.zeros(0, dtype=np.int32)
        lib.call("flmm_scan_group_prepare", scan, _p(Xd), _p(Zk), N, Zk.shape[0], ck.ctypes.data_as(C.c_void_p),
                 units.ctypes.data_as(C.c_void_p) if loco else None, len(units), None)
        lib.call("flmm_scan_rotate_phenos", scan, _p(Yt), N, P, None)
        out = {k: torch.full((M, B), np.nan, dtype=torch.float64, device="cuda") for k in DETAIL}
        max_F = torch.empty(P, dtype=torch.float64, device="cuda")
        n_units = max(len(units), 1)
        ld = torch.empty((n_units, P), dtype=torch.float64, device="cuda")
        if not per_chrom:
            lib.call("flmm_scan_run", scan, _p(Zt), N, M, chrom.ctypes.data_as(C.c_void_p), B, _p(out["f"]),
                     _p(out["beta"]), _p(out["se"]), _p(out["sfve"]), _p(out["nullh2"]), B, _p(max_F), _p(ld), None)
        else:
            max_F.fill_(-np.inf)
            for u, c in enumerate(units):
                sel = np.flatnonzero(chrom == c)
                rows = torch.from_numpy(sel.astype(np.int64)).cuda()
                Zc = Zt[rows].contiguous()
                lib.call("flmm_scan_fit_delta", scan, u, _p(ld[u]), None)
                lib.call("flmm_scan_wald", scan, u, _p(Zc), N, len(sel), _p(rows), B, _p(out["f"]), _p(out["beta"]),
                         _p(out["se"]), _p(out["sfve"]), _p(out["nullh2"]), B, _p(max_F), None)
            torch.cuda.synchronize()
    finally:
        lib.call("flmm_scan_destroy", scan)
    res = {k: v.cpu().numpy() for k, v in out.items()}
    res["max_F"] = max_F.cpu().numpy()
    res["perm_max_F"] = res["max_F"][B:].reshape(B, n_perm)
    res["log_delta"] = ld.cpu().numpy()
    return res


def test_scan_abi_matches_reference_golden(lib, golden):
    g = golden("loco_n150_m1500")
    B, n_perm = g["f"].shape[1], int(g["n_perm"])
    res = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], n_perm)
    assert_scan_close(res, g)
    assert_scan_close(res, g, keys=("perm_max_F",))
    N, D = g["X"].shape
    assert np.abs(orc.neg_log10_p(res["f"], N - D - 1) - orc.neg_log10_p(g["f"], N - D - 1)).max() <= 1e-3


def test_scan_abi_per_chromosome_calls_match_run(lib, golden):
    """fit_delta(k) + wald(k) per chromosome give the same bits as the pipelined run."""
    g = golden("loco_n150_m1500")
    B = g["f"].shape[1]
    a = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], 7)
    b = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], 7, per_chrom=True)
    for k in DETAIL + ("max_F", "log_delta"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    c = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], 7, opts={"pipeline": 0})
    for k in DETAIL + ("max_F", "log_delta"):
        np.testing.assert_array_equal(a[k], c[k], err_msg=k)


def test_scan_abi_kinship_panel_and_single_k(lib, golden):
    g = golden("kin_panel_single_k")
    B, n_perm = g["f"].shape[1], int(g["n_perm"])
    res = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], n_perm, kin=(g["G_kin"], g["chrom_kin"]))
    assert_scan_close(res, g)
    res = _scan(lib, g["G"], g["X"], g["Y"][:, :B], g["chrom"], n_perm, loco=False)
    assert_scan_close(res, g, prefix="sk_")


def test_scan_abi_is_bit_identical_to_the_python_driver(lib):
    """Unsorted chromosome labels, several tiles in every dimension: the C ABI and fasterlmm_gb300.perms issue the
    same kernels on the same operands."""
    from types import SimpleNamespace
    from fasterlmm_gb300 import perms
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(400, 3000, 4, 5, 61, seed=17, config_id=13, chrom_sizes=[900, 700, 1000, 400], k_lo=0,
                     k_hi=40, h2_lo=0.0, h2_hi=0.9)
    perm = np.random.default_rng(3).permutation(3000)
    G, chrom = d.G[:, perm], d.chrom[perm]
    n_perm = 4
    res = _scan(lib, G, d.X, d.Y, chrom, n_perm)
    data = SimpleNamespace(Z=_dev(z_float(G)), X=_dev(d.X), Y=_dev(d.Y), chrom=chrom, Z_kin=None, chrom_kin=None)
    ref, pmf = perms.perm_threshold(data, list(range(61)), n_perm=n_perm, form="fast")
    for k in DETAIL + ("max_F",):
        np.testing.assert_array_equal(res[k], getattr(ref, k).cpu().numpy(), err_msg=k)
