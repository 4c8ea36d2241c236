"""
GPU parity of the split-precision (tensor-core) form.

The split-FP16 products are checked against FP64 products, the fast delta fit against the FP64 golden-section fit
by loss equivalence, the fused Wald kernel against the FP64 Wald kernel, and whole permutation scans against the
reference's golden outputs at its parity tolerance (rtol 1e-5, atol 1e-6; F atol 1e-5) plus the -log10 p gate
|d(-log10 p)| <= 1e-3.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import z_float
from parity import DETAIL, assert_log_delta_equivalent, assert_scan_close

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from fasterlmm_gb300 import build
    build()


def _np(res) -> dict:
    return {k: getattr(res, k).detach().cpu().numpy() for k in DETAIL + ("max_F",)}


def _data(G, X, Y, chrom):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return SimpleNamespace(Z=t(z_float(G)), X=t(X), Y=t(Y), chrom=np.asarray(chrom), Z_kin=None, chrom_kin=None)


@pytest.mark.parametrize("Mr,Nr,K", [(128, 128, 64), (300, 200, 995), (1, 7, 13), (257, 129, 1000)])
def test_split_gemm_matches_fp64(Mr, Nr, K):
    from fasterlmm_gb300 import _lib
    from fasterlmm_gb300.fast import SplitRows, gemm_split
    g = torch.Generator().manual_seed(Mr * 7 + K)
    A = (torch.randn(Mr, K, generator=g, dtype=torch.float64) * torch.logspace(-3, 3, Mr, dtype=torch.float64)[:, None])
    B = torch.randn(Nr, K, generator=g, dtype=torch.float64)
    A, B = A.to(DEV), B.to(DEV)
    ctx = _lib.context(0)
    C = torch.empty(Mr, Nr, dtype=torch.float32, device=DEV)
    gemm_split(ctx, SplitRows.of(A).view(), SplitRows.of(B).view(), C)
    ref = A @ B.T
    scale = (A.abs() @ B.abs().T)
    err = ((C.double() - ref).abs() / scale).max().item()
    assert err < 2e-6, err
    # accumulate into an existing C
    C2 = C.clone()
    gemm_split(ctx, SplitRows.of(A).view(), SplitRows.of(B).view(), C2, accumulate=True)
    torch.testing.assert_close(C2, 2 * C, rtol=1e-6, atol=0)
    _lib.call("flmm_context_check", ctx, None)


def test_fast_delta_fit_is_loss_equivalent(golden):
    from fasterlmm_gb300 import core
    from fasterlmm_gb300.fast import fit_delta_fast
    g = golden("components")
    t = lambda a: torch.from_numpy(a).to(DEV)
    spec = core.fastlmm_compat_rotate(t(g["K"]), t(g["X"]), t(g["Y"]))
    ld, idx = fit_delta_fast(spec.s, spec.UYt.float())
    assert_log_delta_equivalent(ld.cpu().numpy(), g["log_delta"], g["s"], g["UY"])
    ld_grid, _ = fit_delta_fast(spec.s, spec.UYt.float(), refine=False)
    assert np.array_equal(ld_grid.cpu().numpy(), g["log_delta_grid"])


def test_fast_wald_matches_plain_wald():
    """Same spectrum, rotated data and log delta into both Wald kernels."""
    from fasterlmm_gb300 import _lib, core
    from fasterlmm_gb300.fast import WaldOperands, wald_fast
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(333, 3000, 3, 3, 50, seed=5, config_id=12, k_lo=1, k_hi=30, h2_lo=0.0, h2_hi=0.9)
    Zs = orc.standardise_columns(d.Z_float())
    K = orc.grm(Zs[:, d.chrom != 1])
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    spec = core.fastlmm_compat_rotate(t(K), t(d.X), t(d.Y))
    ld = core.fit_delta_grid_compat(spec)
    St = t(Zs[:, d.chrom == 1].T)
    basis = core._BasisView(t(d.X), spec.Xpinv)
    USt = core.rotate_rows(basis.regress_out(St), spec.Ut)
    M, P, n_real = St.shape[0], spec.UYt.shape[0], 40
    rows = torch.arange(M, device=DEV)
    out64, mF64 = core._alloc_outputs(M, n_real, P, spec.s.device)
    core.wald_t(spec.s, spec.UYt, ld, USt, n_real, rows, out64, mF64)
    out32, mF32 = core._alloc_outputs(M, n_real, P, spec.s.device)
    wald_fast(_lib.context(0), WaldOperands(spec.s.device), spec.s, spec.UYt.float(), ld, USt.float(), n_real, rows,
              out32, mF32, log_delta_min=-10.0, log_delta_max=10.0)
    _lib.call("flmm_context_check", _lib.context(0), None)
    for k in DETAIL:
        a, b = out32[k].cpu().numpy(), out64[k].cpu().numpy()
        np.testing.assert_allclose(a, b, rtol=1e-5, atol=1e-5 if k == "f" else 1e-6, err_msg=k)
    np.testing.assert_allclose(mF32.cpu().numpy(), mF64.cpu().numpy(), rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("name", ["loco_n150_m1500", "edge_intercept_only", "edge_rank_deficient"])
def test_fast_perm_threshold_matches_golden(golden, name):
    from fasterlmm_gb300 import perms, post
    g = golden(name)
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    res, pmf = perms.perm_threshold(_data(g["G"], g["X"], g["Y"], g["chrom"]), list(range(B)), n_perm=n_perm,
                                    form="fast")
    assert_scan_close(_np(res), g)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",))
    N, D = g["X"].shape
    nl = post.neg_log10_pvalue(res.f, N - D - 1).cpu().numpy()
    ref = orc.neg_log10_p(g["f"], N - D - 1)
    assert np.abs(nl - ref).max() <= 1e-3


def test_fast_na_groups_and_single_k(golden):
    from fasterlmm_gb300 import perms
    g = golden("na_groups")
    for gi in range(int(g["n_groups"])):
        keep, cols = g[f"g{gi}_keep"], g[f"g{gi}_cols"]
        res, pmf = perms.perm_threshold(_data(g["G"][keep], g["X"][keep], g["Y"][keep][:, cols], g["chrom"]),
                                        list(range(len(cols))), n_perm=int(g["n_perm"]), seed_idx=list(cols),
                                        form="fast")
        assert_scan_close(_np(res), g, prefix=f"g{gi}_")
        assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",), prefix=f"g{gi}_")
    g = golden("kin_panel_single_k")
    B = g["f"].shape[1]
    res, pmf = perms.perm_threshold(_data(g["G"], g["X"], g["Y"], g["chrom"]), list(range(B)), n_perm=int(g["n_perm"]),
                                    loco=False, form="fast")
    assert_scan_close(_np(res), g, prefix="sk_")


def test_fast_larger_case_matches_oracle():
    """Several tiles in every dimension, unsorted chromosome labels, P not a multiple of 128."""
    from fasterlmm_gb300 import perms
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(400, 3000, 4, 5, 61, seed=17, config_id=13, chrom_sizes=[900, 700, 1000, 400], k_lo=0,
                     k_hi=40, h2_lo=0.0, h2_hi=0.9)
    perm = np.random.default_rng(3).permutation(3000)
    G, chrom = d.G[:, perm], d.chrom[perm]
    n_perm = 4
    res, pmf = perms.perm_threshold(_data(G, d.X, d.Y, chrom), list(range(61)), n_perm=n_perm, form="fast")
    ref, rpmf = orc.perm_threshold(z_float(G), d.X, d.Y, chrom, range(61), n_perm=n_perm)
    assert_scan_close(_np(res), ref)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, {"perm_max_F": rpmf}, keys=("perm_max_F",))


@pytest.mark.parametrize("shuffle", [False, True])
def test_fast_streamed_host_outputs_match_device(shuffle):
    """out= with pinned host tensors: rows streamed per chromosome (or copied at the end when labels are unsorted)."""
    from fasterlmm_gb300 import perms
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(300, 2000, 3, 3, 20, seed=23, config_id=14, k_lo=1, k_hi=20)
    G, chrom = d.G, d.chrom
    if shuffle:
        perm = np.random.default_rng(1).permutation(G.shape[1])
        G, chrom = G[:, perm], chrom[perm]
    data = _data(G, d.X, d.Y, chrom)
    n_perm = 3
    ref, ref_pmf = perms.perm_threshold(data, list(range(20)), n_perm=n_perm, form="fast")
    M = G.shape[1]
    out = {k: torch.full((M, 20), np.nan, dtype=torch.float64).pin_memory() for k in DETAIL}
    out["max_F"] = torch.empty(20 * (1 + n_perm), dtype=torch.float64).pin_memory()
    res, pmf = perms.perm_threshold(data, list(range(20)), n_perm=n_perm, form="fast", out=out)
    for k in DETAIL + ("max_F",):
        assert getattr(res, k).data_ptr() == out[k].data_ptr()
        assert torch.equal(getattr(res, k), getattr(ref, k).cpu()), k
    assert torch.equal(pmf, ref_pmf.cpu())


def test_fast_form_with_fp32_eigendecomposition(golden, monkeypatch):
    """
    The FP32 eigendecomposition option: test statistics and -log10 p within the parity tolerance; nullh2 is
    excluded because a flat likelihood turns the decomposition's ~1e-7 error into a larger shift of delta.
    """
    from fasterlmm_gb300 import fast, perms, post
    monkeypatch.setattr(fast, "EIGH_PRECISION", "f32")
    g = golden("loco_n150_m1500")
    B = g["f"].shape[1]
    res, pmf = perms.perm_threshold(_data(g["G"], g["X"], g["Y"], g["chrom"]), list(range(B)), n_perm=int(g["n_perm"]),
                                    form="fast")
    assert_scan_close(_np(res), g, keys=("f", "beta", "se", "sfve", "max_F"))
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",))
    N, D = g["X"].shape
    nl = post.neg_log10_pvalue(res.f, N - D - 1).cpu().numpy()
    assert np.abs(nl - orc.neg_log10_p(g["f"], N - D - 1)).max() <= 1e-3


def test_eigh_refinement_brings_fp32_eigenpairs_to_near_fp64():
    """
    One refinement step: the eigenvalues become Rayleigh quotients of the FP32 vectors (error quadratic in the
    vector error, far below FP32's), and the eigenvector residuals drop by more than an order of magnitude.
    """
    from fasterlmm_gb300 import _lib, fast
    g = torch.Generator().manual_seed(11)
    N, batch = 300, 3
    Z = torch.randn(batch, N, 2 * N, generator=g, dtype=torch.float64)
    K = (Z @ Z.transpose(1, 2)) / (2 * N) + torch.eye(N, dtype=torch.float64)
    K = K.to(DEV)
    ctx = _lib.context(0)
    U32, ev32 = fast._eigh_batched_f32(ctx, K.clone())
    U, ev = fast._eigh_batched_f32_refined(ctx, K.clone())
    ref = torch.linalg.eigvalsh(K)
    assert ev.dtype == torch.float64
    scale = ref.abs().amax(1, keepdim=True)
    rel = ((ev - ref).abs() / scale).max().item()
    rel32 = ((ev32.double() - ref).abs() / scale).max().item()
    assert rel < 1e-8 and rel < rel32 / 100, (rel, rel32)

    def resid(Ur, lam):
        Ud = Ur.double()
        Ud = Ud / Ud.norm(dim=2, keepdim=True)
        R = torch.bmm(Ud, K) - lam.unsqueeze(2) * Ud
        return (R.norm(dim=2) / ref.abs().amax(1, keepdim=True)).max().item()

    r32, r_ref = resid(U32, ev32.double()), resid(U, ev)
    assert r_ref < r32 / 20, (r32, r_ref)
    # the refined rows are stored in FP32: orthonormal to FP32 rounding
    orth = (torch.bmm(U.double(), U.double().transpose(1, 2)) - torch.eye(N, device=DEV, dtype=torch.float64)).abs().max()
    assert orth.item() < 1e-5

