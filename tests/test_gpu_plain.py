"""
GPU parity of the plain (FP64) form against the reference's golden outputs and the CPU oracle.

Every call goes through the C ABI (ctypes) into the sm_103a library.  Tolerances are the reference's parity
convention (tests/parity.py); log delta is compared by loss equivalence because the reference's golden-section
search is itself only determined to FP64 noise.
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


def _np(res) -> dict:
    return {k: getattr(res, k).detach().cpu().numpy() for k in DETAIL + ("max_F",)}


def _data(G, X, Y, chrom, G_kin=None, chrom_kin=None):
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    return SimpleNamespace(Z=t(z_float(G)), X=t(X), Y=t(Y), chrom=np.asarray(chrom),
                           Z_kin=None if G_kin is None else t(z_float(G_kin)), chrom_kin=chrom_kin)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from fasterlmm_gb300 import build
    build()


def _check_ld(res, ref_ld, spectra):
    for i, c in enumerate(sorted(res.log_delta)):
        s, UY = spectra[c]
        assert_log_delta_equivalent(res.log_delta[c].cpu().numpy(), ref_ld[i], s, UY)


def test_standardise_and_grm_match_oracle(golden):
    from fasterlmm_gb300 import core
    g = golden("na_groups")  # has missing calls
    Z = z_float(g["G"])
    Zs = core.standardise_columns(torch.from_numpy(Z).to(DEV)).cpu().numpy()
    np.testing.assert_allclose(Zs, orc.standardise_columns(Z), rtol=1e-12, atol=1e-12)
    K = core.grm(torch.from_numpy(Zs).to(DEV)).cpu().numpy()
    np.testing.assert_allclose(K, orc.grm(Zs), rtol=1e-11, atol=1e-12)
    # the numpy path returns numpy; a float32 tensor comes back float32, as the reference's torch branch returns it
    assert isinstance(core.standardise_columns(Z), np.ndarray)
    Z32 = core.standardise_columns(torch.from_numpy(Z).float().to(DEV))
    assert Z32.dtype == torch.float32 and Z32.shape == Z.shape
    np.testing.assert_allclose(Z32.cpu().numpy(), orc.standardise_columns(Z.astype(np.float32).astype(np.float64)),
                               rtol=1e-6, atol=1e-6)


def test_components_match_golden(golden):
    from fasterlmm_gb300 import core
    g = golden("components")
    t = lambda a: torch.from_numpy(a).to(DEV)
    spec = core.fastlmm_compat_rotate(t(g["K"]), t(g["X"]), t(g["Y"]))
    np.testing.assert_allclose(spec.s.cpu().numpy(), g["s"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(spec.Xpinv.cpu().numpy(), g["Xpinv"], rtol=1e-9, atol=1e-12)
    np.testing.assert_allclose(spec.UY.cpu().numpy() ** 2, g["UY"] ** 2, rtol=1e-8, atol=1e-10)
    assert spec.U_eff.shape == g["U_eff"].shape
    ld_grid = core.fit_delta_grid_compat(spec, refine=False).cpu().numpy()
    assert np.array_equal(ld_grid, g["log_delta_grid"])  # grid argmin bit-exact
    ld = core.fit_delta_grid_compat(spec).cpu().numpy()
    assert_log_delta_equivalent(ld, g["log_delta"], g["s"], g["UY"])
    res = core.snp_wald_scan_compat(spec, t(g["log_delta"]), t(g["Z_std"]), n_real=4)
    assert_scan_close(_np(res), g, rtol=1e-9, atol_scale=1e-3)


@pytest.mark.parametrize("name", ["loco_n150_m1500", "edge_intercept_only", "edge_rank_deficient"])
def test_perm_threshold_matches_golden(golden, name):
    from fasterlmm_gb300 import perms
    g = golden(name)
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    seen = []
    res, pmf = perms.perm_threshold(_data(g["G"], g["X"], g["Y"], g["chrom"]), list(range(B)), n_perm=n_perm,
                                    on_chrom=lambda k, n: seen.append((k, n)))
    n_chr = len(np.unique(g["chrom"]))
    assert seen == [(k + 1, n_chr) for k in range(n_chr)]
    assert pmf.shape == (B, n_perm) and res.f.shape == (g["G"].shape[1], B)
    assert_scan_close(_np(res), g)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",))
    ref, _ = orc.perm_threshold(z_float(g["G"]), g["X"], g["Y"], g["chrom"], range(B), n_perm=n_perm,
                                keep_spectra=True)
    _check_ld(res, g["log_delta"], ref["spectra"])


def test_grid100_loco_matches_golden(golden):
    """Reference LOCO loop with the 100-point [-5, 5] grid; permutation orders are the reference's own."""
    from fasterlmm_gb300 import core, perms
    g = golden("loco_n150_m1500_grid100")
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    N = g["G"].shape[0]
    orders = perms.perm_orders(N, range(B), n_perm)
    assert np.array_equal(orders, g["orders"].transpose(1, 2, 0))  # bit-exact permutation index sets
    Yt = perms.pack_perm_columns(core.transpose(torch.from_numpy(g["Y"][:, :B].copy()).to(DEV)),
                                 torch.from_numpy(orders).to(DEV))
    Zs = core.standardise_columns(torch.from_numpy(z_float(g["G"])).to(DEV))
    res = core.loco_scan_compat(Zs, torch.from_numpy(g["X"]).to(DEV), Yt.T, g["chrom"], n_real=B, n_grid=100,
                                log_delta_min=-5.0, log_delta_max=5.0)
    assert_scan_close(_np(res), g)


def test_kin_panel_and_single_k_match_golden(golden):
    from fasterlmm_gb300 import perms
    g = golden("kin_panel_single_k")
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    data = _data(g["G"], g["X"], g["Y"], g["chrom"], g["G_kin"], g["chrom_kin"])
    res, pmf = perms.perm_threshold(data, list(range(B)), n_perm=n_perm)
    assert_scan_close(_np(res), g)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",))
    data.Z_kin = None
    data.chrom_kin = None
    res, pmf = perms.perm_threshold(data, list(range(B)), n_perm=n_perm, loco=False)
    assert_scan_close(_np(res), g, prefix="sk_")
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",), prefix="sk_")


def test_na_groups_match_golden(golden):
    from fasterlmm_gb300 import perms
    g = golden("na_groups")
    Z = z_float(g["G"])
    for gi in range(int(g["n_groups"])):
        keep, cols = g[f"g{gi}_keep"], g[f"g{gi}_cols"]
        data = _data(g["G"][keep], g["X"][keep], g["Y"][keep][:, cols], g["chrom"])
        assert np.isnan(data.Z.cpu().numpy()).any() == np.isnan(Z[keep]).any()
        res, pmf = perms.perm_threshold(data, list(range(len(cols))), n_perm=int(g["n_perm"]), seed_idx=list(cols))
        assert_scan_close(_np(res), g, prefix=f"g{gi}_")
        assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",), prefix=f"g{gi}_")


def test_loco_inputs_on_cpu_come_back_on_cpu(golden):
    """Host tensors in, host tensors out: the copies go through the device, the compute stays on the GPU."""
    from fasterlmm_gb300 import core
    g = golden("edge_rank_deficient")
    Zs = torch.from_numpy(orc.standardise_columns(z_float(g["G"])))
    res = core.loco_scan_compat(Zs, torch.from_numpy(g["X"]), torch.from_numpy(g["Y"]), g["chrom"], n_real=1)
    assert res.f.device.type == "cpu" and res.f.shape == (Zs.shape[1], 1)
    with pytest.raises(ValueError):
        core.loco_scan_compat(Zs, torch.from_numpy(g["X"]), torch.from_numpy(g["Y"]), g["chrom"], Z_kin=Zs)


def test_n_real_split_and_max_F(golden):
    """n_real = B keeps the leading columns of the full scan; max_F is the column max (reference invariants)."""
    from fasterlmm_gb300 import core
    g = golden("kin_panel_single_k")
    Zs = core.standardise_columns(torch.from_numpy(z_float(g["G"])).to(DEV))
    X = torch.from_numpy(g["X"]).to(DEV)
    Y = torch.from_numpy(g["Y"]).to(DEV)
    full = core.loco_scan_compat(Zs, X, Y, g["chrom"])
    part = core.loco_scan_compat(Zs, X, Y, g["chrom"], n_real=2)
    assert torch.equal(part.f, full.f[:, :2]) and torch.equal(part.max_F, full.max_F)
    torch.testing.assert_close(full.max_F, full.f.max(dim=0).values, rtol=0, atol=0)


def test_larger_random_case_matches_oracle():
    """Several tiles in every kernel dimension, sizes that are not tile multiples, uneven chromosomes."""
    from fasterlmm_gb300.synth import make_dataset
    from fasterlmm_gb300 import perms
    d = make_dataset(301, 2600, 5, 4, 37, seed=7, config_id=11, chrom_sizes=[700, 131, 1000, 69, 700], k_lo=1,
                     k_hi=20, h2_lo=0.0, h2_hi=0.9)
    n_perm = 3
    res, pmf = perms.perm_threshold(_data(d.G, d.X, d.Y, d.chrom), list(range(37)), n_perm=n_perm)
    ref, rpmf = orc.perm_threshold(z_float(d.G), d.X, d.Y, d.chrom, range(37), n_perm=n_perm, keep_spectra=True)
    assert_scan_close(_np(res), ref)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, {"perm_max_F": rpmf}, keys=("perm_max_F",))
    lds = np.stack([ref["log_delta"][c] for c in sorted(ref["log_delta"])])
    _check_ld(res, lds, ref["spectra"])


def test_pvalues_match_scipy(golden):
    import ctypes
    from fasterlmm_gb300 import _lib
    g = golden("loco_n150_m1500")
    N, D = g["X"].shape
    df2 = N - D - 1
    F = np.concatenate([g["f"].ravel(), np.logspace(-6, 5, 2000), [0.0, 1e7]])
    Fd = torch.from_numpy(F).to(DEV)
    out = torch.empty_like(Fd)
    _lib.call("flmm_neglog10_pvalue", ctypes.c_void_p(Fd.data_ptr()), F.size, df2, ctypes.c_void_p(out.data_ptr()),
              None)
    got = out.cpu().numpy()
    ref = orc.neg_log10_p(F, df2)
    fin = np.isfinite(ref)
    np.testing.assert_allclose(got[fin], ref[fin], rtol=1e-10, atol=1e-10)
    assert (got[~fin] > 300).all()  # scipy underflows to p = 0 there; the log-space value stays finite


def test_device_permutation_orders_are_bit_identical():
    """The device PCG64 / SeedSequence / argsort path reproduces numpy's orders exactly, incl. large seeds."""
    from fasterlmm_gb300 import perms
    for N, cols, n_perm, seed in [(150, range(20), 100, 19930909), (1000, [0, 5, 6483], 10, 19930909),
                                  (37, [3, 2**33 + 5], 4, 2**40 + 17), (1, [0], 3, 7),
                                  (2048, [4], 2, 5), (3000, [1, 9], 2, 11)]:  # packed-key sort up to 2048
        dev_o = perms.perm_orders_device(N, cols, n_perm, seed, torch.device(DEV)).cpu().numpy()
        host_o = perms.perm_orders(N, cols, n_perm, seed)
        assert np.array_equal(dev_o, host_o), (N, list(cols)[:3], seed)


def test_permutation_threshold_matches_numpy_quantile(golden):
    """Device threshold = numpy.quantile(f.sf(perm_max_F, 1, df2), 0.05) per phenotype (the CLI's rule)."""
    from fasterlmm_gb300 import post
    g = golden("loco_n150_m1500")
    N, D = g["X"].shape
    thr = post.perm_threshold_p(torch.from_numpy(g["perm_max_F"]).to(DEV), N - D - 1).cpu().numpy()
    np.testing.assert_allclose(thr, g["threshold"], rtol=1e-10, atol=0)
    for q in (0.0, 0.5, 1.0, 0.123):
        ref = [np.quantile(orc.f_sf(g["perm_max_F"][b], N - D - 1), q) for b in range(g["perm_max_F"].shape[0])]
        got = post.perm_threshold_p(torch.from_numpy(g["perm_max_F"]).to(DEV), N - D - 1, q).cpu().numpy()
        np.testing.assert_allclose(got, ref, rtol=1e-10, atol=0)


def test_grouped_driver_matches_golden(golden):
    """The CLI-style grouped scan (one perm_threshold per NaN pattern, full-table seeds) on the reference's fixture."""
    from fasterlmm_gb300.groups import perm_threshold_grouped
    g = golden("na_groups")
    data = _data(g["G"], g["X"], g["Y"], g["chrom"])
    out = perm_threshold_grouped(data, list(range(g["Y"].shape[1])), n_perm=int(g["n_perm"]))
    assert len(out) == int(g["n_groups"])
    for gi, gr in enumerate(out):
        assert gr.cols == g[f"g{gi}_cols"].tolist() and gr.df2 == len(gr.keep) - g["X"].shape[1] - 1
        assert_scan_close(_np(gr.res), g, prefix=f"g{gi}_")
        assert_scan_close({"perm_max_F": gr.perm_max_F.cpu().numpy()}, g, keys=("perm_max_F",), prefix=f"g{gi}_")


def test_lambda_gc_and_rank_by_p_match_scipy(golden):
    """Device post-scan: lambda GC (fasterlmm/inflation.py) and the p-ascending table order, on golden F."""
    import scipy.stats as ss
    from fasterlmm_gb300 import post
    g = golden("loco_n150_m1500")
    N, D = g["X"].shape
    df2 = N - D - 1
    F = g["f"].copy()
    F[3, 2] = np.nan  # a dropped p-value
    lam, n = post.lambda_gc(torch.from_numpy(F).cuda(), df2)
    for b in range(F.shape[1]):
        p = ss.f.sf(F[:, b], 1, df2)
        p = p[~np.isnan(p)]
        ref = np.median(ss.chi2.isf(p, 1)) / ss.chi2.ppf(0.5, 1)
        assert int(n[b].item()) == p.size
        np.testing.assert_allclose(lam[b].item(), ref, rtol=1e-9)
    order = post.rank_by_p(torch.from_numpy(F).cuda(), df2).cpu().numpy()
    for b in range(F.shape[1]):
        p = ss.f.sf(F[:, b], 1, df2)
        assert np.array_equal(np.sort(order[:, b]), np.arange(F.shape[0]))  # a permutation
        pv = p[order[:, b]]
        k = int((~np.isnan(pv)).sum())
        assert np.isnan(pv[k:]).all() and np.all(np.diff(pv[:k]) >= -1e-15 * pv[1:k])  # p ascending, NaN last
        ref = np.argsort(np.where(np.isnan(p), np.inf, p), kind="stable")
        assert (order[:, b] == ref).mean() > 0.99  # the reference's order up to near-ties of the last bits
