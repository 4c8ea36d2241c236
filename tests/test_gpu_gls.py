"""
GPU parity of the plain GLS path (fasterlmm/core.py:89-451) against the reference's own outputs
(tests/golden/plain_*.npz) and the oracle, at the reference's parity tolerance; log delta by loss equivalence.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import z_float
from parity import DETAIL, assert_log_delta_equivalent_gls, assert_scan_close

pytestmark = pytest.mark.gpu
DEV = "cuda"


@pytest.fixture(scope="module", autouse=True)
def _built():
    from fasterlmm_gb300 import build
    build()


def _np(res) -> dict:
    return {k: getattr(res, k).detach().cpu().numpy() for k in DETAIL + ("max_F",)}


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def test_gls_components_match_golden(golden):
    from fasterlmm_gb300 import gls
    g = golden("plain_components")
    spec = gls.rotate(_t(g["K"]), _t(g["X"]), _t(g["Y"]))
    np.testing.assert_allclose(spec.s.cpu().numpy(), g["s"], rtol=1e-7, atol=1e-10)
    np.testing.assert_allclose(spec.X_rot.cpu().numpy() ** 2, g["X_rot"] ** 2, rtol=1e-7, atol=1e-10)
    np.testing.assert_allclose(spec.Y_rot.cpu().numpy() ** 2, g["Y_rot"] ** 2, rtol=1e-7, atol=1e-10)
    # the reference's own spectrum, passed as CPU tensors through the drop-in signatures
    ref = gls.Spectrum(s=torch.from_numpy(g["s"]), U=torch.from_numpy(g["U"]), X_rot=torch.from_numpy(g["X_rot"]),
                       Y_rot=torch.from_numpy(g["Y_rot"]))
    grid = torch.linspace(-10.0, 10.0, 64, dtype=torch.float64)
    for reml, key in ((False, "ml"), (True, "reml")):
        loss = gls._profile_loss(grid, ref.s, ref.X_rot, ref.Y_rot, reml=reml)
        assert loss.device.type == "cpu"
        np.testing.assert_allclose(loss.numpy(), g[f"grid_loss_{key}"], rtol=1e-10, atol=1e-8)
        ld_grid = gls.fit_delta_grid(ref, refine=False, reml=reml)
        assert np.array_equal(ld_grid.numpy(), g[f"log_delta_{key}_grid"])
        ld = gls.fit_delta_grid(ref, reml=reml)
        assert_log_delta_equivalent_gls(ld.numpy(), g[f"log_delta_{key}"], g["s"], g["X_rot"], g["Y_rot"], reml=reml)
        per = gls._profile_loss_per_pheno(ld, ref.s, ref.X_rot, ref.Y_rot, reml=reml)
        np.testing.assert_allclose(per.numpy(), orc.profile_loss_per_pheno(ld.numpy(), g["s"], g["X_rot"], g["Y_rot"],
                                                                           reml=reml), rtol=1e-10)
    for i, dl in enumerate(g["nll_delta"]):
        for p in range(g["Y"].shape[1]):
            v = gls.nLLeval(float(dl), ref.s, ref.X_rot, ref.Y_rot[:, p])
            assert v.ndim == 0
            np.testing.assert_allclose(v.item(), g["nll"][i, p], rtol=1e-10)
    S_rot = torch.from_numpy(g["U"].T @ g["Z_std"])
    res = gls.snp_wald_scan(ref, torch.from_numpy(g["log_delta_ml"]), S_rot, n_real=3)
    for k in DETAIL + ("max_F",):
        np.testing.assert_allclose(getattr(res, k).numpy(), g[k], rtol=1e-9, atol=1e-12, err_msg=k)


def test_gls_loco_and_single_k_match_golden(golden):
    from fasterlmm_gb300 import gls
    g = golden("plain_loco")
    Zs = _t(orc.standardise_columns(z_float(g["G"])))
    B = int(g["n_real"])
    seen = []
    res = gls.loco_scan(Zs, _t(g["X"]), _t(g["Y_all"]), g["chrom"], n_real=B, on_chrom=lambda k, n: seen.append((k, n)))
    n_chr = len(np.unique(g["chrom"]))
    assert seen == [(k + 1, n_chr) for k in range(n_chr)]
    assert_scan_close(_np(res), g)
    res1 = gls.single_k_scan(Zs, _t(g["X"]), _t(g["Y_all"]), n_real=B)
    assert_scan_close(_np(res1), g, prefix="sk_")
    with pytest.raises(ValueError):
        gls.loco_scan(Zs, _t(g["X"]), _t(g["Y_all"]), g["chrom"], Z_kin=Zs)


def test_gls_larger_random_case_matches_oracle():
    """Several tiles in every dimension, unsorted chromosomes, a kinship panel, more covariates."""
    from fasterlmm_gb300 import gls
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(210, 1300, 3, 7, 37, seed=2024, config_id=15, k_lo=0, k_hi=12, h2_lo=0.0, h2_hi=0.9)
    dk = make_dataset(210, 900, 3, 1, 1, seed=2025, config_id=16)
    perm = np.random.default_rng(4).permutation(1300)
    Zs = orc.standardise_columns(d.Z_float()[:, perm])
    chrom = d.chrom[perm]
    Zk = orc.standardise_columns(dk.Z_float())
    ref = orc.loco_scan(Zs, d.X, d.Y, chrom, n_real=30, Z_kin=Zk, chrom_kin=dk.chrom)
    res = gls.loco_scan(_t(Zs), _t(d.X), _t(d.Y), chrom, n_real=30, Z_kin=_t(Zk), chrom_kin=dk.chrom)
    assert_scan_close(_np(res), ref)


def test_gls_rejects_too_many_covariates():
    from fasterlmm_gb300 import _lib, gls
    N, C = 64, 31
    g = torch.Generator().manual_seed(0)
    X = torch.randn(N, C, generator=g, dtype=torch.float64)
    Z = torch.randn(N, 40, generator=g, dtype=torch.float64)
    spec = gls.rotate(_t((Z @ Z.T).numpy() / 40), _t(X.numpy()), _t(torch.randn(N, 2, generator=g, dtype=torch.float64).numpy()))
    with pytest.raises(_lib.FlmmError):
        gls.fit_delta_grid(spec)
