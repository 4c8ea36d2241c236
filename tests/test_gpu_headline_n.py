"""
Parity at the headline sample size.  The golden fixtures are small (N = 150 .. 300); this runs the headline
workload's N = 1,000 samples on three of its chromosomes (15,000 variants) with 16 phenotypes x 10 permutations,
the fast form against the oracle (the reference's algorithm in FP64 numpy, test infrastructure only), and checks the
precision gates the port is held to: relative beta and SE error <= 1e-5 (with the reference's 1e-6 absolute floor),
|d(-log10 p)| <= 1e-3, permutation maxima and thresholds within 1e-4 in -log10 p with the same significance calls,
and every fitted log delta at least as good a fit as the oracle's (loss-equivalent to 1e-9 relative; flat likelihoods leave log delta itself loosely determined).
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import z_float
from parity import compat_loss

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline_case():
    from fasterlmm_gb300 import perms
    from fasterlmm_gb300.synth import make_workload
    d, _ = make_workload("n1000_m100k_b6484_perm10", B=16)
    mask = d.chrom <= np.unique(d.chrom)[2]
    G, chrom, Y, X = d.G[:, mask], d.chrom[mask], d.Y[:, :16], d.X
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    data = SimpleNamespace(Z=t(z_float(G)), Y=t(Y), X=t(X), chrom=chrom, Z_kin=None, chrom_kin=None)
    res, pmf = perms.perm_threshold(data, list(range(16)), n_perm=10, form="fast")
    ref, rpmf = orc.perm_threshold(z_float(G), X, Y, chrom, range(16), n_perm=10, keep_spectra=True)
    return X, res, pmf, ref, rpmf


def test_beta_and_se_within_1e5(headline_case):
    _, res, _, ref, _ = headline_case
    for k in ("beta", "se"):
        np.testing.assert_allclose(getattr(res, k).cpu().numpy(), ref[k], rtol=1e-5, atol=1e-6, err_msg=k)


def test_neg_log10_p_within_1e3(headline_case):
    from fasterlmm_gb300.post import neg_log10_pvalue
    X, res, pmf, ref, rpmf = headline_case
    df2 = X.shape[0] - X.shape[1] - 1
    got = neg_log10_pvalue(res.f, df2).cpu().numpy()
    want = neg_log10_pvalue(torch.from_numpy(ref["f"]).cuda(), df2).cpu().numpy()
    assert np.nanmax(np.abs(got - want)) <= 1e-3
    # the permutation maxima decide the thresholds: same order, -log10 p within the gate
    gp = neg_log10_pvalue(pmf, df2).cpu().numpy()
    wp = neg_log10_pvalue(torch.from_numpy(rpmf).cuda(), df2).cpu().numpy()
    assert np.nanmax(np.abs(gp - wp)) <= 1e-3
    assert (np.argsort(-gp, axis=1, kind="stable") == np.argsort(-wp, axis=1, kind="stable")).mean() > 0.99


def test_top_hits_identical(headline_case):
    """Each real phenotype's ten strongest variants, in order, up to ties within the -log10 p gate."""
    from fasterlmm_gb300.post import neg_log10_pvalue
    X, res, _, ref, _ = headline_case
    df2 = X.shape[0] - X.shape[1] - 1
    got = neg_log10_pvalue(res.f, df2).cpu().numpy()
    want = neg_log10_pvalue(torch.from_numpy(ref["f"]).cuda(), df2).cpu().numpy()
    for j in range(got.shape[1]):
        top_g = np.argsort(-got[:, j], kind="stable")[:10]
        top_w = np.argsort(-want[:, j], kind="stable")[:10]
        differ = top_g != top_w
        # a swapped pair is a tie: the oracle's own values at the two positions within the gate
        assert np.all(np.abs(want[top_g[differ], j] - want[top_w[differ], j]) <= 1e-3), j


def test_log_delta_is_as_good_a_fit(headline_case):
    _, res, _, ref, _ = headline_case
    for c, (s, UY) in ref["spectra"].items():
        ld = res.log_delta[c].cpu().numpy()
        La, Lb = compat_loss(ld, s, UY), compat_loss(ref["log_delta"][c], s, UY)
        assert np.all(La <= Lb + 1e-9 * np.abs(Lb)), c


def test_thresholds_and_calls_at_headline_n(headline_case):
    """The full gate set at the headline sample size: every permutation maximum within 1e-4 in -log10 p, each
    phenotype's 0.05-quantile permutation threshold (fasterlmm/cli.py:128) within 1e-4, and the same significance
    calls except for tests within the gate of the threshold (with beta / SE, the p gate and the top hits again)."""
    from parity import check_gates
    X, res, pmf, ref, rpmf = headline_case
    df2 = X.shape[0] - X.shape[1] - 1
    got = {k: getattr(res, k).cpu().numpy() for k in ("f", "beta", "se")}
    got["perm_max_F"] = pmf.cpu().numpy()
    want = {"f": ref["f"], "beta": ref["beta"], "se": ref["se"], "perm_max_F": rpmf}
    check_gates(got, want, df2, "headline N = 1,000")
