"""
Parity of the split-precision scan where the -log10 p gate is tightest: strong single-variant associations.

-log10 p grows like F / (2 ln 10), so the 1e-3 gate asks for a relative F error below ~5e-3 / F; the FP32 form of
rss = rWr - sWy^2 / sWs loses accuracy like F / df on top of that.  The fast form therefore recomputes every real
test above REFINE_F without the cancelling subtraction (flmm_wald_refine_f32).  These tests hold it to the gate
with half of it to spare:

* N = 1,000 (the headline sample size), three chromosomes of 5,000 variants, single causal variants with h2 from
  0.8 to 0.95 plus polygenic and null phenotypes, ten permutations each, against the oracle (the reference's
  algorithm in FP64 numpy; test infrastructure only) -- RINT-transformed as the CLI does, and raw (F up to ~2e4);
* N = 5,000, three chromosomes of 3,000 variants, against the reference's own FP64 run (tests/golden/strong_n5000.npz,
  inputs regenerated by tests/strong_inputs.py).

Gates: beta and SE within 1e-5 relative (1e-6 absolute floor), |d(-log10 p)| <= 5e-4 on every real test, each
phenotype's ten strongest variants in the same order, the permutation thresholds (the 0.05 quantile of the
permutation minimum p, fasterlmm/cli.py:128) within 1e-4 in -log10, and the same significance calls (p < threshold)
except for tests within the gate of the threshold.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import GOLDEN
from parity import GATE, check_gates, neg_log10_p_gpu
from strong_inputs import N5000, genotype_checksum, strong_dataset

pytestmark = pytest.mark.gpu

SPECS_1000 = [(0.95, 1, 1), (0.9, 1, 2), (0.8, 1, 3), (0.95, 2, 1), (0.6, 3, 2), (0.5, 10, 3), (0.3, 40, 1),
              (0.0, 0, 2)]


def _run_fast(G, X, Y, chrom, n_perm):
    from fasterlmm_gb300 import perms
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    data = SimpleNamespace(Z=t(G.astype(np.float64)), Y=t(Y), X=t(X), chrom=chrom, Z_kin=None, chrom_kin=None)
    res, pmf = perms.perm_threshold(data, list(range(Y.shape[1])), n_perm=n_perm, form="fast")
    torch.cuda.synchronize()
    out = {k: getattr(res, k).cpu().numpy() for k in ("f", "beta", "se", "sfve", "max_F")}
    out["perm_max_F"] = pmf.cpu().numpy()
    return out


def _case_1000(rint: bool):
    G, X, Y, chrom = strong_dataset(1000, [5000, 5000, 5000], 5, SPECS_1000, seed=4242, rint=rint)
    got = _run_fast(G, X, Y, chrom, 10)
    ref, rpmf = orc.perm_threshold(G.astype(np.float64), X, Y, chrom, range(Y.shape[1]), n_perm=10)
    ref = dict(ref)
    ref["perm_max_F"] = rpmf
    return G, X, Y, chrom, got, ref


@pytest.fixture(scope="module")
def case_rint():
    return _case_1000(True)


@pytest.fixture(scope="module")
def case_raw():
    return _case_1000(False)


def test_strong_single_variant_n1000_rint(case_rint):
    *_, got, ref = case_rint
    assert ref["f"].max() > 2000  # the case does reach the tight end of the gate
    check_gates(got, ref, 1000 - 5 - 1, "N=1000 RINT")


def test_strong_single_variant_n1000_raw(case_raw):
    *_, got, ref = case_raw
    assert ref["f"].max() > 10000
    check_gates(got, ref, 1000 - 5 - 1, "N=1000 raw")


def test_reevaluation_is_what_closes_the_gate(case_raw):
    """The same scan without the re-evaluation misses the gate on the strongest tests; with it the error drops."""
    from fasterlmm_gb300 import fast
    G, X, Y, chrom, got, ref = case_raw
    saved = fast.REFINE_F
    fast.REFINE_F = None
    try:
        plain = _run_fast(G, X, Y, chrom, 10)
    finally:
        fast.REFINE_F = saved
    df2 = 1000 - 5 - 1
    e_with = np.abs(neg_log10_p_gpu(got["f"], df2) - neg_log10_p_gpu(ref["f"], df2)).max()
    e_without = np.abs(neg_log10_p_gpu(plain["f"], df2) - neg_log10_p_gpu(ref["f"], df2)).max()
    print(f"max |d(-log10 p)|: {e_without:.3e} without the re-evaluation, {e_with:.3e} with it")
    assert e_with < e_without and e_without > GATE


def test_full_list_falls_back_to_the_chromosome_scan(case_rint):
    """A list too small for the strong tests gives the same outputs through the overflow scan (bit for bit)."""
    from fasterlmm_gb300 import fast
    G, X, Y, chrom, got, _ = case_rint
    saved = fast.REFINE_CAP
    fast.REFINE_CAP = 3
    try:
        small = _run_fast(G, X, Y, chrom, 10)
    finally:
        fast.REFINE_CAP = saved
    for k in got:
        np.testing.assert_array_equal(small[k], got[k], err_msg=k)


def test_strong_signals_n5000_against_reference_golden():
    c = N5000
    with np.load(GOLDEN / "strong_n5000.npz") as z:
        want = {k: z[k] for k in z.files}
    G, X, Y, chrom = strong_dataset(c["N"], c["sizes"], c["D"], c["specs"], seed=c["seed"])
    assert genotype_checksum(G) == int(want["g_checksum"]), "regenerated genotypes differ from the fixture's"
    np.testing.assert_allclose(X, want["X"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(Y, want["Y"], rtol=0, atol=1e-12)
    got = _run_fast(G, X, Y, chrom, c["n_perm"])
    assert want["f"].max() > 5000
    check_gates(got, want, c["N"] - c["D"] - 1, "N=5000")
