"""
GPU parity of the grouped scan (uneven batching): phenotypes in four missingness patterns over 1,600 samples, each
pattern scanned on its own strain subset (groups of 1,057 to 1,600 samples), three phenotypes with forty
permutations among phenotypes with five, against the reference's own FP64 runs (tests/golden/na_groups_n1600.npz,
one perm_threshold per pattern and permutation count; inputs regenerated by tests/strong_inputs.py).

The grouped driver runs each pattern's permutation counts in one joint scan; these tests hold every split result
to the parity gates (beta and SE within rtol 1e-5 / atol 1e-6, |d(-log10 p)| <= 5e-4, top hits, permutation
thresholds), both numeric forms, and the joint scan bit for bit to separate per-count scans.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import GOLDEN
from parity import assert_scan_close, check_gates
from strong_inputs import NA1600, genotype_checksum, na_dataset

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case():
    c = NA1600
    with np.load(GOLDEN / "na_groups_n1600.npz") as z:
        want = {k: z[k] for k in z.files}
    G, X, Y, chrom = na_dataset(c)
    assert genotype_checksum(G) == int(want["g_checksum"]), "regenerated genotypes differ from the fixture's"
    np.testing.assert_allclose(X, want["X"], rtol=0, atol=1e-12)
    np.testing.assert_allclose(Y, want["Y"], rtol=0, atol=1e-12, equal_nan=True)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    data = SimpleNamespace(Z=t(G.astype(np.float64)), Y=t(Y), X=t(X), chrom=chrom, Z_kin=None, chrom_kin=None)
    return c, data, want


def _grouped(case, form):
    from fasterlmm_gb300.groups import perm_threshold_grouped
    c, data, want = case
    out = perm_threshold_grouped(data, list(range(len(c["specs"]))), n_perm=c["n_perm"], n_perm_of=c["n_perm_of"],
                                 form=form)
    torch.cuda.synchronize()
    assert len(out) == int(want["n_runs"])
    return out


def _np(g):
    d = {k: getattr(g.res, k).cpu().numpy() for k in ("f", "beta", "se", "sfve", "max_F")}
    d["perm_max_F"] = g.perm_max_F.cpu().numpy()
    return d


@pytest.mark.parametrize("form", ["fast", "plain"])
def test_grouped_scan_matches_reference_runs(case, form):
    c, _, want = case
    D = c["D"]
    for r, g in enumerate(_grouped(case, form)):
        assert g.keep == want[f"r{r}_keep"].tolist() and g.cols == want[f"r{r}_cols"].tolist()
        assert g.n_perm == int(want[f"r{r}_n_perm"]) and g.perm_max_F.shape == (len(g.cols), g.n_perm)
        got = _np(g)
        ref = {k: want[f"r{r}_{k}"] for k in ("f", "beta", "se", "sfve", "max_F", "perm_max_F")}
        assert_scan_close(got, ref, keys=("f", "beta", "se", "sfve", "max_F", "perm_max_F"))
        check_gates(got, ref, len(g.keep) - D - 1, f"{form} run {r} ({len(g.keep)} samples, {g.n_perm} perms)")
        ld = np.stack([v.cpu().numpy() for _, v in sorted(g.res.log_delta.items())])
        assert ld.shape == want[f"r{r}_log_delta"].shape


def test_joint_count_scan_equals_separate_scans(case):
    """One scan of a pattern's mixed permutation counts gives the bits of one scan per count."""
    from fasterlmm_gb300 import perms
    from fasterlmm_gb300.groups import subset_dataset
    _, data, _ = case
    for g in _grouped(case, "fast"):
        sub = subset_dataset(data, g.keep, g.cols)
        res, pmf = perms.perm_threshold(sub, list(range(len(g.cols))), n_perm=g.n_perm, seed_idx=g.cols, form="fast")
        for k in ("f", "beta", "se", "sfve", "nullh2", "max_F"):
            np.testing.assert_array_equal(getattr(g.res, k).cpu().numpy(), getattr(res, k).cpu().numpy(), err_msg=k)
        np.testing.assert_array_equal(g.perm_max_F.cpu().numpy(), pmf.cpu().numpy())
