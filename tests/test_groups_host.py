"""
CPU tests of the grouped scan's host logic (fasterlmm/cli.py:351-375, fasterlmm/io.py:187-218): the NaN-pattern
grouping and the split of a pattern's columns by permutation count reproduce the runs the reference made for
tests/golden/na_groups_n1600.npz, and the oracle matches that fixture on its mixed-count pattern (which pins the
oracle at N >= 1,000 on a strain subset).
"""
from __future__ import annotations

import numpy as np

import flmm_oracle as orc
from conftest import GOLDEN
from parity import assert_scan_close
from strong_inputs import NA1600, na_dataset


def _fixture():
    with np.load(GOLDEN / "na_groups_n1600.npz") as z:
        return {k: z[k] for k in z.files}


def test_grouping_and_count_split_reproduce_the_reference_runs():
    from fasterlmm_gb300.groups import _count_sets, group_by_na
    c, want = NA1600, _fixture()
    _, _, Y, _ = na_dataset(c)
    runs = []
    for keep, cols in group_by_na(Y, range(Y.shape[1])):
        for js, k in _count_sets(cols, c["n_perm"], c["n_perm_of"]):
            runs.append((keep, [cols[j] for j in js], k))
    assert len(runs) == int(want["n_runs"])
    for r, (keep, cols, k) in enumerate(runs):
        assert keep == want[f"r{r}_keep"].tolist()
        assert cols == want[f"r{r}_cols"].tolist()
        assert k == int(want[f"r{r}_n_perm"])


def test_count_sets_order_and_defaults():
    from fasterlmm_gb300.groups import _count_sets
    assert _count_sets([7, 3, 9, 4], 10, None) == [([0, 1, 2, 3], 10)]
    assert _count_sets([7, 3, 9, 4], 10, {3: 1000, 4: 0}) == [([0, 2], 10), ([1], 1000), ([3], 0)]


def test_oracle_matches_the_reference_on_a_mixed_count_pattern():
    c, want = NA1600, _fixture()
    G, X, Y, chrom = na_dataset(c)
    r = 3  # the 1,057-sample pattern's forty-permutation column
    keep, cols, n_perm = want[f"r{r}_keep"], want[f"r{r}_cols"].tolist(), int(want[f"r{r}_n_perm"])
    Zk = G[keep].astype(np.float64)
    got, pmf = orc.perm_threshold(Zk, X[keep], Y[keep][:, cols], chrom, range(len(cols)), n_perm=n_perm,
                                  seed_idx=cols)
    got = dict(got)
    got["perm_max_F"] = pmf
    assert_scan_close(got, want, keys=("f", "beta", "se", "sfve", "max_F", "perm_max_F"), prefix=f"r{r}_")
