"""
The seeded synthetic inputs that stand in for the reference's datasets (CPU only): determinism, the stated shapes
and distributions (Binomial(2, MAF) dosages, contiguous chromosome blocks, human-proportional sizes, heritability
and causal-count ranges, missingness patterns) and the Blom rank-inverse-normal transform.
"""
from __future__ import annotations

import numpy as np
from scipy.stats import norm

from fasterlmm_gb300.synth import HUMAN_CHROM_MB, chrom_sizes_human, make_dataset, rint_columns


def test_same_seed_same_data_and_config_ids_differ():
    a = make_dataset(60, 300, 3, 3, 4, seed=5, config_id=2)
    b = make_dataset(60, 300, 3, 3, 4, seed=5, config_id=2)
    c = make_dataset(60, 300, 3, 3, 4, seed=5, config_id=3)
    for k in ("G", "X", "Y", "chrom", "h2", "n_causal"):
        np.testing.assert_array_equal(getattr(a, k), getattr(b, k))
    assert not np.array_equal(a.G, c.G)


def test_shapes_and_distributions():
    N, M, B = 2000, 400, 30
    d = make_dataset(N, M, 4, 5, B, seed=9, maf_lo=0.2, h2_lo=0.1, h2_hi=0.6, k_lo=2, k_hi=7)
    assert d.G.shape == (N, M) and d.G.dtype == np.int8 and set(np.unique(d.G)) <= {0, 1, 2}
    assert d.X.shape == (N, 5) and np.all(d.X[:, 0] == 1.0)
    np.testing.assert_array_equal(d.chrom, np.repeat([1, 2, 3, 4], 100))
    # allele frequency of each variant near U[0.2, 0.5] (binomial noise of 2N draws)
    p = d.G.mean(axis=0) / 2
    assert p.min() > 0.2 - 4 * np.sqrt(0.25 / (2 * N)) and p.max() < 0.5 + 4 * np.sqrt(0.25 / (2 * N))
    assert np.all((d.h2 >= 0.1) & (d.h2 <= 0.6)) and np.all((d.n_causal >= 2) & (d.n_causal <= 7))
    assert d.Y.shape == (N, B) and not np.isnan(d.Y).any()


def test_missing_calls_and_phenotype_na_patterns():
    d = make_dataset(300, 200, 2, 3, 40, seed=4, geno_missing_rate=0.02, pheno_na_patterns=4)
    frac = (d.G == -1).mean()
    assert 0.01 < frac < 0.03
    assert np.isnan(d.Z_float()).sum() == (d.G == -1).sum()
    patterns = {np.isnan(d.Y[:, b]).tobytes() for b in range(d.Y.shape[1])}
    assert 1 < len(patterns) <= 4
    assert np.zeros(300, dtype=bool).tobytes() in patterns  # pattern 0: no missing values


def test_human_chromosome_sizes():
    sizes = chrom_sizes_human(500_000)
    assert len(sizes) == 22 and sum(sizes) == 500_000
    w = np.asarray(HUMAN_CHROM_MB, dtype=np.float64)
    np.testing.assert_allclose(np.asarray(sizes), 500_000 * w / w.sum(), atol=1.0)


def test_rint_is_blom_on_ranks_with_nan_kept():
    rng = np.random.default_rng(1)
    Y = rng.gamma(2.0, size=(50, 3))
    Y[[3, 7], 1] = np.nan
    Y[:, 2] = np.round(Y[:, 2])  # ties: average ranks
    R = rint_columns(Y)
    n = 50
    np.testing.assert_allclose(np.sort(R[:, 0]), norm.ppf((np.arange(1, n + 1) - 0.375) / (n + 0.25)), rtol=0, atol=1e-12)
    assert np.isnan(R[[3, 7], 1]).all() and not np.isnan(np.delete(R[:, 1], [3, 7])).any()
    m = 48
    np.testing.assert_allclose(np.sort(np.delete(R[:, 1], [3, 7])), norm.ppf((np.arange(1, m + 1) - 0.375) / (m + 0.25)),
                               atol=1e-12)
    # tied inputs map to one value
    for v in np.unique(Y[:, 2]):
        assert np.ptp(R[Y[:, 2] == v, 2]) == 0.0
