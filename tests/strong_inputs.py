"""
Seeded inputs with strong single-variant associations, drawn so that any numpy reproduces them exactly.

The parity tests of the split-precision scan at large F need inputs that the reference's own FP64 run has been
made on (tests/golden/make_strong_golden.py writes those outputs) while the inputs themselves are regenerated on
the test host instead of being stored.  Only ``Generator.random()`` of numpy's PCG64 is used -- the raw 53-bit
uniform, whose stream numpy keeps fixed -- and everything else is derived from those uniforms by elementary
transforms: Hardy-Weinberg genotypes by inverse CDF, normals by Box-Muller.  A checksum of the genotypes is stored
with the golden outputs so a host whose stream differed would fail loudly instead of comparing different data.

Phenotypes follow the reference's simulator recipe (fasterlmm/sim.py:21-28: standardised causal columns, normal
effects, genetic value rescaled to variance h2, noise of variance 1 - h2), with the causal variants of each
phenotype on one chosen chromosome, then the Blom rank-inverse-normal transform the CLI applies
(fasterlmm/normalize.py:21-52).
"""
from __future__ import annotations

import numpy as np


def _normals(rng: np.random.Generator, n: int) -> np.ndarray:
    u1 = 1.0 - rng.random(n)          # (0, 1]
    u2 = rng.random(n)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def _rint(y: np.ndarray, c: float = 3.0 / 8.0) -> np.ndarray:
    from scipy.stats import norm, rankdata
    ranks = rankdata(y, method="average")
    return norm.ppf((ranks - c) / (y.size - 2 * c + 1))


def genotype_checksum(G: np.ndarray) -> int:
    """Order-dependent checksum of an int8 dosage matrix (exact integer arithmetic)."""
    w = (np.arange(G.shape[1], dtype=np.int64) % 9973) + 1
    return int(((G.astype(np.int64) * w[None, :]).sum(axis=1) * (np.arange(G.shape[0], dtype=np.int64) % 7919 + 1)).sum())


def strong_dataset(N: int, sizes: list[int], D: int, specs: list[tuple[float, int, int]], *, seed: int,
                   rint: bool = True):
    """
    (G (N, M) int8, X (N, D), Y (N, B), chrom (M,)) for phenotypes specs[b] = (h2, k, c): k causal variants on
    chromosome c (1-based) explaining h2 of the variance (k = 0 or h2 = 0: noise only).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    M = int(sum(sizes))
    chrom = np.repeat(np.arange(1, len(sizes) + 1), sizes)
    maf = 0.05 + 0.45 * rng.random(M)
    G = np.empty((N, M), dtype=np.int8)
    for j0 in range(0, M, 4096):
        j1 = min(M, j0 + 4096)
        p = maf[j0:j1]
        u = rng.random((N, j1 - j0))
        G[:, j0:j1] = np.where(u < p * p, 2, np.where(u < 1.0 - (1.0 - p) ** 2, 1, 0)).astype(np.int8)
    X = np.concatenate([np.ones((N, 1)), _normals(rng, N * (D - 1)).reshape(D - 1, N).T], axis=1)
    starts = np.concatenate([[0], np.cumsum(sizes)])
    Y = np.empty((N, len(specs)))
    for b, (h2, k, c) in enumerate(specs):
        e = _normals(rng, N) * np.sqrt(1.0 - h2)
        if k == 0 or h2 == 0.0:
            Y[:, b] = e
        else:
            lo, hi = int(starts[c - 1]), int(starts[c])
            idx = lo + np.unique((rng.random(4 * k) * (hi - lo)).astype(np.int64))[:k]
            Zc = G[:, idx].astype(np.float64)
            Zc = (Zc - Zc.mean(axis=0)) / np.clip(Zc.std(axis=0), 1e-12, None)
            g = Zc @ _normals(rng, idx.size)
            Y[:, b] = g / g.std() * np.sqrt(h2) + e
        if rint:
            Y[:, b] = _rint(Y[:, b])
    return G, X, Y, chrom


# The N = 5,000 case of the golden fixture strong_n5000: three chromosomes of 3,000 variants (each LOCO kinship has
# rank 6,000 > N), two covariates, six phenotypes from a single strong variant to pure noise, ten permutations each.
N5000 = dict(N=5000, sizes=[3000, 3000, 3000], D=3,
             specs=[(0.95, 1, 1), (0.8, 1, 2), (0.9, 2, 3), (0.5, 10, 1), (0.3, 40, 2), (0.0, 0, 1)],
             seed=20250611, n_perm=10)


def na_patterns(N: int, B: int, n_patterns: int, *, frac_lo: float, frac_hi: float, seed: int) -> np.ndarray:
    """
    (B, N) bool missingness of each phenotype: pattern b % n_patterns, pattern 0 complete, pattern p > 0 drops each
    sample with a probability drawn from U[frac_lo, frac_hi] (raw uniforms of its own PCG64 stream).
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    masks = [np.zeros(N, dtype=bool)]
    for _ in range(n_patterns - 1):
        frac = frac_lo + (frac_hi - frac_lo) * rng.random()
        masks.append(rng.random(N) < frac)
    return np.stack([masks[b % n_patterns] for b in range(B)])


# The NaN-group case of the golden fixture na_groups_n1600: 1,600 samples in four missingness patterns (groups of
# about 1,000 to 1,600 samples), four chromosomes of 600-1,200 variants, twelve phenotypes, five permutations each
# except three phenotypes with forty (the uneven permutation counts of a mixed batch).
NA1600 = dict(N=1600, sizes=[1200, 1000, 800, 600], D=3,
              specs=[(0.9, 1, 1), (0.6, 3, 2), (0.5, 10, 3), (0.3, 20, 4), (0.8, 1, 2), (0.2, 5, 1),
                     (0.0, 0, 3), (0.7, 2, 4), (0.4, 8, 1), (0.5, 1, 3), (0.6, 15, 2), (0.1, 3, 4)],
              seed=16001600, na_seed=7700, n_patterns=4, frac_lo=0.1, frac_hi=0.35, n_perm=5,
              n_perm_of={0: 40, 5: 40, 10: 40})


def na_dataset(c: dict = NA1600):
    """(G, X, Y with NaN, chrom) of a NaN-group case."""
    G, X, Y, chrom = strong_dataset(c["N"], c["sizes"], c["D"], c["specs"], seed=c["seed"])
    miss = na_patterns(c["N"], Y.shape[1], c["n_patterns"], frac_lo=c["frac_lo"], frac_hi=c["frac_hi"],
                       seed=c["na_seed"])
    Y = Y.copy()
    Y[miss.T] = np.nan
    return G, X, Y, chrom


# The low-rank case of the golden fixture lowrank_n2000: 2,000 samples, a kinship factor of 400 markers on four
# chromosomes (each LOCO factor has rank ~300 < N, the reference's k < N branch), 3,000 tested variants on the same
# chromosomes, 3 covariates, 6 phenotypes kept in detail and 18 further columns that only feed max_F.
LR2000 = dict(N=2000, sizes=[900, 800, 700, 600], sizes_kin=[120, 110, 90, 80], D=3,
              specs=[(0.9, 1, 1), (0.6, 5, 2), (0.4, 20, 3), (0.8, 2, 4), (0.2, 10, 1), (0.0, 0, 2)],
              n_extra=18, seed=20002000, seed_kin=4004, seed_extra=606)


def lowrank_dataset(c: dict = LR2000):
    """(G test (N, M) int8, X, Y_all (N, B + n_extra), chrom, G_kin (N, k) int8, chrom_kin)."""
    G, X, Y, chrom = strong_dataset(c["N"], c["sizes"], c["D"], c["specs"], seed=c["seed"])
    Gk, _, _, chrom_kin = strong_dataset(c["N"], c["sizes_kin"], c["D"], [], seed=c["seed_kin"])
    rng = np.random.Generator(np.random.PCG64(c["seed_extra"]))
    extra = np.stack([_rint(_normals(rng, c["N"])) for _ in range(c["n_extra"])], axis=1)
    return G, X, np.concatenate([Y, extra], axis=1), chrom, Gk, chrom_kin
