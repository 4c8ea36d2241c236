"""
Seeded synthetic GWAS inputs with the shapes of the scan workloads.

No public dataset is used: genotypes, covariates and phenotypes are drawn here from a fixed seed, following the
recipe of the reference's toy simulator (fasterlmm/sim.py:21-28) widened to per-variant allele frequencies, per
phenotype causal counts and heritabilities, and the Blom rank-inverse-normal transform the CLI applies to
phenotypes (fasterlmm/normalize.py:21-52).

Genotypes are returned as int8 dosages 0/1/2 with -1 marking a missing call, sample-major (N, M), the layout of
the reference's ``AlignedDataset.Z`` (fasterlmm/io.py:123-140) before it is cast to float with NaN for missing.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np

MISSING = -1

# human autosome lengths in Mb (GRCh38, rounded); variant counts of the uneven-chromosome workload are made
# proportional to these
HUMAN_CHROM_MB = [248, 242, 198, 190, 181, 171, 159, 145, 138, 134, 135, 133, 114, 107, 102, 90, 83, 80, 59, 64,
                  47, 51]


@dataclass
class SynthData:
    G: np.ndarray          # (N, M) int8 dosages, -1 = missing
    X: np.ndarray          # (N, D) float64, [intercept | N(0,1) covariates]
    Y: np.ndarray          # (N, B) float64 phenotypes after RINT (NaN where missing)
    chrom: np.ndarray      # (M,) int chromosome label per variant, contiguous blocks 1..n_chrom
    h2: np.ndarray         # (B,) simulated heritability per phenotype
    n_causal: np.ndarray   # (B,) causal variant count per phenotype

    def Z_float(self) -> np.ndarray:
        """(N, M) float64 dosages with NaN for missing calls, the reference's input convention."""
        Z = self.G.astype(np.float64)
        Z[self.G == MISSING] = np.nan
        return Z


def rint_columns(Y: np.ndarray, c: float = 3.0 / 8.0) -> np.ndarray:
    """Blom RINT per column, average ties, NaN kept (fasterlmm/normalize.py:21-52)."""
    from scipy.stats import norm, rankdata
    Y = np.asarray(Y, dtype=np.float64)
    out = np.full_like(Y, np.nan)
    for j in range(Y.shape[1]):
        y = Y[:, j]
        mask = ~np.isnan(y)
        n = int(mask.sum())
        if n == 0:
            continue
        ranks = rankdata(y[mask], method="average")
        out[mask, j] = norm.ppf((ranks - c) / (n - 2 * c + 1))
    return out


def _for_blocks(fn, starts, threads: int) -> None:
    """fn(j0) for every block start, on ``threads`` host threads (numpy releases the GIL in the block work)."""
    starts = list(starts)
    if threads <= 1:
        for j0 in starts:
            fn(j0)
        return
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(threads) as ex:
        list(ex.map(fn, starts))


def _bernoulli_pair_blocks(G: np.ndarray, maf: np.ndarray, step: int, key: tuple, threads: int) -> None:
    N, M = G.shape

    def draw(j0):
        j1 = min(M, j0 + step)
        r = np.random.Generator(np.random.PCG64(np.random.SeedSequence([*key, 1, j0 // step])))
        p = maf[j0:j1]
        blk = (r.random((N, j1 - j0)) < p).astype(np.int8)
        blk += (r.random((N, j1 - j0)) < p).astype(np.int8)
        G[:, j0:j1] = blk

    _for_blocks(draw, range(0, M, step), threads)


def chrom_sizes_even(M: int, n_chrom: int) -> list[int]:
    base, extra = divmod(M, n_chrom)
    return [base + (1 if i < extra else 0) for i in range(n_chrom)]


def chrom_sizes_human(M: int, n_chrom: int = 22) -> list[int]:
    w = np.asarray(HUMAN_CHROM_MB[:n_chrom], dtype=np.float64)
    sizes = np.floor(M * w / w.sum()).astype(int)
    sizes[: M - sizes.sum()] += 1
    return sizes.tolist()


def make_dataset(N: int, M: int, n_chrom: int, D: int, B: int, *, seed: int = 19930909, config_id: int = 0,
                 maf_lo: float = 0.05, h2_lo: float = 0.1, h2_hi: float = 0.8, k_lo: int = 5, k_hi: int = 5,
                 chrom_sizes: list[int] | None = None, geno_missing_rate: float = 0.0,
                 pheno_na_patterns: int = 0, na_frac_hi: float = 0.4, rint: bool = True,
                 block_threads: int = 0) -> SynthData:
    """
    Draw one synthetic dataset.

    Genotypes: Binomial(2, p_j) with p_j ~ U[maf_lo, 0.5]; optional missing calls at ``geno_missing_rate``.
    ``block_threads`` > 0 draws them instead as two Bernoulli(p_j) uniforms per call, each block of 8,192 variants
    from its own PCG64 stream (SeedSequence [seed, config_id, 1, block]) on that many host threads -- the same
    distribution, ~50x faster for the 2.5e9-call workload, independent of the thread count.
    Covariates: intercept plus D - 1 standard normals.  Phenotypes: k ~ U{k_lo..k_hi} causal variants, effects
    N(0, 1), genetic value rescaled to variance h2 (h2 ~ U[h2_lo, h2_hi]; k = 0 or h2 = 0 gives no genetic part),
    noise N(0, 1 - h2), then RINT.  ``pheno_na_patterns`` > 0 assigns each phenotype one of that many missingness
    patterns (pattern 0 has none, the others drop up to ``na_frac_hi`` of the samples).
    """
    rng = np.random.default_rng([seed, config_id])
    sizes = chrom_sizes if chrom_sizes is not None else chrom_sizes_even(M, n_chrom)
    assert sum(sizes) == M
    chrom = np.repeat(np.arange(1, len(sizes) + 1), sizes)
    maf = rng.uniform(maf_lo, 0.5, size=M)
    G = np.empty((N, M), dtype=np.int8)
    step = 8192
    if block_threads > 0:
        _bernoulli_pair_blocks(G, maf, step, (seed, config_id), block_threads)
    else:
        for j0 in range(0, M, step):
            j1 = min(M, j0 + step)
            G[:, j0:j1] = rng.binomial(2, maf[j0:j1], size=(N, j1 - j0)).astype(np.int8)
    if geno_missing_rate > 0:
        miss = rng.random((N, M)) < geno_missing_rate
        G[miss] = MISSING
    X = np.concatenate([np.ones((N, 1)), rng.standard_normal((N, D - 1))], axis=1)

    # per-variant stats over observed calls, used only to standardise the causal columns (in column blocks, so the
    # FP64 copy never holds more than `step` columns)
    obs = G != MISSING
    mu = np.empty(M)
    sd = np.empty(M)

    def stats(j0):
        j1 = min(M, j0 + step)
        Gf = G[:, j0:j1].astype(np.float64)
        ob = obs[:, j0:j1]
        n_obs = np.maximum(ob.sum(axis=0), 1)
        m = np.where(ob, Gf, 0.0).sum(axis=0) / n_obs
        mu[j0:j1] = m
        sd[j0:j1] = np.sqrt(np.where(ob, (Gf - m) ** 2, 0.0).sum(axis=0) / n_obs)

    _for_blocks(stats, range(0, M, step), block_threads)
    sd = np.clip(sd, 1e-12, None)

    h2 = rng.uniform(h2_lo, h2_hi, size=B)
    n_causal = rng.integers(k_lo, k_hi + 1, size=B)
    Y = np.empty((N, B))
    for b in range(B):
        k = int(n_causal[b])
        e = rng.standard_normal(N) * np.sqrt(1.0 - h2[b])
        if k == 0 or h2[b] == 0.0:
            Y[:, b] = e
            continue
        idx = rng.choice(M, size=k, replace=False)
        Zc = np.where(obs[:, idx], (G[:, idx] - mu[idx]) / sd[idx], 0.0)
        g = Zc @ rng.standard_normal(k)
        gs = g.std()
        Y[:, b] = (g / gs * np.sqrt(h2[b]) if gs > 0 else 0.0) + e
    if pheno_na_patterns > 0:
        masks = [np.zeros(N, dtype=bool)]
        for _ in range(pheno_na_patterns - 1):
            frac = rng.uniform(0.0, na_frac_hi)
            masks.append(rng.random(N) < frac)
        pat = rng.integers(0, pheno_na_patterns, size=B)
        for b in range(B):
            Y[masks[pat[b]], b] = np.nan
    if rint:
        Y = rint_columns(Y)
    return SynthData(G=G, X=X, Y=Y, chrom=chrom, h2=h2, n_causal=n_causal)


# the scan workloads, by name: (N, M, n_chrom, D, B, n_perm, grid) and the generator keywords
WORKLOADS = {
    # 150 samples x 1,500 variants over 16 chromosomes, 20 phenotypes x 100 permutations, 100-point grid on [-5, 5]
    "n150_m1500_b20_perm100": dict(N=150, M=1500, n_chrom=16, D=3, B=20, n_perm=100, n_grid=100,
                                   log_delta_min=-5.0, log_delta_max=5.0,
                                   gen=dict(maf_lo=0.05, h2_lo=0.1, h2_hi=0.8, k_lo=5, k_hi=5, config_id=1)),
    # 1,000 samples x 100,000 variants over 20 chromosomes, 6,484 phenotypes x 10 permutations, default grid
    "n1000_m100k_b6484_perm10": dict(N=1000, M=100_000, n_chrom=20, D=5, B=6484, n_perm=10, n_grid=64,
                                     log_delta_min=-10.0, log_delta_max=10.0,
                                     gen=dict(maf_lo=0.01, h2_lo=0.0, h2_hi=0.9, k_lo=0, k_hi=50, config_id=2)),
    # uneven batching: 5,000 samples x 500,000 variants over 22 chromosomes sized like the human autosomes, 2,000
    # phenotypes in 12 missingness patterns (each pattern but the first drops up to 40 % of the samples, so groups
    # have 3,000-5,000 samples); the first 50 phenotypes get 1,000 permutations (n_perm_hi), the rest 10
    "n5000_m500k_b2000_na12": dict(N=5000, M=500_000, n_chrom=22, D=5, B=2000, n_perm=10, n_grid=64,
                                   log_delta_min=-10.0, log_delta_max=10.0, B_hi=50, n_perm_hi=1000, human=True,
                                   gen=dict(maf_lo=0.01, h2_lo=0.0, h2_hi=0.9, k_lo=0, k_hi=50, config_id=3,
                                            pheno_na_patterns=12, na_frac_hi=0.4, block_threads=16)),
}


def make_workload(name: str, *, seed: int = 19930909, B: int | None = None, M: int | None = None) -> tuple[SynthData, dict]:
    """Generate a named workload; ``B`` / ``M`` shrink it for bounded samples (same generator, same seed)."""
    w = dict(WORKLOADS[name])
    gen = dict(w.pop("gen"))
    if B is not None:
        w["B"] = B
    if M is not None:
        w["M"] = M
    if w.get("human"):
        gen["chrom_sizes"] = chrom_sizes_human(w["M"], w["n_chrom"])
    data = make_dataset(w["N"], w["M"], w["n_chrom"], w["D"], w["B"], seed=seed, **gen)
    return data, w


# The low-rank large-cohort shape: a kinship factor of k markers and M tested variants over 22 human-sized
# chromosomes, N samples, B phenotypes (h2 ~ U[0.1, 0.7], 10 causal tested variants each); the permutation columns
# are drawn by the scan's driver.
LOWRANK_WORKLOADS = {
    "n50000_k2000_m1m_b100_perm10": dict(N=50_000, k_kin=2_000, M=1_000_000, n_chrom=22, D=5, B=100, n_perm=10,
                                         n_grid=64, log_delta_min=-10.0, log_delta_max=10.0, config_id=5),
}


@dataclass
class LowRankData:
    Gt: np.ndarray         # (M, N) int8 tested dosages, variant-major (a block of variants is contiguous)
    chrom: np.ndarray      # (M,) chromosome of each tested variant, contiguous blocks 1..n_chrom
    Gk: np.ndarray         # (N, k) int8 kinship-factor dosages
    chrom_kin: np.ndarray  # (k,) chromosome of each kinship marker
    X: np.ndarray          # (N, D)
    Y: np.ndarray          # (N, B) after RINT


def _variant_major_blocks(M: int, N: int, maf: np.ndarray, key: tuple, threads: int, step: int = 2048) -> np.ndarray:
    """(M, N) int8 Binomial(2, maf_m) dosages as two Bernoulli draws per call, each block of `step` variants from
    its own PCG64 stream (SeedSequence [*key, block]); independent of the thread count."""
    Gt = np.empty((M, N), dtype=np.int8)

    def draw(m0):
        m1 = min(M, m0 + step)
        r = np.random.Generator(np.random.PCG64(np.random.SeedSequence([*key, m0 // step])))
        p = maf[m0:m1, None]
        blk = (r.random((m1 - m0, N)) < p).astype(np.int8)
        blk += (r.random((m1 - m0, N)) < p).astype(np.int8)
        Gt[m0:m1] = blk

    _for_blocks(draw, range(0, M, step), threads)
    return Gt


def make_lowrank_workload(name: str, *, seed: int = 19930909, M: int | None = None, B: int | None = None,
                          threads: int = 16) -> tuple[LowRankData, dict]:
    w = dict(LOWRANK_WORKLOADS[name])
    if M is not None:
        w["M"] = M
    if B is not None:
        w["B"] = B
    N, k, Mv, nc, D, Bn = w["N"], w["k_kin"], w["M"], w["n_chrom"], w["D"], w["B"]
    rng = np.random.default_rng([seed, w["config_id"]])
    sizes, sizes_k = chrom_sizes_human(Mv, nc), chrom_sizes_human(k, nc)
    chrom = np.repeat(np.arange(1, nc + 1), sizes)
    chrom_kin = np.repeat(np.arange(1, nc + 1), sizes_k)
    maf = rng.uniform(0.05, 0.5, size=Mv)
    maf_k = rng.uniform(0.05, 0.5, size=k)
    Gt = _variant_major_blocks(Mv, N, maf, (seed, w["config_id"], 1), threads)
    Gk = np.ascontiguousarray(_variant_major_blocks(k, N, maf_k, (seed, w["config_id"], 2), threads).T)
    X = np.concatenate([np.ones((N, 1)), rng.standard_normal((N, D - 1))], axis=1)
    Y = np.empty((N, Bn))
    h2 = rng.uniform(0.1, 0.7, size=Bn)
    for b in range(Bn):
        idx = rng.choice(Mv, size=10, replace=False)
        Zc = Gt[idx].astype(np.float64)
        Zc = (Zc - Zc.mean(axis=1, keepdims=True)) / np.clip(Zc.std(axis=1, keepdims=True), 1e-12, None)
        g = Zc.T @ rng.standard_normal(10)
        Y[:, b] = g / g.std() * np.sqrt(h2[b]) + rng.standard_normal(N) * np.sqrt(1.0 - h2[b])
    return LowRankData(Gt=Gt, chrom=chrom, Gk=Gk, chrom_kin=chrom_kin, X=X, Y=rint_columns(Y)), w
