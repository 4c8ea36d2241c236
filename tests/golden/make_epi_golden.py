"""
Generate tests/golden/epi_batched.npz: outputs of the reference's batched epistasis Wald scan
(``fasterlmm_lux.epi._kernel.snp_wald_scan_batched``, lux/src/fasterlmm_lux/epi/_kernel.py:21-150), run by the
reference itself on CPU in FP64 on seeded inputs.

Usage (in a checkout where the reference is present):
    python tests/golden/make_epi_golden.py [--reference PATH]

The reference's lux package is imported from PATH/lux/src (default: the FASTERLMM_REFERENCE environment variable).
Cases: a generic one with several anchor, phenotype and SNP chunks and a real/permutation split; one where some test
columns are (nearly) collinear with the anchor column, so the rank-deficiency guard zeroes their F (and one with the
guard off); one with 40 covariate columns plus the anchor, as the tier-2 scan runs with many covariates.
"""

from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def make_case(seed: int, K: int, N: int, C: int, P: int, M: int, collinear: int = 0) -> dict:
    rng = np.random.default_rng(seed)
    s = np.sort(rng.gamma(1.0, 1.0, N))[::-1].copy()
    X = rng.standard_normal((K, N, C))
    X[:, :, 0] = 1.0 / np.sqrt(N) * np.sign(rng.standard_normal(N))  # a rotated intercept-like column
    Y = rng.standard_normal((N, P))
    ld = rng.uniform(-3.0, 4.0, P)
    S = rng.standard_normal((K, N, M))
    for k in range(K):
        for j in range(collinear):
            # test column = anchor column (last design column) plus a little noise: denom ~ 0
            S[k, :, j] = X[k, :, -1] * (1.0 + 0.1 * j) + 1e-3 * j * rng.standard_normal(N)
    return dict(s=s, X=X, Y=Y, ld=ld, S=S)


CASES = {
    "generic": dict(seed=11, K=3, N=120, C=5, P=9, M=70, n_real=6, snp_chunk=32, pheno_chunk=4, floor=0.01),
    "collinear": dict(seed=12, K=2, N=90, C=4, P=5, M=40, n_real=5, snp_chunk=16, pheno_chunk=5, floor=0.01,
                      collinear=3),
    "collinear_noguard": dict(seed=12, K=2, N=90, C=4, P=5, M=40, n_real=5, snp_chunk=16, pheno_chunk=5, floor=0.0,
                              collinear=3),
    "wide": dict(seed=13, K=2, N=200, C=41, P=6, M=50, n_real=3, snp_chunk=64, pheno_chunk=6, floor=0.01),
}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH or set FASTERLMM_REFERENCE")
    sys.path.insert(0, str(Path(args.reference) / "lux" / "src"))
    import torch
    from fasterlmm_lux.epi._kernel import snp_wald_scan_batched
    out = {}
    for name, c in CASES.items():
        inp = make_case(c["seed"], c["K"], c["N"], c["C"], c["P"], c["M"], c.get("collinear", 0))
        t = {k: torch.from_numpy(v) for k, v in inp.items()}
        beta, se, chi2, max_f, argmax = snp_wald_scan_batched(
            t["s"], t["X"], t["Y"], t["ld"], t["S"], snp_chunk=c["snp_chunk"], pheno_chunk=c["pheno_chunk"],
            n_real=c["n_real"], denom_floor_rel=c["floor"])
        for k, v in inp.items():
            out[f"{name}/{k}"] = v
        for k, v in dict(beta=beta, se=se, chi2=chi2, max_f=max_f, argmax=argmax).items():
            out[f"{name}/out_{k}"] = v.numpy()
        for k in ("n_real", "snp_chunk", "pheno_chunk", "floor"):
            out[f"{name}/{k}"] = np.asarray(c[k])
    np.savez_compressed(HERE / "epi_batched.npz", **out)
    print("wrote", HERE / "epi_batched.npz")


if __name__ == "__main__":
    main()
