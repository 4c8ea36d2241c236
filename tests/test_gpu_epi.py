"""
The GPU batched epistasis Wald (fasterlmm_gb300.epi.snp_wald_scan_batched) against the reference's own outputs
(tests/golden/epi_batched.npz): the reference's chunking, real/permutation split, near-self guard and 41 design
columns.  Operands are split FP16 with FP32 sums, so the comparison is at 2e-5 relative with the reference's
absolute floors (beta, SE, F away from the planted collinear columns), with the guard's decisions, the maxima and
their columns identical.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

from test_epi_oracle import CASES, compare_epi

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", list(CASES))
def test_epi_batched_matches_reference(golden, case):
    from fasterlmm_gb300.epi import snp_wald_scan_batched
    g = golden("epi_batched")
    get = lambda k: g[f"{case}/{k}"]
    t = lambda k: torch.from_numpy(get(k))
    out = snp_wald_scan_batched(t("s"), t("X"), t("Y"), t("ld"), t("S"), snp_chunk=int(get("snp_chunk")),
                                pheno_chunk=int(get("pheno_chunk")), n_real=int(get("n_real")),
                                denom_floor_rel=float(get("floor")))
    beta, se, F, max_f, arg = (o.numpy() for o in out)
    assert beta.dtype == np.float64 and arg.dtype == np.int64
    # the reference's parity floors (beta / SE 1e-6, F 1e-5 absolute) cover the values near zero
    compare_epi(case, g, beta, se, F, max_f, arg, rtol=2e-5, atol_b=1e-6, atol_f=1e-5)


def test_epi_rank_deficient_anchor_raises():
    """A design with an all-zero column makes A singular: the batch raises LinAlgError, as the reference's does."""
    from fasterlmm_gb300.epi import snp_wald_scan_batched
    rng = np.random.default_rng(0)
    N, C = 40, 3
    X = rng.standard_normal((1, N, C))
    X[0, :, 2] = 0.0  # an exactly zero pivot (a repeated column leaves a rounding-sized one of either sign)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a))
    with pytest.raises(torch.linalg.LinAlgError):
        snp_wald_scan_batched(t(rng.uniform(0.5, 2.0, N)), t(X), t(rng.standard_normal((N, 2))), t(np.zeros(2)),
                              t(rng.standard_normal((1, N, 5))))
