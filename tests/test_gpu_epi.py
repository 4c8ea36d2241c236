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


@pytest.mark.parametrize("N,C,Pc", [(1, 1, 1), (37, 3, 5), (300, 41, 7), (450, 200, 2)])
def test_epi_setup_matches_fp64(N, C, Pc):
    """flmm_epi_setup_f64 (the per-phenotype FP64 setup: weights, Cholesky factor of X^T W X, Q = L^-1 X^T W, the
    X-fit residual row and rWr) against numpy FP64, at one sample, tiny and the largest supported design (C = 200,
    where the kernels' row tile and thread count shrink to fit shared memory); Y's leading dimension is wider than
    the chunk, as for a chunk inside a larger phenotype table."""
    from fasterlmm_gb300 import _lib, build
    build()
    rng = np.random.default_rng(N + C)
    s = rng.uniform(0.1, 3.0, N)
    X = rng.standard_normal((N, C))
    P = Pc + 3
    Y = rng.standard_normal((N, P))
    ld = rng.uniform(-2, 2, P)
    p0 = 2
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    s_d, X_d, Y_d, ld_d = d(s), d(X), d(Y), d(ld)
    R1 = torch.empty((Pc * (C + 1), N), dtype=torch.float64, device="cuda")
    W = torch.empty((Pc, N), dtype=torch.float64, device="cuda")
    rWr = torch.empty(Pc, dtype=torch.float64, device="cuda")
    L = torch.empty(Pc * C * (C + 1) // 2, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.call("flmm_epi_setup_f64", s_d.data_ptr(), N, X_d.data_ptr(), C, C, Y_d[:, p0:].data_ptr(), P,
              ld_d[p0:].data_ptr(), Pc, R1.data_ptr(), W.data_ptr(), rWr.data_ptr(), L.data_ptr(), info.data_ptr(), st)
    torch.cuda.synchronize()
    assert int(info.item()) == 0
    R1, W, rWr, L = (t.cpu().numpy() for t in (R1, W, rWr, L))
    tril = np.tril_indices(C)
    for p in range(Pc):
        w = 1.0 / (s + np.exp(ld[p0 + p]))
        A = X.T @ (w[:, None] * X)
        Lp = np.linalg.cholesky(A)
        Q = np.linalg.solve(Lp, (w[:, None] * X).T)
        bx = np.linalg.solve(A, X.T @ (w * Y[:, p0 + p]))
        r = Y[:, p0 + p] - X @ bx
        np.testing.assert_allclose(W[p], w, rtol=1e-15)
        np.testing.assert_allclose(L[p * len(tril[0]):(p + 1) * len(tril[0])], Lp[tril], rtol=0,
                                   atol=1e-11 * np.abs(Lp).max())
        blk = R1[p * (C + 1):(p + 1) * (C + 1)]
        np.testing.assert_allclose(blk[:C], Q, rtol=0, atol=1e-10 * np.abs(Q).max())
        # the residual's scale is the phenotype's (at N = C it is rounding noise around zero)
        wy = w * Y[:, p0 + p]
        np.testing.assert_allclose(blk[C], w * r, rtol=0, atol=1e-10 * np.abs(wy).max())
        np.testing.assert_allclose(rWr[p], max((w * r * r).sum(), 1e-300), rtol=1e-9,
                                   atol=1e-12 * (wy * Y[:, p0 + p]).sum())
