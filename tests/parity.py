"""
Tolerances and comparison helpers shared by the oracle-pinning and GPU parity tests.

The reference's parity convention is rtol 1e-5 plus atol 1e-6 (reference tests/test_parity.py:20-27).  F is an
O(1..1e4) statistic, so its absolute floor is 1e-5, which moves -log10 p by < 1e-5.

log delta is compared by loss equivalence: the reference fits it by 50 golden-section steps whose last
comparisons are decided by FP64 rounding of the loss, so on flat likelihoods (h2 near 0, log delta near the grid
top) two correct implementations land up to ~1e-3 apart with losses equal to ~1e-12 relative.  A fitted value
passes when it is within ``ld_atol`` of the reference's or its -2 log L is no worse than the reference's by more
than ``loss_rtol`` relative.
"""
from __future__ import annotations

import numpy as np

DETAIL = ("f", "beta", "se", "sfve", "nullh2")
RTOL = 1e-5
# the -log10 p gate of the strong-signal and NaN-group tests: half of the 1e-3 parity bound
GATE = 5e-4
ATOL = {"f": 1e-5, "beta": 1e-6, "se": 1e-6, "sfve": 1e-6, "nullh2": 1e-6, "max_F": 1e-5, "perm_max_F": 1e-5}


def assert_scan_close(got: dict, ref: dict, *, rtol: float = RTOL, keys=DETAIL + ("max_F",), prefix: str = "",
                      atol_scale: float = 1.0):
    for k in keys:
        a = np.asarray(got[k])
        b = np.asarray(ref[prefix + k])
        assert a.shape == b.shape, (k, a.shape, b.shape)
        np.testing.assert_allclose(a, b, rtol=rtol, atol=ATOL[k] * atol_scale, err_msg=k)


def compat_loss(ld: np.ndarray, s: np.ndarray, UY: np.ndarray) -> np.ndarray:
    """(P,) ML -2 log L at one log delta per column (the reference's per-pheno compat loss)."""
    Neff = s.shape[0]
    Sd = s[None, :] + np.exp(ld)[:, None]
    yWy = np.maximum(((UY.T ** 2) / Sd).sum(axis=1), 1e-300)
    return Neff * (np.log(2 * np.pi) + np.log(yWy / Neff) + 1.0) + np.log(Sd).sum(axis=1)


def assert_log_delta_equivalent(ld: np.ndarray, ld_ref: np.ndarray, s: np.ndarray, UY: np.ndarray, *,
                                ld_atol: float = 1e-6, loss_rtol: float = 1e-9):
    ld = np.asarray(ld, dtype=np.float64)
    ld_ref = np.asarray(ld_ref, dtype=np.float64)
    close = np.abs(ld - ld_ref) <= ld_atol
    La = compat_loss(ld, s, UY)
    Lb = compat_loss(ld_ref, s, UY)
    equiv = La <= Lb + loss_rtol * np.abs(Lb)
    bad = ~(close | equiv)
    assert not bad.any(), (f"{bad.sum()} log delta values neither close nor loss-equivalent; worst at "
                           f"{np.flatnonzero(bad)[:5]}: got {ld[bad][:5]}, ref {ld_ref[bad][:5]}, "
                           f"dloss {(La - Lb)[bad][:5]}")


def gls_loss(ld: np.ndarray, s: np.ndarray, X_rot: np.ndarray, Y_rot: np.ndarray, reml: bool = False) -> np.ndarray:
    """(P,) -2 log L of the plain GLS model at one log delta per column (the reference's per-pheno plain loss)."""
    N, C = X_rot.shape
    out = np.empty(len(ld))
    for p, l in enumerate(np.asarray(ld, dtype=np.float64)):
        Sd = s + np.exp(l)
        w = 1.0 / Sd
        A = (X_rot * w[:, None]).T @ X_rot
        u = (X_rot * w[:, None]).T @ Y_rot[:, p]
        rWr = max((w * Y_rot[:, p] ** 2).sum() - u @ np.linalg.solve(A, u), 1e-300)
        if reml:
            out[p] = (N - C) * (np.log(2 * np.pi) + np.log(rWr / (N - C)) + 1.0) + np.log(Sd).sum() + \
                np.linalg.slogdet(A)[1]
        else:
            out[p] = N * (np.log(2 * np.pi) + np.log(rWr / N) + 1.0) + np.log(Sd).sum()
    return out


def assert_log_delta_equivalent_gls(ld, ld_ref, s, X_rot, Y_rot, *, reml: bool = False, ld_atol: float = 1e-6,
                                    loss_rtol: float = 1e-9):
    ld = np.asarray(ld, dtype=np.float64)
    ld_ref = np.asarray(ld_ref, dtype=np.float64)
    close = np.abs(ld - ld_ref) <= ld_atol
    La = gls_loss(ld, s, X_rot, Y_rot, reml)
    Lb = gls_loss(ld_ref, s, X_rot, Y_rot, reml)
    bad = ~(close | (La <= Lb + loss_rtol * np.abs(Lb)))
    assert not bad.any(), (f"{bad.sum()} log delta values neither close nor loss-equivalent; got {ld[bad][:5]}, "
                           f"ref {ld_ref[bad][:5]}, dloss {(La - Lb)[bad][:5]}")


def neg_log10_p_gpu(F, df2):
    """-log10 p of F statistics by the library's own kernel (the scan's p-value path)."""
    import torch
    from fasterlmm_gb300.post import neg_log10_pvalue
    return neg_log10_pvalue(torch.from_numpy(np.ascontiguousarray(F)).cuda(), df2).cpu().numpy()


def check_gates(got: dict, want: dict, df2: int, label: str, gate: float = None) -> float:
    """
    The strong-signal gates: beta and SE within rtol 1e-5 / atol 1e-6, |d(-log10 p)| <= gate on every real test,
    each column's ten strongest variants in the same order (a swap is a tie within the gate), permutation maxima
    within 1e-4 in -log10 p, the 0.05-quantile permutation threshold (fasterlmm/cli.py:128) within 1e-4, and the same
    significance calls except within the gate of the threshold.  Returns the largest |d(-log10 p)|.
    """
    gate = GATE if gate is None else gate
    for k in ("beta", "se"):
        np.testing.assert_allclose(got[k], want[k], rtol=1e-5, atol=1e-6, err_msg=f"{label} {k}")
    gp, wp = neg_log10_p_gpu(got["f"], df2), neg_log10_p_gpu(want["f"], df2)
    err = np.abs(gp - wp)
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err.max() <= gate, f"{label}: |d(-log10 p)| {err.max():.3e} at F = {want['f'][worst]:.1f}"
    # each phenotype's ten strongest variants, in order (a swap is a tie: the reference's values within the gate)
    for j in range(gp.shape[1]):
        tg = np.argsort(-gp[:, j], kind="stable")[:10]
        tw = np.argsort(-wp[:, j], kind="stable")[:10]
        d = tg != tw
        assert np.all(np.abs(wp[tg[d], j] - wp[tw[d], j]) <= gate), (label, j)
    # permutation thresholds and significance calls
    gq, wq = neg_log10_p_gpu(got["perm_max_F"], df2), neg_log10_p_gpu(want["perm_max_F"], df2)
    assert np.abs(gq - wq).max() <= 1e-4, label
    for j in range(gp.shape[1]):
        tg = -np.log10(np.quantile(10.0 ** -gq[j], 0.05))
        tw = -np.log10(np.quantile(10.0 ** -wq[j], 0.05))
        assert abs(tg - tw) <= 1e-4, (label, j, tg, tw)
        sg, sw = gp[:, j] > tg, wp[:, j] > tw
        d = sg != sw
        assert np.all(np.abs(wp[d, j] - tw) <= gate), (label, j, int(d.sum()))
    rb = np.abs(got["beta"] - want["beta"]) / np.maximum(np.abs(want["beta"]), 1e-6)
    print(f"{label}: max F {want['f'].max():.0f}, max |d(-log10 p)| {err.max():.2e}, max rel d(beta) {rb.max():.2e}")
    return float(err.max())
