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
