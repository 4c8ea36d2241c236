"""
CPU oracle for the FaST-ER-LMM fastlmm-compat LOCO association scan.

TEST INFRASTRUCTURE ONLY.  This module is a plain numpy FP64 restatement of the reference's scan path, used as
the checker for the GPU implementation.  Only the test suite (tests/), ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import or run it, and only as the checker or the
timed CPU baseline -- never as the thing measured or shipped.  The product path (``fasterlmm_gb300``) never
imports it and fails loudly when its CUDA library is missing.

Pinning: tests/golden/*.npz hold outputs of the reference itself (the ``fasterlmm`` package, v1.6.2), run on
seeded synthetic inputs by tests/golden/make_golden.py.  tests/test_oracle_golden.py checks every function here
against those fixtures, so this restatement is pinned to the reference's own numbers.

Every function cites the reference file:line it restates (paths inside the reference project).
"""

from __future__ import annotations

import numpy as np

LOG2PI = float(np.log(2.0 * np.pi))


# --------------------------------------------------------------------------------------------------------------
# standardisation and kinship
# --------------------------------------------------------------------------------------------------------------

def pos_floor(dtype=np.float64) -> float:
    """Positive clamp floor: 1e-300 in FP64, 1e-30 otherwise (fasterlmm/core.py:80-86)."""
    return 1e-300 if np.dtype(dtype) == np.float64 else 1e-30


def standardise_columns(Z: np.ndarray) -> np.ndarray:
    """
    Unit standardiser, torch branch order (fasterlmm/io.py:235-246): NaN-aware column mean and population std
    (ddof=0, counts clamped at 1), std == 0 -> inf, subtract / divide, NaN -> 0 after scaling.
    """
    a = np.array(Z, dtype=np.float64, copy=True)
    nan_mask = np.isnan(a)
    a_stats = np.where(nan_mask, 0.0, a)
    n_nonnan = np.maximum((~nan_mask).sum(axis=0), 1).astype(np.float64)
    col_mean = a_stats.sum(axis=0) / n_nonnan
    diff = np.where(nan_mask, 0.0, a_stats - col_mean[None, :])
    col_std = np.sqrt((diff * diff).sum(axis=0) / n_nonnan)
    col_std = np.where(col_std == 0, np.inf, col_std)
    with np.errstate(invalid="ignore"):
        out = (a - col_mean[None, :]) / col_std[None, :]
    return np.where(nan_mask, 0.0, out)


def grm(Z: np.ndarray) -> np.ndarray:
    """K = Z Z^T / M for a pre-standardised Z (fasterlmm/io.py:257-265)."""
    return (Z @ Z.T) / Z.shape[1]


# --------------------------------------------------------------------------------------------------------------
# compat rotation, delta fit, Wald scan
# --------------------------------------------------------------------------------------------------------------

def compat_rotate(K: np.ndarray, X: np.ndarray, Y: np.ndarray) -> dict:
    """
    fastlmm projection rotation (fasterlmm/core.py:487-519): Xpinv = pinv(X); Kp = (I - PX)(K + I)(I - PX);
    eigh; keep eigenpairs D..N-1 with s = max(s - 1, 0); UY = U_eff^T (Y - X Xpinv Y).
    """
    N = K.shape[0]
    D = X.shape[1]
    Xpinv = np.linalg.pinv(X)
    Iperp = np.eye(N) - X @ Xpinv
    Kp = (Iperp @ (K + np.eye(N))) @ Iperp
    s_full, U_full = np.linalg.eigh(Kp)
    s = np.maximum(s_full[D:N] - 1.0, 0.0)
    U_eff = np.ascontiguousarray(U_full[:, D:N])
    Y_r = Y - X @ (Xpinv @ Y)
    UY = U_eff.T @ Y_r
    return {"s": s, "U_eff": U_eff, "X": X, "Xpinv": Xpinv, "UY": UY}


def profile_loss_compat(log_delta: np.ndarray, s: np.ndarray, UY: np.ndarray) -> np.ndarray:
    """(G, P) ML -2 log-likelihood on a grid (fasterlmm/core.py:525-542)."""
    Neff = s.shape[0]
    delta = np.exp(log_delta)
    Sd = s[None, :] + delta[:, None]
    w = 1.0 / Sd
    yWy = w @ (UY * UY)
    rWr = np.maximum(yWy, pos_floor())
    sum_log_Sd = np.log(Sd).sum(axis=1)
    sigma2 = rWr / Neff
    return Neff * (LOG2PI + np.log(sigma2) + 1.0) + sum_log_Sd[:, None]


def profile_loss_compat_per_pheno(log_delta: np.ndarray, s: np.ndarray, UY: np.ndarray) -> np.ndarray:
    """(P,) loss, one log delta per phenotype column (fasterlmm/core.py:545-558)."""
    Neff = s.shape[0]
    delta = np.exp(log_delta)
    Sd = s[None, :] + delta[:, None]
    w = 1.0 / Sd
    yWy = (w * UY.T * UY.T).sum(axis=1)
    rWr = np.maximum(yWy, pos_floor())
    sum_log_Sd = np.log(Sd).sum(axis=1)
    sigma2 = rWr / Neff
    return Neff * (LOG2PI + np.log(sigma2) + 1.0) + sum_log_Sd


def delta_grid(n_grid: int, log_delta_min: float, log_delta_max: float) -> np.ndarray:
    """The grid the reference builds with torch.linspace (fasterlmm/core.py:569)."""
    import torch  # torch.linspace's node values are the ones the reference compares against
    return torch.linspace(log_delta_min, log_delta_max, n_grid, dtype=torch.float64).numpy()


def fit_delta_grid_compat(s: np.ndarray, UY: np.ndarray, *, n_grid: int = 64, log_delta_min: float = -10.0,
                          log_delta_max: float = 10.0, refine: bool = True, return_idx: bool = False):
    """
    Grid argmin then 50 golden-section steps on [grid[i-1], grid[i+1]] (fasterlmm/core.py:561-595).
    The bracket update order, inv_phi constants and final 0.5 (a + b) clamp follow the reference exactly.
    """
    grid = delta_grid(n_grid, log_delta_min, log_delta_max)
    loss = profile_loss_compat(grid, s, UY)
    idx = loss.argmin(axis=0)
    if not refine:
        out = grid[idx]
        return (out, idx) if return_idx else out
    lo_idx = np.clip(idx - 1, 0, n_grid - 1)
    hi_idx = np.clip(idx + 1, 0, n_grid - 1)
    a = grid[lo_idx].copy()
    b = grid[hi_idx].copy()
    inv_phi = 2.0 / (1.0 + 5.0 ** 0.5)
    inv_phi2 = inv_phi * inv_phi
    c = a + inv_phi2 * (b - a)
    d = a + inv_phi * (b - a)
    fc = profile_loss_compat_per_pheno(c, s, UY)
    fd = profile_loss_compat_per_pheno(d, s, UY)
    for _ in range(50):
        cond = fc < fd
        b = np.where(cond, d, b)
        a = np.where(cond, a, c)
        c = a + inv_phi2 * (b - a)
        d = a + inv_phi * (b - a)
        fc = profile_loss_compat_per_pheno(c, s, UY)
        fd = profile_loss_compat_per_pheno(d, s, UY)
    out = np.clip(0.5 * (a + b), log_delta_min, log_delta_max)
    return (out, idx) if return_idx else out


def snp_wald_scan_compat(spec: dict, log_delta: np.ndarray, S: np.ndarray, *, n_real: int | None = None) -> dict:
    """
    Per-(variant, column) Wald test in the projected basis (fasterlmm/core.py:601-671).  The reference tiles the
    pheno / variant axes; tiling does not change the maths (its own chunking-invariance test, tests/
    test_core_compat.py:244-258), so the oracle evaluates one tile.
    """
    s, UY, X, Xpinv, U_eff = spec["s"], spec["UY"], spec["X"], spec["Xpinv"], spec["U_eff"]
    Neff = s.shape[0]
    P = UY.shape[1]
    M = S.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    floor = pos_floor()
    S_r = S - X @ (Xpinv @ S)
    US = U_eff.T @ S_r
    delta = np.exp(log_delta)
    w = 1.0 / (s[None, :] + delta[:, None])
    rWr = np.maximum((w * UY.T * UY.T).sum(axis=1), floor)
    sWy = (w * UY.T) @ US
    sWs = w @ (US * US)
    denom = np.maximum(sWs, floor)
    beta = sWy / denom
    rss = np.maximum(rWr[:, None] - sWy * sWy / denom, floor)
    var_beta = rss / (Neff - 1) / denom
    F = beta * beta / var_beta
    max_F = F.max(axis=1) if M > 0 else np.full(P, -np.inf)
    r = slice(0, n_real)
    sfve = np.sqrt(np.maximum((sWy[r] * sWy[r]) / (denom[r] * rWr[r, None]), 0.0))
    h2 = 1.0 / (1.0 + np.exp(log_delta[:n_real]))
    return {"f": F[r].T.copy(), "beta": beta[r].T.copy(), "se": np.sqrt(var_beta[r]).T.copy(), "sfve": sfve.T.copy(),
            "nullh2": np.broadcast_to(h2[None, :], (M, n_real)).copy(), "max_F": max_F}


def loco_scan_compat(Z: np.ndarray, X: np.ndarray, Y: np.ndarray, chrom: np.ndarray, *, n_real: int | None = None,
                     Z_kin: np.ndarray | None = None, chrom_kin: np.ndarray | None = None, n_grid: int = 64,
                     log_delta_min: float = -10.0, log_delta_max: float = 10.0, refine: bool = True,
                     on_chrom=None, keep_spectra: bool = False) -> dict:
    """
    LOCO driver (fasterlmm/core.py:677-726): per chromosome c, K from the variants not on c (or from the kinship
    panel without c), compat rotation, delta fit, Wald scan of the variants on c, scatter, running genome max.
    The grid options are the reference's fit_delta_grid_compat keywords (fasterlmm/core.py:561-562), which its
    LOCO loop leaves at their defaults (fasterlmm/core.py:715).
    Also returns the per-chromosome log delta, which the reference computes but does not return, and with
    ``keep_spectra`` the per-chromosome (s, UY) used to judge log delta by its loss.
    """
    if (Z_kin is None) != (chrom_kin is None):
        raise ValueError("Z_kin and chrom_kin go together")
    chrom = np.asarray(chrom)
    M = Z.shape[1]
    P = Y.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    out = {k: np.zeros((M, n_real)) for k in ("f", "beta", "se", "sfve", "nullh2")}
    max_F = np.full(P, -np.inf)
    chroms = sorted(np.unique(chrom).tolist())
    log_deltas = {}
    spectra = {}
    for k_idx, c in enumerate(chroms):
        test_mask = chrom == c
        K = grm(Z[:, chrom != c]) if Z_kin is None else grm(Z_kin[:, np.asarray(chrom_kin) != c])
        spec = compat_rotate(K, X, Y)
        ld = fit_delta_grid_compat(spec["s"], spec["UY"], n_grid=n_grid, log_delta_min=log_delta_min,
                                   log_delta_max=log_delta_max, refine=refine)
        log_deltas[c] = ld
        if keep_spectra:
            spectra[c] = (spec["s"], spec["UY"])
        res = snp_wald_scan_compat(spec, ld, Z[:, test_mask], n_real=n_real)
        if n_real > 0:
            for key in out:
                out[key][test_mask, :] = res[key]
        max_F = np.maximum(max_F, res["max_F"])
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(chroms))
    out["max_F"] = max_F
    out["log_delta"] = log_deltas
    if keep_spectra:
        out["spectra"] = spectra
    return out


def single_k_scan_compat(Z: np.ndarray, X: np.ndarray, Y: np.ndarray, *, n_real: int | None = None,
                         Z_kin: np.ndarray | None = None, n_grid: int = 64, log_delta_min: float = -10.0,
                         log_delta_max: float = 10.0, refine: bool = True) -> dict:
    """One K over every kinship variant, one rotation / fit / scan (fasterlmm/core.py:729-740)."""
    K = grm(Z if Z_kin is None else Z_kin)
    spec = compat_rotate(K, X, Y)
    ld = fit_delta_grid_compat(spec["s"], spec["UY"], n_grid=n_grid, log_delta_min=log_delta_min,
                               log_delta_max=log_delta_max, refine=refine)
    res = snp_wald_scan_compat(spec, ld, Z, n_real=n_real)
    res["log_delta"] = ld
    res["spectra"] = {0: (spec["s"], spec["UY"])}
    return res


# --------------------------------------------------------------------------------------------------------------
# plain GLS path: rotation with covariates kept, ML / REML delta fit with a per-delta Cholesky, GLS Wald scan
# --------------------------------------------------------------------------------------------------------------

def eigendecompose(K: np.ndarray, jitter: float = 1e-6) -> tuple[np.ndarray, np.ndarray]:
    """eigh(K + jitter I), eigenvalues clamped at 0 (fasterlmm/core.py:89-102)."""
    s, U = np.linalg.eigh(K + jitter * np.eye(K.shape[0]))
    return np.maximum(s, 0.0), U


def rotate(K: np.ndarray, X: np.ndarray, Y: np.ndarray) -> dict:
    """Spectrum with U^T X and U^T Y (fasterlmm/core.py:105-116)."""
    s, U = eigendecompose(K)
    return {"s": s, "U": U, "X_rot": U.T @ X, "Y_rot": U.T @ Y}


def _gls_terms(w: np.ndarray, X_rot: np.ndarray, Y_rot: np.ndarray):
    """A = X~^T W X~ per row of w, its Cholesky (identity where it fails), u = X~^T W Y~, uAu, yWy."""
    A = np.einsum("gn,nc,nd->gcd", w, X_rot, X_rot)
    C = X_rot.shape[1]
    L = np.empty_like(A)
    bad = np.zeros(A.shape[0], dtype=bool)
    for g in range(A.shape[0]):
        try:
            L[g] = np.linalg.cholesky(A[g])
        except np.linalg.LinAlgError:
            L[g] = np.eye(C)
            bad[g] = True
    return A, L, bad


def profile_loss(log_delta: np.ndarray, s: np.ndarray, X_rot: np.ndarray, Y_rot: np.ndarray, *,
                 reml: bool = False) -> np.ndarray:
    """
    (G, P) -2 log likelihood with beta profiled out by GLS (fasterlmm/core.py:148-187): A = X~^T W X~ per grid
    point, uAu = u^T A^-1 u, rWr = max(yWy - uAu, floor); ML divides by N, REML by N - C and adds log det A.
    Grid points whose A has no Cholesky get +inf.
    """
    N, C = X_rot.shape
    delta = np.exp(log_delta)
    Sd = s[None, :] + delta[:, None]
    w = 1.0 / Sd
    A, L, bad = _gls_terms(w, X_rot, Y_rot)
    logdet_A = 2.0 * np.log(np.diagonal(L, axis1=1, axis2=2)).sum(axis=1)
    u = np.einsum("gn,nc,np->gcp", w, X_rot, Y_rot)
    beta_x = np.stack([np.linalg.solve(L[g].T, np.linalg.solve(L[g], u[g])) for g in range(len(delta))])
    uAu = (u * beta_x).sum(axis=1)
    yWy = w @ (Y_rot * Y_rot)
    rWr = np.maximum(yWy - uAu, pos_floor())
    sum_log_Sd = np.log(Sd).sum(axis=1)
    if reml:
        loss = (N - C) * (LOG2PI + np.log(rWr / (N - C)) + 1.0) + sum_log_Sd[:, None] + logdet_A[:, None]
    else:
        loss = N * (LOG2PI + np.log(rWr / N) + 1.0) + sum_log_Sd[:, None]
    loss[bad, :] = np.inf
    return loss


def profile_loss_per_pheno(log_delta: np.ndarray, s: np.ndarray, X_rot: np.ndarray, Y_rot: np.ndarray, *,
                           reml: bool = False) -> np.ndarray:
    """Column p's loss at its own log_delta[p] (fasterlmm/core.py:190-224)."""
    P = Y_rot.shape[1]
    return np.array([profile_loss(log_delta[p:p + 1], s, X_rot, Y_rot[:, p:p + 1], reml=reml)[0, 0]
                     for p in range(P)])


def nll_eval(delta: float, s: np.ndarray, X_rot: np.ndarray, y_rot: np.ndarray) -> float:
    """ML -2 log likelihood of one phenotype at one delta (fasterlmm/core.py:122-145)."""
    N = X_rot.shape[0]
    w = 1.0 / (s + delta)
    WX = w[:, None] * X_rot
    A = WX.T @ X_rot
    Xy = WX.T @ y_rot
    beta = np.linalg.solve(A, Xy)
    rWr = (y_rot * w * y_rot).sum() - (Xy * beta).sum()
    return float(N * (LOG2PI + np.log(rWr / N) + 1.0) + np.log(s + delta).sum())


def fit_delta_grid(s: np.ndarray, X_rot: np.ndarray, Y_rot: np.ndarray, *, n_grid: int = 64,
                   log_delta_min: float = -10.0, log_delta_max: float = 10.0, refine: bool = True,
                   reml: bool = False, return_idx: bool = False):
    """Grid argmin then 50 golden-section steps on the GLS loss (fasterlmm/core.py:227-264)."""
    grid = delta_grid(n_grid, log_delta_min, log_delta_max)
    loss = profile_loss(grid, s, X_rot, Y_rot, reml=reml)
    idx = loss.argmin(axis=0)
    if not refine:
        out = grid[idx]
        return (out, idx) if return_idx else out
    a = grid[np.clip(idx - 1, 0, n_grid - 1)].copy()
    b = grid[np.clip(idx + 1, 0, n_grid - 1)].copy()
    inv_phi = 2.0 / (1.0 + 5.0 ** 0.5)
    inv_phi2 = inv_phi * inv_phi
    c = a + inv_phi2 * (b - a)
    d = a + inv_phi * (b - a)
    fc = profile_loss_per_pheno(c, s, X_rot, Y_rot, reml=reml)
    fd = profile_loss_per_pheno(d, s, X_rot, Y_rot, reml=reml)
    for _ in range(50):
        cond = fc < fd
        b = np.where(cond, d, b)
        a = np.where(cond, a, c)
        c = a + inv_phi2 * (b - a)
        d = a + inv_phi * (b - a)
        fc = profile_loss_per_pheno(c, s, X_rot, Y_rot, reml=reml)
        fd = profile_loss_per_pheno(d, s, X_rot, Y_rot, reml=reml)
    out = np.clip(0.5 * (a + b), log_delta_min, log_delta_max)
    return (out, idx) if return_idx else out


def snp_wald_scan(spec: dict, log_delta: np.ndarray, S_rot: np.ndarray, *, n_real: int | None = None) -> dict:
    """
    GLS Wald test per (variant, column) with the covariates in the model (fasterlmm/core.py:295-375): per column
    the null fit (A, beta_x, r, rWr), per test B = X~^T W S, quad = B^T A^-1 B, denom = max(sWs - quad, floor),
    num = (W r)^T S, beta = num / denom, var_beta = max(rWr - num^2 / denom, floor) / (N - C - 1) / denom.
    """
    s, X_rot, Y_rot = spec["s"], spec["X_rot"], spec["Y_rot"]
    N, C = X_rot.shape
    P = Y_rot.shape[1]
    M = S_rot.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    floor = pos_floor()
    delta = np.exp(log_delta)
    w = 1.0 / (s[None, :] + delta[:, None])
    A, L, _ = _gls_terms(w, X_rot, Y_rot)
    u = np.einsum("pn,nc,np->pc", w, X_rot, Y_rot)
    beta_x = np.stack([np.linalg.solve(L[p].T, np.linalg.solve(L[p], u[p])) for p in range(P)])
    r = Y_rot - X_rot @ beta_x.T
    rWr = (w * r.T * r.T).sum(axis=1)
    wr = w * r.T
    B = np.einsum("pn,nc,nm->pcm", w, X_rot, S_rot)
    AinvB = np.stack([np.linalg.solve(L[p].T, np.linalg.solve(L[p], B[p])) for p in range(P)])
    sWs = w @ (S_rot * S_rot)
    quad = (B * AinvB).sum(axis=1)
    denom = np.maximum(sWs - quad, floor)
    num = wr @ S_rot
    beta = num / denom
    rss = np.maximum(rWr[:, None] - num * num / denom, floor)
    var_beta = rss / (N - C - 1) / denom
    F = beta * beta / var_beta
    max_F = F.max(axis=1) if M > 0 else np.full(P, -np.inf)
    rr = slice(0, n_real)
    sfve = np.sqrt(np.maximum((num[rr] * num[rr]) / (denom[rr] * rWr[rr, None]), 0.0))
    h2 = 1.0 / (1.0 + np.exp(log_delta[:n_real]))
    return {"f": F[rr].T.copy(), "beta": beta[rr].T.copy(), "se": np.sqrt(var_beta[rr]).T.copy(),
            "sfve": sfve.T.copy(), "nullh2": np.broadcast_to(h2[None, :], (M, n_real)).copy(), "max_F": max_F}


def loco_scan(Z: np.ndarray, X: np.ndarray, Y: np.ndarray, chrom: np.ndarray, *, n_real: int | None = None,
              Z_kin: np.ndarray | None = None, chrom_kin: np.ndarray | None = None, on_chrom=None) -> dict:
    """Plain LOCO driver (fasterlmm/core.py:381-436): per chromosome K_loco, rotate, ML fit, GLS Wald."""
    if (Z_kin is None) != (chrom_kin is None):
        raise ValueError("Z_kin and chrom_kin go together")
    chrom = np.asarray(chrom)
    M = Z.shape[1]
    P = Y.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    out = {k: np.zeros((M, n_real)) for k in ("f", "beta", "se", "sfve", "nullh2")}
    max_F = np.full(P, -np.inf)
    chroms = sorted(np.unique(chrom).tolist())
    log_deltas = {}
    for k_idx, c in enumerate(chroms):
        test_mask = chrom == c
        K = grm(Z[:, chrom != c]) if Z_kin is None else grm(Z_kin[:, np.asarray(chrom_kin) != c])
        spec = rotate(K, X, Y)
        ld = fit_delta_grid(spec["s"], spec["X_rot"], spec["Y_rot"])
        log_deltas[c] = ld
        res = snp_wald_scan(spec, ld, spec["U"].T @ Z[:, test_mask], n_real=n_real)
        if n_real > 0:
            for key in out:
                out[key][test_mask, :] = res[key]
        max_F = np.maximum(max_F, res["max_F"])
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(chroms))
    out["max_F"] = max_F
    out["log_delta"] = log_deltas
    return out


def single_k_scan(Z: np.ndarray, X: np.ndarray, Y: np.ndarray, *, n_real: int | None = None,
                  Z_kin: np.ndarray | None = None) -> dict:
    """Plain whole-genome scan (fasterlmm/core.py:439-451)."""
    spec = rotate(grm(Z if Z_kin is None else Z_kin), X, Y)
    ld = fit_delta_grid(spec["s"], spec["X_rot"], spec["Y_rot"])
    res = snp_wald_scan(spec, ld, spec["U"].T @ Z, n_real=n_real)
    res["log_delta"] = ld
    return res


# --------------------------------------------------------------------------------------------------------------
# low-rank path: kinship factor G (N, k) with k < N, the N - k null directions carried analytically
# --------------------------------------------------------------------------------------------------------------

def lowrank_basis(G: np.ndarray, X: np.ndarray, *, sv_floor: float = 1e-10) -> dict:
    """
    fastlmm's k < N spectral decomposition (fasterlmm/lowrank.py:59-96): G_ = G - X Xpinv G; eigh of G_^T G_
    (k < N) or of G_ G_^T / M_kin (k >= N); keep singular values above sv_floor; U_eff = G_ V / sv, s = sv^2 / M_kin.
    """
    N, k_in = G.shape
    D = X.shape[1]
    Xpinv = np.linalg.pinv(X)
    G_ = G - X @ (Xpinv @ G)
    if k_in < N:
        evals, V = np.linalg.eigh(G_.T @ G_)
        sv = np.sqrt(np.maximum(evals, 0.0))
        keep = sv > sv_floor
        sv, V = sv[keep], V[:, keep]
        U_eff = G_ @ (V / sv)
        s = sv * sv / k_in
    else:
        evals, U = np.linalg.eigh((G_ @ G_.T) / k_in)
        keep = np.maximum(evals, 0.0) > sv_floor * sv_floor / k_in
        s = np.maximum(evals[keep], 0.0)
        U_eff = np.ascontiguousarray(U[:, keep])
    return {"s": s, "U_eff": U_eff, "X": X, "Xpinv": Xpinv, "Neff": N - D}


def rotate_phenos(basis: dict, Y: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """On-rank UY = U_eff^T Y_r and off-rank residual UUY = Y_r - U_eff UY (fasterlmm/lowrank.py:99-111)."""
    Y_r = Y - basis["X"] @ (basis["Xpinv"] @ Y)
    UY = basis["U_eff"].T @ Y_r
    return UY, Y_r - basis["U_eff"] @ UY


def lowrank_rotate(G: np.ndarray, X: np.ndarray, Y: np.ndarray, *, sv_floor: float = 1e-10) -> dict:
    """lowrank_basis + rotate_phenos (fasterlmm/lowrank.py:114-125)."""
    spec = lowrank_basis(G, X, sv_floor=sv_floor)
    spec["UY"], spec["UUY"] = rotate_phenos(spec, Y)
    return spec


def profile_loss_lowrank(log_delta: np.ndarray, s: np.ndarray, UY: np.ndarray, yy_off: np.ndarray,
                         Neff: int) -> np.ndarray:
    """
    (G, P) ML -2 log L of the low-rank model (fasterlmm/lowrank.py:131-151): rWr = sum UY^2 / (s + delta) +
    yy_off / delta, log det = sum log(s + delta) + (Neff - k) log delta.
    """
    k = s.shape[0]
    delta = np.exp(log_delta)
    Sd = s[None, :] + delta[:, None]
    rWr = np.maximum((1.0 / Sd) @ (UY * UY) + yy_off[None, :] / delta[:, None], pos_floor())
    logdet = np.log(Sd).sum(axis=1) + (Neff - k) * np.log(delta)
    return Neff * (LOG2PI + np.log(rWr / Neff) + 1.0) + logdet[:, None]


def profile_loss_lowrank_per_pheno(log_delta: np.ndarray, s: np.ndarray, UY: np.ndarray, yy_off: np.ndarray,
                                   Neff: int) -> np.ndarray:
    """One log delta per column (fasterlmm/lowrank.py:154-169)."""
    k = s.shape[0]
    delta = np.exp(log_delta)
    Sd = s[None, :] + delta[:, None]
    rWr = np.maximum(((1.0 / Sd) * UY.T * UY.T).sum(axis=1) + yy_off / delta, pos_floor())
    logdet = np.log(Sd).sum(axis=1) + (Neff - k) * np.log(delta)
    return Neff * (LOG2PI + np.log(rWr / Neff) + 1.0) + logdet


def fit_delta_grid_lowrank(spec: dict, *, n_grid: int = 64, log_delta_min: float = -10.0,
                           log_delta_max: float = 10.0, refine: bool = True) -> np.ndarray:
    """Grid argmin then 50 golden-section steps on the low-rank loss (fasterlmm/lowrank.py:172-208)."""
    s, UY, Neff = spec["s"], spec["UY"], spec["Neff"]
    yy_off = (spec["UUY"] * spec["UUY"]).sum(axis=0)
    grid = delta_grid(n_grid, log_delta_min, log_delta_max)
    idx = profile_loss_lowrank(grid, s, UY, yy_off, Neff).argmin(axis=0)
    if not refine:
        return grid[idx]
    a = grid[np.clip(idx - 1, 0, n_grid - 1)].copy()
    b = grid[np.clip(idx + 1, 0, n_grid - 1)].copy()
    inv_phi = 2.0 / (1.0 + 5.0 ** 0.5)
    inv_phi2 = inv_phi * inv_phi
    c = a + inv_phi2 * (b - a)
    d = a + inv_phi * (b - a)
    fc = profile_loss_lowrank_per_pheno(c, s, UY, yy_off, Neff)
    fd = profile_loss_lowrank_per_pheno(d, s, UY, yy_off, Neff)
    for _ in range(50):
        cond = fc < fd
        b = np.where(cond, d, b)
        a = np.where(cond, a, c)
        c = a + inv_phi2 * (b - a)
        d = a + inv_phi * (b - a)
        fc = profile_loss_lowrank_per_pheno(c, s, UY, yy_off, Neff)
        fd = profile_loss_lowrank_per_pheno(d, s, UY, yy_off, Neff)
    return np.clip(0.5 * (a + b), log_delta_min, log_delta_max)


def snp_wald_scan_lowrank(spec: dict, log_delta: np.ndarray, S: np.ndarray, *, n_real: int | None = None) -> dict:
    """
    Low-rank Wald scan (fasterlmm/lowrank.py:239-316): every quadratic form has an on-rank part weighted by
    1 / (s + delta) and an off-rank part weighted by 1 / delta (UUS = S_r - U US, UUY as rotated).
    """
    s, UY, UUY, X, Xpinv, U = spec["s"], spec["UY"], spec["UUY"], spec["X"], spec["Xpinv"], spec["U_eff"]
    Neff = spec["Neff"]
    P = UY.shape[1]
    M = S.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    floor = pos_floor()
    delta = np.exp(log_delta)
    w = 1.0 / (s[None, :] + delta[:, None])
    rWr = np.maximum((w * UY.T * UY.T).sum(axis=1) + (UUY * UUY).sum(axis=0) / delta, floor)
    S_r = S - X @ (Xpinv @ S)
    US = U.T @ S_r
    UUS = S_r - U @ US
    sWs = w @ (US * US) + (UUS * UUS).sum(axis=0)[None, :] / delta[:, None]
    denom = np.maximum(sWs, floor)
    sWy = (w * UY.T) @ US + (UUS.T @ UUY).T / delta[:, None]
    beta = sWy / denom
    rss = np.maximum(rWr[:, None] - sWy * sWy / denom, floor)
    var_beta = rss / (Neff - 1) / denom
    F = beta * beta / var_beta
    max_F = F.max(axis=1) if M > 0 else np.full(P, -np.inf)
    r = slice(0, n_real)
    sfve = np.sqrt(np.maximum((sWy[r] * sWy[r]) / (denom[r] * rWr[r, None]), 0.0))
    h2 = 1.0 / (1.0 + np.exp(log_delta[:n_real]))
    return {"f": F[r].T.copy(), "beta": beta[r].T.copy(), "se": np.sqrt(var_beta[r]).T.copy(), "sfve": sfve.T.copy(),
            "nullh2": np.broadcast_to(h2[None, :], (M, n_real)).copy(), "max_F": max_F}


def loco_scan_lowrank(G: np.ndarray, g_chrom: np.ndarray, Z: np.ndarray, z_chrom: np.ndarray, X: np.ndarray,
                      Y: np.ndarray, *, n_real: int | None = None, on_chrom=None) -> dict:
    """Low-rank LOCO driver (fasterlmm/lowrank.py:322-359): the kinship factor drops chromosome c's markers."""
    M = Z.shape[1]
    P = Y.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    out = {k: np.zeros((M, n_real)) for k in ("f", "beta", "se", "sfve", "nullh2")}
    max_F = np.full(P, -np.inf)
    chroms = sorted(np.unique(z_chrom).tolist())
    log_deltas = {}
    for k_idx, c in enumerate(chroms):
        test_mask = np.asarray(z_chrom) == c
        spec = lowrank_rotate(G[:, np.asarray(g_chrom) != c], X, Y)
        ld = fit_delta_grid_lowrank(spec)
        log_deltas[c] = ld
        res = snp_wald_scan_lowrank(spec, ld, Z[:, test_mask], n_real=n_real)
        if n_real > 0:
            for key in out:
                out[key][test_mask, :] = res[key]
        max_F = np.maximum(max_F, res["max_F"])
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(chroms))
    out["max_F"] = max_F
    out["log_delta"] = log_deltas
    return out


def single_k_scan_lowrank(G: np.ndarray, Z: np.ndarray, X: np.ndarray, Y: np.ndarray, *,
                          n_real: int | None = None) -> dict:
    """Low-rank whole-genome scan (fasterlmm/lowrank.py:362-373)."""
    spec = lowrank_rotate(G, X, Y)
    ld = fit_delta_grid_lowrank(spec)
    res = snp_wald_scan_lowrank(spec, ld, Z, n_real=n_real)
    res["log_delta"] = ld
    return res


# --------------------------------------------------------------------------------------------------------------
# PLINK 1 .bed (SNP-major) -- the published file format the reference reads through pysnptools (fasterlmm/io.py:54-67)
# --------------------------------------------------------------------------------------------------------------

def write_bed(prefix: str, G: np.ndarray, *, chrom=None, sid=None, pos=None, iid=None, count_A1: bool = True) -> None:
    """
    Write dosages G (N, M) (NaN or negative = missing) as .bed/.bim/.fam.  With count_A1 a dosage counts the first
    allele: 2 -> 00, 1 -> 10, 0 -> 11; missing -> 01; four samples per byte from the low bits up.
    """
    N, M = G.shape
    chrom = np.ones(M, dtype=int) if chrom is None else np.asarray(chrom)
    sid = [f"v{j}" for j in range(M)] if sid is None else sid
    pos = np.arange(1, M + 1) if pos is None else np.asarray(pos)
    iid = [f"s{i}" for i in range(N)] if iid is None else iid
    with open(f"{prefix}.fam", "w") as fh:
        for s in iid:
            fh.write(f"{s} {s} 0 0 0 -9\n")
    with open(f"{prefix}.bim", "w") as fh:
        for j in range(M):
            fh.write(f"{chrom[j]}\t{sid[j]}\t0\t{int(pos[j])}\tA\tG\n")
    Gf = np.asarray(G, dtype=np.float64)
    miss = ~np.isfinite(Gf) | (Gf < 0)
    a1 = np.where(miss, 0, Gf).astype(np.int64)
    a2 = 2 - a1 if count_A1 else a1
    code = np.select([a2 == 0, a2 == 1, a2 == 2], [0, 2, 3]).astype(np.uint8)
    code[miss] = 1
    bpv = (N + 3) // 4
    pad = np.zeros((bpv * 4, M), dtype=np.uint8)
    pad[:N] = code
    q = pad.reshape(bpv, 4, M)
    rec = (q[:, 0] | (q[:, 1] << 2) | (q[:, 2] << 4) | (q[:, 3] << 6)).T.astype(np.uint8)  # (M, bpv)
    with open(f"{prefix}.bed", "wb") as fh:
        fh.write(bytes([0x6C, 0x1B, 0x01]))
        fh.write(np.ascontiguousarray(rec).tobytes())


def read_bed(prefix: str, *, count_A1: bool = True) -> np.ndarray:
    """(N, M) FP64 dosages, NaN for missing calls, from a SNP-major .bed (the format write_bed writes)."""
    with open(f"{prefix}.fam") as fh:
        N = sum(1 for line in fh if line.strip())
    raw = np.fromfile(f"{prefix}.bed", dtype=np.uint8)
    assert bytes(raw[:3]) == bytes([0x6C, 0x1B, 0x01])
    bpv = (N + 3) // 4
    rec = raw[3:].reshape(-1, bpv)
    codes = np.stack([(rec >> (2 * k)) & 3 for k in range(4)], axis=2).reshape(rec.shape[0], -1)[:, :N].T
    a2 = np.select([codes == 0, codes == 2, codes == 3], [0.0, 1.0, 2.0], np.nan)
    return 2.0 - a2 if count_A1 else a2


# --------------------------------------------------------------------------------------------------------------
# permutations and the batch driver
# --------------------------------------------------------------------------------------------------------------

def perm_orders(N: int, seed_cols, n_perm: int, seed: int = 19930909) -> np.ndarray:
    """
    (N, B, n_perm) int64 row orders: per phenotype a PCG64 stream seeded on [seed, column], n_perm rows of N
    uniforms, argsort along the row (fasterlmm/perms.py:51-55).
    """
    seed_cols = list(seed_cols)
    orders = np.empty((N, len(seed_cols), n_perm), dtype=np.int64)
    for b_pos, p in enumerate(seed_cols):
        rng = np.random.default_rng([seed, int(p)])
        orders[:, b_pos, :] = rng.random((n_perm, N)).argsort(axis=1).T
    return orders


def pack_perms(y_real: np.ndarray, orders: np.ndarray) -> np.ndarray:
    """
    Y_all = [y_real | b0 perms | b1 perms | ...], pheno-major perm columns (fasterlmm/perms.py:56-59).
    """
    N, B = y_real.shape
    n_perm = orders.shape[2]
    y_perms = np.take_along_axis(np.broadcast_to(y_real[:, :, None], (N, B, n_perm)), orders, axis=0)
    return np.concatenate([y_real, y_perms.reshape(N, B * n_perm)], axis=1)


def perm_threshold(Z_raw: np.ndarray, X: np.ndarray, Y: np.ndarray, chrom: np.ndarray, pheno_idx, *,
                   n_perm: int = 100, seed: int = 19930909, loco: bool = True, seed_idx=None,
                   Z_kin_raw: np.ndarray | None = None, chrom_kin: np.ndarray | None = None,
                   n_grid: int = 64, log_delta_min: float = -10.0, log_delta_max: float = 10.0,
                   on_chrom=None, keep_spectra: bool = False) -> tuple[dict, np.ndarray]:
    """
    Batch driver (fasterlmm/perms.py:21-68): standardise Z (and the kinship panel), pack the B real columns with
    their B * n_perm permutation columns, run the LOCO (or single-K) scan with n_real = B, slice perm_max_F.
    """
    Z_std = standardise_columns(Z_raw)
    Z_kin_std = standardise_columns(Z_kin_raw) if Z_kin_raw is not None else None
    pheno_idx = list(pheno_idx)
    B = len(pheno_idx)
    y_real = Y[:, pheno_idx]
    N = y_real.shape[0]
    seed_cols = pheno_idx if seed_idx is None else list(seed_idx)
    orders = perm_orders(N, seed_cols, n_perm, seed)
    Y_all = pack_perms(y_real, orders)
    kw = dict(n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max)
    if loco:
        res = loco_scan_compat(Z_std, X, Y_all, chrom, n_real=B, Z_kin=Z_kin_std, chrom_kin=chrom_kin,
                               on_chrom=on_chrom, keep_spectra=keep_spectra, **kw)
    else:
        res = single_k_scan_compat(Z_std, X, Y_all, n_real=B, Z_kin=Z_kin_std, **kw)
    perm_max_F = res["max_F"][B:].reshape(B, n_perm)
    return res, perm_max_F


# --------------------------------------------------------------------------------------------------------------
# batched epistasis Wald (LUX tier 2)
# --------------------------------------------------------------------------------------------------------------

def epi_wald_batched(s: np.ndarray, X: np.ndarray, Y: np.ndarray, log_delta: np.ndarray, S: np.ndarray, *,
                     n_real: int | None = None, denom_floor_rel: float = 0.01):
    """
    Batched epistasis Wald over K anchors (lux/src/fasterlmm_lux/epi/_kernel.py:21-150): for anchor k the design is
    X[k] (N, C) (shared covariates plus the anchor column), the test columns S[k] (N, M).  Per phenotype p with
    w = 1 / (s + delta_p): A = X^T W X, beta_x = A^-1 X^T W y, r = y - X beta_x, rWr = max(sum w r^2, 1e-300)
    (:74-83); per test column: B = X^T W s_m, quad = B^T A^-1 B, sWs = sum w s_m^2, num = sum w r s_m,
    denom = max(sWs - quad, 1e-300), beta = num / denom, rss = max(rWr - num^2 / denom, 1e-300),
    var_beta = rss / (N - C - 1) / denom, se = sqrt(var_beta), F = beta^2 / var_beta, and F = 0 where
    sWs - quad < denom_floor_rel sWs (:118-133).  Returns beta, se, F (K, M, n_real), max F (K, P) and the first
    test column reaching it (K, P) (:135-139; ties keep the earlier column).
    """
    K, N, C = X.shape
    P = Y.shape[1]
    M = S.shape[2]
    n_real = P if n_real is None else min(n_real, P)
    var_df = N - C - 1
    beta_o = np.empty((K, M, n_real))
    se_o = np.empty((K, M, n_real))
    f_o = np.empty((K, M, n_real))
    max_f = np.full((K, P), -np.inf)
    arg = np.zeros((K, P), dtype=np.int64)
    for k in range(K):
        Xk, Sk = X[k], S[k]
        for p in range(P):
            w = 1.0 / (s + np.exp(log_delta[p]))
            WX = w[:, None] * Xk
            A = WX.T @ Xk
            Ainv = np.linalg.inv(A)
            beta_x = Ainv @ (WX.T @ Y[:, p])
            r = Y[:, p] - Xk @ beta_x
            rWr = max(float(np.sum(w * r * r)), 1e-300)
            B = WX.T @ Sk                       # (C, M)
            quad = np.einsum("cm,cm->m", B, Ainv @ B)
            sWs = w @ (Sk * Sk)
            num = (w * r) @ Sk
            denom_raw = sWs - quad
            denom = np.maximum(denom_raw, 1e-300)
            beta = num / denom
            rss = np.maximum(rWr - num * num / denom, 1e-300)
            var_beta = rss / var_df / denom
            F = beta * beta / var_beta
            if denom_floor_rel > 0.0:
                F = np.where(denom_raw < denom_floor_rel * sWs, 0.0, F)
            j = int(np.argmax(F))
            max_f[k, p], arg[k, p] = F[j], j
            if p < n_real:
                beta_o[k, :, p], se_o[k, :, p], f_o[k, :, p] = beta, np.sqrt(var_beta), F
    return beta_o, se_o, f_o, max_f, arg


# --------------------------------------------------------------------------------------------------------------
# post-scan statistics and NA grouping
# --------------------------------------------------------------------------------------------------------------

def f_sf(F: np.ndarray, df2: int) -> np.ndarray:
    """p = F(1, df2) survival function, as the CLI computes it (fasterlmm/cli.py:405-406)."""
    import scipy.stats as ss
    return ss.f.sf(F, 1, df2)


def neg_log10_p(F: np.ndarray, df2: int) -> np.ndarray:
    """-log10 of the F(1, df2) tail, through scipy's log survival function so huge F does not underflow."""
    import scipy.stats as ss
    return -ss.f.logsf(F, 1, df2) / np.log(10.0)


def perm_quantile_threshold(perm_min_p: np.ndarray, q: float = 0.05) -> float:
    """Genome-wide threshold = linear-interpolated q quantile of the per-perm min p (fasterlmm/cli.py:128)."""
    return float(np.quantile(perm_min_p, q))


def effect_size(beta: np.ndarray, g_var: np.ndarray, p_var: float) -> np.ndarray:
    """EffectSize = beta^2 var(g) / var(y) (fasterlmm/cli.py:131-132)."""
    return beta * beta * g_var / p_var


def group_by_na(Y: np.ndarray, cols) -> list:
    """Group columns by NaN pattern (packbits key), keep rows observed in the group (fasterlmm/io.py:187-203)."""
    mask = np.isnan(Y[:, list(cols)])
    groups: dict = {}
    for j, c in enumerate(cols):
        groups.setdefault(np.packbits(mask[:, j]).tobytes(), []).append(j)
    out = []
    for js in groups.values():
        keep = np.flatnonzero(~mask[:, js[0]]).tolist()
        out.append((keep, [list(cols)[j] for j in js]))
    return out
