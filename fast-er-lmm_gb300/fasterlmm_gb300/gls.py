"""
GPU drop-in for the plain GLS scan path of ``fasterlmm.core`` (the reference's fasterlmm/core.py:89-451).

The plain path keeps the covariates in the model: the kinship K + 1e-6 I is eigendecomposed as is, X and Y are
rotated by U^T, every delta needs the (C, C) Gram A = X~^T W X~ (ML or REML loss), and each test carries the
quadratic form B^T A^-1 B with B = X~^T W s.  Same names, signatures, dataclass and errors as the reference; the work
is done by the FP64 kernels of csrc/flmm_gls.cu (1 <= C <= 30 covariate columns).  No CPU fallback.

Layouts: the kernels read row-major transposes -- Ut (N, N) with one eigenvector per row, Xrt (C, N), Yrt (P, N),
Srt (M, N) -- and ``Spectrum`` exposes the reference's (N, ...) views of them.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import (F64, ScanResult, _alloc_outputs, _chrom_blocks, _cuda_device, _f64, _ptr, _rows_major, _stream,
                   _take_rows, _to_device, _work, gram_t, kinship_from_gram, rotate_rows, transpose)

JITTER = 1e-6  # eigendecompose's diagonal jitter (fasterlmm/core.py:89)


@dataclass
class Spectrum:
    """
    Eigendecomposition with rotated design and phenotypes (fasterlmm/core.py:19-31): s (N,), U (N, N) eigenvectors
    as columns, X_rot = U^T X (N, C), Y_rot = U^T Y (N, P).  U, X_rot and Y_rot are transposed views of ``Ut``,
    ``Xrt`` and ``Yrt``, the layouts the kernels read.
    """
    s: Tensor
    U: Tensor
    X_rot: Tensor
    Y_rot: Tensor
    Ut: Tensor = field(default=None, repr=False)
    Xrt: Tensor = field(default=None, repr=False)
    Yrt: Tensor = field(default=None, repr=False)


def _rows(view: Tensor, rows: Tensor | None, dev: torch.device) -> Tensor:
    """Row-major transpose of an (N, k) view: the stored rows when given, else a transposed copy."""
    return rows if rows is not None else transpose(_f64(view, dev, contiguous=False))


def _spectrum_rows(spec: Spectrum, dev: torch.device) -> tuple[Tensor, Tensor, Tensor]:
    s = _f64(spec.s, dev)
    return s, _rows(spec.X_rot, spec.Xrt, dev), _rows(spec.Y_rot, spec.Yrt, dev)


# ---- eigendecomposition and rotation (fasterlmm/core.py:89-116) ------------------------------------------------

def eigh_rows(K: Tensor, jitter: float = JITTER) -> tuple[Tensor, Tensor]:
    """eigh(K + jitter I) on device, eigenvalues clamped at 0: (s (N,), Ut (N, N) eigenvector rows)."""
    dev = K.device
    N = K.shape[0]
    ctx = _lib.context(dev.index)
    st = _stream(dev)
    A = K.clone()
    _lib.call("flmm_shift_diagonal_f64", _ptr(A), N, N, float(jitter), st)
    evals = torch.empty(N, dtype=F64, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_eigh_workspace_bytes", ctx, N))
    _lib.call("flmm_eigh", ctx, _ptr(A), N, _ptr(evals), w, wb, st)
    s = torch.empty_like(evals)
    _lib.call("flmm_clamp_nonneg_f64", _ptr(evals), N, _ptr(s), st)
    return s, A


def eigendecompose(K: Tensor, jitter: float = JITTER) -> tuple[Tensor, Tensor]:
    """Drop-in for core.eigendecompose (fasterlmm/core.py:89-102): (s, U) with eigenvectors as columns of U."""
    dev = _cuda_device(K)
    s, Ut = eigh_rows(_f64(K, dev), jitter)
    out_dev = K.device if isinstance(K, Tensor) else dev
    if out_dev.type != "cuda":
        return s.to(out_dev), Ut.T.to(out_dev)
    return s, Ut.T


def rotate_t(K: Tensor, X: Tensor, Yt: Tensor) -> tuple[Tensor, Tensor, Tensor, Tensor]:
    """Device rotation: (s, Ut, Xrt (C, N), Yrt (P, N))."""
    s, Ut = eigh_rows(K)
    Xrt = rotate_rows(transpose(X), Ut)
    Yrt = rotate_rows(Yt, Ut)
    return s, Ut, Xrt, Yrt


def rotate(K: Tensor, X: Tensor, Y: Tensor) -> Spectrum:
    """Drop-in for core.rotate (fasterlmm/core.py:105-116)."""
    dev = _cuda_device(K)
    s, Ut, Xrt, Yrt = rotate_t(_f64(K, dev), _f64(X, dev), transpose(_f64(Y, dev)))
    out_dev = K.device if isinstance(K, Tensor) else dev
    mv = (lambda t: t) if out_dev.type == "cuda" else (lambda t: t.to(out_dev))
    return Spectrum(s=mv(s), U=mv(Ut.T), X_rot=mv(Xrt.T), Y_rot=mv(Yrt.T), Ut=Ut, Xrt=Xrt, Yrt=Yrt)


# ---- losses and the delta fit (fasterlmm/core.py:122-264) ------------------------------------------------------

def loss_t(log_delta: Tensor, s: Tensor, Xrt: Tensor, Yrt: Tensor, *, reml: bool = False,
           per_column: bool = False) -> Tensor:
    """(G, P) grid losses, or (P,) at one log delta per column, on device rows."""
    dev = s.device
    N = s.shape[0]
    C = Xrt.shape[0]
    P = Yrt.shape[0]
    G = log_delta.shape[0]
    ld = _f64(log_delta, dev)
    out = torch.empty((P,) if per_column else (G, P), dtype=F64, device=dev)
    if per_column:
        w, wb = None, 0
    else:
        w, wb = _work.get(dev, _lib.query_bytes("flmm_gls_loss_workspace_bytes", N, C, P, G))
    _lib.call("flmm_gls_loss_f64", _ptr(s), N, _ptr(Xrt), Xrt.stride(0), C, _ptr(Yrt), Yrt.stride(0), P, _ptr(ld),
              G, int(per_column), int(bool(reml)), _ptr(out), w, wb, _stream(dev))
    return out


def _profile_loss(log_delta: Tensor, s: Tensor, X_rot: Tensor, Y_rot: Tensor, *, reml: bool = False) -> Tensor:
    """Drop-in for core._profile_loss (fasterlmm/core.py:148-187): (G, P) -2 log L."""
    dev = _cuda_device(s, X_rot, Y_rot)
    out = loss_t(_f64(log_delta, dev), _f64(s, dev), transpose(_f64(X_rot, dev)), transpose(_f64(Y_rot, dev)),
                 reml=reml)
    return out if not isinstance(s, Tensor) or s.is_cuda else out.to(s.device)


def _profile_loss_per_pheno(log_delta: Tensor, s: Tensor, X_rot: Tensor, Y_rot: Tensor, *,
                            reml: bool = False) -> Tensor:
    """Drop-in for core._profile_loss_per_pheno (fasterlmm/core.py:190-224): (P,) at one log delta per column."""
    dev = _cuda_device(s, X_rot, Y_rot)
    out = loss_t(_f64(log_delta, dev), _f64(s, dev), transpose(_f64(X_rot, dev)), transpose(_f64(Y_rot, dev)),
                 reml=reml, per_column=True)
    return out if not isinstance(s, Tensor) or s.is_cuda else out.to(s.device)


def nLLeval(delta, s: Tensor, X_rot: Tensor, y_rot: Tensor) -> Tensor:
    """Drop-in for core.nLLeval (fasterlmm/core.py:122-145): ML -2 log L of one phenotype at one delta (0-d)."""
    dev = _cuda_device(s, X_rot, y_rot)
    ld = torch.log(torch.as_tensor(delta, dtype=F64, device=dev)).reshape(1)
    y = _f64(y_rot, dev).reshape(1, -1)
    out = loss_t(ld, _f64(s, dev), transpose(_f64(X_rot, dev)), y, per_column=True)[0]
    return out if not isinstance(s, Tensor) or s.is_cuda else out.to(s.device)


def fit_delta_t(s: Tensor, Xrt: Tensor, Yrt: Tensor, *, n_grid: int = 64, log_delta_min: float = -10.0,
                log_delta_max: float = 10.0, refine: bool = True, reml: bool = False) -> tuple[Tensor, Tensor]:
    """Grid + golden-section GLS fit on device rows: (log_delta (P,), grid index (P,))."""
    dev = s.device
    N = s.shape[0]
    C = Xrt.shape[0]
    P = Yrt.shape[0]
    ld = torch.empty(P, dtype=F64, device=dev)
    idx = torch.empty(P, dtype=torch.int32, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_gls_workspace_bytes", N, C, P, n_grid))
    _lib.call("flmm_fit_delta_gls_f64", _ptr(s), N, _ptr(Xrt), Xrt.stride(0), C, _ptr(Yrt), Yrt.stride(0), P, n_grid,
              float(log_delta_min), float(log_delta_max), int(bool(refine)), int(bool(reml)), _ptr(ld), _ptr(idx), w,
              wb, _stream(dev))
    return ld, idx


def fit_delta_grid(spectrum: Spectrum, *, n_grid: int = 64, log_delta_min: float = -10.0,
                   log_delta_max: float = 10.0, refine: bool = True, reml: bool = False) -> Tensor:
    """Drop-in for core.fit_delta_grid (fasterlmm/core.py:227-264)."""
    dev = _cuda_device(spectrum.s)
    s, Xrt, Yrt = _spectrum_rows(spectrum, dev)
    ld, _ = fit_delta_t(s, Xrt, Yrt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                        refine=refine, reml=reml)
    return ld if spectrum.s.is_cuda else ld.to(spectrum.s.device)


# ---- Wald scan (fasterlmm/core.py:295-375) ---------------------------------------------------------------------

def wald_t(s: Tensor, Xrt: Tensor, Yrt: Tensor, log_delta: Tensor, Srt: Tensor, n_real: int, rows: Tensor,
           out: dict, max_F: Tensor) -> None:
    """GLS Wald of one rotated variant block Srt (Mc, N) into preallocated outputs at `rows`; raises max_F."""
    dev = s.device
    N = s.shape[0]
    C = Xrt.shape[0]
    P = Yrt.shape[0]
    Mc = Srt.shape[0]
    w, wb = _work.get(dev, _lib.query_bytes("flmm_wald_gls_workspace_bytes", N, C, P))
    _lib.call("flmm_wald_gls_f64", _ptr(s), N, _ptr(Xrt), Xrt.stride(0), C, _ptr(Yrt), Yrt.stride(0), _ptr(log_delta),
              P, n_real, _ptr(Srt), Srt.stride(0), Mc, _ptr(rows), _ptr(out["f"]), _ptr(out["beta"]), _ptr(out["se"]),
              _ptr(out["sfve"]), n_real, _ptr(max_F), w, wb, _stream(dev))
    _lib.call("flmm_fill_nullh2", _ptr(log_delta), n_real, _ptr(rows), Mc, _ptr(out["nullh2"]), n_real, _stream(dev))


def snp_wald_scan(spectrum: Spectrum, log_delta: Tensor, S_rot: Tensor, *, snp_chunk: int | None = None,
                  pheno_chunk: int | None = None, n_real: int | None = None) -> ScanResult:
    """
    Drop-in for core.snp_wald_scan (fasterlmm/core.py:295-375).  S_rot (N, M) is pre-rotated.  snp_chunk /
    pheno_chunk are accepted for signature compatibility; the kernels tile both axes themselves.
    """
    dev = _cuda_device(spectrum.s, S_rot)
    s, Xrt, Yrt = _spectrum_rows(spectrum, dev)
    P = Yrt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    Srt = _rows_major(_f64(S_rot, dev, contiguous=False)).contiguous()
    M = Srt.shape[0]
    out, max_F = _alloc_outputs(M, n_real, P, dev)
    rows = torch.arange(M, dtype=torch.int64, device=dev)
    wald_t(s, Xrt, Yrt, _f64(log_delta, dev), Srt, n_real, rows, out, max_F)
    res = ScanResult(max_F=max_F, **out)
    return _to_device(res, S_rot.device if isinstance(S_rot, Tensor) else dev)


# ---- LOCO / single-K drivers (fasterlmm/core.py:381-451) --------------------------------------------------------

def scan_t(Zt: Tensor, X: Tensor, Yt: Tensor, chrom: np.ndarray, *, n_real: int, on_chrom=None,
           Zt_kin: Tensor | None = None, chrom_kin: np.ndarray | None = None, loco: bool = True) -> ScanResult:
    """
    Plain GLS engine on device tensors: Zt (M, N) standardised tested variants, X (N, C), Yt (P, N).  The Gram of
    every kinship chromosome is computed once and each LOCO kinship is the total minus the chromosome's block.
    """
    dev = Zt.device
    M, N = Zt.shape
    P = Yt.shape[0]
    out, max_F = _alloc_outputs(M, n_real, P, dev)
    kin_Zt = Zt if Zt_kin is None else Zt_kin
    kin_chrom = np.asarray(chrom if Zt_kin is None else chrom_kin)
    test_blocks = _chrom_blocks(chrom, dev)
    if loco:
        kin_blocks = _chrom_blocks(kin_chrom, dev)
        grams = {c: gram_t(_take_rows(kin_Zt, b)) for c, b in kin_blocks.items()}
        Gtot = torch.zeros((N, N), dtype=F64, device=dev)
        for G in grams.values():
            _lib.call("flmm_axpy_f64", N * N, 1.0, _ptr(G), _ptr(Gtot), _stream(dev))
        units = [(c, test_blocks[c]) for c in test_blocks]
    else:
        Gtot = gram_t(kin_Zt)
        grams = {}
        units = [(None, (torch.arange(M, device=dev), slice(0, M)))]
    M_kin = kin_Zt.shape[0]
    log_deltas = {}
    for k_idx, (c, blk) in enumerate(units):
        if c is None:
            K = kinship_from_gram(Gtot, None, M_kin)
        else:
            K = kinship_from_gram(Gtot, grams.get(c), M_kin - int((kin_chrom == c).sum()))
        s, Ut, Xrt, Yrt = rotate_t(K, X, Yt)
        ld, _ = fit_delta_t(s, Xrt, Yrt)
        Srt = rotate_rows(_take_rows(Zt, blk).contiguous(), Ut)
        wald_t(s, Xrt, Yrt, ld, Srt, n_real, blk[0], out, max_F)
        log_deltas[c if c is not None else 0] = ld
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(units))
    return ScanResult(max_F=max_F, log_delta=log_deltas, **out)


def loco_scan(Z: Tensor, X: Tensor, Y: Tensor, chrom: np.ndarray, *, n_real: int | None = None, on_chrom=None,
              Z_kin: Tensor | None = None, chrom_kin: np.ndarray | None = None) -> ScanResult:
    """Drop-in for core.loco_scan (fasterlmm/core.py:381-436); Z (and Z_kin) pre-standardised (N, M)."""
    if (Z_kin is None) != (chrom_kin is None):
        raise ValueError("Z_kin and chrom_kin go together")
    dev = _cuda_device(Z)
    Zt = _rows_major(_f64(Z, dev, contiguous=False))
    Zt_kin = None if Z_kin is None else _rows_major(_f64(Z_kin, dev, contiguous=False))
    Yt = transpose(_f64(Y, dev, contiguous=False))
    P = Yt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    res = scan_t(Zt, _f64(X, dev), Yt, np.asarray(chrom), n_real=n_real, on_chrom=on_chrom, Zt_kin=Zt_kin,
                 chrom_kin=chrom_kin, loco=True)
    return _to_device(res, Z.device if isinstance(Z, Tensor) else dev)


def single_k_scan(Z: Tensor, X: Tensor, Y: Tensor, *, n_real: int | None = None,
                  Z_kin: Tensor | None = None) -> ScanResult:
    """Drop-in for core.single_k_scan (fasterlmm/core.py:439-451)."""
    dev = _cuda_device(Z)
    Zt = _rows_major(_f64(Z, dev, contiguous=False))
    Zt_kin = None if Z_kin is None else _rows_major(_f64(Z_kin, dev, contiguous=False))
    Yt = transpose(_f64(Y, dev, contiguous=False))
    P = Yt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    res = scan_t(Zt, _f64(X, dev), Yt, np.zeros(Zt.shape[0], dtype=np.int64), n_real=n_real, Zt_kin=Zt_kin,
                 loco=False)
    return _to_device(res, Z.device if isinstance(Z, Tensor) else dev)


__all__ = ["Spectrum", "eigendecompose", "rotate", "nLLeval", "_profile_loss", "_profile_loss_per_pheno",
           "fit_delta_grid", "snp_wald_scan", "loco_scan", "single_k_scan"]
