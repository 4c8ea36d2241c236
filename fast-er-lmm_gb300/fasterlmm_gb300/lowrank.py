"""
GPU drop-in for the low-rank path (the reference's fasterlmm/lowrank.py) and its block engine
(fasterlmm/extreme_scan.py).

The kinship is given as a factor G (N, k) of k pruned markers; with k < N the N - k null directions of K never get
an eigenvector and enter every quadratic form with weight 1 / delta.  The basis comes from the k x k Gram of the
covariate-regressed factor (or the N x N kernel when k >= N), exactly as the reference; the delta fit adds the
off-rank sum of squares and (Neff - k) log delta, and the Wald scan treats the off-rank directions as eigen-directions
with s = 0 (csrc/flmm_wald_f64.cu, flmm_wald_lowrank_f64).  FP64 throughout; results come back in the caller's
dtype and on the device of the main input.  No CPU fallback.
"""

from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import (F64, CovariateBasis, ScanResult, _alloc_outputs, _BasisView, _cuda_device, _f64, _ptr,
                   _rows_major, _stream, _to_device, _work, gram_t, kinship_from_gram, rotate_rows, transpose)


@dataclass
class LowRankBasis:
    """fasterlmm/lowrank.py:27-41: s (k,), U_eff (N, k), X (N, D), Xpinv (D, N), Neff = N - D."""
    s: Tensor
    U_eff: Tensor
    X: Tensor
    Xpinv: Tensor
    Neff: int
    Ut: Tensor = field(default=None, repr=False)  # (k, N) rows, U_eff's transpose


@dataclass
class LowRankSpectrum:
    """fasterlmm/lowrank.py:44-56: a basis with one phenotype block rotated, UY (k, P) and UUY (N, P)."""
    s: Tensor
    U_eff: Tensor
    X: Tensor
    Xpinv: Tensor
    Neff: int
    UY: Tensor
    UUY: Tensor
    Ut: Tensor = field(default=None, repr=False)
    UYt: Tensor = field(default=None, repr=False)
    UUYt: Tensor = field(default=None, repr=False)


# ---- basis and rotation (fasterlmm/lowrank.py:59-125) ----------------------------------------------------------

def _eigh_rows(A: Tensor) -> tuple[Tensor, Tensor]:
    dev = A.device
    n = A.shape[0]
    ctx = _lib.context(dev.index)
    V = A.clone()
    evals = torch.empty(n, dtype=F64, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_eigh_workspace_bytes", ctx, n))
    _lib.call("flmm_eigh", ctx, _ptr(V), n, _ptr(evals), w, wb, _stream(dev))
    return evals, V


def basis_t(Gt: Tensor, basis: CovariateBasis, sv_floor: float = 1e-10) -> tuple[Tensor, Tensor]:
    """Device basis from the factor rows Gt (k_in, N): (s (k,), Ut (k, N))."""
    k_in, N = Gt.shape
    Gr = basis.regress_out(Gt)
    if k_in < N:
        evals, V = _eigh_rows(rotate_rows(Gr, Gr))          # eigh of G_^T G_ (k_in, k_in)
        sv = evals.clamp(min=0.0).sqrt()
        keep = torch.nonzero(sv > sv_floor).flatten()
        sv = sv[keep]
        Vk = (V[keep] / sv[:, None]).contiguous()
        Ut = rotate_rows(Vk, transpose(Gr))                # U_eff^T = (V / sv)^T G_^T
        s = sv * sv / k_in
    else:
        evals, U = _eigh_rows(kinship_from_gram(gram_t(Gr), None, k_in))
        keep = torch.nonzero(evals.clamp(min=0.0) > (sv_floor * sv_floor) / k_in).flatten()
        s = evals[keep].clamp(min=0.0)
        Ut = U[keep].contiguous()
    return s.contiguous(), Ut


def rotate_t(Yt: Tensor, Ut: Tensor, basis: CovariateBasis) -> tuple[Tensor, Tensor]:
    """(UYt (P, k), UUYt (P, N)) for device columns Yt (P, N)."""
    Yr = basis.regress_out(Yt)
    UYt = rotate_rows(Yr, Ut)
    UUYt = Yr.clone()
    back = rotate_rows(UYt, transpose(Ut))                 # (P, N) = UY^T U_eff^T
    _lib.call("flmm_axpy_f64", UUYt.numel(), -1.0, _ptr(back), _ptr(UUYt), _stream(Yt.device))
    return UYt, UUYt


def lowrank_basis(G: Tensor, X: Tensor, *, sv_floor: float = 1e-10) -> LowRankBasis:
    """Drop-in for lowrank.lowrank_basis (fasterlmm/lowrank.py:59-96); G column-standardised (N, k)."""
    dev = _cuda_device(G)
    Xd = _f64(X, dev)
    basis = CovariateBasis(Xd)
    s, Ut = basis_t(_rows_major(_f64(G, dev, contiguous=False)).contiguous(), basis, sv_floor)
    N, D = Xd.shape
    return LowRankBasis(s=s, U_eff=Ut.T, X=Xd, Xpinv=basis.Xpinv[:D], Neff=N - D, Ut=Ut)


def _basis_view(b) -> CovariateBasis:
    dev = _cuda_device(b.s)
    return _BasisView(_f64(b.X, dev), _f64(b.Xpinv, dev))


def _ut(b, dev) -> Tensor:
    return b.Ut if getattr(b, "Ut", None) is not None else transpose(_f64(b.U_eff, dev, contiguous=False))


def rotate_phenos(basis: LowRankBasis, Y: Tensor) -> tuple[Tensor, Tensor]:
    """Drop-in for lowrank.rotate_phenos (fasterlmm/lowrank.py:99-111): (UY (k, P), UUY (N, P))."""
    dev = _cuda_device(basis.s, Y)
    UYt, UUYt = rotate_t(transpose(_f64(Y, dev, contiguous=False)), _ut(basis, dev), _basis_view(basis))
    return UYt.T, UUYt.T


def lowrank_rotate(G: Tensor, X: Tensor, Y: Tensor, *, sv_floor: float = 1e-10) -> LowRankSpectrum:
    """Drop-in for lowrank.lowrank_rotate (fasterlmm/lowrank.py:114-125)."""
    b = lowrank_basis(G, X, sv_floor=sv_floor)
    dev = b.s.device
    UYt, UUYt = rotate_t(transpose(_f64(Y, dev, contiguous=False)), b.Ut, _basis_view(b))
    return LowRankSpectrum(s=b.s, U_eff=b.U_eff, X=b.X, Xpinv=b.Xpinv, Neff=b.Neff, UY=UYt.T, UUY=UUYt.T, Ut=b.Ut,
                           UYt=UYt, UUYt=UUYt)


def _spec_rows(spec: LowRankSpectrum, dev) -> tuple[Tensor, Tensor, Tensor, Tensor]:
    s = _f64(spec.s, dev)
    UYt = spec.UYt if spec.UYt is not None else transpose(_f64(spec.UY, dev, contiguous=False))
    UUYt = spec.UUYt if spec.UUYt is not None else transpose(_f64(spec.UUY, dev, contiguous=False))
    return s, _ut(spec, dev), UYt, UUYt


# ---- delta fit (fasterlmm/lowrank.py:172-208) ------------------------------------------------------------------

def fit_delta_t(s: Tensor, UYt: Tensor, UUYt: Tensor, Neff: int, *, n_grid: int = 64, log_delta_min: float = -10.0,
                log_delta_max: float = 10.0, refine: bool = True) -> tuple[Tensor, Tensor]:
    dev = s.device
    k = s.shape[0]
    P = UYt.shape[0]
    st = _stream(dev)
    yy = torch.empty(P, dtype=F64, device=dev)
    _lib.call("flmm_row_sumsq_f64", _ptr(UUYt), UUYt.stride(0), P, UUYt.shape[1], _ptr(yy), st)
    ld = torch.empty(P, dtype=F64, device=dev)
    idx = torch.empty(P, dtype=torch.int32, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_f64_workspace_bytes", k, n_grid))
    _lib.call("flmm_fit_delta_lowrank_f64", _ptr(s), k, _ptr(UYt), UYt.stride(0), _ptr(yy), int(Neff), P, n_grid,
              float(log_delta_min), float(log_delta_max), int(bool(refine)), _ptr(ld), _ptr(idx), w, wb, st)
    return ld, idx


def fit_delta_grid_lowrank(spec: LowRankSpectrum, *, n_grid: int = 64, log_delta_min: float = -10.0,
                           log_delta_max: float = 10.0, refine: bool = True) -> Tensor:
    """Drop-in for lowrank.fit_delta_grid_lowrank (fasterlmm/lowrank.py:172-208)."""
    dev = _cuda_device(spec.s)
    s, _, UYt, UUYt = _spec_rows(spec, dev)
    ld, _ = fit_delta_t(s, UYt, UUYt, spec.Neff, n_grid=n_grid, log_delta_min=log_delta_min,
                        log_delta_max=log_delta_max, refine=refine)
    return ld if spec.s.is_cuda else ld.to(spec.s.device)


# ---- Wald scan (fasterlmm/lowrank.py:239-316) ------------------------------------------------------------------

def wald_t(s: Tensor, Ut: Tensor, UYt: Tensor, UUYt: Tensor, Neff: int, log_delta: Tensor, St: Tensor,
           basis: CovariateBasis, n_real: int, rows: Tensor, out: dict, max_F: Tensor) -> None:
    """Low-rank Wald of a standardised variant block St (Mc, N) into preallocated outputs at `rows`."""
    dev = s.device
    k, N = Ut.shape
    P = UYt.shape[0]
    USt, UUSt = rotate_t(St, Ut, basis)
    Mc = USt.shape[0]
    w, wb = _work.get(dev, _lib.query_bytes("flmm_wald_lowrank_f64_workspace_bytes", k, N, P, Mc))
    _lib.call("flmm_wald_lowrank_f64", _ptr(s), k, _ptr(UYt), UYt.stride(0), _ptr(UUYt), UUYt.stride(0), N, int(Neff),
              _ptr(log_delta), P, n_real, _ptr(USt), USt.stride(0), _ptr(UUSt), UUSt.stride(0), Mc, _ptr(rows),
              _ptr(out["f"]), _ptr(out["beta"]), _ptr(out["se"]), _ptr(out["sfve"]), n_real, _ptr(max_F), w, wb,
              _stream(dev))
    _lib.call("flmm_fill_nullh2", _ptr(log_delta), n_real, _ptr(rows), Mc, _ptr(out["nullh2"]), n_real, _stream(dev))


def snp_wald_scan_lowrank(spec: LowRankSpectrum, log_delta: Tensor, S: Tensor, *, snp_chunk: int | None = None,
                          pheno_chunk: int | None = None, n_real: int | None = None) -> ScanResult:
    """
    Drop-in for lowrank.snp_wald_scan_lowrank (fasterlmm/lowrank.py:239-316).  snp_chunk / pheno_chunk are
    accepted for signature compatibility; the kernels tile both axes themselves.
    """
    dev = _cuda_device(spec.s, S)
    s, Ut, UYt, UUYt = _spec_rows(spec, dev)
    P = UYt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    St = _rows_major(_f64(S, dev, contiguous=False)).contiguous()
    M = St.shape[0]
    out, max_F = _alloc_outputs(M, n_real, P, dev)
    rows = torch.arange(M, dtype=torch.int64, device=dev)
    wald_t(s, Ut, UYt, UUYt, spec.Neff, _f64(log_delta, dev), St, _basis_view(spec), n_real, rows, out, max_F)
    res = ScanResult(max_F=max_F, **out)
    return _as(res, S)


def _as(res: ScanResult, like) -> ScanResult:
    """Results on the device and in the dtype of `like` (the reference returns its input dtype)."""
    dev = like.device if isinstance(like, Tensor) else res.f.device
    dt = like.dtype if isinstance(like, Tensor) and like.is_floating_point() else F64
    res = _to_device(res, dev)
    if dt == F64:
        return res
    return ScanResult(f=res.f.to(dt), beta=res.beta.to(dt), se=res.se.to(dt), sfve=res.sfve.to(dt),
                      nullh2=res.nullh2.to(dt), max_F=res.max_F.to(dt), log_delta=res.log_delta)


# ---- chromosome loops (fasterlmm/lowrank.py:322-373, fasterlmm/extreme_scan.py:28-125) --------------------------

def _loco_scan_core(chroms: list, block_source, M: int, G: Tensor, g_chrom: np.ndarray, X: Tensor, Y: Tensor, *,
                    n_real: int | None, on_chrom, like) -> ScanResult:
    """
    The LOCO loop of fasterlmm/extreme_scan.py:28-77 on the device: per chromosome c the factor drops c's markers,
    the basis, rotation and delta fit are computed once, and every (Z_block (N, Mc), col_idx) that
    block_source(c) yields is scanned against them.
    """
    dev = _cuda_device(G, X, Y)
    Gt = _rows_major(_f64(G, dev, contiguous=False)).contiguous()
    Xd = _f64(X, dev)
    basis = CovariateBasis(Xd)
    Yt = transpose(_f64(Y, dev, contiguous=False))
    N, D = Xd.shape
    P = Yt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    out, max_F = _alloc_outputs(M, n_real, P, dev, zero=True)  # a block reader need not cover every variant
    g_chrom = np.asarray(g_chrom)
    log_deltas = {}
    for k_idx, c in enumerate(chroms):
        keep = torch.from_numpy(np.flatnonzero(g_chrom != c)).to(dev)
        s, Ut = basis_t(Gt.index_select(0, keep), basis)
        UYt, UUYt = rotate_t(Yt, Ut, basis)
        ld, _ = fit_delta_t(s, UYt, UUYt, N - D)
        log_deltas[c] = ld
        for Z_b, cidx in block_source(c):
            St = _rows_major(_f64(Z_b, dev, contiguous=False)).contiguous()
            rows = torch.as_tensor(np.asarray(cidx), dtype=torch.int64).to(dev)
            wald_t(s, Ut, UYt, UUYt, N - D, ld, St, basis, n_real, rows, out, max_F)
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(chroms))
    return _as(ScanResult(max_F=max_F, log_delta=log_deltas, **out), like)


def _blocks(Z: Tensor, z_chrom: np.ndarray, c, block_size: int):
    idx = np.flatnonzero(np.asarray(z_chrom) == c)
    for b0 in range(0, idx.size, block_size):
        cols = idx[b0:b0 + block_size]
        yield Z[:, torch.from_numpy(cols).to(Z.device) if isinstance(Z, Tensor) else cols], cols


def loco_scan_lowrank(G: Tensor, g_chrom: np.ndarray, Z: Tensor, z_chrom: np.ndarray, X: Tensor, Y: Tensor, *,
                      n_real: int | None = None, on_chrom=None) -> ScanResult:
    """Drop-in for lowrank.loco_scan_lowrank (fasterlmm/lowrank.py:322-359); G and Z column-standardised."""
    z_chrom = np.asarray(z_chrom)
    chroms = sorted(np.unique(z_chrom).tolist())
    M = Z.shape[1]
    return _loco_scan_core(chroms, lambda c: _blocks(Z, z_chrom, c, max(M, 1)), M, G, g_chrom, X, Y,
                           n_real=n_real, on_chrom=on_chrom, like=Z)


def single_k_scan_lowrank(G: Tensor, Z: Tensor, X: Tensor, Y: Tensor, *, n_real: int | None = None) -> ScanResult:
    """Drop-in for lowrank.single_k_scan_lowrank (fasterlmm/lowrank.py:362-373)."""
    spec = lowrank_rotate(G, X, Y)
    ld = fit_delta_grid_lowrank(spec)
    return snp_wald_scan_lowrank(spec, ld, Z, n_real=n_real)


def loco_scan_resident(Z: Tensor, z_chrom: np.ndarray, G: Tensor, g_chrom: np.ndarray, X: Tensor, Y: Tensor, *,
                       n_real: int | None = None, block_size: int = 8192, dtype: torch.dtype = torch.float32,
                       on_chrom=None) -> ScanResult:
    """
    Drop-in for extreme_scan.loco_scan_resident (fasterlmm/extreme_scan.py:104-125): the test variants of each
    chromosome are scanned in blocks of block_size against the chromosome's cached spectrum.  The arithmetic is
    FP64; results are returned in ``dtype`` (the reference's FP32 default computes in FP32).
    """
    z_chrom = np.asarray(z_chrom)
    chroms = sorted(set(z_chrom.tolist()))
    like = torch.empty(0, dtype=dtype, device=Z.device if isinstance(Z, Tensor) else "cpu")
    return _loco_scan_core(chroms, lambda c: _blocks(Z, z_chrom, c, block_size), Z.shape[1], G, g_chrom, X, Y,
                           n_real=n_real, on_chrom=on_chrom, like=like)


def loco_scan_blocks(block_source, chroms: list, M: int, G: Tensor, g_chrom: np.ndarray, X: Tensor, Y: Tensor, *,
                     n_real: int | None = None, dtype: torch.dtype = torch.float32, on_chrom=None,
                     device: torch.device | None = None) -> ScanResult:
    """
    The streamed form of fasterlmm/extreme_scan.py:80-101 for any block reader: block_source(c) yields the
    standardised test blocks (Z_block (N, Mc), column indices into the M outputs) of chromosome c, e.g. decoded
    from disk a block at a time, so the N x M genotype matrix never has to be resident.
    """
    like = torch.empty(0, dtype=dtype, device=device or "cpu")
    return _loco_scan_core(list(chroms), block_source, M, G, g_chrom, X, Y, n_real=n_real, on_chrom=on_chrom,
                           like=like)


__all__ = ["LowRankBasis", "LowRankSpectrum", "lowrank_basis", "rotate_phenos", "lowrank_rotate",
           "fit_delta_grid_lowrank", "snp_wald_scan_lowrank", "loco_scan_lowrank", "single_k_scan_lowrank",
           "loco_scan_resident", "loco_scan_blocks"]
