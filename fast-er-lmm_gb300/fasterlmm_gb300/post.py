"""
Post-scan statistics of the CLI (fasterlmm/cli.py:128-132, :405-406) on the device.

pvalue: P(F(1, df2) > F), scipy's f.sf.  neg_log10_pvalue: -log10 of it from the regularized incomplete beta in log
space (finite where f.sf underflows to 0).  perm_threshold_p: the genome-wide threshold, the linear-interpolated q-quantile of the
per-permutation minimum p (monotone in the per-permutation max F).  lambda_gc: the genomic inflation factor
(fasterlmm/inflation.py).  rank_by_p: the p-ascending row order of the output tables.  effect_size: EffectSize.
"""
from __future__ import annotations

import torch
from torch import Tensor

from . import _lib
from .core import F64, _cuda_device, _f64, _ptr, _stream


def neg_log10_pvalue(F: Tensor, df2: int) -> Tensor:
    """-log10 p for every element of F (any shape), FP64, on the device of F (host tensors round-trip)."""
    dev = _cuda_device(F)
    Fd = _f64(F, dev)
    out = torch.empty_like(Fd)
    _lib.call("flmm_neglog10_pvalue", _ptr(Fd), Fd.numel(), int(df2), _ptr(out), _stream(dev))
    return out if not isinstance(F, Tensor) or F.is_cuda else out.to(F.device)


def pvalue(F: Tensor, df2: int) -> Tensor:
    """P(F(1, df2) > F) for every element of F (scipy.stats.f.sf(F, 1, df2), fasterlmm/cli.py:405), FP64, on the
    device of F (host tensors round-trip)."""
    dev = _cuda_device(F)
    Fd = _f64(F, dev)
    out = torch.empty_like(Fd)
    _lib.call("flmm_f_pvalue", _ptr(Fd), Fd.numel(), int(df2), _ptr(out), _stream(dev))
    return out if not isinstance(F, Tensor) or F.is_cuda else out.to(F.device)


def perm_threshold_p(perm_max_F: Tensor, df2: int, q: float = 0.05) -> Tensor:
    """
    (B,) genome-wide p threshold per phenotype: the linear-interpolated q-quantile of P(F(1, df2) > perm_max_F[b])
    over the row's permutations (fasterlmm/cli.py:128), as numpy.quantile(perm_min_p, q).
    """
    dev = _cuda_device(perm_max_F)
    Fm = _f64(perm_max_F, dev)
    B, n_perm = Fm.shape
    out = torch.empty(B, dtype=F64, device=dev)
    _lib.call("flmm_perm_threshold_p", _ptr(Fm), B, n_perm, int(df2), float(q), _ptr(out), _stream(dev))
    return out if not isinstance(perm_max_F, Tensor) or perm_max_F.is_cuda else out.to(perm_max_F.device)


CHI2_1_MEDIAN = 0.45493642311957283  # scipy.stats.chi2.ppf(0.5, 1)


def _nan_median_cols(x: Tensor) -> tuple[Tensor, Tensor]:
    """numpy.median over the non-NaN entries of each column (mean of the two middle values for even counts)."""
    valid = ~torch.isnan(x)
    n = valid.sum(dim=0)
    srt = torch.sort(torch.where(valid, x, torch.full_like(x, float("inf"))), dim=0).values
    lo = ((n - 1).clamp(min=0) // 2).unsqueeze(0)
    hi = (n // 2).clamp(max=x.shape[0] - 1).unsqueeze(0)
    med = 0.5 * (srt.gather(0, lo) + srt.gather(0, hi)).squeeze(0)
    return torch.where(n > 0, med, torch.full_like(med, float("nan"))), n


def lambda_gc(F: Tensor, df2: int) -> tuple[Tensor, Tensor]:
    """
    Genomic inflation factor per phenotype column of F (M, B) (fasterlmm/inflation.py:19-29): median over variants
    of chi2.isf(p, 1) for p = P(F(1, df2) > F), NaN p dropped, divided by chi2.ppf(0.5, 1).  Returns (lambda (B,),
    number of variants used (B,)), on the device of F.
    """
    dev = _cuda_device(F)
    Fd = _f64(F, dev)
    chisq = torch.empty_like(Fd)
    _lib.call("flmm_chisq1_from_f", _ptr(Fd), Fd.numel(), int(df2), _ptr(chisq), _stream(dev))
    med, n = _nan_median_cols(chisq.reshape(Fd.shape[0], -1))
    lam = med / CHI2_1_MEDIAN
    if isinstance(F, Tensor) and not F.is_cuda:
        return lam.to(F.device), n.to(F.device)
    return lam, n


def rank_by_p(F: Tensor, df2: int) -> Tensor:
    """
    Per phenotype column of F (M, B), the variant order of the CLI's output tables (fasterlmm/cli.py:145): p
    ascending with ties (e.g. p underflowing to 0) in variant order, NaN last.  (M, B) int64 indices.
    """
    dev = _cuda_device(F)
    p = pvalue(_f64(F, dev), df2)
    key = torch.where(torch.isnan(p), torch.full_like(p, float("inf")), p)
    order = torch.sort(key, dim=0, stable=True).indices
    return order if not isinstance(F, Tensor) or F.is_cuda else order.to(F.device)


def effect_size(beta: Tensor, g_var: Tensor, p_var: Tensor) -> Tensor:
    """EffectSize = beta^2 var(g) / var(y) per (variant, phenotype) (fasterlmm/cli.py:131-132): elementwise on the
    (M, B) beta with (M,) genotype and (B,) phenotype variances."""
    return beta * beta * g_var[:, None] / p_var[None, :]
