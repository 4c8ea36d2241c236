"""
Post-scan statistics of the CLI (fasterlmm/cli.py:128-132, :405-406) on the device.

neg_log10_pvalue: -log10 P(F(1, df2) > F) from the regularized incomplete beta in log space (finite where scipy's
f.sf underflows to 0).  perm_threshold_p: the genome-wide threshold, the linear-interpolated q-quantile of the
per-permutation minimum p (monotone in the per-permutation max F).
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


def effect_size(beta: Tensor, g_var: Tensor, p_var: Tensor) -> Tensor:
    """EffectSize = beta^2 var(g) / var(y) per (variant, phenotype) (fasterlmm/cli.py:131-132): elementwise on the
    (M, B) beta with (M,) genotype and (B,) phenotype variances."""
    return beta * beta * g_var[:, None] / p_var[None, :]
