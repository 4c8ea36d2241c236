"""
Phenotype missingness groups (fasterlmm/io.py:187-218, fasterlmm/cli.py:351-375).

Phenotypes sharing a NaN pattern share a strain subset, hence one eigendecomposition per chromosome; each group is
scanned on its own rows with its own residual degrees of freedom (df2 = n_rows - D - 1), and its permutations are
seeded on the phenotype's column in the full table so they do not depend on the grouping.
"""
from __future__ import annotations

from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np
import torch

from .perms import perm_threshold


def group_by_na(Y, cols) -> list[tuple[list[int], list[int]]]:
    """
    Group columns by NaN pattern, first-seen order; (keep_rows, cols) per pattern, keep_rows observed in the group
    (fasterlmm/io.py:187-203).  All-NaN columns come back with empty keep_rows.
    """
    Yn = Y.detach().cpu().numpy() if isinstance(Y, torch.Tensor) else np.asarray(Y)
    cols = list(cols)
    mask = np.isnan(Yn[:, cols])
    groups: dict[bytes, list[int]] = {}
    for j in range(len(cols)):
        groups.setdefault(np.packbits(mask[:, j]).tobytes(), []).append(j)
    return [(np.flatnonzero(~mask[:, js[0]]).tolist(), [cols[j] for j in js]) for js in groups.values()]


def subset_dataset(data, rows: list[int], cols: list[int]):
    """Strain subset and phenotype subset of an aligned dataset, tensors kept on their device (fasterlmm/io.py:206-218)."""
    r = torch.as_tensor(rows, dtype=torch.long, device=data.Z.device)
    pick = lambda t: None if t is None else t[r.to(t.device)]
    return SimpleNamespace(Z=pick(data.Z), Y=pick(data.Y)[:, cols], X=pick(data.X), chrom=data.chrom,
                           Z_kin=pick(getattr(data, "Z_kin", None)), chrom_kin=getattr(data, "chrom_kin", None))


@dataclass
class GroupResult:
    keep: list[int]       # strain rows of the group
    cols: list[int]       # full-table phenotype columns of the group
    df2: int              # n_rows - D - 1
    res: object           # ScanResult of the group's real columns
    perm_max_F: torch.Tensor  # (len(cols), n_perm)


def perm_threshold_grouped(data, pheno_idx, *, n_perm: int = 100, seed: int = 19930909, loco: bool = True,
                           form: str = "plain", **kw) -> list[GroupResult]:
    """
    The CLI's grouped scan (fasterlmm/cli.py:351-375): without NaNs one group over every strain; otherwise one
    perm_threshold per NaN pattern on its strain subset, permutations seeded on the full-table column, groups with
    fewer strains than D + 2 skipped.
    """
    pheno_idx = list(pheno_idx)
    D = data.X.shape[1]
    out = []
    for keep, cols in group_by_na(data.Y, pheno_idx):
        df2 = len(keep) - D - 1
        if df2 < 1:
            continue
        sub = subset_dataset(data, keep, cols)
        res, pmf = perm_threshold(sub, list(range(len(cols))), n_perm=n_perm, seed=seed, loco=loco,
                                  seed_idx=cols, form=form, **kw)
        out.append(GroupResult(keep=keep, cols=cols, df2=df2, res=res, perm_max_F=pmf))
    return out
