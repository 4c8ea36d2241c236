"""
Phenotype missingness groups (fasterlmm/io.py:187-218, fasterlmm/cli.py:351-375).

Phenotypes sharing a NaN pattern share a strain subset, hence one eigendecomposition per chromosome; each group is
scanned on its own rows with its own residual degrees of freedom (df2 = n_rows - D - 1), and its permutations are
seeded on the phenotype's column in the full table so they do not depend on the grouping.

Phenotypes of one group may ask for different permutation counts (``n_perm_of``): the reference runs one
perm_threshold per count, each paying the group's eigendecompositions again; here every count's columns join one
scan of the group -- [all real columns | the shuffles of count 1 | the shuffles of count 2 | ...] -- so the group's
kinship eigendecompositions, covariate basis and variant operands are built once.  Each column's statistics do not
depend on the other columns of the scan, so the split results are those of the separate runs.
"""
from __future__ import annotations

from dataclasses import dataclass
from types import SimpleNamespace

import numpy as np
import torch

from .core import ScanResult, _cuda_device, _f64, _to_device, scan_t, standardise_columns_t, transpose
from .perms import pack_perm_columns, perm_orders, perm_orders_device, perm_threshold


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
    n_perm: int = 0       # permutations per column of this result


def _count_sets(cols: list[int], n_perm: int, n_perm_of: dict | None) -> list[tuple[list[int], int]]:
    """Split a group's columns by permutation count, first-seen order: [(positions in cols, count)]."""
    sets: dict[int, list[int]] = {}
    for j, c in enumerate(cols):
        k = int(n_perm if n_perm_of is None else n_perm_of.get(c, n_perm))
        if k < 0:
            raise ValueError(f"negative permutation count for column {c}")
        sets.setdefault(k, []).append(j)
    return [(js, k) for k, js in sets.items()]


def _slice_result(res: ScanResult, r0: int, r1: int, p0: int, p1: int) -> ScanResult:
    """The real columns [r0, r1) and shuffled columns [p0, p1) of a joint scan, as the separate scan returns them."""
    cat = lambda v: torch.cat([v[r0:r1], v[p0:p1]])
    return ScanResult(f=res.f[:, r0:r1], beta=res.beta[:, r0:r1], se=res.se[:, r0:r1], sfve=res.sfve[:, r0:r1],
                      nullh2=res.nullh2[:, r0:r1], max_F=cat(res.max_F),
                      log_delta={c: cat(v) for c, v in res.log_delta.items()})


def perm_threshold_sets(data, sets: list[tuple[list[int], list[int], int]], *, seed: int = 19930909,
                        loco: bool = True, form: str = "plain", timers: dict | None = None,
                        **kw) -> list[tuple[ScanResult, torch.Tensor]]:
    """
    Several perm_threshold batches of one dataset in one scan.  ``sets`` = [(pheno columns of data.Y, seed columns,
    n_perm)]; returns [(ScanResult of the set's real columns, perm_max_F (B_s, n_perm))], each equal to
    ``perm_threshold(data, cols, n_perm=n_perm, seed_idx=seed_cols)`` (fasterlmm/perms.py:21-68).
    """
    dev = _cuda_device(data.Z)
    Zt = standardise_columns_t(data.Z, dev)
    Z_kin = getattr(data, "Z_kin", None)
    Zt_kin = standardise_columns_t(Z_kin, dev) if Z_kin is not None else None
    X = _f64(data.X, dev)
    Y = _f64(data.Y, dev)
    N = Y.shape[0]
    reals = [c for cols, _, _ in sets for c in cols]
    B = len(reals)
    Yt_real = transpose(Y[:, reals].contiguous()) if B else torch.empty((0, N), dtype=torch.float64, device=dev)
    parts, spans, r0, p0 = [Yt_real], [], 0, B
    for cols, seed_cols, n_perm in sets:
        b = len(cols)
        if n_perm and b:
            if N <= 16384:
                orders = perm_orders_device(N, seed_cols, n_perm, seed, dev)
            else:
                orders = torch.from_numpy(perm_orders(N, seed_cols, n_perm, seed)).to(dev)
            parts.append(pack_perm_columns(Yt_real[r0:r0 + b], orders)[b:])
        spans.append((r0, r0 + b, p0, p0 + b * n_perm, n_perm))
        r0, p0 = r0 + b, p0 + b * n_perm
    Yt_all = torch.cat(parts) if len(parts) > 1 else Yt_real
    res = scan_t(Zt, X, Yt_all, np.asarray(data.chrom), n_real=B, Zt_kin=Zt_kin,
                 chrom_kin=getattr(data, "chrom_kin", None), loco=loco, form=form, timers=timers, **kw)
    out_dev = data.Z.device if isinstance(data.Z, torch.Tensor) else dev
    res = _to_device(res, out_dev)
    out = []
    for a0, a1, q0, q1, n_perm in spans:
        r = _slice_result(res, a0, a1, q0, q1)
        out.append((r, r.max_F[a1 - a0:].reshape(a1 - a0, n_perm)))
    return out


def perm_threshold_grouped(data, pheno_idx, *, n_perm: int = 100, seed: int = 19930909, loco: bool = True,
                           form: str = "plain", n_perm_of: dict | None = None, timers: dict | None = None,
                           **kw) -> list[GroupResult]:
    """
    The CLI's grouped scan (fasterlmm/cli.py:351-375): without NaNs one group over every strain; otherwise one
    scan per NaN pattern on its strain subset, permutations seeded on the full-table column, groups with fewer
    strains than D + 2 skipped.  ``n_perm_of`` maps a full-table column to its own permutation count (default
    ``n_perm``); a group's counts share its scan and come back as one GroupResult each, in first-seen order.
    """
    pheno_idx = list(pheno_idx)
    D = data.X.shape[1]
    out = []
    for keep, cols in group_by_na(data.Y, pheno_idx):
        df2 = len(keep) - D - 1
        if df2 < 1:
            continue
        sub = subset_dataset(data, keep, cols)
        sets = _count_sets(cols, n_perm, n_perm_of)
        if len(sets) == 1:
            res, pmf = perm_threshold(sub, list(range(len(cols))), n_perm=sets[0][1], seed=seed, loco=loco,
                                      seed_idx=cols, form=form, timers=timers, **kw)
            out.append(GroupResult(keep=keep, cols=cols, df2=df2, res=res, perm_max_F=pmf, n_perm=sets[0][1]))
            continue
        runs = perm_threshold_sets(sub, [(js, [cols[j] for j in js], k) for js, k in sets], seed=seed, loco=loco,
                                   form=form, timers=timers, **kw)
        for (js, k), (res, pmf) in zip(sets, runs):
            out.append(GroupResult(keep=keep, cols=[cols[j] for j in js], df2=df2, res=res, perm_max_F=pmf, n_perm=k))
    return out
