"""
Phenotype sharding across processes, one GPU each (fasterlmm/cli.py:290-292, 615-642).

The scan has no exchange step: phenotype columns are independent once a chromosome's spectrum exists, so each rank
scans a round-robin slice of the phenotypes on its own GPU with no collective on the data path.  Permutations are
seeded on each phenotype's column in the full table (``seed_idx``), so a sharded run reproduces the unsharded one
column for column.  ``gather_results`` then collects the shards' results on one rank (a result collection after
the scan, over any torch.distributed backend: gloo for host tensors, NCCL for device tensors).
"""

from __future__ import annotations

import torch

from .core import ScanResult


def shard_phenotypes(pheno_list: list, shard_i: int, shard_n: int) -> list:
    """The round-robin slice of rank shard_i out of shard_n (fasterlmm/cli.py:292)."""
    if not 0 <= shard_i < shard_n:
        raise ValueError(f"shard {shard_i} out of range for {shard_n} shards")
    return list(pheno_list)[shard_i::shard_n]


def display_offset(pheno_list: list, shard_i: int, shard_n: int) -> int:
    """Phenotypes carried by the lower-ranked shards, the running count a progress display starts from
    (fasterlmm/cli.py:289-291)."""
    return sum(len(list(pheno_list)[k::shard_n]) for k in range(shard_i))


def perm_threshold_shard(data, pheno_idx: list, shard_i: int, shard_n: int, *, scan=None, **kw):
    """
    Scan this rank's round-robin slice of pheno_idx: (the slice, ScanResult, perm_max_F).  ``scan`` defaults to
    fasterlmm_gb300.perms.perm_threshold; the slice's columns seed their own permutations, as in the full run.
    """
    if scan is None:
        from .perms import perm_threshold as scan
    mine = shard_phenotypes(pheno_idx, shard_i, shard_n)
    res, pmf = scan(data, mine, seed_idx=list(mine), **kw)
    return mine, res, pmf


def gather_results(mine: list, res: ScanResult, perm_max_F: torch.Tensor, pheno_idx: list, *, group=None,
                   dst: int = 0):
    """
    Collect every rank's shard on rank dst and put the columns back in pheno_idx order: (ScanResult over all
    phenotypes, perm_max_F (B, n_perm)) on dst, (None, None) elsewhere.  Uses torch.distributed.gather_object, so
    any backend works; the tensors travel through host memory.
    """
    import torch.distributed as dist
    payload = (list(mine), {k: getattr(res, k).detach().cpu() for k in ("f", "beta", "se", "sfve", "nullh2")},
               perm_max_F.detach().cpu())
    world = dist.get_world_size(group)
    parts = [None] * world if dist.get_rank(group) == dst else None
    dist.gather_object(payload, parts, dst=dst, group=group)
    if parts is None:
        return None, None
    pos = {p: i for i, p in enumerate(pheno_idx)}
    M = parts[0][1]["f"].shape[0]
    B = len(pheno_idx)
    n_perm = parts[0][2].shape[1] if parts[0][2].dim() == 2 else 0
    out = {k: torch.empty((M, B), dtype=torch.float64) for k in ("f", "beta", "se", "sfve", "nullh2")}
    pmf = torch.empty((B, n_perm), dtype=torch.float64)
    max_F = torch.empty(B * (1 + n_perm), dtype=torch.float64)
    for cols, det, pm in parts:
        idx = torch.tensor([pos[c] for c in cols], dtype=torch.long)
        for k in out:
            out[k][:, idx] = det[k].double()
        if len(cols):
            pmf[idx] = pm.double()
    # max_F over [reals | perms]: the reals' maxima are the column maxima of f, the perms' are perm_max_F
    max_F[:B] = out["f"].max(dim=0).values if M else torch.full((B,), float("-inf"), dtype=torch.float64)
    max_F[B:] = pmf.reshape(-1)
    return ScanResult(max_F=max_F, **out), pmf


__all__ = ["shard_phenotypes", "display_offset", "perm_threshold_shard", "gather_results"]
