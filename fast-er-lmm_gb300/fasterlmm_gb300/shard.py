"""
Phenotype sharding across processes, one GPU each (fasterlmm/cli.py:290-292, 615-642).

The scan has no exchange step: phenotype columns are independent once a chromosome's spectrum exists, so each rank
scans a round-robin slice of the phenotypes on its own GPU with no collective on the data path.  Permutations are
seeded on each phenotype's column in the full table (``seed_idx``), so a sharded run reproduces the unsharded one
column for column.  Results leave the ranks the way the reference's do (fasterlmm/cli.py:658-686, its shard
workers write their own phenotypes' files and the parent only merges what is on disk): ``write_shard`` writes a
rank's phenotypes' output files itself, and ``gather_results_files`` reassembles the tables on one rank through a
shared directory, so the process group carries only a barrier and the column lists.  ``gather_results`` does the
same through the process group itself (``gather_object``: every table is pickled through it, which suits small
runs and tests).
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


_KEYS = ("f", "beta", "se", "sfve", "nullh2")


def gather_results_files(shared_dir, mine: list, res: ScanResult, perm_max_F: torch.Tensor, pheno_idx: list, *,
                         group=None, dst: int = 0):
    """
    ``gather_results`` through the filesystem: every rank writes its shard's tables as .npy files into shared_dir
    (a directory all ranks see), one barrier, and rank dst reads them memory-mapped into the assembled result.  The
    process group carries the column lists and the barrier only, never the tables.  Same return values as
    gather_results; the files are removed once dst has read them.
    """
    import numpy as np
    import torch.distributed as dist
    from pathlib import Path
    root = Path(shared_dir)
    root.mkdir(parents=True, exist_ok=True)
    rank = dist.get_rank(group)
    world = dist.get_world_size(group)
    for k in _KEYS:
        np.save(root / f"rank{rank}_{k}.npy", getattr(res, k).detach().double().cpu().numpy())
    np.save(root / f"rank{rank}_perm_max_F.npy", perm_max_F.detach().double().cpu().numpy())
    cols = [None] * world if rank == dst else None
    dist.gather_object(list(mine), cols, dst=dst, group=group)  # also orders every rank's files before dst reads
    if cols is None:
        dist.barrier(group=group)  # dst is done with the files
        return None, None
    pos = {p: i for i, p in enumerate(pheno_idx)}
    B = len(pheno_idx)
    first = np.load(root / "rank0_f.npy", mmap_mode="r")
    M = first.shape[0]
    out = {k: torch.empty((M, B), dtype=torch.float64) for k in _KEYS}
    pmf_parts = [np.load(root / f"rank{r}_perm_max_F.npy") for r in range(world)]
    n_perm = next((pm.shape[1] for pm in pmf_parts if pm.ndim == 2), 0)
    pmf = torch.empty((B, n_perm), dtype=torch.float64)
    for r in range(world):
        if not cols[r]:
            continue
        idx = torch.tensor([pos[c] for c in cols[r]], dtype=torch.long)
        for k in _KEYS:
            out[k][:, idx] = torch.from_numpy(np.ascontiguousarray(np.load(root / f"rank{r}_{k}.npy", mmap_mode="r")))
        pmf[idx] = torch.from_numpy(pmf_parts[r]).reshape(len(cols[r]), n_perm)
    for r in range(world):
        for k in _KEYS + ("perm_max_F",):
            (root / f"rank{r}_{k}.npy").unlink(missing_ok=True)
    dist.barrier(group=group)
    max_F = torch.empty(B * (1 + n_perm), dtype=torch.float64)
    max_F[:B] = out["f"].max(dim=0).values if M else torch.full((B,), float("-inf"), dtype=torch.float64)
    max_F[B:] = pmf.reshape(-1)
    return ScanResult(max_F=max_F, **out), pmf


def write_shard(outdir, mine_names: list, res: ScanResult, perm_max_F: torch.Tensor, df2: int, ctx, p_var, **kw):
    """
    This rank's phenotypes' output files (gwas.tsv, perms.tsv, threshold.txt, lambda_gc.txt per phenotype, through
    output.write_batch) written by the rank itself into outdir, as the reference's shard workers write theirs: the
    files of all ranks together are the unsharded run's, and no table crosses between processes.
    """
    from .output import write_batch
    write_batch(outdir, list(mine_names), res, perm_max_F, df2, ctx, p_var, **kw)


__all__ = ["shard_phenotypes", "display_offset", "perm_threshold_shard", "gather_results", "gather_results_files",
           "write_shard"]
