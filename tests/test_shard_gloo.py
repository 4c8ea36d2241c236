"""
Multi-process paths on CPU with the gloo backend (world size 2, 127.0.0.1): the round-robin phenotype shards,
the gathers that reassemble them in column order (through the process group and through a shared directory), and
bench.py's slowest-rank timing.  The scan itself is a
stand-in here (these tests run without a GPU); its sharded and unsharded results must agree column for column.
"""
from __future__ import annotations

import os
import socket
import sys
from pathlib import Path

import pytest
import torch
import torch.multiprocessing as mp

REPO = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _fake_scan(data, pheno_idx, *, seed_idx, n_perm=3, **kw):
    """Deterministic per-column outputs that depend only on the column's full-table index (its seed column)."""
    from fasterlmm_gb300.core import ScanResult
    M = data["M"]
    cols = torch.tensor(seed_idx, dtype=torch.float64)
    m = torch.arange(M, dtype=torch.float64)[:, None]
    f = (m + 1.0) * (cols[None, :] + 0.5)
    det = {"f": f, "beta": f / 7, "se": f / 11, "sfve": f / 13, "nullh2": 0 * f + cols[None, :] / 100}
    pmf = cols[:, None] * 10 + torch.arange(n_perm, dtype=torch.float64)[None, :]
    max_F = torch.cat([f.max(dim=0).values, pmf.reshape(-1)])
    return ScanResult(max_F=max_F, **det), pmf


def _worker_files(rank, world, port, out_path, shared):
    sys.path[:0] = [str(REPO / "fast-er-lmm_gb300"), str(REPO)]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from fasterlmm_gb300 import shard
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pheno = list(range(3, 14))
        data = {"M": 5}
        mine, res, pmf = shard.perm_threshold_shard(data, pheno, rank, world, scan=_fake_scan)
        full, full_pmf = shard.gather_results_files(shared, mine, res, pmf, pheno)
        if rank == 0:
            ref, ref_pmf = _fake_scan(data, pheno, seed_idx=pheno)
            ok = all(torch.equal(getattr(full, k), getattr(ref, k)) for k in ("f", "beta", "se", "sfve", "nullh2",
                                                                              "max_F"))
            ok = ok and torch.equal(full_pmf, ref_pmf) and not any(Path(shared).iterdir())
            Path(out_path).write_text("ok" if ok else "mismatch")
        else:
            assert full is None
    finally:
        dist.destroy_process_group()


def _worker(rank, world, port, out_path):
    sys.path[:0] = [str(REPO / "fast-er-lmm_gb300"), str(REPO)]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist
    from fasterlmm_gb300 import shard
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        pheno = list(range(3, 14))
        data = {"M": 5}
        mine, res, pmf = shard.perm_threshold_shard(data, pheno, rank, world, scan=_fake_scan)
        assert mine == pheno[rank::world]
        full, full_pmf = shard.gather_results(mine, res, pmf, pheno)
        slowest = bench.max_over_ranks(1.0 + rank, world)
        if rank == 0:
            ref, ref_pmf = _fake_scan(data, pheno, seed_idx=pheno)
            ok = all(torch.equal(getattr(full, k), getattr(ref, k)) for k in ("f", "beta", "se", "sfve", "nullh2",
                                                                              "max_F"))
            ok = ok and torch.equal(full_pmf, ref_pmf) and slowest == float(world)
            ok = ok and shard.display_offset(pheno, 1, world) == len(pheno[0::world])
            Path(out_path).write_text("ok" if ok else "mismatch")
        else:
            assert full is None and slowest == float(world)
    finally:
        dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_sharded_scan_gathers_to_the_unsharded_result(tmp_path):
    out = tmp_path / "result.txt"
    mp.spawn(_worker, args=(2, _free_port(), str(out)), nprocs=2, join=True)
    assert out.read_text() == "ok"


@pytest.mark.timeout(120)
def test_sharded_scan_gathers_through_files(tmp_path):
    """The filesystem gather reassembles the same result, and removes its files."""
    out = tmp_path / "result.txt"
    shared = tmp_path / "shards"
    mp.spawn(_worker_files, args=(2, _free_port(), str(out), str(shared)), nprocs=2, join=True)
    assert out.read_text() == "ok"


def test_shard_slices_are_round_robin():
    from fasterlmm_gb300 import shard
    p = list(range(10))
    assert [shard.shard_phenotypes(p, i, 3) for i in range(3)] == [[0, 3, 6, 9], [1, 4, 7], [2, 5, 8]]
    with pytest.raises(ValueError):
        shard.shard_phenotypes(p, 3, 3)
