"""
PLINK .bed/.bim/.fam input with the genotype decode on the GPU (the reference reads the same files through
pysnptools: fasterlmm/io.py:54-67 for the resident path, fasterlmm/io_stream.py:28-161 for the streamed one).

The .bed stays memory-mapped on the host; a block of variants is copied to the device as its raw 2-bit records
(a quarter byte per call) and decoded there (flmm_bed_decode) into int8 dosages, which flmm_standardise_dosage
turns into the standardised variant-major rows the scans read.  ``chrom_blocks`` feeds
fasterlmm_gb300.lowrank.loco_scan_blocks, so a streamed scan never holds the N x M genotype matrix.

Conventions follow the reference: count_A1 (default) counts the first allele, missing calls are NaN in dosages,
rows are the .fam order filtered to a kept strain set (fasterlmm/io_stream.py:44-57), chromosome codes are numeric
(PLINK's X, Y, XY, MT -> 23, 24, 25, 26), positions are the .bim base-pair column.
"""

from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import F64, _cuda_device, _ptr, _stream

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])  # PLINK 1 .bed, SNP-major
_CHROM_CODES = {"X": 23, "Y": 24, "XY": 25, "MT": 26, "M": 26}


def _chrom_code(c: str) -> float:
    c = c.strip()
    if c.lower().startswith("chr"):
        c = c[3:]
    return float(_CHROM_CODES.get(c.upper(), c))


def read_fam(prefix: str | Path) -> list[str]:
    """Individual ids (second .fam column) in file order."""
    with open(f"{prefix}.fam") as fh:
        return [line.split()[1] for line in fh if line.strip()]


def read_bim(prefix: str | Path) -> dict:
    """chrom (M,) float codes, sid (M,), cm (M,), pos (M,) base pairs, a1 / a2 alleles."""
    chrom, sid, cm, pos, a1, a2 = [], [], [], [], [], []
    with open(f"{prefix}.bim") as fh:
        for line in fh:
            f = line.split()
            if not f:
                continue
            chrom.append(_chrom_code(f[0]))
            sid.append(f[1])
            cm.append(float(f[2]))
            pos.append(float(f[3]))
            a1.append(f[4])
            a2.append(f[5])
    return {"chrom": np.asarray(chrom), "sid": sid, "cm": np.asarray(cm), "pos": np.asarray(pos), "a1": a1, "a2": a2}


@dataclass
class BedFile:
    """A memory-mapped .bed with its metadata, rows aligned to a kept strain set."""
    prefix: str
    records: np.ndarray   # (M, bytes_per_variant) uint8 view of the file past its header
    n_fam: int
    rows: np.ndarray      # (N,) int32 .fam rows of the kept strains, in .fam order
    iid: list
    sid: list
    chrom: np.ndarray
    pos: np.ndarray
    count_A1: bool = True

    @property
    def shape(self) -> tuple[int, int]:
        return len(self.rows), self.records.shape[0]


def open_bed(prefix: str | Path, keep_iid: list | None = None, *, count_A1: bool = True) -> BedFile:
    """
    Open a .bed lazily (fasterlmm/io_stream.py:44-57): metadata is read, genotypes stay on disk.  With keep_iid the
    rows are the .fam rows whose id is in keep_iid, in .fam order.
    """
    prefix = str(prefix)
    fam = read_fam(prefix)
    bim = read_bim(prefix)
    raw = np.memmap(f"{prefix}.bed", dtype=np.uint8, mode="r")
    if raw.size < 3 or bytes(raw[:3]) != BED_MAGIC:
        raise ValueError(f"{prefix}.bed is not a SNP-major PLINK 1 .bed (bad magic bytes)")
    bpv = (len(fam) + 3) // 4
    M = len(bim["sid"])
    if raw.size != 3 + M * bpv:
        raise ValueError(f"{prefix}.bed holds {raw.size - 3} record bytes, expected {M} x {bpv}")
    records = raw[3:].reshape(M, bpv)
    if keep_iid is None:
        rows = np.arange(len(fam), dtype=np.int32)
    else:
        keep = set(map(str, keep_iid))
        rows = np.array([i for i, s in enumerate(fam) if s in keep], dtype=np.int32)
    return BedFile(prefix=prefix, records=records, n_fam=len(fam), rows=rows, iid=[fam[i] for i in rows],
                   sid=bim["sid"], chrom=bim["chrom"], pos=bim["pos"], count_A1=count_A1)


def dosages_t(h: BedFile, cols, dev: torch.device | None = None) -> Tensor:
    """int8 dosages (len(cols), N) on the device, -1 for missing calls."""
    dev = dev or _cuda_device()
    cols = np.asarray(cols, dtype=np.int64)
    N = len(h.rows)
    G = torch.empty((cols.size, N), dtype=torch.int8, device=dev)
    if cols.size == 0 or N == 0:
        return G
    recs = torch.from_numpy(np.ascontiguousarray(h.records[cols])).pin_memory().to(dev, non_blocking=True)
    rows = torch.from_numpy(h.rows).to(dev)
    _lib.call("flmm_bed_decode", _ptr(recs), h.records.shape[1], int(cols.size), h.n_fam, _ptr(rows), N,
              int(bool(h.count_A1)), _ptr(G), N, _stream(dev))
    return G


def standardised_rows(h: BedFile, cols, dev: torch.device | None = None) -> Tensor:
    """Standardised variants (len(cols), N) FP64 on the device, missing calls 0 (fasterlmm/io.py:223-254)."""
    dev = dev or _cuda_device()
    G = dosages_t(h, cols, dev)
    Zt = torch.empty(G.shape, dtype=F64, device=dev)
    if G.numel():
        _lib.call("flmm_standardise_dosage", _ptr(G), G.shape[1], G.shape[1], G.shape[0], _ptr(Zt), G.shape[1],
                  _stream(dev))
    return Zt


def read_dosages(h: BedFile, cols=None) -> np.ndarray:
    """(N, len(cols)) FP64 dosages with NaN for missing calls, like the reference's read_plink (fasterlmm/io.py:54-67)."""
    cols = np.arange(h.records.shape[0]) if cols is None else np.asarray(cols)
    G = dosages_t(h, cols).cpu().numpy().T.astype(np.float64)
    G[G < 0] = np.nan
    return G


def chrom_blocks(h: BedFile, chrom_value, *, block_size: int = 8192, dev: torch.device | None = None):
    """
    Standardised test blocks of one chromosome, (Z_block (N, b), col_idx (b,)), the block source of
    fasterlmm_gb300.lowrank.loco_scan_blocks (fasterlmm/io_stream.py:113-127).
    """
    idx = np.flatnonzero(h.chrom == chrom_value)
    for b0 in range(0, idx.size, block_size):
        cols = idx[b0:b0 + block_size]
        yield standardised_rows(h, cols, dev).T, cols


__all__ = ["BedFile", "open_bed", "read_fam", "read_bim", "dosages_t", "standardised_rows", "read_dosages",
           "chrom_blocks"]
