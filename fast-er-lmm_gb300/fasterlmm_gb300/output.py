"""
Output files of a scan, laid out as the reference CLI writes them (fasterlmm/cli.py:96-161, fasterlmm/bundle.py:36-117,
fasterlmm/inflation.py:32-42), so that a run of this package drops into a pipeline built around the reference's files.

Per phenotype, with per-phenotype directories: ``<outdir>/<pheno>/gwas.tsv`` (the 14 FaST-LMM single_snp columns,
rows in ascending p order with ties in variant order and NaN last), ``perms.tsv`` (the per-permutation minimum p),
``threshold.txt`` (the perm_quantile quantile of those, "%.6e") and, without a bundle, ``lambda_gc.txt`` ("%.6f").
With a bundle, the same table plus ``threshold`` and ``significant`` is appended to a directory of parquet parts
(pyarrow is needed for that route only).  ``lambda_gc.tsv`` collects (Pheno, PhenoIndex, LambdaGC, NVariants) over
the run.

The text tables are formatted by the library's host writer (flmm_write_gwas_tsv / flmm_write_column_tsv, shortest
round-trip digits in pyarrow's notation), which releases the GIL, so phenotypes are written in parallel threads.
``write_batch`` is the CLI's whole post-scan output stage for one batch of phenotypes: p-values, row orders,
permutation thresholds and the inflation factors are computed on the GPU for all phenotypes at once, then each
phenotype's files are written from host copies.  ``write_pheno`` is the per-phenotype call with the reference's
signature (``fasterlmm.cli._write_pheno``) for results already on the host.
"""

from __future__ import annotations

import os
import shutil
import threading
from concurrent.futures import ThreadPoolExecutor
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch
from torch import Tensor

from . import _lib

GWAS_COLUMNS = ["sid_index", "SNP", "Chr", "GenDist", "ChrPos", "PValue", "SnpWeight", "SnpWeightSE", "EffectSize",
                "SnpFractVarExpl", "Mixing", "Nullh2", "Pheno", "PhenoCount"]
BUNDLE_COLUMNS = GWAS_COLUMNS + ["threshold", "significant"]
BUNDLE_FILENAME = "gwas_bundle.parquet"
LAMBDA_FILENAME = "lambda_gc.tsv"
LAMBDA_COLUMNS = ["Pheno", "PhenoIndex", "LambdaGC", "NVariants"]


def _addr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class VariantTable:
    """
    The columns that are the same for every phenotype of a run (the CLI's writer context, fasterlmm/cli.py:248-252):
    variant ids packed as one byte string with offsets, chromosome codes and base-pair positions as FP64, the
    genotype variances that scale EffectSize, and PhenoCount = 1 + n_perm.
    """
    snp_bytes: np.ndarray    # (total,) uint8
    snp_offsets: np.ndarray  # (M + 1,) int64
    chrom: np.ndarray        # (M,) float64
    pos: np.ndarray          # (M,) float64
    g_var: np.ndarray        # (M,) float64
    pheno_count: int
    snp_ids: list | None = None
    _snp_arrow: object = None  # the ids as a pyarrow array, built on the first bundle append

    @classmethod
    def of(cls, snp_ids, chrom, pos, g_var, n_perm: int) -> "VariantTable":
        ids = [str(s) for s in snp_ids]
        enc = [s.encode() for s in ids]
        offsets = np.zeros(len(enc) + 1, dtype=np.int64)
        np.cumsum([len(e) for e in enc], out=offsets[1:])
        buf = np.frombuffer(b"".join(enc) or b"\0", dtype=np.uint8).copy()
        f64 = lambda a: np.ascontiguousarray(np.asarray(a, dtype=np.float64))
        t = cls(snp_bytes=buf, snp_offsets=offsets, chrom=f64(chrom), pos=f64(pos), g_var=f64(g_var),
                pheno_count=1 + int(n_perm), snp_ids=ids)
        if not (t.chrom.shape == t.pos.shape == t.g_var.shape == (len(ids),)):
            raise ValueError("snp ids, chrom, pos and g_var must all have one entry per variant")
        return t

    @property
    def M(self) -> int:
        return self.chrom.shape[0]

    def with_g_var(self, g_var) -> "VariantTable":
        """The same table with another genotype variance vector (a subset of samples, fasterlmm/cli.py:372)."""
        g = np.ascontiguousarray(np.asarray(g_var, dtype=np.float64))
        if g.shape != self.g_var.shape:
            raise ValueError("g_var must have one entry per variant")
        return VariantTable(self.snp_bytes, self.snp_offsets, self.chrom, self.pos, g, self.pheno_count, self.snp_ids)


def format_f64(values) -> list[str]:
    """Text of each value as the output tables write it (shortest round trip, pyarrow's notation)."""
    v = np.ascontiguousarray(np.asarray(values, dtype=np.float64).ravel())
    buf = np.empty(max(1, 40 * v.size), dtype=np.uint8)
    off = np.empty(v.size + 1, dtype=np.int64)
    _lib.call("flmm_format_f64", _addr(v), v.size, _addr(buf), buf.size, _addr(off))
    raw = buf.tobytes()
    return [raw[off[i]:off[i + 1]].decode() for i in range(v.size)]


def write_gwas_tsv(path, table: VariantTable, pheno_name: str, p_col, beta_col, se_col, sfve_col, nullh2_col,
                   p_var: float, order=None) -> None:
    """One phenotype's gwas.tsv from host columns (M,) (or strided views of (M, B) tables); order defaults to the
    ascending-p order."""
    cols = [np.asarray(c, dtype=np.float64) for c in (p_col, beta_col, se_col, sfve_col, nullh2_col)]
    M = table.M
    # a common stride over the five columns: contiguous copies unless they are already equal-strided views
    strides = {c.strides[0] if c.ndim == 1 else None for c in cols}
    if len(strides) != 1 or None in strides or any(c.shape != (M,) for c in cols) or next(iter(strides)) % 8:
        cols = [np.ascontiguousarray(c.reshape(M)) for c in cols]
    ld = cols[0].strides[0] // 8 if M else 1
    if order is None:
        order = np.argsort(cols[0], kind="stable")
    order = np.asarray(order, dtype=np.int64)
    ld_order = order.strides[0] // 8 if order.size else 1
    _lib.call("flmm_write_gwas_tsv", str(path).encode(), M, _addr(table.snp_bytes), _addr(table.snp_offsets),
              _addr(table.chrom), _addr(table.pos), _addr(table.g_var), float(p_var), _addr(cols[0]),
              _addr(cols[1]), _addr(cols[2]), _addr(cols[3]), _addr(cols[4]), ld, _addr(order), ld_order,
              str(pheno_name).encode(), table.pheno_count)


def write_column_tsv(path, header: str, values) -> None:
    v = np.ascontiguousarray(np.asarray(values, dtype=np.float64).ravel())
    _lib.call("flmm_write_column_tsv", str(path).encode(), header.encode(), _addr(v), v.size)


def lambda_gc_host(p) -> tuple[float, int]:
    """Genomic inflation factor of host p-values (fasterlmm/inflation.py:19-29): median of chi2.isf(p, 1) over the
    non-NaN p, divided by chi2.ppf(0.5, 1); (nan, 0) when every p is NaN."""
    from scipy.stats import chi2
    p = np.asarray(p, dtype=np.float64)
    p = p[~np.isnan(p)]
    if p.size == 0:
        return float("nan"), 0
    return float(np.median(chi2.isf(p, 1)) / chi2.ppf(0.5, 1)), int(p.size)


class BundleWriter:
    """
    Streaming parquet bundle (fasterlmm/bundle.py:36-117): a directory of parquet parts, one per writing thread,
    staged in ``<path>.tmp`` and renamed into place by close(), so an interrupted run leaves no half-built bundle.
    Each appended phenotype is one row group.  Needs pyarrow.
    """

    def __init__(self, path) -> None:
        import pyarrow.parquet as pq  # noqa: F401  (fail at construction when pyarrow is absent)
        self._dir = Path(path)
        self._tmp = self._dir.with_name(self._dir.name + ".tmp")
        if self._tmp.is_dir():
            shutil.rmtree(self._tmp)
        elif self._tmp.exists():
            self._tmp.unlink()
        self._tmp.mkdir(parents=True)
        self._local = threading.local()
        self._lock = threading.Lock()
        self._writers: list = []
        self._next = 0

    def append(self, table) -> None:
        import pyarrow.parquet as pq
        w = getattr(self._local, "writer", None)
        if w is None:
            with self._lock:
                w = pq.ParquetWriter(self._tmp / f"gwas-results-part-{self._next:05d}.parquet", table.schema,
                                     compression="snappy")
                self._next += 1
                self._writers.append(w)
            self._local.writer = w
        w.write_table(table)

    def close(self) -> Path:
        for w in self._writers:
            w.close()
        self._writers = []
        if self._dir.is_dir():
            shutil.rmtree(self._dir)
        elif self._dir.exists():
            self._dir.unlink()
        self._tmp.replace(self._dir)
        return self._dir


def _bundle_table(table: VariantTable, pheno_name, p, beta, se, sfve, nullh2, p_var, thresh, order):
    """The bundle's 16-column table of one phenotype, rows in `order` (fasterlmm/cli.py:135-147)."""
    import pyarrow as pa
    o = np.asarray(order, dtype=np.int64)
    pc = np.asarray(p, dtype=np.float64)[o]
    b = np.asarray(beta, dtype=np.float64)[o]
    M = table.M
    if table._snp_arrow is None:
        table._snp_arrow = pa.array(table.snp_ids, type=pa.string())
    pheno = pa.DictionaryArray.from_arrays(pa.array(np.zeros(M, dtype=np.int32)), [str(pheno_name)])
    return pa.table({
        "sid_index": o, "SNP": table._snp_arrow.take(pa.array(o)),
        "Chr": table.chrom[o], "GenDist": pa.nulls(M, pa.float64()), "ChrPos": table.pos[o], "PValue": pc,
        "SnpWeight": b, "SnpWeightSE": np.asarray(se, dtype=np.float64)[o],
        "EffectSize": b * b * table.g_var[o] / p_var, "SnpFractVarExpl": np.asarray(sfve, dtype=np.float64)[o],
        "Mixing": np.zeros(M), "Nullh2": np.asarray(nullh2, dtype=np.float64)[o],
        "Pheno": pheno.cast(pa.string()), "PhenoCount": np.full(M, table.pheno_count, dtype=np.int64),
        "threshold": np.full(M, thresh), "significant": pc < thresh})


def write_pheno(ctx: VariantTable, outdir_str: str, pheno_name: str, p_col, beta_col, se_col, sfve_col, nullh2_col,
                p_var: float, perm_min_p, perm_quantile: float, per_pheno_dirs: bool, bundle_writer=None, *,
                lambda_rows: list | None = None, order=None, thresh: float | None = None,
                lam: tuple[float, int] | None = None) -> None:
    """
    One phenotype's output (fasterlmm/cli.py:114-158), same arguments as the reference's writer with the
    identical-across-phenotypes columns in ``ctx`` (a VariantTable).  ``lambda_rows`` receives (pheno, lambda, n).
    ``order``, ``thresh`` and ``lam`` may be passed in when the device has computed them (write_batch); otherwise
    they are computed here from the host columns as the reference does.
    """
    if thresh is None:
        thresh = float(np.quantile(np.asarray(perm_min_p, dtype=np.float64), perm_quantile))
    if lam is None:
        lam = lambda_gc_host(p_col)
    if lambda_rows is not None:
        lambda_rows.append((pheno_name, lam[0], lam[1]))
    if order is None:
        order = np.argsort(np.asarray(p_col, dtype=np.float64), kind="stable")
    if per_pheno_dirs:
        sub = Path(outdir_str) / str(pheno_name)
        sub.mkdir(parents=True, exist_ok=True)
        write_gwas_tsv(sub / "gwas.tsv", ctx, pheno_name, p_col, beta_col, se_col, sfve_col, nullh2_col, p_var,
                       order)
        write_column_tsv(sub / "perms.tsv", "perm_min_p", perm_min_p)
        (sub / "threshold.txt").write_text(f"{thresh:.6e}\n")
        if bundle_writer is None:
            (sub / "lambda_gc.txt").write_text(f"{lam[0]:.6f}\n")
    if bundle_writer is not None:
        bundle_writer.append(_bundle_table(ctx, pheno_name, p_col, beta_col, se_col, sfve_col, nullh2_col, p_var,
                                           thresh, order))


def write_lambda_table(outdir, shard_i: int | None, rows: list, name_to_idx: dict) -> Path:
    """
    lambda_gc.tsv (lambda_gc.shard{i}.tsv for a shard) in phenotype column order (fasterlmm/inflation.py:32-42):
    header Pheno, PhenoIndex, LambdaGC, NVariants; LambdaGC as "%.6f", NaN as an empty field.
    """
    outdir = Path(outdir)
    path = outdir / (LAMBDA_FILENAME if shard_i is None else f"lambda_gc.shard{shard_i}.tsv")
    lines = ["\t".join(LAMBDA_COLUMNS)]
    for name, idx, lam, n in sorted(((n, name_to_idx[n], lam, nv) for n, lam, nv in rows), key=lambda r: r[1]):
        lam_s = "" if lam != lam else f"{lam:.6f}"
        lines.append(f"{name}\t{idx}\t{lam_s}\t{n}")
    path.write_text("\n".join(lines) + "\n")
    return path


def device_post(res, perm_max_F: Tensor, df2: int, perm_quantile: float = 0.05) -> dict:
    """
    Per-batch post-scan quantities on the device (fasterlmm/cli.py:128-129, :405-406): p (M, B) = P(F(1, df2) > F),
    the ascending-p row order per phenotype (M, B), perm_min_p (B, n_perm), the threshold (B,) and the inflation
    factor with its variant count (B,).  All FP64 / int64 device tensors.
    """
    from .post import lambda_gc, perm_threshold_p, pvalue
    F = res.f
    p = pvalue(F, df2)
    key = torch.where(torch.isnan(p), torch.full_like(p, float("inf")), p)
    order = torch.sort(key, dim=0, stable=True).indices
    pmin = pvalue(perm_max_F, df2)
    thresh = perm_threshold_p(perm_max_F, df2, perm_quantile)
    lam, n = lambda_gc(F, df2)
    return {"p": p, "order": order, "perm_min_p": pmin, "thresh": thresh, "lambda": lam, "n_var": n}


def write_batch(outdir, pheno_names: list, res, perm_max_F: Tensor, df2: int, ctx: VariantTable, p_var, *,
                perm_quantile: float = 0.05, per_pheno_dirs: bool = True, bundle_writer=None,
                lambda_rows: list | None = None, threads: int | None = None) -> None:
    """
    The CLI's output stage for one scanned batch (fasterlmm/cli.py:405-426): device post-scan step for every
    phenotype, one copy of each table to the host, then one write_pheno per phenotype on a thread pool.
    ``res`` is the batch's ScanResult (f, beta, se, sfve, nullh2 of shape (M, B)), ``perm_max_F`` (B, n_perm),
    ``p_var`` (B,) the phenotype variances (ddof 0) that scale EffectSize.
    """
    post = device_post(res, perm_max_F, df2, perm_quantile)
    host = {k: v.cpu().numpy() for k, v in post.items()}
    det = {k: getattr(res, k).double().cpu().numpy() for k in ("beta", "se", "sfve", "nullh2")}
    p_var = np.asarray(p_var.cpu().numpy() if isinstance(p_var, Tensor) else p_var, dtype=np.float64)
    B = len(pheno_names)
    rows = lambda_rows if lambda_rows is not None else []

    def one(j: int) -> None:
        write_pheno(ctx, str(outdir), pheno_names[j], host["p"][:, j], det["beta"][:, j], det["se"][:, j],
                    det["sfve"][:, j], det["nullh2"][:, j], float(p_var[j]), host["perm_min_p"][j], perm_quantile,
                    per_pheno_dirs, bundle_writer, lambda_rows=rows, order=host["order"][:, j],
                    thresh=float(host["thresh"][j]), lam=(float(host["lambda"][j]), int(host["n_var"][j])))

    with ThreadPoolExecutor(max_workers=threads or min(16, os.cpu_count() or 1)) as ex:
        list(ex.map(one, range(B)))


__all__ = ["GWAS_COLUMNS", "BUNDLE_COLUMNS", "VariantTable", "format_f64", "write_gwas_tsv", "write_column_tsv",
           "write_pheno", "write_lambda_table", "BundleWriter", "device_post", "write_batch", "lambda_gc_host"]
