"""
GPU drop-in for ``fasterlmm.perms.perm_threshold`` (the reference's fasterlmm/perms.py:21-68).

A batch of B real phenotypes and their B * n_perm row-shuffled copies run through one LOCO (or single-K) scan;
the per-column genome max F of the shuffled columns is the permutation null.  Row orders are numpy's PCG64 stream
seeded on [seed, column], exactly as the reference draws them, generated and argsorted on the device (or drawn with
numpy on the host for N > 16384), so the permutation index sets are bit-identical; the shuffled columns are
gathered on the device.
"""

from __future__ import annotations

from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import _lib
from .core import ScanResult, _cuda_device, _f64, _ptr, _stream, _to_device, scan_t, standardise_columns_t, \
    transpose


def perm_orders(N: int, seed_cols, n_perm: int, seed: int = 19930909, threads: int = 8) -> np.ndarray:
    """
    (B, n_perm, N) int32 row orders: for column b, ``default_rng([seed, seed_cols[b]]).random((n_perm, N))``
    argsorted along each row (fasterlmm/perms.py:51-55).  Columns are independent streams, drawn in threads.
    """
    seed_cols = [int(p) for p in seed_cols]
    out = np.empty((len(seed_cols), n_perm, N), dtype=np.int32)
    if n_perm == 0 or not seed_cols:
        return out

    def draw(rng_b):
        for b in rng_b:
            out[b] = np.random.default_rng([seed, seed_cols[b]]).random((n_perm, N)).argsort(axis=1)

    nt = max(1, min(threads, len(seed_cols)))
    with ThreadPoolExecutor(nt) as ex:
        list(ex.map(draw, [range(i, len(seed_cols), nt) for i in range(nt)]))
    return out


def perm_orders_device(N: int, seed_cols, n_perm: int, seed: int, dev: torch.device) -> torch.Tensor:
    """(B, n_perm, N) int32 orders drawn on the device, bit-identical to perm_orders (N <= 16384)."""
    seed_cols = [int(p) for p in seed_cols]
    if seed < 0 or any(p < 0 for p in seed_cols):
        raise ValueError("SeedSequence entropy must be non-negative")
    out = torch.empty((len(seed_cols), n_perm, N), dtype=torch.int32, device=dev)
    if seed_cols and n_perm:
        cols = torch.tensor(seed_cols, dtype=torch.int64, device=dev)
        _lib.call("flmm_perm_orders", _ptr(cols), len(seed_cols), int(seed), n_perm, N, _ptr(out), _stream(dev))
    return out


def pack_perm_columns(Yt_real: torch.Tensor, orders: torch.Tensor) -> torch.Tensor:
    """Yt_all (B + B n_perm, N) = [reals | b0 shuffles | b1 shuffles | ...] (fasterlmm/perms.py:56-59)."""
    B, N = Yt_real.shape
    n_perm = orders.shape[1] if orders.ndim == 3 else 0
    Ya = torch.empty((B * (1 + n_perm), N), dtype=torch.float64, device=Yt_real.device)
    _lib.call("flmm_pack_perm_columns", _ptr(Yt_real), Yt_real.stride(0), B, N, _ptr(orders if n_perm else None),
              n_perm, _ptr(Ya), N, _stream(Yt_real.device))
    return Ya


def perm_threshold(data, pheno_idx: list[int], *, n_perm: int = 100, seed: int = 19930909, loco: bool = True,
                   on_chrom=None, seed_idx: list[int] | None = None, n_grid: int = 64, log_delta_min: float = -10.0,
                   log_delta_max: float = 10.0, form: str = "plain", out: dict | None = None,
                   timers: dict | None = None) -> tuple[ScanResult, torch.Tensor]:
    """
    Drop-in for perms.perm_threshold.  ``data`` is the reference's AlignedDataset (or any object with Z, Y, X,
    chrom and optional Z_kin / chrom_kin): raw dosages (N, M) with NaN for missing calls, phenotypes (N, P),
    covariates (N, D).  Returns (ScanResult for the B real columns, perm_max_F (B, n_perm)) on the device of
    data.Z.  The extra keywords select the delta grid and the numeric form (see fasterlmm_gb300.core: "plain" is
    the default here, "fast" the default of the drop-in installer fasterlmm_gb300.shim.install); ``out``
    optionally gives preallocated result tensors (keys f, beta, se, sfve, nullh2 of shape (M, B) and max_F of shape
    (B + B n_perm,), e.g. pinned host memory) that the results are copied into and returned in; ``timers`` is passed
    to the fast engine (CUDA events around its Wald launches).
    """
    dev = _cuda_device(data.Z)
    Zt = standardise_columns_t(data.Z, dev)
    Z_kin = getattr(data, "Z_kin", None)
    chrom_kin = getattr(data, "chrom_kin", None)
    Zt_kin = standardise_columns_t(Z_kin, dev) if Z_kin is not None else None
    X = _f64(data.X, dev)
    pheno_idx = list(pheno_idx)
    B = len(pheno_idx)
    Y = _f64(data.Y, dev)
    N = Y.shape[0]
    Yt_real = transpose(Y[:, pheno_idx].contiguous()) if B else torch.empty((0, N), dtype=torch.float64, device=dev)
    seed_cols = pheno_idx if seed_idx is None else list(seed_idx)
    if N <= 16384:
        orders = perm_orders_device(N, seed_cols, n_perm, seed, dev)
    else:
        orders = torch.from_numpy(perm_orders(N, seed_cols, n_perm, seed)).to(dev)
    Yt_all = pack_perm_columns(Yt_real, orders)
    stream_out = out if (out is not None and form == "fast") else None
    res = scan_t(Zt, X, Yt_all, np.asarray(data.chrom), n_real=B, on_chrom=on_chrom if loco else None,
                 Zt_kin=Zt_kin, chrom_kin=chrom_kin, loco=loco, n_grid=n_grid, log_delta_min=log_delta_min,
                 log_delta_max=log_delta_max, form=form, timers=timers, host_out=stream_out)
    if out is not None and stream_out is None:
        res = copy_into(res, out)
    elif out is None:
        out_dev = data.Z.device if isinstance(data.Z, torch.Tensor) else dev
        res = _to_device(res, out_dev)
    perm_max_F = res.max_F[B:].reshape(B, n_perm)
    return res, perm_max_F


def copy_into(res: ScanResult, out: dict) -> ScanResult:
    """Copy device results into caller-provided tensors (pinned host copies run asynchronously, then sync)."""
    for k in ("f", "beta", "se", "sfve", "nullh2", "max_F"):
        if k in out:
            out[k].copy_(getattr(res, k), non_blocking=True)
    torch.cuda.current_stream().synchronize()
    pick = lambda k: out[k] if k in out else getattr(res, k)
    return ScanResult(f=pick("f"), beta=pick("beta"), se=pick("se"), sfve=pick("sfve"), nullh2=pick("nullh2"),
                      max_F=pick("max_F"), log_delta=res.log_delta)


__all__ = ["perm_threshold", "perm_orders", "pack_perm_columns"]
