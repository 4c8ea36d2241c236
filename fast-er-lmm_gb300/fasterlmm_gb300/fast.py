"""
Split-precision ("fast") form of the LOCO scan engine.

Same algorithm and outputs as the plain form (fasterlmm_gb300.core.scan_t), with the O(N^2 M), O(N Neff P) and
O(Neff P M) products on the tensor cores:

* the kinship Gram of each chromosome, the rotations UY = U_eff^T Y_r and US = U_eff^T S_r, and the Wald sums
  sWy / sWs are split-FP16 tcgen05 products (three MMAs per product, FP32 accumulation, ~21-bit operands);
* the delta fit is an FP32 grid plus a Newton solve of d loss / d log delta = 0 in the reference's bracket;
* the kinship eigendecomposition, the covariate SVD and the projection of K + I stay FP64.

Device layouts: tested variants are grouped by chromosome (a stable reorder, undone by the output row map), so every
chromosome is one contiguous row block of the split variant matrix; the kinship panel is also kept sample-major
with each chromosome's columns starting on a 64-column boundary, so the Gram of a chromosome is one K range.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import F64, CovariateBasis, ScanResult, _alloc_outputs, _ptr, _stream, _work, compat_spectrum, \
    eigh_batched, project_kinship

F16 = torch.float16
F32 = torch.float32

# Precision of the per-chromosome eigendecompositions.
#   "f32r" (default): one FP32 cusolverDnXsyevBatched call for all LOCO kinships, then EIGH_REFINE_STEPS refinement
#          steps of the eigenvectors against the FP64 kinships (flmm_eigh_refine_f32) with FP64 Rayleigh-quotient
#          eigenvalues.  At N = 1,000 the kinship spectrum is a tight bulk (gaps ~1e-4 of its width), where one step
#          leaves beta ~1e-4 off the FP64 result on a fifth of the tests; two steps match the FP64 decomposition's
#          outputs (beta and SE within 1e-5 of the FP64 oracle), a third changes nothing.
#   "f32": the FP32 call alone.  F, beta, SE, SFVE and -log10 p stay inside the parity tolerance, but on phenotypes
#          with a flat likelihood (h2 near 0) the decomposition's ~1e-7 error moves the fitted delta, and with it
#          nullh2 = 1 / (1 + delta), by more than 1e-5 relative; the refinement step removes that.
#   "f64": the FP64 batched call (EIGH_MODE: 1 = cusolverDnXsyevBatched, 2 = syevd side by side on worker streams).
EIGH_PRECISION = "f32r"
EIGH_MODE = 1
# Refinement steps of "f32r": None picks by size -- 2 up to N = 1,024, 3 above (the FP32 decomposition's error grows
# with N: at N = 1,294 two steps left beta of a few hundred tests of a missingness group outside 1e-5 of the
# reference's FP64 result and at N = 5,000 ~1 % of them; three steps match it in both).
EIGH_REFINE_STEPS = None


def refine_steps(N: int) -> int:
    if EIGH_REFINE_STEPS is not None:
        return max(1, int(EIGH_REFINE_STEPS))
    return 2 if N <= 1024 else 3
# Where the exact delta refinement starts: "grid" (the FP32 grid argmin's bracket) or "learned" (the MLP proposal of
# fasterlmm_gb300.learned, bracketed inside the grid argmin's basin; same answers, fewer evaluations per column).
DELTA_PROPOSAL = "grid"
# Run each chromosome's column side (UY rotation, delta fit) on a side stream one chromosome ahead of the Wald scan.
PIPELINE = True
# Real tests whose FP32 F exceeds this are recomputed without the cancelling rss = rWr - sWy^2 / sWs subtraction
# (flmm_wald_refine_f32): the FP32 form's -log10 p error grows like F^2 / df, about 1e-5 at F = 30 and N = 1,000.
# None turns the re-evaluation off.  REFINE_CAP bounds the list of such tests per chromosome (8 bytes each); a
# chromosome with more is recomputed by scanning its stored F.
REFINE_F = 30.0
REFINE_CAP = 1 << 22


def _pad(k: int, m: int = 8) -> int:
    return (k + m - 1) // m * m


class SplitRows:
    """hi / lo FP16 pair of a row-major matrix with one power-of-two scale per row: x ~= (hi + lo) * scale."""

    def __init__(self, rows: int, K: int, dev: torch.device, ld: int | None = None):
        self.rows, self.K = rows, K
        self.ld = ld or _pad(K)
        self.hi = torch.empty((rows, self.ld), dtype=F16, device=dev)
        self.lo = torch.empty((rows, self.ld), dtype=F16, device=dev)
        self.scale = torch.empty(rows, dtype=F32, device=dev)

    @classmethod
    def of(cls, X: Tensor) -> "SplitRows":
        rows, K = X.shape
        out = cls(rows, K, X.device)
        if rows:
            _lib.call("flmm_split_rows_f16", _ptr(X), int(X.dtype == F64), X.stride(0), rows, K, _ptr(out.hi),
                      _ptr(out.lo), out.ld, _ptr(out.scale), _stream(X.device))
        return out

    def view(self, r0: int = 0, rows: int | None = None, k0: int = 0, K: int | None = None) -> "SplitView":
        """A row range and K range of the pair, as raw pointers for the C ABI (keeps the buffers alive)."""
        rows = self.rows - r0 if rows is None else rows
        K = self.K - k0 if K is None else K
        return SplitView(self, (_ptr(self.hi[r0:, k0:]), _ptr(self.lo[r0:, k0:]), _ptr(self.scale[r0:]), self.ld,
                                rows, K))


class SplitView(tuple):
    """(hi, lo, scale, ld, rows, K) pointers of a SplitRows range; holds the owning SplitRows so that the device
    buffers outlive every launch that reads them."""

    def __new__(cls, owner: SplitRows, fields: tuple):
        obj = super().__new__(cls, fields)
        obj.owner = owner
        return obj


def gemm_split(ctx, A: SplitView, B: SplitView, C: Tensor, accumulate: bool = False) -> None:
    """C (Mr, Nr) FP32 = A B^T for split views A, B (from SplitRows.view) with equal K."""
    ah, al, sa, lda, Mr, K = A
    bh, bl, sb, ldb, Nr, Kb = B
    assert K == Kb
    _lib.call("flmm_gemm_split_f16", ctx, ah, al, sa, lda, Mr, bh, bl, sb, ldb, Nr, K, _ptr(C), C.stride(0),
              int(accumulate), _stream(C.device))


def fit_delta_fast(s: Tensor, UYt: Tensor, *, n_grid: int = 64, log_delta_min: float = -10.0,
                   log_delta_max: float = 10.0, refine: bool = True) -> tuple[Tensor, Tensor]:
    dev = s.device
    Neff = s.shape[0]
    P = UYt.shape[0]
    ld = torch.empty(P, dtype=F64, device=dev)
    idx = torch.empty(P, dtype=torch.int32, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_fast_workspace_bytes", Neff, n_grid))
    _lib.call("flmm_fit_delta_fast", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), P, n_grid, float(log_delta_min),
              float(log_delta_max), int(bool(refine)), _ptr(ld), _ptr(idx), w, wb, _stream(dev))
    return ld, idx


def _fit_delta(s: Tensor, UYt: Tensor, **kw) -> tuple[Tensor, Tensor]:
    if DELTA_PROPOSAL == "learned":
        from .learned import fit_delta_learned
        return fit_delta_learned(s, UYt, **kw)
    return fit_delta_fast(s, UYt, **kw)


def _chrom_order(chrom: np.ndarray) -> tuple[np.ndarray | None, list]:
    """Stable grouping by chromosome: (order or None if already grouped, [(c, start, count)] in sorted c)."""
    chrom = np.asarray(chrom)
    order = np.argsort(chrom, kind="stable")
    grouped = chrom[order]
    cs, starts, counts = np.unique(grouped, return_index=True, return_counts=True)
    blocks = [(c.item(), int(a), int(n)) for c, a, n in zip(cs, starts, counts)]
    return (None if np.array_equal(order, np.arange(chrom.size)) else order), blocks


class KinshipPanel:
    """Sample-major split of a standardised panel with 64-aligned chromosome column blocks, and its Grams."""

    def __init__(self, Zt: Tensor, chrom: np.ndarray, ctx):
        dev = Zt.device
        M, N = Zt.shape
        order, blocks = _chrom_order(chrom)
        offs, off = [], 0
        for _, _, n in blocks:
            offs.append(off)
            off += _pad(n, 64)
        Mpad = max(off, 64)
        Zg = torch.zeros((N, Mpad), dtype=F64, device=dev)
        st = _stream(dev)
        src = Zt if order is None else Zt.index_select(0, torch.from_numpy(order).to(dev))
        for (c, a, n), o in zip(blocks, offs):
            if n:
                _lib.call("flmm_transpose_f64", _ptr(src[a:a + n]), N, n, N, _ptr(Zg[:, o:]), Mpad, st)
        del src
        self.split = SplitRows.of(Zg)
        del Zg
        self.M = M
        self.counts = {c: n for (c, _, n) in blocks}
        self.grams: dict = {}
        self.Gtot = torch.zeros((N, N), dtype=F64, device=dev)
        for (c, a, n), o in zip(blocks, offs):
            G = torch.empty((N, N), dtype=F32, device=dev)
            v = self.split.view(0, N, o, n)
            gemm_split(ctx, v, v, G)
            self.grams[c] = G
            _lib.call("flmm_accumulate_f32_f64", N * N, _ptr(G), _ptr(self.Gtot), st)

    def kinship(self, c) -> Tensor:
        """LOCO kinship without chromosome c (c = None: all chromosomes)."""
        N = self.Gtot.shape[0]
        K = torch.empty((N, N), dtype=F64, device=self.Gtot.device)
        Gc = self.grams.get(c) if c is not None else None
        m = self.M - (self.counts.get(c, 0) if c is not None else 0)
        _lib.call("flmm_loco_kinship_f32", _ptr(self.Gtot), _ptr(Gc), N, float(m), _ptr(K), _stream(K.device))
        return K


# sWs interpolation nodes in log delta: spacing and points of the local Lagrange rule (see csrc/flmm_fast.cu)
INTERP_H = 0.25
INTERP_Q = 10


def interp_nodes(lo: float, hi: float) -> tuple[float, int]:
    """(x0, R): R nodes x0 + r h covering [lo, hi] with the margins the 10-point stencil needs at both ends."""
    x0 = lo - (INTERP_Q // 2) * INTERP_H
    R = int(np.ceil((hi - lo) / INTERP_H - 1e-9)) + INTERP_Q + 1
    return x0, R


class WaldOperands:
    """Split operand buffers of the fused Wald kernel, reused across chromosomes (grow-only)."""

    def __init__(self, dev: torch.device):
        self.dev = dev
        self.cols = None
        self.vars = None
        self.flags = None
        self.flag_count = torch.zeros(1, dtype=torch.int32, device=dev)

    def _flags(self, n: int) -> Tensor:
        if self.flags is None or self.flags.shape[0] < n:
            self.flags = torch.empty((max(n, 1), 2), dtype=torch.int32, device=self.dev)
        return self.flags

    def _cols(self, P: int, ldk: int, ldr: int):
        c = self.cols
        if c is None or c[0].shape[0] < P or c[0].shape[1] != ldk or c[2].shape[1] != ldr:
            self.cols = [torch.empty((P, ldk), dtype=F16, device=self.dev) for _ in range(2)] + \
                        [torch.empty((P, ldr), dtype=F16, device=self.dev) for _ in range(2)] + \
                        [torch.empty(P, dtype=F32, device=self.dev) for _ in range(4)]
        return self.cols

    def _vars(self, Mc: int, ldk: int):
        if self.vars is None or self.vars[0].shape[0] < Mc or self.vars[0].shape[1] != ldk:
            self.vars = [torch.empty((Mc, ldk), dtype=F16, device=self.dev) for _ in range(4)] + \
                        [torch.empty(Mc, dtype=F32, device=self.dev) for _ in range(2)]
        return self.vars


def wald_fast(ctx, ops: WaldOperands, s: Tensor, UYt: Tensor, ld: Tensor, USt: Tensor, n_real: int, rows: Tensor,
              out: dict, max_F: Tensor, log_delta_min: float = -10.0, log_delta_max: float = 10.0, mark=None,
              done=None) -> None:
    """
    Fused split-precision Wald of one chromosome (fasterlmm/core.py:601-671).  sWs is interpolated from R nodes in
    log delta covering [log_delta_min, log_delta_max], which must contain every log delta in ``ld``.
    """
    dev = s.device
    st = _stream(dev)
    Neff = s.shape[0]
    P = UYt.shape[0]
    Mc = USt.shape[0]
    ldk = _pad(Neff)
    x0, R = interp_nodes(log_delta_min, log_delta_max)
    ldr = _pad(R)
    s32 = torch.empty(Neff, dtype=F32, device=dev)
    shat = torch.empty(1, dtype=F32, device=dev)
    _lib.call("flmm_convert_f64_f32", Neff, _ptr(s), _ptr(s32), st)
    _lib.call("flmm_mean_f32", _ptr(s), Neff, _ptr(shat), st)
    A1h, A1l, Lh, Ll, sa1, sl, rWr, rWr0 = ops._cols(P, ldk, ldr)
    _lib.call("flmm_wald_split_prep_columns", _ptr(s32), Neff, _ptr(UYt), UYt.stride(0), _ptr(ld), P, _ptr(shat),
              float(x0), INTERP_H, R, _ptr(A1h), _ptr(A1l), ldk, _ptr(Lh), _ptr(Ll), ldr, _ptr(sa1), _ptr(sl),
              _ptr(rWr), _ptr(rWr0), st)
    B1h, B1l, B2h, B2l, sb1, sb2 = ops._vars(Mc, ldk)
    _lib.call("flmm_wald_split_prep_variants", _ptr(USt), USt.stride(0), Mc, Neff, _ptr(B1h), _ptr(B1l), _ptr(B2h),
              _ptr(B2l), ldk, _ptr(sb1), _ptr(sb2), st)
    # node values of sWs~: F (Mc, R) = (US o US) W~^T
    W = torch.empty((R, Neff), dtype=F64, device=dev)
    _lib.call("flmm_wald_interp_nodes", _ptr(s), Neff, _ptr(shat), float(x0), INTERP_H, R, _ptr(W), st)
    Ws = SplitRows.of(W)
    F = torch.empty((Mc, ldr), dtype=F32, device=dev)
    us2 = SplitView(ops, (_ptr(B2h), _ptr(B2l), _ptr(sb2), ldk, Mc, Neff))
    gemm_split(ctx, us2, Ws.view(), F[:, :R])
    Fs = SplitRows.of(F[:, :R])
    refine = REFINE_F is not None and n_real > 0 and Mc > 0
    cap = min(Mc * n_real, REFINE_CAP) if refine else 0
    flags = ops._flags(cap) if refine else None
    slot = mark("wald") if mark else None
    _lib.call("flmm_wald_split_f16", ctx, _ptr(A1h), _ptr(A1l), ldk, _ptr(sa1), _ptr(Lh), _ptr(Ll), ldr, _ptr(sl),
              _ptr(rWr), _ptr(rWr0), P, n_real, _ptr(B1h), _ptr(B1l), ldk, _ptr(sb1), _ptr(Fs.hi), _ptr(Fs.lo), Fs.ld,
              _ptr(Fs.scale), Mc, Neff, R, _ptr(rows), _ptr(out["f"]), _ptr(out["beta"]), _ptr(out["se"]),
              _ptr(out["sfve"]), n_real, _ptr(max_F), float(REFINE_F if refine else float("inf")),
              _ptr(ops.flag_count) if refine else None, _ptr(flags) if refine else None, cap, st)
    if done:
        done(slot)
    if refine:
        slot = mark("refine") if mark else None
        _lib.call("flmm_wald_refine_f32", ctx, _ptr(flags), _ptr(ops.flag_count), cap, float(REFINE_F), _ptr(USt),
                  USt.stride(0), _ptr(UYt), UYt.stride(0), _ptr(s32), _ptr(ld), Neff, Mc, n_real, _ptr(rows),
                  _ptr(out["f"]), _ptr(out["beta"]), _ptr(out["se"]), _ptr(out["sfve"]), n_real, _ptr(max_F), st)
        if done:
            done(slot)
    if "nullh2" in out:  # (the streamed path fills nullh2 rows in host memory instead)
        _lib.call("flmm_fill_nullh2", _ptr(ld), n_real, _ptr(rows), Mc, _ptr(out["nullh2"]), n_real, st)


def scan_t(Zt: Tensor, X: Tensor, Yt: Tensor, chrom: np.ndarray, *, n_real: int, on_chrom=None,
           Zt_kin: Tensor | None = None, chrom_kin: np.ndarray | None = None, loco: bool = True, n_grid: int = 64,
           log_delta_min: float = -10.0, log_delta_max: float = 10.0, refine: bool = True,
           timers: dict | None = None, host_out: dict | None = None) -> ScanResult:
    """
    Fast-form engine on device tensors (same contract as fasterlmm_gb300.core.scan_t).  ``timers``, if given, maps
    a stage name to a list that receives (start, end) CUDA event pairs recorded around that stage.  ``host_out``, if
    given, holds result tensors (keys of ScanResult, e.g. pinned host memory) that are filled while the scan runs:
    each chromosome's result rows are copied on a side stream as soon as its Wald scan is done, so the copies overlap
    the next chromosome's work; the returned ScanResult then holds those tensors.
    """
    dev = Zt.device
    ctx = _lib.context(dev.index)
    st = _stream(dev)
    M, N = Zt.shape
    P = Yt.shape[0]

    def mark(name):
        if timers is None:
            return None
        ev = torch.cuda.Event(enable_timing=True)
        ev.record()
        timers.setdefault(name, []).append([ev, None])
        return timers[name][-1]

    def done(slot):
        if slot is not None:
            ev = torch.cuda.Event(enable_timing=True)
            ev.record()
            slot[1] = ev

    out, max_F = _alloc_outputs(M, n_real, P, dev)
    basis = CovariateBasis(X)
    Ys = SplitRows.of(basis.regress_out(Yt))
    order, blocks = _chrom_order(chrom)
    host_nullh2 = host_out is not None and loco and _RowSink.host_fill_possible(host_out, order, blocks)
    if host_nullh2:
        del out["nullh2"]  # filled in host memory, chromosome by chromosome
        nullh2_row = torch.zeros(1, dtype=torch.int64, device=dev)
    sink = _RowSink(out, host_out, dev, host_nullh2) if host_out is not None else None
    order_t = None if order is None else torch.from_numpy(order).to(dev)
    Zs = SplitRows.of(Zt if order_t is None else Zt.index_select(0, order_t))
    row_map = torch.arange(M, dtype=torch.int64, device=dev) if order_t is None else order_t.to(torch.int64)

    kin = KinshipPanel(Zt if Zt_kin is None else Zt_kin, np.asarray(chrom if Zt_kin is None else chrom_kin), ctx)
    units = [(c, a, n) for (c, a, n) in blocks] if loco else [(None, 0, M)]
    ops = WaldOperands(dev)
    log_deltas = {}
    D = X.shape[1]
    if N <= D:
        raise ValueError(f"need more samples than covariate columns (N={N}, D={D})")
    Neff = N - D
    ldk = _pad(Neff)
    # all projected LOCO kinships first, so their FP64 eigendecompositions run side by side
    slot = mark("eigh")
    Kp = torch.empty((len(units), N, N), dtype=F64, device=dev)
    for k_idx, (c, _, _) in enumerate(units):
        project_kinship(kin.kinship(c), basis, Kp[k_idx])
    if EIGH_PRECISION == "f32r":
        Kp, evals = _eigh_batched_f32_refined(ctx, Kp)
    elif EIGH_PRECISION == "f32":
        Kp, evals = _eigh_batched_f32(ctx, Kp)
    else:
        evals = eigh_batched(Kp, mode=EIGH_MODE)
    done(slot)
    # Column side of chromosome k (its spectrum, eigenvector split, UY rotation and delta fit) runs on a side stream
    # one chromosome ahead of the variant side (US rotation, Wald operand prep, fused Wald) on the main stream, so
    # the delta fit's FP32 work shares the SMs with the tensor-core Wald kernel of the previous chromosome.  Two UY
    # buffers alternate; the side stream reuses one only after the main stream's Wald prep has read it.
    main = torch.cuda.current_stream(dev)
    side = torch.cuda.Stream(device=dev) if PIPELINE else main
    UY_bufs = [torch.empty((P, ldk), dtype=F32, device=dev) for _ in range(2 if PIPELINE else 1)]
    buf_free = [None] * len(UY_bufs)
    # made on the main stream and read on the side stream: their memory is not reused before the side stream's work
    # is done, also when an error ends the scan early
    if side is not main:
        for t in (*UY_bufs, Kp, evals, Ys.hi, Ys.lo, Ys.scale):
            t.record_stream(side)
    start = torch.cuda.Event()
    start.record(main)
    side.wait_event(start)

    def column_side(k_idx: int):
        with torch.cuda.stream(side):
            s_k = _spectrum(evals[k_idx], D)
            Us = SplitRows.of(Kp[k_idx, D:])
            b = k_idx % len(UY_bufs)
            if buf_free[b] is not None:
                side.wait_event(buf_free[b])
            UYt = UY_bufs[b][:, :Neff]
            slot = mark("rotate")
            gemm_split(ctx, Ys.view(), Us.view(), UYt)
            done(slot)
            slot = mark("delta")
            ld_k, _ = _fit_delta(s_k, UYt, n_grid=n_grid, log_delta_min=log_delta_min,
                                 log_delta_max=log_delta_max, refine=refine)
            done(slot)
            ready = torch.cuda.Event()
            ready.record(side)
        return s_k, Us, b, ld_k, ready

    ahead = column_side(0) if units else None
    for k_idx, (c, a, n) in enumerate(units):
        s, Us, b, ld, ready = ahead
        if k_idx + 1 < len(units):
            ahead = column_side(k_idx + 1)
        main.wait_event(ready)
        if side is not main:  # made on the side stream, used on the main stream
            for t in (s, ld, Us.hi, Us.lo, Us.scale):
                t.record_stream(main)
        USt = torch.empty((n, ldk), dtype=F32, device=dev)
        gemm_split(ctx, Zs.view(a, n), Us.view(), USt[:, :Neff])
        wald_fast(ctx, ops, s, UY_bufs[b][:, :Neff], ld, USt[:, :Neff], n_real, row_map[a:a + n], out, max_F,
                  log_delta_min=log_delta_min, log_delta_max=log_delta_max, mark=mark, done=done)
        buf_free[b] = torch.cuda.Event()
        buf_free[b].record(main)
        log_deltas[c if c is not None else 0] = ld
        if sink is not None:
            sink.push(order, a, n)
            if host_nullh2 and n:
                vh, vd = sink.mapped_vec(n_real)
                _lib.call("flmm_fill_nullh2", _ptr(ld), n_real, _ptr(nullh2_row), 1, vd, n_real, st)
                sink.push_nullh2(vh, n_real, order, a, n)
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(units))
    _lib.call("flmm_context_check", ctx, st)
    if sink is not None:
        return sink.finish(max_F, log_deltas)
    return ScanResult(max_F=max_F, log_delta=log_deltas, **out)


def _eigh_batched_f32(ctx, Kp: Tensor) -> tuple[Tensor, Tensor]:
    """FP32 eigendecomposition of a (batch, N, N) FP64 stack: (eigenvector rows (batch, N, N) FP32, evals FP32)."""
    dev = Kp.device
    batch, N, _ = Kp.shape
    st = _stream(dev)
    A = torch.empty((batch, N, N), dtype=F32, device=dev)
    _lib.call("flmm_convert_f64_f32", A.numel(), _ptr(Kp), _ptr(A), st)
    evals = torch.empty((batch, N), dtype=F32, device=dev)
    nbytes = _lib.query_bytes("flmm_eigh_batched_f32_workspace_bytes", ctx, N, batch)
    w, wb = _work.get(dev, nbytes)
    _lib.call("flmm_eigh_batched_f32", ctx, _ptr(A), N, batch, _ptr(evals), w, wb, st)
    return A, evals


def _eigh_batched_f32_refined(ctx, Kp: Tensor) -> tuple[Tensor, Tensor]:
    """FP32 eigendecomposition plus refine_steps(N) refinement steps: (eigenvector rows FP32, ascending FP64 evals,
    the Rayleigh quotients of the last step's input vectors)."""
    dev = Kp.device
    batch, N, _ = Kp.shape
    U, _ = _eigh_batched_f32(ctx, Kp)
    U_ref = torch.empty_like(U)
    evals = torch.empty((batch, N), dtype=F64, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_eigh_refine_workspace_bytes", N, batch))
    for _ in range(refine_steps(N)):
        _lib.call("flmm_eigh_refine_f32", _ptr(Kp), _ptr(U), _ptr(U_ref), _ptr(evals), N, batch, w, wb,
                  _stream(dev))
        U, U_ref = U_ref, U
    return U, evals


def _spectrum(evals: Tensor, D: int) -> Tensor:
    if evals.dtype == F64:
        return compat_spectrum(evals, D)
    N = evals.shape[0]
    s = torch.empty(N - D, dtype=F64, device=evals.device)
    _lib.call("flmm_compat_spectrum_f32", _ptr(evals), N, D, _ptr(s), _stream(evals.device))
    return s


# mapped host buffers for the streamed nullh2 vectors, by size, kept for the process (host_alloc is slow)
_MAPPED_FREE: dict = {}


class _RowSink:
    """
    Copies finished result rows into caller tensors on a side stream.  A chromosome whose rows are contiguous in
    the caller's variant order is copied as soon as its scan is queued; other rows (unsorted chromosome labels)
    and max_F are copied at the end.

    nullh2 repeats one value per (chromosome, phenotype) over the chromosome's rows.  When every chromosome's rows
    are contiguous and the caller's nullh2 lives in host memory, only each chromosome's (n_real,) vector crosses the
    link and host threads fill its rows (flmm_fill_rows_host_f64) while the GPU runs on: a fifth of the result bytes
    never leave the device.
    """

    KEYS = ("f", "beta", "se", "sfve", "nullh2")
    # Row fills and result copies both write host memory.  Per step of the 1,000 x 100,000 x 71,324 scan (e2e, median
    # of 4): fills deferred until the copies drained 197 ms, fills beside the copies on 2 x 8 threads 227 ms (the
    # copies slowed from 5.4 to ~8 ms per chromosome), on one worker of 2 threads 173 ms (the copies keep most of
    # the bandwidth and the fills finish with them).
    FILL_THREADS = 2
    FILL_WORKERS = 1

    def __init__(self, out: dict, host_out: dict, dev: torch.device, host_nullh2: bool = False):
        self.out, self.host, self.dev = out, host_out, dev
        self.stream = torch.cuda.Stream(device=dev)
        # mapped host buffers of the (n_real,) nullh2 vectors, written by the kernel that forms them: a copy would
        # queue on the copy engine behind the earlier chromosomes' result copies
        self.mapped = []
        self.pending = []  # row ranges not copied early
        self.host_nullh2 = host_nullh2
        self.fills = []
        self.pool = None
        if host_nullh2:
            from concurrent.futures import ThreadPoolExecutor
            self.pool = ThreadPoolExecutor(max_workers=self.FILL_WORKERS)

    @staticmethod
    def host_fill_possible(host_out: dict | None, order, blocks) -> bool:
        h = (host_out or {}).get("nullh2")
        if h is None or h.is_cuda or not h.is_contiguous() or h.dtype != F64:
            return False
        return order is None or all(np.array_equal(order[a:a + n], np.arange(order[a], order[a] + n))
                                    for _, a, n in blocks if n)

    def mapped_vec(self, n_real: int) -> tuple[int, int]:
        """A mapped host buffer of n_real doubles: (host address, device address)."""
        nbytes = 8 * max(n_real, 1)
        free = _MAPPED_FREE.setdefault(nbytes, [])
        if free:
            hp, dp = free.pop()
        else:
            h, d = C.c_void_p(), C.c_void_p()
            _lib.call("flmm_host_alloc_mapped", nbytes, C.byref(h), C.byref(d))
            hp, dp = h.value, d.value
        self.mapped.append((nbytes, hp, dp))
        return hp, dp

    def push_nullh2(self, vec_host: int, n_real: int, order, a: int, n: int) -> None:
        """Fill one chromosome's n rows of the host nullh2 table from its vector, which the kernel just queued on the
        current stream writes into the mapped buffer at vec_host."""
        if n == 0:
            return
        r0 = a if order is None else int(order[a])
        done = torch.cuda.Event()
        done.record(torch.cuda.current_stream(self.dev))
        dst = self.host["nullh2"]
        ld = dst.stride(0)

        def fill():
            done.synchronize()
            _lib.call("flmm_fill_rows_host_f64", dst.data_ptr() + 8 * r0 * ld, ld, n, vec_host, n_real,
                      self.FILL_THREADS)

        self.fills.append((self.pool.submit(fill), None, None))

    def push(self, order, a: int, n: int) -> None:
        if n == 0:
            return
        r0 = a if order is None else int(order[a])
        if order is not None and not np.array_equal(order[a:a + n], np.arange(r0, r0 + n)):
            self.pending.append(None)
            return
        ev = torch.cuda.Event()
        ev.record(torch.cuda.current_stream(self.dev))
        self.stream.wait_event(ev)
        with torch.cuda.stream(self.stream):
            for k in self.KEYS:
                if k in self.host and k in self.out:
                    self.host[k][r0:r0 + n].copy_(self.out[k][r0:r0 + n], non_blocking=True)

    def finish(self, max_F: Tensor, log_deltas: dict) -> ScanResult:
        main = torch.cuda.current_stream(self.dev)
        if self.pending:  # at least one chromosome was not contiguous: copy everything once more at the end
            for k in self.KEYS:
                if k in self.host and k in self.out:
                    self.host[k].copy_(self.out[k], non_blocking=True)
        if "max_F" in self.host:
            self.host["max_F"].copy_(max_F, non_blocking=True)
        main.synchronize()
        self.stream.synchronize()
        for f, _, _ in self.fills:
            f.result()
        if self.pool is not None:
            self.pool.shutdown(wait=True)
        for nbytes, hp, dp in self.mapped:
            _MAPPED_FREE.setdefault(nbytes, []).append((hp, dp))
        self.mapped = []
        pick = lambda k, t: self.host[k] if k in self.host else t
        res = {k: pick(k, v) for k, v in self.out.items()}
        if self.host_nullh2:
            res["nullh2"] = self.host["nullh2"]
        return ScanResult(max_F=pick("max_F", max_F), log_delta=log_deltas, **res)
