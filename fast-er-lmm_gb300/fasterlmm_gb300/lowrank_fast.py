"""
Split-precision form of the low-rank LOCO scan (the reference's fasterlmm/lowrank.py:239-373 and the block engine
of fasterlmm/extreme_scan.py:29-80), for cohorts whose kinship is given by a factor G (N, k) of k markers.

Per LOCO chromosome c the kinship markers of c are dropped and the basis is formed as the reference does
(lowrank.py:59-96): the covariate-regressed factor's k x k Gram -- here the submatrix of one Gram of all markers,
formed once in FP64 -- is decomposed in FP64, and U_eff = G_ V / sv (on the tensor cores, split FP16); the
phenotype rotation UY = U_eff^T Y_r and the FP64 low-rank delta fit follow (lowrank.py:99-208).  Test variants then
arrive in blocks (a resident matrix, or int8 dosages streamed from pinned host memory, decoded and standardised on
the device while the previous block is scanned) and every block runs two split-FP16 tensor-core products and the
fused Wald kernel of the full-rank form:

    US = U_eff^T S_r,  UUS = S_r - U_eff US          (K = N and K = k; lowrank.py:287-289)
    sWy = [w~ o UY | c UUY] . [US | UUS]             (K = k + N; lowrank.py:296)
    sWs = interpolated [US^2 | ||UUS||^2] . [w~ | c](x)

with w~ = (shat + delta) / (s + delta), c = (shat + delta) / delta and the phenotypes' residuals UUY = Y_r - U_eff UY
formed once per chromosome (csrc/flmm_lowrank_fast.cu), and the F test on N - D - 1 degrees of freedom
(lowrank.py:270).  Real tests with F above fast.REFINE_F are recomputed without the FP32 rss cancellation
(flmm_lr_wald_refine), as in the full-rank form.
"""
from __future__ import annotations

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import F64, CovariateBasis, ScanResult, _alloc_outputs, _cuda_device, _f64, _ptr, _stream, _work, \
    kinship_from_gram, rotate_rows, transpose
from . import fast
from .fast import F16, F32, INTERP_H, SplitRows, WaldOperands, _pad, gemm_split, interp_nodes
from .lowrank import _eigh_rows

SV_FLOOR = 1e-10
BLOCK = 8192  # variants per streamed block


class _MarkerPanel:
    """The kinship factor's covariate-regressed marker rows, sample-major and split, with every chromosome's columns
    starting on a 64-column boundary (so one chromosome is one K range), and the FP64 Gram of all markers."""

    def __init__(self, Gk: Tensor, g_chrom: np.ndarray, basis: CovariateBasis, ctx):
        dev = Gk.device
        N, k_all = Gk.shape
        g_chrom = np.asarray(g_chrom)
        self.order = np.argsort(g_chrom, kind="stable")
        chroms, starts, counts = np.unique(g_chrom[self.order], return_index=True, return_counts=True)
        self.blocks = {c.item(): (int(a), int(n)) for c, a, n in zip(chroms, starts, counts)}
        offs, off = {}, 0
        for c, (a, n) in self.blocks.items():
            offs[c] = off
            off += _pad(n, 64)
        self.offs, self.k_pad, self.k_all = offs, max(off, 64), k_all
        Gt = transpose(Gk[:, torch.from_numpy(self.order).to(dev)].contiguous())  # (k_all, N) in chromosome order
        self.Grt = basis.regress_out(Gt)                                           # G_ rows, FP64
        self.gram = rotate_rows(self.Grt, self.Grt)                               # G_^T G_ (k_all, k_all), FP64
        padded = torch.zeros((self.k_pad, N), dtype=F64, device=dev)
        for c, (a, n) in self.blocks.items():
            padded[offs[c]:offs[c] + n] = self.Grt[a:a + n]
        self.split_T = SplitRows.of(transpose(padded))                            # (N, k_pad) sample-major
        self.N = N
        self.decomposed = {}  # chromosome -> (ascending evals (k_in,) FP64, eigenvector rows (k_in, k_in))

    def decompose_loco(self, chroms, ctx) -> None:
        """Eigendecompositions of the LOCO marker Grams of every chromosome in `chroms`, in one batched call of the
        library's FP32 solver with the refinement steps (FP64-accurate eigenpairs) instead of one FP64 decomposition
        per chromosome.  The Grams differ in size by the left-out chromosome, so each is padded to the largest with
        -rho I (rho above every Gram's row sums, so the padding's eigenvalues lie below the Grams' non-negative
        spectra) and its k_in largest eigenpairs are kept.  Only where the batched solver covers the size (below
        2,500) and the basis takes the Gram branch (k_in < N)."""
        todo = [c for c in chroms if c in self.blocks and c not in self.decomposed]
        sizes = {c: self.k_all - self.blocks[c][1] for c in todo}
        todo = [c for c in todo if 0 < sizes[c] < self.N]
        if len(todo) < 2:
            return
        k_max = max(sizes.values())
        if k_max >= 2500:
            return
        dev = self.gram.device
        A = torch.zeros((len(todo), k_max, k_max), dtype=F64, device=dev)
        rho = 0.0
        for b, c in enumerate(todo):
            idx = torch.from_numpy(self.kept(c)).to(dev)
            Gc = self.gram.index_select(0, idx).index_select(1, idx)
            A[b, :sizes[c], :sizes[c]] = Gc
            rho = max(rho, float(Gc.abs().sum(dim=1).max()))
        rho = 2.0 * rho + 1.0
        for b, c in enumerate(todo):
            k_in = sizes[c]
            if k_in < k_max:
                d = torch.arange(k_in, k_max, device=dev)
                A[b, d, d] = -rho
        U, evals = fast._eigh_batched_f32_refined(ctx, A)
        for b, c in enumerate(todo):
            k_in = sizes[c]
            lo = k_max - k_in  # the padding's eigenpairs come first (ascending order)
            self.decomposed[c] = (evals[b, lo:].contiguous(), U[b, lo:, :k_in].double().contiguous())

    def kept(self, c) -> np.ndarray:
        """Marker positions (in chromosome order) of the kinship without chromosome c (c = None: all)."""
        if c is None or c not in self.blocks:
            return np.arange(self.k_all)
        a, n = self.blocks[c]
        return np.concatenate([np.arange(0, a), np.arange(a + n, self.k_all)])

    def basis(self, c, ctx) -> tuple[Tensor, Tensor, Tensor]:
        """(s (k,), Ut (k, N) FP32, U_eff (N, k) FP32) of the kinship without chromosome c
        (fasterlmm/lowrank.py:75-96)."""
        dev = self.gram.device
        keep = self.kept(c)
        k_in, N = keep.size, self.N
        if k_in >= N:  # the reference's k >= N branch: the N x N kernel decomposed directly
            Gc = self.Grt[torch.from_numpy(keep).to(dev)]
            evals, U = _eigh_rows(kinship_from_gram(rotate_rows(transpose(Gc), transpose(Gc)), None, k_in))
            sel = torch.nonzero(evals.clamp(min=0.0) > (SV_FLOOR * SV_FLOOR) / k_in).flatten()
            Us = U[sel].contiguous()
            return evals[sel].clamp(min=0.0).contiguous(), Us.float(), transpose(Us).float()
        if c in self.decomposed:
            evals, V = self.decomposed.pop(c)
        else:
            idx = torch.from_numpy(keep).to(dev)
            evals, V = _eigh_rows(self.gram.index_select(0, idx).index_select(1, idx).contiguous())
        sv = evals.clamp(min=0.0).sqrt()
        sel = torch.nonzero(sv > SV_FLOOR).flatten()
        sv = sv[sel]
        Vk = V[sel] / sv[:, None]                                                 # (k, k_in) FP64
        # Ut = Vk G_^T: scatter Vk's columns to the padded marker layout (chromosome c's columns stay zero)
        A = torch.zeros((Vk.shape[0], self.k_pad), dtype=F64, device=dev)
        col = 0
        for cc, (a, n) in self.blocks.items():
            if cc == c:
                continue
            A[:, self.offs[cc]:self.offs[cc] + n] = Vk[:, col:col + n]
            col += n
        As = SplitRows.of(A)
        Ut = torch.empty((Vk.shape[0], N), dtype=F32, device=dev)
        gemm_split(ctx, As.view(), self.split_T.view(), Ut)
        Ueff = torch.empty((N, Vk.shape[0]), dtype=F32, device=dev)  # the same products, transposed
        gemm_split(ctx, self.split_T.view(), As.view(), Ueff)
        return (sv * sv / k_in).contiguous(), Ut, Ueff


def dosage_blocks(Gt_host: Tensor, rows_of: dict, dev: torch.device, block: int = BLOCK):
    """
    Block source over int8 dosages Gt_host (M, N) in pinned host memory (0/1/2, -1 missing), variant-major: for a
    chromosome c, yields (Zt (Mc, N) FP64 standardised, output rows (Mc,) int64) of its variants (rows_of[c], sorted
    and contiguous) block by block.  Each block is copied on a side stream into one of two device buffers while the
    previous block is scanned, then decoded and standardised (flmm_standardise_dosage) on the caller's stream.
    """
    N = Gt_host.shape[1]
    copy = torch.cuda.Stream(device=dev)
    bufs = [torch.empty((block, N), dtype=torch.int8, device=dev) for _ in range(2)]
    ready = [torch.cuda.Event() for _ in range(2)]
    free = [None, None]
    main = torch.cuda.current_stream(dev)

    def source(c):
        r = rows_of.get(c)
        if r is None or r.size == 0:
            return
        a, n = int(r[0]), int(r.size)
        starts = list(range(a, a + n, block))

        def issue(i):
            j0 = starts[i]
            m = min(block, a + n - j0)
            b = i % 2
            with torch.cuda.stream(copy):
                if free[b] is not None:
                    copy.wait_event(free[b])
                bufs[b][:m].copy_(Gt_host[j0:j0 + m], non_blocking=True)
                ready[b].record(copy)
            return j0, m, b

        pending = issue(0)
        for i in range(len(starts)):
            j0, m, b = pending
            if i + 1 < len(starts):
                pending = issue(i + 1)
            main.wait_event(ready[b])
            Zt = torch.empty((m, N), dtype=F64, device=dev)
            _lib.call("flmm_standardise_dosage", _ptr(bufs[b]), N, N, m, _ptr(Zt), N, _stream(dev))
            ev = torch.cuda.Event()
            ev.record(main)
            free[b] = ev
            yield Zt, torch.arange(j0, j0 + m, dtype=torch.int64, device=dev)

    return source


def loco_scan_blocks_fast(Gk: Tensor, g_chrom: np.ndarray, block_source, M: int, chroms, X: Tensor, Y: Tensor, *,
                          n_real: int | None = None, loco: bool = True, n_grid: int = 64, log_delta_min: float = -10.0,
                          log_delta_max: float = 10.0, on_chrom=None, timers: dict | None = None) -> ScanResult:
    """
    Low-rank LOCO scan (fasterlmm/extreme_scan.py:29-80) in the split-precision form.  Gk (N, k) the standardised
    kinship factor with marker chromosome labels g_chrom; block_source(c) yields (Zt (Mc, N) standardised test
    variants, output rows (Mc,) int64 device) for chromosome c (every variant when loco is False and c is None);
    outputs (M, n_real) and max_F (P,) on the device.
    """
    dev = _cuda_device(Gk)
    ctx = _lib.context(dev.index)
    st = _stream(dev)
    Gk, Xd, Yd = _f64(Gk, dev, contiguous=False), _f64(X, dev), _f64(Y, dev)
    N, D = Xd.shape
    P = Yd.shape[1]
    n_real = P if n_real is None else min(n_real, P)
    Neff = N - D

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

    slot = mark("basis")
    basis = CovariateBasis(Xd)
    Yrt = basis.regress_out(transpose(Yd))                                    # (P, N) FP64
    Yrs = SplitRows.of(Yrt)
    panel = _MarkerPanel(Gk, g_chrom, basis, ctx)
    if loco:
        panel.decompose_loco(list(chroms), ctx)
    done(slot)
    out, max_F = _alloc_outputs(M, n_real, P, dev, zero=True)
    ops = WaldOperands(dev)  # the strong-test list
    x0, R = interp_nodes(log_delta_min, log_delta_max)
    ldr = _pad(R)
    log_deltas = {}
    units = list(chroms) if loco else [None]
    for u_idx, c in enumerate(units):
        slot = mark("basis")
        s, Ut, Ueff = panel.basis(c if loco else None, ctx)
        k = s.shape[0]
        Us, Ues = SplitRows.of(Ut), SplitRows.of(Ueff)
        done(slot)
        slot = mark("rotate")
        UYt = torch.empty((P, k), dtype=F32, device=dev)
        gemm_split(ctx, Yrs.view(), Us.view(), UYt)
        UY64 = torch.zeros((P, k), dtype=F64, device=dev)
        _lib.call("flmm_accumulate_f32_f64", UY64.numel(), _ptr(UYt), _ptr(UY64), st)
        # off-rank residuals UUY = Y_r - U_eff UY and their sums of squares (fasterlmm/lowrank.py:110)
        C1 = torch.empty((P, N), dtype=F32, device=dev)
        gemm_split(ctx, SplitRows.of(UYt).view(), Ues.view(), C1)
        UUYt = torch.empty((P, N), dtype=F64, device=dev)
        yy_off = torch.empty(P, dtype=F64, device=dev)
        _lib.call("flmm_lr_residual", _ptr(Yrt), N, _ptr(C1), N, P, N, _ptr(UUYt), N, _ptr(yy_off), st)
        del C1
        done(slot)
        slot = mark("delta")
        ld = torch.empty(P, dtype=F64, device=dev)
        idx = torch.empty(P, dtype=torch.int32, device=dev)
        w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_f64_workspace_bytes", k, n_grid))
        _lib.call("flmm_fit_delta_lowrank_f64", _ptr(s), k, _ptr(UY64), k, _ptr(yy_off), int(Neff), P, n_grid,
                  float(log_delta_min), float(log_delta_max), 1, _ptr(ld), _ptr(idx), w, wb, st)
        done(slot)
        log_deltas[c if loco else 0] = ld
        # column side of the fused scan: [(w~ - c) o UY | c Y_r] split, Lagrange weights, rWr
        s32 = torch.empty(k, dtype=F32, device=dev)
        shat = torch.empty(1, dtype=F32, device=dev)
        _lib.call("flmm_convert_f64_f32", k, _ptr(s), _ptr(s32), st)
        _lib.call("flmm_mean_f32", _ptr(s), k, _ptr(shat), st)
        K1 = k + N
        lda = _pad(K1)
        A1h = torch.empty((P, lda), dtype=F16, device=dev)
        A1l = torch.empty((P, lda), dtype=F16, device=dev)
        Lh = torch.empty((P, ldr), dtype=F16, device=dev)
        Ll = torch.empty((P, ldr), dtype=F16, device=dev)
        sa1, sl, rWr, rWr0 = (torch.empty(P, dtype=F32, device=dev) for _ in range(4))
        _lib.call("flmm_lr_prep_columns", _ptr(s32), k, _ptr(UYt), k, _ptr(UUYt), N, N, _ptr(yy_off), _ptr(ld), P,
                  _ptr(shat), float(x0), INTERP_H, R, _ptr(A1h), _ptr(A1l), lda, _ptr(Lh), _ptr(Ll), ldr, _ptr(sa1),
                  _ptr(sl), _ptr(rWr), _ptr(rWr0), st)
        ldw = _pad(k + 1)
        W = torch.zeros((R, ldw), dtype=F64, device=dev)
        _lib.call("flmm_lr_interp_nodes", _ptr(s), k, _ptr(shat), float(x0), INTERP_H, R, _ptr(W), ldw, st)
        Ws = SplitRows.of(W[:, :k + 1])
        for Zt, rows in block_source(c):
            Mc = Zt.shape[0]
            if Mc == 0:
                continue
            slot = mark("rotate")
            # S_r first: U_eff can hold directions of the covariates (the reference keeps every eigenvector above
            # its floor), so US = U_eff^T S_r, not U_eff^T S (lowrank.py:287-288)
            Sr = basis.regress_out(Zt)
            del Zt
            Zs = SplitRows.of(Sr)
            USt = torch.empty((Mc, k), dtype=F32, device=dev)
            gemm_split(ctx, Zs.view(), Us.view(), USt)
            Ct = torch.empty((Mc, N), dtype=F32, device=dev)                 # U_eff US, for UUS = S_r - U_eff US
            gemm_split(ctx, SplitRows.of(USt).view(), Ues.view(), Ct)
            del Zs
            done(slot)
            slot = mark("wald")
            B1h = torch.empty((Mc, lda), dtype=F16, device=dev)
            B1l = torch.empty((Mc, lda), dtype=F16, device=dev)
            B2 = SplitRows(Mc, k + 1, dev, ld=ldw)
            sb1 = torch.empty(Mc, dtype=F32, device=dev)
            _lib.call("flmm_lr_prep_variants", _ptr(USt), k, _ptr(Sr), Sr.stride(0), _ptr(Ct), N, Mc, k, N,
                      None, N, 0,
                      _ptr(B1h), _ptr(B1l), lda, _ptr(sb1), _ptr(B2.hi), _ptr(B2.lo), ldw, _ptr(B2.scale), st)
            F = torch.empty((Mc, ldr), dtype=F32, device=dev)
            gemm_split(ctx, B2.view(), Ws.view(), F[:, :R])
            Fs = SplitRows.of(F[:, :R])
            refine = fast.REFINE_F is not None and n_real > 0
            cap = min(Mc * n_real, fast.REFINE_CAP) if refine else 0
            flags = ops._flags(cap) if refine else None
            _lib.call("flmm_wald_split_f16_df", ctx, _ptr(A1h), _ptr(A1l), lda, _ptr(sa1), _ptr(Lh), _ptr(Ll), ldr,
                      _ptr(sl), _ptr(rWr), _ptr(rWr0), P, n_real, _ptr(B1h), _ptr(B1l), lda, _ptr(sb1), _ptr(Fs.hi),
                      _ptr(Fs.lo), Fs.ld, _ptr(Fs.scale), Mc, K1, R, _ptr(rows), _ptr(out["f"]), _ptr(out["beta"]),
                      _ptr(out["se"]), _ptr(out["sfve"]), n_real, _ptr(max_F),
                      float(fast.REFINE_F if refine else float("inf")), _ptr(ops.flag_count) if refine else None,
                      _ptr(flags) if refine else None, cap, int(N - D - 1), st)
            if refine:  # strong real tests recomputed without the FP32 rss cancellation
                _lib.call("flmm_lr_wald_refine", _ptr(flags), _ptr(ops.flag_count), cap, float(fast.REFINE_F),
                          _ptr(USt), k, _ptr(UYt), k, _ptr(Sr), Sr.stride(0), _ptr(Ct), N, _ptr(UUYt), N, _ptr(s32),
                          _ptr(ld), k, N, Mc, n_real, int(N - D - 1), _ptr(rows), _ptr(out["f"]), _ptr(out["beta"]),
                          _ptr(out["se"]), _ptr(out["sfve"]), n_real, _ptr(max_F), st)
            _lib.call("flmm_fill_nullh2", _ptr(ld), n_real, _ptr(rows), Mc, _ptr(out["nullh2"]), n_real, st)
            done(slot)
        if on_chrom is not None:
            on_chrom(u_idx + 1, len(units))
    _lib.call("flmm_context_check", ctx, st)
    return ScanResult(max_F=max_F, log_delta=log_deltas, **out)


def resident_blocks(Zt: Tensor, z_chrom: np.ndarray, block: int = BLOCK):
    """Block source over a resident standardised variant-major matrix Zt (M, N) on the device."""
    z_chrom = np.asarray(z_chrom)
    dev = Zt.device

    def source(c):
        sel = np.arange(z_chrom.size) if c is None else np.flatnonzero(z_chrom == c)
        for j in range(0, sel.size, block):
            r = sel[j:j + block]
            rows = torch.from_numpy(r.astype(np.int64)).to(dev)
            yield Zt.index_select(0, rows), rows

    return source


def loco_scan_lowrank_fast(G: Tensor, g_chrom: np.ndarray, Z: Tensor, z_chrom: np.ndarray, X: Tensor, Y: Tensor, *,
                           n_real: int | None = None, on_chrom=None, **kw) -> ScanResult:
    """Split-precision form of lowrank.loco_scan_lowrank (fasterlmm/lowrank.py:320-359): G, Z column-standardised
    (N, k) and (N, M) with their chromosome labels."""
    dev = _cuda_device(G, Z)
    Zt = transpose(_f64(Z, dev, contiguous=False).contiguous())
    chroms = sorted(np.unique(np.asarray(z_chrom)).tolist())
    return loco_scan_blocks_fast(_f64(G, dev), g_chrom, resident_blocks(Zt, z_chrom), Zt.shape[0], chroms, X, Y,
                                 n_real=n_real, on_chrom=on_chrom, **kw)


def single_k_scan_lowrank_fast(G: Tensor, Z: Tensor, X: Tensor, Y: Tensor, *, n_real: int | None = None,
                               **kw) -> ScanResult:
    """Split-precision form of lowrank.single_k_scan_lowrank (fasterlmm/lowrank.py:362-373)."""
    dev = _cuda_device(G, Z)
    Zt = transpose(_f64(Z, dev, contiguous=False).contiguous())
    g_chrom = np.zeros(G.shape[1], dtype=np.int64)
    return loco_scan_blocks_fast(_f64(G, dev), g_chrom, resident_blocks(Zt, np.zeros(Zt.shape[0])), Zt.shape[0],
                                 [None], X, Y, n_real=n_real, loco=False, **kw)
