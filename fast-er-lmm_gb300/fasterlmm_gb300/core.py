"""
GPU drop-in for the fastlmm-compat scan path of ``fasterlmm.core`` (the reference's fasterlmm/core.py:454-740).

Same function names, signatures, dataclasses, argument meaning and error behaviour as the reference; the work is
done by the CUDA library (include/fasterlmm_gb300.h) on one GB300.  Tensors may live on any device: they are moved
to the current CUDA device, and results come back on the device of the main input (Z, or K for the rotation),
FP64 like the reference.  There is no CPU fallback: without a CUDA device or the built library every call raises.

Two numeric forms run the same algorithm:

* ``form="plain"``: FP64 end to end, with the reference's operation order and its 50-step golden-section search.
* ``form="fast"``: split-precision tensor-core rotation and Wald kernels with FP32 accumulation, an FP32 grid
  followed by a safeguarded Newton refinement of log delta whose sums are compensated FP32 (log delta itself is
  carried in FP64; see fasterlmm_gb300.fast).

Called directly, every driver defaults to ``form="plain"``, the reference's own arithmetic.  The drop-in
installer (fasterlmm_gb300.shim.install) binds ``form="fast"`` unless told otherwise, since the fast form is
the one held to the scan's stated tolerances (beta/SE rtol 1e-5, |d(-log10 p)| <= 1e-3) at full speed.

Beyond the reference's keywords, the LOCO / single-K drivers accept the delta-grid options of
fit_delta_grid_compat (n_grid, log_delta_min, log_delta_max, refine), which the reference's loop leaves at their
defaults (fasterlmm/core.py:715), and ``form``.  The per-chromosome log delta of the last scan is kept on the
returned ScanResult as ``log_delta`` (a dict chromosome -> (P,) tensor), which the reference computes but drops.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np
import torch
from torch import Tensor

from . import _lib

F64 = torch.float64


# ---- result types (fasterlmm/core.py:34-48, 466-484) ---------------------------------------------------------

@dataclass
class ScanResult:
    """Per-(variant, real column) Wald outputs (M, n_real) and the per-column genome max F (P,)."""
    f: Tensor
    beta: Tensor
    se: Tensor
    sfve: Tensor
    nullh2: Tensor
    max_F: Tensor
    log_delta: dict = field(default_factory=dict, repr=False)


@dataclass
class CompatSpectrum:
    """
    Projected eigendecomposition (fasterlmm/core.py:466-484).  s (Neff,), U_eff (N, Neff), X (N, D), Xpinv (D, N),
    UY (Neff, P).  U_eff and UY are transposed views of ``Ut`` (Neff, N) and ``UYt`` (P, Neff), the layouts the
    kernels read.
    """
    s: Tensor
    U_eff: Tensor
    X: Tensor
    Xpinv: Tensor
    UY: Tensor
    Ut: Tensor = field(default=None, repr=False)
    UYt: Tensor = field(default=None, repr=False)


# ---- plumbing ------------------------------------------------------------------------------------------------

def _ptr(t: Tensor | None) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


def _stream(dev: torch.device) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)


def _cuda_device(*tensors) -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("fasterlmm_gb300 needs a CUDA device (GB300, sm_103a); there is no CPU fallback")
    for t in tensors:
        if isinstance(t, Tensor) and t.is_cuda:
            return t.device
    return torch.device("cuda", torch.cuda.current_device())


def _f64(t, dev: torch.device, contiguous: bool = True) -> Tensor:
    if isinstance(t, np.ndarray):
        t = torch.from_numpy(np.ascontiguousarray(t))
    t = t.to(device=dev, dtype=F64)
    return t.contiguous() if contiguous else t


class _Work:
    """Per-device grow-only scratch buffer handed to the library's `work` arguments."""

    def __init__(self):
        self.buf: dict[torch.device, Tensor] = {}

    def get(self, dev: torch.device, nbytes: int) -> tuple[C.c_void_p, int]:
        b = self.buf.get(dev)
        if b is None or b.numel() < nbytes:
            b = torch.empty(max(nbytes, 1 << 20), dtype=torch.uint8, device=dev)
            self.buf[dev] = b
        b.record_stream(torch.cuda.current_stream(dev))  # freed only after every stream that used it is done
        return C.c_void_p(b.data_ptr()), b.numel()


_work = _Work()


def transpose(A: Tensor) -> Tensor:
    """(rows, cols) FP64 CUDA tensor -> contiguous (cols, rows) by the library's transpose kernel."""
    A = A.contiguous()
    rows, cols = A.shape
    out = torch.empty((cols, rows), dtype=F64, device=A.device)
    _lib.call("flmm_transpose_f64", _ptr(A), cols, rows, cols, _ptr(out), rows, _stream(A.device))
    return out


def _rows_major(Z: Tensor) -> Tensor:
    """(N, M) matrix -> (M, N) contiguous variant-major copy (free when Z is already a transposed view)."""
    if Z.T.is_contiguous():
        return Z.T
    return transpose(Z)


# ---- standardisation and kinship (fasterlmm/io.py:223-265) ------------------------------------------------------

def standardise_columns_t(Z, dev: torch.device | None = None) -> Tensor:
    """Unit-standardise (N, M) dosages with NaN for missing calls; returns the variant-major (M, N) tensor."""
    dev = dev or _cuda_device(Z)
    Zd = _f64(Z, dev)
    N, M = Zd.shape
    Zt = torch.empty((M, N), dtype=F64, device=dev)
    _lib.call("flmm_standardise_f64", _ptr(Zd), M, N, M, _ptr(Zt), N, _stream(dev))
    return Zt


def standardise_columns(arr):
    """Drop-in for io.standardise_columns (fasterlmm/io.py:223-254): same shape and type back.  Computed in FP64; a
    floating-point tensor comes back in its own dtype, as the reference's torch branch returns it (io.py:235-246),
    and an array as FP64, as its numpy branch does."""
    src_dev = arr.device if isinstance(arr, Tensor) else None
    Zt = standardise_columns_t(arr)
    out = Zt.T
    if isinstance(arr, np.ndarray):
        return out.cpu().numpy()
    if arr.is_floating_point() and arr.dtype != F64:
        out = out.to(arr.dtype)
    return out if src_dev is None or src_dev.type == "cuda" else out.to(src_dev)


def gram_t(Zt: Tensor, out: Tensor | None = None, accumulate: bool = False) -> Tensor:
    """G (N, N) = Zt^T Zt in FP64 for a variant-major block Zt (M, N)."""
    M, N = Zt.shape
    if out is None:
        out = torch.empty((N, N), dtype=F64, device=Zt.device)
    if M == 0 and not accumulate:
        out.zero_()
        return out
    _lib.call("flmm_gram_f64", _ptr(Zt), Zt.stride(0), M, N, 1.0 if accumulate else 0.0, _ptr(out), N,
              _stream(Zt.device))
    return out


def kinship_from_gram(Gtot: Tensor, Gc: Tensor | None, m_loco: int) -> Tensor:
    N = Gtot.shape[0]
    K = torch.empty_like(Gtot)
    _lib.call("flmm_loco_kinship", _ptr(Gtot), _ptr(Gc), N, N, float(m_loco), _ptr(K), _stream(Gtot.device))
    return K


def grm(Z: Tensor) -> Tensor:
    """Drop-in for io.grm (fasterlmm/io.py:257-265): K = Z Z^T / M for a standardised (N, M) Z."""
    dev = _cuda_device(Z)
    Zt = _rows_major(_f64(Z, dev, contiguous=False))
    G = gram_t(Zt)
    K = kinship_from_gram(G, None, Zt.shape[0])
    return K if not isinstance(Z, Tensor) or Z.is_cuda else K.to(Z.device)


# ---- compat rotation (fasterlmm/core.py:487-519) ----------------------------------------------------------------

class CovariateBasis:
    """Device thin SVD of X: Qx (D, N) orthonormal rows spanning range(X) (zero past the rank), Xpinv (D, N)."""

    def __init__(self, X: Tensor):
        dev = X.device
        self.X = X
        N, D = X.shape
        if N < D:
            raise ValueError(f"need at least as many samples as covariate columns (N={N}, D={D})")
        ctx = _lib.context(dev.index)
        nbytes = _lib.query_bytes("flmm_covariate_basis_workspace_bytes", ctx, N, D)
        self.Qx = torch.empty((D, N), dtype=F64, device=dev)
        self.Xpinv = torch.empty((D, N), dtype=F64, device=dev)
        self.rank = torch.zeros(1, dtype=torch.int32, device=dev)
        w, wb = _work.get(dev, nbytes)
        _lib.call("flmm_covariate_basis", ctx, _ptr(X), N, D, _ptr(self.Qx), _ptr(self.Xpinv), _ptr(self.rank), w,
                  wb, _stream(dev))

    def regress_out(self, At: Tensor) -> Tensor:
        """Row-wise OLS regress-out R = A - X Xpinv A for A given as rows (rows, N)."""
        rows, N = At.shape
        R = torch.empty_like(At)
        if rows:
            _lib.call("flmm_regress_out", _ptr(At), At.stride(0), rows, N, _ptr(self.X), self.X.shape[1],
                      _ptr(self.Xpinv), _ptr(R), N, _stream(At.device))
        return R


def project_kinship(K: Tensor, basis: CovariateBasis, out: Tensor) -> Tensor:
    """out (N, N) = (I - PX)(K + I)(I - PX) (fasterlmm/core.py:499-506)."""
    dev = K.device
    N = K.shape[0]
    D = basis.X.shape[1]
    w, wb = _work.get(dev, _lib.query_bytes("flmm_project_kinship_workspace_bytes", N, D))
    _lib.call("flmm_project_kinship", _ptr(K), K.stride(0), _ptr(basis.Qx), N, D, _ptr(out), N, w, wb, _stream(dev))
    return out


def eigh_batched(A: Tensor, mode: int = 1, slot: int = -1, evals: Tensor | None = None,
                 work: Tensor | None = None) -> Tensor:
    """
    In-place FP64 eigendecomposition of a (batch, N, N) stack on the current stream: eigenvector rows overwrite A;
    returns evals (batch, N).  ``slot`` >= 0 uses a worker cuSOLVER handle and ``work`` a private workspace, for
    batches that run on another stream next to work that uses the shared scratch buffer.
    """
    dev = A.device
    batch, N, _ = A.shape
    ctx = _lib.context(dev.index)
    if evals is None:
        evals = torch.empty((batch, N), dtype=F64, device=dev)
    nbytes = _lib.query_bytes("flmm_eigh_batched_workspace_bytes", ctx, N, batch, mode)
    if work is None:
        w, wb = _work.get(dev, nbytes)
    else:
        assert work.numel() >= nbytes
        w, wb = C.c_void_p(work.data_ptr()), work.numel()
    _lib.call("flmm_eigh_batched", ctx, _ptr(A), N, batch, _ptr(evals), mode, slot, w, wb, _stream(dev))
    return evals


def compat_spectrum(evals: Tensor, D: int) -> Tensor:
    N = evals.shape[0]
    s = torch.empty(N - D, dtype=F64, device=evals.device)
    _lib.call("flmm_compat_spectrum", _ptr(evals), N, D, _ptr(s), _stream(evals.device))
    return s


def compat_eigh(K: Tensor, basis: CovariateBasis) -> tuple[Tensor, Tensor]:
    """Projected kinship eigendecomposition: s (Neff,) and Ut (Neff, N) (fasterlmm/core.py:498-515)."""
    dev = K.device
    N = K.shape[0]
    D = basis.X.shape[1]
    if N <= D:
        raise ValueError(f"need more samples than covariate columns (N={N}, D={D})")
    ctx = _lib.context(dev.index)
    st = _stream(dev)
    Kp = torch.empty((N, N), dtype=F64, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_project_kinship_workspace_bytes", N, D))
    _lib.call("flmm_project_kinship", _ptr(K), K.stride(0), _ptr(basis.Qx), N, D, _ptr(Kp), N, w, wb, st)
    evals = torch.empty(N, dtype=F64, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_eigh_workspace_bytes", ctx, N))
    _lib.call("flmm_eigh", ctx, _ptr(Kp), N, _ptr(evals), w, wb, st)
    s = torch.empty(N - D, dtype=F64, device=dev)
    _lib.call("flmm_compat_spectrum", _ptr(evals), N, D, _ptr(s), st)
    return s, Kp[D:]


def rotate_rows(At: Tensor, Ut: Tensor) -> Tensor:
    """(rows, N) x (Neff, N)^T -> (rows, Neff) in FP64."""
    rows, N = At.shape
    Neff = Ut.shape[0]
    out = torch.empty((rows, Neff), dtype=F64, device=At.device)
    if rows:
        _lib.call("flmm_gemm_nt_f64", _ptr(At), At.stride(0), _ptr(Ut), Ut.stride(0), _ptr(out), Neff, rows, Neff, N,
                  1.0, _stream(At.device))
    return out


def fastlmm_compat_rotate(K: Tensor, X: Tensor, Y: Tensor) -> CompatSpectrum:
    """Drop-in for core.fastlmm_compat_rotate (fasterlmm/core.py:487-519)."""
    dev = _cuda_device(K)
    Kd, Xd, Yd = _f64(K, dev), _f64(X, dev), _f64(Y, dev)
    basis = CovariateBasis(Xd)
    s, Ut = compat_eigh(Kd, basis)
    UYt = rotate_rows(basis.regress_out(transpose(Yd)), Ut)
    out_dev = K.device if isinstance(K, Tensor) else dev
    mv = (lambda t: t) if out_dev.type == "cuda" else (lambda t: t.to(out_dev))
    return CompatSpectrum(s=mv(s), U_eff=mv(Ut.T), X=mv(Xd), Xpinv=mv(basis.Xpinv[: Xd.shape[1]]), UY=mv(UYt.T),
                          Ut=Ut, UYt=UYt)


# ---- delta fit (fasterlmm/core.py:561-595) ---------------------------------------------------------------------

def fit_delta_t(s: Tensor, UYt: Tensor, *, n_grid: int = 64, log_delta_min: float = -10.0,
                log_delta_max: float = 10.0, refine: bool = True) -> tuple[Tensor, Tensor]:
    """FP64 grid + golden-section fit on device tensors; returns (log_delta (P,), grid index (P,))."""
    dev = s.device
    Neff = s.shape[0]
    P = UYt.shape[0]
    ld = torch.empty(P, dtype=F64, device=dev)
    idx = torch.empty(P, dtype=torch.int32, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_f64_workspace_bytes", Neff, n_grid))
    _lib.call("flmm_fit_delta_f64", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), P, n_grid, float(log_delta_min),
              float(log_delta_max), int(bool(refine)), _ptr(ld), _ptr(idx), w, wb, _stream(dev))
    return ld, idx


def fit_delta_grid_compat(spec: CompatSpectrum, *, n_grid: int = 64, log_delta_min: float = -10.0,
                          log_delta_max: float = 10.0, refine: bool = True) -> Tensor:
    """Drop-in for core.fit_delta_grid_compat (fasterlmm/core.py:561-595)."""
    dev = _cuda_device(spec.s)
    s = _f64(spec.s, dev)
    UYt = spec.UYt if spec.UYt is not None else transpose(_f64(spec.UY, dev))
    ld, _ = fit_delta_t(s, UYt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                        refine=refine)
    return ld if spec.s.is_cuda else ld.to(spec.s.device)


# ---- Wald scan (fasterlmm/core.py:601-671) ---------------------------------------------------------------------

def wald_t(s: Tensor, UYt: Tensor, log_delta: Tensor, USt: Tensor, n_real: int, rows: Tensor, out: dict,
           max_F: Tensor) -> None:
    """FP64 fused Wald of one variant block into preallocated (M, n_real) outputs at `rows`; raises max_F."""
    dev = s.device
    Neff = s.shape[0]
    P = UYt.shape[0]
    Mc = USt.shape[0]
    w, wb = _work.get(dev, _lib.query_bytes("flmm_wald_f64_workspace_bytes", P, Neff))
    _lib.call("flmm_wald_f64", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), _ptr(log_delta), P, n_real, _ptr(USt),
              USt.stride(0), Mc, _ptr(rows), _ptr(out["f"]), _ptr(out["beta"]), _ptr(out["se"]), _ptr(out["sfve"]),
              n_real, _ptr(max_F), w, wb, _stream(dev))
    _lib.call("flmm_fill_nullh2", _ptr(log_delta), n_real, _ptr(rows), Mc, _ptr(out["nullh2"]), n_real, _stream(dev))


def _alloc_outputs(M: int, n_real: int, P: int, dev: torch.device, zero: bool = False) -> tuple[dict, Tensor]:
    """(M, n_real) detail outputs and max_F (P,) = -inf.  The scans write every detail element, so the detail is left
    uninitialised unless ``zero`` (callers whose variant blocks may not cover all M rows)."""
    alloc = torch.zeros if zero else torch.empty
    out = {k: alloc((M, n_real), dtype=F64, device=dev) for k in ("f", "beta", "se", "sfve", "nullh2")}
    max_F = torch.empty(P, dtype=F64, device=dev)
    _lib.call("flmm_fill_f64", _ptr(max_F), P, float("-inf"), _stream(dev))
    return out, max_F


def snp_wald_scan_compat(spec: CompatSpectrum, log_delta: Tensor, S: Tensor, *, snp_chunk: int = 4096,
                         pheno_chunk: int = 256, n_real: int | None = None) -> ScanResult:
    """
    Drop-in for core.snp_wald_scan_compat (fasterlmm/core.py:601-671).  snp_chunk / pheno_chunk are accepted for
    signature compatibility; the fused kernel tiles both axes itself and the result does not depend on tiling.
    """
    dev = _cuda_device(spec.s, S)
    s = _f64(spec.s, dev)
    UYt = spec.UYt if spec.UYt is not None else transpose(_f64(spec.UY, dev))
    Ut = spec.Ut if spec.Ut is not None else transpose(_f64(spec.U_eff, dev))
    basis = _BasisView(_f64(spec.X, dev), _f64(spec.Xpinv, dev))
    P = UYt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    St = _rows_major(_f64(S, dev, contiguous=False))
    M = St.shape[0]
    USt = rotate_rows(basis.regress_out(St), Ut)
    out, max_F = _alloc_outputs(M, n_real, P, dev)
    rows = torch.arange(M, dtype=torch.int64, device=dev)
    ld = _f64(log_delta, dev)
    wald_t(s, UYt, ld, USt, n_real, rows, out, max_F)
    res = ScanResult(max_F=max_F, **out)
    return _to_device(res, S.device if isinstance(S, Tensor) else dev)


class _BasisView(CovariateBasis):
    """A CovariateBasis around an existing (X, Xpinv) pair."""

    def __init__(self, X: Tensor, Xpinv: Tensor):
        self.X, self.Xpinv = X, Xpinv


def _to_device(res: ScanResult, dev: torch.device) -> ScanResult:
    if dev.type == "cuda":
        return res
    return ScanResult(f=res.f.to(dev), beta=res.beta.to(dev), se=res.se.to(dev), sfve=res.sfve.to(dev),
                      nullh2=res.nullh2.to(dev), max_F=res.max_F.to(dev),
                      log_delta={k: v.to(dev) for k, v in res.log_delta.items()})


# ---- LOCO / single-K drivers (fasterlmm/core.py:677-740) --------------------------------------------------------

def _chrom_blocks(chrom: np.ndarray, dev: torch.device) -> dict:
    """chromosome -> (row index tensor on device, contiguous slice or None), chromosomes in sorted order."""
    chrom = np.asarray(chrom)
    blocks = {}
    for c in sorted(np.unique(chrom).tolist()):
        idx = np.flatnonzero(chrom == c)
        sl = slice(int(idx[0]), int(idx[-1]) + 1) if idx[-1] - idx[0] + 1 == idx.size else None
        blocks[c] = (torch.from_numpy(idx).to(dev), sl)
    return blocks


def _take_rows(Zt: Tensor, blk) -> Tensor:
    idx, sl = blk
    return Zt[sl] if sl is not None else Zt.index_select(0, idx)


def scan_t(Zt: Tensor, X: Tensor, Yt: Tensor, chrom: np.ndarray, *, n_real: int, on_chrom=None,
           Zt_kin: Tensor | None = None, chrom_kin: np.ndarray | None = None, loco: bool = True, n_grid: int = 64,
           log_delta_min: float = -10.0, log_delta_max: float = 10.0, refine: bool = True,
           form: str = "plain", timers: dict | None = None, host_out: dict | None = None) -> ScanResult:
    """
    Core engine on device tensors: Zt (M, N) standardised tested variants, X (N, D), Yt (P, N) columns, chromosome
    labels (M,).  The kinship Gram of every chromosome is computed once and each LOCO kinship is the total minus
    the chromosome's own block; the covariate basis and the OLS regress-out of the phenotypes are computed once.
    ``host_out`` (fast form only) streams the results into caller tensors while the scan runs (fast.scan_t).
    """
    if form == "fast":
        from . import fast
        return fast.scan_t(Zt, X, Yt, chrom, n_real=n_real, on_chrom=on_chrom, Zt_kin=Zt_kin, chrom_kin=chrom_kin,
                           loco=loco, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                           refine=refine, timers=timers, host_out=host_out)
    if host_out is not None:
        raise ValueError("host_out is only supported by the fast form")
    if form != "plain":
        raise ValueError(f"unknown form {form!r} (expected 'plain' or 'fast')")
    dev = Zt.device
    M, N = Zt.shape
    P = Yt.shape[0]
    out, max_F = _alloc_outputs(M, n_real, P, dev)
    basis = CovariateBasis(X)
    Yrt = basis.regress_out(Yt)
    kin_Zt = Zt if Zt_kin is None else Zt_kin
    kin_chrom = np.asarray(chrom if Zt_kin is None else chrom_kin)
    test_blocks = _chrom_blocks(chrom, dev)
    log_deltas = {}
    if loco:
        kin_blocks = _chrom_blocks(kin_chrom, dev)
        grams = {c: gram_t(_take_rows(kin_Zt, b)) for c, b in kin_blocks.items()}
        Gtot = torch.zeros((N, N), dtype=F64, device=dev)
        for G in grams.values():
            _lib.call("flmm_axpy_f64", N * N, 1.0, _ptr(G), _ptr(Gtot), _stream(dev))
        units = [(c, test_blocks[c]) for c in test_blocks]
    else:
        Gtot = gram_t(kin_Zt)
        units = [(None, (torch.arange(M, device=dev), slice(0, M)))]
    M_kin = kin_Zt.shape[0]
    for k_idx, (c, blk) in enumerate(units):
        if c is None:
            K = kinship_from_gram(Gtot, None, M_kin)
        else:
            Gc = grams.get(c)
            m_c = int((kin_chrom == c).sum())
            K = kinship_from_gram(Gtot, Gc, M_kin - m_c)
        s, Ut = compat_eigh(K, basis)
        UYt = rotate_rows(Yrt, Ut)
        ld, _ = fit_delta_t(s, UYt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                            refine=refine)
        USt = rotate_rows(basis.regress_out(_take_rows(Zt, blk)), Ut)
        wald_t(s, UYt, ld, USt, n_real, blk[0], out, max_F)
        log_deltas[c if c is not None else 0] = ld
        if on_chrom is not None:
            on_chrom(k_idx + 1, len(units))
    return ScanResult(max_F=max_F, log_delta=log_deltas, **out)


def loco_scan_compat(Z: Tensor, X: Tensor, Y: Tensor, chrom: np.ndarray, *, n_real: int | None = None,
                     on_chrom=None, Z_kin: Tensor | None = None, chrom_kin: np.ndarray | None = None,
                     n_grid: int = 64, log_delta_min: float = -10.0, log_delta_max: float = 10.0,
                     refine: bool = True, form: str = "plain") -> ScanResult:
    """Drop-in for core.loco_scan_compat (fasterlmm/core.py:677-726); Z (and Z_kin) pre-standardised (N, M)."""
    if (Z_kin is None) != (chrom_kin is None):
        raise ValueError("Z_kin and chrom_kin go together")
    dev = _cuda_device(Z)
    Zt = _rows_major(_f64(Z, dev, contiguous=False))
    Zt_kin = None if Z_kin is None else _rows_major(_f64(Z_kin, dev, contiguous=False))
    Yt = transpose(_f64(Y, dev, contiguous=False))
    P = Yt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    res = scan_t(Zt, _f64(X, dev), Yt, np.asarray(chrom), n_real=n_real, on_chrom=on_chrom, Zt_kin=Zt_kin,
                 chrom_kin=chrom_kin, loco=True, n_grid=n_grid, log_delta_min=log_delta_min,
                 log_delta_max=log_delta_max, refine=refine, form=form)
    return _to_device(res, Z.device if isinstance(Z, Tensor) else dev)


def single_k_scan_compat(Z: Tensor, X: Tensor, Y: Tensor, *, n_real: int | None = None,
                         Z_kin: Tensor | None = None, n_grid: int = 64, log_delta_min: float = -10.0,
                         log_delta_max: float = 10.0, refine: bool = True, form: str = "plain") -> ScanResult:
    """Drop-in for core.single_k_scan_compat (fasterlmm/core.py:729-740)."""
    dev = _cuda_device(Z)
    Zt = _rows_major(_f64(Z, dev, contiguous=False))
    Zt_kin = None if Z_kin is None else _rows_major(_f64(Z_kin, dev, contiguous=False))
    Yt = transpose(_f64(Y, dev, contiguous=False))
    P = Yt.shape[0]
    n_real = P if n_real is None else min(n_real, P)
    M = Zt.shape[0]
    res = scan_t(Zt, _f64(X, dev), Yt, np.zeros(M, dtype=np.int64), n_real=n_real, Zt_kin=Zt_kin, loco=False,
                 n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max, refine=refine, form=form)
    return _to_device(res, Z.device if isinstance(Z, Tensor) else dev)
