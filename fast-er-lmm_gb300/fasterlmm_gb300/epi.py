"""
Batched epistasis Wald scan over K anchors (LUX tier 2): ``snp_wald_scan_batched`` with the signature and outputs of
the reference's lux/src/fasterlmm_lux/epi/_kernel.py:21-150, on the GPU.

For anchor k the design X[k] (N, C) holds the shared rotated covariates and the rotated anchor column, and S[k]
(N, M) the rotated test columns (anchor x partner products).  Per phenotype chunk the small dense algebra runs in
FP64 in the library's setup kernels (flmm_epi_setup_f64: A_p = X^T W_p X, its Cholesky factor L_p,
Q_p = L_p^-1 X^T W_p, the X-fit residual r_p and rWr; 1 <= C <= 200);
the work that scales with the test columns runs on the tensor cores as two split-FP16 products
(csrc/flmm_fast.cu, FP32 accumulation): G1 = [Q_p; (w_p o r_p)] S (C + 1 rows per phenotype) and G2 = W (S o S);
csrc/flmm_epi.cu turns them into beta, SE, F, the near-self guard and the running maximum.  Quadratic forms are
sums of squares of Q_p S, so no (C, Mc) solve is formed per test column.

Precision: operands carry ~22 bits (split FP16), sums FP32, the final formulas FP64.  Against the reference run in
FP64 the outputs agree to ~1e-5 relative away from near-collinear test columns (where sWs - quad is small against
sWs and any implementation's beta is rounding noise; the guard zeroes their F).  A Cholesky failure (a pivot that is
not positive) raises torch.linalg.LinAlgError for the whole call once the scan has run, like the reference's
batched call.
"""
from __future__ import annotations

import torch
from torch import Tensor

from . import _lib
from .core import F64, _cuda_device, _ptr, _stream
from .fast import SplitRows, gemm_split

F32 = torch.float32


def snp_wald_scan_batched(s: Tensor, X_rot_batched: Tensor, Y_rot: Tensor, log_delta: Tensor, S_rot_batched: Tensor,
                          *, snp_chunk: int = 4096, pheno_chunk: int = 256, n_real: int | None = None,
                          use_fp16_inner: bool = False, denom_floor_rel: float = 0.01):
    """
    K anchors at once (lux/src/fasterlmm_lux/epi/_kernel.py:21-150).  Returns (beta, se, chi2) of shape
    (K, M, n_real) on the CPU in the inputs' dtype, and the per-phenotype maximum F (K, P) with the first test
    column reaching it (K, P), on the CPU.  ``use_fp16_inner`` is accepted for signature compatibility: the inner
    products always run on the tensor cores here.
    """
    del use_fp16_inner
    dev = _cuda_device(s)
    dtype = s.dtype
    ctx = _lib.context(dev.index)
    K, N, C = X_rot_batched.shape
    P = Y_rot.shape[1]
    M = S_rot_batched.shape[2]
    n_real = P if n_real is None else min(n_real, P)
    var_df = N - C - 1
    st = _stream(dev)
    s64 = s.to(dev, F64).contiguous()
    Y64 = Y_rot.to(dev, F64).contiguous()
    ld64 = log_delta.to(dev, F64).contiguous()
    beta_d = torch.empty((K, M, n_real), dtype=F64, device=dev)
    se_d = torch.empty_like(beta_d)
    f_d = torch.empty_like(beta_d)
    max_f = torch.full((K, P), float("-inf"), dtype=F64, device=dev)
    argmax = torch.zeros((K, P), dtype=torch.int64, device=dev)
    info = torch.zeros(1, dtype=torch.int32, device=dev)
    snp_chunk = max(1, int(snp_chunk))
    pheno_chunk = max(1, int(pheno_chunk))
    Pmax = min(pheno_chunk, P)
    R1 = torch.empty((Pmax * (C + 1), N), dtype=F64, device=dev)
    w = torch.empty((Pmax, N), dtype=F64, device=dev)
    rWr = torch.empty(Pmax, dtype=F64, device=dev)
    Lw = torch.empty(Pmax * C * (C + 1) // 2, dtype=F64, device=dev)
    for k in range(K):
        Xk = X_rot_batched[k].to(dev, F64).contiguous()    # (N, C)
        Sk = S_rot_batched[k].to(dev, F64)                  # (N, M)
        St = Sk.t().contiguous()                            # (M, N): test columns as rows
        St_split = SplitRows.of(St)
        S2_split = SplitRows.of(St * St)
        for p0 in range(0, P, pheno_chunk):
            p1 = min(p0 + pheno_chunk, P)
            Pc = p1 - p0
            # per phenotype: w, A = X^T W X = L L^T, Q = L^-1 X^T W, the X-fit residual row w o r and rWr
            _lib.call("flmm_epi_setup_f64", _ptr(s64), N, _ptr(Xk), Xk.stride(0), C, _ptr(Y64[:, p0:]),
                      Y64.stride(0), _ptr(ld64[p0:]), Pc, _ptr(R1), _ptr(w), _ptr(rWr), _ptr(Lw), _ptr(info), st)
            R1_split = SplitRows.of(R1[:Pc * (C + 1)])
            W_split = SplitRows.of(w[:Pc])
            for m0 in range(0, M, snp_chunk):
                Mc = min(snp_chunk, M - m0)
                G1 = torch.empty((Pc * (C + 1), Mc), dtype=F32, device=dev)
                G2 = torch.empty((Pc, Mc), dtype=F32, device=dev)
                gemm_split(ctx, R1_split.view(), St_split.view(m0, Mc), G1)
                gemm_split(ctx, W_split.view(), S2_split.view(m0, Mc), G2)
                _lib.call("flmm_epi_wald_f32", _ptr(G1), G1.stride(0), _ptr(G2), G2.stride(0), _ptr(rWr), Pc, C,
                          Mc, m0, p0, n_real, float(var_df), float(denom_floor_rel), _ptr(beta_d[k]), _ptr(se_d[k]),
                          _ptr(f_d[k]), n_real, _ptr(max_f[k]), _ptr(argmax[k]), st)
    _lib.call("flmm_context_check", ctx, st)
    if int(info.item()):
        raise torch.linalg.LinAlgError("snp_wald_scan_batched: X^T W X is not positive definite for some anchor "
                                       "and phenotype (the Cholesky factorisation failed)")
    out = lambda t: t.to("cpu", dtype)
    return out(beta_d), out(se_d), out(f_d), out(max_f), argmax.cpu()


__all__ = ["snp_wald_scan_batched"]
