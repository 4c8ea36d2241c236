"""
GPU tests of the eigenvector refinement's FP64-accurate product W = U~ A^T (flmm_refine_product): the tensor-core
form (exact digit planes on FP16 MMAs, csrc/flmm_ozaki.cu) and the double-FP32 form against an FP64 product of the
same U~ on kinship-like matrices, including sizes that are not multiples of the tiles or of eight, several
matrices per batch, and reductions longer than one launch (N > 1,024, added in FP64 across launches); U~ is U
rounded to 28 bits below each row's largest element.  The FP64 product is numpy's (BLAS) product of the same
operands, whose summation error is ~sqrt(N) 2^-53 of sum |u||a|, far below the tolerances.  A refinement step
through the default form reaches FP64 eigenvalues.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _case(N, batch, seed, odd_rows=True):
    rng = np.random.default_rng(seed)
    A, U = [], []
    for b in range(batch):
        Z = rng.standard_normal((N, 2 * N))
        K = Z @ Z.T / (2 * N)
        K = (K + K.T) / 2
        w, V = np.linalg.eigh(K)
        Ub = (V.T + 1e-6 * rng.standard_normal((N, N))).astype(np.float32)
        if odd_rows and N > 8:
            Ub[3] *= np.float32(1e-3)  # a row far below the others' scale
            Ub[5, ::2] = 0.0           # and one with zeros
        A.append(K)
        U.append(Ub)
    return np.stack(A), np.stack(U)


def _product(A, U, form):
    from fasterlmm_gb300 import _lib
    batch, N, _ = A.shape
    Ad = torch.from_numpy(A).cuda()
    Ud = torch.from_numpy(U).cuda()
    Ut = torch.empty_like(Ud)
    W = torch.empty_like(Ad)
    wb = _lib.query_bytes("flmm_refine_product_workspace_bytes", N, batch)
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    st = torch.cuda.current_stream().cuda_stream
    _lib.call("flmm_refine_product", Ud.data_ptr(), Ad.data_ptr(), N, batch, form, Ut.data_ptr(), W.data_ptr(),
              work.data_ptr(), wb, st)
    torch.cuda.synchronize()
    return Ut.cpu().numpy(), W.cpu().numpy()


@pytest.mark.parametrize("N,batch", [(8, 2), (301, 3), (1000, 2), (1100, 2)])
def test_refine_product_matches_fp64(N, batch):
    from fasterlmm_gb300 import build
    build()
    A, U = _case(N, batch, seed=N)
    for form, tol in ((0, 1e-13), (1, 2e-12)):
        Ut, W = _product(A, U, form)
        for b in range(batch):
            rowmax = np.abs(U[b]).max(axis=1, keepdims=True)
            rowmax[rowmax == 0] = 1
            if form == 1:
                np.testing.assert_array_equal(Ut[b], U[b])
            else:
                # U~ rounds at 2^-27 of each row's largest element; elements within 2^-3 of it are exact
                assert np.all(np.abs(Ut[b] - U[b]) <= 2.0 ** -27 * rowmax)
                big = np.abs(U[b]) >= rowmax / 8
                np.testing.assert_array_equal(Ut[b][big], U[b][big])
            ref = Ut[b].astype(np.float64) @ A[b].T
            scale = np.abs(Ut[b].astype(np.float64)) @ np.abs(A[b]).T
            scale[scale == 0] = 1
            err = (np.abs(W[b] - ref) / scale).max()
            assert err <= tol, (form, err)


def test_refinement_step_agrees_across_product_forms():
    """Both forms' products agree with the FP64 product of U to the rounding of U~, and one refinement step through
    the default (tensor-core) form returns the input's Rayleigh quotients and brings eigenvectors perturbed by 1e-6
    to FP64 eigenvalues within 1e-10 of the largest."""
    from fasterlmm_gb300 import build, _lib
    build()
    N, batch = 600, 2
    A, U = _case(N, batch, seed=7, odd_rows=False)
    Ad = torch.from_numpy(A).cuda()
    wb = _lib.query_bytes("flmm_eigh_refine_workspace_bytes", N, batch)
    st = torch.cuda.current_stream().cuda_stream
    outs = []
    for form in (0, 1):
        # the product's form is read once per process from the environment, so call the product entry point to
        # compare the forms: the step is W = product, then the FP32 corrections, identical for both
        Ut, W = _product(A, U, form)
        outs.append((Ut, W))
    # the forms' products of their own U~ agree with the FP64 product of U to the rounding of U~ (2^-27 relative)
    for b in range(batch):
        full = U[b].astype(np.float64) @ A[b].T
        for Ut, W in outs:
            assert np.abs(W[b] - full).max() <= 2.0 ** -26 * np.abs(full).max() * np.sqrt(N)
    # and the refinement entry point runs end to end with the default (tensor-core) form
    Ud = torch.from_numpy(U).cuda()
    Uo = torch.empty_like(Ud)
    ev = torch.empty((batch, N), dtype=torch.float64, device="cuda")
    work = torch.empty(wb, dtype=torch.uint8, device="cuda")
    _lib.call("flmm_eigh_refine_f32", Ad.data_ptr(), Ud.data_ptr(), Uo.data_ptr(), ev.data_ptr(), N, batch,
              work.data_ptr(), wb, st)
    torch.cuda.synchronize()
    Ut0 = outs[0][0]
    for b in range(batch):
        ref = np.linalg.eigvalsh(A[b])
        lam = np.abs(ref).max()
        # evals are the FP64 Rayleigh quotients of the step's input vectors U~ (error O(N eps^2) against FP64 eigh)
        Ui = Ut0[b].astype(np.float64)
        rq_in = np.einsum("jn,jn->j", Ui @ A[b], Ui) / np.einsum("jn,jn->j", Ui, Ui)
        np.testing.assert_allclose(ev[b].cpu().numpy(), rq_in, rtol=0, atol=1e-12 * lam)
        # the refined vectors' quotients match FP64 eigh to the FP32 rounding of the output vectors
        Ub = Uo[b].double().cpu().numpy()
        rq = np.einsum("jn,jn->j", Ub @ A[b], Ub) / np.einsum("jn,jn->j", Ub, Ub)
        np.testing.assert_allclose(rq, ref, rtol=0, atol=1e-10 * lam)
        assert np.abs(rq - ref).max() < np.abs(rq_in - ref).max() / 10
        R = A[b] @ Ub.T - Ub.T * ref
        assert np.abs(R).max() <= 1e-6 * lam
