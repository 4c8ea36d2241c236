"""
GPU tests of the library's own batched FP32 eigensolver (csrc/flmm_eigh_own.cu, behind flmm_eigh_batched_f32 for
N < 2,500): residual, orthogonality and eigenvalues against numpy's FP64 eigh on kinship-like matrices, projected
kinships with an exact null space (the D covariate directions) and a repeated eigenvalue, and the tiny sizes where
the tridiagonalisation has no reflector; after the fast form's refinement steps the eigenvalues agree with FP64 to
the refinement's accuracy.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _kinships(N, batch, seed, project=0, repeat=False):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(batch):
        M = max(2 * N, 8)
        Z = rng.standard_normal((N, M))
        K = Z @ Z.T / M
        if project:
            X = np.concatenate([np.ones((N, 1)), rng.standard_normal((N, project - 1))], axis=1)
            Q, _ = np.linalg.qr(X)
            P = np.eye(N) - Q @ Q.T
            K = P @ K @ P
        if repeat and N > 12:
            w, V = np.linalg.eigh(K)
            w[10] = w[11]
            K = (V * w) @ V.T
        out.append((K + K.T) / 2)
    return np.stack(out)


def _own(K):
    from fasterlmm_gb300 import fast
    from fasterlmm_gb300 import _lib
    Kd = torch.from_numpy(K).cuda()
    U, ev = fast._eigh_batched_f32(_lib.context(0), Kd)
    torch.cuda.synchronize()
    return U.double().cpu().numpy(), ev.double().cpu().numpy()


@pytest.mark.parametrize("N,batch,project,repeat", [(1, 2, 0, False), (2, 2, 0, False), (3, 3, 0, False),
                                                    (64, 3, 0, False), (257, 2, 3, True), (1000, 4, 5, False)])
def test_own_eigensolver_residual_and_orthogonality(N, batch, project, repeat):
    from fasterlmm_gb300 import build
    build()
    K = _kinships(N, batch, seed=N + batch, project=project, repeat=repeat)
    U, ev = _own(K)
    for b in range(batch):
        nrm = max(np.abs(np.linalg.eigvalsh(K[b])).max(), 1e-30)
        ref = np.linalg.eigvalsh(K[b])
        assert np.all(np.diff(ev[b]) >= -1e-6 * nrm), "eigenvalues not ascending"
        np.testing.assert_allclose(ev[b], ref, rtol=0, atol=2e-5 * nrm)
        R = K[b] @ U[b].T - U[b].T * ev[b]
        assert np.abs(R).max() <= 5e-5 * nrm, np.abs(R).max() / nrm
        O = U[b] @ U[b].T - np.eye(N)
        assert np.abs(O).max() <= 5e-5, np.abs(O).max()


def test_own_eigensolver_then_refinement_reaches_fp64():
    from fasterlmm_gb300 import _lib, build, fast
    build()
    K = _kinships(1000, 3, seed=7, project=5)
    U, ev = fast._eigh_batched_f32_refined(_lib.context(0), torch.from_numpy(K).cuda())
    torch.cuda.synchronize()
    ev = ev.cpu().numpy()
    for b in range(3):
        ref = np.linalg.eigvalsh(K[b])
        # the kept spectrum (above the D null directions) to near FP64 accuracy
        np.testing.assert_allclose(ev[b][5:], ref[5:], rtol=1e-10, atol=1e-12)
