"""
GPU tests of the learned delta proposal: the training kernels against the CPU oracle (oracle/flmm_mlp_oracle.py),
a short training run, and what the trained network gains over the fit without it (grid evaluations saved at the
grid path's answers).
"""
from __future__ import annotations

from pathlib import Path
from types import SimpleNamespace

import numpy as np
import pytest
import torch

import flmm_mlp_oracle as mo
import flmm_oracle as orc
from parity import assert_log_delta_equivalent, assert_scan_close

pytestmark = pytest.mark.gpu
DEV = "cuda"
WEIGHTS = Path(__file__).resolve().parents[1] / "fast-er-lmm_gb300" / "fasterlmm_gb300" / "delta_mlp.npz"
BLOCKS = {"W1": (0, 8320), "b1": (8320, 8448), "W2": (8448, 24832), "b2": (24832, 24960), "w3": (24960, 25088),
          "b3": (25088, 25089)}


@pytest.fixture(scope="module", autouse=True)
def _built():
    from fasterlmm_gb300 import build
    build()


def _problem(seed=5, n_x=3000, batch=2048):
    from fasterlmm_gb300.learned import init_params
    rng = np.random.default_rng(seed)
    params = init_params(seed).astype(np.float64) + rng.normal(0.0, 0.02, mo.N_PARAMS)
    X = rng.normal(0.0, 1.0, (n_x, mo.N_IN))
    y = rng.normal(0.0, 2.0, n_x)
    rows = rng.integers(0, n_x, batch).astype(np.int32)
    rows[7], rows[100] = -1, n_x + 3  # indices outside the matrix contribute nothing
    return params.astype(np.float32), X.astype(np.float32), y.astype(np.float32), rows


def _gpu_grad(params, X, y, rows, bf16):
    from fasterlmm_gb300 import learned
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    g, loss = learned.mlp_grad(t(params), t(X), t(y), t(rows), huber_beta=0.1, bf16=bf16)
    return g.cpu().numpy().astype(np.float64), float(loss.item())


def _oracle_grad(params, X, y, rows, bf16):
    valid = rows[(rows >= 0) & (rows < X.shape[0])]
    loss, g = mo.loss_and_grad(params.astype(np.float64), X[valid].astype(np.float64), y[valid].astype(np.float64),
                               huber_beta=0.1, bf16=bf16)
    scale = valid.size / rows.size  # the kernel's mean is over the whole minibatch
    return g * scale, loss * scale


# FP32 operands: the kernel's FP32 sums against FP64 (~1e-6 normwise measured).  BF16 operands: where an FP32
# activation or back-propagated gradient lies within its FP32-vs-FP64 difference of a BF16 rounding boundary, the two
# sides round it to neighbouring BF16 values (2^-8 apart), and those flips move the gradient by ~3e-3 normwise.
@pytest.mark.parametrize("bf16,tol", [(False, 2e-5), (True, 1e-2)])
def test_mlp_gradient_matches_the_oracle(bf16, tol):
    """flmm_mlp_grad against the FP64 restatement with the same rounding points, block by block (normwise)."""
    params, X, y, rows = _problem()
    g, loss = _gpu_grad(params, X, y, rows, bf16)
    go, lo = _oracle_grad(params, X, y, rows, bf16)
    assert abs(loss - lo) <= 1e-5 * abs(lo)
    for name, (a, b) in BLOCKS.items():
        err = np.linalg.norm(g[a:b] - go[a:b]) / np.linalg.norm(go[a:b])
        assert err <= tol, (name, err)


def test_bf16_operands_are_rounded_and_gradient_is_deterministic():
    params, X, y, rows = _problem(seed=9)
    g16, _ = _gpu_grad(params, X, y, rows, True)
    g32, _ = _gpu_grad(params, X, y, rows, False)
    assert np.linalg.norm(g16 - g32) / np.linalg.norm(g32) > 1e-3  # BF16 rounding is visible
    g16b, _ = _gpu_grad(params, X, y, rows, True)
    np.testing.assert_array_equal(g16, g16b)  # fixed-order reduction of the per-CTA partials


def test_adamw_step_matches_the_oracle():
    from fasterlmm_gb300 import _lib
    rng = np.random.default_rng(2)
    p = rng.normal(0, 0.1, mo.N_PARAMS)
    g = rng.normal(0, 1e-2, mo.N_PARAMS)
    m = rng.normal(0, 1e-3, mo.N_PARAMS)
    v = rng.uniform(0, 1e-4, mo.N_PARAMS)
    t = lambda a: torch.from_numpy(a.astype(np.float32)).to(DEV)
    tp, tg, tm, tv = t(p), t(g), t(m), t(v)
    _lib.call("flmm_mlp_adamw", tp.data_ptr(), tg.data_ptr(), tm.data_ptr(), tv.data_ptr(), 7, 1e-3, 0.9, 0.999, 1e-8,
              1e-4, torch.cuda.current_stream().cuda_stream)
    f32 = lambda x: float(np.float32(x))  # the kernel receives its hyperparameters as FP32 values
    po, mo_, vo = mo.adamw_step(p.astype(np.float32).astype(np.float64), g.astype(np.float32).astype(np.float64),
                                m.astype(np.float32).astype(np.float64), v.astype(np.float32).astype(np.float64), 7,
                                lr=f32(1e-3), beta1=f32(0.9), beta2=f32(0.999), eps=f32(1e-8),
                                weight_decay=f32(1e-4))
    # FP32 update against FP64: a few FP32 roundings of the weight and of the step (which can nearly cancel it)
    p32 = p.astype(np.float32).astype(np.float64)
    err = np.abs(tp.cpu().numpy() - po)
    assert np.all(err <= 1e-6 * np.abs(po) + 2e-5 * np.abs(po - p32) + 1e-12), err.max()
    # m = beta1 m + (1 - beta1) g can nearly cancel: bound its error by the terms' magnitudes
    m32, g32 = m.astype(np.float32).astype(np.float64), g.astype(np.float32).astype(np.float64)
    assert np.all(np.abs(tm.cpu().numpy() - mo_) <= 1e-6 * (0.9 * np.abs(m32) + 0.1 * np.abs(g32)))
    np.testing.assert_allclose(tv.cpu().numpy(), vo, rtol=1e-5, atol=1e-13)


def test_training_kernels_fit_a_teacher_network():
    """fit_mlp (own gradient + AdamW kernels, BF16 operands) learns the outputs of a network of the same shape."""
    from fasterlmm_gb300 import learned
    rng = np.random.default_rng(4)
    X = rng.normal(0.0, 1.0, (8192, mo.N_IN))
    teacher = learned.init_params(99).astype(np.float64) * 3.0
    y = mo.forward(teacher, X)
    y = (y - y.mean()) / y.std()
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(DEV)
    params, losses = learned.fit_mlp(t(X), t(y), np.arange(7168), steps=600, batch=1024, seed=3)
    assert np.isfinite(losses).all()
    assert losses[-30:].mean() < 0.25 * losses[:30].mean(), (losses[:30].mean(), losses[-30:].mean())
    # held-out rows: the trained network beats predicting the mean by a wide margin
    pred = mo.forward(params.cpu().numpy().astype(np.float64), X[7168:], bf16=False)
    assert np.mean((pred - y[7168:]) ** 2) < 0.3


def _untrained_model(dev):
    from fasterlmm_gb300 import learned
    params = torch.from_numpy(learned.init_params(12345))
    arrays = learned.export_weights(params, np.zeros(mo.N_IN, np.float32), np.ones(mo.N_IN, np.float32))
    return learned.DeltaMLP(arrays, dev)


@pytest.mark.skipif(not WEIGHTS.exists(), reason="proposal weights not trained")
def test_trained_proposal_saves_grid_evaluations_at_the_grid_paths_answers():
    """
    The gain of the trained network over the fit without it: the same log delta as the full-grid path (loss
    equivalent), with most grid evaluations skipped; an untrained network of the same shape saves far fewer (its
    columns fall back to the full grid), and no sampled audit finds a better node outside a window.
    """
    from fasterlmm_gb300 import core, fast, learned
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(500, 4000, 1, 3, 400, seed=41, config_id=17, k_lo=0, k_hi=60, h2_lo=0.0, h2_hi=0.95)
    Zs = orc.standardise_columns(d.Z_float())
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    spec = core.fastlmm_compat_rotate(t(orc.grm(Zs)), t(d.X), t(d.Y))
    UYt = spec.UYt.float().contiguous()
    ld_grid, _ = fast.fit_delta_fast(spec.s, UYt)
    s64, UY64 = spec.s.cpu().numpy(), spec.UYt.T.cpu().numpy()
    gains = {}
    for name, model in (("trained", learned.DeltaMLP.load(torch.device(DEV))), ("untrained", _untrained_model(DEV))):
        stats = {}
        ld, _ = learned.fit_delta_learned(spec.s, UYt, model=model, stats=stats)
        assert_log_delta_equivalent(ld.cpu().numpy(), ld_grid.cpu().numpy(), s64, UY64, ld_atol=1e-6,
                                    loss_rtol=1e-10)
        gains[name] = learned.grid_evaluations(stats)
        assert gains[name]["audits_lost"] == 0
    assert gains["trained"]["saved_fraction"] >= 0.5, gains
    assert gains["trained"]["saved_fraction"] > gains["untrained"]["saved_fraction"] + 0.2, gains


@pytest.mark.skipif(not WEIGHTS.exists(), reason="proposal weights not trained")
def test_learned_fit_in_the_scan_keeps_the_reference_goldens(golden, monkeypatch):
    from fasterlmm_gb300 import fast, perms
    from conftest import z_float
    monkeypatch.setattr(fast, "DELTA_PROPOSAL", "learned")
    g = golden("loco_n150_m1500")
    B = g["f"].shape[1]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    data = SimpleNamespace(Z=t(z_float(g["G"])), X=t(g["X"]), Y=t(g["Y"]), chrom=g["chrom"], Z_kin=None,
                           chrom_kin=None)
    res, pmf = perms.perm_threshold(data, list(range(B)), n_perm=int(g["n_perm"]), form="fast")
    out = {k: getattr(res, k).cpu().numpy() for k in ("f", "beta", "se", "sfve", "nullh2", "max_F")}
    assert_scan_close(out, g)
    assert_scan_close({"perm_max_F": pmf.cpu().numpy()}, g, keys=("perm_max_F",))
