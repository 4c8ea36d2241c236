"""
The MLP training oracle (oracle/flmm_mlp_oracle.py) pinned by finite differences of its own loss, and its BF16
rounding and AdamW step checked on known values.  CPU only.
"""
from __future__ import annotations

import numpy as np

import flmm_mlp_oracle as mo


def _problem(seed=3, n=40):
    rng = np.random.default_rng(seed)
    params = rng.normal(0.0, 0.15, mo.N_PARAMS)
    X = rng.normal(0.0, 1.0, (n, mo.N_IN))
    y = rng.normal(0.0, 1.0, n)
    return params, X, y


def test_gradient_matches_central_differences():
    params, X, y = _problem()
    beta = 0.1
    loss, grad = mo.loss_and_grad(params, X, y, huber_beta=beta)
    # residuals away from the smooth-L1 kink, so the loss is smooth at the step used
    d = mo.forward(params, X) - y
    assert np.all(np.abs(np.abs(d) - beta) > 1e-3)
    rng = np.random.default_rng(11)
    h = 1e-6
    idx = np.concatenate([rng.choice(np.arange(s, s + n), 12, replace=False) for s, n in
                          ((0, 8320), (8320, 128), (8448, 16384), (24832, 128), (24960, 128))] + [[25088]])
    for i in idx:
        e = np.zeros_like(params)
        e[i] = h
        fd = (mo.loss_and_grad(params + e, X, y, huber_beta=beta)[0] -
              mo.loss_and_grad(params - e, X, y, huber_beta=beta)[0]) / (2 * h)
        assert abs(fd - grad[i]) <= 1e-7 + 1e-5 * abs(grad[i]), (i, fd, grad[i])


def test_layout_and_bf16_rounding():
    assert mo.N_PARAMS == 25089
    p = np.arange(mo.N_PARAMS, dtype=np.float64)
    u = mo.unpack(p)
    assert u["W1"][1, 0] == 65 and u["b1"][0] == 8320 and u["W2"][0, 0] == 8448 and u["b3"] == 25088
    np.testing.assert_array_equal(mo.pack(u), p)
    # 1 + 2^-8 is halfway between two BF16 values: ties go to the even one (1.0); 1 + 3 * 2^-8 rounds up
    x = np.array([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 1.0 + 2.0 ** -9])
    np.testing.assert_array_equal(mo.round_bf16(x), [1.0, 1.0 + 2.0 ** -6, -2.5, 1.0])


def test_adamw_first_step_moves_each_weight_by_lr():
    params, _, _ = _problem()
    g = np.linspace(-1, 1, mo.N_PARAMS) + 0.5
    w, m, v = mo.adamw_step(params, g, np.zeros_like(g), np.zeros_like(g), 1, lr=1e-3, weight_decay=0.0, eps=1e-12)
    # after one bias-corrected step mhat / sqrt(vhat) = sign(g)
    np.testing.assert_allclose(w - params, -1e-3 * np.sign(g), rtol=1e-6)
