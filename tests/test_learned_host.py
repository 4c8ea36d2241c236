"""
Host logic of the learned delta proposal (CPU only): the parameter layout shared by the training kernels and the
oracle, the folding of the input standardisation into the exported inference weights, and the grid-evaluation
summary of a learned fit.
"""
from __future__ import annotations

import numpy as np
import torch

import flmm_mlp_oracle as mo
from fasterlmm_gb300 import learned


def test_parameter_layout_matches_the_oracle():
    p = learned.init_params(3)
    assert p.dtype == np.float32 and p.size == learned.MLP_PARAMS == mo.N_PARAMS
    ours = learned.unpack_params(p)
    theirs = mo.unpack(p.astype(np.float64))
    for name, _ in mo.SHAPES:
        np.testing.assert_array_equal(ours[name], theirs[name].astype(np.float32))
    # U(-1/sqrt(fan_in), 1/sqrt(fan_in)) per layer
    assert np.abs(ours["W1"]).max() <= 1 / np.sqrt(learned.N_FEATURES)
    assert np.abs(ours["W2"]).max() <= 1 / np.sqrt(128) and np.abs(ours["w3"]).max() <= 1 / np.sqrt(128)
    assert not np.array_equal(learned.init_params(3), learned.init_params(4))


def test_exported_weights_fold_the_input_standardisation():
    """forward(raw x; exported weights) == forward((x - mu) / sd; trained weights)."""
    rng = np.random.default_rng(8)
    params = learned.init_params(5)
    X = rng.normal(2.0, 3.0, (50, learned.N_FEATURES)).astype(np.float32)
    mu, sd = X.mean(axis=0), X.std(axis=0) + 1e-6
    arrays = learned.export_weights(torch.from_numpy(params), mu, sd)
    flat = mo.pack({"W1": arrays["W1"], "b1": arrays["b1"], "W2": arrays["W2"], "b2": arrays["b2"],
                    "w3": arrays["w3"], "b3": arrays["b3"]})
    want = mo.forward(params.astype(np.float64), (X.astype(np.float64) - mu) / sd)
    got = mo.forward(flat, X.astype(np.float64))
    np.testing.assert_allclose(got, want, rtol=1e-5, atol=1e-5)  # the folded weights are stored in FP32


def test_grid_evaluation_summary():
    stats = {"counters": torch.tensor([10, 4, 0, 700], dtype=torch.int32), "P": 100, "n_grid": 64}
    g = learned.grid_evaluations(stats)
    assert g["grid_evaluations"] == 700 + 10 * 64 and g["full_grid_evaluations"] == 6400
    assert g["fallback_rate"] == 0.1 and g["audited"] == 4 and g["audits_lost"] == 0
    assert abs(g["saved_fraction"] - (1 - 1340 / 6400)) < 1e-12
