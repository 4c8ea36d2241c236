"""
CPU oracle for the training arithmetic of the learned delta proposal's MLP.

TEST INFRASTRUCTURE ONLY.  The proposal network has no counterpart in the reference (FaST-ER-LMM fits delta by a
grid search plus golden-section refinement, fasterlmm/core.py:561-595), so there is no reference output to pin this
file to.  It restates, in numpy FP64, the forward pass, the back-propagated gradient of the mean smooth-L1 loss and
the AdamW step that the library's training kernels compute, with the same BF16 rounding points, so that the GPU
gradients can be checked against it.  It is pinned by finite differences of its own loss (tests/test_mlp_oracle.py).
Only tests/ use it; the product path never imports it.

Parameter layout (one flat array, FLMM_MLP_PARAMS = 25,089 values):
    W1 (128, 65) | b1 (128) | W2 (128, 128) | b2 (128) | w3 (128) | b3 (1)
"""

from __future__ import annotations

import numpy as np

N_IN, N_HID = 65, 128
SHAPES = (("W1", (N_HID, N_IN)), ("b1", (N_HID,)), ("W2", (N_HID, N_HID)), ("b2", (N_HID,)), ("w3", (N_HID,)),
          ("b3", ()))
N_PARAMS = sum(int(np.prod(s)) for _, s in SHAPES)

GELU_C = 0.7978845608028654  # sqrt(2 / pi)
GELU_A = 0.044715


def unpack(params: np.ndarray) -> dict:
    """Views of the flat parameter array by name."""
    out, off = {}, 0
    for name, shape in SHAPES:
        n = int(np.prod(shape))
        out[name] = params[off:off + n].reshape(shape)
        off += n
    return out


def pack(parts: dict) -> np.ndarray:
    return np.concatenate([np.asarray(parts[name], dtype=np.float64).reshape(-1) for name, _ in SHAPES])


def round_bf16(x: np.ndarray) -> np.ndarray:
    """Round to BF16 (nearest, ties to even) via FP32, returned as float64 values."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def gelu(x: np.ndarray) -> np.ndarray:
    return 0.5 * x * (1.0 + np.tanh(GELU_C * (x + GELU_A * x ** 3)))


def gelu_grad(x: np.ndarray) -> np.ndarray:
    t = np.tanh(GELU_C * (x + GELU_A * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * GELU_C * (1.0 + 3.0 * GELU_A * x * x)


def forward(params: np.ndarray, X: np.ndarray, *, bf16: bool = False) -> np.ndarray:
    """Network output (n,) for feature rows X (n, 65)."""
    return _forward(params, X, bf16)[-1]


def _forward(params, X, bf16):
    op = round_bf16 if bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    p = unpack(np.asarray(params, dtype=np.float64))
    x = op(X)
    W1, W2, w3 = op(p["W1"]), op(p["W2"]), op(p["w3"])
    z1 = x @ W1.T + p["b1"]
    a1 = op(gelu(z1))
    z2 = a1 @ W2.T + p["b2"]
    a2 = op(gelu(z2))
    o = a2 @ w3 + p["b3"]
    return op, x, W2, w3, z1, a1, z2, a2, o


def loss_and_grad(params: np.ndarray, X: np.ndarray, y: np.ndarray, *, huber_beta: float = 0.1,
                  bf16: bool = False) -> tuple[float, np.ndarray]:
    """
    Mean smooth-L1 loss over the rows and its gradient with respect to the flat parameters, with the training
    kernels' rounding points: with bf16, the inputs, weights, activations and the pre-activation gradients dz are
    rounded to BF16 where they enter a product (bias gradients sum the rounded dz).
    """
    op, x, W2, w3, z1, a1, z2, a2, o = _forward(params, X, bf16)
    n = X.shape[0]
    d = o - np.asarray(y, dtype=np.float64)
    small = np.abs(d) < huber_beta
    loss = float(np.where(small, 0.5 * d * d / huber_beta, np.abs(d) - 0.5 * huber_beta).sum() / n)
    g = np.where(small, d / huber_beta, np.sign(d)) / n
    dz2 = op(g[:, None] * w3[None, :] * gelu_grad(z2))
    dz1 = op((dz2 @ W2) * gelu_grad(z1))
    grads = {"W1": dz1.T @ x, "b1": dz1.sum(axis=0), "W2": dz2.T @ a1, "b2": dz2.sum(axis=0), "w3": a2.T @ g,
             "b3": g.sum()}
    return loss, pack(grads)


def adamw_step(params: np.ndarray, grad: np.ndarray, m: np.ndarray, v: np.ndarray, step: int, *, lr: float,
               beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, weight_decay: float = 1e-2):
    """One AdamW step (decoupled weight decay, bias-corrected moments): returns (params, m, v)."""
    w = params * (1.0 - lr * weight_decay)
    m = beta1 * m + (1.0 - beta1) * grad
    v = beta2 * v + (1.0 - beta2) * grad * grad
    mhat = m / (1.0 - beta1 ** step)
    vhat = v / (1.0 - beta2 ** step)
    return w - lr * mhat / (np.sqrt(vhat) + eps), m, v
