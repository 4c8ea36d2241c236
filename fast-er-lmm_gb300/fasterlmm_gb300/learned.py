"""
Learned delta proposal for the fast delta fit (no counterpart in the reference, whose fit is a grid argmin plus a
golden-section search).

A small MLP (65 -> 128 -> 128 -> 1, tanh-GELU) maps cheap features of each rotated column -- the log energy
fractions of UY^2 over 32 equal-count bins of the ascending spectrum, the log mean eigenvalue per bin, log Neff --
to a proposed log delta.  The fit's grid search then collapses to a narrow bracket: each column evaluates the grid
loss at the 2 HALF_WIDTH + 1 nodes nearest its proposal.  A window argmin on the window's edge sends the column to
the full grid; a sampled audit (every AUDIT_STRIDE-th column evaluates the full grid) sends every column there if
a node outside a window wins.  The exact Newton refinement then runs from the chosen node, as in the grid path
(csrc/flmm_delta_learned.cu), so the proposal saves grid evaluations without moving the answer.

The weights (``delta_mlp.npz`` beside this file) are produced by ``python -m fasterlmm_gb300.learned train`` on a
GB300: seeded synthetic datasets (N from 300 to 2,000, 1 to 6 covariates, h2 uniform on [0, 0.95], 0 to 100 causal
variants, each phenotype plus one permuted copy), labels from the exact fit on a 200-point grid, trained by the
library's own kernels (csrc/flmm_mlp_train.cu: minibatch gradient with BF16 operands and FP32 accumulation, AdamW
on FP32 master weights).
"""

from __future__ import annotations

import argparse
import json
import time
from pathlib import Path

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .core import F64, CovariateBasis, _ptr, _stream, _work, gram_t, kinship_from_gram, project_kinship, \
    standardise_columns_t, transpose

F32 = torch.float32
WEIGHTS = Path(__file__).resolve().parent / "delta_mlp.npz"
N_FEATURES = 65


class DeltaMLP:
    """The proposal network's weights on one device (the layout flmm_delta_mlp_f32 reads)."""

    _cache: dict = {}

    def __init__(self, arrays: dict, dev: torch.device):
        t = lambda k: torch.from_numpy(np.ascontiguousarray(arrays[k], dtype=np.float32)).to(dev)
        self.W1, self.b1, self.W2, self.b2, self.w3 = t("W1"), t("b1"), t("W2"), t("b2"), t("w3")
        self.b3 = float(arrays["b3"])
        assert self.W1.shape == (128, N_FEATURES) and self.W2.shape == (128, 128) and self.w3.shape == (128,)

    @classmethod
    def load(cls, dev: torch.device, path: Path = WEIGHTS) -> "DeltaMLP":
        key = (str(path), str(dev))
        if key not in cls._cache:
            with np.load(path) as z:
                cls._cache[key] = cls({k: z[k] for k in z.files}, dev)
        return cls._cache[key]


def features_t(s: Tensor, UYt: Tensor) -> Tensor:
    """(P, 65) FP32 features of device columns UYt (P, Neff) FP32 against the ascending spectrum s (Neff,) FP64."""
    P, Neff = UYt.shape
    feats = torch.empty((P, N_FEATURES), dtype=F32, device=s.device)
    _lib.call("flmm_delta_features_f32", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), P, _ptr(feats), _stream(s.device))
    return feats


def propose_t(feats: Tensor, model: DeltaMLP, lo: float, hi: float) -> Tensor:
    P = feats.shape[0]
    x = torch.empty(P, dtype=F64, device=feats.device)
    _lib.call("flmm_delta_mlp_f32", _ptr(feats), P, _ptr(model.W1), _ptr(model.b1), _ptr(model.W2), _ptr(model.b2),
              _ptr(model.w3), model.b3, float(lo), float(hi), _ptr(x), _stream(feats.device))
    return x


# Narrow bracket: grid nodes evaluated on each side of the proposal's nearest node, and the audit rate (every
# AUDIT_STRIDE-th column also evaluates the full grid; a lost audit sends every column of the call to the full grid).
HALF_WIDTH = 3
AUDIT_STRIDE = 64


def fit_delta_learned(s: Tensor, UYt: Tensor, *, n_grid: int = 64, log_delta_min: float = -10.0,
                      log_delta_max: float = 10.0, refine: bool = True, model: DeltaMLP | None = None,
                      stats: dict | None = None, half_width: int = HALF_WIDTH,
                      audit_stride: int = AUDIT_STRIDE) -> tuple[Tensor, Tensor]:
    """
    Fast delta fit with the grid search collapsed to the proposal's bracket (flmm_fit_delta_learned):
    (log_delta (P,), grid index (P,)), same contract as fast.fit_delta_fast.  ``stats``, if given, receives the
    device counters (int32[4]: fallback columns, audited columns, audits lost, grid nodes evaluated by the window
    and audit pass); see :func:`grid_evaluations` for the totals.
    """
    from .fast import fit_delta_fast
    dev = s.device
    P, Neff = UYt.shape
    if Neff < 32:  # too few samples for the features: the grid path
        return fit_delta_fast(s, UYt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                              refine=refine)
    model = model or DeltaMLP.load(dev)
    ld = torch.empty(P, dtype=F64, device=dev)
    idx = torch.empty(P, dtype=torch.int32, device=dev)
    cnt = torch.empty(4, dtype=torch.int32, device=dev)
    w, wb = _work.get(dev, _lib.query_bytes("flmm_fit_delta_learned_workspace_bytes", Neff, n_grid, P))
    _lib.call("flmm_fit_delta_learned", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), P, n_grid, float(log_delta_min),
              float(log_delta_max), int(bool(refine)), _ptr(model.W1), _ptr(model.b1), _ptr(model.W2),
              _ptr(model.b2), _ptr(model.w3), model.b3, int(half_width), int(audit_stride), _ptr(ld), _ptr(idx),
              _ptr(cnt), w, wb, _stream(dev))
    if stats is not None:
        stats.update(counters=cnt, P=P, n_grid=n_grid)
    return ld, idx


def grid_evaluations(stats: dict) -> dict:
    """Host summary of a learned fit's counters: grid-node loss evaluations against the full grid's P * n_grid."""
    fb, audited, lost, window = (int(v) for v in stats["counters"].cpu().tolist())
    P, G = stats["P"], stats["n_grid"]
    done = window + fb * G
    return {"columns": P, "fallback": fb, "fallback_rate": fb / max(P, 1), "audited": audited, "audits_lost": lost,
            "grid_evaluations": done, "full_grid_evaluations": P * G, "saved_fraction": 1.0 - done / max(P * G, 1)}


# ---- training ------------------------------------------------------------------------------------------------

def _columns(rng: np.random.Generator, dev: torch.device, N: int, M: int, D: int, B: int, seed: int):
    """One synthetic single-kinship dataset -> (s, UYt FP32) through the fast form's own rotation."""
    from .fast import SplitRows, _eigh_batched_f32_refined, _spectrum, gemm_split
    from .synth import make_dataset
    d = make_dataset(N, M, 1, D, B, seed=seed, config_id=31, maf_lo=0.01, h2_lo=0.0, h2_hi=0.95, k_lo=0, k_hi=100)
    Y = d.Y.copy()
    perm = np.stack([rng.permutation(N) for _ in range(B)], axis=1)
    Y = np.concatenate([Y, np.take_along_axis(Y, perm, axis=0)], axis=1)  # each phenotype plus one permuted copy
    ctx = _lib.context(dev.index)
    Zt = standardise_columns_t(torch.from_numpy(d.Z_float()).to(dev), dev)
    X = torch.from_numpy(d.X).to(dev)
    basis = CovariateBasis(X)
    Kp = torch.empty((1, N, N), dtype=F64, device=dev)
    project_kinship(kinship_from_gram(gram_t(Zt), None, M), basis, Kp[0])
    U, ev = _eigh_batched_f32_refined(ctx, Kp)
    s = _spectrum(ev[0], D)
    Ut = U[0, D:]
    Yr = basis.regress_out(transpose(torch.from_numpy(Y).to(dev)))
    UYt = torch.empty((Yr.shape[0], N - D), dtype=F32, device=dev)
    gemm_split(ctx, SplitRows.of(Yr).view(), SplitRows.of(Ut).view(), UYt)
    return s, UYt


def make_training_set(n_sets: int, seed: int, dev: torch.device) -> tuple[np.ndarray, np.ndarray]:
    """Features and exact-fit labels (200-point grid on [-10, 10]) from n_sets seeded synthetic datasets."""
    from .fast import fit_delta_fast
    rng = np.random.default_rng(seed)
    feats, labels = [], []
    for k in range(n_sets):
        N = int(rng.choice([300, 500, 800, 1000, 1500, 2000]))
        M = int(min(50_000, rng.integers(2 * N, 30 * N)))
        D = int(rng.integers(1, 7))
        s, UYt = _columns(rng, dev, N, M, D, 300, seed=seed * 1000 + k)
        ld, _ = fit_delta_fast(s, UYt, n_grid=200)
        feats.append(features_t(s, UYt).cpu().numpy())
        labels.append(ld.cpu().numpy())
    return np.concatenate(feats), np.concatenate(labels)


MLP_PARAMS = 25089  # FLMM_MLP_PARAMS: W1 (128, 65) | b1 (128) | W2 (128, 128) | b2 (128) | w3 (128) | b3
_LAYOUT = (("W1", (128, N_FEATURES)), ("b1", (128,)), ("W2", (128, 128)), ("b2", (128,)), ("w3", (128,)), ("b3", ()))


def init_params(seed: int) -> np.ndarray:
    """Flat FP32 parameters, each layer U(-1/sqrt(fan_in), 1/sqrt(fan_in)) like a freshly made linear layer."""
    rng = np.random.default_rng(seed)
    parts = []
    for name, shape in _LAYOUT:
        fan_in = N_FEATURES if name in ("W1", "b1") else 128
        bound = 1.0 / np.sqrt(fan_in)
        parts.append(rng.uniform(-bound, bound, int(np.prod(shape))))
    out = np.concatenate(parts).astype(np.float32)
    assert out.size == MLP_PARAMS
    return out


def unpack_params(flat: np.ndarray) -> dict:
    out, off = {}, 0
    for name, shape in _LAYOUT:
        n = int(np.prod(shape))
        out[name] = np.asarray(flat[off:off + n], dtype=np.float32).reshape(shape)
        off += n
    return out


def mlp_grad(params: Tensor, X: Tensor, y: Tensor, rows: Tensor, *, huber_beta: float = 0.1, bf16: bool = True,
             grad: Tensor | None = None, loss: Tensor | None = None) -> tuple[Tensor, Tensor]:
    """Gradient of the mean smooth-L1 loss over X[rows] on the device (flmm_mlp_grad): (grad, loss)."""
    dev = params.device
    batch = rows.numel()
    grad = torch.empty(MLP_PARAMS, dtype=F32, device=dev) if grad is None else grad
    loss = torch.empty(1, dtype=F32, device=dev) if loss is None else loss
    w, wb = _work.get(dev, _lib.query_bytes("flmm_mlp_grad_workspace_bytes", batch))
    _lib.call("flmm_mlp_grad", _ptr(params), _ptr(X), X.stride(0), X.shape[0], _ptr(y), _ptr(rows), batch,
              float(huber_beta), int(bool(bf16)), _ptr(grad), _ptr(loss), w, wb, _stream(dev))
    return grad, loss


def fit_mlp(X: Tensor, y: Tensor, train_rows: np.ndarray, *, steps: int, batch: int = 2048, lr: float = 2e-3,
            weight_decay: float = 1e-4, huber_beta: float = 0.1, seed: int = 0, bf16: bool = True) -> tuple:
    """
    Train the proposal MLP with the library's own kernels: per step a minibatch gradient (flmm_mlp_grad, BF16
    operands, FP32 accumulation) and an AdamW step on the FP32 master weights (flmm_mlp_adamw), cosine-annealed
    learning rate.  X (n, 65) FP32 features (already standardised), y (n,) FP32 labels on the device.
    Returns (FP32 master parameters (MLP_PARAMS,) on the device, per-step minibatch losses as numpy).
    """
    dev = X.device
    rng = np.random.default_rng(seed)
    params = torch.from_numpy(init_params(seed)).to(dev)
    m = torch.zeros_like(params)
    v = torch.zeros_like(params)
    grad = torch.empty_like(params)
    losses = torch.empty(steps, dtype=F32, device=dev)
    picks = rng.integers(0, len(train_rows), (steps, batch))
    rows = torch.from_numpy(np.asarray(train_rows, dtype=np.int32)[picks]).to(dev)
    st = _stream(dev)
    for k in range(steps):
        mlp_grad(params, X, y, rows[k], huber_beta=huber_beta, bf16=bf16, grad=grad, loss=losses[k:k + 1])
        lr_k = lr * 0.5 * (1.0 + np.cos(np.pi * k / steps))
        _lib.call("flmm_mlp_adamw", _ptr(params), _ptr(grad), _ptr(m), _ptr(v), k + 1, float(lr_k), 0.9, 0.999,
                  1e-8, float(weight_decay), st)
    return params, losses.cpu().numpy()


def export_weights(params: Tensor, mu: np.ndarray, sd: np.ndarray) -> dict:
    """Inference arrays for flmm_delta_mlp_f32, with the input standardisation (x - mu) / sd folded into layer 1."""
    p = unpack_params(params.cpu().numpy())
    W1 = p["W1"] / sd[None, :]
    b1 = p["b1"] - W1 @ mu
    return {"W1": W1.astype(np.float32), "b1": b1.astype(np.float32), "W2": p["W2"], "b2": p["b2"], "w3": p["w3"],
            "b3": np.float32(p["b3"])}


def train(out: Path, *, n_sets: int = 48, steps: int = 4000, seed: int = 20240601) -> dict:
    """Train the proposal MLP on the device with the library's kernels and write its weights to ``out``."""
    dev = torch.device("cuda", torch.cuda.current_device())
    t0 = time.time()
    X, y = make_training_set(n_sets, seed, dev)
    t_data = time.time() - t0
    n = X.shape[0]
    rng = np.random.default_rng(seed + 1)
    order = rng.permutation(n)
    n_val = max(1, n // 10)
    val, tr = order[:n_val], order[n_val:]
    mu, sd = X[tr].mean(axis=0), X[tr].std(axis=0) + 1e-6
    Xt = torch.from_numpy(((X - mu) / sd).astype(np.float32)).to(dev)
    yt = torch.from_numpy(y.astype(np.float32)).to(dev)
    t1 = time.time()
    params, losses = fit_mlp(Xt, yt, tr, steps=steps, seed=seed)
    torch.cuda.synchronize()
    t_fit = time.time() - t1
    arrays = export_weights(params, mu, sd)
    model = DeltaMLP(arrays, dev)
    feats_val = torch.from_numpy(X[val].astype(np.float32)).to(dev)
    pv = propose_t(feats_val, model, -1e30, 1e30).cpu().numpy()
    err = np.abs(pv - y[val])
    info = {"samples": int(n), "train_s": time.time() - t0, "data_s": t_data, "fit_s": t_fit, "steps": steps,
            "loss_first": float(losses[:50].mean()), "loss_last": float(losses[-50:].mean()),
            "val_abs_err_median": float(np.median(err)), "val_abs_err_p90": float(np.quantile(err, 0.9)),
            "val_within_0.1": float((err < 0.1).mean()), "trainer": "flmm_mlp_grad + flmm_mlp_adamw (BF16 operands)"}
    np.savez(out, **arrays, info=json.dumps(info))
    return info


# ---- the learned-proposal configuration: training and held-out evaluation at one cohort shape -------------------

def _simulate(Zt: Tensor, B: int, seed: int) -> Tensor:
    """B phenotypes (B, N) on the device from standardised genotypes Zt (M, N) by the method's simulator recipe
    (fasterlmm/sim.py:21-28) with per-phenotype h2 ~ U[0, 0.95], 1-500 causal variants and effects N(0, h2 / k)."""
    M, N = Zt.shape
    rng = np.random.default_rng([seed, 4, 1])
    Yt = torch.empty((B, N), dtype=F64, device=Zt.device)
    for b in range(B):
        h2 = rng.uniform(0.0, 0.95)
        k = int(rng.integers(1, 501))
        idx = torch.from_numpy(rng.choice(M, size=k, replace=False)).to(Zt.device)
        beta = torch.from_numpy(rng.standard_normal(k) * np.sqrt(h2 / k)).to(Zt.device)
        noise = torch.from_numpy(rng.standard_normal(N) * np.sqrt(1.0 - h2)).to(Zt.device)
        Yt[b] = beta @ Zt.index_select(0, idx) + noise
    return Yt


def config4(out_weights: Path, *, N: int = 2000, M: int = 50_000, n_train: int = 20_000, n_eval: int = 10_000,
            n_perm: int = 100, steps: int = 4000, n_grid: int = 200, seed: int = 20250404, wald_variants: int = 2000,
            timers: bool = True) -> dict:
    """
    Train the proposal on n_train phenotypes of one simulated cohort (N x M, single kinship of all variants; labels
    from the exact fit on an n_grid-point grid) with the library's training kernels, then evaluate it on n_eval
    held-out phenotypes x (1 + n_perm) columns against the full grid: grid evaluations saved, fallback rate, lost
    audits, |d log delta|, and |d(-log10 p)| of a fused Wald scan of `wald_variants` variants under either fit.
    """
    from .core import ScanResult
    from .fast import SplitRows, WaldOperands, _eigh_batched_f32_refined, _spectrum, fit_delta_fast, gemm_split, \
        wald_fast
    from .perms import pack_perm_columns, perm_orders_device
    from .post import neg_log10_pvalue
    dev = torch.device("cuda", torch.cuda.current_device())
    ctx = _lib.context(dev.index)
    from .synth import make_dataset
    t0 = time.time()
    d = make_dataset(N, M, 22, 1, 1, seed=seed, config_id=4, maf_lo=0.05, k_lo=1, k_hi=1)
    Zt = standardise_columns_t(torch.from_numpy(d.Z_float()).to(dev), dev)
    del d
    Yt = _simulate(Zt, n_train + n_eval, seed)
    t_sim = time.time() - t0
    X = torch.ones((N, 1), dtype=F64, device=dev)
    basis = CovariateBasis(X)
    Kp = torch.empty((1, N, N), dtype=F64, device=dev)
    project_kinship(kinship_from_gram(gram_t(Zt), None, M), basis, Kp[0])
    U, ev = _eigh_batched_f32_refined(ctx, Kp)
    D = 1
    s = _spectrum(ev[0], D)
    Us = SplitRows.of(U[0, D:])

    def rotate(Yt):
        Yr = basis.regress_out(Yt)
        out = torch.empty((Yr.shape[0], N - D), dtype=F32, device=dev)
        gemm_split(ctx, SplitRows.of(Yr).view(), Us.view(), out)
        return out

    # training: features and exact-fit labels of the training phenotypes
    UY_tr = rotate(Yt[:n_train])
    lab, _ = fit_delta_fast(s, UY_tr, n_grid=n_grid)
    X_tr = features_t(s, UY_tr).cpu().numpy()
    y_tr = lab.cpu().numpy()
    mu, sd = X_tr.mean(axis=0), X_tr.std(axis=0) + 1e-6
    Xt = torch.from_numpy(((X_tr - mu) / sd).astype(np.float32)).to(dev)
    yt = torch.from_numpy(y_tr.astype(np.float32)).to(dev)
    t1 = time.time()
    params, losses = fit_mlp(Xt, yt, np.arange(n_train), steps=steps, seed=seed)
    torch.cuda.synchronize()
    t_fit = time.time() - t1
    arrays = export_weights(params, mu, sd)
    model = DeltaMLP(arrays, dev)
    # held-out evaluation: each phenotype with n_perm shuffles (numpy's PCG64 orders, as the scan draws them)
    cols = list(range(n_train, n_train + n_eval))
    orders = perm_orders_device(N, cols, n_perm, 19930909, dev)
    Yt_all = pack_perm_columns(Yt[n_train:].contiguous(), orders)
    UY = rotate(Yt_all)
    del Yt_all
    P = UY.shape[0]
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    fit_delta_fast(s, UY[:1024], n_grid=n_grid)  # warm both paths
    fit_delta_learned(s, UY[:1024], n_grid=n_grid, model=model)
    e0.record()
    ld_full, _ = fit_delta_fast(s, UY, n_grid=n_grid)
    e1.record()
    stats: dict = {}
    ld_l, _ = fit_delta_learned(s, UY, n_grid=n_grid, model=model, stats=stats)
    e2.record()
    torch.cuda.synchronize()
    g = grid_evaluations(stats)
    dld = (ld_l - ld_full).abs().cpu().numpy()
    # Wald scan of a block of variants under either fit: -log10 p of the real columns and the permutation maxima
    rows = torch.arange(wald_variants, dtype=torch.int64, device=dev)
    USt = torch.empty((wald_variants, N - D), dtype=F32, device=dev)
    gemm_split(ctx, SplitRows.of(Zt[:wald_variants]).view(), Us.view(), USt)
    ops = WaldOperands(dev)
    res = {}
    for tag, ld in (("full", ld_full), ("learned", ld_l)):
        out = {k: torch.zeros((wald_variants, n_eval), dtype=F64, device=dev) for k in ("f", "beta", "se", "sfve")}
        max_F = torch.full((P,), float("-inf"), dtype=F64, device=dev)
        wald_fast(ctx, ops, s, UY, ld, USt, n_eval, rows, out, max_F)
        res[tag] = (neg_log10_pvalue(out["f"], N - D - 1), neg_log10_pvalue(max_F, N - D - 1))
    dp = (res["learned"][0] - res["full"][0]).abs().max().item()
    dq = (res["learned"][1] - res["full"][1]).abs().max().item()
    rec = {"cohort": {"N": N, "M": M, "chromosomes": 22, "kinship": "single, all variants", "covariates": "intercept"},
           "training": {"phenotypes": n_train, "labels": f"exact fit from the {n_grid}-point grid argmin",
                        "steps": steps, "trainer": "flmm_mlp_grad + flmm_mlp_adamw (BF16 operands, FP32 master)",
                        "fit_s": round(t_fit, 2), "loss_first": float(losses[:50].mean()),
                        "loss_last": float(losses[-50:].mean())},
           "evaluation": {"phenotypes": n_eval, "permutations": n_perm, "columns": P, **g,
                          "abs_d_log_delta_median": float(np.median(dld)),
                          "abs_d_log_delta_p99": float(np.quantile(dld, 0.99)),
                          "abs_d_log_delta_max": float(dld.max()),
                          "wald_variants": wald_variants, "max_abs_d_neglog10p_real": dp,
                          "max_abs_d_neglog10p_perm_max": dq,
                          "fit_ms_full_grid": e0.elapsed_time(e1), "fit_ms_learned": e1.elapsed_time(e2)},
           "simulate_s": round(t_sim, 1)}
    np.savez(out_weights, **arrays, info=json.dumps(rec))
    return rec


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description="train (and evaluate) the learned delta proposal")
    ap.add_argument("cmd", choices=["train", "config4"])
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--sets", type=int, default=48)
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--n-train", type=int, default=20_000)
    ap.add_argument("--n-eval", type=int, default=10_000)
    ap.add_argument("--n-perm", type=int, default=100)
    args = ap.parse_args(argv)
    from . import build
    build()
    if args.cmd == "train":
        print(json.dumps(train(Path(args.out), n_sets=args.sets, steps=args.steps)), flush=True)
    else:
        print(json.dumps(config4(Path(args.out), n_train=args.n_train, n_eval=args.n_eval, n_perm=args.n_perm,
                                 steps=args.steps)), flush=True)


if __name__ == "__main__":
    main()
