"""
Learned delta proposal for the fast delta fit (no counterpart in the reference, whose fit is a grid argmin plus a
golden-section search).

A small MLP (65 -> 128 -> 128 -> 1, tanh-GELU) maps cheap features of each rotated column -- the log energy
fractions of UY^2 over 32 equal-count bins of the ascending spectrum, the log mean eigenvalue per bin, log Neff --
to a proposed log delta.  The exact refinement then starts there: a proposal inside the FP32 grid argmin's basin
splits it, the half holding the stationary point is confirmed by one derivative sign, and the fast fit's
safeguarded Newton iteration runs in that half from the proposal; columns where that fails take the grid
refinement unchanged (csrc/flmm_delta_learned.cu).  The proposal therefore changes how many evaluations a column
needs, not the answer: results equal the grid path's to the Newton tolerance.

The weights (``delta_mlp.npz`` beside this file) are produced by ``python -m fasterlmm_gb300.learned train`` on a
GB300: seeded synthetic datasets (N from 300 to 2,000, 1 to 6 covariates, h2 uniform on [0, 0.95], 0 to 100 causal
variants, each phenotype plus one permuted copy), labels from the exact fit on a 200-point grid, trained in BF16
with FP32 master weights.
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


def fit_delta_learned(s: Tensor, UYt: Tensor, *, n_grid: int = 64, log_delta_min: float = -10.0,
                      log_delta_max: float = 10.0, refine: bool = True, model: DeltaMLP | None = None,
                      stats: dict | None = None) -> tuple[Tensor, Tensor]:
    """
    Fast delta fit with the learned proposal: (log_delta (P,), grid index (P,)), same contract as
    fast.fit_delta_fast.  ``stats``, if given, receives the number of columns that fell back to the grid path.
    """
    from .fast import fit_delta_fast
    dev = s.device
    ld_grid, idx = fit_delta_fast(s, UYt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max,
                                  refine=False)
    if not refine or UYt.shape[1] < 32:
        if refine:  # too few samples for the features: the grid refinement
            return fit_delta_fast(s, UYt, n_grid=n_grid, log_delta_min=log_delta_min, log_delta_max=log_delta_max)
        return ld_grid, idx
    model = model or DeltaMLP.load(dev)
    st = _stream(dev)
    P, Neff = UYt.shape
    x = propose_t(features_t(s, UYt), model, log_delta_min, log_delta_max)
    grid = torch.empty(n_grid, dtype=F64, device=dev)
    _lib.call("flmm_delta_grid_nodes", float(log_delta_min), float(log_delta_max), n_grid, _ptr(grid), st)
    ld = torch.empty(P, dtype=F64, device=dev)
    nfb = torch.zeros(1, dtype=torch.int32, device=dev)
    _lib.call("flmm_newton_from_proposal", _ptr(s), Neff, _ptr(UYt), UYt.stride(0), P, _ptr(grid), n_grid, _ptr(idx),
              _ptr(x), _ptr(ld), _ptr(nfb), st)
    if stats is not None:
        stats["fallback"] = nfb
    return ld, idx


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


def train(out: Path, *, n_sets: int = 48, steps: int = 4000, seed: int = 20240601) -> dict:
    """Train the proposal MLP (BF16 autocast, FP32 master weights) and write its weights to ``out``."""
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
    Xt = torch.from_numpy((X - mu) / sd).float().to(dev)
    yt = torch.from_numpy(y).float().to(dev)
    torch.manual_seed(seed)
    net = torch.nn.Sequential(torch.nn.Linear(N_FEATURES, 128), torch.nn.GELU(approximate="tanh"),
                              torch.nn.Linear(128, 128), torch.nn.GELU(approximate="tanh"),
                              torch.nn.Linear(128, 1)).to(dev)
    opt = torch.optim.AdamW(net.parameters(), lr=2e-3, weight_decay=1e-4)
    sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps)
    tr_t = torch.from_numpy(tr).to(dev)
    for step in range(steps):
        b = tr_t[torch.randint(0, tr_t.numel(), (2048,), device=dev)]
        with torch.autocast("cuda", dtype=torch.bfloat16):
            pred = net(Xt[b]).squeeze(1)
        loss = torch.nn.functional.smooth_l1_loss(pred.float(), yt[b], beta=0.1)
        opt.zero_grad(set_to_none=True)
        loss.backward()
        opt.step()
        sched.step()
    with torch.no_grad():
        pv = net(Xt[torch.from_numpy(val).to(dev)]).squeeze(1).float()
        err = (pv - yt[torch.from_numpy(val).to(dev)]).abs().cpu().numpy()
    W1 = net[0].weight.detach().float().cpu().numpy() / sd[None, :]  # fold the input standardisation into layer 1
    b1 = net[0].bias.detach().float().cpu().numpy() - W1 @ mu
    info = {"samples": int(n), "train_s": time.time() - t0, "data_s": t_data,
            "val_abs_err_median": float(np.median(err)), "val_abs_err_p90": float(np.quantile(err, 0.9)),
            "val_within_0.1": float((err < 0.1).mean())}
    np.savez(out, W1=W1.astype(np.float32), b1=b1.astype(np.float32),
             W2=net[2].weight.detach().float().cpu().numpy(), b2=net[2].bias.detach().float().cpu().numpy(),
             w3=net[4].weight.detach().float().cpu().numpy()[0], b3=np.float32(net[4].bias.item()),
             info=json.dumps(info))
    return info


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description="train the learned delta proposal")
    ap.add_argument("cmd", choices=["train"])
    ap.add_argument("--out", default=str(WEIGHTS))
    ap.add_argument("--sets", type=int, default=48)
    ap.add_argument("--steps", type=int, default=4000)
    args = ap.parse_args(argv)
    from . import build
    build()
    print(json.dumps(train(Path(args.out), n_sets=args.sets, steps=args.steps)), flush=True)


if __name__ == "__main__":
    main()
