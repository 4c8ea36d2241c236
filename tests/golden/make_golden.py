"""
Generate the golden fixtures in tests/golden/ by running the reference implementation itself.

Usage (in a checkout where the reference is present):
    python tests/golden/make_golden.py [--reference PATH]

The reference (the ``fasterlmm`` package, v1.6.2) is imported from PATH (default: the FASTERLMM_REFERENCE
environment variable).  Its modules ``fasterlmm.io`` and ``fasterlmm.normalize`` import pandas at module top
although the scan path never calls it; when pandas is not installed an empty stand-in package is put on sys.path
for the import.  Nothing in the reference is modified: the per-chromosome log delta, which the reference computes
but does not return, is observed by wrapping ``fasterlmm.core.fit_delta_grid_compat`` for the duration of a call.

Each fixture holds the seeded synthetic inputs (int8 genotypes, covariates, phenotypes, chromosome labels) and the
reference's FP64 outputs.  The files are small (a few MB in total) so they travel with the repository; the GPU
tests read them without needing the reference.
"""

from __future__ import annotations

import argparse
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "fast-er-lmm_gb300"))

from fasterlmm_gb300.synth import make_dataset, make_workload  # noqa: E402


def _import_reference(path: str):
    try:
        import pandas  # noqa: F401
    except ImportError:
        stub = Path(tempfile.mkdtemp()) / "pandas"
        stub.mkdir()
        (stub / "__init__.py").write_text("")
        sys.path.insert(0, str(stub.parent))
    sys.path.insert(0, path)
    import torch
    import fasterlmm.core as core
    import fasterlmm.io as fio
    import fasterlmm.perms as perms
    torch.set_num_threads(max(1, os.cpu_count() or 1))
    return core, fio, perms, torch


class _DeltaRecorder:
    """Wraps core.fit_delta_grid_compat to record each call's output (one call per chromosome)."""

    def __init__(self, core):
        self.core = core
        self.orig = core.fit_delta_grid_compat
        self.calls = []

    def __enter__(self):
        def wrapped(spec, **kw):
            out = self.orig(spec, **kw)
            self.calls.append((spec.s.clone(), out.clone()))
            return out
        self.core.fit_delta_grid_compat = wrapped
        return self

    def __exit__(self, *exc):
        self.core.fit_delta_grid_compat = self.orig


def _dataset(fio, torch, d, Z_kin=None, chrom_kin=None):
    Zf = d.Z_float()
    return fio.AlignedDataset(iid=[str(i) for i in range(Zf.shape[0])], Z=torch.from_numpy(Zf),
                              Y=torch.from_numpy(d.Y.copy()), X=torch.from_numpy(d.X.copy()), chrom=d.chrom,
                              pos=np.arange(Zf.shape[1]), snp_id=[str(i) for i in range(Zf.shape[1])],
                              pheno_names=[f"p{i}" for i in range(d.Y.shape[1])],
                              Z_kin=None if Z_kin is None else torch.from_numpy(Z_kin), chrom_kin=chrom_kin)


def _res_dict(res, prefix=""):
    return {prefix + k: getattr(res, k).numpy() for k in ("f", "beta", "se", "sfve", "nullh2", "max_F")}


def _perm_case(core, fio, perms, torch, d, pheno_idx, n_perm, *, loco=True, seed=19930909, seed_idx=None,
               Z_kin=None, chrom_kin=None):
    data = _dataset(fio, torch, d, Z_kin, chrom_kin)
    with _DeltaRecorder(core) as rec:
        res, pmf = perms.perm_threshold(data, list(pheno_idx), n_perm=n_perm, seed=seed, loco=loco,
                                        seed_idx=seed_idx)
    out = _res_dict(res)
    out["perm_max_F"] = pmf.numpy()
    out["log_delta"] = np.stack([c[1].numpy() for c in rec.calls])
    out["s_chrom"] = np.concatenate([c[0].numpy() for c in rec.calls])
    return out


def _scipy_post(out, df2, B):
    import scipy.stats as ss
    p = ss.f.sf(out["f"], 1, df2)
    pmin = ss.f.sf(out["perm_max_F"], 1, df2)
    thr = np.array([np.quantile(pmin[b], 0.05) for b in range(B)]) if pmin.shape[1] > 0 else np.zeros(B)
    return {"p": p, "perm_min_p": pmin, "threshold": thr, "neglog10p": -ss.f.logsf(out["f"], 1, df2) / np.log(10)}


def _inputs(d):
    return {"G": d.G, "X": d.X, "Y": d.Y, "chrom": d.chrom}


class _PlainDeltaRecorder:
    """Wraps core.fit_delta_grid (the plain LOCO loop calls it once per chromosome) to record its outputs."""

    def __init__(self, core):
        self.core = core
        self.orig = core.fit_delta_grid
        self.calls = []

    def __enter__(self):
        def wrapped(spec, **kw):
            out = self.orig(spec, **kw)
            self.calls.append(out.clone())
            return out
        self.core.fit_delta_grid = wrapped
        return self

    def __exit__(self, *exc):
        self.core.fit_delta_grid = self.orig


def _plain_fixtures(core, fio, torch):
    """The plain GLS path (fasterlmm/core.py:89-451): components, the LOCO driver and the single-K driver."""
    # components on a toy single-K problem: rotation, ML / REML grid losses, fits, GLS Wald, nLLeval
    rng = np.random.default_rng(78)
    Nt, Mt, Pt = 48, 160, 5
    Zc = fio.standardise_columns(torch.from_numpy(rng.normal(size=(Nt, Mt))))
    Kc = (Zc @ Zc.T) / Mt
    Xc = torch.from_numpy(np.concatenate([np.ones((Nt, 1)), rng.normal(size=(Nt, 2))], axis=1))
    Yc = torch.from_numpy(rng.normal(size=(Nt, Pt)))
    spec = core.rotate(Kc, Xc, Yc)
    grid = torch.linspace(-10.0, 10.0, 64, dtype=torch.float64)
    ld_ml = core.fit_delta_grid(spec)
    ld_ml_grid = core.fit_delta_grid(spec, refine=False)
    ld_reml = core.fit_delta_grid(spec, reml=True)
    ld_reml_grid = core.fit_delta_grid(spec, refine=False, reml=True)
    S_rot = spec.U.T @ Zc
    wres = core.snp_wald_scan(spec, ld_ml, S_rot, n_real=3)
    wres_t = core.snp_wald_scan(spec, ld_ml, S_rot, n_real=3, snp_chunk=23, pheno_chunk=2)
    nll_d = np.array([0.05, 1.0, 7.5])
    nll = np.array([[core.nLLeval(float(dl), spec.s, spec.X_rot, spec.Y_rot[:, p]).item() for p in range(Pt)]
                    for dl in nll_d])
    np.savez_compressed(HERE / "plain_components.npz", Z_std=Zc.numpy(), K=Kc.numpy(), X=Xc.numpy(), Y=Yc.numpy(),
                        s=spec.s.numpy(), X_rot=spec.X_rot.numpy(), Y_rot=spec.Y_rot.numpy(), U=spec.U.numpy(),
                        grid_loss_ml=core._profile_loss(grid, spec.s, spec.X_rot, spec.Y_rot).numpy(),
                        grid_loss_reml=core._profile_loss(grid, spec.s, spec.X_rot, spec.Y_rot, reml=True).numpy(),
                        log_delta_ml=ld_ml.numpy(), log_delta_ml_grid=ld_ml_grid.numpy(),
                        log_delta_reml=ld_reml.numpy(), log_delta_reml_grid=ld_reml_grid.numpy(),
                        nll_delta=nll_d, nll=nll, **_res_dict(wres), **_res_dict(wres_t, "tiled_"))

    # the LOCO driver on real columns followed by permuted copies (n_real split), and the single-K driver
    d = make_dataset(120, 900, 6, 3, 6, seed=31337, config_id=8, k_lo=2, k_hi=10)
    B, n_perm = 6, 3
    N = d.X.shape[0]
    orders = np.stack([np.random.default_rng([19930909, b]).random((n_perm, N)).argsort(axis=1) for b in range(B)])
    y_real = d.Y[:, :B]
    Y_all = np.concatenate([y_real] + [y_real[orders[b, k], b][:, None] for b in range(B) for k in range(n_perm)],
                           axis=1)
    Z_std = fio.standardise_columns(torch.from_numpy(d.Z_float()))
    X = torch.from_numpy(d.X.copy())
    seen = []
    with _PlainDeltaRecorder(core) as rec:
        res = core.loco_scan(Z_std, X, torch.from_numpy(Y_all), d.chrom, n_real=B, on_chrom=lambda k, n: seen.append(k))
    res1 = core.single_k_scan(Z_std, X, torch.from_numpy(Y_all), n_real=B)
    np.savez_compressed(HERE / "plain_loco.npz", **_inputs(d), Y_all=Y_all, n_real=B, **_res_dict(res),
                        log_delta=np.stack([c.numpy() for c in rec.calls]), n_chrom_seen=len(seen),
                        **_res_dict(res1, "sk_"))


def _lowrank_fixtures(ref_path, fio, torch):
    """The low-rank path (fasterlmm/lowrank.py) and its resident block engine (fasterlmm/extreme_scan.py)."""
    import fasterlmm.lowrank as lr
    import fasterlmm.extreme_scan as xs
    rng = np.random.default_rng(91)
    # components: k < N (the k x k Gram branch) and k >= N (the N x N branch)
    Nt, Pt = 90, 4
    Xc = torch.from_numpy(np.concatenate([np.ones((Nt, 1)), rng.normal(size=(Nt, 2))], axis=1))
    Yc = torch.from_numpy(rng.normal(size=(Nt, Pt)))
    S = fio.standardise_columns(torch.from_numpy(rng.integers(0, 3, size=(Nt, 70)).astype(np.float64)))
    out = {"X": Xc.numpy(), "Y": Yc.numpy(), "S": S.numpy()}
    for tag, k in (("lo", 40), ("hi", 120)):
        G = fio.standardise_columns(torch.from_numpy(rng.integers(0, 3, size=(Nt, k)).astype(np.float64)))
        spec = lr.lowrank_rotate(G, Xc, Yc)
        yy_off = (spec.UUY * spec.UUY).sum(dim=0)
        grid = torch.linspace(-10.0, 10.0, 64, dtype=torch.float64)
        ld = lr.fit_delta_grid_lowrank(spec)
        res = lr.snp_wald_scan_lowrank(spec, ld, S, n_real=2)
        out.update({f"{tag}_G": G.numpy(), f"{tag}_s": spec.s.numpy(), f"{tag}_UY": spec.UY.numpy(),
                    f"{tag}_UUY": spec.UUY.numpy(), f"{tag}_Neff": spec.Neff,
                    f"{tag}_grid_loss": lr._profile_loss_lowrank(grid, spec.s, spec.UY, yy_off, spec.Neff).numpy(),
                    f"{tag}_log_delta": ld.numpy(), f"{tag}_log_delta_grid": lr.fit_delta_grid_lowrank(spec, refine=False).numpy(),
                    **_res_dict(res, f"{tag}_")})
    np.savez_compressed(HERE / "lowrank_components.npz", **out)

    # LOCO over a pruned kinship factor, real + permuted columns, the single-K driver and the resident block
    # engine (FP64 and its FP32 default) with blocks that split chromosomes
    d = make_dataset(100, 700, 5, 3, 5, seed=777, config_id=9, k_lo=2, k_hi=8)
    dk = make_dataset(100, 300, 5, 1, 1, seed=778, config_id=10)
    B, n_perm = 5, 2
    N = d.X.shape[0]
    orders = np.stack([np.random.default_rng([19930909, b]).random((n_perm, N)).argsort(axis=1) for b in range(B)])
    y_real = d.Y[:, :B]
    Y_all = np.concatenate([y_real] + [y_real[orders[b, k], b][:, None] for b in range(B) for k in range(n_perm)],
                           axis=1)
    Z = fio.standardise_columns(torch.from_numpy(d.Z_float()))
    G = fio.standardise_columns(torch.from_numpy(dk.Z_float()))
    X = torch.from_numpy(d.X.copy())
    Yt = torch.from_numpy(Y_all)
    res = lr.loco_scan_lowrank(G, dk.chrom, Z, d.chrom, X, Yt, n_real=B)
    res1 = lr.single_k_scan_lowrank(G, Z, X, Yt, n_real=B)
    res64 = xs.loco_scan_resident(Z, d.chrom, G, dk.chrom, X, Yt, n_real=B, block_size=37, dtype=torch.float64)
    res32 = xs.loco_scan_resident(Z.float(), d.chrom, G, dk.chrom, X, Yt, n_real=B, block_size=37)
    np.savez_compressed(HERE / "lowrank_loco.npz", **_inputs(d), G_kin=dk.G, chrom_kin=dk.chrom, Y_all=Y_all,
                        n_real=B, **_res_dict(res), **_res_dict(res1, "sk_"), **_res_dict(res64, "res64_"),
                        **{k: v.astype(np.float32) for k, v in _res_dict(res32, "res32_").items()})


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    ap.add_argument("--only", choices=["compat", "plain", "lowrank"], default=None,
                    help="write only the compat-path, the plain-GLS or the low-rank fixtures")
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH (or set FASTERLMM_REFERENCE) to the reference checkout")
    core, fio, perms, torch = _import_reference(args.reference)
    if args.only in (None, "plain"):
        _plain_fixtures(core, fio, torch)
    if args.only in (None, "lowrank"):
        _lowrank_fixtures(args.reference, fio, torch)
    if args.only in ("plain", "lowrank"):
        return

    # 1. the 150 x 1,500 / 16-chromosome workload through perm_threshold, reference defaults (64-pt grid)
    d, w = make_workload("n150_m1500_b20_perm100")
    B, n_perm = w["B"], w["n_perm"]
    out = _perm_case(core, fio, perms, torch, d, range(B), n_perm)
    N, D = d.X.shape
    out.update(_scipy_post(out, N - D - 1, B))
    np.savez_compressed(HERE / "loco_n150_m1500.npz", **_inputs(d), n_perm=n_perm, **out)

    # 2. same data, the 100-point grid on [-5, 5]: the reference's LOCO loop (fasterlmm/core.py:707-726) driven
    #    with explicit fit_delta_grid_compat keywords, since loco_scan_compat does not forward them
    Zt = torch.from_numpy(d.Z_float())
    Z_std = fio.standardise_columns(Zt)
    X = torch.from_numpy(d.X)
    orders = np.empty((N, B, n_perm), dtype=np.int64)
    for b in range(B):
        rng = np.random.default_rng([19930909, b])
        orders[:, b, :] = rng.random((n_perm, N)).argsort(axis=1).T
    y_real = torch.from_numpy(d.Y[:, :B].copy())
    y_perms = torch.gather(y_real.unsqueeze(2).expand(N, B, n_perm), 0, torch.from_numpy(orders)).reshape(N, -1)
    Y_all = torch.cat([y_real, y_perms], dim=1)
    M = Zt.shape[1]
    maxF = torch.full((Y_all.shape[1],), float("-inf"), dtype=torch.float64)
    lds = []
    detail = {k: torch.zeros(M, B, dtype=torch.float64) for k in ("f", "beta", "se", "sfve", "nullh2")}
    for c in sorted(np.unique(d.chrom).tolist()):
        tm = d.chrom == c
        K = fio.grm(Z_std[:, d.chrom != c])
        spec = core.fastlmm_compat_rotate(K, X, Y_all)
        ld = core.fit_delta_grid_compat(spec, n_grid=100, log_delta_min=-5.0, log_delta_max=5.0)
        lds.append(ld.numpy())
        res = core.snp_wald_scan_compat(spec, ld, Z_std[:, tm], n_real=B)
        for k in detail:
            detail[k][tm, :] = getattr(res, k)
        maxF = torch.maximum(maxF, res.max_F)
    np.savez_compressed(HERE / "loco_n150_m1500_grid100.npz", **_inputs(d), n_perm=n_perm, orders=orders.astype(np.int16),
                        **{k: v.numpy() for k, v in detail.items()}, max_F=maxF.numpy(), log_delta=np.stack(lds))

    # 3. component fixtures: compat rotation, delta grid (refine on / off), Wald scan, on a toy single-K problem
    #    with an arbitrary 4-column design (the shape the reference's own unit tests use)
    rng = np.random.default_rng(77)
    Nt, Mt, Pt = 40, 150, 6
    Zc = fio.standardise_columns(torch.from_numpy(rng.normal(size=(Nt, Mt))))
    Kc = (Zc @ Zc.T) / Mt
    Xc = torch.from_numpy(np.concatenate([np.ones((Nt, 1)), rng.normal(size=(Nt, 3))], axis=1))
    Yc = torch.from_numpy(rng.normal(size=(Nt, Pt)))
    spec = core.fastlmm_compat_rotate(Kc, Xc, Yc)
    ld_ref = core.fit_delta_grid_compat(spec)
    ld_grid = core.fit_delta_grid_compat(spec, refine=False)
    grid_loss = core._profile_loss_compat(torch.linspace(-10.0, 10.0, 64, dtype=torch.float64), spec.s, spec.UY)
    wres = core.snp_wald_scan_compat(spec, ld_ref, Zc, n_real=4)
    wres_t = core.snp_wald_scan_compat(spec, ld_ref, Zc, n_real=4, snp_chunk=17, pheno_chunk=2)
    np.savez_compressed(HERE / "components.npz", Z_std=Zc.numpy(), K=Kc.numpy(), X=Xc.numpy(), Y=Yc.numpy(),
                        s=spec.s.numpy(), UY=spec.UY.numpy(), Xpinv=spec.Xpinv.numpy(), U_eff=spec.U_eff.numpy(),
                        log_delta=ld_ref.numpy(), log_delta_grid=ld_grid.numpy(), grid_loss=grid_loss.numpy(),
                        **_res_dict(wres), **_res_dict(wres_t, "tiled_"))

    # 4. missing data: genotype missing calls + 3 phenotype NA patterns, run the CLI's grouped path
    #    (fasterlmm/cli.py:351-375): per NA group a strain subset and perm_threshold with seed_idx
    d = make_dataset(120, 900, 6, 3, 9, seed=424242, config_id=3, geno_missing_rate=0.02, pheno_na_patterns=3,
                     k_lo=2, k_hi=8)
    Yt = torch.from_numpy(d.Y.copy())
    groups = fio.group_by_na(Yt, list(range(d.Y.shape[1])))
    data = _dataset(fio, torch, d)
    gout = {}
    for gi, (keep, cols) in enumerate(groups):
        sub = fio.subset_dataset(data, keep, cols)
        res, pmf = perms.perm_threshold(sub, list(range(len(cols))), n_perm=7, seed=19930909, seed_idx=cols)
        gout.update({f"g{gi}_{k}": v for k, v in _res_dict(res).items()})
        gout[f"g{gi}_perm_max_F"] = pmf.numpy()
        gout[f"g{gi}_keep"] = np.asarray(keep, dtype=np.int32)
        gout[f"g{gi}_cols"] = np.asarray(cols, dtype=np.int32)
    np.savez_compressed(HERE / "na_groups.npz", **_inputs(d), n_groups=len(groups), n_perm=7, **gout)

    # 5. separate kinship panel (Z_kin / chrom_kin) and the single-K branch
    d = make_dataset(90, 600, 5, 2, 4, seed=5150, config_id=4, k_lo=3, k_hi=6)
    dk = make_dataset(90, 800, 5, 2, 1, seed=6160, config_id=5)
    out = _perm_case(core, fio, perms, torch, d, range(4), 6, Z_kin=dk.Z_float(), chrom_kin=dk.chrom)
    out1 = _perm_case(core, fio, perms, torch, d, range(4), 6, loco=False)
    np.savez_compressed(HERE / "kin_panel_single_k.npz", **_inputs(d), G_kin=dk.G, chrom_kin=dk.chrom, n_perm=6,
                        **out, **{"sk_" + k: v for k, v in out1.items()})

    # 6. edge cases: intercept-only design, a monomorphic variant, a one-variant chromosome, one phenotype,
    #    no permutations; and a rank-deficient design (duplicated covariate) for the drop-D quirk
    d = make_dataset(64, 300, 4, 1, 1, seed=99, config_id=6, chrom_sizes=[1, 120, 100, 79], k_lo=2, k_hi=2)
    d.G[:, 5] = 1  # monomorphic: std 0 -> inf -> standardised column of zeros
    out = _perm_case(core, fio, perms, torch, d, [0], 0)
    np.savez_compressed(HERE / "edge_intercept_only.npz", **_inputs(d), n_perm=0, **out)
    d = make_dataset(64, 300, 3, 3, 2, seed=98, config_id=7, k_lo=2, k_hi=4)
    d.X[:, 2] = d.X[:, 1]  # rank(X) = 2 < D = 3
    out = _perm_case(core, fio, perms, torch, d, [0, 1], 3)
    np.savez_compressed(HERE / "edge_rank_deficient.npz", **_inputs(d), n_perm=3, **out)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
