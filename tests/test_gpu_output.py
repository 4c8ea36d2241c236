"""
GPU side of the output stage: the device p-value against scipy's f.sf, and write_batch (device post-scan step for
a whole batch, then the per-phenotype files) against the same files written from host-computed quantities.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_pvalue_matches_scipy():
    from scipy.stats import f as fdist
    from fasterlmm_gb300.post import pvalue
    rng = np.random.default_rng(3)
    F = np.concatenate([10.0 ** rng.uniform(-8, 4, 20000), [0.0, -1.0, np.nan, np.inf, 1e-300, 5.0, 3000.0]])
    for df2 in (3, 146, 993, 4999):
        got = pvalue(torch.from_numpy(F).cuda(), df2).cpu().numpy()
        want = fdist.sf(F, 1, df2)
        ok = want > 1e-290
        np.testing.assert_allclose(got[ok], want[ok], rtol=1e-11, atol=0)
        assert np.all(got[~ok & ~np.isnan(want)] < 1e-280)
        assert np.isnan(got[np.isnan(F)]).all()
        assert got[F == 0.0][0] == 1.0 and got[F == -1.0][0] == 1.0 and got[np.isinf(F)][0] == 0.0


def _scan(golden):
    from types import SimpleNamespace
    from fasterlmm_gb300 import perms
    from conftest import z_float
    g = golden("loco_n150_m1500")
    dev = torch.device("cuda")
    data = SimpleNamespace(Z=torch.from_numpy(z_float(g["G"])).to(dev), Y=torch.from_numpy(g["Y"]).to(dev),
                           X=torch.from_numpy(g["X"]).to(dev), chrom=g["chrom"], Z_kin=None, chrom_kin=None)
    B = g["Y"].shape[1]
    res, pmf = perms.perm_threshold(data, list(range(B)), n_perm=20, form="fast")
    return g, res, pmf


def test_write_batch_files(golden, tmp_path):
    from scipy.stats import f as fdist
    from fasterlmm_gb300.output import VariantTable, lambda_gc_host, write_batch, write_lambda_table
    g, res, pmf = _scan(golden)
    M, B = res.f.shape
    N, D = g["X"].shape
    df2 = N - D - 1
    rng = np.random.default_rng(5)
    ctx = VariantTable.of([f"v{i}" for i in range(M)], g["chrom"].astype(np.float64),
                          np.arange(M, dtype=np.float64) * 100.0, rng.uniform(0.1, 0.5, M), n_perm=20)
    p_var = g["Y"].var(axis=0)
    names = [f"ph{j}" for j in range(B)]
    rows = []
    write_batch(tmp_path, names, res, pmf, df2, ctx, p_var, per_pheno_dirs=True, lambda_rows=rows, threads=4)
    F = res.f.cpu().numpy()
    p_host = fdist.sf(F, 1, df2)
    pmin_host = fdist.sf(pmf.cpu().numpy(), 1, df2)
    for j, name in enumerate(names):
        lines = (tmp_path / name / "gwas.tsv").read_text().splitlines()
        assert lines[0].split("\t")[:6] == ["sid_index", "SNP", "Chr", "GenDist", "ChrPos", "PValue"]
        body = [ln.split("\t") for ln in lines[1:]]
        assert len(body) == M
        sid = np.array([int(r[0]) for r in body])
        pv = np.array([float(r[5]) for r in body])
        # rows: a permutation of the variants in ascending written p, ties in variant order, NaN last
        assert sorted(sid) == list(range(M))
        p_by_variant = np.empty(M)
        p_by_variant[sid] = pv
        np.testing.assert_array_equal(sid, np.argsort(p_by_variant, kind="stable"))
        np.testing.assert_allclose(pv, p_host[sid, j], rtol=1e-11)
        assert all(r[1] == f"v{s}" and r[3] == "" and r[10] == "0" and r[12] == name and r[13] == "21"
                   for r, s in zip(body, sid))
        np.testing.assert_array_equal(np.array([float(r[6]) for r in body]), res.beta[sid, j].cpu().numpy())
        thresh = float((tmp_path / name / "threshold.txt").read_text())
        np.testing.assert_allclose(thresh, np.quantile(pmin_host[j], 0.05), rtol=1e-6)  # "%.6e" text
        perms_txt = (tmp_path / name / "perms.tsv").read_text().splitlines()
        assert perms_txt[0] == "perm_min_p"
        np.testing.assert_allclose(np.array(perms_txt[1:], dtype=float), pmin_host[j], rtol=1e-11)
        lam = float((tmp_path / name / "lambda_gc.txt").read_text())
        np.testing.assert_allclose(lam, lambda_gc_host(p_host[:, j])[0], rtol=1e-6, atol=1e-6)
    assert sorted(r[0] for r in rows) == sorted(names)
    text = write_lambda_table(tmp_path, None, rows, {n: i for i, n in enumerate(names)}).read_text().splitlines()
    assert [t.split("\t")[0] for t in text[1:]] == names


def test_sharded_writes_match_the_unsharded_files(golden, tmp_path):
    """Each rank writing its own round-robin phenotypes' files (shard.write_shard, the reference's shard-worker
    layout, fasterlmm/cli.py:292) gives the same files, byte for byte, as one unsharded write of the whole batch:
    a phenotype's files depend on its own columns only."""
    from fasterlmm_gb300 import shard
    from fasterlmm_gb300.core import ScanResult
    from fasterlmm_gb300.output import VariantTable, write_batch
    g, res, pmf = _scan(golden)
    M, B = res.f.shape
    N, D = g["X"].shape
    df2 = N - D - 1
    rng = np.random.default_rng(7)
    ctx = VariantTable.of([f"v{i}" for i in range(M)], g["chrom"].astype(np.float64),
                          np.arange(M, dtype=np.float64) * 100.0, rng.uniform(0.1, 0.5, M), n_perm=20)
    p_var = g["Y"].var(axis=0)
    names = [f"ph{j}" for j in range(B)]
    whole = tmp_path / "whole"
    parts = tmp_path / "parts"
    write_batch(whole, names, res, pmf, df2, ctx, p_var, per_pheno_dirs=True, threads=4)
    for r in range(2):  # the two ranks of a world of two, one after the other
        mine = shard.shard_phenotypes(list(range(B)), r, 2)
        idx = torch.tensor(mine, device=res.f.device)
        cols = {k: getattr(res, k).index_select(1, idx) for k in ("f", "beta", "se", "sfve", "nullh2")}
        pmf_r = pmf.index_select(0, idx)
        res_r = ScanResult(max_F=torch.cat([cols["f"].max(dim=0).values, pmf_r.reshape(-1)]), **cols)
        shard.write_shard(parts, [names[j] for j in mine], res_r, pmf_r, df2, ctx, p_var[mine], per_pheno_dirs=True,
                          threads=4)
    for name in names:
        for f in ("gwas.tsv", "perms.tsv", "threshold.txt", "lambda_gc.txt"):
            assert (parts / name / f).read_bytes() == (whole / name / f).read_bytes(), (name, f)
