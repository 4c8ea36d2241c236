"""
GPU parity of the split-precision low-rank scan (fasterlmm_gb300.lowrank_fast) against the reference's own FP64 runs:
the 100-sample fixture of the reference's k >= N branch (tests/golden/lowrank_loco.npz) and the 2,000-sample
fixture of its k < N branch with strong single-variant signals (tests/golden/lowrank_n2000.npz, made by
tests/golden/make_lowrank_golden.py; inputs regenerated by tests/strong_inputs.py).

Gates: beta and SE within rtol 1e-5 / atol 1e-6, nullh2 within 1e-5, |d(-log10 p)| <= 5e-4 on every real test and
on the genome maxima of the other columns; and int8 dosages streamed block by block from pinned host memory give
the bits of the resident path.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from conftest import GOLDEN, z_float
from parity import GATE, neg_log10_p_gpu
from strong_inputs import LR2000, genotype_checksum, lowrank_dataset

pytestmark = pytest.mark.gpu


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _check(res, g, df2, prefix="", label=""):
    got = {k: getattr(res, k).cpu().numpy() for k in ("f", "beta", "se", "sfve", "nullh2", "max_F")}
    for k in ("beta", "se"):
        np.testing.assert_allclose(got[k], g[prefix + k], rtol=1e-5, atol=1e-6, err_msg=f"{label} {k}")
    np.testing.assert_allclose(got["nullh2"], g[prefix + "nullh2"], rtol=1e-5, atol=1e-6, err_msg=f"{label} nullh2")
    for k in ("f", "max_F"):
        e = np.abs(neg_log10_p_gpu(got[k], df2) - neg_log10_p_gpu(g[prefix + k], df2))
        assert e.max() <= GATE, f"{label} {k}: |d(-log10 p)| {e.max():.2e} (max F {g[prefix + k].max():.0f})"
    return got


def test_lowrank_fast_k_ge_n_fixture(golden):
    from fasterlmm_gb300 import build, lowrank_fast
    build()
    g = golden("lowrank_loco")
    Zs = orc.standardise_columns(z_float(g["G"]))
    Gs = orc.standardise_columns(z_float(g["G_kin"]))
    B = int(g["n_real"])
    N, D = g["X"].shape
    res = lowrank_fast.loco_scan_lowrank_fast(_t(Gs), g["chrom_kin"], _t(Zs), g["chrom"], _t(g["X"]), _t(g["Y_all"]),
                                              n_real=B)
    _check(res, g, N - D - 1, label="LOCO")
    res1 = lowrank_fast.single_k_scan_lowrank_fast(_t(Gs), _t(Zs), _t(g["X"]), _t(g["Y_all"]), n_real=B)
    _check(res1, g, N - D - 1, prefix="sk_", label="single-K")


@pytest.fixture(scope="module")
def lr2000():
    c = LR2000
    with np.load(GOLDEN / "lowrank_n2000.npz") as z:
        want = {k: z[k] for k in z.files}
    G, X, Y, chrom, Gk, chrom_kin = lowrank_dataset(c)
    assert genotype_checksum(G) == int(want["g_checksum"]) and genotype_checksum(Gk) == int(want["gk_checksum"])
    np.testing.assert_allclose(Y, want["Y"], rtol=0, atol=1e-12)
    return c, G, X, Y, chrom, Gk, chrom_kin, want


def test_lowrank_fast_k_lt_n_strong_signals(lr2000):
    from fasterlmm_gb300 import build, lowrank_fast
    build()
    c, G, X, Y, chrom, Gk, chrom_kin, want = lr2000
    Zs = orc.standardise_columns(G.astype(np.float64))
    Gs = orc.standardise_columns(Gk.astype(np.float64))
    B, N, D = int(want["n_real"]), c["N"], c["D"]
    res = lowrank_fast.loco_scan_lowrank_fast(_t(Gs), chrom_kin, _t(Zs), chrom, _t(X), _t(Y), n_real=B)
    got = _check(res, want, N - D - 1, label="LOCO N=2000")
    assert want["f"].max() > 1000
    for j in range(B):  # each phenotype's ten strongest variants in order, up to ties within the gate
        gp = neg_log10_p_gpu(got["f"][:, j], N - D - 1)
        wp = neg_log10_p_gpu(want["f"][:, j], N - D - 1)
        tg, tw = np.argsort(-gp, kind="stable")[:10], np.argsort(-wp, kind="stable")[:10]
        d = tg != tw
        assert np.all(np.abs(wp[tg[d]] - wp[tw[d]]) <= GATE), j
    res1 = lowrank_fast.single_k_scan_lowrank_fast(_t(Gs), _t(Zs), _t(X), _t(Y), n_real=B)
    _check(res1, want, N - D - 1, prefix="sk_", label="single-K N=2000")


def test_streamed_dosage_blocks_match_resident(lr2000):
    """int8 dosages in pinned host memory, copied block by block on a side stream and standardised on the device,
    give the bits of the resident FP64 path (blocks of 512 split every chromosome)."""
    from fasterlmm_gb300 import build, lowrank_fast
    from fasterlmm_gb300.core import transpose
    build()
    c, G, X, Y, chrom, Gk, chrom_kin, _ = lr2000
    dev = torch.device("cuda", 0)
    Gs = orc.standardise_columns(Gk.astype(np.float64))
    B = len(c["specs"])
    Gt_host = torch.from_numpy(np.ascontiguousarray(G.T)).pin_memory()
    rows_of = {int(ch): np.flatnonzero(chrom == ch) for ch in np.unique(chrom)}
    chroms = sorted(rows_of)
    src = lowrank_fast.dosage_blocks(Gt_host, rows_of, dev, block=512)
    a = lowrank_fast.loco_scan_blocks_fast(_t(Gs), chrom_kin, src, G.shape[1], chroms, _t(X), _t(Y), n_real=B)
    Zt = torch.empty((G.shape[1], G.shape[0]), dtype=torch.float64, device=dev)
    from fasterlmm_gb300 import _lib
    Gt_dev = Gt_host.to(dev)
    _lib.call("flmm_standardise_dosage", Gt_dev.data_ptr(), G.shape[0], G.shape[0], G.shape[1], Zt.data_ptr(),
              G.shape[0], None)
    b = lowrank_fast.loco_scan_blocks_fast(_t(Gs), chrom_kin, lowrank_fast.resident_blocks(Zt, chrom, block=512),
                                           G.shape[1], chroms, _t(X), _t(Y), n_real=B)
    torch.cuda.synchronize()
    for k in ("f", "beta", "se", "sfve", "nullh2", "max_F"):
        np.testing.assert_array_equal(getattr(a, k).cpu().numpy(), getattr(b, k).cpu().numpy(), err_msg=k)
