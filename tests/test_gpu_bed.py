"""
GPU decode of PLINK .bed files (csrc/flmm_bed.cu) against the oracle's restatement of the format, and a streamed
low-rank scan fed from a .bed block by block against the resident scan of the same data.
"""
from __future__ import annotations

import numpy as np
import pytest
import torch

import flmm_oracle as orc
from parity import DETAIL

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from fasterlmm_gb300 import build
    build()


def _dataset_bed(tmp_path, N=201, M=1500, miss=0.02):
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(N, M, 4, 3, 6, seed=808, config_id=18, k_lo=1, k_hi=10, geno_missing_rate=miss)
    prefix = str(tmp_path / "geno")
    orc.write_bed(prefix, d.Z_float(), chrom=d.chrom)
    return d, prefix


@pytest.mark.parametrize("count_A1", [True, False])
def test_bed_decode_matches_format(tmp_path, count_A1):
    from fasterlmm_gb300 import bedio
    d, prefix = _dataset_bed(tmp_path)
    h = bedio.open_bed(prefix, count_A1=count_A1)
    got = bedio.read_dosages(h)
    ref = orc.read_bed(prefix, count_A1=count_A1)
    assert np.array_equal(np.isnan(got), np.isnan(ref)) and np.array_equal(np.nan_to_num(got), np.nan_to_num(ref))
    Zt = bedio.standardised_rows(h, np.arange(ref.shape[1])).cpu().numpy()
    np.testing.assert_allclose(Zt.T, orc.standardise_columns(ref), rtol=1e-12, atol=1e-12)
    # an aligned strain subset, rows in .fam order
    keep = [h.iid[i] for i in (199, 5, 77, 150, 0)]
    hs = bedio.open_bed(prefix, keep_iid=keep, count_A1=count_A1)
    rows = [0, 5, 77, 150, 199]
    assert hs.iid == [h.iid[i] for i in rows]
    sub = bedio.read_dosages(hs, [3, 999, 10])
    assert np.array_equal(np.nan_to_num(sub, nan=-7), np.nan_to_num(ref[rows][:, [3, 999, 10]], nan=-7))


def test_streamed_lowrank_scan_from_bed_equals_resident(tmp_path):
    from fasterlmm_gb300 import bedio, lowrank
    d, prefix = _dataset_bed(tmp_path)
    h = bedio.open_bed(prefix)
    Z = orc.standardise_columns(orc.read_bed(prefix))
    kin = np.arange(0, Z.shape[1], 7)                     # a strided kinship panel
    G = torch.from_numpy(Z[:, kin]).cuda()
    X, Y = torch.from_numpy(d.X).cuda(), torch.from_numpy(d.Y).cuda()
    chroms = sorted(np.unique(h.chrom).tolist())
    streamed = lowrank.loco_scan_blocks(lambda c: bedio.chrom_blocks(h, c, block_size=333), chroms, Z.shape[1], G,
                                        h.chrom[kin], X, Y, n_real=4, dtype=torch.float64, device=torch.device("cuda"))
    resident = lowrank.loco_scan_lowrank(G, h.chrom[kin], torch.from_numpy(Z).cuda(), h.chrom, X, Y, n_real=4)
    for k in DETAIL + ("max_F",):
        np.testing.assert_allclose(getattr(streamed, k).cpu().numpy(), getattr(resident, k).cpu().numpy(),
                                   rtol=1e-10, atol=1e-12, err_msg=k)
