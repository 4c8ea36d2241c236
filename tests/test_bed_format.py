"""
CPU checks of the PLINK .bed restatement in the oracle and of the package's .bim/.fam parsing (no GPU): the
encoder/decoder round trip, both allele conventions, ragged sample counts, missing calls, metadata.
"""
from __future__ import annotations

import numpy as np
import pytest

import flmm_oracle as orc


@pytest.mark.parametrize("N", [1, 4, 7, 130])
@pytest.mark.parametrize("count_A1", [True, False])
def test_bed_roundtrip(tmp_path, N, count_A1):
    rng = np.random.default_rng(N)
    G = rng.integers(0, 3, size=(N, 9)).astype(np.float64)
    G[rng.random(G.shape) < 0.1] = np.nan
    prefix = str(tmp_path / "x")
    orc.write_bed(prefix, G, count_A1=count_A1)
    back = orc.read_bed(prefix, count_A1=count_A1)
    assert np.array_equal(np.isnan(back), np.isnan(G))
    assert np.array_equal(np.nan_to_num(back, nan=-1), np.nan_to_num(G, nan=-1))
    # the other convention reads 2 - dosage
    other = orc.read_bed(prefix, count_A1=not count_A1)
    assert np.array_equal(np.nan_to_num(other, nan=-1), np.where(np.isnan(G), -1, 2 - G))


def test_bim_fam_metadata(tmp_path):
    from fasterlmm_gb300 import bedio
    prefix = str(tmp_path / "m")
    G = np.zeros((5, 3))
    orc.write_bed(prefix, G, chrom=[1, 2, 23], sid=["a", "b", "c"], pos=[10, 20, 30], iid=["p", "q", "r", "s", "t"])
    assert bedio.read_fam(prefix) == ["p", "q", "r", "s", "t"]
    bim = bedio.read_bim(prefix)
    assert bim["sid"] == ["a", "b", "c"] and np.array_equal(bim["chrom"], [1, 2, 23]) and np.array_equal(bim["pos"], [10, 20, 30])
    h = bedio.open_bed(prefix, keep_iid=["t", "q"])
    assert h.iid == ["q", "t"] and list(h.rows) == [1, 4] and h.shape == (2, 3)
    assert bedio._chrom_code("chrX") == 23.0 and bedio._chrom_code("MT") == 26.0
