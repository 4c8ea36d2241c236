"""
GPU tests of the split products' kernel forms and tile orders (flmm_tc_config): every CTA-pair / single-CTA form and
every raster group gives the default's results bit for bit, and the autotuner records the shapes it tuned.
"""
from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu
DEV = "cuda"
CHOICES = [(1, 1), (1, 2), (1, 3), (1, 8), (0, 1), (0, 2), (0, 4)]


@pytest.fixture(autouse=True)
def _restore_mode():
    from fasterlmm_gb300 import _lib, build
    build()
    yield
    _lib.tc_config(1)  # the library's initial mode


def test_split_gemm_bits_do_not_depend_on_kernel_form_or_tile_order():
    from fasterlmm_gb300 import _lib
    from fasterlmm_gb300.fast import SplitRows, gemm_split
    g = torch.Generator().manual_seed(3)
    Mr, Nr, K = 1000, 700, 995  # 4 x 6 pair tiles, 8 x 6 single-CTA tiles
    A = SplitRows.of(torch.randn(Mr, K, generator=g, dtype=torch.float64).to(DEV))
    B = SplitRows.of(torch.randn(Nr, K, generator=g, dtype=torch.float64).to(DEV))
    ctx = _lib.context(0)

    def run():
        C = torch.full((Mr, Nr), float("nan"), dtype=torch.float32, device=DEV)
        gemm_split(ctx, A.view(), B.view(), C)
        return C

    _lib.tc_config(0)
    ref = run()
    assert torch.isfinite(ref).all()
    for pair, group in CHOICES:
        _lib.tc_config(2, pair, group)
        assert torch.equal(run(), ref), (pair, group)
    _lib.tc_config(1)
    assert torch.equal(run(), ref)
    tuned = [r for r in _lib.autotune_report() if r["kernel"] == "gemm" and (r["rows"], r["cols"], r["K"]) == (Mr, Nr, K)]
    assert len(tuned) == 1 and tuned[0]["ms"] > 0 and tuned[0]["ms"] <= tuned[0]["default_ms"] + 1e-9
    _lib.call("flmm_context_check", ctx, None)


def test_fused_wald_bits_do_not_depend_on_kernel_form_or_tile_order():
    """A fast-form scan whose chromosomes span several variant tiles, under every choice and the autotuner."""
    from fasterlmm_gb300 import _lib, perms
    from fasterlmm_gb300.synth import make_dataset
    d = make_dataset(200, 1400, 2, 3, 60, seed=8, config_id=23, k_lo=1, k_hi=8)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(DEV)
    data = SimpleNamespace(Z=t(d.Z_float()), X=t(d.X), Y=t(d.Y), chrom=d.chrom, Z_kin=None, chrom_kin=None)

    def scan():
        res, pmf = perms.perm_threshold(data, list(range(60)), n_perm=5, form="fast")
        return {k: getattr(res, k).cpu().numpy() for k in ("f", "beta", "se", "sfve", "max_F")} | {"pmf": pmf.cpu().numpy()}

    _lib.tc_config(0)
    ref = scan()
    for pair, group in CHOICES:
        _lib.tc_config(2, pair, group)
        got = scan()
        for k in ref:
            np.testing.assert_array_equal(got[k], ref[k], err_msg=f"{k} pair={pair} group={group}")
    _lib.tc_config(1)
    got = scan()
    for k in ref:
        np.testing.assert_array_equal(got[k], ref[k], err_msg=k)
    assert any(r["kernel"] == "wald" and r["cols"] == 700 for r in _lib.autotune_report())
