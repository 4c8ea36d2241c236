"""
The oracle's restatement of the batched epistasis Wald (LUX tier 2) against the reference's own outputs
(tests/golden/epi_batched.npz, made by tests/golden/make_epi_golden.py).  CPU only.

The "collinear" cases plant test columns that copy the anchor column (exactly, or up to 1e-3 noise); there
sWs - quad is rounding noise, so beta, SE and (without the guard) F are meaningless in any implementation and are
not compared; with the guard on, F is 0 there in both.
"""
from __future__ import annotations

import numpy as np
import pytest

import flmm_oracle as orc

CASES = {"generic": 0, "collinear": 3, "collinear_noguard": 3, "wide": 0}


def compare_epi(case, g, beta, se, F, max_f, arg, *, rtol, atol_b=1e-12, atol_f=1e-10):
    get = lambda k: g[f"{case}/{k}"]
    planted = CASES[case]
    ok = np.s_[:, planted:, :]
    np.testing.assert_allclose(beta[ok], get("out_beta")[ok], rtol=rtol, atol=atol_b, err_msg="beta")
    np.testing.assert_allclose(se[ok], get("out_se")[ok], rtol=rtol, atol=atol_b, err_msg="se")
    if float(get("floor")) > 0:
        np.testing.assert_allclose(F, get("out_chi2"), rtol=rtol, atol=atol_f, err_msg="F")
        np.testing.assert_allclose(max_f, get("out_max_f"), rtol=rtol, atol=atol_f, err_msg="max F")
        np.testing.assert_array_equal(arg, get("out_argmax"))
    else:
        np.testing.assert_allclose(F[ok], get("out_chi2")[ok], rtol=rtol, atol=atol_f, err_msg="F")
        # where the reference's maximum is a regular column, it is the maximum over the regular columns
        keep = np.isfinite(get("out_max_f")) & (get("out_argmax") >= planted)
        Fr = F[:, planted:, :]
        np.testing.assert_allclose(Fr.max(axis=1)[keep], get("out_max_f")[keep], rtol=rtol, atol=atol_f,
                                   err_msg="max F")
        np.testing.assert_array_equal((Fr.argmax(axis=1) + planted)[keep], get("out_argmax")[keep])


@pytest.mark.parametrize("case", list(CASES))
def test_epi_oracle_matches_reference(golden, case):
    g = golden("epi_batched")
    get = lambda k: g[f"{case}/{k}"]
    with np.errstate(over="ignore", divide="ignore", invalid="ignore"):
        out = orc.epi_wald_batched(get("s"), get("X"), get("Y"), get("ld"), get("S"), n_real=int(get("n_real")),
                                   denom_floor_rel=float(get("floor")))
    compare_epi(case, g, *out, rtol=1e-8)
