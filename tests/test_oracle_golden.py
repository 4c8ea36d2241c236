"""
Pin the CPU oracle (oracle/flmm_oracle.py) to the reference's own outputs in tests/golden/*.npz.

The fixtures were produced by the reference implementation (tests/golden/make_golden.py); the oracle is a numpy
restatement with its own summation order and LAPACK call.  Everything that does not go through the golden-section
search agrees to FP64 rounding; log delta is judged by loss equivalence (tests/parity.py) and the scan outputs by
the reference's parity tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import flmm_oracle as orc
from conftest import z_float
from parity import DETAIL, assert_log_delta_equivalent, assert_scan_close


def _close(a, b, rtol=1e-7, atol=1e-9):
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def _check_log_delta(res, ref_ld):
    for i, c in enumerate(sorted(res["log_delta"])):
        s, UY = res["spectra"][c]
        assert_log_delta_equivalent(res["log_delta"][c], ref_ld[i], s, UY)


def test_oracle_components(golden):
    g = golden("components")
    spec = orc.compat_rotate(g["K"], g["X"], g["Y"])
    _close(spec["s"], g["s"], atol=1e-10)
    _close(spec["Xpinv"], g["Xpinv"], atol=1e-12)
    # UY depends on the basis only through eigenvector signs: compare the sign-invariant squares and the loss
    _close(spec["UY"] ** 2, g["UY"] ** 2, atol=1e-10)
    grid = orc.delta_grid(64, -10.0, 10.0)
    _close(orc.profile_loss_compat(grid, spec["s"], spec["UY"]), g["grid_loss"], rtol=1e-12, atol=1e-9)
    ld_grid = orc.fit_delta_grid_compat(spec["s"], spec["UY"], refine=False)
    assert np.array_equal(ld_grid, g["log_delta_grid"])  # the grid argmin is exact
    ld = orc.fit_delta_grid_compat(spec["s"], spec["UY"])
    assert_log_delta_equivalent(ld, g["log_delta"], spec["s"], spec["UY"])
    res = orc.snp_wald_scan_compat(spec, g["log_delta"], g["Z_std"], n_real=4)
    for k in DETAIL + ("max_F",):
        _close(res[k], g[k])
        _close(res[k], g["tiled_" + k])  # the reference's tiled run (17-variant x 2-column chunks)


@pytest.mark.parametrize("name", ["loco_n150_m1500", "edge_intercept_only", "edge_rank_deficient"])
def test_oracle_perm_threshold(golden, name):
    g = golden(name)
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    seen = []
    res, pmf = orc.perm_threshold(z_float(g["G"]), g["X"], g["Y"], g["chrom"], range(B), n_perm=n_perm,
                                  on_chrom=lambda k, n: seen.append((k, n)), keep_spectra=True)
    n_chr = len(np.unique(g["chrom"]))
    assert seen == [(k + 1, n_chr) for k in range(n_chr)]
    _check_log_delta(res, g["log_delta"])
    assert_scan_close(res, g)
    assert_scan_close({"perm_max_F": pmf}, g, keys=("perm_max_F",))


def test_oracle_grid100(golden):
    g = golden("loco_n150_m1500_grid100")
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    N = g["G"].shape[0]
    orders = orc.perm_orders(N, range(B), n_perm)
    assert np.array_equal(orders, g["orders"].astype(np.int64))  # permutation index sets are bit-exact
    Y_all = orc.pack_perms(g["Y"][:, :B], orders)
    res = orc.loco_scan_compat(orc.standardise_columns(z_float(g["G"])), g["X"], Y_all, g["chrom"], n_real=B,
                               n_grid=100, log_delta_min=-5.0, log_delta_max=5.0, keep_spectra=True)
    _check_log_delta(res, g["log_delta"])
    assert_scan_close(res, g)


def test_oracle_post_scan(golden):
    g = golden("loco_n150_m1500")
    N, D = g["X"].shape
    df2 = N - D - 1
    _close(orc.f_sf(g["f"], df2), g["p"], rtol=1e-12, atol=0)
    _close(orc.neg_log10_p(g["f"], df2), g["neglog10p"], rtol=1e-12, atol=1e-12)
    thr = [orc.perm_quantile_threshold(g["perm_min_p"][b]) for b in range(g["f"].shape[1])]
    _close(np.asarray(thr), g["threshold"], rtol=1e-12, atol=0)


def test_oracle_kin_panel_and_single_k(golden):
    g = golden("kin_panel_single_k")
    B = g["f"].shape[1]
    n_perm = int(g["n_perm"])
    res, pmf = orc.perm_threshold(z_float(g["G"]), g["X"], g["Y"], g["chrom"], range(B), n_perm=n_perm,
                                  Z_kin_raw=z_float(g["G_kin"]), chrom_kin=g["chrom_kin"], keep_spectra=True)
    _check_log_delta(res, g["log_delta"])
    assert_scan_close(res, g)
    assert_scan_close({"perm_max_F": pmf}, g, keys=("perm_max_F",))
    res, pmf = orc.perm_threshold(z_float(g["G"]), g["X"], g["Y"], g["chrom"], range(B), n_perm=n_perm, loco=False)
    _check_log_delta({"log_delta": {0: res["log_delta"]}, "spectra": res["spectra"]}, g["sk_log_delta"])
    assert_scan_close(res, g, prefix="sk_")
    assert_scan_close({"perm_max_F": pmf}, g, keys=("perm_max_F",), prefix="sk_")
    with pytest.raises(ValueError):
        orc.loco_scan_compat(np.zeros((4, 4)), np.ones((4, 1)), np.zeros((4, 1)), np.arange(4), Z_kin=np.zeros((4, 4)))


def test_oracle_na_groups(golden):
    g = golden("na_groups")
    Z = z_float(g["G"])
    groups = orc.group_by_na(g["Y"], list(range(g["Y"].shape[1])))
    assert len(groups) == int(g["n_groups"])
    for gi, (keep, cols) in enumerate(groups):
        assert np.array_equal(keep, g[f"g{gi}_keep"]) and np.array_equal(cols, g[f"g{gi}_cols"])
        res, pmf = orc.perm_threshold(Z[keep], g["X"][keep], g["Y"][keep][:, cols], g["chrom"], range(len(cols)),
                                      n_perm=int(g["n_perm"]), seed_idx=cols)
        assert_scan_close(res, g, prefix=f"g{gi}_")
        assert_scan_close({"perm_max_F": pmf}, g, keys=("perm_max_F",), prefix=f"g{gi}_")


def test_group_by_na_host_logic_matches_reference_groups(golden):
    """The package's host grouping (no GPU needed) reproduces the reference's groups on its NA fixture."""
    from fasterlmm_gb300.groups import group_by_na
    g = golden("na_groups")
    groups = group_by_na(g["Y"], list(range(g["Y"].shape[1])))
    assert len(groups) == int(g["n_groups"])
    for gi, (keep, cols) in enumerate(groups):
        assert keep == g[f"g{gi}_keep"].tolist() and cols == g[f"g{gi}_cols"].tolist()
    # all-NaN column -> empty keep rows; a column without NaN -> every row
    Y = np.array([[1.0, np.nan], [2.0, np.nan], [3.0, np.nan]])
    assert group_by_na(Y, [0, 1]) == [([0, 1, 2], [0]), ([], [1])]


def test_oracle_plain_components(golden):
    """The plain GLS restatement against the reference's rotate / _profile_loss / fit_delta_grid / snp_wald_scan."""
    from parity import assert_log_delta_equivalent_gls
    g = golden("plain_components")
    spec = orc.rotate(g["K"], g["X"], g["Y"])
    _close(spec["s"], g["s"], atol=1e-10)
    # rotated data depend on the basis only through eigenvector signs
    _close(spec["X_rot"] ** 2, g["X_rot"] ** 2, atol=1e-10)
    _close(spec["Y_rot"] ** 2, g["Y_rot"] ** 2, atol=1e-10)
    s, Xr, Yr = g["s"], g["X_rot"], g["Y_rot"]
    grid = orc.delta_grid(64, -10.0, 10.0)
    _close(orc.profile_loss(grid, s, Xr, Yr), g["grid_loss_ml"], rtol=1e-10, atol=1e-8)
    _close(orc.profile_loss(grid, s, Xr, Yr, reml=True), g["grid_loss_reml"], rtol=1e-10, atol=1e-8)
    for reml, key in ((False, "ml"), (True, "reml")):
        assert np.array_equal(orc.fit_delta_grid(s, Xr, Yr, refine=False, reml=reml), g[f"log_delta_{key}_grid"])
        ld = orc.fit_delta_grid(s, Xr, Yr, reml=reml)
        assert_log_delta_equivalent_gls(ld, g[f"log_delta_{key}"], s, Xr, Yr, reml=reml)
    for i, dl in enumerate(g["nll_delta"]):
        for p in range(Yr.shape[1]):
            np.testing.assert_allclose(orc.nll_eval(float(dl), s, Xr, Yr[:, p]), g["nll"][i, p], rtol=1e-10)
    S_rot = g["U"].T @ g["Z_std"]
    res = orc.snp_wald_scan({"s": s, "X_rot": Xr, "Y_rot": Yr}, g["log_delta_ml"], S_rot, n_real=3)
    for k in DETAIL + ("max_F",):
        _close(res[k], g[k])
        _close(res[k], g["tiled_" + k])


def test_oracle_plain_loco_and_single_k(golden):
    g = golden("plain_loco")
    Zs = orc.standardise_columns(z_float(g["G"]))
    B = int(g["n_real"])
    seen = []
    res = orc.loco_scan(Zs, g["X"], g["Y_all"], g["chrom"], n_real=B, on_chrom=lambda k, n: seen.append(k))
    assert len(seen) == int(g["n_chrom_seen"])
    assert_scan_close(res, g)
    ref_ld = g["log_delta"]
    for i, c in enumerate(sorted(res["log_delta"])):
        assert np.abs(res["log_delta"][c] - ref_ld[i]).max() < 1e-3
    res1 = orc.single_k_scan(Zs, g["X"], g["Y_all"], n_real=B)
    assert_scan_close(res1, g, prefix="sk_")


def test_oracle_lowrank_components(golden):
    """Low-rank restatement vs the reference's lowrank_rotate / loss / fit / Wald, both rank branches."""
    g = golden("lowrank_components")
    for tag in ("lo", "hi"):
        spec = orc.lowrank_rotate(g[f"{tag}_G"], g["X"], g["Y"])
        assert spec["Neff"] == int(g[f"{tag}_Neff"])
        # In the k >= N branch the reference keeps eigenvalues above (1e-10)^2 / k, which admits O(1e-17) rounding
        # noise of the projected-out directions; how many such directions are kept varies with rounding, and a kept
        # noise direction (s ~ 0, weight 1 / delta) counts exactly like an off-rank one.  Compare the real spectrum
        # and the loss, which does not depend on that split.
        big, gbig = spec["s"] > 1e-12, g[f"{tag}_s"] > 1e-12
        _close(spec["s"][big], g[f"{tag}_s"][gbig], atol=1e-10)
        _close(spec["UY"][big] ** 2, g[f"{tag}_UY"][gbig] ** 2, atol=1e-10)
        grid = orc.delta_grid(64, -10.0, 10.0)
        for s_, UY_, UUY_ in ((spec["s"], spec["UY"], spec["UUY"]), (g[f"{tag}_s"], g[f"{tag}_UY"], g[f"{tag}_UUY"])):
            _close(orc.profile_loss_lowrank(grid, s_, UY_, (UUY_ ** 2).sum(axis=0), spec["Neff"]),
                   g[f"{tag}_grid_loss"], rtol=1e-10, atol=1e-9)
        ref = {**spec, "s": g[f"{tag}_s"], "UY": g[f"{tag}_UY"], "UUY": g[f"{tag}_UUY"]}
        assert np.array_equal(orc.fit_delta_grid_lowrank(ref, refine=False), g[f"{tag}_log_delta_grid"])
        ld = orc.fit_delta_grid_lowrank(ref)
        assert np.abs(ld - g[f"{tag}_log_delta"]).max() < 1e-3
        res = orc.snp_wald_scan_lowrank(spec, g[f"{tag}_log_delta"], g["S"], n_real=2)
        for k in DETAIL + ("max_F",):
            _close(res[k], g[f"{tag}_{k}"])


def test_oracle_lowrank_loco_single_k_and_resident(golden):
    g = golden("lowrank_loco")
    Z = orc.standardise_columns(z_float(g["G"]))
    G = orc.standardise_columns(z_float(g["G_kin"]))
    B = int(g["n_real"])
    seen = []
    res = orc.loco_scan_lowrank(G, g["chrom_kin"], Z, g["chrom"], g["X"], g["Y_all"], n_real=B,
                                on_chrom=lambda k, n: seen.append(k))
    assert seen == list(range(1, len(np.unique(g["chrom"])) + 1))
    assert_scan_close(res, g)
    assert_scan_close(res, g, prefix="res64_")  # the reference's resident block engine gives the same scan
    res1 = orc.single_k_scan_lowrank(G, Z, g["X"], g["Y_all"], n_real=B)
    assert_scan_close(res1, g, prefix="sk_")
