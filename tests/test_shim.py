"""
CPU test of the drop-in installer: it rebinds exactly the names the reference's callers look up (including the
copies imported by name into fasterlmm.perms and fasterlmm.cli) and restores them.  Uses stand-in modules.
"""
from __future__ import annotations

import types


def _fake(name, attrs):
    m = types.ModuleType(name)
    for a in attrs:
        setattr(m, a, object())
    return m


def test_install_and_uninstall_rebind_reference_names():
    from fasterlmm_gb300 import perms, shim
    from fasterlmm_gb300 import gls
    core = _fake("fasterlmm.core", ["loco_scan_compat", "single_k_scan_compat", "fastlmm_compat_rotate",
                                   "fit_delta_grid_compat", "snp_wald_scan_compat", "grm", "rotate", "fit_delta_grid",
                                   "snp_wald_scan", "loco_scan", "single_k_scan", "nLLeval", "_profile_loss",
                                   "Spectrum"])
    extreme = _fake("fasterlmm.extreme", ["Spectrum", "fit_delta_grid", "snp_wald_scan"])
    pmod = _fake("fasterlmm.perms", ["loco_scan_compat", "single_k_scan_compat", "perm_threshold"])
    cli = _fake("fasterlmm.cli", ["perm_threshold"])
    import sys
    sys.modules.update({"fasterlmm.core": core, "fasterlmm.perms": pmod, "fasterlmm.cli": cli})
    try:
        orig = (core.loco_scan_compat, pmod.perm_threshold, cli.perm_threshold, core.grm)
        orig_ext = extreme.fit_delta_grid
        patched = shim.install(form="fast", modules={"core": core, "perms": pmod, "cli": cli, "extreme": extreme})
        assert core.loco_scan is gls.loco_scan and core.nLLeval is gls.nLLeval and core.Spectrum is gls.Spectrum
        assert extreme.fit_delta_grid is gls.fit_delta_grid and "fasterlmm.extreme.snp_wald_scan" in patched
        assert "fasterlmm.perms.perm_threshold" in patched and "fasterlmm.cli.perm_threshold" in patched
        assert core.loco_scan_compat.keywords == {"form": "fast"}
        assert pmod.perm_threshold.func is perms.perm_threshold
        assert pmod.loco_scan_compat.keywords == {"form": "fast"}
        assert core.grm is orig[3]  # names outside the scan path are left alone
        shim.uninstall()
        assert (core.loco_scan_compat, pmod.perm_threshold, cli.perm_threshold) == orig[:3]
        assert extreme.fit_delta_grid is orig_ext
    finally:
        for k in ("fasterlmm.core", "fasterlmm.perms", "fasterlmm.cli"):
            sys.modules.pop(k, None)


def test_cli_writer_is_routed_through_output_module(golden, tmp_path):
    """With outputs=True the CLI's per-phenotype writer writes the reference's files through this package."""
    import numpy as np
    from fasterlmm_gb300 import build, shim
    build()
    g = golden("output_files")
    calls = []
    cli = types.ModuleType("fasterlmm.cli")
    cli._write_pheno = lambda *a, **k: calls.append(a)
    shim.install(form="fast", modules={"cli": cli}, outputs=True)
    try:
        M, n_perm = int(g["M"]), int(g["n_perm"])
        ctx = {"snp_id": list(g["snp"]), "chrom": g["chrom"], "pos": g["pos"], "g_var": g["g_var"],
               "sid_index": np.arange(M), "gendist": None, "mixing": np.zeros(M),
               "phenocount": np.full(M, 1 + n_perm), "pheno_idx": None, "lambda_rows": []}
        for j, name in enumerate(g["pheno"]):
            cli._write_pheno({**ctx}, str(tmp_path), str(name), p_col=g["p"][:, j], beta_col=g["beta"][:, j],
                             se_col=g["se"][:, j], sfve_col=g["sfve"][:, j], nullh2_col=g["nullh2"][:, j],
                             p_var=float(g["p_var"][j]), perm_min_p=g["perm_min_p"][j],
                             perm_quantile=float(g["perm_quantile"]), per_pheno_dirs=True, bundle_writer=None)
            for fname in ("gwas.tsv", "perms.tsv", "threshold.txt", "lambda_gc.txt"):
                assert (tmp_path / str(name) / fname).read_bytes() == bytes(g[f"file_{j}_{fname}"])
        assert [r[0] for r in ctx["lambda_rows"]] == [str(n) for n in g["pheno"]]
        cli._write_pheno({**ctx, "clump": {"z": None}}, str(tmp_path), "x", None, None, None, None, None, 1.0, None,
                         0.05, True, None)
        assert len(calls) == 1  # clumping goes to the original writer
    finally:
        shim.uninstall()
    assert not hasattr(cli._write_pheno, "__wrapped__") and cli._write_pheno(1) is None and len(calls) == 2


def test_lux_batched_wald_is_rebound():
    from fasterlmm_gb300 import epi, shim
    kern = _fake("fasterlmm_lux.epi._kernel", ["snp_wald_scan_batched"])
    scan = _fake("fasterlmm_lux.epi.scan", ["snp_wald_scan_batched", "scan_tier2"])
    orig = scan.snp_wald_scan_batched
    patched = shim.install(form="fast", modules={"lux_kernel": kern, "lux_scan": scan})
    try:
        assert scan.snp_wald_scan_batched is epi.snp_wald_scan_batched
        assert kern.snp_wald_scan_batched is epi.snp_wald_scan_batched
        assert "fasterlmm_lux.epi.scan.snp_wald_scan_batched" in patched
    finally:
        shim.uninstall()
    assert scan.snp_wald_scan_batched is orig
