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
    core = _fake("fasterlmm.core", ["loco_scan_compat", "single_k_scan_compat", "fastlmm_compat_rotate",
                                   "fit_delta_grid_compat", "snp_wald_scan_compat", "grm"])
    pmod = _fake("fasterlmm.perms", ["loco_scan_compat", "single_k_scan_compat", "perm_threshold"])
    cli = _fake("fasterlmm.cli", ["perm_threshold"])
    import sys
    sys.modules.update({"fasterlmm.core": core, "fasterlmm.perms": pmod, "fasterlmm.cli": cli})
    try:
        orig = (core.loco_scan_compat, pmod.perm_threshold, cli.perm_threshold, core.grm)
        patched = shim.install(form="fast", modules={"core": core, "perms": pmod, "cli": cli})
        assert "fasterlmm.perms.perm_threshold" in patched and "fasterlmm.cli.perm_threshold" in patched
        assert core.loco_scan_compat.keywords == {"form": "fast"}
        assert pmod.perm_threshold.func is perms.perm_threshold
        assert pmod.loco_scan_compat.keywords == {"form": "fast"}
        assert core.grm is orig[3]  # names outside the scan path are left alone
        shim.uninstall()
        assert (core.loco_scan_compat, pmod.perm_threshold, cli.perm_threshold) == orig[:3]
    finally:
        for k in ("fasterlmm.core", "fasterlmm.perms", "fasterlmm.cli"):
            sys.modules.pop(k, None)
