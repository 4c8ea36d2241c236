"""
Install this package's GPU scan under an existing ``fasterlmm`` (FaST-ER-LMM) installation.

``install()`` rebinds, in the reference's own modules, the names its callers look up at call time:
``fasterlmm.core.{loco_scan_compat, single_k_scan_compat, fastlmm_compat_rotate, fit_delta_grid_compat,
snp_wald_scan_compat}``, the copies ``fasterlmm.perms`` imported by name (fasterlmm/perms.py:17), and
``perm_threshold`` in ``fasterlmm.perms`` and in ``fasterlmm.cli`` when that module is loaded (it imports the
function by name).  The plain GLS names of ``fasterlmm.core`` (rotate, eigendecompose, nLLeval, _profile_loss,
_profile_loss_per_pheno, fit_delta_grid, snp_wald_scan, loco_scan, single_k_scan; fasterlmm/core.py:89-451) and
the copies ``fasterlmm.extreme`` imported by name (fasterlmm/extreme.py:19) are rebound to the GLS kernels, and
the low-rank names of ``fasterlmm.lowrank`` and the copies ``fasterlmm.extreme_scan`` imported (fasterlmm/
extreme_scan.py:21-22) to the low-rank kernels, so the streamed engine's block loop runs its math on the GPU.  The
CLI and any user code that goes through those names then runs on the GPU unchanged.  ``uninstall()`` restores
the originals.  The CLI's per-phenotype writer ``fasterlmm.cli._write_pheno`` is rebound to fasterlmm_gb300.output,
whose files are byte-identical to the reference's.  When the LUX epistasis modules are loaded, their batched Wald
(``fasterlmm_lux.epi._kernel.snp_wald_scan_batched`` and the copy ``fasterlmm_lux.epi.scan`` imported by name) is
rebound to fasterlmm_gb300.epi.
"""
from __future__ import annotations

import functools
import sys

_saved: dict = {}  # (module name, attribute) -> (module, original value)

_CORE_NAMES = ("loco_scan_compat", "single_k_scan_compat", "fastlmm_compat_rotate", "fit_delta_grid_compat",
               "snp_wald_scan_compat")
_GLS_NAMES = ("eigendecompose", "rotate", "nLLeval", "_profile_loss", "_profile_loss_per_pheno", "fit_delta_grid",
              "snp_wald_scan", "loco_scan", "single_k_scan", "Spectrum")
_LOWRANK_NAMES = ("LowRankBasis", "LowRankSpectrum", "lowrank_basis", "rotate_phenos", "lowrank_rotate",
                  "fit_delta_grid_lowrank", "snp_wald_scan_lowrank", "loco_scan_lowrank", "single_k_scan_lowrank",
                  "loco_scan_resident")


def _set(mod, name, value):
    key = (mod.__name__, name)
    if key not in _saved:
        _saved[key] = (mod, getattr(mod, name))
    setattr(mod, name, value)


def install(form: str = "fast", modules: dict | None = None, outputs: bool = True) -> list[str]:
    """
    Patch the reference's modules (imported from sys.modules, or given as ``modules`` = {"core": ..., "perms":
    ..., "cli": ...}).  ``form`` picks the numeric form of the scan drivers; ``outputs`` also routes the CLI's
    per-phenotype writer through fasterlmm_gb300.output.  Returns the patched qualified names.
    """
    from . import core, gls, lowrank, perms
    mods = dict(modules or {})
    if not mods:
        import importlib
        mods["core"] = importlib.import_module("fasterlmm.core")
        mods["perms"] = importlib.import_module("fasterlmm.perms")
        for key in ("cli", "extreme", "lowrank", "extreme_scan"):
            if f"fasterlmm.{key}" in sys.modules:
                mods[key] = sys.modules[f"fasterlmm.{key}"]
        for key, name in (("lux_kernel", "fasterlmm_lux.epi._kernel"), ("lux_scan", "fasterlmm_lux.epi.scan")):
            if name in sys.modules:
                mods[key] = sys.modules[name]
    ours = {
        "loco_scan_compat": functools.partial(core.loco_scan_compat, form=form),
        "single_k_scan_compat": functools.partial(core.single_k_scan_compat, form=form),
        "fastlmm_compat_rotate": core.fastlmm_compat_rotate,
        "fit_delta_grid_compat": core.fit_delta_grid_compat,
        "snp_wald_scan_compat": core.snp_wald_scan_compat,
    }
    patched = []
    for name in _CORE_NAMES:
        if hasattr(mods.get("core"), name):
            _set(mods["core"], name, ours[name])
            patched.append(f"{mods['core'].__name__}.{name}")
    for name in _GLS_NAMES:
        for key in ("core", "extreme"):
            m = mods.get(key)
            if m is not None and hasattr(m, name):
                _set(m, name, getattr(gls, name))
                patched.append(f"{m.__name__}.{name}")
    for name in _LOWRANK_NAMES:
        for key in ("lowrank", "extreme_scan"):
            m = mods.get(key)
            if m is not None and hasattr(m, name):
                _set(m, name, getattr(lowrank, name))
                patched.append(f"{m.__name__}.{name}")
    from . import epi
    for key in ("lux_kernel", "lux_scan"):
        m = mods.get(key)
        if m is not None and hasattr(m, "snp_wald_scan_batched"):
            _set(m, "snp_wald_scan_batched", epi.snp_wald_scan_batched)
            patched.append(f"{m.__name__}.snp_wald_scan_batched")
    cli = mods.get("cli")
    if outputs and cli is not None and hasattr(cli, "_write_pheno"):
        key = (cli.__name__, "_write_pheno")
        _set(cli, "_write_pheno", _cli_writer(_saved[key][1] if key in _saved else cli._write_pheno))
        patched.append(f"{cli.__name__}._write_pheno")
    pt = functools.partial(perms.perm_threshold, form=form)
    for key in ("perms", "cli"):
        m = mods.get(key)
        if m is None:
            continue
        for name in ("loco_scan_compat", "single_k_scan_compat"):
            if hasattr(m, name):
                _set(m, name, ours[name])
                patched.append(f"{m.__name__}.{name}")
        if hasattr(m, "perm_threshold"):
            _set(m, "perm_threshold", pt)
            patched.append(f"{m.__name__}.perm_threshold")
    return patched


def _cli_writer(original):
    """
    Stand-in for fasterlmm.cli._write_pheno (fasterlmm/cli.py:114-158) that writes through fasterlmm_gb300.output.
    The CLI's writer context is turned into a VariantTable once per (ids, genotype variances) pair; calls with LD
    clumping on (the optional LDGroup column) go to the original writer.
    """
    from .output import VariantTable, write_pheno
    cache: dict = {}

    def write(ctx, outdir_str, pheno_name, p_col, beta_col, se_col, sfve_col, nullh2_col, p_var, perm_min_p,
              perm_quantile, per_pheno_dirs, bundle_writer):
        if ctx.get("clump") is not None:
            return original(ctx, outdir_str, pheno_name, p_col, beta_col, se_col, sfve_col, nullh2_col, p_var,
                            perm_min_p, perm_quantile, per_pheno_dirs, bundle_writer)
        key = (id(ctx["snp_id"]), id(ctx["g_var"]))
        hit = cache.get(key)
        if hit is None or hit[0] is not ctx["snp_id"] or hit[1] is not ctx["g_var"]:
            ids = ctx["snp_id"].to_pylist() if hasattr(ctx["snp_id"], "to_pylist") else list(ctx["snp_id"])
            table = VariantTable.of(ids, ctx["chrom"], ctx["pos"], ctx["g_var"], int(ctx["phenocount"][0]) - 1)
            if len(cache) > 8:
                cache.clear()
            hit = cache[key] = (ctx["snp_id"], ctx["g_var"], table)  # the objects are kept so their ids stay theirs
        write_pheno(hit[2], outdir_str, pheno_name, p_col, beta_col, se_col, sfve_col, nullh2_col, p_var,
                    perm_min_p, perm_quantile, per_pheno_dirs, bundle_writer, lambda_rows=ctx["lambda_rows"])

    return write


def uninstall() -> None:
    for (_, name), (mod, value) in list(_saved.items()):
        setattr(mod, name, value)
    _saved.clear()
