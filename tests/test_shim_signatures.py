"""
The drop-in's public names against the reference's own signatures (tests/golden/signatures.json, written by
tests/golden/make_signatures.py from an import of the reference): every function the installer rebinds takes the
reference's parameters in the reference's order, with the same kinds and defaults, and adds only keyword
parameters that have defaults; the dataclasses carry the reference's fields in order.  Then install() on modules
that hold exactly the reference's names rebinds each of them.
"""
from __future__ import annotations

import dataclasses
import inspect
import json
import types
from pathlib import Path

import pytest

SIGS = json.loads((Path(__file__).parent / "golden" / "signatures.json").read_text())


def _ours(qualname):
    from fasterlmm_gb300 import core, gls, lowrank, perms, shim
    mod, name = qualname.rsplit(".", 1)
    if mod == "fasterlmm.core":
        return getattr(core if name in shim._CORE_NAMES else gls, name)
    return getattr({"fasterlmm.perms": perms, "fasterlmm.lowrank": lowrank}[mod], name)


@pytest.mark.parametrize("qualname", sorted(SIGS))
def test_signature_matches_reference(qualname):
    ref = SIGS[qualname]
    ours = _ours(qualname)
    if "dataclass" in ref:
        assert dataclasses.is_dataclass(ours)
        assert [f.name for f in dataclasses.fields(ours)][:len(ref["dataclass"])] == ref["dataclass"]
        return
    params = list(inspect.signature(ours).parameters.values())
    assert len(params) >= len(ref["params"]), qualname
    for p, r in zip(params, ref["params"]):
        assert p.name == r["name"] and p.kind.name == r["kind"], (qualname, p, r)
        want = r["default"]
        got = None if p.default is inspect.Parameter.empty else repr(p.default)
        assert got == want, (qualname, p.name, got, want)
    for p in params[len(ref["params"]):]:
        assert p.kind is inspect.Parameter.KEYWORD_ONLY and p.default is not inspect.Parameter.empty, (qualname, p)


def test_install_rebinds_every_reference_name():
    from fasterlmm_gb300 import shim
    mods = {}
    for qualname in SIGS:
        mod, name = qualname.rsplit(".", 1)
        m = mods.setdefault(mod, types.ModuleType(mod))
        setattr(m, name, object())
    originals = {q: getattr(mods[q.rsplit(".", 1)[0]], q.rsplit(".", 1)[1]) for q in SIGS}
    patched = shim.install(modules={"core": mods["fasterlmm.core"], "perms": mods["fasterlmm.perms"],
                                    "lowrank": mods["fasterlmm.lowrank"]}, outputs=False)
    try:
        for q, orig in originals.items():
            mod, name = q.rsplit(".", 1)
            assert q in patched, q
            assert getattr(mods[mod], name) is not orig, q
    finally:
        shim.uninstall()
    for q, orig in originals.items():
        mod, name = q.rsplit(".", 1)
        assert getattr(mods[mod], name) is orig, q
