"""
Record the reference's public signatures for the names the drop-in installer rebinds, as tests/golden/signatures.json.

Usage (in a checkout where the reference is present):
    python tests/golden/make_signatures.py [--reference PATH]

The reference (the ``fasterlmm`` package) is imported from PATH (default: the FASTERLMM_REFERENCE environment
variable), with the same empty pandas stand-in as make_golden.py when pandas is absent.  For every function the
installer (fasterlmm_gb300.shim) rebinds in fasterlmm.core, fasterlmm.perms and fasterlmm.lowrank, the file holds
its parameters (name, kind, default as repr, or null when there is none); for the dataclasses, their field names
in order.  tests/test_shim_signatures.py checks the drop-in against this file without the reference present.
"""
from __future__ import annotations

import argparse
import dataclasses
import inspect
import json
import os
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO / "fast-er-lmm_gb300"))
sys.path.insert(0, str(HERE))

from make_golden import _import_reference  # noqa: E402
from fasterlmm_gb300 import shim  # noqa: E402


def _describe(obj):
    if dataclasses.is_dataclass(obj):
        return {"dataclass": [f.name for f in dataclasses.fields(obj)]}
    params = []
    for p in inspect.signature(obj).parameters.values():
        params.append({"name": p.name, "kind": p.kind.name,
                       "default": None if p.default is inspect.Parameter.empty else repr(p.default)})
    return {"params": params}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("FASTERLMM_REFERENCE", ""))
    args = ap.parse_args()
    if not args.reference:
        sys.exit("pass --reference PATH (or set FASTERLMM_REFERENCE) to the reference checkout")
    _import_reference(args.reference)
    import importlib
    out = {}
    names = {"fasterlmm.core": shim._CORE_NAMES + shim._GLS_NAMES, "fasterlmm.perms": ("perm_threshold",),
             "fasterlmm.lowrank": shim._LOWRANK_NAMES}
    for modname, attrs in names.items():
        mod = importlib.import_module(modname)
        for a in attrs:
            if hasattr(mod, a):
                out[f"{modname}.{a}"] = _describe(getattr(mod, a))
    (HERE / "signatures.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"wrote {len(out)} signatures")


if __name__ == "__main__":
    main()
