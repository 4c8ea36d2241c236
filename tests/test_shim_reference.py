"""
CPU test of the drop-in installer against the real reference package (not stand-ins): it imports the reference
(an empty stand-in for pandas, which fasterlmm/io.py:14 and fasterlmm/normalize.py:15 import at module top but the
scan never calls), runs ``shim.install()`` on its actual modules and checks

* every rebound name in fasterlmm.core, fasterlmm.perms (including the copies it imports by name,
  fasterlmm/perms.py:17), fasterlmm.lowrank and fasterlmm.extreme_scan now resolves to this package;
* each replacement accepts every call the reference's function accepts: the reference's parameters appear in the
  same order, of the same kind, with the same defaults; any extra parameter of ours is keyword-only or defaulted;
* ``uninstall()`` puts the reference's own objects back.

It runs in a child interpreter so the imported reference does not leak into the other tests' modules, and is
skipped where the reference is absent (FASTERLMM_REFERENCE names a checkout; by default it is the offline install
under baseline/_ref).
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
# the reference package: FASTERLMM_REFERENCE (a checkout), else its offline install under baseline/_ref
REF = Path(os.environ.get("FASTERLMM_REFERENCE", str(REPO / "baseline" / "_ref")))

CHILD = r"""
import inspect, json, sys, tempfile, pathlib, functools
stub = pathlib.Path(tempfile.mkdtemp()) / "pandas"; stub.mkdir(); (stub / "__init__.py").write_text("")
sys.path[:0] = [str(stub.parent), sys.argv[1], sys.argv[2]]
import fasterlmm.core as core, fasterlmm.perms as perms, fasterlmm.lowrank as lowrank, fasterlmm.extreme_scan as xs
from fasterlmm_gb300 import shim
mods = {"core": core, "perms": perms, "lowrank": lowrank, "extreme_scan": xs}
before = {(m, n): getattr(mod, n) for m, mod in mods.items() for n in dir(mod) if not n.startswith("__")}
patched = shim.install(form="fast", outputs=False)
report = {"patched": patched, "problems": [], "extras": {}}
def target(obj):
    return obj.func if isinstance(obj, functools.partial) else obj
for q in patched:
    mname, name = q.rsplit(".", 1)
    key = mname.split(".", 1)[1]
    if key not in mods:
        continue
    new, old = getattr(mods[key], name), before[(key, name)]
    if not target(new).__module__.startswith("fasterlmm_gb300"):
        report["problems"].append(f"{q} not rebound")
    if inspect.isclass(old) or not callable(old):
        continue
    ps_old = list(inspect.signature(old).parameters.values())
    sig_new = inspect.signature(new)
    ps_new = list(sig_new.parameters.values())
    for i, p in enumerate(ps_old):
        if i >= len(ps_new):
            report["problems"].append(f"{q}: missing {p.name}")
            continue
        n = ps_new[i]
        if (n.name, n.kind) != (p.name, p.kind):
            report["problems"].append(f"{q}: parameter {i} is {n.name}/{n.kind}, reference {p.name}/{p.kind}")
        elif p.default is not inspect.Parameter.empty and repr(n.default) != repr(p.default):
            report["problems"].append(f"{q}: default of {p.name} {n.default!r} != {p.default!r}")
    extra = ps_new[len(ps_old):]
    for n in extra:
        if n.kind is not inspect.Parameter.KEYWORD_ONLY and n.default is inspect.Parameter.empty:
            report["problems"].append(f"{q}: extra parameter {n.name} is required")
    report["extras"][q] = [n.name for n in extra]
shim.uninstall()
for (key, name), obj in before.items():
    if getattr(mods[key], name) is not obj:
        report["problems"].append(f"fasterlmm.{key}.{name} not restored")
print(json.dumps(report))
"""


@pytest.mark.skipif(not (REF / "fasterlmm" / "core.py").exists(), reason="the reference is neither checked out nor installed")
def test_install_on_the_real_reference_modules():
    r = subprocess.run([sys.executable, "-c", CHILD, str(REF), str(REPO / "fast-er-lmm_gb300")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    rep = json.loads(r.stdout.strip().splitlines()[-1])
    must = {"fasterlmm.core.loco_scan_compat", "fasterlmm.core.single_k_scan_compat",
            "fasterlmm.core.fastlmm_compat_rotate", "fasterlmm.core.fit_delta_grid_compat",
            "fasterlmm.core.snp_wald_scan_compat", "fasterlmm.perms.perm_threshold",
            "fasterlmm.perms.loco_scan_compat", "fasterlmm.core.loco_scan", "fasterlmm.lowrank.loco_scan_lowrank"}
    assert must <= set(rep["patched"]), sorted(must - set(rep["patched"]))
    assert not rep["problems"], rep["problems"]
