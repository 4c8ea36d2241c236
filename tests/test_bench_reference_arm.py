"""
CPU test of ``bench.py --impl reference``: the reference arm runs on a host without a GPU and prints one JSON line
with the keys the benchmark contract asks for (impl, cpu_baseline, e2e with zero copy bytes), on a tiny sample.
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parents[1]


def test_reference_arm_prints_its_line():
    r = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--B", "8", "--M", "2000"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-3000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "tests/s"
    assert line["cpu_baseline"]["kind"] in ("port", "reference") and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["steps"] == 1 and line["warmup"] == 1


def test_cpu_path_is_the_installed_reference_where_present(tmp_path, monkeypatch):
    """The CPU baseline times the reference's own functions when the package is installed under baseline/_ref,
    and the oracle port otherwise; both run a tiny sample to the end."""
    import pytest
    sys.path.insert(0, str(REPO))
    import bench
    d, w = bench.make_inputs(8, 2000)
    monkeypatch.setattr(bench, "REF_DIR", tmp_path)  # an empty directory: no install
    kind, ref, _ = bench._cpu_kind()
    assert kind == "port" and ref is None
    dt, n = bench.cpu_sample_run(d, w, 4, 1, None)
    assert dt > 0 and n > 0
    monkeypatch.setattr(bench, "REF_DIR", REPO / "baseline" / "_ref")
    if not (REPO / "baseline" / "_ref" / "fasterlmm" / "core.py").exists():
        pytest.skip("the reference is not installed under baseline/_ref")
    kind, ref, _ = bench._cpu_kind()
    assert kind == "reference" and ref[0].__name__ == "fasterlmm.core"
    dt2, n2 = bench.cpu_sample_run(d, w, 4, 1, ref)
    assert dt2 > 0 and n2 == n
    assert "pandas" not in sys.modules or sys.modules["pandas"].__dict__.get("__file__")  # no stand-in left behind
