"""
Shared pytest setup.

Marker ``gpu``: tests that need a CUDA device (run with ``-m gpu``); everything else runs on a CPU-only host.
The package lives in ``fast-er-lmm_gb300/`` and the CPU oracle in ``oracle/``; both are put on sys.path here.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

REPO = Path(__file__).resolve().parents[1]
GOLDEN = REPO / "tests" / "golden"
for p in (REPO / "fast-er-lmm_gb300", REPO / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    """Loader for the committed reference fixtures: golden('loco_n150_m1500') -> dict of arrays."""
    cache = {}

    def load(name):
        if name not in cache:
            with np.load(GOLDEN / f"{name}.npz") as z:
                cache[name] = {k: z[k] for k in z.files}
        return cache[name]
    return load


def z_float(G: np.ndarray) -> np.ndarray:
    """int8 dosages with -1 for missing -> float64 with NaN (the reference's genotype convention)."""
    Z = G.astype(np.float64)
    Z[G < 0] = np.nan
    return Z
