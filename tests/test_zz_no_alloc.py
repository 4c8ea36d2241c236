"""
GPU test of flmm_fit_delta_fast_noalloc, the delta-fit entry point that allocates nothing.

It is meant for callers that cannot give the library device memory (all of it owned by another pool, or a
latency-critical loop that may not call cudaMalloc); its scratch is a fixed array inside the library, shared by all
calls on a device.  The test drives it through the C ABI on two calls in a row -- different sizes and data, so the
second call runs over the first call's leftover scratch -- and checks each against flmm_fit_delta_fast with
caller-provided workspace on the same inputs (same kernels, so the results must be identical), plus the size limit.
The file name makes pytest collect it last.
"""
from __future__ import annotations

import ctypes as C

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from fasterlmm_gb300 import _lib, build
    build()
    return _lib


def _inputs(Neff, P, seed):
    g = torch.Generator().manual_seed(seed)
    s = (torch.rand(Neff, generator=g, dtype=torch.float64) * 2.0 + 0.05).cuda()
    s[: Neff // 10] = 0.0  # some zero eigenvalues, as a rank-deficient kinship gives
    UYt = torch.randn(P, Neff, generator=g, dtype=torch.float32).cuda()
    UYt[:, : Neff // 3] *= 3.0
    return s, UYt


def _fit(lib, s, UYt, n_grid, lo, hi, noalloc, refine=1):
    Neff = s.shape[0]
    P = UYt.shape[0]
    ld = torch.full((max(P, 1),), float("nan"), dtype=torch.float64, device="cuda")
    idx = torch.full((max(P, 1),), -1, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    if noalloc:
        lib.call("flmm_fit_delta_fast_noalloc", p(s), Neff, p(UYt), UYt.stride(0), P, n_grid, lo, hi, refine, p(ld),
                 p(idx), None)
    else:
        nbytes = lib.query_bytes("flmm_fit_delta_fast_workspace_bytes", Neff, n_grid)
        work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        lib.call("flmm_fit_delta_fast", p(s), Neff, p(UYt), UYt.stride(0), P, n_grid, lo, hi, refine, p(ld), p(idx),
                 p(work), nbytes, None)
    torch.cuda.synchronize()
    return ld.cpu(), idx.cpu()


def test_noalloc_matches_workspace_entry_on_two_calls(lib):
    calls = [(995, 700, 64, -10.0, 10.0, 1), (150, 257, 100, -5.0, 5.0, 2)]
    for Neff, P, n_grid, lo, hi, seed in calls:
        s, UYt = _inputs(Neff, P, seed)
        ld_ref, idx_ref = _fit(lib, s, UYt, n_grid, lo, hi, noalloc=False)
        ld, idx = _fit(lib, s, UYt, n_grid, lo, hi, noalloc=True)
        assert torch.isfinite(ld).all() and (idx >= 0).all()
        assert torch.equal(idx, idx_ref)
        torch.testing.assert_close(ld, ld_ref, rtol=0, atol=0)


def test_noalloc_rejects_oversized_requests(lib):
    s, UYt = _inputs(5000, 4, 3)
    with pytest.raises(lib.FlmmError) as e:
        _fit(lib, s, UYt, 400, -10.0, 10.0, noalloc=True)  # 400 * 5000 floats > 4 MiB
    assert e.value.status == 4 and "fixed" in str(e.value)


def test_noalloc_edge_cases_match_workspace_entry(lib):
    """No columns, grid-only fits, and minima outside the bracket (the edge and binary-search branches)."""
    s, UYt = _inputs(300, 1, 4)
    ld = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
    idx = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    lib.call("flmm_fit_delta_fast_noalloc", p(s), 300, p(UYt), 300, 0, 64, -10.0, 10.0, 1, p(ld), p(idx), None)
    torch.cuda.synchronize()
    assert torch.isnan(ld).all() and (idx == -1).all()  # P = 0: nothing written
    s, UYt = _inputs(300, 129, 5)
    for refine in (0, 1):
        a = _fit(lib, s, UYt, 64, -10.0, 10.0, noalloc=False, refine=refine)
        b = _fit(lib, s, UYt, 64, -10.0, 10.0, noalloc=True, refine=refine)
        assert torch.equal(a[1], b[1]) and torch.equal(a[0], b[0])
    # a narrow window [-1, 1]: most columns' minima lie outside it, so the fit ends at a window edge
    a = _fit(lib, s, UYt, 16, -1.0, 1.0, noalloc=False)
    b = _fit(lib, s, UYt, 16, -1.0, 1.0, noalloc=True)
    assert torch.equal(a[1], b[1]) and torch.equal(a[0], b[0])
    assert ((a[1] == 0) | (a[1] == 15)).any()


def test_noalloc_limit_is_the_workspace_size(lib):
    """The exact limit: calls whose workspace query is at most 4 MiB run, one grid node more is refused."""
    limit = 4 << 20
    Neff = 4096
    fits = [g for g in range(200, 300) if lib.query_bytes("flmm_fit_delta_fast_workspace_bytes", Neff, g) <= limit]
    g_max = max(fits)
    s, UYt = _inputs(Neff, 3, 6)
    a = _fit(lib, s, UYt, g_max, -10.0, 10.0, noalloc=False)
    b = _fit(lib, s, UYt, g_max, -10.0, 10.0, noalloc=True)
    assert torch.equal(a[0], b[0])
    with pytest.raises(lib.FlmmError) as e:
        _fit(lib, s, UYt, g_max + 1, -10.0, 10.0, noalloc=True)
    assert e.value.status == 4
