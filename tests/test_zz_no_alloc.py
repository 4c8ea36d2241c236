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


def _fit(lib, s, UYt, n_grid, lo, hi, noalloc):
    Neff = s.shape[0]
    P = UYt.shape[0]
    ld = torch.full((P,), float("nan"), dtype=torch.float64, device="cuda")
    idx = torch.full((P,), -1, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    if noalloc:
        lib.call("flmm_fit_delta_fast_noalloc", p(s), Neff, p(UYt), UYt.stride(0), P, n_grid, lo, hi, 1, p(ld), p(idx),
                 None)
    else:
        nbytes = lib.query_bytes("flmm_fit_delta_fast_workspace_bytes", Neff, n_grid)
        work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
        lib.call("flmm_fit_delta_fast", p(s), Neff, p(UYt), UYt.stride(0), P, n_grid, lo, hi, 1, p(ld), p(idx),
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
