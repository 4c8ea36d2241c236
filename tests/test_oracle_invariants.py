"""
The reference's own structural tests of the compat scan, restated against the CPU oracle (CPU only): the drop-D
shapes of the compat spectrum (reference tests/test_core_compat.py:87-114), the UY identity (:129-142), grid-node
landing without refinement (:174-186), max_F as the column maximum of F (:214-223), nullh2 = 1 / (1 + delta)
(:228), the n_real split (:261-282), a refined fit never worse than its grid node (tests/test_core_plain.py:
114-127, here for the compat loss), and the permutation seeding rules (tests/test_perms.py:26-36, 98-141).
"""
from __future__ import annotations

import numpy as np
import pytest

import flmm_oracle as orc
from fasterlmm_gb300.synth import make_dataset


@pytest.fixture(scope="module")
def case():
    d = make_dataset(80, 400, 2, 3, 6, seed=12, config_id=5, k_lo=1, k_hi=6, h2_lo=0.0, h2_hi=0.9)
    Z = orc.standardise_columns(d.Z_float())
    K = orc.grm(Z[:, d.chrom == 2])
    spec = orc.compat_rotate(K, d.X, d.Y)
    return d, Z, K, spec


def test_drop_d_shapes_and_clamped_spectrum(case):
    d, _, _, spec = case
    N, D = d.X.shape
    assert spec["s"].shape == (N - D,) and spec["U_eff"].shape == (N, N - D) and spec["UY"].shape == (N - D, 6)
    assert spec["Xpinv"].shape == (D, N)
    assert np.all(spec["s"] >= 0.0) and np.all(np.diff(spec["s"]) >= -1e-12)
    # the kept eigenvectors are orthonormal and orthogonal to the covariates
    U = spec["U_eff"]
    np.testing.assert_allclose(U.T @ U, np.eye(N - D), atol=1e-10)
    np.testing.assert_allclose(d.X.T @ U, 0.0, atol=1e-8)


def test_uy_identity(case):
    d, _, _, spec = case
    U, X, Y = spec["U_eff"], d.X, d.Y
    # U_eff is orthogonal to range(X), so U_eff^T Y_r = U_eff^T Y
    np.testing.assert_allclose(spec["UY"], U.T @ (Y - X @ np.linalg.pinv(X) @ Y), atol=1e-10)
    np.testing.assert_allclose(spec["UY"], U.T @ Y, atol=1e-8)


def test_grid_node_landing_and_refinement_no_worse(case):
    _, _, _, spec = case
    s, UY = spec["s"], spec["UY"]
    grid = orc.delta_grid(64, -10.0, 10.0)
    ld0, idx = orc.fit_delta_grid_compat(s, UY, refine=False, return_idx=True)
    np.testing.assert_array_equal(ld0, grid[idx])
    ld = orc.fit_delta_grid_compat(s, UY)
    L0 = orc.profile_loss_compat_per_pheno(ld0, s, UY)
    L1 = orc.profile_loss_compat_per_pheno(ld, s, UY)
    assert np.all(L1 <= L0 + 1e-9 * np.abs(L0))
    assert np.all(np.abs(ld - ld0) <= (grid[1] - grid[0]) + 1e-12)  # inside the argmin's bracket


def test_max_f_nullh2_and_n_real_split(case):
    d, Z, _, spec = case
    ld = orc.fit_delta_grid_compat(spec["s"], spec["UY"])
    S = Z[:, d.chrom == 1]
    full = orc.snp_wald_scan_compat(spec, ld, S)
    np.testing.assert_array_equal(full["max_F"], full["f"].max(axis=0))
    np.testing.assert_allclose(full["nullh2"], np.broadcast_to(1.0 / (1.0 + np.exp(ld)), full["nullh2"].shape))
    part = orc.snp_wald_scan_compat(spec, ld, S, n_real=2)
    for k in ("f", "beta", "se", "sfve", "nullh2"):
        np.testing.assert_array_equal(part[k], full[k][:, :2])
    np.testing.assert_array_equal(part["max_F"], full["max_F"])  # max_F covers every column


@pytest.fixture(scope="module")
def perm_case():
    d = make_dataset(60, 240, 3, 2, 5, seed=21, config_id=6, k_lo=1, k_hi=4)
    return d.Z_float(), d.X, d.Y, d.chrom


def _pt(case, cols, **kw):
    Z, X, Y, chrom = case
    return orc.perm_threshold(Z, X, Y, chrom, cols, **kw)


def test_permutation_seeding_like_the_reference(perm_case):
    """Reference tests/test_perms.py:26-36, 98-141: same seed identical, other seed differs, a phenotype keeps its
    permutation null when batched, reordered or scanned as a subset seeded with its full-table column."""
    r0, p0 = _pt(perm_case, [0, 1], n_perm=4)
    _, p1 = _pt(perm_case, [0, 1], n_perm=4)
    np.testing.assert_array_equal(p0, p1)
    _, p_other = _pt(perm_case, [0, 1], n_perm=4, seed=7)
    assert not np.array_equal(p0, p_other)
    # batching stability (same rounding tolerance as the reference's own test)
    r_solo, p_solo = _pt(perm_case, [0], n_perm=4)
    np.testing.assert_allclose(p0[0], p_solo[0], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(r0["f"][:, 0], r_solo["f"][:, 0], rtol=1e-7, atol=1e-9)
    # order independence: rows follow the requested order, each phenotype keeps its own permutations
    _, p10 = _pt(perm_case, [1, 0], n_perm=4)
    np.testing.assert_allclose(p10[0], p0[1], rtol=1e-7, atol=1e-9)
    np.testing.assert_allclose(p10[1], p0[0], rtol=1e-7, atol=1e-9)
    # seed_idx: a one-column subset seeded with its full-table column gets the same permutations
    Z, X, Y, chrom = perm_case
    _, p_plain = orc.perm_threshold(Z, X, Y, chrom, [3], n_perm=3)
    _, p_sub = orc.perm_threshold(Z, X, Y[:, [3]], chrom, [0], n_perm=3, seed_idx=[3])
    _, p_unseeded = orc.perm_threshold(Z, X, Y[:, [3]], chrom, [0], n_perm=3)
    np.testing.assert_allclose(p_sub, p_plain, rtol=1e-7, atol=1e-9)
    assert not np.allclose(p_unseeded, p_plain)
