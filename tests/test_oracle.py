"""The oracle (CPU restatement) pinned against the reference.

1. Bit-exact agreement with golden vectors recorded from the reference's own
   translation units (tests/golden/make_golden.py).
2. When oracle/_ref/libmgref.so exists (this container), a direct
   comparison with the reference on fresh inputs.
3. The reference unit tests of this path, restated on the oracle:
   tests/testLaph4.cc, testBatchLaph4.cc, testMGkernels.cc,
   testTradeGhostValues.cc and testGramMatrix.cc.
"""
import numpy as np
import pytest

import oracle as O
from helpers import golden
from mgmol_gb300 import synth


@pytest.fixture(scope="module")
def G():
    return golden()


@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_stencils_match_reference_vectors(G, tag, dt):
    n = tuple(int(x) for x in G["stencil_n"])
    ll = tuple(float(x) for x in G["stencil_ll"])
    psi = G["stencil_psi"].astype(dt)
    for t in range(5):
        assert np.array_equal(O.fd_apply(n, ll, t, psi), G[f"fd{t}_{tag}"]), f"lap_type {t}"
    assert np.array_equal(O.rhs_mehr(n, ll, psi), G[f"rhs_{tag}"])
    assert np.array_equal(O.hpsi(n, ll, 0, psi, G["stencil_V"]), G[f"hpsi_{tag}"])
    r = O.restrict(n, ll, psi)
    assert np.array_equal(r, G[f"restrict_{tag}"])
    assert np.array_equal(O.extend(n, ll, r), G[f"extend_{tag}"])


@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
@pytest.mark.parametrize("lap", [0, 2, 4])
def test_precond_matches_reference_vectors(G, tag, dt, lap):
    n = tuple(int(x) for x in G["pc_n"])
    ll = tuple(float(x) for x in G["pc_ll"])
    out = O.precond(n, ll, lap, 2, float(G["pc_gamma"]), G["pc_res"].astype(dt))
    assert np.array_equal(out, G[f"pc{lap}_{tag}"])


@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_residual_matches_reference_vectors(G, tag, dt):
    n = tuple(int(x) for x in G["res_n"])
    ll = tuple(float(x) for x in G["res_ll"])
    psi = G["res_psi"].astype(dt)
    th = G["res_theta"]
    assert np.array_equal(O.mult_matrix(psi, th), G[f"mm_{tag}"])
    hp = G[f"res_hpsi_{tag}"]
    assert np.array_equal(O.residual(n, ll, psi, hp, th), G[f"res_{tag}"])


@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_matb_and_normalize_match_reference_vectors(G, tag, dt):
    n = tuple(int(x) for x in G["res_n"])
    ll = tuple(float(x) for x in G["res_ll"])
    psi = G["res_psi"].astype(dt)
    assert np.array_equal(O.matb(n, ll, psi), G[f"matb_{tag}"])
    out, d = O.normalize(n, ll, psi)
    assert np.array_equal(out, G[f"norm_psi_{tag}"])
    assert np.array_equal(d, G[f"norm_diag_{tag}"])


@pytest.mark.parametrize("name", ["conv", "collinear", "repeat"])
@pytest.mark.parametrize("m", [1, 3])
@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_anderson_matches_reference_vectors(G, name, m, tag, dt):
    got = O.anderson(G["and_x0"].astype(dt), G[f"and_f_{name}"].astype(dt), m, 1.0, 0.02,
                     G["and_invs"], fscale=0.5)
    assert np.array_equal(got, G[f"and_{name}_m{m}_{tag}"])


@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_rho_matches_reference_vectors(G, tag, dt):
    n = tuple(int(x) for x in G["res_n"])
    ll = tuple(float(x) for x in G["res_ll"])
    rho, charge, t = O.rho(n, ll, G["res_psi"].astype(dt), G["rho_X"])
    assert np.array_equal(rho, G[f"rho_{tag}"])
    vel = np.prod([a / b for a, b in zip(ll, n)])
    assert abs(charge - vel * G[f"rho_{tag}"].sum()) < 1e-12 * abs(charge)
    # rescaled to a charge within 2 %: the density scales by nel / charge
    scaled, c2, t2 = O.rho(n, ll, G["res_psi"].astype(dt), G["rho_X"], nel=1.01 * charge)
    assert abs(t2 - 1.01) < 1e-12 and np.allclose(scaled, 1.01 * rho, rtol=1e-14, atol=0)
    with pytest.raises(RuntimeError):
        O.rho(n, ll, G["res_psi"].astype(dt), G["rho_X"], nel=1.1 * charge)


def test_update_hb_oracle_vs_numpy():
    rng = np.random.default_rng(5)
    A = rng.standard_normal((9, 9))
    S = A @ A.T + 9 * np.eye(9)
    th = rng.standard_normal((9, 9))
    # only the lower triangle of S is read
    S_low = np.tril(S) + np.triu(rng.standard_normal((9, 9)), 1)
    hb = O.update_hb(S_low, th)
    ref = 0.5 * (S @ th) + 0.5 * (S @ th).T
    assert np.array_equal(hb, hb.T)
    assert np.max(np.abs(hb - ref)) < 1e-12 * np.max(np.abs(ref))


@pytest.mark.parametrize("lap", range(5))
def test_mgm_matches_reference_vectors(G, lap):
    n = tuple(int(x) for x in G["mgm_n"])
    ll = tuple(float(x) for x in G["mgm_ll"])
    vh, info = O.mgm(n, ll, lap, G["mgm_vh0"], G["mgm_rho"], max_sweeps=6, tol=1e-10)
    assert np.array_equal(vh, G[f"mgm{lap}_vh"])
    ref = G[f"mgm{lap}_info"]
    got = [info["final_residual"], info["final_relative_residual"], info["residual_reduction"],
           info["nb_sweeps"], info["converged"]]
    assert np.array_equal(np.array(got, dtype=np.float64), ref)
    if lap == 0:
        vf, _ = O.mgm(n, ll, 0, G["mgm_vh0"].astype(np.float32), G["mgm_rho"].astype(np.float32),
                      max_sweeps=3, tol=1e-10)
        assert np.array_equal(vf, G["mgm0_vh_f"])


def test_masks_match_reference_vectors(G):
    n = tuple(int(x) for x in G["pc_n"])
    ll = tuple(float(x) for x in G["pc_ll"])
    st, vals = O.mask_build(n, ll, 1, 3, G["mask_centers"], G["mask_radii"], func=0)
    assert np.array_equal(st, G["mask_state"])
    for l in range(3):
        assert np.array_equal(vals[l], G[f"mask_values_{l}"])
    st1, vals1 = O.mask_build(n, ll, 1, 1, G["mask_centers"], G["mask_radii"], func=1)
    assert np.array_equal(st1, G["mask1_state"])
    assert np.array_equal(vals1[0], G["mask1_values_0"])
    out = O.precond(n, ll, 0, 2, float(G["pc_gamma"]), G["pc_res"], masks=(st, vals))
    assert np.array_equal(out, G["pc0_masked_d"])


needs_ref = pytest.mark.skipif(O.ref_lib() is None, reason="reference pinning build absent")


@needs_ref
@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_oracle_equals_reference_fresh_inputs(dt):
    n = (12, 16, 8)
    ll = (12 * 0.3, 16 * 0.3, 8 * 0.3)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 2, 4242)
    psi = psi.astype(dt)
    V = synth.gaussian_wells(n, ll, 4, 4242)
    for t in range(5):
        assert np.array_equal(O.fd_apply(n, ll, t, psi), O.fd_apply(n, ll, t, psi, ref=True))
    assert np.array_equal(O.hpsi(n, ll, 0, psi, V), O.hpsi(n, ll, 0, psi, V, ref=True))
    a = O.precond(n, ll, 0, 1, 0.25, psi)
    b = O.precond(n, ll, 0, 1, 0.25, psi, ref=True)
    assert np.array_equal(a, b)


def _sin_field(n, ll):
    """u = sum_i sin(2 pi x_i / L_i) and its exact -Lap (tests/testLaph4.cc:30-82)."""
    x = [np.arange(n[i]) * ll[i] / n[i] for i in range(3)]
    X, Y, Z = np.meshgrid(*x, indexing="ij")
    k = [2 * np.pi / ll[i] for i in range(3)]
    u = np.sin(k[0] * X) + np.sin(k[1] * Y) + np.sin(k[2] * Z)
    lap = k[0] ** 2 * np.sin(k[0] * X) + k[1] ** 2 * np.sin(k[1] * Y) + k[2] ** 2 * np.sin(k[2] * Z)
    return u.reshape(1, -1), lap.reshape(1, -1)


def test_laph4_sine_margin():
    """tests/testLaph4.cc: 32x24x20 periodic grid, L = 2, margin 2e-3."""
    n = (32, 24, 20)
    ll = (2.0, 2.0, 2.0)
    u, lap = _sin_field(n, ll)
    for t in (2, 3, 4):
        out = O.fd_apply(n, ll, t, u)
        assert np.max(np.abs(out - lap)) / np.max(np.abs(lap)) < 2e-3
    # Mehrstellen: -Lap_M u approximates B(-Lap u)
    out = O.fd_apply(n, ll, 0, u)
    blap = O.rhs_mehr(n, ll, lap)
    assert np.max(np.abs(out - blap)) / np.max(np.abs(blap)) < 2e-3


def test_batch_laph4_sine_margin():
    """tests/testBatchLaph4.cc: the same check on a batch of 10 functions."""
    n = (32, 24, 20)
    ll = (2.0, 2.0, 2.0)
    u, lap = _sin_field(n, ll)
    U = np.repeat(u, 10, axis=0) * np.arange(1, 11)[:, None]
    out = O.fd_apply(n, ll, 2, U)
    for i in range(10):
        assert np.max(np.abs(out[i] - (i + 1) * lap[0])) < 2e-3 * (i + 1) * np.max(np.abs(lap))


def test_mgkernels_constants():
    """tests/testMGkernels.cc: constants i*1.11 survive restrict then extend to 1e-8."""
    n = (32, 24, 20)
    ll = (3.2, 2.4, 2.0)
    U = np.stack([np.full(n[0] * n[1] * n[2], i * 1.11) for i in range(5)])
    c = O.restrict(n, ll, U)
    assert np.max(np.abs(c - np.repeat(np.arange(5)[:, None] * 1.11, c.shape[1], 1))) < 1e-8
    f = O.extend(n, ll, c)
    assert np.max(np.abs(f - U)) < 1e-8


def test_trade_preserves_norm():
    """tests/testTradeGhostValues.cc: ghost fill leaves the interior norm
    unchanged and fills ghosts with periodic images (ghosts 1..2)."""
    for g in (1, 2):
        n = (32, 24, 20)
        ll = (3.2, 2.4, 2.0)
        rng = np.random.default_rng(7)
        u = rng.standard_normal((1, n[0] * n[1] * n[2]))
        # -Lap of a random field with ghost widths 1 (2nd) and 2 (4th) uses
        # exactly the ghost values; compare with a numpy periodic roll
        t = 1 if g == 1 else 2
        out = O.fd_apply(n, ll, t, u)
        U = u.reshape(n)
        h = [ll[i] / n[i] for i in range(3)]
        ref = np.zeros_like(U)
        for ax in range(3):
            ih = 1.0 / (h[ax] * h[ax])
            if t == 1:
                ref += ih * (2 * U - np.roll(U, 1, ax) - np.roll(U, -1, ax))
            else:
                ref += ih / 12.0 * (30 * U - 16 * (np.roll(U, 1, ax) + np.roll(U, -1, ax))
                                    + (np.roll(U, 2, ax) + np.roll(U, -2, ax)))
        assert np.max(np.abs(out.reshape(n) - ref)) < 1e-9 * np.max(np.abs(ref))


def test_gram_matrix_cholesky_and_loewdin():
    """tests/testGramMatrix.cc restated on one task: random SPD n = 213,
    L L^T - S <= 1e-14 relative, S^-1 S = I."""
    n = 213
    rng = np.random.default_rng(213)
    A = rng.standard_normal((n, n))
    S = A @ A.T / n + np.eye(n)
    info, L = O.potrf(S)
    assert info == 0
    assert np.max(np.abs(L @ L.T - S)) <= 1e-14 * np.max(np.abs(S)) * n
    Sinv = O.inverse_from_chol(L)
    assert np.max(np.abs(Sinv @ S - np.eye(n))) < 1e-12
    # a non-SPD matrix reports its failing pivot instead of aborting
    S2 = S.copy()
    S2[5, 5] = -1.0
    info2, _ = O.potrf(S2)
    assert info2 > 0


@pytest.mark.parametrize("case", ["a", "b"])
@pytest.mark.parametrize("tag,dt", [("d", np.float64), ("f", np.float32)])
def test_gram_and_hmat_match_reference_golden(case, tag, dt):
    """S and H bit for bit against the reference's getLocalOverlap /
    computeLocalProduct through LocalMatrices2DistMatrix (its 1e-14 filter
    drops the far pairs of case b).  For FP32 orbitals the reference's
    USE_MP path keeps each product in a float local matrix; the oracle's
    usemp form restates it, and its default FP64 sum is within that
    rounding."""
    g = golden()
    n = tuple(int(x) for x in g[f"sh{case}_n"])
    h = float(g[f"sh{case}_ll"][0]) / n[0]
    vel = h ** 3
    p = g[f"sh{case}_psi"].astype(dt)
    hp = g[f"sh{case}_hpsi_{tag}"]
    S_ref, H_ref = g[f"sh{case}_S_{tag}"], g[f"sh{case}_H_{tag}"]
    assert np.array_equal(O.gram(p, vel, usemp=True), S_ref)
    assert np.array_equal(O.hmat(p, hp, vel, usemp=True), H_ref)
    if case == "b":
        assert np.count_nonzero(S_ref == 0) > 0
    if dt == np.float32:
        # the FP64 sum the mixed-precision GPU path is measured against
        mask = S_ref != 0
        S = O.gram(p, vel)
        assert np.max(np.abs(S - S_ref)[mask] / np.abs(S_ref)[mask]) <= 2.0 ** -24
        assert np.array_equal(S == 0, S_ref == 0)
    if O.ref_lib() is not None:
        assert np.array_equal(O.gram(p, vel, ref=True), S_ref)
        assert np.array_equal(O.hmat(p, hp, vel, ref=True), H_ref)


def test_gram_and_hmat_oracle_vs_numpy():
    n = (8, 8, 8)
    ll = (2.8, 2.8, 2.8)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 6, 99)
    vel = (0.35 ** 3)
    S = O.gram(psi, vel)
    ref = psi @ psi.T * vel
    ref[np.abs(ref) <= 1e-14] = 0
    assert np.max(np.abs(S - ref)) < 1e-13 * np.max(np.abs(ref))
    H = O.hmat(psi, 2 * psi, vel)
    assert np.max(np.abs(H - 2 * ref)) < 1e-13 * np.max(np.abs(ref))


def test_set_gamma():
    """OrbitalsPreconditioning::setGamma arithmetic."""
    g = O.set_gamma(0.05, 2, -0.3, -1.2)
    d = 0.05 * 4 ** 3
    assert abs(g - 1.0 / (2.0 / d + abs(-0.3 + 1.2))) < 1e-15
