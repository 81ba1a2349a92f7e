"""Parity of the multigrid transfers, masks and the V-cycle preconditioner
(CUDA through the C ABI) with the oracle; masks bit-exact."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F32, TOL_F64, golden, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


@pytest.mark.parametrize("n", [(16, 12, 20), (32, 32, 32), (8, 4, 6)])
def test_restrict_prolong(n):
    ll = tuple(x * 0.35 for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 3, 5)
    ctx = capi.Context(n, ll)
    c = ctx.restrict(_dev(psi))
    c_ref = O.restrict(n, ll, psi)
    assert rel_err(c.cpu().numpy(), c_ref) < TOL_F64
    f = ctx.prolong(_dev(c_ref))
    assert rel_err(f.cpu().numpy(), O.extend(n, ll, c_ref)) < TOL_F64
    c32 = ctx.restrict(_dev(psi, np.float32))
    assert rel_err(c32.cpu().numpy(), c_ref) < TOL_F32


def test_transfer_constants_exact():
    """tests/testMGkernels.cc on the GPU: constants survive restrict+extend."""
    n = (32, 24, 20)
    ctx = capi.Context(n, (3.2, 2.4, 2.0))
    U = torch.stack([torch.full((n[0] * n[1] * n[2],), i * 1.11, dtype=torch.float64) for i in range(5)]).cuda()
    f = ctx.prolong(ctx.restrict(U))
    assert float((f - U).abs().max()) < 1e-8


@pytest.mark.parametrize("lap", [0, 2, 4])
def test_precond_golden(lap):
    G = golden()
    n = tuple(int(x) for x in G["pc_n"])
    ll = tuple(float(x) for x in G["pc_ll"])
    ctx = capi.Context(n, ll)
    g = float(G["pc_gamma"])
    out = ctx.precond_mg(_dev(G["pc_res"]), lap, 2, g).cpu().numpy()
    assert rel_err(out, G[f"pc{lap}_d"]) < TOL_F64
    out32 = ctx.precond_mg(_dev(G["pc_res"], np.float32), lap, 2, g).cpu().numpy()
    assert rel_err(out32, G[f"pc{lap}_d"]) < 1e-4


@pytest.mark.parametrize("n,maxl,lap", [((32, 32, 32), 2, 0), ((64, 32, 48), 2, 0),
                                         ((32, 32, 32), 1, 4), ((32, 16, 32), 0, 0),
                                         ((64, 64, 64), 3, 2)])
def test_precond_vs_oracle(n, maxl, lap):
    ll = tuple(x * 0.35 for x in n)
    res, _, _ = synth.gaussian_orbitals(n, ll, 3, 21)
    ctx = capi.Context(n, ll)
    ref = O.precond(n, ll, lap, maxl, 0.37, res)
    out = ctx.precond_mg(_dev(res), lap, maxl, 0.37).cpu().numpy()
    assert rel_err(out, ref) < TOL_F64


def test_precond_chunked_equals_unchunked():
    n = (32, 32, 32)
    ll = (11.2,) * 3
    res, _, _ = synth.gaussian_orbitals(n, ll, 7, 8)
    ctx = capi.Context(n, ll)
    a = ctx.precond_mg(_dev(res), 0, 2, 0.3)
    b = ctx.precond_mg(_dev(res), 0, 2, 0.3, chunk=3)
    assert torch.equal(a, b)


def test_masks_bit_exact_vs_reference_vectors():
    G = golden()
    n = tuple(int(x) for x in G["pc_n"])
    ll = tuple(float(x) for x in G["pc_ll"])
    ctx = capi.Context(n, ll)
    M = capi.Masks(ctx, 3, G["mask_centers"], G["mask_radii"], func=0, kind=0, mesh_ghosts=1)
    for l in range(3):
        st, dense = M.expand(l)
        assert np.array_equal(st, G["mask_state"][l])
        assert np.array_equal(dense.cpu().numpy(), G[f"mask_values_{l}"]), f"level {l}"
    M1 = capi.Masks(ctx, 1, G["mask_centers"], G["mask_radii"], func=1, kind=1, mesh_ghosts=1)
    st, dense = M1.expand(0)
    assert np.array_equal(st, G["mask1_state"][0])
    assert np.array_equal(dense.cpu().numpy(), G["mask1_values_0"])


@pytest.mark.parametrize("n,ng,seed", [((64, 64, 64), 1, 1003), ((48, 40, 32), 4, 77)])
def test_masks_bit_exact_vs_oracle(n, ng, seed):
    ll = tuple(x * 0.3 for x in n)
    _, centers, _ = synth.gaussian_orbitals(n, ll, 12, seed)
    radii = synth.mask_radii(12, seed, 2.0, 6.0)
    radii[0] = 200.0  # state 1 (mask identically one)
    ctx = capi.Context(n, ll)
    st_ref, vals_ref = O.mask_build(n, ll, ng, 3, centers, radii, func=0)
    M = capi.Masks(ctx, 3, centers, radii, func=0, kind=0, mesh_ghosts=ng)
    for l in range(3):
        st, dense = M.expand(l)
        assert np.array_equal(st, st_ref[l])
        d = dense.cpu().numpy()
        for f in range(12):
            if st_ref[l][f] == 2:
                assert np.array_equal(d[f], vals_ref[l][f]), (l, f)


def test_mask_apply_and_masked_precond():
    G = golden()
    n = tuple(int(x) for x in G["pc_n"])
    ll = tuple(float(x) for x in G["pc_ll"])
    ctx = capi.Context(n, ll)
    M = capi.Masks(ctx, 3, G["mask_centers"], G["mask_radii"], func=0, kind=0, mesh_ghosts=1)
    out = ctx.precond_mg(_dev(G["pc_res"]), 0, 2, float(G["pc_gamma"]), masks=M).cpu().numpy()
    assert rel_err(out, G["pc0_masked_d"]) < TOL_F64
    # apply alone
    u = _dev(G["pc_res"] * 3.0)
    M.apply(u, 0)
    st, vals = O.mask_build(n, ll, 1, 3, G["mask_centers"], G["mask_radii"], func=0)
    ref = O.mask_apply(n, 0, st, vals, G["pc_res"] * 3.0, kind=0)
    assert np.array_equal(u.cpu().numpy(), ref)


def test_masked_precond_float32():
    n = (32, 32, 32)
    ll = (9.6,) * 3
    res, centers, _ = synth.gaussian_orbitals(n, ll, 4, 31)
    radii = synth.mask_radii(4, 31, 3.0, 5.0)
    ctx = capi.Context(n, ll)
    st, vals = O.mask_build(n, ll, 1, 3, centers, radii, func=0, dtype=np.float32)
    ref = O.precond(n, ll, 0, 2, 0.3, res.astype(np.float32), masks=(st, vals))
    M = capi.Masks(ctx, 3, centers, radii, func=0, kind=0, dtype=torch.float32)
    out = ctx.precond_mg(_dev(res, np.float32), 0, 2, 0.3, masks=M).cpu().numpy()
    assert rel_err(out, ref) < 1e-4


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-14), (np.float32, 2e-6)])
def test_precond_update_fused(dt, tol):
    """psi += alpha P(res) through the last fine sweep equals the V-cycle
    followed by an axpy (the update of ABPG::update_states)."""
    n = (32, 32, 32)
    ll = tuple(x * 0.3 for x in n)
    res, _, _ = synth.gaussian_orbitals(n, ll, 5, 61)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 5, 62)
    ctx = capi.Context(n, ll)
    r = _dev(res, dt)
    corr = ctx.precond_mg(r, 0, 2, 0.3)
    ref = _dev(psi, dt)
    capi.axpy(0.5, corr, ref)
    got = _dev(psi, dt)
    ctx.precond_update(r, got, 0.5, 0, 2, 0.3)
    assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) < tol
    # without coarse levels (the update rides on the last coarsest-level sweep)
    c0 = ctx.precond_mg(r, 0, 0, 0.3)
    ref0 = _dev(psi, dt)
    capi.axpy(0.5, c0, ref0)
    got0 = _dev(psi, dt)
    ctx.precond_update(r, got0, 0.5, 0, 0, 0.3)
    assert rel_err(got0.cpu().numpy(), ref0.cpu().numpy()) < tol
    # with a caller scratch block for the fine-level iterate
    got = _dev(psi, dt)
    ctx.precond_update(r, got, 0.5, 0, 2, 0.3, work=torch.empty_like(r))
    assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) < tol
    # through the masked V-cycle too
    centers = np.array([[4.8, 4.8, 4.8]] * 5)
    radii = np.full(5, 3.0)
    masks = capi.Masks(ctx, 3, centers, radii, dtype=torch.float64 if dt == np.float64 else torch.float32)
    corr = ctx.precond_mg(r, 0, 2, 0.3, masks=masks)
    ref = _dev(psi, dt)
    capi.axpy(0.5, corr, ref)
    got = _dev(psi, dt)
    ctx.precond_update(r, got, 0.5, 0, 2, 0.3, masks=masks)
    assert rel_err(got.cpu().numpy(), ref.cpu().numpy()) < tol


def test_precond_leading_dimension_above_points():
    """Blocks whose functions are spaced wider than the grid (ld > points)."""
    n = (16, 16, 16)
    ll = tuple(x * 0.35 for x in n)
    res, _, _ = synth.gaussian_orbitals(n, ll, 4, 63)
    ctx = capi.Context(n, ll)
    npts = ctx.npts
    wide = torch.zeros((4, npts + 96), dtype=torch.float64, device="cuda")
    wide[:, :npts] = _dev(res)
    out_wide = torch.full((4, npts + 96), 7.0, dtype=torch.float64, device="cuda")
    ctx.precond_mg(wide[:, :npts], 0, 2, 0.3, out=out_wide[:, :npts])
    ref = ctx.precond_mg(_dev(res), 0, 2, 0.3)
    assert torch.equal(out_wide[:, :npts], ref)
    assert torch.all(out_wide[:, npts:] == 7.0)


def test_masks_update_after_centres_move():
    """MasksSet::update: the set rebuilt for moved centres and new radii is
    bit-identical to a fresh one (and to the oracle), through the same
    handle; a correction-mask set (profile one, GridMaskMult) applied to a
    block as LocGridOrbitals::applyCorrMask does matches the oracle."""
    n = (48, 40, 32)
    ll = tuple(x * 0.3 for x in n)
    _, centers, _ = synth.gaussian_orbitals(n, ll, 10, 91)
    radii = synth.mask_radii(10, 91, 2.0, 6.0)
    ctx = capi.Context(n, ll)
    M = capi.Masks(ctx, 3, centers, radii, func=0, kind=0, mesh_ghosts=2)
    rng = np.random.default_rng(92)
    moved = (centers + rng.uniform(-1.0, 1.0, centers.shape)) % np.asarray(ll)
    radii2 = radii * 1.1
    M.update(moved, radii2)
    fresh = capi.Masks(ctx, 3, moved, radii2, func=0, kind=0, mesh_ghosts=2)
    st_ref, vals_ref = O.mask_build(n, ll, 2, 3, moved, radii2, func=0)
    for l in range(3):
        st, dense = M.expand(l)
        st2, dense2 = fresh.expand(l)
        assert np.array_equal(st, st2) and np.array_equal(st, st_ref[l])
        assert np.array_equal(dense.cpu().numpy(), dense2.cpu().numpy())
        d = dense.cpu().numpy()
        for f in range(10):
            if st_ref[l][f] == 2:
                assert np.array_equal(d[f], vals_ref[l][f]), (l, f)
    # correction masks: profile one, multiplied in
    C = capi.Masks(ctx, 1, moved, radii2 * 1.5, func=1, kind=1, mesh_ghosts=2)
    res, _, _ = synth.gaussian_orbitals(n, ll, 10, 93)
    u = _dev(res)
    C.apply(u, 0)
    st1, vals1 = O.mask_build(n, ll, 2, 1, moved, radii2 * 1.5, func=1)
    ref = O.mask_apply(n, 0, st1, vals1, res, kind=1)
    assert np.array_equal(u.cpu().numpy(), ref)
