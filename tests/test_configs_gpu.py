"""The workload configurations at their stated sizes, through the C ABI.

C1  plain FP64: 64 orbitals on a 64^3 periodic grid, h = 0.35, seed 1001,
    8 wells; Mehrstellen H psi with B(V psi), the V-cycle on the residual
    (maxlevels 2: three grids), S, H and B against the oracle to 1e-12.
C2  FP32 orbitals: 512 on 128^3, h = 0.3, 32 wells, del2_8th; H psi in
    FP32, S and H in split-BF16x3 and TF32 against the FP64 path (these
    cross 64 split-K ranges of the tensor-core kernel, so its FP64 atomic
    reduction is exercised) and on the CUDA cores in FP32 with
    double-float totals, and the FP64 Cholesky of S.
C3  1536 localized orbitals on 160^3, h = 0.3, mask radii U[4, 8] bohr,
    seed 1003: the masks bit for bit against the oracle's GridMask::init
    restatement, and the fused localized step against the oracle chain on
    a subset of the orbitals.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


def test_c1_plain_fp64_at_the_stated_size():
    n = (64, 64, 64)
    ll = tuple(0.35 * x for x in n)
    nf = 64
    psi, _, _ = synth.gaussian_orbitals(n, ll, nf, 1001)
    V = synth.gaussian_wells(n, ll, 8, 1001)
    ctx = capi.Context(n, ll)
    dpsi, dV = _dev(psi), _dev(V)
    hp = ctx.hpsi(dpsi, dV, capi.LAP_MEHR4, True)
    hp_ref = O.hpsi(n, ll, 0, psi, V)
    assert rel_err(hp.cpu().numpy(), hp_ref) < TOL_F64
    S = ctx.gram(dpsi).cpu().numpy()
    H = ctx.hmat(dpsi, hp).cpu().numpy()
    B = ctx.matb(dpsi).cpu().numpy()
    S_ref = O.gram(psi, ctx.vel)
    H_ref = O.hmat(psi, hp_ref, ctx.vel)
    assert rel_err(S, S_ref) < TOL_F64
    assert rel_err(H, H_ref) < TOL_F64
    assert rel_err(B, O.matb(n, ll, psi)) < TOL_F64
    # the residual with theta = S^-1 H, then the V-cycle on it
    Sinv = np.linalg.inv(S_ref)
    th = O.theta(Sinv, H_ref)
    res = ctx.residual(dpsi, hp, _dev(th))
    res_ref = O.residual(n, ll, psi, hp_ref, th)
    assert rel_err(res.cpu().numpy(), res_ref) < TOL_F64
    gamma = ctx.gamma(capi.LAP_MEHR4, 2, float(V.max()), float(V.min()))
    out = ctx.precond_mg(_dev(res_ref), capi.LAP_MEHR4, 2, gamma).cpu().numpy()
    assert rel_err(out, O.precond(n, ll, 0, 2, gamma, res_ref)) < TOL_F64


def test_c2_mixed_products_at_the_stated_size():
    n = (128, 128, 128)
    ll = tuple(0.3 * x for x in n)
    nf = 512
    ctx = capi.Context(n, ll)
    psi64, _, _ = synth.gaussian_orbitals_device(n, ll, nf, 1002, torch.float64)
    V64 = synth.gaussian_wells_device(n, ll, 32, 1002)
    psi32 = psi64.float()
    hp64 = ctx.hpsi(psi64, V64, capi.LAP_8TH, False)
    hp32 = ctx.hpsi(psi32, V64.float(), capi.LAP_8TH, False)
    e_h = float((hp32.double() - hp64).abs().max() / hp64.abs().max())
    assert e_h < 2e-6
    # the FP64 path (FP64 orbitals), and FP64 products of the FP32 blocks
    # (the product error alone)
    S_all, H_all = ctx.gram_hmat(psi64, hp64, capi.GEMM_FP64)
    del psi64, hp64
    S64, H64 = ctx.gram_hmat(psi32.double(), hp32.double(), capi.GEMM_FP64)
    sc, hc = float(S64.abs().max()), float(H64.abs().max())
    for mode, tol in ((capi.GEMM_BF16X3, 3e-5), (capi.GEMM_TF32, 1e-3)):
        S, H = ctx.gram_hmat(psi32, hp32, mode)
        for Sr, Hr in ((S64, H64), (S_all, H_all)):
            assert float((S - Sr).abs().max()) / sc < tol, mode
            assert float((H - Hr).abs().max()) / hc < tol, mode
        assert torch.equal(S, S.T)
        del S, H
    # FP32 products on the CUDA cores: 8-term chains, 128-term FP32 sums,
    # double-float totals
    S, H = ctx.gram_hmat(psi32, hp32, capi.GEMM_FP32)
    assert float((S - S64).abs().max()) / sc < 1e-7
    assert float((H - H64).abs().max()) / hc < 1e-7
    del S, H
    L = torch.tril(ctx.cholesky(S_all.clone()))
    assert float((L @ L.T - S_all).abs().max()) / sc < 1e-14


def test_c3_masks_bit_exact_at_the_stated_size():
    n = (160, 160, 160)
    ll = tuple(0.3 * x for x in n)
    nf = 1536
    rng = np.random.default_rng(1003)
    centers = rng.uniform(0.0, 1.0, size=(nf, 3)) * np.asarray(ll)[None, :]
    radii = synth.mask_radii(nf, 1003, 4.0, 8.0)
    ctx = capi.Context(n, ll)
    M = capi.Masks(ctx, 1, centers, radii, func=0, kind=0, dtype=torch.float32)
    st, dense = M.expand(0)
    for f0 in range(0, nf, 256):
        f1 = min(nf, f0 + 256)
        st_ref, vals_ref = O.mask_build(n, ll, 1, 1, centers[f0:f1], radii[f0:f1], func=0,
                                        dtype=np.float32)
        assert np.array_equal(st[f0:f1], st_ref[0])
        assert torch.equal(dense[f0:f1], torch.from_numpy(vals_ref[0]).cuda()), (f0, f1)
        del vals_ref


def test_c3_local_step_at_the_stated_size():
    """The fused localized step for 12 of the configuration's orbitals on
    the 160^3 grid against the whole-grid oracle chain (H psi, residual with
    the correction mask, two masked Jacobi sweeps)."""
    n = (160, 160, 160)
    ll = tuple(0.3 * x for x in n)
    nf = 12
    psi, centers, _ = synth.gaussian_orbitals(n, ll, nf, 1003)
    radii = synth.mask_radii(nf, 1003, 4.0, 8.0)
    ctx = capi.Context(n, ll)
    masks = capi.Masks(ctx, 1, centers, radii, func=0, kind=0, dtype=torch.float32)
    corr = capi.Masks(ctx, 1, centers, radii, func=1, kind=1, dtype=torch.float32)
    loc = capi.Local(ctx, masks, corr)
    V = synth.gaussian_wells(n, ll, 32, 1003).astype(np.float32)
    phi = 0.6 * psi + 0.1 * np.roll(psi, 1, axis=0)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()  # noqa: E731
    psi_p = loc.gather(f32(psi))
    phi_p = loc.gather(f32(phi))
    gamma = ctx.gamma(0, 2, float(V.max()), -0.5)
    u_p, w_p = loc.step(psi_p, phi_p, f32(V), gamma)
    u = loc.scatter(u_p).cpu().numpy()
    w = loc.scatter(w_p).cpu().numpy()
    psi0 = loc.scatter(psi_p).cpu().numpy().astype(np.float64)
    phi0 = loc.scatter(phi_p).cpu().numpy().astype(np.float64)
    st_o, v_o = O.mask_build(n, ll, 1, 1, centers, radii, func=0)
    st_c, v_c = O.mask_build(n, ll, 1, 1, centers, radii, func=1)
    r0 = O.mask_apply(n, 0, st_c, v_c,
                      O.rhs_mehr(n, ll, phi0) - O.hpsi(n, ll, 0, psi0, V.astype(np.float64)), kind=1)
    jf = O.jacobi_factor(n, ll, 0)
    u1 = O.mask_apply(n, 0, st_o, v_o, gamma * r0 - jf * (O.fd_apply(n, ll, 0, gamma * r0) - r0),
                      kind=0)
    w1 = O.fd_apply(n, ll, 0, u1) - r0
    u2 = O.mask_apply(n, 0, st_o, v_o, u1 - jf * w1, kind=0)
    w2 = O.mask_apply(n, 0, st_o, v_o, O.fd_apply(n, ll, 0, u1) - r0, kind=0)
    assert rel_err(u, u2) < 1e-4
    assert rel_err(w, w2) < 1e-4
