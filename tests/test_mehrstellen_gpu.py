"""The Mehrstellen projected matrices and the normalization on the GPU vs
the oracle: computeMatB (B = Psi^T (B Psi) vel), updateHB, normalize, the
normalization factors from the Gram diagonal, and the update with a column
scale folded in.

Error bars (relative to max |reference|) are those of the products:
FP64 mode 1e-12; FP32 CUDA cores 2e-5; tensor-core modes as in the Gram
tests (TF32 2e-3, BF16X3 2e-5, FP16X3 5e-6).  The normalization of FP64
blocks agrees to 1e-12 (the device sums the squares in another order, a
tree instead of the reference's sequential loop, which moves diagS and its
inverse square root by up to ~P ulps for P points); FP32 blocks to one FP32
ulp.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = {capi.GEMM_FP64: TOL_F64, capi.GEMM_FP32: 2e-5, capi.GEMM_TF32: 2e-3,
       capi.GEMM_BF16X3: 2e-5, capi.GEMM_FP16X3: 5e-6}


def _dev(a, dt):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


def _setup(grid, nf, seed):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, seed, sigma=(0.9, 1.3))
    return ll, psi, capi.Context(grid, ll)


@pytest.mark.parametrize("mode", sorted(TOL))
@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 24), ((32, 24, 20), 150), ((10, 12, 14), 20)])
def test_matb_matches_oracle(mode, grid, nf):
    """(10, 12, 14): points not a multiple of 64 and rows not of whole
    vectors, so B Psi is formed in FP32 and split afterwards; the others
    write the BF16 planes from the stencil directly."""
    ll, psi, ctx = _setup(grid, nf, 61)
    dt = np.float64 if mode == capi.GEMM_FP64 else np.float32
    p = psi.astype(dt)
    B = ctx.matb(_dev(p, dt), mode=mode).cpu().numpy()
    ref = O.matb(grid, ll, p)
    assert np.array_equal(B, B.T)
    # the device forms the lower triangle; the oracle both
    assert rel_err(np.tril(B), np.tril(ref)) < TOL[mode]
    assert rel_err(B, ref) < max(TOL[mode], 1e-7 if dt == np.float32 else 0)


@pytest.mark.parametrize("mode", [capi.GEMM_FP64, capi.GEMM_BF16X3, capi.GEMM_FP16X3])
def test_matb_work_blocks_and_chunks(mode):
    """B Psi formed in the caller's block, in a 7-function block, and in the
    context's block (more than 512 functions: several chunks) agree."""
    grid, nf = (16, 16, 16), 600
    ll, psi, ctx = _setup(grid, nf, 62)
    dt = np.float64 if mode == capi.GEMM_FP64 else np.float32
    p = _dev(psi, dt)
    a = ctx.matb(p, mode=mode).cpu().numpy()
    b = ctx.matb(p, mode=mode, work=torch.empty_like(p)).cpu().numpy()
    c = ctx.matb(p, mode=mode, work=torch.empty_like(p[:7])).cpu().numpy()
    tol = 1e-13 if mode == capi.GEMM_FP64 else 1e-6
    assert rel_err(b, a) < tol and rel_err(c, a) < tol
    ref = O.matb(grid, ll, psi.astype(dt))
    assert rel_err(np.tril(a), np.tril(ref)) < TOL[mode]


@pytest.mark.parametrize("mode", [capi.GEMM_FP64, capi.GEMM_FP32, capi.GEMM_BF16X3])
def test_gram_hmat_matb_equals_separate(mode):
    grid, nf = (20, 20, 20), 130
    ll, psi, ctx = _setup(grid, nf, 63)
    V = synth.gaussian_wells(grid, ll, 4, 63)
    dt = np.float64 if mode == capi.GEMM_FP64 else np.float32
    p = _dev(psi, dt)
    hp = ctx.hpsi(p, torch.from_numpy(V).cuda().to(p.dtype))
    S, H, B = ctx.gram_hmat_matb(p, hp, mode=mode, work=torch.empty_like(p))
    tol = 1e-13 if mode == capi.GEMM_FP64 else 1e-6
    assert rel_err(S.cpu().numpy(), ctx.gram(p, mode).cpu().numpy()) < tol
    assert rel_err(H.cpu().numpy(), ctx.hmat(p, hp, mode).cpu().numpy()) < tol
    assert rel_err(B.cpu().numpy(), ctx.matb(p, mode).cpu().numpy()) < tol


def test_matb_rejects_bad_work():
    grid, nf = (16, 16, 16), 8
    ll, psi, ctx = _setup(grid, nf, 64)
    p = _dev(psi, np.float64)
    with pytest.raises(capi.MgxError):
        ctx.matb(p, mode=capi.GEMM_FP64, work=p)


def test_update_hb_matches_oracle():
    rng = np.random.default_rng(65)
    n = 200
    A = rng.standard_normal((n, n))
    S = A @ A.T / n + np.eye(n)
    th = rng.standard_normal((n, n))
    ctx = capi.Context((16, 16, 16), (5.6,) * 3)
    S_low = np.tril(S) + np.triu(rng.standard_normal((n, n)), 1)  # upper part unread
    hb = ctx.update_hb(_dev(S_low, np.float64), _dev(th, np.float64)).cpu().numpy()
    ref = O.update_hb(S_low, th)
    assert np.array_equal(hb, hb.T)
    assert rel_err(hb, ref) < TOL_F64


@pytest.mark.parametrize("dt", [np.float64, np.float32])
def test_normalize_matches_oracle(dt):
    grid, nf = (24, 16, 20), 9
    ll, psi, ctx = _setup(grid, nf, 66)
    p = (3.0 * psi).astype(dt)
    d = _dev(p, dt)
    diag = ctx.normalize(d).cpu().numpy()
    ref, rdiag = O.normalize(grid, ll, p)
    # a sequential and a tree sum of P squares differ by up to ~P ulps in the
    # worst case (the reference's own sum carries that error)
    assert rel_err(diag, rdiag) < 1e-12
    got = d.cpu().numpy()
    if dt == np.float64:
        # alpha = diagS^-1/2 carries the relative error of the reordered sum
        assert rel_err(got, ref) < 1e-12
    else:
        # FP32: the same rounding of alpha * x, alpha equal to ~1e-16
        ulp = np.spacing(np.abs(ref).astype(np.float32))
        assert np.all(np.abs(got - ref) <= ulp)
    # normalized: vel |psi_i|^2 = 1
    again = ctx.normalize(d).cpu().numpy()
    assert np.max(np.abs(again - 1.0)) < (1e-12 if dt == np.float64 else 1e-6)


def test_normalize_rejects_zero_function():
    grid, nf = (16, 16, 16), 4
    ll, psi, ctx = _setup(grid, nf, 67)
    psi[2] = 0.0
    d = _dev(psi, np.float64)
    with pytest.raises(capi.MgxError) as e:
        ctx.normalize(d)
    assert e.value.status == capi.MGX_NOT_SPD
    assert np.array_equal(d.cpu().numpy(), psi)


def test_normalize_scales_from_gram():
    grid, nf = (16, 16, 16), 10
    ll, psi, ctx = _setup(grid, nf, 68)
    p = _dev(2.5 * psi, np.float64)
    S = ctx.gram(p)
    d = ctx.normalize_scales(S).cpu().numpy()
    _, diag = O.normalize(grid, ll, 2.5 * psi)
    assert rel_err(d, 1.0 / np.sqrt(diag)) < 1e-12


@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-13), (np.float32, 2e-6)])
def test_precond_update_with_column_scale(dt, tol):
    """psi_j <- d_j (psi_j + alpha P(res)_j) equals V-cycle, axpy and scale."""
    grid, nf = (16, 16, 16), 6
    ll, psi, ctx = _setup(grid, nf, 69)
    res, _, _ = synth.gaussian_orbitals(grid, ll, nf, 70)
    r = _dev(res, dt)
    scale = torch.linspace(0.5, 1.5, nf, dtype=torch.float64, device="cuda")
    got = _dev(psi, dt)
    ctx.precond_update(r, got, 0.5, 0, 2, 0.3, psi_scale=scale)
    corr = ctx.precond_mg(r, 0, 2, 0.3).cpu().numpy().astype(np.float64)
    ref = scale.cpu().numpy()[:, None] * (psi.astype(dt).astype(np.float64) + 0.5 * corr)
    assert rel_err(got.cpu().numpy(), ref) < tol
    # no coarse levels: the update (and its scale) sits in the only sweep
    got0 = _dev(psi, dt)
    ctx.precond_update(r, got0, 0.5, 0, 0, 0.3, psi_scale=scale)
    corr0 = ctx.precond_mg(r, 0, 0, 0.3).cpu().numpy().astype(np.float64)
    ref0 = scale.cpu().numpy()[:, None] * (psi.astype(dt).astype(np.float64) + 0.5 * corr0)
    assert rel_err(got0.cpu().numpy(), ref0) < tol
