"""The electronic density (mgx_rho, Rho<T>::computeRho for non-orthogonal
orbitals with the reference's charge rescaling) on the GPU vs the oracle,
which the reference vectors pin bit for bit.

Error bars (relative to max |rho|): FP64 products 1e-12; FP32 orbitals
with FP64 accumulation (the reference's MPgemmNN) 1e-6; tensor-core modes
those of the products (BF16X3 6e-5, FP16X3 5e-6, TF32 2e-3), reduced in
the product's epilogue.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = {capi.GEMM_FP32: 2e-5, capi.GEMM_TF32: 2e-3, capi.GEMM_BF16X3: 6e-5,
       capi.GEMM_FP16X3: 5e-6}


def _case(grid, nf, seed):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, seed, sigma=(0.9, 1.3))
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((nf, nf))
    X = 2.0 * (A @ A.T / nf + np.eye(nf)) / nf
    return ll, psi, X


@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 12), ((24, 16, 20), 70)])
def test_rho_fp64(grid, nf):
    ll, psi, X = _case(grid, nf, 81)
    ctx = capi.Context(grid, ll)
    rho, q = ctx.rho(torch.from_numpy(psi).cuda(), torch.from_numpy(X).cuda())
    ref, rq, _ = O.rho(grid, ll, psi, X)
    assert rel_err(rho.cpu().numpy(), ref) < 1e-12
    assert abs(q - rq) < 1e-12 * abs(rq)


@pytest.mark.parametrize("mode", [capi.GEMM_FP64, capi.GEMM_FP32, capi.GEMM_TF32,
                                  capi.GEMM_BF16X3, capi.GEMM_FP16X3])
@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 40), ((32, 24, 20), 300)])
def test_rho_fp32_modes(mode, grid, nf):
    ll, psi, X = _case(grid, nf, 82)
    ctx = capi.Context(grid, ll)
    p32 = psi.astype(np.float32)
    rho, _ = ctx.rho(torch.from_numpy(p32).cuda(), torch.from_numpy(X).cuda(), mode=mode)
    ref, _, _ = O.rho(grid, ll, p32, X)
    assert rel_err(rho.cpu().numpy(), ref) < (1e-6 if mode == capi.GEMM_FP64 else TOL[mode])


def test_rho_work_chunks_and_rescaling():
    grid, nf = (16, 16, 16), 30
    ll, psi, X = _case(grid, nf, 83)
    ctx = capi.Context(grid, ll)
    d = torch.from_numpy(psi).cuda()
    Xd = torch.from_numpy(X).cuda()
    a, q = ctx.rho(d, Xd)
    b, _ = ctx.rho(d, Xd, work=torch.empty_like(d[:7]))
    assert rel_err(b.cpu().numpy(), a.cpu().numpy()) < 1e-15
    # nel within 2 % of the charge: rescaled; beyond: refused, rho unscaled
    c, q2 = ctx.rho(d, Xd, nel=0.99 * q)
    assert abs(q2 - q) < 1e-12 * q
    assert rel_err(c.cpu().numpy(), 0.99 * a.cpu().numpy()) < 1e-14
    ref, _, _ = O.rho(grid, ll, psi, X, nel=0.99 * q)
    assert rel_err(c.cpu().numpy(), ref) < 1e-12
    with pytest.raises(capi.MgxError):
        ctx.rho(d, Xd, nel=1.5 * q)
