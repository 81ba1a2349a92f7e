"""Gram / H matrices, FP64 Cholesky, inverse and trace on the GPU vs the
oracle and the restated tests/testGramMatrix.cc checks."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


@pytest.mark.parametrize("n,nf", [((16, 16, 16), 5), ((32, 24, 16), 70), ((16, 16, 16), 130)])
def test_gram_hmat_fp64(n, nf):
    ll = tuple(x * 0.35 for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, nf, 17)
    V = synth.gaussian_wells(n, ll, 8, 17)
    ctx = capi.Context(n, ll)
    S = ctx.gram(_dev(psi)).cpu().numpy()
    S_ref = O.gram(psi, ctx.vel)
    assert rel_err(S, S_ref) < TOL_F64
    assert np.array_equal(S, S.T)
    hp = O.hpsi(n, ll, 0, psi, V)
    H = ctx.hmat(_dev(psi), _dev(hp)).cpu().numpy()
    assert rel_err(H, O.hmat(psi, hp, ctx.vel)) < TOL_F64


def test_gram_fp32_cuda_cores():
    n, nf = (32, 32, 32), 40
    ll = tuple(x * 0.3 for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, nf, 3)
    ctx = capi.Context(n, ll)
    S = ctx.gram(_dev(psi, np.float32), mode=capi.GEMM_FP32).cpu().numpy()
    S_ref = O.gram(psi.astype(np.float32), ctx.vel)
    # FP32 products: 8-term chains, 128-term FP32 sums, double-float total
    assert rel_err(S, S_ref) < 1e-8


def test_cholesky_inverse_trace():
    """testGramMatrix.cc restated: n = 213, L L^T = S to 1e-14, S^-1 S = I."""
    n = 213
    rng = np.random.default_rng(213)
    A = rng.standard_normal((n, n))
    S = A @ A.T / n + np.eye(n)
    ctx = capi.Context((8, 8, 8), (1, 1, 1))
    L = ctx.cholesky(_dev(S)).cpu().numpy()
    assert np.max(np.abs(np.triu(L, 1))) == 0.0
    assert np.max(np.abs(L @ L.T - S)) <= 1e-14 * np.max(np.abs(S)) * n
    info, L_ref = O.potrf(S)
    assert rel_err(L, L_ref) < 1e-12
    Sinv = ctx.inverse_from_cholesky(_dev(L)).cpu().numpy()
    assert np.max(np.abs(Sinv @ S - np.eye(n))) < 1e-12
    H = rng.standard_normal((n, n))
    H = H + H.T
    tr = float(ctx.trace_prod(_dev(H), _dev(Sinv)).cpu()[0])
    ref = O.trace_prod(H, Sinv)
    assert abs(tr - ref) < 1e-12 * max(1.0, abs(ref))


def test_cholesky_reports_not_spd():
    n = 100
    S = np.eye(n)
    S[70, 70] = -2.0
    ctx = capi.Context((8, 8, 8), (1, 1, 1))
    with pytest.raises(capi.MgxError) as e:
        ctx.cholesky(_dev(S))
    assert e.value.status == capi.MGX_NOT_SPD
    assert "71" in str(e.value)
    # the context stays usable
    L = ctx.cholesky(_dev(np.eye(n) * 4.0)).cpu().numpy()
    assert np.allclose(L, 2.0 * np.eye(n))


@pytest.mark.parametrize("n", [64, 130, 512])
def test_gram_pipeline_on_orbitals(n):
    grid = (16, 16, 16)
    ll = (5.6, 5.6, 5.6)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, n, 5, sigma=(0.8, 1.2))
    ctx = capi.Context(grid, ll)
    S = ctx.gram(_dev(psi))
    S_np = S.cpu().numpy()
    w = np.linalg.eigvalsh(S_np)
    if w[0] <= 0:
        pytest.skip("random orbitals not independent at this size")
    L = ctx.cholesky(S)
    Sinv = ctx.inverse_from_cholesky(L).cpu().numpy()
    assert np.max(np.abs(Sinv @ S_np - np.eye(n))) < 1e-9 * np.linalg.cond(S_np)


@pytest.mark.parametrize("n", [64, 213, 512])
def test_theta_from_cholesky(n):
    """theta = S^-1 H by substitution equals the inverse-then-multiply path
    (GramMatrix::computeInverse + ProjectedMatrices::updateTheta) and its
    trace the energy tr(S^-1 H)."""
    rng = np.random.default_rng(n)
    A = rng.standard_normal((n, n))
    S = A @ A.T / n + np.eye(n)
    H = rng.standard_normal((n, n))
    H = H + H.T
    ctx = capi.Context((8, 8, 8), (1, 1, 1))
    L = ctx.cholesky(_dev(S))
    th, tr = ctx.theta_from_cholesky(L, _dev(H))
    Sinv = O.inverse_from_chol(L.cpu().numpy())
    ref = O.theta(Sinv, H)
    assert rel_err(th.cpu().numpy(), ref) < 1e-12 * max(1.0, np.linalg.cond(S) / 10)
    t = float(tr.cpu()[0])
    tref = O.trace_prod(H, Sinv)
    assert abs(t - tref) < 1e-12 * max(1.0, abs(tref)) * n


@pytest.mark.parametrize("case", ["a", "b"])
def test_gram_hmat_match_reference_golden(case):
    """The GPU's FP64 S and H against the reference's own getLocalOverlap /
    computeLocalProduct and LocalMatrices2DistMatrix (recorded vectors):
    1e-12 relative and the same entries dropped by the 1e-14 filter; for
    FP32 orbitals (split-BF16x3 on the tensor cores) the product tolerance,
    against the reference's USE_MP matrices."""
    from helpers import golden
    g = golden()
    n = tuple(int(x) for x in g[f"sh{case}_n"])
    ll = tuple(float(x) for x in g[f"sh{case}_ll"])
    ctx = capi.Context(n, ll)
    psi = g[f"sh{case}_psi"]
    S = ctx.gram(_dev(psi)).cpu().numpy()
    H = ctx.hmat(_dev(psi), _dev(g[f"sh{case}_hpsi_d"])).cpu().numpy()
    S_ref, H_ref = g[f"sh{case}_S_d"], g[f"sh{case}_H_d"]
    assert rel_err(S, S_ref) < TOL_F64
    assert rel_err(H, H_ref) < TOL_F64
    assert np.array_equal(S == 0, S_ref == 0)
    assert np.array_equal(H == 0, H_ref == 0)
    p32 = _dev(psi, np.float32)
    S32 = ctx.gram(p32, mode=capi.GEMM_BF16X3).cpu().numpy()
    H32 = ctx.hmat(p32, _dev(g[f"sh{case}_hpsi_f"], np.float32), mode=capi.GEMM_BF16X3).cpu().numpy()
    assert rel_err(S32, g[f"sh{case}_S_f"]) < 2e-5
    assert rel_err(H32, g[f"sh{case}_H_f"]) < 2e-5
