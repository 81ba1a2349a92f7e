"""Theta, Psi Theta and the residual (computeResidualUsingHPhi) on the GPU
vs the oracle.

Error bars, relative to max |reference|:
  FP64 mode, FP64 orbitals                                    <= 1e-12
  FP64 mode, FP32 orbitals (FP64 accumulation, FP32 result)   <= 3e-7
  FP32 CUDA-core mode (FP32 FMA)                              <= 2e-5
  BF16X3 tensor cores                                         <= 6e-5
  FP16X3 tensor cores (scaled fp16 hi / lo, 2^-22 split; the
  FP32 accumulation sets the bar)                             <= 5e-6
  TF32 tensor cores                                           <= 2e-3
The BF16X3 bar: each operand is hi + lo with |x - hi - lo| <= 2^-16 |x|
(bf16 unit roundoff 2^-8, twice), so one product carries up to ~2^-15
relative error; with theta close to diagonal a single term dominates each
output and nothing averages it out (the Gram sums over grid points do).
"""
import os

import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = {capi.GEMM_FP32: 2e-5, capi.GEMM_TF32: 2e-3, capi.GEMM_BF16X3: 6e-5,
       capi.GEMM_FP16X3: 5e-6}


def _dev(a, dt=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


def _theta(nf, seed):
    rng = np.random.default_rng(seed)
    return np.eye(nf) + rng.standard_normal((nf, nf)) / nf


def test_theta_reads_lower_triangle():
    n = 150
    rng = np.random.default_rng(150)
    A = rng.standard_normal((n, n))
    Sinv = A @ A.T / n + np.eye(n)
    H = rng.standard_normal((n, n))
    junk = np.tril(Sinv) + np.triu(np.full((n, n), 7.0), 1)
    ctx = capi.Context((8, 8, 8), (1, 1, 1))
    th = ctx.theta(_dev(junk), _dev(H)).cpu().numpy()
    assert rel_err(th, O.theta(Sinv, H)) < TOL_F64
    assert rel_err(th, Sinv @ H) < TOL_F64


@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 5), ((15, 13, 11), 70), ((16, 16, 16), 130)])
def test_mult_matrix_fp64(grid, nf):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 31)
    th = _theta(nf, 31)
    ctx = capi.Context(grid, ll)
    out = ctx.mult_matrix(_dev(psi), _dev(th)).cpu().numpy()
    assert rel_err(out, O.mult_matrix(psi, th)) < TOL_F64


def test_mult_matrix_fp32_orbitals_fp64_accumulation():
    grid, nf = (16, 16, 16), 96
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 4)
    p32 = psi.astype(np.float32)
    th = _theta(nf, 4)
    ctx = capi.Context(grid, ll)
    out = ctx.mult_matrix(_dev(p32, np.float32), _dev(th)).cpu().numpy()
    ref = O.mult_matrix(p32, th)
    assert ref.dtype == np.float32
    assert rel_err(out, ref) < 3e-7


@pytest.mark.parametrize("mode", [capi.GEMM_FP32, capi.GEMM_TF32, capi.GEMM_BF16X3,
                                  capi.GEMM_FP16X3])
@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 64), ((15, 13, 11), 37), ((32, 24, 20), 200),
                                     ((20, 20, 20), 300)])
def test_mult_matrix_fp32_modes(mode, grid, nf):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 8)
    p32 = psi.astype(np.float32)
    th = _theta(nf, 8)
    ctx = capi.Context(grid, ll)
    out = ctx.mult_matrix(_dev(p32, np.float32), _dev(th), mode=mode).cpu().numpy()
    ref = O.mult_matrix(p32.astype(np.float64), th)
    assert rel_err(out, ref) < TOL[mode]


def test_mult_matrix_tc_chunks_match():
    """Point chunks of the tensor-core product give the same bits as one pass."""
    grid, nf = (24, 24, 20), 260
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 12)
    p = _dev(psi, np.float32)
    th = _dev(_theta(nf, 12))
    ctx = capi.Context(grid, ll)
    one = ctx.mult_matrix(p, th, mode=capi.GEMM_BF16X3)
    os.environ["MGX_PSI_THETA_CHUNK"] = "1000"   # 8 tiles of 128 points per chunk
    try:
        many = ctx.mult_matrix(p, th, mode=capi.GEMM_BF16X3)
    finally:
        del os.environ["MGX_PSI_THETA_CHUNK"]
    assert torch.equal(one, many)


@pytest.mark.parametrize("apply_B", [1, 0])
@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 8), ((15, 13, 11), 70)])
def test_residual_fp64(apply_B, grid, nf):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 21)
    V = synth.gaussian_wells(grid, ll, 5, 21)
    hp = O.hpsi(grid, ll, 0, psi, V)
    th = _theta(nf, 21)
    ref = O.residual(grid, ll, psi, hp, th, apply_B)
    ctx = capi.Context(grid, ll)
    res = ctx.residual(_dev(psi), _dev(hp), _dev(th), apply_B=apply_B).cpu().numpy()
    assert rel_err(res, ref) < TOL_F64
    # in place on hpsi, with a caller work block
    hd = _dev(hp)
    work = torch.empty_like(hd)
    ctx.residual(_dev(psi), hd, _dev(th), apply_B=apply_B, work=work, out=hd)
    assert rel_err(hd.cpu().numpy(), ref) < TOL_F64


@pytest.mark.parametrize("mode", [capi.GEMM_FP64, capi.GEMM_FP32, capi.GEMM_BF16X3,
                                  capi.GEMM_FP16X3])
def test_residual_fp32(mode):
    grid, nf = (16, 16, 16), 130
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 22)
    V = synth.gaussian_wells(grid, ll, 5, 22)
    p32 = psi.astype(np.float32)
    hp = O.hpsi(grid, ll, 0, p32, V).astype(np.float32)
    th = _theta(nf, 22)
    ref = O.residual(grid, ll, p32.astype(np.float64), hp.astype(np.float64), th, 1)
    ctx = capi.Context(grid, ll)
    res = ctx.residual(_dev(p32, np.float32), _dev(hp, np.float32), _dev(th), mode=mode).cpu().numpy()
    scale = max(np.max(np.abs(ref)), np.max(np.abs(hp)))
    err = np.max(np.abs(res - ref)) / scale
    assert err < (3e-7 if mode == capi.GEMM_FP64 else TOL[mode])


@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 40), ((32, 24, 20), 300), ((10, 12, 14), 70)])
def test_psi_theta_reuses_gram_conversion(grid, nf):
    """With mgx_set_reuse_conversion on, Psi Theta reads the Gram product's
    BF16 planes of the same block as an MN-major operand; the result is that
    of the converting path.  Another block is not taken for the converted
    one."""
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 29)
    p32 = psi.astype(np.float32)
    ctx = capi.Context(grid, ll)
    d = _dev(p32, np.float32)
    th = _theta(nf, 30)
    thd = _dev(th)
    l0 = capi.launches()
    ref = ctx.mult_matrix(d, thd, capi.GEMM_BF16X3).cpu().numpy()
    n_convert = capi.launches() - l0
    ctx.set_reuse_conversion(True)
    ctx.gram(d, capi.GEMM_BF16X3)
    l0 = capi.launches()
    got = ctx.mult_matrix(d, thd, capi.GEMM_BF16X3).cpu().numpy()
    # the reusing product launches no conversion of psi
    assert capi.launches() - l0 < n_convert
    assert rel_err(got, ref) < 1e-6
    assert rel_err(got, O.mult_matrix(p32, th)) < TOL[capi.GEMM_BF16X3]
    # column chunks of the residual read the same planes
    hp = _dev(O.hpsi(grid, ll, 0, p32, synth.gaussian_wells(grid, ll, 3, 29)), np.float32)
    full = ctx.residual(d, hp, thd, capi.GEMM_BF16X3).cpu().numpy()
    thc = torch.from_numpy(np.ascontiguousarray(th.T)).cuda()
    part = ctx.residual_cols(d, hp[: nf // 2], thc[: nf // 2].contiguous(), capi.GEMM_BF16X3)
    assert rel_err(part.cpu().numpy(), full[: nf // 2]) < 1e-6
    ref_res = O.residual(grid, ll, p32, hp.cpu().numpy(), th)
    assert rel_err(full, ref_res) < TOL[capi.GEMM_BF16X3]
    # a different block goes through its own conversion
    d2 = 2 * d
    got2 = ctx.mult_matrix(d2, thd, capi.GEMM_BF16X3).cpu().numpy()
    assert rel_err(got2, 2 * ref) < 1e-6


def test_residual_rejects_aliases():
    grid, nf = (8, 8, 8), 3
    ctx = capi.Context(grid, (2.8, 2.8, 2.8))
    a = torch.zeros((nf, 512), dtype=torch.float64, device="cuda")
    b = torch.zeros_like(a)
    th = torch.eye(nf, dtype=torch.float64, device="cuda")
    with pytest.raises(capi.MgxError):
        ctx.residual(a, b, th, out=a)
    with pytest.raises(capi.MgxError):
        ctx.residual(a, b, th, work=b)
    with pytest.raises(capi.MgxError):
        ctx.mult_matrix(a, th, mode=capi.GEMM_BF16X3)   # needs FP32 orbitals


def _oracle_step(grid, ll, psi, V, alpha, gamma, lap_type=0):
    """The reference's iteration as a chain of oracle calls: normalize, then
    H psi, S, H, (Mehrstellen) B; S^-1; theta = B^-1 H and HB = sym(S theta)
    (Mehrstellen) or theta = S^-1 H and HB = H; energy tr(HB S^-1);
    residual, V-cycle, update."""
    vel = np.prod([l / n for l, n in zip(ll, grid)])
    psi, _ = O.normalize(grid, ll, psi)
    hp = O.hpsi(grid, ll, lap_type, psi, V)
    S = O.gram(psi, vel)
    H = O.hmat(psi, hp, vel)
    info, L = O.potrf(S)
    assert info == 0
    Sinv = O.inverse_from_chol(L)
    if lap_type == 0:
        B = O.matb(grid, ll, psi)
        info, LB = O.potrf(B)
        assert info == 0
        th = O.theta(O.inverse_from_chol(LB), H)
        e = O.trace_prod(O.update_hb(S, th), Sinv)
    else:
        th = O.theta(Sinv, H)
        e = O.trace_prod(H, Sinv)
    res = O.residual(grid, ll, psi, hp, th, 1 if lap_type == 0 else 0)
    corr = O.precond(grid, ll, lap_type, 2, gamma, res)
    return psi + alpha * corr, e, res, corr


@pytest.mark.parametrize("fuse", [False, True])
def test_abpg_step_fp64_matches_oracle_chain(fuse):
    """One full sweep (normalize, H psi, S / H / B, Cholesky, inverses,
    theta = B^-1 H, HB, energy, residual, V-cycle, update) in FP64 against
    the same chain of oracle calls; fused, the normalization rides on the
    update."""
    from mgmol_gb300.sweep import OrbitalSweep
    grid, nf = (16, 16, 16), 12
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 41, sigma=(0.9, 1.3))
    psi = psi * np.linspace(0.7, 1.6, nf)[:, None]      # not normalized on entry
    V = synth.gaussian_wells(grid, ll, 4, 41)
    ctx = capi.Context(grid, ll)
    sw = OrbitalSweep(ctx, torch.from_numpy(V), nf, mode="plain", maxlevels=2, fuse_update=fuse)
    pd = _dev(psi)
    e = float(sw.run(pd).cpu()[0])
    ref, e_ref, res, corr = _oracle_step(grid, ll, psi, V, sw.alpha, sw.gamma)
    assert abs(e - e_ref) < 1e-11 * abs(e_ref)
    if not fuse:
        assert rel_err(sw.hpsi.cpu().numpy(), res) < TOL_F64
        assert rel_err(sw.corr.cpu().numpy(), corr) < TOL_F64
    assert rel_err(pd.cpu().numpy(), ref) < TOL_F64


def test_abpg_anderson_steps_match_oracle_chain():
    """Four ABPG steps with Anderson extrapolation (m = 2, the accelerated
    branch of update_states) in FP64 against the oracle chain with its own
    stateful AndersonMix; the blocks are normalized before every step as
    the reference does, so the history holds unnormalized iterates."""
    from mgmol_gb300.sweep import OrbitalSweep
    grid, nf = (16, 16, 16), 8
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 44, sigma=(0.9, 1.3))
    V = synth.gaussian_wells(grid, ll, 4, 44)
    ctx = capi.Context(grid, ll)
    sw = OrbitalSweep(ctx, torch.from_numpy(V), nf, mode="plain", maxlevels=2, anderson_m=2)
    assert not sw.fuse_update
    pd = _dev(psi)
    x = np.ascontiguousarray(psi.copy())
    mix = O.AndersonState(2, 1.0, x.shape, np.float64)
    vel = ctx.vel
    for step in range(4):
        e = float(sw.run(pd).cpu()[0])
        x[:] = O.normalize(grid, ll, x)[0]
        hp = O.hpsi(grid, ll, 0, x, V)
        S = O.gram(x, vel)
        H = O.hmat(x, hp, vel)
        Sinv = O.inverse_from_chol(O.potrf(S)[1])
        th = O.theta(O.inverse_from_chol(O.potrf(O.matb(grid, ll, x))[1]), H)
        e_ref = O.trace_prod(O.update_hb(S, th), Sinv)
        corr = O.precond(grid, ll, 0, 2, sw.gamma, O.residual(grid, ll, x, hp, th, 1))
        mix.step(x, corr, vel, np.diag(Sinv), sw.alpha)
        assert abs(e - e_ref) < 1e-11 * abs(e_ref), step
        assert rel_err(pd.cpu().numpy(), x) < 1e-11, step
    mix.close()
    assert sw.last_mix["mm"] >= 1


def test_abpg_step_other_operator_matches_oracle_chain():
    """lap_type 2 (4th order, no B): theta = S^-1 H, HB = H, res = psi theta - H psi."""
    from mgmol_gb300.sweep import OrbitalSweep
    grid, nf = (16, 16, 16), 10
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 42, sigma=(0.9, 1.3))
    V = synth.gaussian_wells(grid, ll, 4, 42)
    ctx = capi.Context(grid, ll)
    sw = OrbitalSweep(ctx, torch.from_numpy(V), nf, mode="plain", lap_type=2, maxlevels=2)
    pd = _dev(psi)
    e = float(sw.run(pd).cpu()[0])
    ref, e_ref, _, _ = _oracle_step(grid, ll, psi, V, sw.alpha, sw.gamma, lap_type=2)
    assert abs(e - e_ref) < 1e-11 * abs(e_ref)
    assert rel_err(pd.cpu().numpy(), ref) < TOL_F64


@pytest.mark.parametrize("mode,gemm", [("plain", capi.GEMM_FP64), ("mixed", capi.GEMM_BF16X3)])
def test_abpg_step_lean_schedule_matches_full(mode, gemm):
    """The column-chunked schedule (residual / preconditioner over chunks of
    output functions) and the schedule with the update fused into the
    preconditioner move psi as the full-block schedule does."""
    from mgmol_gb300.sweep import OrbitalSweep
    grid, nf = (16, 16, 16), 12
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 43, sigma=(0.9, 1.3))
    psi = O.normalize(grid, ll, psi)[0]
    V = torch.from_numpy(synth.gaussian_wells(grid, ll, 4, 43))
    dt = np.float64 if mode == "plain" else np.float32
    ctx = capi.Context(grid, ll)
    a, b = _dev(psi, dt), _dev(psi, dt)
    full = OrbitalSweep(ctx, V, nf, mode=mode, gemm=gemm, maxlevels=2, fuse_update=False)
    fused = OrbitalSweep(ctx, V, nf, mode=mode, gemm=gemm, maxlevels=2)
    lean = OrbitalSweep(ctx, V, nf, mode=mode, gemm=gemm, maxlevels=2, chunk_funcs=5)
    c = _dev(psi, dt)
    ea = float(full.run(a).cpu()[0])
    eb = float(lean.run(b).cpu()[0])
    fused.run(c)
    # the split-K Gram sums K slices with atomics, so S and H (and what
    # follows) agree to rounding between runs, not bit for bit
    assert abs(ea - eb) <= 1e-13 * abs(ea)
    tol = 1e-12 if mode == "plain" else 1e-6
    assert rel_err(b.cpu().numpy(), a.cpu().numpy()) < tol
    assert rel_err(lean.correction().cpu().numpy(), full.correction().cpu().numpy()) < tol * 100
    # the update fused into the last smoothing sweep moves psi the same way;
    # its normalization factors come from the diagonal of the step's own
    # Gram matrix, whose product error (BF16X3: ~1e-6) scales whole columns,
    # so the blocks are compared after normalizing both
    na = O.normalize(grid, ll, a.cpu().numpy().astype(np.float64))[0]
    nc = O.normalize(grid, ll, c.cpu().numpy().astype(np.float64))[0]
    assert rel_err(nc, na) < (1e-12 if mode == "plain" else 1e-6)
