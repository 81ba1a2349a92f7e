"""Tensor-core (tcgen05) Gram / H matrices vs the FP64 oracle.

Error bars, relative to max |S| (resp. max |H|):
  TF32   (10-bit mantissa products, FP32 accumulation)        <= 2e-3
  BF16X3 (hi*hi + hi*lo + lo*hi, FP32 accumulation)           <= 2e-5
  FP16X3 (scaled fp16 hi / lo, split error 2^-22)             <= 5e-6
The FP16X3 bar is set by the FP32 accumulation over up to 32768 K
elements per output tile (measured 3.2e-6 at K = 65536), not by its split.
and the FP32 CUDA-core mode for comparison <= 1e-5.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = {capi.GEMM_TF32: 2e-3, capi.GEMM_BF16X3: 2e-5, capi.GEMM_FP16X3: 5e-6}


def _dev(a, dt=np.float32):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


@pytest.mark.parametrize("mode", [capi.GEMM_TF32, capi.GEMM_BF16X3, capi.GEMM_FP16X3])
@pytest.mark.parametrize("grid,nf", [((16, 16, 16), 64), ((32, 24, 20), 200), ((20, 20, 20), 130),
                                     ((64, 32, 32), 300)])
def test_tc_gram_hmat(mode, grid, nf):
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 23)
    V = synth.gaussian_wells(grid, ll, 6, 23)
    ctx = capi.Context(grid, ll)
    p32 = psi.astype(np.float32)
    S = ctx.gram(_dev(p32), mode=mode).cpu().numpy()
    S_ref = O.gram(p32, ctx.vel)
    assert np.array_equal(S, S.T)
    assert rel_err(S, S_ref) < TOL[mode]
    hp = O.hpsi(grid, ll, 0, p32, V)
    H = ctx.hmat(_dev(p32), _dev(hp), mode=mode).cpu().numpy()
    H_ref = O.hmat(p32, hp, ctx.vel)
    assert rel_err(H, H_ref) < TOL[mode]


def test_tc_gram_odd_sizes():
    """K not a multiple of the K block, n not a multiple of 128."""
    grid = (15, 13, 11)
    ll = tuple(x * 0.3 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, 37, 2)
    ctx = capi.Context(grid, ll)
    p32 = psi.astype(np.float32)
    for mode in (capi.GEMM_TF32, capi.GEMM_BF16X3, capi.GEMM_FP16X3):
        S = ctx.gram(_dev(p32), mode=mode).cpu().numpy()
        assert rel_err(S, O.gram(p32, ctx.vel)) < TOL[mode]


def test_bf16x3_beats_tf32():
    grid = (32, 32, 32)
    ll = tuple(x * 0.3 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, 128, 9)
    ctx = capi.Context(grid, ll)
    p32 = psi.astype(np.float32)
    ref = O.gram(p32, ctx.vel)
    e_tf = rel_err(ctx.gram(_dev(p32), mode=capi.GEMM_TF32).cpu().numpy(), ref)
    e_b3 = rel_err(ctx.gram(_dev(p32), mode=capi.GEMM_BF16X3).cpu().numpy(), ref)
    assert e_b3 < e_tf / 10


@pytest.mark.parametrize("mode", [capi.GEMM_TF32, capi.GEMM_BF16X3, capi.GEMM_FP32, capi.GEMM_FP64])
def test_fused_gram_hmat_equals_separate(mode):
    """mgx_gram_hmat (one conversion of Psi, H in column chunks of 512)
    agrees with the separate calls; n > 512 exercises the chunking."""
    grid = (16, 16, 12)
    ll = tuple(x * 0.35 for x in grid)
    nf = 600
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 41)
    V = synth.gaussian_wells(grid, ll, 6, 41)
    ctx = capi.Context(grid, ll)
    dt = np.float64 if mode == capi.GEMM_FP64 else np.float32
    p = psi.astype(dt)
    hp = O.hpsi(grid, ll, 0, p, V)
    S, H = ctx.gram_hmat(_dev(p, dt), _dev(hp, dt), mode=mode)
    S2 = ctx.gram(_dev(p, dt), mode=mode)
    H2 = ctx.hmat(_dev(p, dt), _dev(hp, dt), mode=mode)
    tol = {capi.GEMM_TF32: 2e-3, capi.GEMM_BF16X3: 2e-5, capi.GEMM_FP32: 1e-5, capi.GEMM_FP64: 1e-12}[mode]
    assert rel_err(S.cpu().numpy(), S2.cpu().numpy()) < tol
    assert rel_err(H.cpu().numpy(), H2.cpu().numpy()) < tol
    assert rel_err(H.cpu().numpy(), O.hmat(p, hp, ctx.vel)) < tol
    assert rel_err(S.cpu().numpy(), O.gram(p, ctx.vel)) < tol
