"""Parity of the CUDA stencils (through the C ABI) with the oracle.

FP64 kernels vs the FP64 oracle: 1e-12 relative (normwise, max |diff| over
max |ref|).  FP32 kernels compute in FP32 and are compared with the FP64
oracle at 2e-5 relative.  Sizes cover the staged (bulk-copy) path, the
direct path (small / odd z lines), ragged grids and the x-chunk wrap.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F32, TOL_F64, golden, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu

CASES = [
    ((16, 12, 20), 0.35, 3),   # ragged, direct path for some ops
    ((32, 32, 32), 0.35, 4),   # staged path
    ((24, 16, 40), 0.30, 2),   # ragged staged
    ((8, 8, 8), 0.35, 2),      # tiny: direct path
    ((40, 36, 64), 0.3, 3),    # x chunk not dividing nx
]


def _inputs(n, h, nf, seed=11):
    ll = tuple(n[i] * h for i in range(3))
    psi, _, _ = synth.gaussian_orbitals(n, ll, nf, seed)
    V = synth.gaussian_wells(n, ll, 6, seed)
    return ll, psi, V


def _dev(a, dt):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


@pytest.mark.parametrize("n,h,nf", CASES)
@pytest.mark.parametrize("lap", [0, 1, 2, 3, 4])
def test_fd_apply(n, h, nf, lap):
    ll, psi, _ = _inputs(n, h, nf)
    ctx = capi.Context(n, ll)
    ref = O.fd_apply(n, ll, lap, psi)
    out = ctx.fd_apply(_dev(psi, np.float64), lap).cpu().numpy()
    assert rel_err(out, ref) < TOL_F64
    out32 = ctx.fd_apply(_dev(psi, np.float32), lap).cpu().numpy()
    assert rel_err(out32, ref) < TOL_F32


@pytest.mark.parametrize("n,h,nf", CASES)
def test_rhs_mehr(n, h, nf):
    ll, psi, _ = _inputs(n, h, nf)
    ctx = capi.Context(n, ll)
    ref = O.rhs_mehr(n, ll, psi)
    assert rel_err(ctx.rhs_mehr(_dev(psi, np.float64)).cpu().numpy(), ref) < TOL_F64
    assert rel_err(ctx.rhs_mehr(_dev(psi, np.float32)).cpu().numpy(), ref) < TOL_F32


@pytest.mark.parametrize("n,h,nf", CASES)
@pytest.mark.parametrize("lap,apply_B", [(0, 1), (0, 0), (2, 1), (4, 1), (1, 1)])
def test_hpsi(n, h, nf, lap, apply_B):
    ll, psi, V = _inputs(n, h, nf)
    ctx = capi.Context(n, ll)
    ref = O.hpsi(n, ll, lap, psi, V, apply_B=apply_B)
    out = ctx.hpsi(_dev(psi, np.float64), _dev(V, np.float64), lap, bool(apply_B)).cpu().numpy()
    assert rel_err(out, ref) < TOL_F64
    # FP32 orbitals with FP32 and with FP64 potential
    for vdt in (np.float32, np.float64):
        out32 = ctx.hpsi(_dev(psi, np.float32), _dev(V, vdt), lap, bool(apply_B)).cpu().numpy()
        assert rel_err(out32, ref) < TOL_F32


def test_hpsi_matches_reference_golden():
    G = golden()
    n = tuple(int(x) for x in G["stencil_n"])
    ll = tuple(float(x) for x in G["stencil_ll"])
    ctx = capi.Context(n, ll)
    out = ctx.hpsi(_dev(G["stencil_psi"], np.float64), _dev(G["stencil_V"], np.float64)).cpu().numpy()
    assert rel_err(out, G["hpsi_d"]) < TOL_F64
    for t in range(5):
        o = ctx.fd_apply(_dev(G["stencil_psi"], np.float64), t).cpu().numpy()
        assert rel_err(o, G[f"fd{t}_d"]) < TOL_F64


def test_leading_dimension_padding():
    """BlockVector-style padded columns (ld > numpt)."""
    n, h, nf = (32, 16, 24), 0.3, 3
    ll, psi, V = _inputs(n, h, nf)
    np_ = psi.shape[1]
    ld = np_ + 40
    big = torch.zeros((nf, ld), dtype=torch.float64, device="cuda")
    big[:, :np_] = torch.from_numpy(psi).cuda()
    out = torch.full_like(big, 7.0)
    ctx = capi.Context(n, ll)
    ctx.fd_apply(big[:, :np_], 0, out=out[:, :np_])
    ref = O.fd_apply(n, ll, 0, psi)
    assert rel_err(out[:, :np_].cpu().numpy(), ref) < TOL_F64
    assert torch.all(out[:, np_:] == 7.0)


def test_empty_batch_is_a_no_op():
    n = (16, 16, 16)
    ctx = capi.Context(n, (5.6, 5.6, 5.6))
    u = torch.zeros((0, 4096), dtype=torch.float64, device="cuda")
    assert ctx.fd_apply(u, 0).shape == (0, 4096)


# ---------------------------------------------------------------- drop-in ghosted
def _ghosted(u, n, g):
    nf = u.shape[0]
    G = np.zeros((nf, n[0] + 2 * g, n[1] + 2 * g, n[2] + 2 * g), dtype=u.dtype)
    U = u.reshape(nf, *n)
    G[:, g:-g, g:-g, g:-g] = U
    return G


@pytest.mark.parametrize("lap,g", [(0, 1), (1, 1), (2, 2), (3, 3), (4, 4), (0, 2)])
def test_dropin_fdkernel_del2(lap, g):
    n, h, nf = (16, 12, 20), 0.35, 3
    ll, psi, _ = _inputs(n, h, nf)
    Gh = torch.from_numpy(_ghosted(psi, n, g)).cuda()
    capi.trade_boundaries(n, ll, g, Gh, nf)
    B = torch.zeros_like(Gh)
    capi.fdkernel_del2(n, ll, g, lap, Gh, B, nf)
    out = B[:, g:-g, g:-g, g:-g].reshape(nf, -1).cpu().numpy()
    assert rel_err(out, O.fd_apply(n, ll, lap, psi)) < TOL_F64
    # ghosts of the output untouched
    assert float(B[:, :g].abs().max()) == 0.0


def test_dropin_trade_is_periodic_image():
    n, g = (6, 5, 7), 2
    ll = (6 * 0.3, 5 * 0.3, 7 * 0.3)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((2, n[0] * n[1] * n[2]))
    Gh = torch.from_numpy(_ghosted(u, n, g)).cuda()
    capi.trade_boundaries(n, ll, g, Gh, 2)
    ref = np.pad(u.reshape(2, *n), ((0, 0), (g, g), (g, g), (g, g)), mode="wrap")
    assert np.array_equal(Gh.cpu().numpy(), ref)


def test_dropin_rhs_and_transfers():
    n, h, nf = (16, 12, 20), 0.35, 2
    ll, psi, _ = _inputs(n, h, nf)
    g = 1
    Gh = torch.from_numpy(_ghosted(psi, n, g)).cuda()
    capi.trade_boundaries(n, ll, g, Gh, nf)
    R = torch.zeros((nf, n[0] * n[1] * n[2]), dtype=torch.float64, device="cuda")
    capi.fdkernel_rhs_mehr1(n, ll, g, Gh, R, 0, nf)
    assert rel_err(R.cpu().numpy(), O.rhs_mehr(n, ll, psi)) < TOL_F64
    cn = tuple(x // 2 for x in n)
    C = torch.zeros((nf, cn[0] + 2, cn[1] + 2, cn[2] + 2), dtype=torch.float64, device="cuda")
    capi.mgkernel_restrict3d(n, ll, g, Gh, C, nf)
    c_ref = O.restrict(n, ll, psi)
    assert rel_err(C[:, 1:-1, 1:-1, 1:-1].reshape(nf, -1).cpu().numpy(), c_ref) < TOL_F64
    capi.trade_boundaries(cn, ll, g, C, nf)
    F = torch.zeros_like(Gh)
    capi.mgkernel_extend3d(n, ll, g, C, F, nf)
    e_ref = O.extend(n, ll, c_ref)
    assert rel_err(F[:, 1:-1, 1:-1, 1:-1].reshape(nf, -1).cpu().numpy(), e_ref) < TOL_F64
