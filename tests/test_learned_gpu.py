"""The learned preconditioner on the GPU (mgx_unet_*, mgx_precond_learned,
mgx_precond_mg_warm): forward pass, loss, gradients and the Adam step
against the float64 CPU oracle (oracle/unet_oracle.py); training on the
V-cycle's pairs; the per-function fallback; and what the trained network
gains in the block preconditioned-gradient iteration."""
import numpy as np
import pytest
import torch

import unet_oracle as UO
from helpers import rel_err
from mgmol_gb300 import capi, learned, synth

pytestmark = pytest.mark.gpu

# FP32 activations and accumulation against the float64 oracle with the
# same BF16 weights
TOL_FWD = 2e-5
TOL_GRAD = 2e-4


def _dev(a, dt=np.float32):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


def _fields(n, nfunc, seed):
    ll = tuple(x * 0.4 for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, nfunc, seed)
    psi -= psi.mean(axis=1, keepdims=True)
    return ll, psi


@pytest.mark.parametrize("n", [(16, 16, 16), (8, 24, 12), (32, 16, 40)])
def test_forward_matches_oracle(n):
    ll, x = _fields(n, 3, 11)
    ctx = capi.Context(n, ll)
    net = capi.UNet(ctx)
    p = UO.init_params(5)
    net.set_params(p)
    y = net.forward(_dev(x)).cpu().numpy()
    y_ref = UO.forward(n, p, x)
    assert rel_err(y, y_ref) < TOL_FWD


def test_forward_strided_block():
    n = (16, 16, 16)
    ll, x = _fields(n, 4, 12)
    ctx = capi.Context(n, ll)
    net = capi.UNet(ctx)
    p = UO.init_params(6)
    net.set_params(p)
    big = torch.zeros((4, ctx.npts + 64), dtype=torch.float32, device="cuda")
    big[:, :ctx.npts] = _dev(x)
    out = torch.zeros_like(big)
    net.forward(big[:, :ctx.npts], out=out[:, :ctx.npts])
    assert rel_err(out[:, :ctx.npts].cpu().numpy(), UO.forward(n, p, x)) < TOL_FWD
    assert float(out[:, ctx.npts:].abs().max()) == 0.0


@pytest.mark.parametrize("n", [(16, 16, 16), (8, 12, 16)])
def test_loss_and_gradient_match_oracle(n):
    ll, x = _fields(n, 3, 13)
    _, t = _fields(n, 3, 14)
    ctx = capi.Context(n, ll)
    net = capi.UNet(ctx)
    p = UO.init_params(7)
    net.set_params(p)
    loss, grad = net.loss_grad(_dev(x), _dev(t))
    l_ref, g_ref = UO.loss_grad(n, p, x, t)
    assert abs(float(loss) - l_ref) < 1e-5 * abs(l_ref)
    g = grad.cpu().numpy()
    o = 0
    for ci, co, _ in UO.LAYERS:
        k = ci * co * 27
        assert rel_err(g[o:o + k], g_ref[o:o + k]) < TOL_GRAD, (ci, co)
        o += k


def test_adam_step_matches_oracle():
    n = (16, 16, 16)
    ll, x = _fields(n, 2, 15)
    _, t = _fields(n, 2, 16)
    ctx = capi.Context(n, ll)
    net = capi.UNet(ctx)
    p = UO.init_params(8)
    net.set_params(p)
    pd = p.astype(np.float64)
    m = np.zeros_like(pd)
    v = np.zeros_like(pd)
    for step in (1, 2):
        _, grad = net.loss_grad(_dev(x), _dev(t))
        g = grad.cpu().numpy().astype(np.float64)
        net.adam(grad, 1e-3)
        pd, m, v = UO.adam(pd, g, m, v, step, 1e-3)
        got = net.get_params().cpu().numpy()
        assert np.abs(got - pd).max() < 1e-6 * np.abs(pd).max()
        pd = got.astype(np.float64)


def test_warm_vcycle_from_gamma_res_is_the_vcycle():
    n = (32, 32, 32)
    ll, x = _fields(n, 3, 17)
    ctx = capi.Context(n, ll)
    g = ctx.gamma(0, 2, 0.0, 0.0)
    r = _dev(x)
    plain = ctx.precond_mg(r, 0, 2, g)
    warm = (r * np.float32(g)).contiguous()
    ctx.precond_mg_warm(r, warm, 0, 2)
    assert rel_err(warm.cpu().numpy(), plain.cpu().numpy()) < 1e-6


def test_fallback_with_an_untrained_net_is_the_vcycle():
    """A zero network gives the zero correction (reduction 1): every
    function falls back, and the result is the V-cycle's, bit for bit."""
    n = (32, 32, 32)
    ll, x = _fields(n, 5, 18)
    ctx = capi.Context(n, ll)
    g = ctx.gamma(0, 2, 0.0, 0.0)
    net = capi.UNet(ctx)
    net.set_params(np.zeros(capi.UNET_PARAMS, np.float32))
    r = _dev(x)
    tau = np.zeros(5)
    out, red, nfb = capi.precond_learned(ctx, net, r, 0, 2, g, tau, mode=capi.LEARNED_REPLACE)
    plain = ctx.precond_mg(r, 0, 2, g)
    assert nfb == 5
    assert torch.equal(out, plain)
    assert np.all(tau > 0) and np.all(tau < 1)
    np.testing.assert_allclose(red, tau)
    # with tau known, the next call keeps every fallback without a refresh
    out2, red2, nfb2 = capi.precond_learned(ctx, net, r, 0, 2, g, tau, mode=capi.LEARNED_REPLACE)
    assert nfb2 == 5 and torch.equal(out2, plain)


def test_training_and_gain_in_the_block_iteration():
    """Trains on the plain iteration's (residual, V-cycle correction) pairs,
    then runs the block preconditioned-gradient iteration to 1e-6 with the
    V-cycle and with the learned warm start (refreshed fallback, so each
    step is at least as good as the V-cycle's from the same iterate)."""
    n = (32, 32, 32)
    ll = tuple(x * 0.4 for x in n)
    ctx = capi.Context(n, ll)
    lap, maxl = 0, 2
    g = ctx.gamma(lap, maxl, 0.0, 0.0)
    solver = learned.BlockSolver(ctx, lap, maxl, g)
    net = capi.UNet(ctx)
    net.set_params(learned.init_params(1))
    first = None
    for k in range(3):
        f = learned.rhs_block(n, ll, 16, 300 + k)
        tr = learned.train_on_iteration(solver, net, f, 25, 1e-3, 4, reps=2)
        first = tr.losses[0] if first is None else first
    assert tr.losses[-1] < 0.5 * first, (first, tr.losses[-1])

    f = learned.rhs_block(n, ll, 8, 400)
    its_plain, _ = solver.run(f, solver.vcycle, tol=1e-6, maxit=400)
    pc = learned.Learned(solver, net, refresh=True)
    its_learned, _ = solver.run(f, pc, tol=1e-6, maxit=400)
    print("iterations plain", its_plain, "learned", its_learned, "fallbacks", pc.fallbacks,
          "of", pc.functions)
    assert (its_plain <= 400).all()
    assert np.median(its_learned) <= np.median(its_plain)
