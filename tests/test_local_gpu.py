"""Localized orbitals (mgx_local_*): box-local storage on the mask boxes and
the fused fine-level step (H psi, the masked residual, two masked Jacobi
sweeps) against the oracle chain of the pinned operators on the whole grid;
every column shape, with and without the CUDA graph, gives the same bits."""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _setup(n, h, nf, seed, rlo, rhi):
    ll = tuple(h * x for x in n)
    psi, centers, _ = synth.gaussian_orbitals(n, ll, nf, seed)
    rng = np.random.default_rng(seed + 1)
    radii = rng.uniform(rlo, rhi, size=nf)
    ctx = capi.Context(n, ll)
    masks = capi.Masks(ctx, 1, centers, radii, func=0, kind=0, dtype=torch.float32)
    corr = capi.Masks(ctx, 1, centers, radii, func=1, kind=1, dtype=torch.float32)
    loc = capi.Local(ctx, masks, corr)
    V = synth.gaussian_wells(n, ll, 6, seed).astype(np.float32)
    phi = 0.6 * psi + 0.1 * np.roll(psi, 1, axis=0)
    return ll, ctx, loc, centers, radii, psi, phi, V


def test_gather_scatter_round_trip():
    n = (32, 32, 32)
    _, ctx, loc, _, _, psi, _, _ = _setup(n, 0.35, 5, 31, 1.5, 2.5)
    full = torch.from_numpy(psi.astype(np.float32)).cuda()
    packed = loc.gather(full)
    back = loc.scatter(packed)
    assert loc.total == int(loc.offsets[-1])
    for f in range(5):
        o, e = loc.boxes[f, :3], loc.boxes[f, 3:]
        assert np.all(e + 6 <= np.array(n))
        idx = np.ix_(*[(o[i] + np.arange(e[i])) % n[i] for i in range(3)])
        got = back[f].cpu().numpy().reshape(n)
        np.testing.assert_array_equal(got[idx], psi[f].astype(np.float32).reshape(n)[idx])
        mask = np.ones(n, bool)
        mask[idx] = False
        assert np.all(got[mask] == 0)


@pytest.mark.parametrize("shape", [1, 2, 5])
@pytest.mark.parametrize("n,h,nf,r", [((32, 32, 32), 0.35, 6, (1.5, 2.5)),
                                       ((40, 32, 48), 0.3, 9, (1.2, 2.0))])
def test_local_step_matches_oracle_chain(n, h, nf, r, shape):
    ll, ctx, loc, centers, radii, psi, phi, V = _setup(n, h, nf, 41, *r)
    loc.set_config(shape, 2, True)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    psi_p = loc.gather(f32(psi))
    phi_p = loc.gather(f32(phi))
    gamma = ctx.gamma(0, 2, float(V.max()), -0.5)
    u_p, w_p = loc.step(psi_p, phi_p, f32(V), gamma)
    u = loc.scatter(u_p).cpu().numpy()
    w = loc.scatter(w_p).cpu().numpy()

    # the oracle chain on the whole grid, from the orbitals as stored
    psi0 = loc.scatter(psi_p).cpu().numpy().astype(np.float64)
    phi0 = loc.scatter(phi_p).cpu().numpy().astype(np.float64)
    st_o, v_o = O.mask_build(n, ll, 1, 1, centers, radii, func=0)
    st_c, v_c = O.mask_build(n, ll, 1, 1, centers, radii, func=1)
    hp = O.hpsi(n, ll, 0, psi0, V.astype(np.float64), apply_B=1)
    res = O.mask_apply(n, 0, st_c, v_c, O.rhs_mehr(n, ll, phi0) - hp, kind=1)
    jf = O.jacobi_factor(n, ll, 0)
    u0 = gamma * res
    u1 = O.mask_apply(n, 0, st_o, v_o, u0 - jf * (O.fd_apply(n, ll, 0, u0) - res), kind=0)
    w1 = O.fd_apply(n, ll, 0, u1) - res
    u2 = O.mask_apply(n, 0, st_o, v_o, u1 - jf * w1, kind=0)
    wm = O.mask_apply(n, 0, st_o, v_o, w1, kind=0)
    assert rel_err(u, u2) < 1e-4
    assert rel_err(w, wm) < 1e-4


def test_every_configuration_gives_the_same_bits():
    n = (32, 32, 32)
    _, ctx, loc, _, _, psi, phi, V = _setup(n, 0.35, 7, 51, 1.5, 2.5)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    psi_p, phi_p, Vd = loc.gather(f32(psi)), loc.gather(f32(phi)), f32(V)
    ref = None
    for shape in range(6):
        for ctas in (1, 4):
            for graph in (False, True):
                loc.set_config(shape, ctas, graph)
                u, w = loc.step(psi_p, phi_p, Vd, 0.01)
                if ref is None:
                    ref = (u.clone(), w.clone())
                assert torch.equal(u, ref[0]) and torch.equal(w, ref[1]), (shape, ctas, graph)
    # a replayed graph with new input values gives the new result
    loc.set_config(1, 2, True)
    u1, w1 = torch.empty_like(u), torch.empty_like(w)
    loc.step(psi_p, phi_p, Vd, 0.01, u=u1, w=w1)
    psi_p.mul_(2.0)
    phi_p.mul_(2.0)
    loc.step(psi_p, phi_p, Vd, 0.01, u=u1, w=w1)
    loc.set_config(1, 2, False)
    u2, w2 = loc.step(psi_p, phi_p, Vd, 0.01)
    assert torch.equal(u1, u2) and torch.equal(w1, w2)


def test_tuner_picks_a_resident_configuration():
    n = (32, 32, 32)
    _, ctx, loc, _, _, psi, phi, V = _setup(n, 0.35, 8, 61, 1.5, 2.5)
    f32 = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    psi_p, phi_p, Vd = loc.gather(f32(psi)), loc.gather(f32(phi)), f32(V)
    u, w = loc.empty(), loc.empty()
    ms, (shape, ctas, graph) = loc.tune(psi_p, phi_p, Vd, 0.01, u, w)
    assert ms.size == 24 and np.all(ms[ms >= 0] > 0)
    assert ms[4 * shape + (1, 2, 3, 4).index(ctas)] == ms[ms >= 0].min()
    assert graph == 1


def test_box_wider_than_the_grid_is_refused():
    n = (16, 16, 16)
    ll = tuple(0.35 * x for x in n)
    ctx = capi.Context(n, ll)
    c = np.array([[2.0, 2.0, 2.0]])
    r = np.array([2.5])
    masks = capi.Masks(ctx, 1, c, r, func=0, kind=0, dtype=torch.float32)
    corr = capi.Masks(ctx, 1, c, r, func=1, kind=1, dtype=torch.float32)
    with pytest.raises(capi.MgxError):
        capi.Local(ctx, masks, corr)
