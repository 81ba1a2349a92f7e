"""mgx_sincos_diag (the centres and spreads of SpreadsAndCenters) against the
oracle's restatement of SinCosOps::computeDiag, FP64 and FP32 blocks,
normalized and not; the same bits on repeated calls; centres and spreads
from the library's elements against the oracle's."""
import numpy as np
import pytest
import torch

import oracle as O
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,h,nf", [((32, 28, 36), 0.35, 5), ((64, 64, 64), 0.35, 40),
                                    ((48, 40, 24), 0.3, 300)])
@pytest.mark.parametrize("dt", [torch.float64, torch.float32])
def test_sincos_diag_matches_the_oracle(n, h, nf, dt):
    ll = tuple(x * h for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, nf, 71)
    ctx = capi.Context(n, ll)
    d = torch.from_numpy(psi).to(dtype=dt, device="cuda")
    host = d.double().cpu().numpy()
    for normalized in (False, True):
        got = ctx.sincos_diag(d, normalized).cpu().numpy()
        ref = O.sincos_diag(n, ll, host, normalized)
        assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
        again = ctx.sincos_diag(d, normalized).cpu().numpy()
        assert np.array_equal(got, again)
    x, spread = ctx.centers_spreads(d)
    xr, sr = O.centers_spreads(ll, O.sincos_diag(n, ll, host))
    assert np.max(np.abs(x - xr)) < 1e-10 and np.max(np.abs(spread - sr)) < 1e-10


def test_centres_follow_the_seeded_orbitals():
    n = (64, 64, 64)
    ll = tuple(x * 0.35 for x in n)
    psi, centers, _ = synth.gaussian_orbitals(n, ll, 16, 1001)
    ctx = capi.Context(n, ll)
    x, _ = ctx.centers_spreads(torch.from_numpy(psi).cuda())
    d = x - np.asarray(centers)
    d -= np.asarray(ll)[None, :] * np.round(d / np.asarray(ll)[None, :])
    assert np.max(np.abs(d)) < 0.1
