"""mgx_hpsi_gram_hmat_matb (H psi made inside the H product and written
straight into its split-BF16x3 operand planes) against the separate calls
mgx_hpsi + mgx_gram_hmat_matb: H psi bit for bit, S, H and B to the FP64
reduction order, across several 512-function chunks; the fallback shapes
(no vector kernel, other product modes); and one sweep each way."""
import numpy as np
import pytest
import torch

from mgmol_gb300 import capi, synth
from mgmol_gb300.sweep import OrbitalSweep

pytestmark = pytest.mark.gpu


def _inputs(n, h, nf, seed):
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, nf, seed, torch.float32)
    V = synth.gaussian_wells_device(n, ll, 8, seed).float().contiguous()
    return ctx, psi, V


@pytest.mark.parametrize("n,nf", [((32, 32, 32), 600), ((32, 28, 36), 40), ((30, 26, 34), 20)])
@pytest.mark.parametrize("mode", [capi.GEMM_BF16X3, capi.GEMM_TF32])
def test_fused_matches_separate_calls(n, nf, mode):
    ctx, psi, V = _inputs(n, 0.35, nf, 17)
    hp_ref = ctx.hpsi(psi, V, capi.LAP_MEHR4, True)
    S0, H0, B0 = ctx.gram_hmat_matb(psi, hp_ref, mode)
    hp = torch.empty_like(psi)
    S1, H1, B1 = ctx.hpsi_gram_hmat_matb(psi, V, hp, mode)
    assert torch.equal(hp, hp_ref)
    for a, b in ((S1, S0), (H1, H0), (B1, B0)):
        assert float((a - b).abs().max()) <= 1e-12 * float(b.abs().max())


def test_sweep_with_and_without_the_fused_call():
    n = (48, 48, 48)
    ll = tuple(x * 0.35 for x in n)
    ctx = capi.Context(n, ll)
    V = synth.gaussian_wells_device(n, ll, 8, 1001)
    psi0, _, _ = synth.gaussian_orbitals_device(n, ll, 32, 1001, torch.float32)
    out = []
    for fuse in (True, False):
        sw = OrbitalSweep(ctx, V, 32, mode="mixed", gemm=capi.GEMM_BF16X3, fuse_hpsi=fuse)
        assert sw.fuse_hpsi == fuse
        psi = psi0.clone()
        e = [float(sw.run(psi).cpu()[0]) for _ in range(3)]
        out.append((np.asarray(e), psi))
    (e1, p1), (e2, p2) = out
    assert np.allclose(e1, e2, rtol=1e-10, atol=0)
    assert float((p1 - p2).abs().max()) <= 1e-5 * float(p2.abs().max())
