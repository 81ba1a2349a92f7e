"""pb::Mgm (the multigrid Poisson solver) on the GPU vs the oracle and the
reference's own golden vectors.

FP64: the field to 1e-12 relative, the same number of V-cycles and the same
convergence flag, the residual norms to 1e-9 relative (they measure a
residual that is itself ~1e-4..1e-7 of the right-hand side, so the FMA-level
differences of the GPU stencils show there first).  FP32: 1e-5 relative.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import TOL_F64, golden, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _dev(a, dt=np.float64):
    return torch.from_numpy(np.ascontiguousarray(a.astype(dt))).cuda()


@pytest.mark.parametrize("lap", range(5))
def test_mgm_matches_reference_vectors(lap):
    G = golden()
    n = tuple(int(x) for x in G["mgm_n"])
    ll = tuple(float(x) for x in G["mgm_ll"])
    ctx = capi.Context(n, ll)
    vh = _dev(G["mgm_vh0"])
    info = ctx.mgm(vh, _dev(G["mgm_rho"]), lap_type=lap, max_sweeps=6, tol=1e-10)
    ref = G[f"mgm{lap}_info"]
    assert rel_err(vh.cpu().numpy(), G[f"mgm{lap}_vh"]) < TOL_F64
    assert info["nb_sweeps"] == int(ref[3])
    assert info["converged"] == int(ref[4])
    for k, i in (("final_residual", 0), ("final_relative_residual", 1), ("residual_reduction", 2)):
        assert abs(info[k] - ref[i]) <= 1e-9 * abs(ref[i]), k


@pytest.mark.parametrize("lap,n", [(0, (32, 32, 32)), (0, (64, 48, 40)), (1, (24, 24, 24)),
                                   (4, (32, 32, 16)), (2, (40, 24, 8))])
def test_mgm_vs_oracle(lap, n):
    ll = tuple(x * 0.3 for x in n)
    rho = synth.gaussian_wells(n, ll, 5, 77)
    rho = rho - rho.mean()
    vh0 = np.zeros_like(rho)
    ref, ri = O.mgm(n, ll, lap, vh0, rho, max_sweeps=8, tol=1e-9)
    ctx = capi.Context(n, ll)
    vh = _dev(vh0)
    info = ctx.mgm(vh, _dev(rho), lap_type=lap, max_sweeps=8, tol=1e-9)
    assert info["levels"] == ri["levels"]
    assert info["nb_sweeps"] == ri["nb_sweeps"]
    assert bool(info["converged"]) == ri["converged"]
    assert rel_err(vh.cpu().numpy(), ref) < TOL_F64


def test_mgm_fp32():
    G = golden()
    n = tuple(int(x) for x in G["mgm_n"])
    ll = tuple(float(x) for x in G["mgm_ll"])
    ctx = capi.Context(n, ll)
    vh = _dev(G["mgm_vh0"], np.float32)
    ctx.mgm(vh, _dev(G["mgm_rho"], np.float32), lap_type=0, max_sweeps=3, tol=1e-10)
    assert rel_err(vh.cpu().numpy(), G["mgm0_vh_f"]) < 1e-5


def test_mgm_converges_and_stops_early():
    n = (64, 64, 64)
    ll = (19.2,) * 3
    rho = synth.gaussian_wells(n, ll, 8, 5)
    rho = rho - rho.mean()
    ctx = capi.Context(n, ll)
    vh = torch.zeros(n[0] * n[1] * n[2], dtype=torch.float64, device="cuda")
    info = ctx.mgm(vh, _dev(rho), lap_type=0, max_sweeps=30, tol=1e-8)
    assert info["converged"] == 1
    assert info["final_relative_residual"] < 1e-8
    assert info["nb_sweeps"] < 30
    # a second solve from the converged field stops at once
    again = ctx.mgm(vh, _dev(rho), lap_type=0, max_sweeps=30, tol=1e-8)
    assert again["nb_sweeps"] == 0 and again["converged"] == 1


def test_mgm_rejects_bad_arguments():
    ctx = capi.Context((8, 8, 8), (2.0, 2.0, 2.0))
    a = torch.zeros(512, dtype=torch.float64, device="cuda")
    with pytest.raises(capi.MgxError):
        ctx.mgm(a, a)                       # vh and rho alias
    with pytest.raises(capi.MgxError):
        ctx.mgm(a, torch.zeros_like(a), lap_type=4, ghosts=2)   # ghosts below radius
