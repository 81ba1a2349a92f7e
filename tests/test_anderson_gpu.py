"""Anderson extrapolation of the orbital update (mgx_anderson_*) on the GPU
vs the oracle restatement of AndersonMix<T>::update, which the
reference-vector tests pin bit for bit to the reference's own code.

The device sums each dot product in another order than the reference's
sequential MPdot, so the coefficients differ in the last bits; blocks agree
to 1e-12 (FP64) and 1e-6 (FP32) relative to their largest value over a
whole sequence of updates, history shortening included.
"""
import numpy as np
import pytest
import torch

import oracle as O
from helpers import rel_err
from mgmol_gb300 import capi

pytestmark = pytest.mark.gpu

GRID = (8, 8, 10)
LL = (2.4, 2.4, 3.0)


def _sequences(kind, nf, npt, ns, seed):
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((nf, npt))
    if kind == "conv":
        return np.stack([(0.6 ** s) * rng.standard_normal((nf, npt)) for s in range(ns)])
    if kind == "collinear":
        return np.stack([(0.7 ** s) * (g + 1e-3 * rng.standard_normal((nf, npt)))
                         for s in range(ns)])
    return np.stack([(1.0 + 1e-4 * s) * g + 1e-6 * rng.standard_normal((nf, npt))
                     for s in range(ns)])


def _run_gpu(ctx, x0, fseq, m, invs, fscale):
    x = torch.from_numpy(np.ascontiguousarray(x0)).cuda()
    mix = capi.Anderson(ctx, m, 1.0, x)
    out, infos = [], []
    for s in range(fseq.shape[0]):
        invS = torch.diag(torch.from_numpy(invs[s])).cuda().contiguous()
        f = torch.from_numpy(np.ascontiguousarray(fseq[s])).cuda()
        infos.append(mix.update(x, f, fscale, invS))
        out.append(x.cpu().numpy().copy())
    mix.close()
    return np.stack(out), infos


@pytest.mark.parametrize("kind", ["conv", "collinear", "repeat"])
@pytest.mark.parametrize("m", [0, 1, 2, 3, 8])
@pytest.mark.parametrize("dt,tol", [(np.float64, 1e-12), (np.float32, 1e-6)])
def test_anderson_matches_oracle(kind, m, dt, tol):
    ctx = capi.Context(GRID, LL)
    nf, ns = 6, 10
    rng = np.random.default_rng(11)
    x0 = rng.standard_normal((nf, ctx.npts)).astype(dt)
    fseq = _sequences(kind, nf, ctx.npts, ns, 12).astype(dt)
    invs = 1.0 + 0.2 * rng.random((ns, nf))
    got, infos = _run_gpu(ctx, x0, fseq, m, invs, 0.5)
    ref = O.anderson(x0, fseq, m, 1.0, ctx.vel, invs, fscale=0.5)
    for s in range(ns):
        assert rel_err(got[s], ref[s]) < tol, f"step {s}"
    assert infos[0]["mm"] == 0 and all(0 <= i["mm"] <= m for i in infos)
    if kind == "repeat" and m > 1:
        # repeated residuals make the history nearly dependent: the
        # reference's safeguards shorten it
        assert sum(i["reductions"] for i in infos) > 0


def test_anderson_first_update_and_restart():
    """Without history the update is x += fscale f, also after restart."""
    ctx = capi.Context(GRID, LL)
    rng = np.random.default_rng(13)
    x0 = rng.standard_normal((3, ctx.npts)).astype(np.float32)
    f0 = rng.standard_normal((3, ctx.npts)).astype(np.float32)
    x = torch.from_numpy(x0.copy()).cuda()
    f = torch.from_numpy(f0).cuda()
    fbar = torch.empty_like(f)
    mix = capi.Anderson(ctx, 2, 1.0, x)
    info = mix.update(x, f, 0.5, None, fbar=fbar)
    assert info["mm"] == 0
    ref = x0 + (0.5 * f0.astype(np.float64)).astype(np.float32)
    assert np.array_equal(x.cpu().numpy(), ref)
    assert np.array_equal(fbar.cpu().numpy(), (0.5 * f0.astype(np.float64)).astype(np.float32))
    invS = torch.eye(3, dtype=torch.float64, device="cuda")
    # the same residual again leaves f - f_0 = 0: a singular history matrix
    with pytest.raises(capi.MgxError) as e:
        mix.update(x, f, 0.5, invS)
    assert e.value.status == capi.MGX_NOT_SPD
    assert mix.update(x, 0.5 * f, 0.5, invS)["mm"] == 1
    mix.restart()
    x1 = x.cpu().numpy()
    assert mix.update(x, f, 0.5, invS)["mm"] == 0
    assert np.array_equal(x.cpu().numpy(), x1 + (0.5 * f0.astype(np.float64)).astype(np.float32))
    mix.close()


def test_anderson_rejects_bad_arguments():
    ctx = capi.Context(GRID, LL)
    x = torch.zeros((2, ctx.npts), dtype=torch.float64, device="cuda")
    with pytest.raises(capi.MgxError):
        capi.Anderson(ctx, capi.ANDERSON_MAX_M + 1, 1.0, x)
    mix = capi.Anderson(ctx, 1, 1.0, x)
    with pytest.raises(capi.MgxError):
        mix.update(x, x, 1.0, None)
    f = torch.ones_like(x)
    mix.update(x, f, 1.0, None)
    with pytest.raises(capi.MgxError):
        mix.update(x, f, 1.0, None)         # the second update needs S^-1
    # the refused update left the history as it was
    invS = torch.eye(2, dtype=torch.float64, device="cuda")
    assert mix.update(x, 2 * f, 1.0, invS)["mm"] == 1
    mix.close()
