"""The localized-orbital workload: N orbitals on their mask boxes and the
fused fine-level step (mgx_local_step: H psi, the masked residual and the two
masked Jacobi pre-sweeps of the V-cycle, one persistent kernel launched as
a CUDA graph, tile shape and CTAs per SM picked by mgx_local_tune).

Orbitals are the workload's seeded Gaussians restricted to the level-0 box
of a GridMaskMax mask of seeded radius U[4, 8] bohr (gaussianDecay), with
the correction masks of profile one; phi = lambda_j psi_j stands in for the
column of Psi Theta (the step's cost does not depend on its values).

CLI (one JSON line):
    python -m mgmol_gb300.local --grid 160 160 160 --h 0.3 --nfunc 1536
"""
import argparse
import json
import sys

import numpy as np
import torch

from . import capi, synth

# algorithmic bytes per box point: psi, phi, V, two mask values read; u, w written
BYTES_PER_POINT = 7 * 4
# the kernel variants of mgx_local_tune: (largest column TY x TZ, fitted to each
# box, planes per march step)
VARIANTS = [("24x32", 1), ("16x32", 1), ("32x32", 1), ("24x32", 2), ("16x32", 2), ("32x32", 2)]


def build(n, h, nfunc, seed, rlo=4.0, rhi=8.0, chunk=128):
    ll = tuple(h * x for x in n)
    ctx = capi.Context(n, ll)
    g = torch.Generator(device="cuda")
    g.manual_seed(int(seed))
    L = torch.tensor(ll, dtype=torch.float64, device="cuda")
    centers = (torch.rand((nfunc, 3), generator=g, dtype=torch.float64, device="cuda") * L)
    centers = centers.cpu().numpy()
    radii = synth.mask_radii(nfunc, seed, rlo, rhi)
    masks = capi.Masks(ctx, 1, centers, radii, func=0, kind=0, dtype=torch.float32)
    corr = capi.Masks(ctx, 1, centers, radii, func=1, kind=1, dtype=torch.float32)
    loc = capi.Local(ctx, masks, corr)
    # the orbitals: Gaussians of width U[1, 2] around the mask centres,
    # generated on the whole grid a chunk at a time and gathered to the boxes
    psi = loc.empty()
    sig = 1.0 + torch.rand(nfunc, generator=g, dtype=torch.float64, device="cuda")
    xs = [torch.arange(n[i], dtype=torch.float64, device="cuda") * (ll[i] / n[i]) for i in range(3)]
    full = torch.zeros((nfunc, ctx.npts), dtype=torch.float32, device="cuda")
    c = torch.from_numpy(centers).cuda()
    for f0 in range(0, nfunc, chunk):
        f1 = min(nfunc, f0 + chunk)
        d2 = []
        for i in range(3):
            d = xs[i][None, :] - c[f0:f1, i:i + 1]
            d = d - L[i] * torch.round(d / L[i])
            d2.append(d * d)
        r2 = d2[0][:, :, None, None] + d2[1][:, None, :, None] + d2[2][:, None, None, :]
        s = sig[f0:f1][:, None, None, None]
        full[f0:f1] = torch.exp(-r2 / (2.0 * s * s)).reshape(f1 - f0, -1).float()
    loc.gather(full, out=psi)
    del full
    lam = (-0.5 + 0.2 * torch.rand(nfunc, generator=g, device="cuda")).cpu().numpy()
    phi = psi.clone()
    for f in range(nfunc):
        a, b = int(loc.offsets[f]), int(loc.offsets[f + 1])
        phi[a:b] *= float(lam[f])
    V = torch.from_numpy(synth.gaussian_wells(n, ll, 64, seed).astype(np.float32)).cuda()
    gamma = ctx.gamma(0, 2, float(V.max()), -0.5)
    return ctx, loc, (masks, corr), psi, phi, V, gamma


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", type=int, nargs=3, default=[160, 160, 160])
    ap.add_argument("--h", type=float, default=0.3)
    ap.add_argument("--nfunc", type=int, default=1536)
    ap.add_argument("--seed", type=int, default=1003)
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--config", type=int, nargs=2, default=None, metavar=("VARIANT", "CTAS"),
                    help="skip the tuner: kernel variant and CTAs per SM")
    a = ap.parse_args(argv)
    n = tuple(a.grid)
    ctx, loc, keep, psi, phi, V, gamma = build(n, a.h, a.nfunc, a.seed)
    u, w = loc.empty(), loc.empty()
    if a.config:
        loc.set_config(a.config[0], a.config[1], True)
        ms, cfg = np.zeros(0), loc.config()
    else:
        ms, cfg = loc.tune(psi, phi, V, gamma, u, w)
    loc.step(psi, phi, V, gamma, u=u, w=w)
    torch.cuda.synchronize()
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    for _ in range(a.reps):
        loc.step(psi, phi, V, gamma, u=u, w=w)
    e1.record(s)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / a.reps
    vols = loc.boxes[:, 3].astype(np.int64) * loc.boxes[:, 4] * loc.boxes[:, 5]
    gbs = loc.total * BYTES_PER_POINT / (t * 1e-3) / 1e9
    out = {"workload": "localized step", "grid": list(n), "h": a.h, "nfunc": a.nfunc,
           "box_points_total": int(loc.total), "box_points_mean": float(vols.mean()),
           "box_points_min": int(vols.min()), "box_points_max": int(vols.max()),
           "ms_per_step": t, "algorithmic_GBps": gbs, "bytes_per_point": BYTES_PER_POINT,
           "config": {"column": VARIANTS[cfg[0]][0], "planes_per_step": VARIANTS[cfg[0]][1],
                      "ctas_per_sm": cfg[1],
                      "graph": bool(cfg[2])},
           "tune_ms": [round(float(x), 4) for x in ms],
           "whole_grid_points": a.nfunc * ctx.npts}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)
