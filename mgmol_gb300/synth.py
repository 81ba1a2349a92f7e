"""Seeded synthetic orbitals and local potentials (host side, numpy).

The workloads of this package are synthetic: each orbital is a Gaussian
exp(-|r - c|^2 / (2 sigma^2)) under the periodic minimum image, sigma uniform
in [1, 2] bohr, centre uniform in the box, multiplied pointwise by
(1 + 0.05 N(0,1)).  The local potential is a sum of Gaussian wells of depth
U[-2, -0.5] Ha and width 1.5 bohr.  Grid points sit at r = (i h) with the
origin at 0, matching pb::Grid with a zero origin (src/pb/Grid.cc:18-96).

The random stream is numpy's counter-based Philox generator keyed by the
seed; orbitals and potential use separate streams (seed, seed + 50000).
Device-side generation of the same distributions for the large workloads
lives in csrc (mgx_synth_*), which is the path bench.py uses.
"""
import numpy as np


def _coords(n, ll):
    h = [ll[i] / n[i] for i in range(3)]
    return [np.arange(n[i], dtype=np.float64) * h[i] for i in range(3)]


def _min_image_sq(x, c, L):
    d = x - c
    d = d - L * np.round(d / L)
    return d * d


def gaussian_orbitals(n, ll, nfunc, seed, dtype=np.float64, noise=0.05,
                      sigma=(1.0, 2.0)):
    """Returns (psi[nfunc, nx*ny*nz], centers[nfunc,3], sigmas[nfunc])."""
    rng = np.random.Generator(np.random.Philox(key=seed))
    centers = rng.uniform(0.0, 1.0, size=(nfunc, 3)) * np.asarray(ll)[None, :]
    sig = rng.uniform(sigma[0], sigma[1], size=nfunc)
    xs = _coords(n, ll)
    psi = np.empty((nfunc, n[0] * n[1] * n[2]), dtype=dtype)
    for f in range(nfunc):
        dx = _min_image_sq(xs[0], centers[f, 0], ll[0])
        dy = _min_image_sq(xs[1], centers[f, 1], ll[1])
        dz = _min_image_sq(xs[2], centers[f, 2], ll[2])
        r2 = dx[:, None, None] + dy[None, :, None] + dz[None, None, :]
        g = np.exp(-r2 / (2.0 * sig[f] * sig[f]))
        g *= 1.0 + noise * rng.standard_normal(g.shape)
        psi[f] = g.reshape(-1).astype(dtype)
    return psi, centers, sig


def gaussian_wells(n, ll, nwells, seed, width=1.5, depth=(-2.0, -0.5)):
    """Local potential V (Hartree) on the grid, flattened, float64."""
    rng = np.random.Generator(np.random.Philox(key=seed + 50000))
    R = rng.uniform(0.0, 1.0, size=(nwells, 3)) * np.asarray(ll)[None, :]
    d = rng.uniform(depth[0], depth[1], size=nwells)
    xs = _coords(n, ll)
    V = np.zeros((n[0], n[1], n[2]))
    for k in range(nwells):
        dx = _min_image_sq(xs[0], R[k, 0], ll[0])
        dy = _min_image_sq(xs[1], R[k, 1], ll[1])
        dz = _min_image_sq(xs[2], R[k, 2], ll[2])
        r2 = dx[:, None, None] + dy[None, :, None] + dz[None, None, :]
        V += d[k] * np.exp(-r2 / (2.0 * width * width))
    return V.reshape(-1)


def mask_radii(nfunc, seed, lo=4.0, hi=8.0):
    """Seeded localization radii U[lo, hi] bohr."""
    rng = np.random.Generator(np.random.Philox(key=seed + 70000))
    return rng.uniform(lo, hi, size=nfunc)


def gaussian_orbitals_device(n, ll, nfunc, seed, dtype, device="cuda", noise=0.05,
                             sigma=(1.0, 2.0), chunk=32):
    """The same distributions as gaussian_orbitals, generated on the GPU with
    torch's seeded device generator (used for the large benchmark blocks,
    where host generation and upload would dominate).  Returns the block
    (nfunc, nx*ny*nz) on `device`."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    L = torch.tensor(ll, dtype=torch.float64, device=device)
    centers = torch.rand((nfunc, 3), generator=g, dtype=torch.float64, device=device) * L
    sig = sigma[0] + (sigma[1] - sigma[0]) * torch.rand(nfunc, generator=g, dtype=torch.float64,
                                                        device=device)
    xs = [torch.arange(n[i], dtype=torch.float64, device=device) * (ll[i] / n[i]) for i in range(3)]
    out = torch.empty((nfunc, n[0] * n[1] * n[2]), dtype=dtype, device=device)
    for f0 in range(0, nfunc, chunk):
        f1 = min(nfunc, f0 + chunk)
        c = centers[f0:f1]
        d2 = []
        for i in range(3):
            d = xs[i][None, :] - c[:, i:i + 1]
            d = d - L[i] * torch.round(d / L[i])
            d2.append(d * d)
        r2 = (d2[0][:, :, None, None] + d2[1][:, None, :, None] + d2[2][:, None, None, :])
        s = sig[f0:f1][:, None, None, None]
        gv = torch.exp(-r2 / (2.0 * s * s))
        gv *= 1.0 + noise * torch.randn(gv.shape, generator=g, dtype=torch.float64, device=device)
        out[f0:f1] = gv.reshape(f1 - f0, -1).to(dtype)
    return out, centers, sig


def gaussian_wells_device(n, ll, nwells, seed, device="cuda", width=1.5, depth=(-2.0, -0.5)):
    """Sum of Gaussian wells on the GPU (float64, flattened)."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed) + 50000)
    L = torch.tensor(ll, dtype=torch.float64, device=device)
    R = torch.rand((nwells, 3), generator=g, dtype=torch.float64, device=device) * L
    dep = depth[0] + (depth[1] - depth[0]) * torch.rand(nwells, generator=g, dtype=torch.float64,
                                                        device=device)
    xs = [torch.arange(n[i], dtype=torch.float64, device=device) * (ll[i] / n[i]) for i in range(3)]
    V = torch.zeros((n[0], n[1], n[2]), dtype=torch.float64, device=device)
    for k in range(nwells):
        d2 = []
        for i in range(3):
            d = xs[i] - R[k, i]
            d = d - L[i] * torch.round(d / L[i])
            d2.append(d * d)
        r2 = d2[0][:, None, None] + d2[1][None, :, None] + d2[2][None, None, :]
        V += dep[k] * torch.exp(-r2 / (2.0 * width * width))
    return V.reshape(-1)
