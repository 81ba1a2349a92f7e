"""Snapshots of device arrays: an orbital block larger than the 64 MiB
staging chunks streams out and back bit for bit, and the learned
preconditioner's weights restore a network that gives the same output."""
import numpy as np
import pytest
import torch

from mgmol_gb300 import capi, restart, synth

pytestmark = pytest.mark.gpu


def test_device_block_round_trip(tmp_path):
    n = (96, 96, 96)
    ll = tuple(0.3 * x for x in n)
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, 48, 9, torch.float32)   # 170 MB
    V = synth.gaussian_wells_device(n, ll, 8, 9)
    p = tmp_path / "block.bin"
    restart.save(p, grid=(n, ll), meta={"orbitals": 48}, psi=psi, V=V)
    back = torch.empty_like(psi)
    restart.load(p, "psi", out=back)
    assert torch.equal(back, psi)
    assert torch.equal(restart.load(p, "V", device="cuda"), V)


def test_learned_weights_restore_the_network(tmp_path):
    import sys
    import os
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(__file__)), "oracle"))
    import unet_oracle as UO
    n = (32, 32, 32)
    ctx = capi.Context(n, tuple(0.35 * x for x in n))
    net = capi.UNet(ctx)
    net.set_params(UO.init_params(3))
    x = torch.randn((2, ctx.npts), dtype=torch.float32, device="cuda")
    for _ in range(2):
        net.train_step(x, 0.5 * x, 1e-3)
    y = net.forward(x)
    p = tmp_path / "net.bin"
    restart.save(p, meta={"network": "unet"}, unet=net.get_params())
    net2 = capi.UNet(ctx)
    net2.set_params(restart.load(p, "unet").numpy())
    assert torch.equal(net2.forward(x), y)
