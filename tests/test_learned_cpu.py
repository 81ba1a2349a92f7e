"""CPU checks of the learned preconditioner's oracle (oracle/unet_oracle.py):
its restriction and prolongation are the pinned V-cycle transfers, its
autograd gradient agrees with finite differences, and the bias-free
network is positively homogeneous."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import oracle as O  # noqa: E402
import unet_oracle as L  # noqa: E402


def _tensor(u, n):
    return torch.from_numpy(u).reshape(u.shape[0], 1, *n)


def test_transfers_are_the_vcycle_transfers():
    n = (8, 12, 16)
    ll = (4.0, 6.0, 8.0)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((3, n[0] * n[1] * n[2]))
    nc = tuple(v // 2 for v in n)
    r = L.restrict(_tensor(u, n)).reshape(3, -1).numpy()
    np.testing.assert_allclose(r, O.restrict(n, ll, u), rtol=0, atol=1e-14)
    c = rng.standard_normal((3, nc[0] * nc[1] * nc[2]))
    p = L.prolong(_tensor(c, nc)).reshape(3, -1).numpy()
    np.testing.assert_allclose(p, O.extend(n, ll, c), rtol=0, atol=1e-14)


def test_restriction_adjoint_is_prolongation_over_eight():
    # the identity the backward pass of mgx_learn.cu relies on: R^T = P / 8
    n = (8, 8, 8)
    rng = np.random.default_rng(4)
    u = torch.from_numpy(rng.standard_normal((1, 1, *n)))
    c = torch.from_numpy(rng.standard_normal((1, 1, 4, 4, 4)))
    lhs = float((L.restrict(u) * c).sum())
    rhs = float((u * L.prolong(c)).sum()) / 8.0
    assert abs(lhs - rhs) < 1e-12 * abs(lhs)


def test_autograd_gradient_matches_finite_differences():
    n = (8, 8, 8)
    rng = np.random.default_rng(5)
    p = torch.from_numpy(L.init_params(7).astype(np.float64))
    x = torch.from_numpy(rng.standard_normal((2, 1, *n)))
    t = torch.from_numpy(rng.standard_normal((2, 1, *n)))

    def loss(q):
        e = L.net_normalized(x, L.split(q)) - t
        return (e * e).mean()

    q = p.clone().requires_grad_(True)
    loss(q).backward()
    g = q.grad.numpy()
    h = 1e-6
    offs = np.cumsum([0] + [ci * co * 27 for ci, co, _ in L.LAYERS])
    for layer in range(6):
        i = int(offs[layer] + 5)
        e = torch.zeros_like(p)
        e[i] = h
        fd = (float(loss(p + e)) - float(loss(p - e))) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (layer, fd, g[i])


def test_network_is_positively_homogeneous():
    n = (8, 8, 8)
    rng = np.random.default_rng(6)
    p = L.init_params(8)
    x = rng.standard_normal((2, 512))
    y1 = L.forward(n, p, x)
    y2 = L.forward(n, p, 3.5 * x)
    np.testing.assert_allclose(y2, 3.5 * y1, rtol=1e-12, atol=1e-12 * np.abs(y1).max())
