"""CPU oracle of the learned preconditioner's network -- TEST
INFRASTRUCTURE ONLY (tests/, __graft_entry__.smoke() and bench.py's CPU leg
use it as the checker; the product never imports it).

A float64 restatement, on the CPU in torch with autograd for the
gradients, of the 3-level 3-D convolutional U-Net that
mgmol_gb300/csrc/mgx_learn.cu runs on the GPU.  The reference has no
learned preconditioner; what ties this network to the reference is its
down- and upsampling, which are the V-cycle's full-weighting restriction
and trilinear prolongation (src/pb/MGkernels.cc:28-283), checked against
this directory's pinned restatement (oracle.restrict / oracle.extend) by
tests/test_learned_cpu.py.

Fields: arrays (nfunc, nx * ny * nz), points x-slowest / z-fastest, on a
periodic grid; the network works on (N, C, nx, ny, nz) tensors.

Layers (bias-free 3x3x3 cross-correlations, periodic; channels in -> out,
level): E0 1->16 @0, E1 16->32 @1, E2 32->64 @2, D2 64->32 @2,
D1 32->16 @1, D0 16->1 @0:
    a0 = relu(E0 x)          a1 = relu(E1 R a0)     a2 = relu(E2 R a1)
    s1 = relu(P D2 a2 + a1)  s0 = relu(P D1 s1 + a0) y = D0 s0
with x the input divided by its RMS and the output multiplied by it.
Weights as used on the GPU: the FP32 master values rounded to BF16.
"""
import numpy as np
import torch
import torch.nn.functional as F

LAYERS = [(1, 16, 0), (16, 32, 1), (32, 64, 2), (64, 32, 2), (32, 16, 1), (16, 1, 0)]
NPARAM = sum(ci * co * 27 for ci, co, _ in LAYERS)
assert NPARAM == 139104

_R1 = np.array([0.25, 0.5, 0.25])
_P1 = np.array([0.5, 1.0, 0.5])


def _k3(v):
    return torch.tensor(np.einsum("a,b,c->abc", v, v, v), dtype=torch.float64).view(1, 1, 3, 3, 3)


_RK = _k3(_R1)
_PK = _k3(_P1)


def init_params(seed):
    """He-normal initial weights (fan-in 27 * cin), FP32."""
    rng = np.random.default_rng(seed)
    out = []
    for ci, co, _ in LAYERS:
        out.append(rng.standard_normal(ci * co * 27) * np.sqrt(2.0 / (27 * ci)))
    return np.concatenate(out).astype(np.float32)


def bf16_round(p):
    """FP32 values rounded to BF16 (round to nearest even), as float64."""
    t = torch.from_numpy(np.asarray(p, dtype=np.float32).copy())
    return t.to(torch.bfloat16).to(torch.float64)


def split(p):
    """The six weight tensors (cout, cin, 3, 3, 3) of a parameter vector."""
    ws, o = [], 0
    for ci, co, _ in LAYERS:
        n = ci * co * 27
        ws.append(p[o:o + n].view(co, ci, 3, 3, 3))
        o += n
    return ws


def _pad(x):
    return F.pad(x, (1, 1, 1, 1, 1, 1), mode="circular")


def conv(x, w):
    return F.conv3d(_pad(x), w)


def restrict(x):
    """Full weighting, fine (N, C, n) -> coarse (N, C, n / 2), periodic."""
    N, C = x.shape[:2]
    y = F.conv3d(_pad(x.reshape(N * C, 1, *x.shape[2:])), _RK, stride=2)
    return y.reshape(N, C, *y.shape[2:])


def prolong(x):
    """Trilinear prolongation, coarse (N, C, n) -> fine (N, C, 2 n), periodic."""
    N, C = x.shape[:2]
    n = x.shape[2:]
    z = torch.zeros(N * C, 1, 2 * n[0], 2 * n[1], 2 * n[2], dtype=x.dtype)
    z[:, :, ::2, ::2, ::2] = x.reshape(N * C, 1, *n)
    y = F.conv3d(_pad(z), _PK)
    return y.reshape(N, C, *y.shape[2:])


def net_normalized(xh, ws):
    """The network on RMS-normalized inputs (N, 1, nx, ny, nz)."""
    W0, W1, W2, W3, W4, W5 = ws
    a0 = F.relu(conv(xh, W0))
    a1 = F.relu(conv(restrict(a0), W1))
    a2 = F.relu(conv(restrict(a1), W2))
    s1 = F.relu(prolong(conv(a2, W3)) + a1)
    s0 = F.relu(prolong(conv(s1, W4)) + a0)
    return conv(s0, W5)


def _fields(x, n):
    x = torch.as_tensor(np.asarray(x, dtype=np.float64))
    return x.reshape(-1, 1, n[0], n[1], n[2])


def _rms(x):
    s = torch.sqrt((x * x).mean(dim=(1, 2, 3, 4), keepdim=True))
    return torch.where(s > 0, s, torch.ones_like(s))


def forward(n, params, x):
    """net(x) for fields x (nfunc, npts): s * net_normalized(x / s)."""
    ws = split(bf16_round(params))
    xt = _fields(x, n)
    s = _rms(xt)
    with torch.no_grad():
        y = net_normalized(xt / s, ws) * s
    return y.reshape(xt.shape[0], -1).numpy()


def loss_grad(n, params, x, t):
    """(loss, grad): loss = mean over functions and points of
    (net_normalized(x / s) - t / s)^2 and its gradient with respect to the
    BF16-rounded weights (float64, length NPARAM)."""
    p = bf16_round(params).requires_grad_(True)
    ws = split(p)
    xt = _fields(x, n)
    tt = _fields(t, n)
    s = _rms(xt)
    e = net_normalized(xt / s, ws) - tt / s
    loss = (e * e).mean()
    loss.backward()
    return float(loss.detach()), p.grad.numpy().copy()


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step in float64; returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1 = 1.0 / (1.0 - b1 ** step)
    c2 = 1.0 / (1.0 - b2 ** step)
    return params - lr * (m * c1) / (np.sqrt(v * c2) + eps), m, v
