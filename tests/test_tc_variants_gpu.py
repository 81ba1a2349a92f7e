"""The tensor-core product kernels in their other launch forms, each in a
fresh process (the library reads the choice once): the split-K products
(S, H, B) on the persistent two-accumulator kernel (MGX_TC_PERSIST_SPLITK=1),
every product on one CTA per output tile (MGX_TC_PERSIST=0), and the
split-K tiles in column order (MGX_TC_TILE_ORDER=col), against the FP64
oracle at the split-BF16x3 error bars."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import sys
import numpy as np
import torch
sys.path.insert(0, ROOT)
sys.path.insert(0, ROOT + "/oracle")
import oracle as O
from mgmol_gb300 import capi, synth

def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))

n = (32, 24, 20)
ll = tuple(x * 0.35 for x in n)
psi, _, _ = synth.gaussian_orbitals(n, ll, 200, 23)
V = synth.gaussian_wells(n, ll, 6, 23)
p32 = psi.astype(np.float32)
ctx = capi.Context(n, ll)
dp = torch.from_numpy(p32).cuda()
hp = ctx.hpsi(dp, torch.from_numpy(V.astype(np.float32)).cuda())
S, H = ctx.gram_hmat(dp, hp, capi.GEMM_BF16X3)
assert rel(S.cpu().numpy(), O.gram(p32, ctx.vel)) < 2e-5, "S"
assert rel(H.cpu().numpy(), O.hmat(p32, hp.cpu().numpy().astype(np.float64), ctx.vel)) < 2e-5, "H"
B = ctx.matb(dp, capi.GEMM_BF16X3)
assert rel(np.tril(B.cpu().numpy()), np.tril(O.matb(n, ll, p32.astype(np.float64)))) < 2e-5, "B"
th = np.eye(200) + np.random.default_rng(3).standard_normal((200, 200)) / 200
out = ctx.mult_matrix(dp, torch.from_numpy(th).cuda(), capi.GEMM_BF16X3)
ref = O.mult_matrix(p32.astype(np.float64), th)
assert rel(out.cpu().numpy(), ref) < 6e-5, "Psi Theta"
print("variant ok")
"""


@pytest.mark.parametrize("env", [{"MGX_TC_PERSIST_SPLITK": "1"}, {"MGX_TC_PERSIST": "0"},
                                 {"MGX_TC_TILE_ORDER": "col"}])
def test_product_kernel_launch_forms(env):
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT))],
                       env={**os.environ, **env}, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "variant ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
