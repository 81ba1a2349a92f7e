"""The V-cycle with the residual of each level's second pre-sweep
restricted inside that sweep's kernel (the default) against the V-cycle
with the residual stored and restricted by its own kernel
(MGX_FUSED_RESTRICT=0), the V-cycle with both pre-sweeps and both
post-sweeps of a level each in one kernel against single sweeps
(MGX_TWO_SWEEPS=0; the pre-sweep pair where it pays, everywhere it runs,
and nowhere; blocks of 256 and 512 threads), the post-sweep pair starting from the coarse-grid correction
formed on chip (MGX_PAIR_PROLONG=1) against the prolongation kernel, and
the FP32 prolongation with four z points per
thread against the pair form (MGX_PROLONG4=0), each in a fresh process
(the library reads the choice once): the same bits, FP64 and FP32, on
grids whose tile rows and x chunks end unevenly, plain, warm-started, in
chunks and with the update fused into the last sweep; and the fused FP64
V-cycle against the oracle."""
import os
import subprocess
import sys

import numpy as np
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

outs = {}
for n, nf, maxl in (((32, 28, 36), 5, 2), ((48, 40, 24), 3, 1), ((64, 64, 64), 4, 2)):
    ll = tuple(x * 0.35 for x in n)
    res, _, _ = synth.gaussian_orbitals(n, ll, nf, 61)
    ctx = capi.Context(n, ll)
    for dt in (torch.float64, torch.float32):
        for lap in (0, 1, 2):
            rin = torch.from_numpy(res).to(dtype=dt, device="cuda")
            o = ctx.precond_mg(rin, lap, maxl, 0.3)
            outs[f"{n}_{dt}_{lap}"] = o.cpu().numpy()
            # a warm start (the first sweep from the iterate out holds)
            outs[f"warm_{n}_{dt}_{lap}"] = ctx.precond_mg_warm(rin, o.clone(), lap, maxl).cpu().numpy()
            # chunks of two functions
            outs[f"chunk_{n}_{dt}_{lap}"] = ctx.precond_mg(rin, lap, maxl, 0.3, chunk=2).cpu().numpy()
            # the update fused into the last sweep, with the column scale
            psi = torch.flip(rin, (0,)).contiguous()
            sc = torch.linspace(0.5, 1.5, nf, dtype=torch.float64, device="cuda")
            ctx.precond_update(rin, psi, -0.3, lap, maxl, 0.3, psi_scale=sc)
            outs[f"upd_{n}_{dt}_{lap}"] = psi.cpu().numpy()
    ref = O.precond(n, ll, 0, maxl, 0.3, res)
    got = outs[f"{n}_{torch.float64}_0"]
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) < 1e-12, n
np.savez(OUT, **outs)
print("vcycle ok")
"""


def _run(tmp_path, env, tag):
    out = str(tmp_path / f"{tag}.npz")
    r = subprocess.run([sys.executable, "-c", SCRIPT.replace("ROOT", repr(ROOT)).replace("OUT", repr(out))],
                       env={**os.environ, **env}, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "vcycle ok" in r.stdout, r.stdout[-2000:] + r.stderr[-2000:]
    return np.load(out)


def test_fused_restriction_gives_the_same_bits(tmp_path):
    a = _run(tmp_path, {"MGX_FUSED_RESTRICT": "1"}, "fused")
    b = _run(tmp_path, {"MGX_FUSED_RESTRICT": "0"}, "separate")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k


def test_prolongation_four_wide_gives_the_same_bits(tmp_path):
    a = _run(tmp_path, {"MGX_PROLONG4": "1"}, "four")
    b = _run(tmp_path, {"MGX_PROLONG4": "0"}, "pair")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k


@pytest.mark.parametrize("pre_pair,threads", [("auto", "auto"), ("1", "256"), ("0", "auto"),
                                              ("1", "512")])
def test_paired_sweeps_give_the_same_bits(tmp_path, pre_pair, threads):
    env = {"MGX_TWO_SWEEPS": "1"}
    if threads != "auto":
        env["MGX_JJ_THREADS"] = threads
    if pre_pair != "auto":
        env["MGX_PRE_PAIR"] = pre_pair
    a = _run(tmp_path, env, "pairs")
    b = _run(tmp_path, {"MGX_TWO_SWEEPS": "0"}, "single")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k


def test_folded_prolongation_gives_the_same_bits(tmp_path):
    a = _run(tmp_path, {"MGX_PAIR_PROLONG": "1"}, "folded")
    b = _run(tmp_path, {"MGX_PAIR_PROLONG": "0"}, "kernel")
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k]), k
