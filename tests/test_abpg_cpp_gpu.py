"""The C++ host driver of one quench iteration (mgmol_gb300/cpp/abpg_step.h,
AbpgStep<T>) through tests/cpp/test_abpg.cpp: FP64 against the oracle chain
of the reference's iteration (normalize, H psi, S / H / B, theta = B^-1 H,
HB, energy, residual, V-cycle, update), in the fused, unfused and
column-chunked schedules; FP32 with split-BF16x3 products against the
Python schedule of the same kernels (mgmol_gb300/sweep.py)."""
import os
import subprocess

import numpy as np
import pytest
import torch

from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth
from test_residual_gpu import _oracle_step

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_abpg_test():
    capi.load()
    out = os.path.join(ROOT, "mgmol_gb300", "_build", "test_abpg")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    libdir = os.path.join(ROOT, "mgmol_gb300")
    cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "mgmol_gb300", "cpp"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "cpp", "test_abpg.cpp"),
           "-o", out, "-L", libdir, "-lmgx", f"-Wl,-rpath,{libdir}", "-L", os.path.join(CUDA, "lib64"),
           "-lcudart", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run(tmp_path, grid, ll, V, psi, steps, fuse, chunk, gemm, gamma):
    exe = build_abpg_test()
    nf = psi.shape[0]
    dt = 0 if psi.dtype == np.float64 else 1
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        np.array(list(grid) + [nf, dt, steps, int(fuse), chunk, gemm], dtype=np.int32).tofile(f)
        np.array(list(ll) + [float(V.min()), float(V.max()), gamma], dtype=np.float64).tofile(f)
        np.ascontiguousarray(V, dtype=np.float64).tofile(f)
        np.ascontiguousarray(psi).tofile(f)
    r = subprocess.run([exe, str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    raw = np.fromfile(outp, dtype=np.uint8)
    e = raw[: 8 * steps].view(np.float64)
    g = raw[8 * steps: 8 * steps + 8].view(np.float64)[0]
    out = raw[8 * steps + 8:].view(psi.dtype).reshape(psi.shape)
    return e, g, out


def test_abpg_driver_compiles():
    assert os.path.exists(build_abpg_test())


@pytest.mark.gpu
@pytest.mark.parametrize("fuse,chunk", [(True, 0), (False, 0), (False, 5)])
def test_abpg_driver_fp64_matches_oracle_chain(tmp_path, fuse, chunk):
    grid, nf = (16, 16, 16), 12
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 41, sigma=(0.9, 1.3))
    psi = psi * np.linspace(0.7, 1.6, nf)[:, None]      # not normalized on entry
    V = synth.gaussian_wells(grid, ll, 4, 41)
    e, gamma, out = _run(tmp_path, grid, ll, V, psi, 1, fuse, chunk, capi.GEMM_FP64, 0.0)
    ref, e_ref, _, _ = _oracle_step(grid, ll, psi, V, 0.5, gamma)
    assert abs(e[0] - e_ref) < 1e-11 * abs(e_ref)
    assert rel_err(out, ref) < TOL_F64


@pytest.mark.gpu
def test_abpg_driver_fp32_matches_python_schedule(tmp_path):
    from mgmol_gb300.sweep import OrbitalSweep
    grid, nf = (32, 32, 32), 40
    ll = tuple(x * 0.35 for x in grid)
    psi, _, _ = synth.gaussian_orbitals(grid, ll, nf, 43)
    V = synth.gaussian_wells(grid, ll, 6, 43)
    ctx = capi.Context(grid, ll)
    sw = OrbitalSweep(ctx, torch.from_numpy(V), nf, mode="mixed", gemm=capi.GEMM_BF16X3)
    pd = torch.from_numpy(psi.astype(np.float32)).cuda()
    e_py = [float(sw.run(pd).cpu()[0]) for _ in range(3)]
    e, _, out = _run(tmp_path, grid, ll, V.astype(np.float32).astype(np.float64),
                     psi.astype(np.float32), 3, True, 0, capi.GEMM_BF16X3, sw.gamma)
    # the same kernels in the same order; the split-K FP64 atomics sum in
    # either order
    np.testing.assert_allclose(e, e_py, rtol=1e-9)
    assert rel_err(out, pd.cpu().numpy()) < 1e-5
