"""The allocation-free V-cycle entry point, mgx_precond_mg_static.

Callers that cannot allocate device memory (under a memory pool they do
not own, or in a process that forbids device allocations after start-up)
use this entry point; its scratch is a fixed 64 MiB device array inside the
library.  This file is collected last
so that a failure here never hides another test; it passes alone in a fresh
process as well as after the rest of the suite.
"""
import ctypes

import numpy as np
import pytest
import torch

from helpers import TOL_F64, rel_err
from mgmol_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _static(ctx, res, lap_type, maxlevels, gamma, chunk=0):
    """Calls mgx_precond_mg_static through the C ABI."""
    L = capi.load()
    out = torch.empty_like(res)
    prm = capi.PrecondParams(lap_type, maxlevels, float(gamma), int(chunk))
    dt = capi.F64 if res.dtype == torch.float64 else capi.F32
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = L.mgx_precond_mg_static(ctx.handle, ctypes.byref(prm), dt, ctypes.c_void_p(res.data_ptr()),
                                 res.stride(0), ctypes.c_void_p(out.data_ptr()), res.shape[0], None, stream)
    assert st == capi.MGX_OK, L.mgx_last_error_string().decode()
    return out


@pytest.mark.parametrize("dtype,tol", [(torch.float64, TOL_F64), (torch.float32, 1e-6)])
def test_static_vcycle_matches_allocating_entry_point(dtype, tol):
    # 32^3, FP64: about 0.67 MB of scratch per function, so 130 functions
    # take two chunks of the 64 MiB array
    n = (32, 32, 32)
    ll = tuple(x * 0.35 for x in n)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 130, 77)
    res = torch.from_numpy(psi).to(dtype=dtype, device="cuda")
    ctx = capi.Context(n, ll)
    ref = ctx.precond_mg(res, capi.LAP_MEHR4, 2, 0.3).cpu().numpy()
    first = _static(ctx, res, capi.LAP_MEHR4, 2, 0.3).cpu().numpy()
    second = _static(ctx, res, capi.LAP_MEHR4, 2, 0.3).cpu().numpy()
    assert rel_err(first, ref) < tol
    assert rel_err(second, ref) < tol
    assert np.array_equal(first, second)


def test_static_vcycle_rejects_functions_larger_than_the_scratch():
    # one FP32 function on 192^3 with two coarse levels needs about 72 MB
    n = (192, 192, 192)
    ctx = capi.Context(n, tuple(x * 0.25 for x in n))
    L = capi.load()
    prm = capi.PrecondParams(capi.LAP_MEHR4, 2, 0.3, 0)
    res = torch.zeros((1, n[0] * n[1] * n[2]), dtype=torch.float32, device="cuda")
    out = torch.empty_like(res)
    st = L.mgx_precond_mg_static(ctx.handle, ctypes.byref(prm), capi.F32, ctypes.c_void_p(res.data_ptr()),
                                 res.stride(0), ctypes.c_void_p(out.data_ptr()), 1, None, None)
    assert st == capi.MGX_BAD_ARG
    assert b"static scratch" in L.mgx_last_error_string()
