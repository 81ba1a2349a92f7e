"""C-ABI checks that need no GPU: the library loads, exports exactly the
entry points include/mgx.h declares, and its host-only logic behaves."""
import ctypes
import os
import re
import subprocess

import pytest

from mgmol_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            names |= set(re.findall(r"^(?:int|const char\*|unsigned long long)\s+(mgx_\w+)\(", txt, re.M))
    return names


def test_library_exports_every_declared_symbol():
    capi.load()
    out = subprocess.run(["nm", "-D", "--defined-only", capi.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if re.search(r"\sT\smgx_", l)}
    declared = _declared()
    assert declared, "no declarations parsed"
    assert declared == exported, (declared ^ exported)
    assert declared == set(capi.EXPORTS)


def test_build_recipe_targets_sm103a_only():
    """The recipe compiles and links for sm_103a and nothing else; the
    loaded module's architecture is checked on the GPU (test_build_gpu)."""
    from mgmol_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_precond_gamma_host_logic():
    """mgx_precond_gamma is host arithmetic: setGamma with Laph4M invDiag."""
    import oracle as O
    g = capi.Grid.make((64, 64, 64), (22.4, 22.4, 22.4))
    out = ctypes.c_double()
    st = capi.load().mgx_precond_gamma(ctypes.byref(g), 0, 2, -0.5, -1.7, ctypes.byref(out))
    assert st == capi.MGX_OK
    h = 22.4 / 64
    inv_diag = 1.0 / ((4.0 / 3.0) * 3.0 / (h * h))
    assert abs(out.value - O.set_gamma(inv_diag, 2, -0.5, -1.7)) < 1e-15 * out.value


def test_bad_arguments_are_reported_not_aborted():
    L = capi.load()
    g = capi.Grid.make((16, 16, 16), (4.0, 4.0, 4.0), bc=(1, 0, 1))
    h = ctypes.c_void_p()
    assert L.mgx_create(ctypes.byref(g), ctypes.byref(h)) == capi.MGX_UNSUPPORTED
    assert b"periodic" in L.mgx_last_error_string()
    g2 = capi.Grid.make((0, 16, 16), (4.0, 4.0, 4.0))
    assert L.mgx_create(ctypes.byref(g2), ctypes.byref(h)) == capi.MGX_BAD_ARG
    assert L.mgx_fd_apply(None, 0, 0, None, 0, None, 1, None) == capi.MGX_BAD_ARG
    out = ctypes.c_double()
    assert L.mgx_precond_gamma(ctypes.byref(capi.Grid.make((8, 8, 8), (1, 1, 1))), 9, 1, 0.0, 0.0,
                               ctypes.byref(out)) == capi.MGX_BAD_ARG


def test_learned_and_local_entry_points_check_their_arguments():
    """Entry points of the learned preconditioner and the localized orbitals
    refuse NULL handles and inconsistent arguments before any device work."""
    L = capi.load()
    h = ctypes.c_void_p()
    assert L.mgx_unet_create(None, ctypes.byref(h)) == capi.MGX_BAD_ARG
    assert L.mgx_unet_forward(None, None, 0, None, 1, None) == capi.MGX_BAD_ARG
    assert L.mgx_unet_loss_grad(None, None, None, 0, 1, None, None, None) == capi.MGX_BAD_ARG
    prm = capi.AdamParams(1e-3, 0.9, 0.999, 1e-8)
    assert L.mgx_unet_adam(None, None, ctypes.byref(prm), None) == capi.MGX_BAD_ARG
    assert L.mgx_unet_train_step(None, None, None, 0, 1, ctypes.byref(prm), None, None) \
        == capi.MGX_BAD_ARG
    pp = capi.PrecondParams(0, 2, 0.1, 0)
    assert L.mgx_precond_learned(None, None, ctypes.byref(pp), None, 0, None, 1, 0, None, None,
                                 None, None) == capi.MGX_BAD_ARG
    assert L.mgx_precond_mg_warm(None, ctypes.byref(pp), 0, None, 0, None, 1, None, None) \
        == capi.MGX_BAD_ARG
    assert L.mgx_local_create(None, None, None, ctypes.byref(h)) == capi.MGX_BAD_ARG
    assert L.mgx_local_step(None, None, None, None, 0.1, None, None, None) == capi.MGX_BAD_ARG
    assert L.mgx_local_set_config(None, 0, 2, 1) == capi.MGX_BAD_ARG
    assert L.mgx_local_layout(None, None, None, None) == capi.MGX_BAD_ARG
    assert capi.UNET_PARAMS == sum(ci * co * 27 for ci, co in
                                   ((1, 16), (16, 32), (32, 64), (64, 32), (32, 16), (16, 1)))
