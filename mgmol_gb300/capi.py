"""ctypes binding of the mgx C ABI (include/mgx.h) with torch device tensors.

This is the Python face of the library used by the tests and the benchmark;
C++ callers use include/mgx.h directly or the MGmol-shaped adaptor classes in
mgmol_gb300/cpp/.  The shared library is the in-tree mgmol_gb300/libmgx.so
built for sm_103a; there is no other implementation behind these calls, and
importing fails loudly when the library cannot be loaded.

Orbital blocks are torch tensors of shape (nfunc, nx*ny*nz) (or (nx*ny*nz,)
for one function), float64 or float32, on the CUDA device, points x-slowest
and z-fastest.  Matrices are (n, n) float64 tensors, column-major as in the
C ABI (use .T to read them row-major; S and S^-1 are symmetric).
"""
import ctypes
import os

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmgx.so")

MGX_OK, MGX_BAD_ARG, MGX_NOT_SPD, MGX_NONFINITE, MGX_TIMEOUT, MGX_CUDA_ERROR, \
    MGX_UNSUPPORTED, MGX_NO_MEMORY = range(8)
F64, F32 = 0, 1
GEMM_FP64, GEMM_FP32, GEMM_TF32, GEMM_BF16X3, GEMM_FP16X3 = 0, 1, 2, 3, 4
LAP_MEHR4, LAP_2ND, LAP_4TH, LAP_6TH, LAP_8TH = 0, 1, 2, 3, 4

_STATUS = {0: "MGX_OK", 1: "MGX_BAD_ARG", 2: "MGX_NOT_SPD", 3: "MGX_NONFINITE", 4: "MGX_TIMEOUT",
           5: "MGX_CUDA_ERROR", 6: "MGX_UNSUPPORTED", 7: "MGX_NO_MEMORY"}


class MgxError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")
        self.status = status


class Grid(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("ll", ctypes.c_double * 3), ("bc", ctypes.c_int * 3)]

    @staticmethod
    def make(n, ll, bc=(1, 1, 1)):
        g = Grid()
        for i in range(3):
            g.n[i] = int(n[i])
            g.ll[i] = float(ll[i])
            g.bc[i] = int(bc[i])
        return g


class PrecondParams(ctypes.Structure):
    _fields_ = [("lap_type", ctypes.c_int), ("maxlevels", ctypes.c_int), ("gamma", ctypes.c_double),
                ("chunk", ctypes.c_int)]


class MgmParams(ctypes.Structure):
    _fields_ = [("lap_type", ctypes.c_int), ("max_levels", ctypes.c_int),
                ("max_sweeps", ctypes.c_int), ("tol", ctypes.c_double), ("nu1", ctypes.c_int),
                ("nu2", ctypes.c_int), ("ghosts", ctypes.c_int)]


class MgmResult(ctypes.Structure):
    _fields_ = [("final_residual", ctypes.c_double), ("final_relative_residual", ctypes.c_double),
                ("residual_reduction", ctypes.c_double), ("nb_sweeps", ctypes.c_int),
                ("converged", ctypes.c_int), ("levels", ctypes.c_int)]


ANDERSON_MAX_M = 8


class AndersonInfo(ctypes.Structure):
    _fields_ = [("mm", ctypes.c_int), ("reductions", ctypes.c_int),
                ("theta", ctypes.c_double * ANDERSON_MAX_M)]


class Dataset(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char_p), ("type", ctypes.c_int), ("ndim", ctypes.c_int),
                ("shape", ctypes.c_size_t * 4), ("data", ctypes.c_void_p)]


SNAP_F64, SNAP_F32, SNAP_I32, SNAP_U8 = 0, 1, 2, 3


class AdamParams(ctypes.Structure):
    _fields_ = [("lr", ctypes.c_float), ("beta1", ctypes.c_float), ("beta2", ctypes.c_float),
                ("eps", ctypes.c_float)]


UNET_PARAMS = 139104
LEARNED_REPLACE, LEARNED_WARM, LEARNED_REFRESH = 0, 1, 2

_LIB = None
_vp = ctypes.c_void_p
_i = ctypes.c_int
_sz = ctypes.c_size_t
_d = ctypes.c_double
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)

_SIGS = {
    "mgx_create": [ctypes.POINTER(Grid), ctypes.POINTER(_vp)],
    "mgx_destroy": [_vp],
    "mgx_fdkernel_del2": [ctypes.POINTER(Grid), _i, _i, _i, _vp, _vp, _sz, _vp],
    "mgx_fdkernel_rhs_mehr1": [ctypes.POINTER(Grid), _i, _i, _vp, _vp, _i, _sz, _vp],
    "mgx_mgkernel_restrict3d": [ctypes.POINTER(Grid), _i, _i, _vp, _vp, _sz, _vp],
    "mgx_mgkernel_extend3d": [ctypes.POINTER(Grid), _i, _i, _vp, _vp, _sz, _vp],
    "mgx_trade_boundaries": [ctypes.POINTER(Grid), _i, _i, _vp, _sz, _vp],
    "mgx_axpy": [_sz, _d, _i, _vp, _vp, _vp],
    "mgx_kernel_arch": [ctypes.POINTER(_i)],
    "mgx_regions_move_to": [_i, _dp, _dp, _dp, ctypes.POINTER(ctypes.c_float)],
    "mgx_regions_update_radii": [_i, _dp, ctypes.c_float, ctypes.POINTER(ctypes.c_float),
                                 ctypes.POINTER(ctypes.c_float)],
    "mgx_sincos_diag": [_vp, _i, _vp, _sz, _i, _i, _vp, _vp],
    "mgx_pack_functions": [ctypes.POINTER(Grid), _i, _i, _dp, ctypes.POINTER(ctypes.c_float), _i,
                           _i, ctypes.POINTER(_i), ctypes.POINTER(_i)],
    "mgx_fd_apply": [_vp, _i, _i, _vp, _sz, _vp, _i, _vp],
    "mgx_rhs_mehr": [_vp, _i, _vp, _sz, _vp, _i, _vp],
    "mgx_hpsi": [_vp, _i, _i, _vp, _sz, _vp, _i, _vp, _i, _i, _vp],
    "mgx_mg_restrict": [_vp, _i, _i, _vp, _vp, _i, _vp],
    "mgx_mg_prolong": [_vp, _i, _i, _vp, _vp, _i, _vp],
    "mgx_precond_mg": [_vp, ctypes.POINTER(PrecondParams), _i, _vp, _sz, _vp, _i, _vp, _vp],
    "mgx_precond_mg_update": [_vp, ctypes.POINTER(PrecondParams), _i, _vp, _sz, _vp, _d, _vp, _i,
                              _vp, _vp, _vp],
    "mgx_precond_mg_static": [_vp, ctypes.POINTER(PrecondParams), _i, _vp, _sz, _vp, _i, _vp, _vp],
    "mgx_precond_gamma": [ctypes.POINTER(Grid), _i, _i, _d, _d, _dp],
    "mgx_masks_create": [_vp, _i, _i, _dp, _dp, _i, _i, _i, _i, ctypes.POINTER(_vp), _vp],
    "mgx_masks_destroy": [_vp],
    "mgx_masks_update": [_vp, _vp, _dp, _dp, _vp],
    "mgx_masks_apply": [_vp, _vp, _i, _vp, _sz, _i, _vp],
    "mgx_masks_expand": [_vp, _i, _vp, _ip, _vp],
    "mgx_gram": [_vp, _i, _vp, _sz, _i, _vp, _vp],
    "mgx_hmat": [_vp, _i, _vp, _vp, _sz, _i, _vp, _vp],
    "mgx_gram_hmat": [_vp, _i, _vp, _vp, _sz, _i, _vp, _vp, _vp],
    "mgx_matb": [_vp, _i, _vp, _sz, _i, _vp, _vp, _i, _vp],
    "mgx_gram_hmat_matb": [_vp, _i, _vp, _vp, _sz, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "mgx_hpsi_gram_hmat_matb": [_vp, _i, _vp, _vp, _vp, _sz, _i, _vp, _vp, _vp, _vp, _i, _vp],
    "mgx_update_hb": [_vp, _i, _vp, _vp, _vp, _vp],
    "mgx_normalize": [_vp, _i, _vp, _sz, _i, _vp, _vp],
    "mgx_normalize_scales": [_vp, _i, _vp, _vp, _vp],
    "mgx_cholesky": [_vp, _i, _vp, _ip, _vp],
    "mgx_cholesky_async": [_vp, _i, _vp, _vp, _vp],
    "mgx_set_reuse_conversion": [_vp, _i],
    "mgx_timing_enable": [_i],
    "mgx_timing_read": [_i, _dp, _ip],
    "mgx_inverse_from_cholesky": [_vp, _i, _vp, _vp, _vp],
    "mgx_trace_prod": [_vp, _i, _vp, _vp, _vp, _vp],
    "mgx_theta": [_vp, _i, _vp, _vp, _vp, _vp],
    "mgx_copy": [_vp, _vp, _sz, _vp],
    "mgx_theta_from_cholesky": [_vp, _i, _vp, _vp, _vp, _vp, _vp],
    "mgx_mult_matrix": [_vp, _i, _i, _vp, _sz, _i, _vp, _vp, _vp],
    "mgx_residual": [_vp, _i, _i, _vp, _vp, _sz, _i, _vp, _i, _vp, _vp, _vp],
    "mgx_residual_cols": [_vp, _i, _i, _vp, _vp, _sz, _i, _vp, _i, _i, _vp, _vp, _vp],
    "mgx_mgm": [_vp, ctypes.POINTER(MgmParams), _i, _vp, _vp, ctypes.POINTER(MgmResult), _vp],
    "mgx_rho": [_vp, _i, _i, _vp, _sz, _i, _vp, _d, _vp, _dp, _vp, _i, _vp],
    "mgx_anderson_create": [_vp, _i, _d, _i, _sz, _i, ctypes.POINTER(_vp)],
    "mgx_anderson_destroy": [_vp],
    "mgx_anderson_restart": [_vp],
    "mgx_anderson_update": [_vp, _vp, _vp, _d, _vp, _vp, ctypes.POINTER(AndersonInfo), _vp],
    "mgx_precond_mg_warm": [_vp, ctypes.POINTER(PrecondParams), _i, _vp, _sz, _vp, _i, _vp, _vp],
    "mgx_unet_create": [_vp, ctypes.POINTER(_vp)],
    "mgx_unet_destroy": [_vp],
    "mgx_unet_set_params": [_vp, _vp, _vp],
    "mgx_unet_get_params": [_vp, _vp, _vp],
    "mgx_unet_forward": [_vp, _vp, _sz, _vp, _i, _vp],
    "mgx_unet_loss_grad": [_vp, _vp, _vp, _sz, _i, _vp, _vp, _vp],
    "mgx_unet_adam": [_vp, _vp, ctypes.POINTER(AdamParams), _vp],
    "mgx_unet_train_step": [_vp, _vp, _vp, _sz, _i, ctypes.POINTER(AdamParams), _vp, _vp],
    "mgx_local_create": [_vp, _vp, _vp, ctypes.POINTER(_vp)],
    "mgx_local_destroy": [_vp],
    "mgx_local_layout": [_vp, ctypes.POINTER(_sz), ctypes.POINTER(_sz), _ip],
    "mgx_local_gather": [_vp, _vp, _sz, _vp, _vp],
    "mgx_local_scatter": [_vp, _vp, _vp, _sz, _vp],
    "mgx_local_step": [_vp, _vp, _vp, _vp, _d, _vp, _vp, _vp],
    "mgx_local_tune": [_vp, _vp, _vp, _vp, _d, _vp, _vp, _dp, _ip, _vp],
    "mgx_local_set_config": [_vp, _i, _i, _i],
    "mgx_local_get_config": [_vp, _ip, _ip, _ip],
    "mgx_precond_learned": [_vp, _vp, ctypes.POINTER(PrecondParams), _vp, _sz, _vp, _i, _i, _dp,
                            _dp, _ip, _vp],
    "mgx_snapshot_write": [ctypes.c_char_p, ctypes.POINTER(Grid), ctypes.c_char_p, _i,
                           ctypes.POINTER(Dataset), _vp],
    "mgx_snapshot_header": [ctypes.c_char_p, ctypes.c_char_p, _sz, ctypes.POINTER(_sz)],
    "mgx_snapshot_read": [ctypes.c_char_p, ctypes.c_char_p, _vp, _sz, _vp],
}

# every entry point declared in include/mgx.h
EXPORTS = sorted(list(_SIGS) + ["mgx_last_error_string", "mgx_kernel_launch_count"])


def load(path=LIB_PATH):
    """Loads libmgx.so (building it first when nvcc is available)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(path):
        from . import build as _b
        _b.build()
    if not os.path.exists(path):
        raise ImportError(f"mgx library not found at {path}")
    L = ctypes.CDLL(path)
    for name, args in _SIGS.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.mgx_last_error_string.restype = ctypes.c_char_p
    L.mgx_last_error_string.argtypes = []
    L.mgx_kernel_launch_count.restype = ctypes.c_ulonglong
    L.mgx_kernel_launch_count.argtypes = []
    _LIB = L
    return L


def _check(status):
    if status != MGX_OK:
        raise MgxError(status, load().mgx_last_error_string().decode())


def launches():
    return int(load().mgx_kernel_launch_count())


def regions_move_to(centers, targets, cell):
    """LocalizationRegions::moveTo (mgx_regions_move_to): new centres
    (nfunc x 3) and the largest move before the 1-bohr cap."""
    import numpy as np
    c = np.array(centers, dtype=np.float64, order="C").reshape(-1, 3)
    t = np.ascontiguousarray(targets, dtype=np.float64).reshape(-1, 3)
    if t.shape != c.shape:
        raise ValueError("one target per centre")
    cl = np.ascontiguousarray(cell, dtype=np.float64)
    mx = ctypes.c_float()
    _check(load().mgx_regions_move_to(c.shape[0], c.ctypes.data_as(_dp), t.ctypes.data_as(_dp),
                                      cl.ctypes.data_as(_dp), ctypes.byref(mx)))
    return c, mx.value


def regions_update_radii(spreads, ratio):
    """LocalizationRegions::updateRadii (mgx_regions_update_radii): FP32
    radii ratio x spread and their mean radius."""
    import numpy as np
    sp = np.ascontiguousarray(spreads, dtype=np.float64).reshape(-1)
    r = np.zeros(sp.size, dtype=np.float32)
    mean = ctypes.c_float()
    _check(load().mgx_regions_update_radii(sp.size, sp.ctypes.data_as(_dp), ctypes.c_float(ratio),
                                           r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                           ctypes.byref(mean)))
    return r, mean.value


def pack_functions(n, ll, centers, radii, subdivx, rlf=False, ghosts=1):
    """FunctionsPacking of one task (mgx_pack_functions): the colour of each
    orbital and the number of colours.  centers (nfunc x 3, bohr) and radii
    (nfunc, stored as FP32 like the reference's localization regions)."""
    import numpy as np
    c = np.ascontiguousarray(centers, dtype=np.float64).reshape(-1, 3)
    r = np.ascontiguousarray(radii, dtype=np.float32).reshape(-1)
    if c.shape[0] != r.shape[0]:
        raise ValueError("one radius per centre")
    nf = r.shape[0]
    colors = np.zeros(max(nf, 1), dtype=np.int32)
    nc = _i()
    g = Grid.make(n, ll)
    _check(load().mgx_pack_functions(ctypes.byref(g), int(ghosts), nf, c.ctypes.data_as(_dp),
                                     r.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                     int(subdivx), 1 if rlf else 0,
                                     colors.ctypes.data_as(ctypes.POINTER(_i)),
                                     ctypes.byref(nc)))
    return colors[:nf].copy(), nc.value


def kernel_arch():
    """major * 10 + minor of the architecture the library's kernels were
    compiled for, as the CUDA runtime reports it for the loaded module."""
    v = _i()
    _check(load().mgx_kernel_arch(ctypes.byref(v)))
    return v.value


TIMING_TC_SPLITK, TIMING_TC_STORE = 1, 2


def timing_enable(on):
    """Brackets every tensor-core product launch with CUDA events."""
    _check(load().mgx_timing_enable(1 if on else 0))


def timing_read(cls):
    """(total device ms, launches) of one timing class since its last read."""
    ms = ctypes.c_double()
    n = ctypes.c_int()
    _check(load().mgx_timing_read(int(cls), ctypes.byref(ms), ctypes.byref(n)))
    return ms.value, n.value


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _dtype(t):
    if t.dtype == torch.float64:
        return F64
    if t.dtype == torch.float32:
        return F32
    raise TypeError(f"unsupported dtype {t.dtype}")


def _block(t, npts):
    """(pointer, ld, nfunc) of an orbital block tensor."""
    if not t.is_cuda:
        raise ValueError("orbital block must be a CUDA tensor")
    if t.dim() == 1:
        if t.numel() != npts or t.stride(0) != 1:
            raise ValueError("bad single-function block")
        return ctypes.c_void_p(t.data_ptr()), npts, 1
    if t.dim() != 2 or t.shape[1] != npts or t.stride(1) != 1:
        raise ValueError(f"block must be (nfunc, {npts}) with unit point stride")
    return ctypes.c_void_p(t.data_ptr()), t.stride(0), t.shape[0]


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def axpy(alpha, x, y, stream=None):
    """y += alpha x over whole blocks of the same dtype (mgx_axpy)."""
    if x.dtype != y.dtype or x.numel() != y.numel() or not (x.is_contiguous() and y.is_contiguous()):
        raise ValueError("axpy wants contiguous blocks of one dtype and size")
    _check(load().mgx_axpy(x.numel(), float(alpha), _dtype(x), _ptr(x), _ptr(y), _stream(stream)))
    return y


def copy(dst, src, stream=None):
    """dst <- src (same byte size; either may be a pinned host tensor) with
    the library's SM-driven copy (mgx_copy)."""
    nb = src.numel() * src.element_size()
    if dst.numel() * dst.element_size() != nb or not (dst.is_contiguous() and src.is_contiguous()):
        raise ValueError("copy wants contiguous tensors of one byte size")
    _check(load().mgx_copy(_ptr(dst), _ptr(src), nb, _stream(stream)))
    return dst


class Context:
    """An mgx context: grid geometry plus device workspaces."""

    def __init__(self, n, ll):
        self.n = tuple(int(x) for x in n)
        self.ll = tuple(float(x) for x in ll)
        self.grid = Grid.make(self.n, self.ll)
        self.npts = self.n[0] * self.n[1] * self.n[2]
        h = ctypes.c_void_p()
        _check(load().mgx_create(ctypes.byref(self.grid), ctypes.byref(h)))
        self.handle = h

    def set_reuse_conversion(self, on):
        """mgx_set_reuse_conversion: Psi Theta products may read the last
        Gram-type product's BF16 conversion of the same (unchanged) block."""
        _check(load().mgx_set_reuse_conversion(self.handle, 1 if on else 0))

    def close(self):
        if getattr(self, "handle", None):
            load().mgx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def h(self):
        return tuple(self.ll[i] / self.n[i] for i in range(3))

    @property
    def vel(self):
        h = self.h
        return h[0] * h[1] * h[2]

    def level_points(self, level):
        return (self.n[0] >> level) * (self.n[1] >> level) * (self.n[2] >> level)

    # ------------------------------------------------------------ stencils
    def fd_apply(self, u, lap_type, out=None, stream=None):
        p, ld, nf = _block(u, self.npts)
        out = torch.empty_like(u) if out is None else out
        po, ldo, _ = _block(out, self.npts)
        assert ldo == ld
        _check(load().mgx_fd_apply(self.handle, lap_type, _dtype(u), p, ld, po, nf, _stream(stream)))
        return out

    def rhs_mehr(self, u, out=None, stream=None):
        p, ld, nf = _block(u, self.npts)
        out = torch.empty_like(u) if out is None else out
        _check(load().mgx_rhs_mehr(self.handle, _dtype(u), p, ld, _ptr(out), nf, _stream(stream)))
        return out

    def hpsi(self, psi, V, lap_type=LAP_MEHR4, apply_B=True, out=None, stream=None):
        p, ld, nf = _block(psi, self.npts)
        out = torch.empty_like(psi) if out is None else out
        if V.numel() != self.npts or not V.is_contiguous():
            raise ValueError("V must be contiguous with one value per grid point")
        _check(load().mgx_hpsi(self.handle, lap_type, _dtype(psi), p, ld, _ptr(V), _dtype(V),
                               _ptr(out), nf, 1 if apply_B else 0, _stream(stream)))
        return out

    def restrict(self, fine, level=0, stream=None):
        nf = 1 if fine.dim() == 1 else fine.shape[0]
        out = torch.empty((nf, self.level_points(level + 1)), dtype=fine.dtype, device=fine.device)
        _check(load().mgx_mg_restrict(self.handle, level, _dtype(fine), _ptr(fine), _ptr(out), nf,
                                      _stream(stream)))
        return out

    def prolong(self, coarse, level=0, stream=None):
        nf = 1 if coarse.dim() == 1 else coarse.shape[0]
        out = torch.empty((nf, self.level_points(level)), dtype=coarse.dtype, device=coarse.device)
        _check(load().mgx_mg_prolong(self.handle, level, _dtype(coarse), _ptr(coarse), _ptr(out), nf,
                                     _stream(stream)))
        return out

    # ------------------------------------------------------------ preconditioner
    def precond_mg(self, res, lap_type, maxlevels, gamma, masks=None, chunk=0, out=None,
                   stream=None):
        p, ld, nf = _block(res, self.npts)
        out = torch.empty_like(res) if out is None else out
        prm = PrecondParams(lap_type, maxlevels, float(gamma), int(chunk))
        _check(load().mgx_precond_mg(self.handle, ctypes.byref(prm), _dtype(res), p, ld, _ptr(out), nf,
                                     masks.handle if masks is not None else None, _stream(stream)))
        return out

    def precond_mg_warm(self, res, out, lap_type, maxlevels, masks=None, chunk=0, stream=None):
        """out <- V-cycle(res) started from the iterate out holds."""
        p, ld, nf = _block(res, self.npts)
        po, ldo, _ = _block(out, self.npts)
        assert ldo == ld
        prm = PrecondParams(lap_type, maxlevels, 0.0, int(chunk))
        _check(load().mgx_precond_mg_warm(self.handle, ctypes.byref(prm), _dtype(res), p, ld, po, nf,
                                          masks.handle if masks is not None else None,
                                          _stream(stream)))
        return out

    def precond_update(self, res, psi, alpha, lap_type, maxlevels, gamma, masks=None, chunk=0,
                       work=None, psi_scale=None, stream=None):
        """psi += alpha * V-cycle(res) (the update fused into the last sweep);
        with psi_scale (FP64 device vector, one value per function) psi_j =
        psi_scale[j] * (psi_j + alpha * V-cycle(res)_j); work: optional
        scratch block of res's shape."""
        p, ld, nf = _block(res, self.npts)
        pp, ldp, _ = _block(psi, self.npts)
        assert ldp == ld
        if psi_scale is not None and (psi_scale.dtype != torch.float64 or psi_scale.numel() < nf
                                      or not psi_scale.is_contiguous()):
            raise ValueError("psi_scale must be a contiguous FP64 vector of nfunc values")
        prm = PrecondParams(lap_type, maxlevels, float(gamma), int(chunk))
        _check(load().mgx_precond_mg_update(self.handle, ctypes.byref(prm), _dtype(res), p, ld, pp,
                                            float(alpha), _ptr(psi_scale), nf,
                                            masks.handle if masks is not None else None,
                                            _ptr(work), _stream(stream)))
        return psi

    def gamma(self, lap_type, mg_levels, vmax, small_eig):
        g = ctypes.c_double()
        _check(load().mgx_precond_gamma(ctypes.byref(self.grid), lap_type, mg_levels, vmax, small_eig,
                                        ctypes.byref(g)))
        return g.value

    # ------------------------------------------------------------ Gram / H
    def gram(self, psi, mode=GEMM_FP64, out=None, stream=None):
        p, ld, nf = _block(psi, self.npts)
        S = torch.empty((nf, nf), dtype=torch.float64, device=psi.device) if out is None else out
        _check(load().mgx_gram(self.handle, mode, p, ld, nf, _ptr(S), _stream(stream)))
        return S

    def hmat(self, psi, hpsi, mode=GEMM_FP64, out=None, stream=None):
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, _ = _block(hpsi, self.npts)
        assert ldh == ld
        H = torch.empty((nf, nf), dtype=torch.float64, device=psi.device) if out is None else out
        _check(load().mgx_hmat(self.handle, mode, p, ph, ld, nf, _ptr(H), _stream(stream)))
        # column-major H(i,j) = <psi_i, hpsi_j>; return the row-major view
        return H.T

    def gram_hmat(self, psi, hpsi, mode=GEMM_FP64, S=None, H=None, stream=None):
        """(S, H) with H returned as the row-major view (H[i, j] = <psi_i, hpsi_j>)."""
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, _ = _block(hpsi, self.npts)
        assert ldh == ld
        S = torch.empty((nf, nf), dtype=torch.float64, device=psi.device) if S is None else S
        H = torch.empty((nf, nf), dtype=torch.float64, device=psi.device) if H is None else H
        _check(load().mgx_gram_hmat(self.handle, mode, p, ph, ld, nf, _ptr(S), _ptr(H), _stream(stream)))
        return S, H.T

    def _work(self, work, ld, dtype):
        """(pointer, functions) of a B Psi work block (None: owned by ctx)."""
        if work is None:
            return None, 0
        pw, ldw, nw = _block(work, self.npts)
        if ldw != ld and nw > 1:
            raise ValueError("work must have the leading dimension of psi")
        if work.dtype != dtype:
            raise ValueError("work must have the orbital type")
        return pw, nw

    def matb(self, psi, mode=GEMM_FP64, work=None, out=None, stream=None):
        """B = Psi^T (B Psi) * vel (computeMatB), symmetric FP64 (nfunc, nfunc);
        work: optional (k, npts) block for B Psi, k >= 1 functions."""
        p, ld, nf = _block(psi, self.npts)
        B = torch.empty((nf, nf), dtype=torch.float64, device=psi.device) if out is None else out
        pw, nw = self._work(work, ld, psi.dtype)
        _check(load().mgx_matb(self.handle, mode, p, ld, nf, _ptr(B), pw, nw, _stream(stream)))
        return B

    def gram_hmat_matb(self, psi, hpsi, mode=GEMM_FP64, S=None, H=None, B=None, work=None,
                       stream=None):
        """(S, H, B) in one call, H as the row-major view."""
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, _ = _block(hpsi, self.npts)
        assert ldh == ld
        mk = lambda: torch.empty((nf, nf), dtype=torch.float64, device=psi.device)  # noqa: E731
        S = mk() if S is None else S
        H = mk() if H is None else H
        B = mk() if B is None else B
        pw, nw = self._work(work, ld, psi.dtype)
        _check(load().mgx_gram_hmat_matb(self.handle, mode, p, ph, ld, nf, _ptr(S), _ptr(H), _ptr(B),
                                         pw, nw, _stream(stream)))
        return S, H.T, B

    def hpsi_gram_hmat_matb(self, psi, V, hpsi, mode=GEMM_BF16X3, S=None, H=None, B=None,
                            work=None, stream=None):
        """H psi into hpsi (Mehrstellen with B(V psi), FP32) and (S, H, B) in
        one call (mgx_hpsi_gram_hmat_matb); H as the row-major view."""
        if psi.dtype != torch.float32 or V.dtype != torch.float32 or hpsi.dtype != torch.float32:
            raise ValueError("FP32 block, potential and H psi")
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, _ = _block(hpsi, self.npts)
        assert ldh == ld
        if V.numel() != self.npts or not V.is_contiguous():
            raise ValueError("V must be one contiguous field of the grid")
        mk = lambda: torch.empty((nf, nf), dtype=torch.float64, device=psi.device)  # noqa: E731
        S = mk() if S is None else S
        H = mk() if H is None else H
        B = mk() if B is None else B
        pw, nw = self._work(work, ld, psi.dtype)
        _check(load().mgx_hpsi_gram_hmat_matb(self.handle, mode, p, _ptr(V), ph, ld, nf, _ptr(S),
                                              _ptr(H), _ptr(B), pw, nw, _stream(stream)))
        return S, H.T, B

    def update_hb(self, S, theta, stream=None):
        """HB = sym(S theta) (ProjectedMatricesMehrstellen::updateHB); row-major
        tensors in and out, S read from its lower triangle."""
        n = S.shape[0]
        Sc = self._colmajor(S)
        tc = self._colmajor(theta)
        out = torch.empty((n, n), dtype=torch.float64, device=S.device)
        _check(load().mgx_update_hb(self.handle, n, _ptr(Sc), _ptr(tc), _ptr(out), _stream(stream)))
        return out.T

    def normalize(self, psi, diag=None, stream=None):
        """LocGridOrbitals::normalize in place; returns diagS (FP64 device)."""
        p, ld, nf = _block(psi, self.npts)
        d = torch.empty(nf, dtype=torch.float64, device=psi.device) if diag is None else diag
        _check(load().mgx_normalize(self.handle, _dtype(psi), p, ld, nf, _ptr(d), _stream(stream)))
        return d

    def normalize_scales(self, S, out=None, stream=None):
        """1 / sqrt(diag(S)) as an FP64 device vector."""
        n = S.shape[0]
        if S.stride() != (n, 1) and S.stride() != (1, n):
            raise ValueError("S must be a dense (n, n) tensor")
        d = torch.empty(n, dtype=torch.float64, device=S.device) if out is None else out
        _check(load().mgx_normalize_scales(self.handle, n, _ptr(S), _ptr(d), _stream(stream)))
        return d

    def cholesky(self, S, stream=None, info=None):
        """Lower factor L (returned as a row-major tensor) of symmetric S.
        With info (a device int32 tensor) nothing waits for the
        factorization: info receives 0 or the pivot index on the stream."""
        n = S.shape[0]
        A = S.T.contiguous().clone()
        if info is not None:
            if info.dtype != torch.int32 or not info.is_cuda:
                raise ValueError("info must be a device int32 tensor")
            _check(load().mgx_cholesky_async(self.handle, n, _ptr(A), _ptr(info), _stream(stream)))
            return A.T
        info = ctypes.c_int(0)
        st = load().mgx_cholesky(self.handle, n, _ptr(A), ctypes.byref(info), _stream(stream))
        if st != MGX_OK:
            raise MgxError(st, load().mgx_last_error_string().decode() + f" (info={info.value})")
        return A.T

    def inverse_from_cholesky(self, L, stream=None):
        n = L.shape[0]
        Lc = L.T.contiguous()
        out = torch.empty((n, n), dtype=torch.float64, device=L.device)
        _check(load().mgx_inverse_from_cholesky(self.handle, n, _ptr(Lc), _ptr(out), _stream(stream)))
        return out.T

    def trace_prod(self, H, Sinv, stream=None):
        n = H.shape[0]
        Hc = H.T.contiguous()
        Sc = Sinv.T.contiguous()
        out = torch.empty(1, dtype=torch.float64, device=H.device)
        _check(load().mgx_trace_prod(self.handle, n, _ptr(Hc), _ptr(Sc), _ptr(out), _stream(stream)))
        return out

    def residual_cols(self, psi, hpsi, theta_cols, mode=GEMM_FP64, apply_B=True, work=None,
                      out=None, stream=None):
        """Residual of ncols output functions: theta_cols is the column-major
        (ncols, nfunc) slice theta[:, j0:j0+ncols].T (contiguous), hpsi and out
        (ncols, npts) views of the chunk; out may be hpsi."""
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, nc = _block(hpsi, self.npts)
        if theta_cols.shape != (nc, nf) or not theta_cols.is_contiguous():
            raise ValueError("theta_cols must be a contiguous (ncols, nfunc) tensor")
        out = torch.empty_like(hpsi) if out is None else out
        _check(load().mgx_residual_cols(self.handle, mode, _dtype(psi), p, ph, ld, nf,
                                        _ptr(theta_cols), nc, 1 if apply_B else 0, _ptr(work),
                                        _ptr(out), _stream(stream)))
        return out

    # ------------------------------------------------------------ density
    def rho(self, psi, X, mode=GEMM_FP64, nel=0.0, out=None, work=None, stream=None):
        """Rho<T>::computeRho: (rho, charge) with rho(p) = sum_j (Psi X)_j(p)
        psi_j(p) (X a row-major FP64 tensor), rescaled to nel electrons when
        nel > 0."""
        p, ld, nf = _block(psi, self.npts)
        rho = torch.empty(self.npts, dtype=torch.float64, device=psi.device) if out is None else out
        Xc = self._colmajor(X)
        q = ctypes.c_double()
        pw, nw = (None, 0) if work is None else _block(work, self.npts)[0::2]
        _check(load().mgx_rho(self.handle, mode, _dtype(psi), p, ld, nf, _ptr(Xc), float(nel),
                              _ptr(rho), ctypes.byref(q), pw, nw, _stream(stream)))
        return rho, q.value

    # ------------------------------------------------------------ centres
    def sincos_diag(self, psi, normalized=False, out=None, stream=None):
        """The diagonal position-matrix elements of the block (mgx_sincos_diag):
        an (nfunc, 6) FP64 device tensor, columns cos x, sin x, cos y, sin y,
        cos z, sin z (scaled by L / (2 pi))."""
        p, ld, nf = _block(psi, self.npts)
        import torch
        out = torch.empty((nf, 6), dtype=torch.float64, device=psi.device) if out is None else out
        _check(load().mgx_sincos_diag(self.handle, _dtype(psi), p, ld, nf, 1 if normalized else 0,
                                      _ptr(out), _stream(stream)))
        return out

    def centers_spreads(self, psi, normalized=False, stream=None):
        """Centres (nfunc x 3, in [0, L)) and spreads (nfunc) of the orbitals,
        SpreadsAndCenters::computeCenter / computeSpread from sincos_diag."""
        import numpy as np
        a = self.sincos_diag(psi, normalized, stream=stream).cpu().numpy()
        ll = np.asarray(self.ll)
        lby2pi = ll * (0.5 / np.pi)
        c, s = a[:, 0::2], a[:, 1::2]
        x = lby2pi[None, :] * np.arctan2(s, c)
        x = np.where(x < 0., x + ll[None, :], x)
        spread2 = (lby2pi[None, :] ** 2 - c * c - s * s).sum(axis=1)
        return x, np.sqrt(spread2)

    # ------------------------------------------------------------ Poisson
    def mgm(self, vh, rho, lap_type=LAP_MEHR4, max_levels=10, max_sweeps=10, tol=1e-16, nu1=2,
            nu2=2, ghosts=0, stream=None):
        """pb::Mgm on one field: vh (device, npts values) is solved in place;
        returns the result fields as a dict."""
        if vh.numel() != self.npts or rho.numel() != self.npts:
            raise ValueError("vh and rho need one value per grid point")
        if not (vh.is_contiguous() and rho.is_contiguous()) or vh.dtype != rho.dtype:
            raise ValueError("vh and rho must be contiguous and of one dtype")
        prm = MgmParams(lap_type, max_levels, max_sweeps, float(tol), nu1, nu2, ghosts)
        res = MgmResult()
        _check(load().mgx_mgm(self.handle, ctypes.byref(prm), _dtype(vh), _ptr(vh), _ptr(rho),
                              ctypes.byref(res), _stream(stream)))
        return {k: getattr(res, k) for k, _ in MgmResult._fields_}

    # ------------------------------------------------------------ residual
    def theta(self, Sinv, H, stream=None):
        """theta = Sinv H (row-major tensors in and out; Sinv read from its
        lower triangle)."""
        n = H.shape[0]
        Sc = Sinv.T.contiguous()
        Hc = H.T.contiguous()
        out = torch.empty((n, n), dtype=torch.float64, device=H.device)
        _check(load().mgx_theta(self.handle, n, _ptr(Sc), _ptr(Hc), _ptr(out), _stream(stream)))
        return out.T

    def theta_from_cholesky(self, L, H, stream=None):
        """(theta, trace): theta = S^-1 H from the row-major lower factor L of
        S (as returned by cholesky) by substitution; trace = tr(theta)."""
        n = H.shape[0]
        Lc = L.T.contiguous()
        Hc = H.T.contiguous()
        out = torch.empty((n, n), dtype=torch.float64, device=H.device)
        tr = torch.empty(1, dtype=torch.float64, device=H.device)
        _check(load().mgx_theta_from_cholesky(self.handle, n, _ptr(Lc), _ptr(Hc), _ptr(out),
                                              _ptr(tr), _stream(stream)))
        return out.T, tr

    @staticmethod
    def _colmajor(theta):
        t = theta.T
        return t if t.is_contiguous() else t.contiguous()

    def mult_matrix(self, psi, theta, mode=GEMM_FP64, out=None, stream=None):
        """out_j = sum_i psi_i theta[i, j] (theta a row-major FP64 tensor)."""
        p, ld, nf = _block(psi, self.npts)
        out = torch.empty_like(psi) if out is None else out
        po, ldo, _ = _block(out, self.npts)
        assert ldo == ld
        tc = self._colmajor(theta)
        _check(load().mgx_mult_matrix(self.handle, mode, _dtype(psi), p, ld, nf, _ptr(tc), po,
                                      _stream(stream)))
        return out

    def residual(self, psi, hpsi, theta, mode=GEMM_FP64, apply_B=True, work=None, out=None,
                 stream=None):
        """res = B(psi) theta - hpsi (apply_B) or psi theta - hpsi; out may be hpsi."""
        p, ld, nf = _block(psi, self.npts)
        ph, ldh, _ = _block(hpsi, self.npts)
        assert ldh == ld
        out = torch.empty_like(psi) if out is None else out
        tc = self._colmajor(theta)
        _check(load().mgx_residual(self.handle, mode, _dtype(psi), p, ph, ld, nf, _ptr(tc),
                                   1 if apply_B else 0, _ptr(work), _ptr(out), _stream(stream)))
        return out


class Anderson:
    """AndersonMix of an orbital block: m history pairs owned by the library
    (mgx_anderson_*)."""

    def __init__(self, ctx, m, beta, x):
        _, ld, nf = _block(x, ctx.npts)
        self.ctx = ctx
        self.nfunc = nf
        self.handle = ctypes.c_void_p()
        _check(load().mgx_anderson_create(ctx.handle, int(m), float(beta), _dtype(x), ld, nf,
                                          ctypes.byref(self.handle)))

    def update(self, x, f, fscale=1.0, invS=None, fbar=None, stream=None):
        """x moves by one Anderson step with the residual fscale * f; invS:
        the FP64 device S^-1 whose diagonal weights the dot products.
        Returns {"mm", "reductions", "theta"}."""
        px, ldx, nf = _block(x, self.ctx.npts)
        pf, ldf, _ = _block(f, self.ctx.npts)
        if nf != self.nfunc or ldf != ldx:
            raise ValueError("x and f must be blocks of the mixer's shape")
        if invS is not None and (invS.dtype != torch.float64 or not invS.is_contiguous()):
            raise ValueError("invS must be a contiguous FP64 (n, n) tensor")
        info = AndersonInfo()
        _check(load().mgx_anderson_update(self.handle, px, pf, float(fscale), _ptr(invS), _ptr(fbar),
                                          ctypes.byref(info), _stream(stream)))
        return {"mm": info.mm, "reductions": info.reductions,
                "theta": [info.theta[j] for j in range(max(info.mm, 0))]}

    def restart(self):
        _check(load().mgx_anderson_restart(self.handle))

    def close(self):
        if self.handle:
            load().mgx_anderson_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Masks:
    """Localization masks (GridMaskMax / GridMaskMult) of nfunc orbitals."""

    def __init__(self, ctx, nlevels, centers, radii, func=0, kind=0, mesh_ghosts=1,
                 dtype=torch.float64, stream=None):
        import numpy as np
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1))
        r = np.ascontiguousarray(np.asarray(radii, dtype=np.float64).reshape(-1))
        self.nfunc = r.shape[0]
        self.nlevels = nlevels
        self.ctx = ctx
        self.dtype = dtype
        h = ctypes.c_void_p()
        _check(load().mgx_masks_create(ctx.handle, nlevels, self.nfunc, c.ctypes.data_as(_dp),
                                       r.ctypes.data_as(_dp), func, kind, mesh_ghosts,
                                       F64 if dtype == torch.float64 else F32, ctypes.byref(h),
                                       _stream(stream)))
        self.handle = h

    def update(self, centers, radii, stream=None):
        """MasksSet::update: the masks rebuilt for moved centres / new radii."""
        import numpy as np
        c = np.ascontiguousarray(np.asarray(centers, dtype=np.float64).reshape(-1))
        r = np.ascontiguousarray(np.asarray(radii, dtype=np.float64).reshape(-1))
        if r.shape[0] != self.nfunc or c.shape[0] != 3 * self.nfunc:
            raise ValueError("update needs nfunc centres and radii")
        _check(load().mgx_masks_update(self.ctx.handle, self.handle, c.ctypes.data_as(_dp),
                                       r.ctypes.data_as(_dp), _stream(stream)))
        return self

    def apply(self, u, level, stream=None):
        p, ld, nf = _block(u, self.ctx.level_points(level))
        _check(load().mgx_masks_apply(self.ctx.handle, self.handle, level, p, ld, nf, _stream(stream)))
        return u

    def expand(self, level, stream=None):
        """(state int array, dense values tensor (nfunc, level points))."""
        import numpy as np
        dense = torch.empty((self.nfunc, self.ctx.level_points(level)), dtype=self.dtype, device="cuda")
        st = np.zeros(self.nfunc, dtype=np.int32)
        _check(load().mgx_masks_expand(self.handle, level, _ptr(dense), st.ctypes.data_as(_ip),
                                       _stream(stream)))
        return st, dense

    def close(self):
        if getattr(self, "handle", None):
            load().mgx_masks_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- drop-in (ghosted)
def fdkernel_del2(n, ll, ghosts, lap_type, v, b, nfunc, stream=None):
    g = Grid.make(n, ll)
    _check(load().mgx_fdkernel_del2(ctypes.byref(g), ghosts, lap_type, _dtype(v), _ptr(v), _ptr(b),
                                    nfunc, _stream(stream)))


def fdkernel_rhs_mehr1(n, ll, ghosts, v, rhs, rhs_ghosts, nfunc, stream=None):
    g = Grid.make(n, ll)
    _check(load().mgx_fdkernel_rhs_mehr1(ctypes.byref(g), ghosts, _dtype(v), _ptr(v), _ptr(rhs),
                                         rhs_ghosts, nfunc, _stream(stream)))


def trade_boundaries(n, ll, ghosts, u, nfunc, stream=None):
    g = Grid.make(n, ll)
    _check(load().mgx_trade_boundaries(ctypes.byref(g), ghosts, _dtype(u), _ptr(u), nfunc,
                                       _stream(stream)))


def mgkernel_restrict3d(n, ll, ghosts, fine, coarse, nfunc, stream=None):
    g = Grid.make(n, ll)
    _check(load().mgx_mgkernel_restrict3d(ctypes.byref(g), ghosts, _dtype(fine), _ptr(fine),
                                          _ptr(coarse), nfunc, _stream(stream)))


def mgkernel_extend3d(n, ll, ghosts, coarse, fine, nfunc, stream=None):
    g = Grid.make(n, ll)
    _check(load().mgx_mgkernel_extend3d(ctypes.byref(g), ghosts, _dtype(coarse), _ptr(coarse),
                                        _ptr(fine), nfunc, _stream(stream)))


class UNet:
    """The learned preconditioner's network on a context's grid
    (mgx_unet_*): FP32 master weights, BF16 in the convolutions."""

    def __init__(self, ctx):
        self.ctx = ctx
        self.handle = ctypes.c_void_p()
        _check(load().mgx_unet_create(ctx.handle, ctypes.byref(self.handle)))
        self._loss = torch.zeros(1, dtype=torch.float64, device="cuda")

    def __del__(self):
        if getattr(self, "handle", None) and _LIB is not None:
            _LIB.mgx_unet_destroy(self.handle)
            self.handle = None

    def set_params(self, p, stream=None):
        p = torch.as_tensor(p, dtype=torch.float32).cuda().contiguous()
        if p.numel() != UNET_PARAMS:
            raise ValueError(f"{UNET_PARAMS} parameters expected")
        _check(load().mgx_unet_set_params(self.handle, _ptr(p), _stream(stream)))
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()

    def get_params(self, stream=None):
        p = torch.empty(UNET_PARAMS, dtype=torch.float32, device="cuda")
        _check(load().mgx_unet_get_params(self.handle, _ptr(p), _stream(stream)))
        return p

    def forward(self, x, out=None, stream=None):
        px, ld, nf = _block(x, self.ctx.npts)
        out = torch.empty_like(x) if out is None else out
        po, ldo, _ = _block(out, self.ctx.npts)
        assert ldo == ld and x.dtype == torch.float32
        _check(load().mgx_unet_forward(self.handle, px, ld, po, nf, _stream(stream)))
        return out

    def loss_grad(self, x, target, grad=None, stream=None):
        """(loss tensor, grad tensor) of mean((net(x/s) - target/s)^2)."""
        px, ld, nf = _block(x, self.ctx.npts)
        pt, ldt, _ = _block(target, self.ctx.npts)
        assert ldt == ld
        grad = torch.empty(UNET_PARAMS, dtype=torch.float32, device="cuda") if grad is None else grad
        loss = torch.empty(1, dtype=torch.float64, device="cuda")
        _check(load().mgx_unet_loss_grad(self.handle, px, pt, ld, nf, _ptr(grad), _ptr(loss),
                                         _stream(stream)))
        return loss, grad

    def adam(self, grad, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        prm = AdamParams(lr, beta1, beta2, eps)
        _check(load().mgx_unet_adam(self.handle, _ptr(grad), ctypes.byref(prm), _stream(stream)))

    def train_step(self, x, target, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        """One loss / gradient / Adam step; returns the loss as a device tensor."""
        px, ld, nf = _block(x, self.ctx.npts)
        pt, ldt, _ = _block(target, self.ctx.npts)
        assert ldt == ld
        prm = AdamParams(lr, beta1, beta2, eps)
        loss = torch.empty(1, dtype=torch.float64, device="cuda")
        _check(load().mgx_unet_train_step(self.handle, px, pt, ld, nf, ctypes.byref(prm), _ptr(loss),
                                          _stream(stream)))
        return loss


def precond_learned(ctx, net, res, lap_type, maxlevels, gamma, tau, mode=LEARNED_WARM, chunk=0,
                    out=None, stream=None):
    """The learned correction of res with the V-cycle as per-function
    fallback (mgx_precond_learned).  tau: float64 numpy array (nfunc), the
    V-cycle's residual reduction per function, updated in place.  Returns
    (out, reduction per function, number of fallbacks)."""
    p, ld, nf = _block(res, ctx.npts)
    out = torch.empty_like(res) if out is None else out
    po, ldo, _ = _block(out, ctx.npts)
    assert ldo == ld and res.dtype == torch.float32
    if tau.dtype != np.float64 or tau.size < nf or not tau.flags["C_CONTIGUOUS"]:
        raise ValueError("tau must be a contiguous float64 array of nfunc values")
    red = np.zeros(nf)
    nfb = ctypes.c_int()
    prm = PrecondParams(lap_type, maxlevels, float(gamma), int(chunk))
    _check(load().mgx_precond_learned(ctx.handle, net.handle, ctypes.byref(prm), p, ld, po, nf,
                                      int(mode), tau.ctypes.data_as(_dp), red.ctypes.data_as(_dp),
                                      ctypes.byref(nfb), _stream(stream)))
    return out, red, nfb.value


class Local:
    """Localized orbitals on their mask boxes (mgx_local_*): packed box-local
    FP32 blocks and the fused fine-level step."""

    def __init__(self, ctx, masks, corr):
        self.ctx = ctx
        self._keep = (masks, corr)
        self.handle = ctypes.c_void_p()
        _check(load().mgx_local_create(ctx.handle, masks.handle, corr.handle,
                                       ctypes.byref(self.handle)))
        self.nfunc = masks.nfunc
        tot = ctypes.c_size_t()
        self.offsets = np.zeros(self.nfunc + 1, dtype=np.uint64)
        self.boxes = np.zeros(6 * self.nfunc, dtype=np.int32)
        _check(load().mgx_local_layout(self.handle, ctypes.byref(tot),
                                       self.offsets.ctypes.data_as(ctypes.POINTER(_sz)),
                                       self.boxes.ctypes.data_as(_ip)))
        self.total = tot.value
        self.boxes = self.boxes.reshape(self.nfunc, 6)

    def __del__(self):
        if getattr(self, "handle", None) and _LIB is not None:
            _LIB.mgx_local_destroy(self.handle)
            self.handle = None

    def empty(self):
        return torch.empty(max(self.total, 1), dtype=torch.float32, device="cuda")

    def gather(self, full, out=None, stream=None):
        p, ld, nf = _block(full, self.ctx.npts)
        assert nf == self.nfunc and full.dtype == torch.float32
        out = self.empty() if out is None else out
        _check(load().mgx_local_gather(self.handle, p, ld, _ptr(out), _stream(stream)))
        return out

    def scatter(self, packed, out=None, stream=None):
        out = (torch.zeros((self.nfunc, self.ctx.npts), dtype=torch.float32, device="cuda")
               if out is None else out)
        p, ld, nf = _block(out, self.ctx.npts)
        _check(load().mgx_local_scatter(self.handle, _ptr(packed), p, ld, _stream(stream)))
        return out

    def step(self, psi, phi, V, gamma, u=None, w=None, stream=None):
        u = self.empty() if u is None else u
        w = self.empty() if w is None else w
        _check(load().mgx_local_step(self.handle, _ptr(psi), _ptr(phi), _ptr(V), float(gamma),
                                     _ptr(u), _ptr(w), _stream(stream)))
        return u, w

    def tune(self, psi, phi, V, gamma, u, w, stream=None):
        """Times the candidates and keeps the fastest; returns (times in ms
        per candidate, (shape, ctas_per_sm, graph))."""
        ms = np.zeros(64)
        n = ctypes.c_int(64)
        _check(load().mgx_local_tune(self.handle, _ptr(psi), _ptr(phi), _ptr(V), float(gamma),
                                     _ptr(u), _ptr(w), ms.ctypes.data_as(_dp), ctypes.byref(n),
                                     _stream(stream)))
        return ms[:n.value].copy(), self.config()

    def config(self):
        a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        _check(load().mgx_local_get_config(self.handle, ctypes.byref(a), ctypes.byref(b),
                                           ctypes.byref(c)))
        return a.value, b.value, c.value

    def set_config(self, shape, ctas_per_sm, graph=True):
        _check(load().mgx_local_set_config(self.handle, int(shape), int(ctas_per_sm),
                                           1 if graph else 0))
