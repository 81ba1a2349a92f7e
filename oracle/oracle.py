"""ctypes front end of the oracle -- TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liborc.so`` (the CPU restatement in mgx_oracle.cpp) and, when
present, ``oracle/_ref/libmgref.so`` (the reference MGmol's own hot-path
translation units compiled against single-task shims by build_ref.sh).
Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it.

All arrays are numpy, orbital-major (nfunc, nx*ny*nz), points x-slowest /
z-fastest, which is the ghost-free BlockVector layout of src/BlockVector.h.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_ORC = None
_REF = None

_dp = ctypes.POINTER(ctypes.c_double)
_fp = ctypes.POINTER(ctypes.c_float)
_ip = ctypes.POINTER(ctypes.c_int)


def build():
    """Compile liborc.so (quick, plain make)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _ORC
    if _ORC is None:
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            build()
        _ORC = ctypes.CDLL(path)
        _ORC.orc_set_gamma.restype = ctypes.c_double
        _ORC.orc_jacobi_factor.restype = ctypes.c_double
        _ORC.orc_trace_prod.restype = ctypes.c_double
    return _ORC


def ref_lib():
    """The reference's own code (None when it was not built here)."""
    global _REF
    if _REF is None:
        path = os.path.join(HERE, "_ref", "libmgref.so")
        if not os.path.exists(path):
            return None
        _REF = ctypes.CDLL(path)
    return _REF


def _p(a):
    a = np.ascontiguousarray(a)
    if a.dtype == np.float64:
        return a.ctypes.data_as(_dp)
    if a.dtype == np.float32:
        return a.ctypes.data_as(_fp)
    if a.dtype == np.int32:
        return a.ctypes.data_as(_ip)
    raise TypeError(a.dtype)


def _grid(n, ll):
    return (ctypes.c_int * 3)(*n), (ctypes.c_double * 3)(*ll)


def _sfx(a):
    return "d" if a.dtype == np.float64 else "f"


def _call(L, name, *args):
    rc = getattr(L, name)(*args)
    if rc != 0:
        raise RuntimeError(f"{name} returned {rc}")


# The reference's batched FDkernelDel2_6th / FDkernelDel2_8th initialise the
# x offset once outside the function loop (src/pb/FDkernels.cc:298,341 and
# :391,442), so for nfunc > 1 every function after the first is addressed
# dim0 planes too far.  The reference is therefore called one function at a
# time for lap types 3 and 4; the oracle implements the per-function operator.
_PER_FUNCTION = (3, 4)


def fd_apply(n, ll, lap_type, u, ref=False):
    if ref and lap_type in _PER_FUNCTION and np.asarray(u).shape[0] > 1:
        return np.concatenate([fd_apply(n, ll, lap_type, u[i:i + 1], ref=True)
                               for i in range(u.shape[0])])
    L = ref_lib() if ref else lib()
    pre = "ref" if ref else "orc"
    u = np.ascontiguousarray(u)
    out = np.zeros_like(u)
    gn, gl = _grid(n, ll)
    _call(L, f"{pre}_fd_apply_{_sfx(u)}", gn, gl, lap_type, u.shape[0], _p(u), _p(out))
    return out


def rhs_mehr(n, ll, u, ref=False):
    L = ref_lib() if ref else lib()
    pre = "ref" if ref else "orc"
    u = np.ascontiguousarray(u)
    out = np.zeros_like(u)
    gn, gl = _grid(n, ll)
    _call(L, f"{pre}_rhs_mehr_{_sfx(u)}", gn, gl, u.shape[0], _p(u), _p(out))
    return out


def hpsi(n, ll, lap_type, psi, V, apply_B=1, ref=False):
    psi = np.ascontiguousarray(psi)
    V = np.ascontiguousarray(V, dtype=np.float64)
    out = np.zeros_like(psi)
    gn, gl = _grid(n, ll)
    if ref:
        assert lap_type == 0 and apply_B == 1
        _call(ref_lib(), f"ref_hpsi_mehr_{_sfx(psi)}", gn, gl, psi.shape[0], _p(psi), _p(V), _p(out))
    else:
        _call(lib(), f"orc_hpsi_{_sfx(psi)}", gn, gl, lap_type, apply_B, psi.shape[0], _p(psi), _p(V), _p(out))
    return out


def restrict(n, ll, u, ref=False):
    L = ref_lib() if ref else lib()
    pre = "ref" if ref else "orc"
    u = np.ascontiguousarray(u)
    out = np.zeros((u.shape[0], (n[0] // 2) * (n[1] // 2) * (n[2] // 2)), dtype=u.dtype)
    gn, gl = _grid(n, ll)
    _call(L, f"{pre}_restrict_{_sfx(u)}", gn, gl, u.shape[0], _p(u), _p(out))
    return out


def extend(n, ll, c, ref=False):
    """n is the FINE grid."""
    L = ref_lib() if ref else lib()
    pre = "ref" if ref else "orc"
    c = np.ascontiguousarray(c)
    out = np.zeros((c.shape[0], n[0] * n[1] * n[2]), dtype=c.dtype)
    gn, gl = _grid(n, ll)
    _call(L, f"{pre}_extend_{_sfx(c)}", gn, gl, c.shape[0], _p(c), _p(out))
    return out


def mask_build(n, ll, ng, nlevels, centers, radii, func=0, ref=False, dtype=np.float64):
    """Masks of every orbital at levels 0..nlevels-1 (func 0 gaussianDecay,
    1 one).  Returns (state[nlevels, nfunc], values list per level
    [nfunc, level_points])."""
    centers = np.ascontiguousarray(centers, dtype=np.float64)
    radii = np.ascontiguousarray(radii, dtype=np.float64)
    nf = radii.shape[0]
    sizes = [(n[0] >> l) * (n[1] >> l) * (n[2] >> l) for l in range(nlevels)]
    state = np.zeros(nlevels * nf, dtype=np.int32)
    gn, gl = _grid(n, ll)
    if ref:
        vals = np.zeros(sum(sizes) * nf, dtype=np.float64)
        _call(ref_lib(), "ref_mask_build", gn, gl, ng, nlevels, nf, _p(centers), _p(radii), func,
              _p(state), _p(vals))
        vals = vals.astype(dtype)
    else:
        vals = np.zeros(sum(sizes) * nf, dtype=dtype)
        _call(lib(), f"orc_mask_build_{_sfx(vals)}", gn, gl, ng, nlevels, nf, _p(centers), _p(radii),
              func, _p(state), _p(vals))
    out, off = [], 0
    for s in sizes:
        out.append(vals[off:off + nf * s].reshape(nf, s))
        off += nf * s
    return state.reshape(nlevels, nf), out


def mask_apply(n, level, state, values, u, kind=0):
    """Apply level masks (from mask_build) to ghost-free data u (copy)."""
    u = np.array(u, copy=True)
    nl = state.shape[0]
    flat = np.ascontiguousarray(np.concatenate([v.reshape(-1) for v in values]).astype(u.dtype))
    st = np.ascontiguousarray(state.reshape(-1), dtype=np.int32)
    gn = (ctypes.c_int * 3)(*n)
    _call(lib(), f"orc_mask_apply_{_sfx(u)}", gn, level, nl, u.shape[0], kind, _p(st), _p(flat), _p(u))
    return u


def precond(n, ll, lap_type, maxlevels, gamma, res, masks=None, kind=0, ref=False):
    """OrbitalsPreconditioning::precond_mg on a residual block.  masks: for the
    oracle, (state, values) from mask_build; for the reference, (centers,
    radii) (it builds its own GridMask objects)."""
    res = np.ascontiguousarray(res)
    out = np.zeros_like(res)
    gn, gl = _grid(n, ll)
    nf = res.shape[0]
    if ref and lap_type in _PER_FUNCTION and nf > 1:
        parts = []
        for i in range(nf):
            m = None if masks is None else (np.asarray(masks[0])[i:i + 1], np.asarray(masks[1])[i:i + 1])
            parts.append(precond(n, ll, lap_type, maxlevels, gamma, res[i:i + 1], m, kind, ref=True))
        return np.concatenate(parts)
    if ref:
        if masks is None:
            c = np.zeros(3)
            r = np.zeros(1)
            nm = 0
        else:
            c, r = (np.ascontiguousarray(m, dtype=np.float64) for m in masks)
            nm = nf
        _call(ref_lib(), f"ref_precond_{_sfx(res)}", gn, gl, lap_type, maxlevels, ctypes.c_double(gamma),
              nf, _p(res), _p(out), nm, _p(c), _p(r), kind)
        return out
    if masks is None:
        _call(lib(), f"orc_precond_{_sfx(res)}", gn, gl, lap_type, maxlevels, ctypes.c_double(gamma),
              nf, _p(res), _p(out), kind, None, None)
    else:
        state, values = masks
        flat = np.ascontiguousarray(np.concatenate([v.reshape(-1) for v in values]).astype(res.dtype))
        st = np.ascontiguousarray(state.reshape(-1), dtype=np.int32)
        _call(lib(), f"orc_precond_{_sfx(res)}", gn, gl, lap_type, maxlevels, ctypes.c_double(gamma),
              nf, _p(res), _p(out), kind, _p(st), _p(flat))
    return out


def set_gamma(inv_diag, mg_levels, vmax, small_eig):
    return lib().orc_set_gamma(ctypes.c_double(inv_diag), mg_levels, ctypes.c_double(vmax),
                               ctypes.c_double(small_eig))


def jacobi_factor(n, ll, lap_type):
    gn, gl = _grid(n, ll)
    return lib().orc_jacobi_factor(gn, gl, lap_type)


def gram(psi, vel, ref=False, usemp=False):
    """S = psi^T psi * vel with the 1e-14 filter (symmetric).  ref=True runs
    the reference's own LocalMatrices / LocalMatrices2DistMatrix code; for
    FP32 orbitals that is the USE_MP path, which keeps the product in a
    float local matrix (src/LocGridOrbitals.cc:1584-1602).  usemp=True
    restates that path for FP32 orbitals; the default keeps the FP64 sum
    (the stricter reference for the mixed-precision GPU path)."""
    psi = np.ascontiguousarray(psi)
    nf, npt = psi.shape
    S = np.zeros((nf, nf))
    if usemp and psi.dtype == np.float32 and not ref:
        _call(lib(), "orc_product_f_usemp", _p(psi), _p(psi), ctypes.c_long(npt), nf,
              ctypes.c_long(npt), ctypes.c_double(vel), _p(S))
        return S.T.copy()
    if ref:
        _call(ref_lib(), f"ref_gram_{_sfx(psi)}", npt, nf, _p(psi), npt, ctypes.c_double(vel), _p(S))
        return S.T.copy()
    _call(lib(), f"orc_gram_{_sfx(psi)}", _p(psi), ctypes.c_long(npt), nf, ctypes.c_long(npt),
          ctypes.c_double(vel), _p(S))
    return S


def hmat(psi, hpsi_, vel, ref=False, usemp=False):
    """H[i, j] = <psi_i, hpsi_j> * vel with the 1e-14 filter; ref and usemp
    as in gram."""
    psi = np.ascontiguousarray(psi)
    hpsi_ = np.ascontiguousarray(hpsi_, dtype=psi.dtype)
    nf, npt = psi.shape
    H = np.zeros((nf, nf))
    if usemp and psi.dtype == np.float32 and not ref:
        _call(lib(), "orc_product_f_usemp", _p(psi), _p(hpsi_), ctypes.c_long(npt), nf,
              ctypes.c_long(npt), ctypes.c_double(vel), _p(H))
    elif ref:
        _call(ref_lib(), f"ref_hmat_{_sfx(psi)}", npt, nf, _p(psi), _p(hpsi_), npt,
              ctypes.c_double(vel), _p(H))
    else:
        _call(lib(), f"orc_hmat_{_sfx(psi)}", _p(psi), _p(hpsi_), ctypes.c_long(npt), nf,
              ctypes.c_long(npt), ctypes.c_double(vel), _p(H))
    # H is column-major (j*n+i) = H(i,j); return H[i, j]
    return H.T.copy()


def potrf(S):
    """Lower Cholesky factor of S (column-major inside; numpy in/out)."""
    n = S.shape[0]
    A = np.ascontiguousarray(np.asarray(S, dtype=np.float64).T.copy())
    info = lib().orc_potrf(n, _p(A))
    return info, A.T.copy()


def inverse_from_chol(L):
    n = L.shape[0]
    Lc = np.ascontiguousarray(L.T)
    out = np.zeros((n, n))
    _call(lib(), "orc_inverse_from_chol", n, _p(Lc), _p(out))
    return out.T.copy()


def trace_prod(H, Sinv):
    n = H.shape[0]
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.float64).T)
    Sc = np.ascontiguousarray(np.asarray(Sinv, dtype=np.float64).T)
    return lib().orc_trace_prod(n, _p(Hc), _p(Sc))


def theta(Sinv, H):
    """theta = S^-1 H (row-major numpy in/out)."""
    n = Sinv.shape[0]
    Sc = np.ascontiguousarray(np.asarray(Sinv, dtype=np.float64).T)
    Hc = np.ascontiguousarray(np.asarray(H, dtype=np.float64).T)
    out = np.zeros((n, n))
    _call(lib(), "orc_theta", n, _p(Sc), _p(Hc), _p(out))
    return out.T.copy()


def mult_matrix(psi, th, ref=False):
    """out_j = sum_i psi_i theta[i, j] (theta row-major numpy)."""
    psi = np.ascontiguousarray(psi)
    nf, npt = psi.shape
    tc = np.ascontiguousarray(np.asarray(th, dtype=np.float64).T)
    out = np.zeros_like(psi)
    if ref:
        _call(ref_lib(), f"ref_mult_matrix_{_sfx(psi)}", npt, nf, _p(psi), _p(tc), _p(out))
        return out
    _call(lib(), f"orc_mult_matrix_{_sfx(psi)}", _p(psi), ctypes.c_long(npt), nf, ctypes.c_long(npt),
          _p(tc), _p(out))
    return out


def residual(n, ll, psi, hpsi_, th, apply_B=1, ref=False):
    """res = (B psi) theta - hpsi (computeResidualUsingHPhi)."""
    psi = np.ascontiguousarray(psi)
    hpsi_ = np.ascontiguousarray(hpsi_, dtype=psi.dtype)
    tc = np.ascontiguousarray(np.asarray(th, dtype=np.float64).T)
    out = np.zeros_like(psi)
    gn, gl = _grid(n, ll)
    if ref:
        assert apply_B
        _call(ref_lib(), f"ref_residual_{_sfx(psi)}", gn, gl, psi.shape[0], _p(psi), _p(hpsi_),
              _p(tc), _p(out))
        return out
    _call(lib(), f"orc_residual_{_sfx(psi)}", gn, gl, apply_B, psi.shape[0], _p(psi), _p(hpsi_),
          _p(tc), _p(out))
    return out


def mgm(n, ll, lap_type, vh, rho, ghosts=0, cogr=10, max_sweeps=10, tol=1e-16, nu1=2, nu2=2,
        ref=False):
    """pb::Mgm on one field: returns (vh after the solve, info dict).  ghosts:
    ghost width of the fine grid (0: the operator's)."""
    L = ref_lib() if ref else lib()
    pre = "ref" if ref else "orc"
    vh = np.array(vh, copy=True).reshape(-1)
    rho = np.ascontiguousarray(rho, dtype=vh.dtype).reshape(-1)
    ng = ghosts if ghosts > 0 else {0: 1, 1: 1, 2: 2, 3: 3, 4: 4}[lap_type]
    out = np.zeros(6)
    gn, gl = _grid(n, ll)
    _call(L, f"{pre}_mgm_{_sfx(vh)}", gn, gl, lap_type, ng, cogr, max_sweeps, ctypes.c_double(tol),
          nu1, nu2, _p(vh), _p(rho), _p(out))
    info = {"final_residual": out[0], "final_relative_residual": out[1],
            "residual_reduction": out[2], "nb_sweeps": int(out[3]), "converged": bool(out[4])}
    if not ref:
        info["levels"] = int(out[5])
    return vh, info


def matb(n, ll, psi, ref=False):
    """B = psi^T (B psi) * vel (LocGridOrbitals::computeMatB), both
    triangles; row-major numpy (nfunc, nfunc)."""
    psi = np.ascontiguousarray(psi)
    nf = psi.shape[0]
    B = np.zeros((nf, nf))
    gn, gl = _grid(n, ll)
    name = f"ref_matb_{_sfx(psi)}" if ref else f"orc_matb_{_sfx(psi)}"
    _call(ref_lib() if ref else lib(), name, gn, gl, nf, _p(psi), _p(B))
    return B.T.copy()


def normalize(n, ll, psi, ref=False):
    """LocGridOrbitals::normalize: returns (normalized copy of psi, diagS)."""
    out = np.array(psi, copy=True, order="C")
    nf = out.shape[0]
    d = np.zeros(nf)
    gn, gl = _grid(n, ll)
    name = f"ref_normalize_{_sfx(out)}" if ref else f"orc_normalize_{_sfx(out)}"
    _call(ref_lib() if ref else lib(), name, gn, gl, nf, _p(out), _p(d))
    return out, d


def update_hb(S, th):
    """HB = sym(S theta) (ProjectedMatricesMehrstellen::updateHB), row-major."""
    n = S.shape[0]
    Sc = np.ascontiguousarray(np.asarray(S, dtype=np.float64).T)
    tc = np.ascontiguousarray(np.asarray(th, dtype=np.float64).T)
    out = np.zeros((n, n))
    _call(lib(), "orc_update_hb", n, _p(Sc), _p(tc), _p(out))
    return out.T.copy()


def anderson(x0, fseq, m, beta, vel, invs, fscale=1.0, ref=False):
    """nsteps AndersonMix updates of x0 (nfunc, npts) with the residuals
    fscale * fseq[s] (nsteps, nfunc, npts); invs (nsteps, nfunc) the weights
    (S^-1)(k, k) of each step.  Returns x after every update."""
    x0 = np.ascontiguousarray(x0)
    fseq = np.ascontiguousarray(fseq, dtype=x0.dtype)
    invs = np.ascontiguousarray(invs, dtype=np.float64)
    ns, nf, npt = fseq.shape
    out = np.zeros((ns, nf, npt), dtype=x0.dtype)
    L = ref_lib() if ref else lib()
    name = f"{'ref' if ref else 'orc'}_anderson_{_sfx(x0)}"
    _call(L, name, npt, nf, m, ctypes.c_double(beta), ctypes.c_double(vel), _p(invs), _p(x0), ns,
          _p(fseq), ctypes.c_double(fscale), _p(out))
    return out


class AndersonState:
    """The oracle's AndersonMix kept across steps (for an iteration whose
    residuals depend on x)."""

    def __init__(self, m, beta, shape, dtype):
        self.sfx = "d" if np.dtype(dtype) == np.float64 else "f"
        L = lib()
        new = getattr(L, f"orc_anderson_new_{self.sfx}")
        new.restype = ctypes.c_void_p
        self.h = ctypes.c_void_p(new(m, ctypes.c_double(beta), ctypes.c_long(int(np.prod(shape)))))
        self.shape = shape

    def step(self, x, f, vel, invs_diag, fscale):
        """x (numpy, updated in place) moves by one update with fscale * f."""
        nf, npt = self.shape
        invs_diag = np.ascontiguousarray(invs_diag, dtype=np.float64)
        f = np.ascontiguousarray(f, dtype=x.dtype)
        _call(lib(), f"orc_anderson_step_{self.sfx}", self.h, npt, nf, ctypes.c_double(vel),
              _p(invs_diag), _p(x), _p(f), ctypes.c_double(fscale))
        return x

    def close(self):
        if self.h:
            getattr(lib(), f"orc_anderson_free_{self.sfx}")(self.h)
            self.h = None


def rho(n, ll, psi, X, nel=0.0, ref=False):
    """Density of the block with density matrix X (row-major numpy, n x n):
    (rho, charge, factor); the reference arm returns the unscaled density of
    its own MPgemmNN and loop (charge and factor None)."""
    psi = np.ascontiguousarray(psi)
    nf, npt = psi.shape
    Xc = np.ascontiguousarray(np.asarray(X, dtype=np.float64).T)
    out = np.zeros(npt)
    if ref:
        _call(ref_lib(), f"ref_rho_{_sfx(psi)}", npt, nf, _p(psi), _p(Xc), _p(out))
        return out, None, None
    gn, gl = _grid(n, ll)
    info = np.zeros(2)
    rc = getattr(lib(), f"orc_rho_{_sfx(psi)}")(gn, gl, nf, _p(psi), _p(Xc), ctypes.c_double(nel),
                                                 _p(out), _p(info))
    if rc != 0:
        raise RuntimeError("density charge off by more than 2%")
    return out, info[0], info[1]


# ------------------------------------------------------------ function packing
def pack_overlap(n, ll, centers, radii, subdivx, ghosts=1):
    """The orbital overlap pattern of FunctionsPacking with one task (uint8
    nfunc x nfunc, diagonal set).  Restates the subdomain geometry of
    LocalizationRegions::setupSubdomainGeometry (src/LocalizationRegions.cc:
    935-967: lattice L, margin ghosts (|h| + 1e-8), mesh lattice L - h),
    computeSubdivOverlapGids (:1039-1099: each region, radius r + margin
    rounded to float as LRData holds it, listed in every x sub-box whose
    closest point lies within it) and overlap (:1103-1119: a shared
    sub-box).  Pure Python loops, small cases."""
    h = [ll[i] / n[i] for i in range(3)]
    div = [ll[i] - h[i] for i in range(3)]
    delta = (np.sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) + 1.e-8) * float(ghosts)
    loc = ll[0] / subdivx
    nf = len(radii)
    inbox = np.zeros((nf, subdivx), dtype=bool)
    for f in range(nf):
        radius = np.float32(np.float64(np.float32(radii[f])) + delta)
        r2 = float(radius * radius)  # float product, as the reference's
        for iloc in range(subdivx):
            cc = [0.5 * ((2 * iloc + 1) * loc), 0.5 * div[1], 0.5 * div[2]]
            t = [float(centers[f][i]) for i in range(3)]
            for i in range(3):
                while t[i] >= cc[i] + 0.5 * ll[i]:
                    t[i] -= ll[i]
                while t[i] < cc[i] - 0.5 * ll[i]:
                    t[i] += ll[i]
            p = list(t)
            if p[0] < iloc * loc:
                p[0] = iloc * loc
            if p[1] < 0.:
                p[1] = 0.
            if p[2] < 0.:
                p[2] = 0.
            if p[0] > (iloc + 1) * loc - h[0]:
                p[0] = (iloc + 1) * loc - h[0]
            if p[1] > div[1]:
                p[1] = div[1]
            if p[2] > div[2]:
                p[2] = div[2]
            d2 = (p[0] - t[0]) * (p[0] - t[0]) + (p[1] - t[1]) * (p[1] - t[1]) \
                + (p[2] - t[2]) * (p[2] - t[2])
            inbox[f, iloc] = d2 < r2
    ov = (inbox.astype(np.int32) @ inbox.T.astype(np.int32)) > 0
    np.fill_diagonal(ov, True)
    return ov.astype(np.uint8)


def _sort_desc(a, b, lo, hi):
    """quicksortI_h2l (src/tools/coloring.cc): a descending, b alongside."""
    i, j = lo, hi
    x = a[(lo + hi) // 2]
    while True:
        while a[i] > x:
            i += 1
        while a[j] < x:
            j -= 1
        if i <= j:
            a[i], a[j] = a[j], a[i]
            b[i], b[j] = b[j], b[i]
            i += 1
            j -= 1
        if not i <= j:
            break
    if lo < j:
        _sort_desc(a, b, lo, j)
    if i < hi:
        _sort_desc(a, b, i, hi)


def pack_colors(overlap, rlf=False):
    """The colouring of FunctionsPacking::getColors (src/FunctionsPacking.cc:
    79-158) on an overlap pattern: greedyColor (degree order of
    quicksortI_h2l, then greedyMC's smallest free colour) or colorRLF
    (src/tools/coloring.cc).  Returns (colour per function, colours)."""
    ov = np.asarray(overlap).astype(bool)
    nf = ov.shape[0]
    color = [-1] * nf
    if not rlf:
        deg = [int(ov[i].sum()) for i in range(nf)]
        order = list(range(nf))
        if nf:
            _sort_desc(deg, order, 0, nf - 1)
        ncol = 0
        for v in order:
            taken = {color[j] for j in range(nf) if ov[v, j] and color[j] >= 0}
            top = max(taken) if taken else -1
            c = 0
            while c <= top and c in taken:
                c += 1
            color[v] = c
            ncol = max(ncol, c + 1)
        return np.asarray(color, dtype=np.int32), ncol
    unc = list(range(nf))
    ncol = 0
    while unc:
        v0, best = -1, -1
        for j in unc:  # the multimap keeps the last of equal degrees
            d = sum(1 for i in unc if ov[i, j])
            if d > 0 and d >= best:
                v0, best = j, d
        unc.remove(v0)
        color[v0] = ncol
        u = [i for i in unc if ov[i, v0]]
        v = [i for i in unc if not ov[i, v0]]
        while v:
            u0, bu = -1, -1
            for j in v:
                d = sum(1 for i in u if ov[i, j])
                if d >= bu:
                    u0, bu = j, d
            color[u0] = ncol
            unc.remove(u0)
            u += [i for i in v if ov[i, u0]]
            v = [i for i in v if not ov[i, u0]]
        ncol += 1
    return np.asarray(color, dtype=np.int32), ncol


def ref_pack_colors(overlap, rlf=False):
    """The same colouring by the reference's own coloring.cc (None when the
    reference was not built here)."""
    L = ref_lib()
    if L is None:
        return None
    ov = np.ascontiguousarray(overlap, dtype=np.uint8)
    nf = ov.shape[0]
    colors = np.zeros(max(nf, 1), dtype=np.int32)
    nc = ctypes.c_int()
    rc = L.ref_pack_colors(nf, ov.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)),
                           1 if rlf else 0, colors.ctypes.data_as(_ip), ctypes.byref(nc))
    if rc != 0:
        raise RuntimeError("ref_pack_colors failed")
    return colors[:nf].copy(), nc.value


# ------------------------------------------------------------ centres and spreads
def sincos_tables(n, ll, ref=False):
    """pb::Grid::getSinCosFunctions (src/pb/Grid.cc:244-282) in FP64, one
    task: per direction cos(i 2 pi / n) L / (2 pi), then sin; concatenated
    as cos x, sin x, cos y, sin y, cos z, sin z.  ref: the reference's own
    Grid (None when it was not built here)."""
    if ref:
        L = ref_lib()
        if L is None:
            return None
        out = np.zeros(2 * sum(n))
        L.ref_sincos_tables((ctypes.c_int * 3)(*n), (ctypes.c_double * 3)(*ll), _p(out))
        return out
    import math
    parts = []
    for d in range(3):
        alpha = ll[d] * (0.5 * (1.0 / math.pi))
        hh = 2. * math.pi / float(n[d])
        parts.append([math.cos(float(i) * hh) * alpha for i in range(n[d])])
        parts.append([math.sin(float(i) * hh) * alpha for i in range(n[d])])
    return np.asarray(sum(parts, []))


def sincos_diag(n, ll, psi, normalized=False):
    """SinCosOps::computeDiag (src/SinCosOps.cc:733-826) with one task and
    one subdomain: per orbital the six sums vel sum psi^2 t, divided by the
    norm vel sum psi^2 unless normalized (FP64, (nfunc, 6))."""
    t = sincos_tables(n, ll)
    nx, ny, nz = n
    cx, sx = t[0:nx], t[nx:2 * nx]
    cy, sy = t[2 * nx:2 * nx + ny], t[2 * nx + ny:2 * nx + 2 * ny]
    cz, sz = t[2 * nx + 2 * ny:2 * nx + 2 * ny + nz], t[2 * nx + 2 * ny + nz:]
    vel = (ll[0] / nx) * (ll[1] / ny) * (ll[2] / nz)
    a = np.asarray(psi, dtype=np.float64).reshape(-1, nx, ny, nz) ** 2
    out = np.stack([np.einsum("fxyz,x->f", a, cx), np.einsum("fxyz,x->f", a, sx),
                    np.einsum("fxyz,y->f", a, cy), np.einsum("fxyz,y->f", a, sy),
                    np.einsum("fxyz,z->f", a, cz), np.einsum("fxyz,z->f", a, sz)], axis=1)
    if normalized:
        return vel * out
    norm = vel * a.reshape(a.shape[0], -1).sum(axis=1)
    return vel * out / norm[:, None]


def centers_spreads(ll, a):
    """SpreadsAndCenters::computeCenter and computeSpread
    (src/SpreadsAndCenters.cc:26-104) from the (nfunc, 6) elements."""
    import math
    ll = np.asarray(ll, dtype=np.float64)
    lby2pi = ll * (0.5 * (1.0 / math.pi))
    c, s = a[:, 0::2], a[:, 1::2]
    x = lby2pi[None, :] * np.arctan2(s, c)
    x = np.where(x < 0., x + ll[None, :], x)
    return x, np.sqrt((lby2pi[None, :] ** 2 - c * c - s * s).sum(axis=1))


# ------------------------------------------------------------ localization regions
def regions_move_to(centers, targets, cell):
    """LocalizationRegions::moveTo (src/LocalizationRegions.cc:405-450) with
    Vector3D::vminimage (src/tools/Vector3D.cc:32-63, periodic): (new
    centres, largest move as float)."""
    import math
    c = [list(map(float, x)) for x in np.asarray(centers, dtype=np.float64).reshape(-1, 3)]
    t = np.asarray(targets, dtype=np.float64).reshape(-1, 3)
    mx = np.float32(0.)
    for f in range(len(c)):
        d = []
        for i in range(3):
            r = math.fmod(float(t[f][i]) - c[f][i], float(cell[i]))
            ax2 = 0.5 * float(cell[i])
            if r > ax2:
                r -= float(cell[i])
            elif r < -ax2:
                r += float(cell[i])
            d.append(r)
        nrm = np.float32(math.sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]))
        if nrm > mx:
            mx = nrm
        if nrm > 1.:
            d = [x / float(nrm) for x in d]
        for i in range(3):
            c[f][i] += d[i]
    return np.asarray(c), float(mx)


def regions_update_radii(spreads, ratio):
    """LocalizationRegions::updateRadii and getMeanRadius (:332-366): FP32
    radii ratio x spread and the cube root of their mean cube (FP32)."""
    r = np.asarray([np.float32(float(np.float32(ratio)) * float(s)) for s in spreads],
                   dtype=np.float32)
    rcube = np.float32(0.)
    for a in r:
        rcube = np.float32(rcube + np.float32(a * a * a))
    return r, float(np.cbrt(np.float32(rcube / np.float32(len(r)))))
