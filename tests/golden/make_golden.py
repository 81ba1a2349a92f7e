"""Records golden vectors from the reference MGmol's own hot-path code.

Runs the reference translation units compiled unmodified against single-task
shims (oracle/build_ref.sh -> oracle/_ref/libmgref.so, built from the MGmol
source tree in this container) on small seeded inputs, and stores inputs and
outputs in tests/golden/ref_vectors.npz.  tests/test_oracle.py checks the
oracle restatement against these vectors; the GPU tests check the CUDA
kernels against the oracle.  Re-run after changing the generator:

    oracle/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from mgmol_gb300 import synth  # noqa: E402


def main():
    if O.ref_lib() is None:
        raise SystemExit("oracle/_ref/libmgref.so missing: run oracle/build_ref.sh first")
    out = {}
    # ragged grid, all operators, both precisions
    n = (16, 12, 20)
    ll = (16 * 0.35, 12 * 0.35, 20 * 0.35)
    psi, centers, _ = synth.gaussian_orbitals(n, ll, 3, 1001)
    V = synth.gaussian_wells(n, ll, 8, 1001)
    out["stencil_n"] = np.array(n)
    out["stencil_ll"] = np.array(ll)
    out["stencil_psi"] = psi
    out["stencil_V"] = V
    for tag, dt in (("d", np.float64), ("f", np.float32)):
        p = psi.astype(dt)
        for t in range(5):
            out[f"fd{t}_{tag}"] = O.fd_apply(n, ll, t, p, ref=True)
        out[f"rhs_{tag}"] = O.rhs_mehr(n, ll, p, ref=True)
        out[f"hpsi_{tag}"] = O.hpsi(n, ll, 0, p, V, ref=True)
        out[f"restrict_{tag}"] = O.restrict(n, ll, p, ref=True)
        out[f"extend_{tag}"] = O.extend(n, ll, out[f"restrict_{tag}"], ref=True)
    # V-cycle preconditioner, 3 grids (16^3 coarsest 4^3), three operators
    n = (16, 16, 16)
    ll = (16 * 0.35,) * 3
    res, centers, _ = synth.gaussian_orbitals(n, ll, 3, 1002)
    out["pc_n"] = np.array(n)
    out["pc_ll"] = np.array(ll)
    out["pc_res"] = res
    out["pc_gamma"] = np.array(0.3)
    for tag, dt in (("d", np.float64), ("f", np.float32)):
        for t in (0, 2, 4):
            out[f"pc{t}_{tag}"] = O.precond(n, ll, t, 2, 0.3, res.astype(dt), ref=True)
    # masks (GridMaskMax, gaussianDecay) at 3 levels, and the masked V-cycle
    radii = synth.mask_radii(3, 1003, 1.5, 3.0)
    out["mask_centers"] = centers
    out["mask_radii"] = radii
    st, vals = O.mask_build(n, ll, 1, 3, centers, radii, func=0, ref=True)
    out["mask_state"] = st
    for l, v in enumerate(vals):
        out[f"mask_values_{l}"] = v
    st1, vals1 = O.mask_build(n, ll, 1, 1, centers, radii, func=1, ref=True)
    out["mask1_state"] = st1
    out["mask1_values_0"] = vals1[0]
    out["pc0_masked_d"] = O.precond(n, ll, 0, 2, 0.3, res, masks=(centers, radii), ref=True)
    # Psi Theta (MPgemmNN) and the Mehrstellen residual B(psi) theta - hpsi
    n = (16, 12, 20)
    ll = (16 * 0.35, 12 * 0.35, 20 * 0.35)
    psi, _, _ = synth.gaussian_orbitals(n, ll, 7, 1004)
    V = synth.gaussian_wells(n, ll, 4, 1004)
    rng = np.random.default_rng(1004)
    th = np.eye(7) + rng.standard_normal((7, 7)) / 7
    out["res_n"] = np.array(n)
    out["res_ll"] = np.array(ll)
    out["res_psi"] = psi
    out["res_theta"] = th
    Xr = rng.standard_normal((7, 7))
    out["rho_X"] = 2.0 * (Xr @ Xr.T / 7 + np.eye(7))
    for tag, dt in (("d", np.float64), ("f", np.float32)):
        p = psi.astype(dt)
        hp = O.hpsi(n, ll, 0, p, V, ref=True)
        out[f"res_hpsi_{tag}"] = hp
        out[f"mm_{tag}"] = O.mult_matrix(p, th, ref=True)
        out[f"res_{tag}"] = O.residual(n, ll, p, hp, th, ref=True)
        # computeMatB and normalize on the same block
        out[f"matb_{tag}"] = O.matb(n, ll, p, ref=True)
        # the density of the block with a density matrix (unscaled)
        out[f"rho_{tag}"] = O.rho(n, ll, p, out["rho_X"], ref=True)[0]
        out[f"norm_psi_{tag}"], out[f"norm_diag_{tag}"] = O.normalize(n, ll, p, ref=True)
    # pb::Mgm on one field, every operator (6 V-cycles, nu1 = nu2 = 2)
    n = (16, 12, 20)
    ll = (16 * 0.4, 12 * 0.4, 20 * 0.4)
    rho = synth.gaussian_wells(n, ll, 6, 1005)
    rho = rho - rho.mean()
    vh0 = 0.1 * synth.gaussian_wells(n, ll, 3, 1006)
    out["mgm_n"] = np.array(n)
    out["mgm_ll"] = np.array(ll)
    out["mgm_rho"] = rho
    out["mgm_vh0"] = vh0
    for t in range(5):
        vh, info = O.mgm(n, ll, t, vh0, rho, max_sweeps=6, tol=1e-10, ref=True)
        out[f"mgm{t}_vh"] = vh
        out[f"mgm{t}_info"] = np.array([info["final_residual"], info["final_relative_residual"],
                                        info["residual_reduction"], info["nb_sweeps"],
                                        info["converged"]])
    vh, info = O.mgm(n, ll, 0, vh0.astype(np.float32), rho.astype(np.float32), max_sweeps=3,
                     tol=1e-10, ref=True)
    out["mgm0_vh_f"] = vh
    # AndersonMix<T>::update on residual sequences: a converging one, a
    # nearly collinear one (the determinant safeguard shortens the history)
    # and one with repeated residuals (coefficients outside [-3, 0.5])
    rng = np.random.default_rng(1007)
    nf, npt, ns = 5, 640, 9
    x0 = rng.standard_normal((nf, npt))
    g = rng.standard_normal((nf, npt))
    seqs = {
        "conv": np.stack([(0.6 ** s) * rng.standard_normal((nf, npt)) for s in range(ns)]),
        "collinear": np.stack([(0.7 ** s) * (g + 1e-3 * rng.standard_normal((nf, npt)))
                               for s in range(ns)]),
        "repeat": np.stack([(1.0 + 1e-4 * s) * g + 1e-6 * rng.standard_normal((nf, npt))
                            for s in range(ns)]),
    }
    invs = 1.0 + 0.2 * rng.random((ns, nf))
    out["and_x0"] = x0
    out["and_invs"] = invs
    for name, fs in seqs.items():
        out[f"and_f_{name}"] = fs
        for tag, dt in (("d", np.float64), ("f", np.float32)):
            for m in (1, 3):
                out[f"and_{name}_m{m}_{tag}"] = O.anderson(x0.astype(dt), fs.astype(dt), m, 1.0,
                                                           0.02, invs, fscale=0.5, ref=True)
    # S and H as getLocalOverlap / computeLocalProduct form them, summed by
    # LocalMatrices2DistMatrix (1e-14 filter): a dense case and narrow,
    # well separated orbitals whose far pairs the filter drops
    for case, (n, h, sig, nf, seed) in {"a": ((16, 12, 20), 0.35, (1.0, 2.0), 7, 1004),
                                        "b": ((24, 24, 24), 0.6, (0.5, 0.6), 6, 1006)}.items():
        ll = tuple(x * h for x in n)
        psi, _, _ = synth.gaussian_orbitals(n, ll, nf, seed, sigma=sig)
        V = synth.gaussian_wells(n, ll, 4, seed)
        out[f"sh{case}_n"] = np.array(n)
        out[f"sh{case}_ll"] = np.array(ll)
        out[f"sh{case}_psi"] = psi
        out[f"sh{case}_V"] = V
        for tag, dt in (("d", np.float64), ("f", np.float32)):
            p = psi.astype(dt)
            hp = O.hpsi(n, ll, 0, p, V, ref=True).astype(dt)
            out[f"sh{case}_hpsi_{tag}"] = hp
            out[f"sh{case}_S_{tag}"] = O.gram(p, h ** 3, ref=True)
            out[f"sh{case}_H_{tag}"] = O.hmat(p, hp, h ** 3, ref=True)
    np.savez_compressed(os.path.join(HERE, "ref_vectors.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_vectors.npz"), len(out), "arrays")


if __name__ == "__main__":
    main()
