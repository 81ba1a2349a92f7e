"""Energy agreement of the mixed-precision sweep with the plain FP64 sweep.

    python -m mgmol_gb300.accuracy --grid 192 192 192 --nfunc 256 --iters 30

The FP64 run and one mixed run per GEMM mode start from the same seeded
orbitals and potential and take the same number of ABPG steps (normalize,
H psi, S / H / B, theta, residual, V-cycle, update).  The energy of a step
is the band-structure term of ProjectedMatrices::getEigSum, tr(HB S^-1) in
Rydberg (with --theta gram, tr(S^-1 H)); the report gives it per step, the
differences in Hartree (Ry / 2) and the condition number of the normalized
block's S at the first and last step, one JSON line.
"""
import argparse
import json
import sys
import time

import torch

from . import capi, synth
from .sweep import OrbitalSweep

GEMM = {"fp32": capi.GEMM_FP32, "tf32": capi.GEMM_TF32, "bf16x3": capi.GEMM_BF16X3,
        "fp16x3": capi.GEMM_FP16X3}


def _trajectory(ctx, V, n, ll, nfunc, iters, seed, mode, gemm, lean, gamma, use_matb=True):
    dt = torch.float64 if mode == "plain" else torch.float32
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float64)
    psi = psi.to(dt)
    sw = OrbitalSweep(ctx, V, nfunc, mode=mode, gemm=gemm, chunk_funcs=lean,
                      use_matb=use_matb)
    if gamma is not None:
        sw.gamma = gamma
    energies, conds = [], []
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for it in range(iters):
        e = sw.run(psi)
        energies.append(float(e.cpu()[0]))
        if it in (0, iters - 1):
            S = sw.S
            if sw.fuse_update:
                # the step ran on the block before its normalization
                S = sw.dscale[:, None] * S * sw.dscale[None, :]
            w = torch.linalg.eigvalsh(S)
            conds.append(float(w[-1] / w[0]))
    torch.cuda.synchronize()
    out = {"energies_ry": energies, "seconds": time.perf_counter() - t0, "gamma": sw.gamma,
           "cond_S": conds}
    del sw, psi
    torch.cuda.empty_cache()
    return out


def run(grid, h, nfunc, iters, gemms, wells, seed, lean=0, use_matb=True):
    n = tuple(grid)
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    V = synth.gaussian_wells_device(n, ll, wells, seed)
    plain = _trajectory(ctx, V, n, ll, nfunc, iters, seed, "plain", capi.GEMM_FP64, lean, None,
                        use_matb)
    res = {"grid": list(n), "h": h, "orbitals": nfunc, "iters": iters,
           "theta": "B^-1 H" if use_matb else "S^-1 H",
           "E_plain_ry": plain["energies_ry"], "cond_S_plain": plain["cond_S"],
           "plain_s_per_step": plain["seconds"] / iters, "mixed": {}}
    for g in gemms:
        mixed = _trajectory(ctx, V, n, ll, nfunc, iters, seed, "mixed", GEMM[g], 0,
                            plain["gamma"], use_matb)
        dE = [abs(a - b) / 2 for a, b in zip(plain["energies_ry"], mixed["energies_ry"])]
        res["mixed"][g] = {"max_abs_dE_ha": max(dE), "first_abs_dE_ha": dE[0],
                           "final_abs_dE_ha": dE[-1], "dE_ha_per_step": dE,
                           "E_mixed_ry": mixed["energies_ry"],
                           "s_per_step": mixed["seconds"] / iters}
    return res


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, nargs=3, default=[96, 96, 96])
    ap.add_argument("--h", type=float, default=0.25)
    ap.add_argument("--nfunc", type=int, default=256)
    ap.add_argument("--iters", type=int, default=30)
    ap.add_argument("--gemm", default="bf16x3",
                    help="comma-separated GEMM modes of the mixed runs (" + ", ".join(sorted(GEMM)) + ")")
    ap.add_argument("--wells", type=int, default=16)
    ap.add_argument("--seed", type=int, default=1005)
    ap.add_argument("--lean", type=int, default=0, help="column chunk of the FP64 run (0 = full)")
    ap.add_argument("--theta", default="b", choices=["b", "gram"],
                    help="b: theta = B^-1 H (Mehrstellen, as the reference); gram: S^-1 H")
    args = ap.parse_args(argv)
    gemms = [g for g in args.gemm.split(",") if g]
    for g in gemms:
        if g not in GEMM:
            raise SystemExit(f"unknown GEMM mode {g}")
    res = run(args.grid, args.h, args.nfunc, args.iters, gemms, args.wells, args.seed, args.lean,
              args.theta == "b")
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
