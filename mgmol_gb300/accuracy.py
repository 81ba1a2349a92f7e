"""Energy agreement of the mixed-precision sweep with the plain FP64 sweep.

    python -m mgmol_gb300.accuracy --grid 192 192 192 --nfunc 256 --iters 30

Both runs start from the same seeded orbitals and potential and take the
same number of ABPG steps (H psi, S and H, theta, residual, V-cycle,
update).  The energy of a step is the band-structure term tr(S^-1 H)
(ProjectedMatrices::getEigSum, Rydberg); the report gives it per step for
both runs and the largest difference in Hartree (Ry / 2), one JSON line.
"""
import argparse
import json
import sys
import time

import torch

from . import capi, synth
from .sweep import OrbitalSweep

GEMM = {"fp32": capi.GEMM_FP32, "tf32": capi.GEMM_TF32, "bf16x3": capi.GEMM_BF16X3}


def run(grid, h, nfunc, iters, gemm, wells, seed, lean=0):
    n = tuple(grid)
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    V = synth.gaussian_wells_device(n, ll, wells, seed)
    out = {}
    for mode in ("plain", "mixed"):
        dt = torch.float64 if mode == "plain" else torch.float32
        psi, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float64)
        psi = psi.to(dt)
        sw = OrbitalSweep(ctx, V, nfunc, mode=mode,
                          gemm=capi.GEMM_FP64 if mode == "plain" else GEMM[gemm],
                          chunk_funcs=lean if mode == "plain" else 0)
        # both modes use the FP64 run's preconditioner scale
        if mode == "mixed":
            sw.gamma = out["plain"]["gamma"]
        energies = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(iters):
            e = sw.run(psi)
            energies.append(float(e.cpu()[0]))
        torch.cuda.synchronize()
        out[mode] = {"energies_ry": energies, "seconds": time.perf_counter() - t0,
                     "gamma": sw.gamma}
        del sw, psi
        torch.cuda.empty_cache()
    dE = [abs(a - b) / 2 for a, b in zip(out["plain"]["energies_ry"], out["mixed"]["energies_ry"])]
    return {
        "grid": list(n), "h": h, "orbitals": nfunc, "iters": iters, "gemm": gemm,
        "max_abs_dE_ha": max(dE), "final_abs_dE_ha": dE[-1], "dE_ha_per_step": dE,
        "E_plain_ry": out["plain"]["energies_ry"], "E_mixed_ry": out["mixed"]["energies_ry"],
        "plain_s_per_step": out["plain"]["seconds"] / iters,
        "mixed_s_per_step": out["mixed"]["seconds"] / iters,
    }


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--grid", type=int, nargs=3, default=[96, 96, 96])
    ap.add_argument("--h", type=float, default=0.25)
    ap.add_argument("--nfunc", type=int, default=256)
    ap.add_argument("--iters", type=int, default=30)
    ap.add_argument("--gemm", default="bf16x3", choices=sorted(GEMM))
    ap.add_argument("--wells", type=int, default=16)
    ap.add_argument("--seed", type=int, default=1005)
    ap.add_argument("--lean", type=int, default=0, help="column chunk of the FP64 run (0 = full)")
    args = ap.parse_args(argv)
    res = run(args.grid, args.h, args.nfunc, args.iters, args.gemm, args.wells, args.seed,
              args.lean)
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
