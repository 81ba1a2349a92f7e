"""Errors of the mixed-precision H psi, S and H against the FP64 path at a
full configuration (one JSON line).

    python -m mgmol_gb300.errors --grid 128 128 128 --h 0.3 --nfunc 512 --lap 4

The FP64 path (FP64 orbitals, H psi and products on the FP64 units) is the
reference here; its kernels equal the CPU oracle to 1e-12 relative in the
tests, and the oracle itself cannot finish this size in reasonable time.
The mixed path takes the same orbitals rounded to FP32, H psi in FP32 and S,
H in each tensor-core mode.  Two errors are given for S and H: against the
FP64 products of the FP64 orbitals (everything the mixed path changes), and
against the FP64 products of the FP32-rounded orbitals (the product alone).
Then the FP64 Cholesky of S on the GPU, with its factor's residual.
"""
import argparse
import json
import sys

import torch

from . import capi, synth

MODES = {"bf16x3": capi.GEMM_BF16X3, "tf32": capi.GEMM_TF32, "fp16x3": capi.GEMM_FP16X3,
         "fp32": capi.GEMM_FP32}


def _err(a, b):
    d = float((a - b).abs().max())
    return {"max_abs": d, "rel_to_max": d / float(b.abs().max())}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", type=int, nargs=3, default=[128, 128, 128])
    ap.add_argument("--h", type=float, default=0.3)
    ap.add_argument("--nfunc", type=int, default=512)
    ap.add_argument("--wells", type=int, default=32)
    ap.add_argument("--lap", type=int, default=4)
    ap.add_argument("--seed", type=int, default=1002)
    a = ap.parse_args(argv)
    n = tuple(a.grid)
    ll = tuple(x * a.h for x in n)
    ctx = capi.Context(n, ll)
    apply_B = a.lap == capi.LAP_MEHR4
    psi64, _, _ = synth.gaussian_orbitals_device(n, ll, a.nfunc, a.seed, torch.float64)
    V64 = synth.gaussian_wells_device(n, ll, a.wells, a.seed)
    psi32 = psi64.float()
    hp64 = ctx.hpsi(psi64, V64, a.lap, apply_B)
    hp32 = ctx.hpsi(psi32, V64.float(), a.lap, apply_B)
    out = {"grid": list(n), "h": a.h, "nfunc": a.nfunc, "lap_type": a.lap,
           "hpsi_fp32": _err(hp32.double(), hp64)}
    S64, H64 = ctx.gram_hmat(psi64, hp64, capi.GEMM_FP64)
    # FP64 products of the FP32-rounded inputs: the reference for the product error alone
    S64r, H64r = ctx.gram_hmat(psi32.double(), hp32.double(), capi.GEMM_FP64)
    for name, mode in MODES.items():
        S, H = ctx.gram_hmat(psi32, hp32, mode)
        out[name] = {"S": _err(S, S64), "H": _err(H, H64),
                     "S_product_only": _err(S, S64r), "H_product_only": _err(H, H64r)}
        del S, H
    L = ctx.cholesky(S64.clone())
    Lt = torch.tril(L)
    out["cholesky_fp64"] = {"residual_rel": float((Lt @ Lt.T - S64).abs().max() / S64.abs().max())}
    torch.cuda.synchronize()
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)
