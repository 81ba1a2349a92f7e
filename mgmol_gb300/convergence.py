"""Converged energy of the mixed-precision sweep against the plain FP64 sweep.

    python -m mgmol_gb300.convergence --grid 48 48 48 --h 0.35 --nfunc 32 --wells 8

MGmol stops its electronic iterations on the change of the eigenvalue sum
(DFTsolver<T>::checkConvergenceEnergy, src/DFTsolver.cc:138-167):
sum_eig = 2 getEigSum in Ry (src/DFTsolver.cc:202-203), deig = |sum_eig[k]
- sum_eig[k-1]|, deig2 = max(deig, previous deig) (1e9 before the first
change, src/DFTsolver.cc:220-225), converged when step > 1 and deig2 <
conv_tol.  In Hartree sum_eig is tr(HB S^-1) (the trace in Ry, times the
occupation 2, over 2), so the tolerances here are Hartree on that number.

Two iterations start from the same seeded orbitals and potential:
  plain  FP64 orbitals, stencils, products and V-cycle (152 s per sweep at
         2048 orbitals on 192^3), stopped by the test on its own energies;
  mixed  FP32 orbitals and stencils with split-BF16x3 tensor-core products
         (0.72 s per sweep there), stopped by the same test on energies
         evaluated to FP64-class accuracy (energy_accurate): the sweep's
         own energy carries a bias and a sweep-to-sweep noise from its FP32
         stencils and FP32-accumulated products (about 1e-3 Ha and 3e-5 Ha
         at 256 orbitals on 96^3) that the test at 1e-6 Ha cannot see
         through, while its orbitals follow the FP64 trajectory closely.
The report gives both converged energies and their gap, the sweeps and the
seconds of each path, the accurate energies against the plain trajectory at
the same sweep, and one full FP64 evaluation of the final mixed block.
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


class EnergyTest:
    """DFTsolver's convergence test on the eigenvalue sum, in Hartree.

    push(e_ry) takes the sweep's tr(HB S^-1) in Ry; sum_eig in Hartree is
    the same number (2 x tr Ry / 2).  Returns True once step > 1 and the
    larger of the last two changes is below tol."""

    def __init__(self, tol_ha):
        self.tol = float(tol_ha)
        self.energies = []
        self.deig = 1e9
        self.deig2 = 1e9

    def push(self, e_ry):
        self.energies.append(float(e_ry))
        step = len(self.energies) - 1
        if step > 0:
            old = self.deig
            self.deig = abs(self.energies[-1] - self.energies[-2])
            self.deig2 = max(self.deig, old)
        return step > 1 and self.deig2 < self.tol


def iterate(sw, psi, tol_ha, max_steps):
    """Sweeps until the energy test holds or max_steps sweeps ran.  The
    sweep that reports convergence has already moved psi on (the reference
    breaks before its update); the energy it reports is that of the block
    it started from.  Returns (EnergyTest, sweeps, converged)."""
    test = EnergyTest(tol_ha)
    for k in range(max_steps):
        e = sw.run(psi)
        if test.push(float(e.cpu()[0])):
            return test, k + 1, True
    return test, max_steps, False


def energy_fp64(ctx, V64, psi, nfunc, gamma):
    """tr(HB S^-1) of a block in FP64: the block promoted to FP64, H psi, S,
    H, B and the dense algebra on the FP64 units, no update."""
    p = psi.to(torch.float64).contiguous()
    sw = OrbitalSweep(ctx, V64, nfunc, mode="plain", gamma=gamma)
    e = float(sw.run(p, update=False).cpu()[0])
    del sw, p
    return e


def _trace_binv_h(S, H, B):
    """tr(HB S^-1) with HB = sym(S B^-1 H), i.e. tr(B^-1 H), on the host in FP64."""
    import numpy as np
    Hn = H.cpu().numpy() if hasattr(H, "cpu") else H
    Bn = B.cpu().numpy() if hasattr(B, "cpu") else B
    return float(np.trace(np.linalg.solve(Bn, Hn)))


def evaluation_errors(ctx, V64, psi32):
    """Energy of one FP32 block evaluated with each combination of stencil
    precision (FP64 on the promoted block, FP64 rounded to FP32, FP32) and
    product mode (FP64, FP32 CUDA cores, split-BF16x3, TF32); the dense
    algebra is the same FP64 host solve for all.  Returns {name: E} in the
    units of the sweep's energy, with "fp64" the exact evaluation."""
    p64 = psi32.to(torch.float64)
    V32 = V64.to(torch.float32)
    hp64 = ctx.hpsi(p64, V64, capi.LAP_MEHR4, True)
    bp64 = ctx.rhs_mehr(p64)
    hp32 = ctx.hpsi(psi32, V32, capi.LAP_MEHR4, True)
    bp32 = ctx.rhs_mehr(psi32)
    stencils = {"st64": (hp64, bp64), "st64r32": (hp64.float(), bp64.float()),
                "st32": (hp32, bp32)}
    out = {}
    for sname, (hp, bp) in stencils.items():
        for pname, mode in (("pr64", capi.GEMM_FP64), ("fp32", capi.GEMM_FP32),
                            ("bf16x3", capi.GEMM_BF16X3), ("tf32", capi.GEMM_TF32)):
            if mode == capi.GEMM_FP64:
                a, hb, bb = p64, hp.to(torch.float64), bp.to(torch.float64)
            else:
                if sname == "st64":
                    continue
                a, hb, bb = psi32, hp, bp
            S = ctx.gram(a, mode)
            H = ctx.hmat(a, hb, mode)
            B = ctx.hmat(a, bb, mode)
            out[f"{sname}+{pname}"] = _trace_binv_h(S, H, B)
    out["fp64"] = out.pop("st64+pr64")
    # the FP32 Mehrstellen operator on a constant field (its row sum)
    one = torch.ones((1, ctx.npts), dtype=torch.float32, device=psi32.device)
    out["rowsum_f32_lap"] = float(ctx.fd_apply(one, capi.LAP_MEHR4).abs().max())
    out["rowsum_f32_B_minus_1"] = float((ctx.rhs_mehr(one) - 1).abs().max())
    return out


def energy_accurate(ctx, V64, psi32, chunk=64, hp=None, bp=None):
    """tr(B^-1 H) of an FP32 block to FP64-class accuracy at FP32 cost.

    H psi and B psi come from the FP64 stencils applied to chunks of the
    block promoted to FP64, each kept as two FP32 blocks, hi = fl32(x) and
    lo = fl32(x - hi), so that nothing of the FP64 result is lost to the
    FP32 storage.  H = Psi^T (H Psi) vel and B = Psi^T (B Psi) vel are then
    the CUDA-core FP32 products of Psi with hi, whose sums end in
    double-float (MGX_GEMM_FP32), plus the split-BF16x3 tensor-core products
    of Psi with lo (2^-24 of the total, so their own 1e-5 error does not
    show); the Cholesky of B, theta = B^-1 H and its trace in FP64.  The
    sweep's own energy differs: its FP32 stencils and split-K tensor-core
    products carry an error that grows with the points per orbital and the
    number of orbitals.  hp, bp: optional FP32 blocks of psi32's shape, the
    hi and lo halves of one operator's result (H psi, then B psi)."""
    nf = psi32.shape[0]
    hi = torch.empty_like(psi32) if hp is None else hp
    lo = torch.empty_like(psi32) if bp is None else bp

    def product(apply):
        for f0 in range(0, nf, chunk):
            f1 = min(nf, f0 + chunk)
            r = apply(psi32[f0:f1].to(torch.float64))
            hi[f0:f1] = r.to(torch.float32)
            lo[f0:f1] = (r - hi[f0:f1].to(torch.float64)).to(torch.float32)
            del r
        # the library's product workspaces come from cudaMalloc, not from
        # torch's cache: hand back what the FP64 chunks held
        torch.cuda.empty_cache()
        return ctx.hmat(psi32, hi, capi.GEMM_FP32) + ctx.hmat(psi32, lo, capi.GEMM_BF16X3)

    H = product(lambda p: ctx.hpsi(p, V64, capi.LAP_MEHR4, True))
    B = product(lambda p: ctx.rhs_mehr(p))
    _, tr = ctx.theta_from_cholesky(ctx.cholesky(B), H)
    return float(tr.cpu()[0])


def converge_mixed(ctx, V64, sw, psi, tol_ha, every=10, max_steps=2000):
    """The mixed-precision iteration stopped by the reference's energy test.

    The sweeps run in mixed precision (sw, FP32 block psi).  Their own
    energies are too noisy for the test at small tolerances, so the energy
    of the block is evaluated with energy_accurate: every `every` sweeps
    while the mean change per sweep over that stride is at or above tol,
    then after every sweep until DFTsolver's test (EnergyTest) holds on
    those consecutive energies.  Returns a dict with the sweeps run, the
    accurate evaluations made, the sampled (sweep, energy) pairs, the final
    energy and whether the test held."""
    samples = []
    test = EnergyTest(tol_ha)
    fine = False
    prev = None
    k = 0
    converged = False
    while k <= max_steps:
        if fine or k % every == 0:
            # the sweep's H psi and work blocks are free between sweeps
            e = energy_accurate(ctx, V64, psi, hp=sw.hpsi, bp=sw.corr) \
                if sw.corr.shape == psi.shape else energy_accurate(ctx, V64, psi)
            samples.append((k, e))
            if fine:
                if test.push(e):
                    converged = True
                    break
            else:
                if prev is not None and abs(e - prev) / every < tol_ha:
                    fine = True
                    test.push(e)
                prev = e
        if k == max_steps:
            break
        sw.run(psi)
        k += 1
    return {"sweeps": k, "evaluations": len(samples), "samples": samples,
            "E_ha": samples[-1][1], "converged": converged}


def run(grid, h, nfunc, wells, seed, tol_ha=1e-8, max_plain=2000, max_mixed=2000,
        gemm="bf16x3", every=10, diagnose=False):
    """The plain FP64 iteration and the mixed one from the same orbitals,
    each stopped by the reference's energy test at tol_ha; their energies,
    sweeps and times, and the gap between the two converged energies."""
    n = tuple(grid)
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    V64 = synth.gaussian_wells_device(n, ll, wells, seed)
    psi0, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float64)
    gamma = ctx.gamma(capi.LAP_MEHR4, 2, float(V64.max()), float(V64.min()))
    out = {"grid": list(n), "h": h, "orbitals": nfunc, "wells": wells, "seed": seed,
           "tol_ha": tol_ha, "gemm": gemm, "every": every}

    psi = psi0.clone()
    sw = OrbitalSweep(ctx, V64, nfunc, mode="plain", gamma=gamma)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tp, kp, cp = iterate(sw, psi, tol_ha, max_plain)
    torch.cuda.synchronize()
    tplain = time.perf_counter() - t0
    out["plain"] = {"sweeps": kp, "converged": cp, "E_ha": tp.energies[-1], "seconds": tplain,
                    "energies_ha": tp.energies}
    del sw, psi

    psi = psi0.to(torch.float32)
    sw = OrbitalSweep(ctx, V64, nfunc, mode="mixed", gemm=GEMM[gemm], gamma=gamma)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = converge_mixed(ctx, V64, sw, psi, tol_ha, every, max_mixed)
    torch.cuda.synchronize()
    m["seconds"] = time.perf_counter() - t0
    m["abs_dE_vs_plain_ha"] = abs(m["E_ha"] - tp.energies[-1])
    # the accurate energies against the plain trajectory at the same sweep
    track = [abs(e - tp.energies[k]) for k, e in m["samples"] if k < len(tp.energies)]
    m["max_abs_dE_same_sweep_ha"] = max(track) if track else None
    if diagnose:
        out["evaluation"] = evaluation_errors(ctx, V64, psi)
    out["mixed"] = m
    # one FP64 evaluation of the final mixed block (FP64 orbitals, stencils
    # and products): what energy_accurate stands in for
    out["mixed_final_fp64_ha"] = energy_fp64(ctx, V64, psi, nfunc, gamma)
    out["accurate_vs_fp64_ha"] = abs(out["mixed_final_fp64_ha"] - energy_accurate(ctx, V64, psi))
    out["time_ratio_plain_over_mixed"] = tplain / m["seconds"]
    del sw, psi
    torch.cuda.empty_cache()
    return out


def evaluation_check(grid, h, nfunc, wells, seed, sweeps=20, gemm="bf16x3"):
    """After `sweeps` mixed sweeps from the seeded orbitals: the sweep's own
    energy, energy_accurate and a full FP64 evaluation of the same block,
    with the seconds of the two evaluations (Hartree)."""
    n = tuple(grid)
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    V64 = synth.gaussian_wells_device(n, ll, wells, seed)
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float32)
    gamma = ctx.gamma(capi.LAP_MEHR4, 2, float(V64.max()), float(V64.min()))
    sw = OrbitalSweep(ctx, V64, nfunc, mode="mixed", gemm=GEMM[gemm], gamma=gamma)
    for _ in range(sweeps):
        sw.run(psi)
    e_sweep = float(sw.run(psi, update=False).cpu()[0])
    del sw
    torch.cuda.empty_cache()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_acc = energy_accurate(ctx, V64, psi)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    e64 = energy_fp64(ctx, V64, psi, nfunc, gamma)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    # FP64 products of H psi and B psi rounded to FP32: the share of the
    # accurate evaluation's error that the rounding of its stencil outputs
    # makes (the rest is its FP32 products)
    p64 = psi.to(torch.float64)
    hp = ctx.hpsi(p64, V64, capi.LAP_MEHR4, True).float().double()
    H = ctx.hmat(p64, hp, capi.GEMM_FP64)
    del hp
    bp = ctx.rhs_mehr(p64).float().double()
    B = ctx.hmat(p64, bp, capi.GEMM_FP64)
    del bp, p64
    _, tr = ctx.theta_from_cholesky(ctx.cholesky(B), H)
    e_r = float(tr.cpu()[0])
    return {"grid": list(n), "h": h, "orbitals": nfunc, "sweeps": sweeps, "E_sweep_ha": e_sweep,
            "E_accurate_ha": e_acc, "E_fp64_ha": e64, "sweep_minus_fp64_ha": e_sweep - e64,
            "accurate_minus_fp64_ha": e_acc - e64, "rounded_stencils_minus_fp64_ha": e_r - e64,
            "accurate_s": t1 - t0, "fp64_s": t2 - t1}


def mixed_only(grid, h, nfunc, wells, seed, tol_ha, max_mixed, gemm="bf16x3", every=10):
    """The mixed iteration alone, stopped by the energy test on accurate
    energies or after max_mixed sweeps (for sizes where the plain FP64
    iteration cannot be run to convergence): the sampled accurate energies,
    the sweeps, the seconds, and the last mean change per sweep."""
    n = tuple(grid)
    ll = tuple(x * h for x in n)
    ctx = capi.Context(n, ll)
    V64 = synth.gaussian_wells_device(n, ll, wells, seed)
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float32)
    gamma = ctx.gamma(capi.LAP_MEHR4, 2, float(V64.max()), float(V64.min()))
    sw = OrbitalSweep(ctx, V64, nfunc, mode="mixed", gemm=GEMM[gemm], gamma=gamma)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = converge_mixed(ctx, V64, sw, psi, tol_ha, every, max_mixed)
    torch.cuda.synchronize()
    m["seconds"] = time.perf_counter() - t0
    sm = m["samples"]
    m["last_change_per_sweep_ha"] = (abs(sm[-1][1] - sm[-2][1]) / max(1, sm[-1][0] - sm[-2][0])
                                     if len(sm) > 1 else None)
    m.update({"grid": list(n), "h": h, "orbitals": nfunc, "tol_ha": tol_ha})
    return m


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", type=int, nargs=3, default=[48, 48, 48])
    ap.add_argument("--h", type=float, default=0.35)
    ap.add_argument("--nfunc", type=int, default=32)
    ap.add_argument("--wells", type=int, default=8)
    ap.add_argument("--seed", type=int, default=1001)
    ap.add_argument("--tol", type=float, default=1e-8, help="Hartree, both paths")
    ap.add_argument("--max-plain", type=int, default=2000)
    ap.add_argument("--max-mixed", type=int, default=2000)
    ap.add_argument("--every", type=int, default=10,
                    help="sweeps between accurate energies while far from convergence")
    ap.add_argument("--gemm", default="bf16x3", choices=sorted(GEMM))
    ap.add_argument("--diagnose", action="store_true",
                    help="energy of the final mixed block under each evaluation precision")
    ap.add_argument("--mixed-only", action="store_true",
                    help="no plain FP64 run: the mixed iteration to --tol or --max-mixed sweeps")
    ap.add_argument("--eval-only", type=int, default=0, metavar="SWEEPS",
                    help="no convergence runs: the three evaluations of the block after this "
                         "many mixed sweeps")
    a = ap.parse_args(argv)
    if a.mixed_only:
        print(json.dumps(mixed_only(a.grid, a.h, a.nfunc, a.wells, a.seed, a.tol, a.max_mixed,
                                    a.gemm, a.every)), flush=True)
        return 0
    if a.eval_only:
        print(json.dumps(evaluation_check(a.grid, a.h, a.nfunc, a.wells, a.seed, a.eval_only,
                                          a.gemm)), flush=True)
        return 0
    res = run(a.grid, a.h, a.nfunc, a.wells, a.seed, a.tol, a.max_plain, a.max_mixed, a.gemm,
              a.every, a.diagnose)
    print(json.dumps(res), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
