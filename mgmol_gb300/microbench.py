"""Per-kernel timing of the orbital hot path at a chosen shape.

    python -m mgmol_gb300.microbench gram_hmat --grid 96 96 32 --nfunc 2048
    python -m mgmol_gb300.microbench all --grid 192 192 192 --nfunc 256

Each operation runs through the C ABI on device-resident synthetic inputs
(seeded Gaussian orbitals and wells), `--warmup` untimed and `--reps` timed
calls bracketed by CUDA events on the current stream; one JSON line per
operation gives milliseconds per call and the achieved rate against the
algorithmic work (flop for the products, bytes for the stencil passes).
"""
import argparse
import json
import sys

import torch

from . import capi, synth
from .sweep import vcycle_bytes

GEMM = {"fp64": capi.GEMM_FP64, "fp32": capi.GEMM_FP32, "tf32": capi.GEMM_TF32,
        "bf16x3": capi.GEMM_BF16X3, "fp16x3": capi.GEMM_FP16X3}


def _time(fn, warmup, reps):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("op", choices=["gram", "hmat", "gram_hmat", "matb", "gram_hmat_matb", "mult",
                                   "residual", "hpsi", "precond", "mgm", "dense", "dense_b",
                                   "dense_parts", "normalize", "mult_reuse", "h2d", "h2d_kernel",
                                   "all"])
    ap.add_argument("--streams", type=int, default=1, help="h2d: concurrent copy streams")
    ap.add_argument("--grid", type=int, nargs=3, default=[96, 96, 32])
    ap.add_argument("--h", type=float, default=0.25)
    ap.add_argument("--nfunc", type=int, default=2048)
    ap.add_argument("--gemm", default="bf16x3", choices=sorted(GEMM))
    ap.add_argument("--fp64", action="store_true", help="FP64 orbitals (GEMM mode fp64)")
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--reps", type=int, default=5)
    args = ap.parse_args(argv)
    torch.manual_seed(0)

    n = tuple(args.grid)
    ll = tuple(x * args.h for x in n)
    N = args.nfunc
    dt = torch.float64 if args.fp64 else torch.float32
    mode = capi.GEMM_FP64 if args.fp64 else GEMM[args.gemm]
    ctx = capi.Context(n, ll)
    npts = ctx.npts
    s = 8 if args.fp64 else 4
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, N, 11, dt)
    V = synth.gaussian_wells_device(n, ll, 16, 11).to(dt)
    hpsi = ctx.hpsi(psi, V)
    torch.cuda.synchronize()
    ops = ["gram", "hmat", "gram_hmat", "matb", "gram_hmat_matb", "mult", "residual", "hpsi",
           "precond", "dense", "dense_b", "normalize", "mgm"] \
        if args.op == "all" else [args.op]
    out = []
    for op in ops:
        if op == "gram":
            ms = _time(lambda: ctx.gram(psi, mode), args.warmup, args.reps)
            work, unit = N * (N + 1) * npts, "TFLOP/s"
        elif op == "hmat":
            ms = _time(lambda: ctx.hmat(psi, hpsi, mode), args.warmup, args.reps)
            work, unit = 2.0 * N * N * npts, "TFLOP/s"
        elif op == "gram_hmat":
            ms = _time(lambda: ctx.gram_hmat(psi, hpsi, mode), args.warmup, args.reps)
            work, unit = N * (N + 1) * npts + 2.0 * N * N * npts, "TFLOP/s"
        elif op == "matb":
            wb = torch.empty_like(psi)
            ms = _time(lambda: ctx.matb(psi, mode, work=wb), args.warmup, args.reps)
            del wb
            work, unit = N * (N + 1) * npts, "TFLOP/s"
        elif op == "gram_hmat_matb":
            wb = torch.empty_like(psi)
            ms = _time(lambda: ctx.gram_hmat_matb(psi, hpsi, mode, work=wb), args.warmup, args.reps)
            del wb
            work, unit = 2 * N * (N + 1) * npts + 2.0 * N * N * npts, "TFLOP/s"
        elif op == "dense_parts":
            # each FP64 piece of the dense phase on its own (N from --nfunc)
            S, H, Bm = ctx.gram_hmat_matb(psi, hpsi, mode)
            L = ctx.cholesky(S)
            Sinv = ctx.inverse_from_cholesky(L).contiguous()
            th = ctx.theta(Sinv, H)
            parts = {
                "cholesky": (lambda: ctx.cholesky(S), N ** 3 / 3),
                "inverse_from_cholesky": (lambda: ctx.inverse_from_cholesky(L), N ** 3),
                "theta_symm": (lambda: ctx.theta(Sinv, H), 2 * N ** 3),
                "theta_from_cholesky": (lambda: ctx.theta_from_cholesky(L, H), 2 * N ** 3),
                "update_hb": (lambda: ctx.update_hb(S, th), 2 * N ** 3),
                "trace_prod": (lambda: ctx.trace_prod(H, Sinv), 2 * N ** 2),
            }
            for name, (fn, fl) in parts.items():
                pms = _time(fn, args.warmup, args.reps)
                line = {"op": "dense_parts", "part": name, "nfunc": N, "ms": pms,
                        "achieved": fl / (pms * 1e-3) / 1e12, "unit": "TFLOP/s"}
                out.append(line)
                print(json.dumps(line), flush=True)
            continue
        elif op == "normalize":
            ms = _time(lambda: ctx.normalize(psi), args.warmup, args.reps)
            work, unit = 3 * N * npts * s, "GB/s"
        elif op == "mult_reuse":
            # Psi Theta reading the Gram product's conversion of psi (MN-major A)
            th = (torch.eye(N, dtype=torch.float64, device="cuda")
                  + torch.randn(N, N, dtype=torch.float64, device="cuda") / N)
            dst = torch.empty_like(psi)
            ctx.set_reuse_conversion(True)
            ctx.gram(psi, mode)
            ms = _time(lambda: ctx.mult_matrix(psi, th, mode, out=dst), args.warmup, args.reps)
            ctx.set_reuse_conversion(False)
            del dst
            work, unit = 2.0 * N * N * npts, "TFLOP/s"
        elif op in ("mult", "residual"):
            th = (torch.eye(N, dtype=torch.float64, device="cuda")
                  + torch.randn(N, N, dtype=torch.float64, device="cuda") / N)
            dst = torch.empty_like(psi)
            if op == "mult":
                ms = _time(lambda: ctx.mult_matrix(psi, th, mode, out=dst), args.warmup, args.reps)
            else:
                work_blk = torch.empty_like(psi)
                ms = _time(lambda: ctx.residual(psi, hpsi, th, mode, True, work=work_blk, out=dst),
                           args.warmup, args.reps)
                del work_blk
            del dst
            work, unit = 2.0 * N * N * npts, "TFLOP/s"
        elif op == "hpsi":
            dst = torch.empty_like(psi)
            ms = _time(lambda: ctx.hpsi(psi, V, out=dst), args.warmup, args.reps)
            del dst
            work, unit = N * npts * 2 * s + npts * s, "GB/s"
        elif op == "precond":
            dst = torch.empty_like(psi)
            gamma = ctx.gamma(capi.LAP_MEHR4, 2, float(V.max()), float(V.min()))
            ms = _time(lambda: ctx.precond_mg(hpsi, capi.LAP_MEHR4, 2, gamma, out=dst),
                       args.warmup, args.reps)
            del dst
            work, unit = vcycle_bytes(N, npts, s, 2), "GB/s"
        elif op == "dense":
            S, H = ctx.gram_hmat(psi, hpsi, mode)

            def dense():
                L = ctx.cholesky(S)
                Sinv = ctx.inverse_from_cholesky(L)
                ctx.trace_prod(H, Sinv.contiguous())
                ctx.theta(Sinv, H)
            ms = _time(dense, args.warmup, args.reps)
            work, unit = (N ** 3 / 3 + 4 * N ** 3 / 3 + 2 * N ** 3), "TFLOP/s"
        elif op == "dense_b":
            # the dense algebra of the Mehrstellen step: S^-1, theta = B^-1 H by
            # substitution, HB = sym(S theta), tr(HB S^-1)
            S, H, Bm = ctx.gram_hmat_matb(psi, hpsi, mode)

            def dense_b():
                Sinv = ctx.inverse_from_cholesky(ctx.cholesky(S)).contiguous()
                th, _ = ctx.theta_from_cholesky(ctx.cholesky(Bm), H)
                ctx.trace_prod(ctx.update_hb(S, th), Sinv)
            ms = _time(dense_b, args.warmup, args.reps)
            work, unit = (2 * N ** 3 / 3 + 4 * N ** 3 / 3 + 2 * N ** 3 + 2 * N ** 3), "TFLOP/s"
        elif op == "h2d":
            # pinned host block -> device block, split over --streams streams
            host = torch.empty(psi.shape, dtype=dt, pin_memory=True)
            host.copy_(psi)
            dst = torch.empty_like(psi)
            streams = [torch.cuda.Stream() for _ in range(args.streams)]
            parts = list(zip(host.chunk(args.streams), dst.chunk(args.streams)))

            def copy():
                cur = torch.cuda.current_stream()
                for st, (h, d) in zip(streams, parts):
                    st.wait_stream(cur)
                    with torch.cuda.stream(st):
                        d.copy_(h, non_blocking=True)
                for st in streams:
                    cur.wait_stream(st)
            ms = _time(copy, 1, args.reps)
            work, unit = host.numel() * host.element_size(), "GB/s"
            del host, dst
        elif op == "h2d_kernel":
            host = torch.empty(psi.shape, dtype=dt, pin_memory=True)
            host.copy_(psi)
            dst = torch.empty_like(psi)
            ms = _time(lambda: capi.copy(dst, host), 1, args.reps)
            assert torch.equal(dst, psi)
            work, unit = host.numel() * host.element_size(), "GB/s"
            del host, dst
        elif op == "mgm":
            rho = V[0:npts].double() - V.double().mean()
            vh = torch.zeros(npts, dtype=torch.float64, device="cuda")

            def solve():
                vh.zero_()
                ctx.mgm(vh, rho, max_sweeps=10, tol=1e-10)
            ms = _time(solve, 1, max(1, args.reps // 2))
            work, unit = None, None
        rate = None
        if work is not None:
            scale = 1e12 if unit == "TFLOP/s" else 1e9
            rate = work / (ms * 1e-3) / scale
        line = {"op": op, "grid": list(n), "nfunc": N, "dtype": "f64" if args.fp64 else "f32",
                "gemm": "fp64" if args.fp64 else args.gemm, "ms": ms, "achieved": rate, "unit": unit}
        out.append(line)
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
