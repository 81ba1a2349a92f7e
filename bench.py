"""Orbital-sweep benchmark of the GB300 implementation of MGmol's hot path.

One step = one orbital sweep over all N orbitals, the reference's
iteration for a Mehrstellen operator: normalization of the block, H psi
(Mehrstellen operator and B(V psi)), the S, H and B matrices, FP64
Cholesky / inverse of S, theta = B^-1 H, HB and the energy tr(HB S^-1), the
residual B(psi) theta - H psi, one V-cycle preconditioner application and
the orbital update, on seeded synthetic orbitals.  --theta gram runs the
form with theta = S^-1 H and energy tr(S^-1 H) instead (no B matrix).

Default workload: 2048 orbitals on a 192^3 periodic grid (h = 0.25 bohr,
FP32 orbitals, 64 Gaussian wells) -- the configuration the metric is quoted
on.  Inputs (58 GB of orbitals) are far larger than the 126 MB L2, so no L2
flush is needed between steps.

Output: one JSON line (see the keys below).  --impl reference times the
CPU implementation of the same sweep (the oracle port of the reference's
algorithm, all host cores) on a bounded sample and extrapolates to the
workload; under torchrun only rank 0 runs it.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    # name: grid, h, nfunc, wells, lap_type, seed
    "c5": dict(n=(192, 192, 192), h=0.25, nfunc=2048, wells=64, seed=1005,
               workload="full sweep at scale: 2048 orbitals, 192^3, h=0.25, Mehrstellen"),
    "c1": dict(n=(64, 64, 64), h=0.35, nfunc=64, wells=8, seed=1001,
               workload="plain FP64 case: 64 orbitals, 64^3, h=0.35, Mehrstellen"),
    "c5_256": dict(n=(192, 192, 192), h=0.25, nfunc=256, wells=64, seed=1005,
                   workload="profiling slice: 256 orbitals on the 192^3 grid, h=0.25, Mehrstellen, FP32"),
    "c5_32": dict(n=(192, 192, 192), h=0.25, nfunc=32, wells=64, seed=1005,
                  workload="profiling slice: 32 orbitals on the 192^3 grid, h=0.25, Mehrstellen, FP32"),
    "medium": dict(n=(64, 64, 64), h=0.25, nfunc=512, wells=16, seed=8,
                   workload="medium sweep: 512 orbitals, 64^3, Mehrstellen, FP32 (profiling case)"),
    "small": dict(n=(64, 64, 64), h=0.25, nfunc=256, wells=16, seed=7,
                  workload="small sweep: 256 orbitals, 64^3, Mehrstellen, FP32"),
}
METRIC = "orbital sweeps/s (ABPG step: normalize, Hpsi, S/H/B, theta, residual, precond, update)"


# DRAM bytes (read + write) per split-K gram_kernel launch at the 2048-orbital
# 192^3 workload in split-BF16x3 (row tile order), measured once with ncu
# over the nine launches of one sweep (dram__bytes_read.sum +
# dram__bytes_write.sum, one pass); the operand planes read once would be
# 6.12e10 B per launch
SPLITK_DRAM_BYTES_PER_LAUNCH = 7.479e10
SPLITK_ALGO_BYTES_PER_LAUNCH = 6.122e10


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        import statistics
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), d.get(
            "bf16_tflops_sustained", 1700.0), "measured"
    return 6800.0, 1900.0, 1700.0, "fallback"


# --------------------------------------------------------------------- CPU leg
def _omp_threads(n):
    """Sets the OpenMP thread count of the oracle's parallel regions entered
    from this thread (the oracle links the process's one OpenMP runtime)."""
    import ctypes
    for name in ("libgomp.so.1", "libgomp.so"):
        try:
            ctypes.CDLL(name).omp_set_num_threads(int(n))
            return True
        except OSError:
            continue
    return False


def cpu_sweep_estimate(cfg, sample_funcs=4, products=True):
    """Times the oracle port of one sweep on `sample_funcs` orbitals of the
    workload grid and extrapolates to N: normalize, H psi, the B psi of
    computeMatB, the V-cycle and the residual stencil scale with N; S, H, B
    and Psi Theta with N^2 (B as the reference forms it, full N x N).  The
    N x N FP64 algebra is not timed (a few GFLOP against the products' tens
    of TFLOP).  Returns the seconds of the linear and the quadratic part per
    sweep (the quadratic part only when `products`)."""
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from mgmol_gb300 import synth

    n = cfg["n"]
    ll = tuple(x * cfg["h"] for x in n)
    N = cfg["nfunc"]
    psi, _, _ = synth.gaussian_orbitals(n, ll, sample_funcs, cfg["seed"], dtype=np.float32)
    V = synth.gaussian_wells(n, ll, cfg["wells"], cfg["seed"])
    vel = (cfg["h"]) ** 3
    t0 = time.perf_counter()
    O.normalize(n, ll, psi)
    hp = O.hpsi(n, ll, 0, psi, V)
    O.rhs_mehr(n, ll, psi)
    O.precond(n, ll, 0, 2, 0.2, hp)
    # the linear part of the residual (B applied to the product) and the update
    th = np.eye(sample_funcs)
    O.residual(n, ll, psi, hp.astype(np.float32), th, 1)
    t1 = time.perf_counter()
    lin = (t1 - t0) * (N / sample_funcs)
    if not products:
        return {"linear_s": lin, "quadratic_s": None, "sample_s": t1 - t0}
    # S, H and Psi Theta on a 128-orbital x 2^19-point slab: time per
    # (pair, point) of each product
    ns, ks = 128, min(1 << 19, n[0] * n[1] * n[2])
    rng = np.random.default_rng(0)
    slab = rng.standard_normal((ns, ks)).astype(np.float32)
    t3 = time.perf_counter()
    O.gram(slab, vel)
    O.hmat(slab, slab, vel)
    t4 = time.perf_counter()
    O.mult_matrix(slab, np.eye(ns))
    t5 = time.perf_counter()
    P = n[0] * n[1] * n[2]
    pairs_s = ns * (ns + 1) / 2 + ns * ns
    per_pair_point = (t4 - t3) / (pairs_s * ks)
    per_mm = (t5 - t4) / (ns * ns * ks)
    quad = per_pair_point * (N * (N + 1) / 2 + 2 * N * N) * P + per_mm * N * N * P
    return {"linear_s": lin, "quadratic_s": quad, "sample_s": (t1 - t0) + (t5 - t3)}


def cpu_baseline(cfg, sample_funcs, reps=1, as_written_funcs=4):
    """The CPU baseline of one sweep: the median of `reps` samples of the
    oracle port on all host threads (orbital-parallel stencils), and the
    reference as written, whose Mehrstellen kernels (FDkernelDel2_4th_Mehr,
    FDkernelRHS_4th_Mehr1, src/pb/FDkernels.cc:447-584) carry no OpenMP:
    the stencil phases timed on one thread, the products (threaded BLAS in
    the reference) on all threads."""
    import statistics
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    samples = [cpu_sweep_estimate(cfg, sample_funcs) for _ in range(max(1, reps))]
    per = statistics.median(s["linear_s"] + s["quadratic_s"] for s in samples)
    quad = statistics.median(s["quadratic_s"] for s in samples)
    out = {
        "value": 1.0 / per, "unit": "sweeps/s", "cores": cores, "kind": "port",
        "sample": (f"oracle port of the reference loops (FP32 data, FP64 accumulation as the "
                   f"USE_MP build), {cores} threads, median of {len(samples)}: normalize, H psi, "
                   f"B psi, V-cycle and the residual stencil on {sample_funcs} of {cfg['nfunc']} "
                   f"orbitals ({cfg['n'][0]}^3), scaled by N; S, H, B and Psi Theta timed on a "
                   f"128-orbital x 524288-point slab, scaled by pairs x points; N x N FP64 "
                   f"algebra not timed; one sample took {samples[0]['sample_s']:.1f} s"),
        "seconds_per_sweep": per,
    }
    if as_written_funcs:
        aw = as_written(cfg, quad, cores, as_written_funcs)
        if aw:
            out["as_written"] = aw
    return out


def as_written(cfg, quad_s, cores, funcs=4):
    """The reference as written: its stencil phases on one thread (sampled
    on `funcs` orbitals, scaled by N) plus the products' `quad_s` seconds on
    all threads; None when the OpenMP runtime cannot be reached."""
    if not _omp_threads(1):
        return None
    try:
        lin1 = cpu_sweep_estimate(cfg, funcs, products=False)["linear_s"]
    finally:
        _omp_threads(cores)
    return {"value": 1.0 / (lin1 + quad_s), "unit": "sweeps/s", "cores": cores,
            "sample": (f"stencil phases on 1 thread ({funcs} orbitals, scaled by N), products "
                       f"on {cores} threads as in the main sample")}


def slowest_replica_ms(ms, world, device):
    """Replicas only: every rank times its own copy of the workload; the job
    takes as long as its slowest rank (max over ranks, a collective on
    `device`, which is the rank's GPU under NCCL and the CPU under gloo)."""
    if world <= 1:
        return float(ms)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def job_sweeps_per_s(ms, world):
    """Whole-job throughput: every rank swept its own block once per step."""
    return world * 1e3 / ms


def _config(cfg, args, use_matb=None, chunk=0, net=False, world=1):
    """The config object of the JSON line (the same keys for both arms)."""
    mode = args.mode
    return {"workload": cfg["workload"], "grid": list(cfg["n"]), "h": cfg["h"],
            "orbitals": cfg["nfunc"], "mode": mode,
            "gemm": args.gemm if mode == "mixed" else "fp64", "lap_type": "mehrstellen",
            "precond": "learned U-Net, warm-started V-cycle, per-function V-cycle fallback"
            if net else "V-cycle 2 coarse levels",
            "theta": "B^-1 H (ProjectedMatricesMehrstellen)"
            if (args.theta == "b" if use_matb is None else use_matb)
            else "S^-1 H (ProjectedMatrices)",
            "schedule": f"column chunks of {chunk}" if chunk else "full blocks",
            "l2": "inputs larger than L2 (no flush)", "parallelism": f"replicas x{world}"}


def run_reference(args, cfg):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return 0
    import statistics
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    cores = int(os.environ["OMP_NUM_THREADS"])
    # each step is one bounded sample of the sweep on the host cores
    per, quad = [], []
    first = None
    for _ in range(args.steps):
        e = cpu_sweep_estimate(cfg, sample_funcs=args.cpu_sample)
        first = first or e
        per.append(e["linear_s"] + e["quadratic_s"])
        quad.append(e["quadratic_s"])
    sec = statistics.median(per)
    aw = as_written(cfg, statistics.median(quad), cores) if args.as_written else None
    line = {
        "impl": "reference", "metric": METRIC, "value": 1.0 / sec, "unit": "sweeps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sec, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": _config(cfg, args, chunk=0),
        "cpu_baseline": {
            "value": 1.0 / sec, "unit": "sweeps/s", "cores": cores, "kind": "port",
            "sample": (f"oracle port of the reference loops (FP32 data, FP64 accumulation as "
                       f"the USE_MP build), {cores} threads, median of {len(per)} samples: "
                       f"stencil phases on {args.cpu_sample} of {cfg['nfunc']} orbitals scaled "
                       f"by N, products on a 128-orbital x 524288-point slab scaled by pairs x "
                       f"points; N x N FP64 algebra not timed; one sample took "
                       f"{first['sample_s']:.1f} s")},
        "e2e": {"value": 1.0 / sec, "unit": "sweeps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if aw:
        line["cpu_baseline"]["as_written"] = aw
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------- GPU leg
def run_gpu(args, cfg):
    import torch
    import torch.distributed as dist
    from mgmol_gb300 import capi, synth
    from mgmol_gb300.sweep import OrbitalSweep, vcycle_bytes

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    capi.load()

    n = cfg["n"]
    ll = tuple(x * cfg["h"] for x in n)
    N = cfg["nfunc"]
    mode = args.mode
    dt = torch.float64 if mode == "plain" else torch.float32
    gemm = {"fp64": capi.GEMM_FP64, "fp32": capi.GEMM_FP32, "tf32": capi.GEMM_TF32,
            "bf16x3": capi.GEMM_BF16X3, "fp16x3": capi.GEMM_FP16X3}[args.gemm if mode == "mixed" else "fp64"]
    ctx = capi.Context(n, ll)
    # replicas only: every rank runs the same workload on its own GPU
    psi, _, _ = synth.gaussian_orbitals_device(n, ll, N, cfg["seed"] + rank, dt)
    V = synth.gaussian_wells_device(n, ll, cfg["wells"], cfg["seed"])
    lean = args.lean
    if lean < 0:
        # three full blocks plus the GEMM workspace must fit, else walk the
        # residual / preconditioner in chunks of 128 functions
        free, _ = torch.cuda.mem_get_info()
        block = N * ctx.npts * (8 if mode == "plain" else 4)
        lean = 0 if 3.6 * block < free else 128
    net = None
    if args.precond == "learned":
        # the learned preconditioner, trained during the warm-up sweeps on
        # the (residual, V-cycle correction) pairs they make
        from mgmol_gb300 import learned as lrn
        net = capi.UNet(ctx)
        net.set_params(lrn.init_params(cfg["seed"]))
    sw = OrbitalSweep(ctx, V, N, mode=mode, gemm=gemm, precond_chunk=args.chunk,
                      chunk_funcs=lean, use_matb=args.theta == "b", learned=net,
                      fuse_hpsi=not args.no_fuse_hpsi)
    torch.cuda.synchronize()

    train = {"pairs": 0, "steps": 0, "loss_first": None, "loss_last": None}
    if net is not None:
        sw.use_learned = False
        gen = torch.Generator(device="cpu")
        gen.manual_seed(cfg["seed"])

        def on_pair(res, corr):
            rows = torch.randperm(N, generator=gen)[: args.train_pairs].tolist()
            if not rows:
                return
            for b0 in range(0, len(rows), 4):
                idx = rows[b0:b0 + 4]
                loss = net.train_step(res[idx].contiguous(), corr[idx].contiguous(), 1e-3)
                train["steps"] += 1
                if train["loss_first"] is None:
                    train["loss_first"] = float(loss)
            train["loss_last"] = float(loss)
            train["pairs"] += len(rows)
        sw.on_pair = on_pair
    for _ in range(args.warmup):
        sw.run(psi)
    torch.cuda.synchronize()
    if net is not None:
        sw.on_pair = None
        sw.use_learned = True

    clocks = ClockSampler(local)
    clocks.start()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = capi.launches()
    # CUDA events around every tensor-core product launch, on its stream
    capi.timing_read(capi.TIMING_TC_SPLITK)
    capi.timing_read(capi.TIMING_TC_STORE)
    capi.timing_enable(True)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    start.record()
    for _ in range(args.steps):
        e = sw.run(psi, timed=True)
    stop.record()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches = capi.launches() - l0
    fallbacks_timed = sw.fallbacks
    capi.timing_enable(False)
    tk_ms, tk_n = capi.timing_read(capi.TIMING_TC_SPLITK)
    ts_ms, ts_n = capi.timing_read(capi.TIMING_TC_STORE)
    ms = start.elapsed_time(stop) / args.steps
    clocks.stop()
    phases = sw.phase_ms()
    energy = float(e.cpu()[0])
    ms = slowest_replica_ms(ms, world, "cuda")

    # end to end through the C ABI with host buffers: pinned host orbitals
    # copied in each step, energy and S read back
    e2e = None
    if args.e2e:
        host = torch.empty(psi.shape, dtype=dt, pin_memory=True)
        host.copy_(psi)
        dev = psi  # the device block is overwritten by the upload each step
        s_host = torch.empty((N, N), dtype=torch.float64, pin_memory=True)
        e_host = torch.empty(1, dtype=torch.float64, pin_memory=True)
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        ksteps = args.steps
        for _ in range(ksteps):
            capi.copy(dev, host)   # SM-driven copy of the pinned host block
            ee = sw.run(dev)
            e_host.copy_(ee, non_blocking=True)
            s_host.copy_(sw.S, non_blocking=True)
        t1.record()
        torch.cuda.synchronize()
        ms_e2e = slowest_replica_ms(t0.elapsed_time(t1) / ksteps, world, "cuda")
        e2e = {"value": job_sweeps_per_s(ms_e2e, world), "unit": "sweeps/s",
               "h2d_bytes_per_step": int(host.numel() * host.element_size()),
               "d2h_bytes_per_step": int(8 + N * N * 8), "steps": ksteps}

    # the energy gate: the accurate energy of the final block against the
    # sweep's own, at this workload; and both iterations run to convergence
    # on a small configuration
    echeck = None
    use_matb, sched_chunk = sw.use_matb, sw.chunk
    if args.energy_check and mode == "mixed" and use_matb:
        from mgmol_gb300 import convergence
        V64 = V.to(torch.float64) if V.dtype != torch.float64 else V
        e_sweep = float(sw.run(psi, update=False).cpu()[0])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_acc = convergence.energy_accurate(ctx, V64, psi, chunk=64, hp=sw.hpsi, bp=sw.corr)
        t_acc = time.perf_counter() - t0
        del V64
        echeck = {"workload": {"E_sweep_ha": e_sweep, "E_accurate_ha": e_acc,
                               "sweep_minus_accurate_ha": e_sweep - e_acc,
                               "accurate_evaluation_s": t_acc}}
        del sw, psi
        torch.cuda.empty_cache()
        g = convergence.run((48, 48, 48), 0.35, 32, 8, 1001, tol_ha=1e-8)
        echeck["converged"] = {
            "config": "32 orbitals on 48^3, h=0.35, 8 wells, seed 1001; DFTsolver energy test "
                      "at 1e-8 Ha on both paths",
            "plain_sweeps": g["plain"]["sweeps"], "mixed_sweeps": g["mixed"]["sweeps"],
            "mixed_accurate_evaluations": g["mixed"]["evaluations"],
            "E_plain_ha": g["plain"]["E_ha"], "E_mixed_ha": g["mixed"]["E_ha"],
            "abs_dE_ha": g["mixed"]["abs_dE_vs_plain_ha"],
            "max_abs_dE_same_sweep_ha": g["mixed"]["max_abs_dE_same_sweep_ha"],
            "plain_s": g["plain"]["seconds"], "mixed_s": g["mixed"]["seconds"],
            "converged": bool(g["plain"]["converged"] and g["mixed"]["converged"])}

    if rank != 0:
        return 0
    hbm, bf16, bf16s, peak_kind = _peaks()
    npts = n[0] * n[1] * n[2]
    s = 4 if dt == torch.float32 else 8
    # algorithmic work per sweep phase
    hpsi_bytes = N * npts * 2 * s + npts * s
    # S and B lower triangles including the diagonal, H full
    gram_flops = (2 if use_matb else 1) * N * (N + 1) * npts + 2.0 * N * N * npts
    shares = {k: v / sum(phases.values()) for k, v in phases.items()}
    dominant = max(phases, key=phases.get)
    # the tensor-core kernels themselves (event-timed launches inside the
    # timed sweeps): split-BF16x3 issues 3 bf16 MMAs per algorithmic
    # multiply-add, so "issued" is 3x the algorithmic rate in that mode
    nprod = 3 if (mode == "mixed" and args.gemm in ("bf16x3", "fp16x3")) else 1
    psi_theta_flops = 2.0 * N * N * npts
    kernels = {}
    if tk_n:
        k_ms = tk_ms / args.steps
        kernels["gram_kernel split-K (S, H, B)"] = {
            "launches_per_sweep": tk_n / args.steps, "ms_per_sweep": k_ms,
            "algorithmic_tflops": gram_flops / (k_ms * 1e-3) / 1e12,
            "issued_tflops": nprod * gram_flops / (k_ms * 1e-3) / 1e12}
    if ts_n:
        k_ms = ts_ms / args.steps
        kernels["gram_kernel store (Psi Theta)"] = {
            "launches_per_sweep": ts_n / args.steps, "ms_per_sweep": k_ms,
            "algorithmic_tflops": psi_theta_flops / (k_ms * 1e-3) / 1e12,
            "issued_tflops": nprod * psi_theta_flops / (k_ms * 1e-3) / 1e12}
    if dominant == "gram" and tk_n:
        k_ms = tk_ms / tk_n                       # one launch on average
        per_launch = gram_flops / (tk_n / args.steps)
        achieved = per_launch / (k_ms * 1e-3) / 1e12
        # timed inside a seconds-long loop of sweeps: the sustained peak
        roof = {"kernel": "gram_kernel (tcgen05 split-K: S, H, B)", "bound": "tensor",
                "achieved": achieved, "peak": bf16s, "peak_burst": bf16, "unit": "TFLOP/s",
                "frac": achieved / bf16s,
                "traffic": (SPLITK_DRAM_BYTES_PER_LAUNCH
                            if (cfg["workload"] == CONFIGS["c5"]["workload"] and mode == "mixed"
                                and args.gemm == "bf16x3") else None),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of the nine "
                                  "split-K launches of one sweep, averaged per launch; algorithmic "
                                  f"{SPLITK_ALGO_BYTES_PER_LAUNCH:.3e} B per launch",
                "issued_frac": nprod * achieved / bf16s,
                "algorithmic": f"{gram_flops:.3e} flop per sweep (S{' and B' if use_matb else ''} "
                               f"lower incl. diagonal + H) over {tk_n / args.steps:.0f} launches"}
    elif dominant == "gram":
        achieved = gram_flops / (phases["gram"] * 1e-3) / 1e12
        roof = {"kernel": "gram+hmat phase", "bound": "tensor", "achieved": achieved, "peak": bf16,
                "unit": "TFLOP/s", "frac": achieved / bf16, "traffic": None,
                "algorithmic": f"{gram_flops:.3e} flop per sweep (S{' and B' if use_matb else ''} "
                               f"lower incl. diagonal + H)"}
    elif dominant == "residual":
        rflops = 2.0 * N * N * npts
        achieved = rflops / (phases["residual"] * 1e-3) / 1e12
        roof = {"kernel": "residual (psi theta + B)", "bound": "tensor", "achieved": achieved,
                "peak": bf16, "unit": "TFLOP/s", "frac": achieved / bf16, "traffic": None,
                "algorithmic": f"{rflops:.3e} flop per sweep (psi theta)"}
    elif dominant == "hpsi":
        achieved = hpsi_bytes / (phases["hpsi"] * 1e-3) / 1e9
        roof = {"kernel": "hpsi", "bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "traffic": None,
                "algorithmic": f"{hpsi_bytes:.3e} B per sweep"}
    else:
        pc_bytes = vcycle_bytes(N, npts, s, 2)
        achieved = pc_bytes / (phases["precond"] * 1e-3) / 1e9
        roof = {"kernel": "precond_mg", "bound": "hbm", "achieved": achieved, "peak": hbm,
                "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                "algorithmic": f"{pc_bytes:.3e} B per sweep"}
    roof["peak_kind"] = peak_kind
    line = {
        "metric": METRIC, "value": job_sweeps_per_s(ms, world), "unit": "sweeps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32" if dt == torch.float32 else "f64",
        "data": "synthetic (seeded Gaussian orbitals and wells generated on the device)",
        "config": _config(cfg, args, use_matb=use_matb, chunk=sched_chunk, net=net is not None,
                          world=world),
        "phases_ms": phases, "phase_share": shares, "energy_trace_ry": energy,
        "roofline": roof, "tensor_kernels": kernels, "gpu_launches": launches,
        "clocks": clocks.summary(),
    }
    if net is not None:
        line["learned"] = {"train": train, "fallbacks_per_sweep": fallbacks_timed / args.steps,
                           "functions": N}
    if e2e:
        line["e2e"] = e2e
    if echeck:
        line["energy_check"] = echeck
    if not args.no_cpu:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(cfg, args.cpu_sample).items()
                                if k != "seconds_per_sweep"}
    print(json.dumps(line), flush=True)
    return 0


# ----------------------------------------------------------- per-kernel timing
def _time(fn, warmup, reps):
    import torch
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


def micro(argv=None):
    """Per-kernel timing at a chosen shape (python bench.py --micro OP ...):
    each operation through the C ABI on device-resident seeded inputs,
    --warmup untimed and --reps timed calls between CUDA events on the
    current stream; one JSON line per operation with milliseconds per call
    and the rate on its algorithmic work (flop for the products, bytes for
    the stencil passes)."""
    import torch
    from mgmol_gb300 import capi, synth
    from mgmol_gb300.sweep import vcycle_bytes
    GEMM = {"fp64": capi.GEMM_FP64, "fp32": capi.GEMM_FP32, "tf32": capi.GEMM_TF32,
            "bf16x3": capi.GEMM_BF16X3, "fp16x3": capi.GEMM_FP16X3}
    ap = argparse.ArgumentParser(prog="bench.py --micro")
    ap.add_argument("op", choices=["gram", "hmat", "gram_hmat", "matb", "gram_hmat_matb", "mult",
                                   "residual", "hpsi", "precond", "mgm", "dense", "dense_b",
                                   "dense_parts", "normalize", "mult_reuse", "h2d", "h2d_kernel",
                                   "centers", "all"])
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
        elif op == "centers":
            # the position-matrix diagonal of SpreadsAndCenters: the block read once
            ms = _time(lambda: ctx.sincos_diag(psi), args.warmup, args.reps)
            work, unit = N * npts * s, "GB/s"
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



def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="c5", choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="mixed", choices=["mixed", "plain"])
    ap.add_argument("--gemm", default="bf16x3", choices=["fp32", "tf32", "bf16x3", "fp16x3"])
    ap.add_argument("--chunk", type=int, default=0, help="V-cycle orbital chunk (0 = auto)")
    ap.add_argument("--no-fuse-hpsi", action="store_true",
                    help="H psi as its own pass and its conversion for the H product separate")
    ap.add_argument("--theta", default="b", choices=["b", "gram"],
                    help="b: theta = B^-1 H as the reference for a Mehrstellen operator; "
                         "gram: theta = S^-1 H")
    ap.add_argument("--lean", type=int, default=-1,
                    help="residual / preconditioner column chunk (0 = full blocks, -1 = auto)")
    ap.add_argument("--cpu-sample", type=int, default=32,
                    help="orbitals of the timed CPU sample of the linear phases")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precond", default="vcycle", choices=["vcycle", "learned"],
                    help="learned: the U-Net preconditioner with V-cycle fallback, trained "
                         "during the warm-up sweeps")
    ap.add_argument("--train-pairs", type=int, default=256,
                    help="pairs per warm-up sweep the learned preconditioner trains on")
    ap.add_argument("--no-e2e", dest="e2e", action="store_false")
    ap.add_argument("--no-energy-check", dest="energy_check", action="store_false",
                    help="skip the accurate energy of the final block and the small "
                         "converged comparison of the two paths")
    ap.add_argument("--as-written", action="store_true",
                    help="reference arm: also time the stencil phases on one thread")
    if len(sys.argv) > 1 and sys.argv[1] == "--micro":
        return micro(sys.argv[2:])
    args = ap.parse_args()
    cfg = CONFIGS[args.config]
    if args.impl == "reference":
        return run_reference(args, cfg)
    return run_gpu(args, cfg)


if __name__ == "__main__":
    sys.exit(main())
