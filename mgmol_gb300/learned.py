"""The learned preconditioner: training of the library's U-Net
(mgx_unet_*, csrc/mgx_learn.cu) on (residual, V-cycle correction) pairs
that the library's own V-cycle produces, and its use inside a block
preconditioned-gradient iteration with the V-cycle as per-function
fallback (mgx_precond_learned).

The iteration is the preconditioned gradient method on the block of
systems that the orbital V-cycle preconditions (Preconditioning<T>::mg,
src/Preconditioning.cc:155-216, with the fine operator A of lap_type,
periodic, right-hand sides of zero mean):

    r = f - A x ;  x += omega P(r)

with P the plain V-cycle (mgx_precond_mg, started from gamma r as
OrbitalsPreconditioning::precond_mg does) or the learned correction, and
omega the step (1; ABPG's 0.5 * precond_factor is 0.5).  x and
r are FP64, so that |r| can fall to 1e-6 |f|; P works on the FP32 residual
like the reference's float preconditioner.

Training pairs come from the plain iteration itself: every residual it
forms and the V-cycle's correction of it.  They are consumed as they are
made (a few Adam steps per batch of pairs) instead of being stored.

CLI (one JSON line):
    python -m mgmol_gb300.learned --grid 128 128 128 --h 0.3 --train-funcs 512 \\
        --train-iters 40 --test-funcs 64 --lap 4
"""
import argparse
import json
import sys
import time

import numpy as np
import torch

from . import capi, synth


def rhs_block(n, ll, nfunc, seed):
    """Zero-mean right-hand sides: the seeded Gaussian orbitals of the
    workload, minus their means (FP64, device)."""
    f, _, _ = synth.gaussian_orbitals_device(n, ll, nfunc, seed, torch.float64)
    f -= f.mean(dim=1, keepdim=True)
    return f


def init_params(seed):
    """He-normal initial weights (fan-in 27 * cin) in the parameter order of
    mgx_unet (the six 3x3x3 kernels, [out][in][x][y][z])."""
    rng = np.random.default_rng(seed)
    out = []
    for ci, co in ((1, 16), (16, 32), (32, 64), (64, 32), (32, 16), (16, 1)):
        out.append(rng.standard_normal(ci * co * 27) * np.sqrt(2.0 / (27 * ci)))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == capi.UNET_PARAMS
    return p


class BlockSolver:
    """The block preconditioned-gradient iteration for A x = f."""

    def __init__(self, ctx, lap_type, maxlevels, gamma, chunk=0, omega=1.0):
        self.ctx = ctx
        self.lap = lap_type
        self.maxlevels = maxlevels
        self.gamma = gamma
        self.chunk = chunk
        self.omega = omega

    def vcycle(self, r32, out=None):
        return self.ctx.precond_mg(r32, self.lap, self.maxlevels, self.gamma, chunk=self.chunk,
                                   out=out)

    def run(self, f, precond, tol=1e-6, maxit=200, on_pair=None):
        """Iterates until every |r_j| <= tol |f_j| or maxit steps.  precond(r32)
        returns the FP32 correction; on_pair(r32, c) sees each pair.  Returns
        (iterations per function (maxit + 1 where not reached), history of
        the largest relative residual)."""
        nf = f.shape[0]
        fn = torch.linalg.vector_norm(f, dim=1)
        x = torch.zeros_like(f)
        r = f.clone()
        its = np.full(nf, maxit + 1)
        hist = []
        r32 = torch.empty(f.shape, dtype=torch.float32, device=f.device)
        for k in range(maxit + 1):
            rel = (torch.linalg.vector_norm(r, dim=1) / fn).cpu().numpy()
            hist.append(float(rel.max()))
            newly = (rel <= tol) & (its > maxit)
            its[newly] = k
            if (its <= maxit).all() or k == maxit:
                break
            r32.copy_(r)
            c = precond(r32)
            if on_pair is not None:
                on_pair(r32, c)
            x.add_(c.double(), alpha=self.omega)
            self.ctx.fd_apply(x, self.lap, out=r)
            torch.sub(f, r, out=r)
        return its, hist


class Learned:
    """The learned correction with the V-cycle as fallback, as a precond
    callable for BlockSolver.run."""

    def __init__(self, solver, net, mode=capi.LEARNED_WARM, refresh=False):
        self.s = solver
        self.net = net
        self.mode = mode | (capi.LEARNED_REFRESH if refresh else 0)
        self.tau = None
        self.fallbacks = 0
        self.calls = 0
        self.functions = 0

    def __call__(self, r32):
        nf = r32.shape[0]
        if self.tau is None or self.tau.size != nf:
            self.tau = np.zeros(nf)
        out, red, nfb = capi.precond_learned(self.s.ctx, self.net, r32, self.s.lap,
                                             self.s.maxlevels, self.s.gamma, self.tau,
                                             mode=self.mode, chunk=self.s.chunk)
        self.fallbacks += nfb
        self.calls += 1
        self.functions += nf
        return out


class Trainer:
    """Adam on minibatches of the pairs handed to it."""

    def __init__(self, net, lr=1e-3, batch=4, steps_per_pair_batch=1):
        self.net = net
        self.lr = lr
        self.batch = batch
        self.reps = steps_per_pair_batch
        self.losses = []
        self.steps = 0

    def __call__(self, x, y):
        nf = x.shape[0]
        perm = torch.randperm(nf, device=x.device)
        for _ in range(self.reps):
            for b0 in range(0, nf, self.batch):
                idx = perm[b0:b0 + self.batch]
                xb = x[idx].contiguous()
                yb = y[idx].contiguous()
                loss = self.net.train_step(xb, yb, self.lr)
                self.steps += 1
                if self.steps % 16 == 1:
                    self.losses.append(float(loss))


def train_on_iteration(solver, net, f, iters, lr, batch, reps=1):
    """Runs the plain iteration for `iters` steps on f and trains the net on
    every (residual, V-cycle correction) pair it makes."""
    tr = Trainer(net, lr=lr, batch=batch, steps_per_pair_batch=reps)
    solver.run(f, solver.vcycle, tol=0.0, maxit=iters, on_pair=tr)
    return tr


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--grid", type=int, nargs=3, default=[128, 128, 128])
    ap.add_argument("--h", type=float, default=0.3)
    ap.add_argument("--lap", type=int, default=4)
    ap.add_argument("--maxlevels", type=int, default=2)
    ap.add_argument("--train-funcs", type=int, default=512)
    ap.add_argument("--train-chunk", type=int, default=64,
                    help="functions iterated together while generating pairs")
    ap.add_argument("--train-iters", type=int, default=40)
    ap.add_argument("--batch", type=int, default=4)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--test-funcs", type=int, default=64)
    ap.add_argument("--tol", type=float, default=1e-6)
    ap.add_argument("--maxit", type=int, default=300)
    ap.add_argument("--omega", type=float, default=1.0)
    ap.add_argument("--mode", choices=["warm", "replace"], default="warm")
    ap.add_argument("--refresh", action="store_true",
                    help="run the V-cycle on every function at every step (exact fallback)")
    ap.add_argument("--seed", type=int, default=1004)
    ap.add_argument("--save", default=None, help="write the trained weights (.npy)")
    ap.add_argument("--load", default=None, help="start from these weights (.npy)")
    a = ap.parse_args(argv)

    n = tuple(a.grid)
    ll = tuple(x * a.h for x in n)
    ctx = capi.Context(n, ll)
    gamma = ctx.gamma(a.lap, a.maxlevels, 0.0, 0.0)
    solver = BlockSolver(ctx, a.lap, a.maxlevels, gamma, omega=a.omega)
    net = capi.UNet(ctx)
    net.set_params(np.load(a.load) if a.load else init_params(a.seed))

    # training on the plain iteration's pairs, generated chunk by chunk
    t0 = time.time()
    pairs = 0
    losses = []
    for f0 in range(0, a.train_funcs, a.train_chunk):
        nc = min(a.train_chunk, a.train_funcs - f0)
        f = rhs_block(n, ll, nc, a.seed + 100 + f0)
        tr = train_on_iteration(solver, net, f, a.train_iters, a.lr, a.batch)
        losses += tr.losses
        pairs += nc * a.train_iters
        del f
    torch.cuda.synchronize()
    t_train = time.time() - t0
    if a.save:
        np.save(a.save, net.get_params().cpu().numpy())

    # the test block: plain against learned (warm start, fallback)
    f = rhs_block(n, ll, a.test_funcs, a.seed + 200)
    res = {}
    mode = capi.LEARNED_WARM if a.mode == "warm" else capi.LEARNED_REPLACE
    for name, pc in (("plain", solver.vcycle),
                     ("learned", Learned(solver, net, mode=mode, refresh=a.refresh))):
        torch.cuda.synchronize()
        t1 = time.time()
        its, hist = solver.run(f, pc, tol=a.tol, maxit=a.maxit)
        torch.cuda.synchronize()
        dt = time.time() - t1
        res[name] = {"iterations_median": float(np.median(its)), "iterations_max": int(its.max()),
                     "reached": int((its <= a.maxit).sum()), "seconds": dt,
                     "final_residual": hist[-1]}
        if name == "learned":
            res[name]["fallbacks"] = pc.fallbacks
            res[name]["function_calls"] = pc.functions

    # time of one application to the test block
    r32 = f.float()
    for name, fn in (("vcycle", lambda: solver.vcycle(r32)), ("net", lambda: net.forward(r32))):
        fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(3):
            fn()
        e1.record()
        torch.cuda.synchronize()
        res[f"ms_{name}"] = e0.elapsed_time(e1) / 3
    out = {"grid": list(n), "h": a.h, "lap_type": a.lap, "omega": a.omega, "mode": a.mode,
           "refresh": a.refresh, "train_funcs": a.train_funcs,
           "pairs": pairs, "train_seconds": t_train, "loss_first": losses[0] if losses else None,
           "loss_last": losses[-1] if losses else None, "test_funcs": a.test_funcs, "tol": a.tol,
           **res}
    print(json.dumps(out))
    return out


if __name__ == "__main__":
    sys.exit(0 if main() else 1)
