"""One orbital sweep of MGmol's hot path, composed from the C-ABI kernels.

A sweep over the N orbitals of a block Psi is one iteration of the
DFTsolver loop with the ABPG stepper (src/DFTsolver.cc:262-400,
ABPG<T>::updateWF / update_states, src/ABPG.cc:37-140), for a Mehrstellen
operator (lap_type 0, ProjectedMatricesMehrstellen, src/MGmol.cc:243-254):
  0. normalize Psi (LocGridOrbitals::normalize, src/LocGridOrbitals.cc:
     2230-2311, which the reference runs after every update);
  1. H psi       (Hamiltonian<T>::applyLocal, src/Hamiltonian.cc:85-159);
  2. S, H, B     (LocGridOrbitals::computeGram / Hamiltonian::addHlocalij /
                  LocGridOrbitals::computeMatB, src/LocGridOrbitals.cc:
                  1428-1738, src/Hamiltonian.cc:227-239);
  3. FP64 dense algebra: Cholesky and inverse of S (GramMatrix::updateLS /
     computeInverse, src/GramMatrix.cc:75-191); Cholesky of B and
     theta = B^-1 H (ProjectedMatricesMehrstellen::computeInvB /
     updateTheta); HB = sym(S theta) (updateHB) and the energy
     tr(HB S^-1) (ProjectedMatrices::getEigSum, src/ProjectedMatrices.cc:
     550-566).  For the other operators (and, with use_matb=False, for the
     Mehrstellen operator too) theta = S^-1 H and HB = H
     (ProjectedMatrices::updateTheta / setHB2H);
  4. the residual res = B(psi) theta - H psi (MGmol::computeResidualUsingHPhi,
     src/MGmol.cc:1227-1290), written over H psi;
  5. one V-cycle preconditioner application on the residual
     (OrbitalsPreconditioning<T>::precond_mg, src/OrbitalsPreconditioning.cc:86-117);
  6. psi += alpha * P(res), alpha = 0.5 * precond_factor (the non-accelerated
     branch of ABPG<T>::update_states).

With the fused update (the default) step 0 costs no pass over the block:
the step runs on the block as it came out of the previous update, and the
normalization factors d_i = S(i,i)^-1/2 of that block (the diagonal of its
own Gram matrix) scale the update instead, psi_i <- d_i (psi_i + alpha
P(res)_i).  Every quantity of the step is covariant under that column
scaling (theta -> D^-1 theta D, res -> res D, tr(HB S^-1) unchanged), so the
result is the reference's normalize-then-step to rounding; the block handed
back is the reference's block after update_states, before its normalize.
The unfused schedules call mgx_normalize explicitly first.

Every step runs on the GPU through mgmol_gb300.capi; the only host work is
the launch sequence and the Cholesky status read-back.

Two precision modes:
  "plain": FP64 orbitals, FP64 stencils, FP64 products, FP64 V-cycle;
  "mixed": FP32 orbitals and stencils with an FP32 potential, Gram / H / B
           and Psi Theta in the requested GEMM mode, FP32 V-cycle; FP64
           Cholesky / inverse / trace / theta in both.
"""
import numpy as np
import torch

from . import capi


def vcycle_bytes(N, npts, s, maxlevels):
    """Minimal HBM bytes of one V-cycle application on N functions of npts
    points (element size s), following the kernel schedule: level 0 -- first
    sweep from f (read f, write v), second pre-sweep (read v, f; write v, w),
    restriction (read w, write the coarse rhs), prolongation-correction (read
    coarse, read and write v), two post-sweeps (read v, f; write v); coarse
    levels add a zero fill of v and 4 sweeps on the coarsest grid."""
    total = 0.0
    for l in range(maxlevels + 1):
        P = N * npts / 8 ** l
        if l == maxlevels:
            total += P * s * (1 + 4 * 3)
            continue
        first = 2 if l == 0 else 1 + 3       # level 0 starts from f; others zero-fill
        total += P * s * (first + 4 + 1.125 + 2.125 + 2 * 3)
    return total



class OrbitalSweep:
    """One ABPG step per run() on a device block of orbitals.

    chunk_funcs > 0 selects the memory-lean schedule: the residual and the
    preconditioner walk the block in chunks of that many output functions
    (mgx_residual_cols), each chunk's correction is parked in its slice of
    the H psi block, and one update closes the step.  The block then needs
    psi, H psi and two chunk buffers instead of three full blocks, which is
    what lets the FP64 path hold 2048 orbitals on 192^3 in one GPU."""

    PHASES = ("normalize", "hpsi", "gram", "dense", "residual", "precond", "update")

    def __init__(self, ctx, V, nfunc, mode="mixed", gemm=None, lap_type=capi.LAP_MEHR4,
                 maxlevels=2, gamma=None, precond_chunk=0, precond_factor=1.0,
                 chunk_funcs=0, fuse_update=True, use_matb=True, anderson_m=0,
                 anderson_beta=1.0, learned=None, learned_mode=capi.LEARNED_WARM,
                 fuse_hpsi=True, device="cuda"):
        self.ctx = ctx
        self.mode = mode
        self.lap_type = lap_type
        self.maxlevels = maxlevels
        self.nfunc = nfunc
        self.dtype = torch.float64 if mode == "plain" else torch.float32
        self.gemm = gemm if gemm is not None else (capi.GEMM_FP64 if mode == "plain" else capi.GEMM_FP32)
        self.V = V.to(device=device, dtype=self.dtype).contiguous()
        npts = ctx.npts
        self.chunk = int(chunk_funcs) if chunk_funcs and chunk_funcs < nfunc else 0
        self.hpsi = torch.empty((nfunc, npts), dtype=self.dtype, device=device)
        if self.chunk:
            self.corr = torch.empty((self.chunk, npts), dtype=self.dtype, device=device)
            self.work = torch.empty((self.chunk, npts), dtype=self.dtype, device=device)
        else:
            self.corr = torch.empty((nfunc, npts), dtype=self.dtype, device=device)
            self.work = None
        self.S = torch.empty((nfunc, nfunc), dtype=torch.float64, device=device)
        self.Hm = torch.empty((nfunc, nfunc), dtype=torch.float64, device=device)
        # Mehrstellen: the residual applies B; with use_matb (the reference's
        # ProjectedMatricesMehrstellen) theta = B^-1 H with the matrix B of the
        # generalized eigenproblem, else theta = S^-1 H (ProjectedMatrices)
        self.mehr = lap_type == capi.LAP_MEHR4
        self.use_matb = self.mehr and bool(use_matb)
        self.Bm = torch.empty((nfunc, nfunc), dtype=torch.float64, device=device) \
            if self.use_matb else None
        # H psi made inside the H product (its chunks written straight into
        # the product's split-BF16x3 operand planes): FP32 Mehrstellen with
        # B(V psi) and the B matrix, split-BF16x3 products
        self.fuse_hpsi = bool(fuse_hpsi) and mode == "mixed" and self.use_matb \
            and self.gemm == capi.GEMM_BF16X3
        self.dscale = torch.empty(nfunc, dtype=torch.float64, device=device)
        self.diagS = torch.empty(nfunc, dtype=torch.float64, device=device)
        self.precond_chunk = precond_chunk
        # the update psi += alpha P(res) inside the last fine-level sweep
        # (full-block schedule without Anderson mixing only; the chunked one
        # defers the update)
        self.anderson_m = int(anderson_m)
        # the learned preconditioner (a capi.UNet) in place of the V-cycle,
        # the V-cycle as per-function fallback (mgx_precond_learned); off
        # while use_learned is False, when on_pair(res, corr), if set, sees
        # every residual block and its V-cycle correction (training)
        self.learned = learned
        self.learned_mode = learned_mode
        self.use_learned = learned is not None
        self.on_pair = None
        self.tau = np.zeros(nfunc)
        self.fallbacks = 0
        self.fuse_update = (bool(fuse_update) and not self.chunk and self.anderson_m == 0
                            and learned is None)
        self.anderson_beta = float(anderson_beta)
        self.mixer = None
        # the S side of the dense algebra (Cholesky and inverse of S, HB and
        # the energy) runs on a second stream with its own context, next to
        # the critical path theta = B^-1 H -> residual -> V-cycle
        # (high priority: its blocks are scheduled as soon as SMs free up
        # beside the residual and the V-cycle, instead of after them)
        self.side = torch.cuda.Stream(device=device, priority=-1) if self.use_matb else None
        self.side_after_theta = True
        self.sctx = capi.Context(ctx.n, ctx.ll) if self.use_matb else None
        self.info = torch.zeros(2, dtype=torch.int32, device=device)
        self.Sinv = None
        # psi does not change between the Gram products and Psi Theta: the
        # residual reads the Gram's BF16 conversion of psi
        ctx.set_reuse_conversion(True)
        self.alpha = 0.5 * precond_factor
        self.theta = None
        if gamma is None:
            vmax = float(self.V.max())
            gamma = ctx.gamma(lap_type, maxlevels, vmax, float(self.V.min()))
        self.gamma = gamma
        self.marks = []
        self.timed_runs = 0

    def _mark(self, timed, phase=None):
        """Closes the open phase interval and opens `phase` (None: close only)."""
        if not timed:
            return
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        if self.marks and self.marks[-1][2] is None:
            self.marks[-1][2] = e
        if phase is not None:
            self.marks.append([phase, e, None])

    def run(self, psi, timed=False, update=True, accelerate=None):
        """One sweep; psi is updated in place (unless update is False).
        With anderson_m > 0 the update is the Anderson extrapolation
        (accelerate, default on) or the plain step (accelerate False, the
        history untouched), as ABPG<T>::update_states switches.
        Returns the device tensor holding the energy tr(HB S^-1) (Ry)."""
        ctx = self.ctx
        lazy = self.fuse_update and update
        if accelerate is None:
            accelerate = self.anderson_m > 0
        if accelerate and self.mixer is None:
            if self.anderson_m <= 0:
                raise ValueError("acceleration needs anderson_m > 0")
            self.mixer = capi.Anderson(ctx, self.anderson_m, self.anderson_beta, psi)
        if not lazy:
            self._mark(timed, "normalize")
            ctx.normalize(psi, diag=self.diagS)
        if self.fuse_hpsi:
            # H psi inside the H product: its time counts in the gram phase
            self._mark(timed, "gram")
            ctx.hpsi_gram_hmat_matb(psi, self.V, self.hpsi, self.gemm, S=self.S, H=self.Hm,
                                    B=self.Bm, work=self.work if self.chunk else self.corr)
        else:
            self._mark(timed, "hpsi")
            ctx.hpsi(psi, self.V, self.lap_type, True, out=self.hpsi)
            self._mark(timed, "gram")
            if self.use_matb:
                ctx.gram_hmat_matb(psi, self.hpsi, self.gemm, S=self.S, H=self.Hm, B=self.Bm,
                                   work=self.work if self.chunk else self.corr)
            else:
                ctx.gram_hmat(psi, self.hpsi, self.gemm, S=self.S, H=self.Hm)
        self._mark(timed, "dense")
        # Hm holds H column-major; the matrix calls want the row-major view
        H = self.Hm.T
        if self.use_matb:
            main = torch.cuda.current_stream()
            self.side.wait_stream(main)
            # computeInvB + updateTheta: theta = B^-1 H from the factor of B
            self.theta, _ = ctx.theta_from_cholesky(ctx.cholesky(self.Bm, info=self.info[0:1]), H)
            theta_done = torch.cuda.Event()
            theta_done.record(main)
            with torch.cuda.stream(self.side):
                # computeGramAndInvS, updateHB and getEigSum beside the
                # residual and the V-cycle; started after theta, so that the
                # FP64 work of the critical path does not share the FP64
                # units with it (side_after_theta False: beside theta too)
                if self.side_after_theta:
                    self.side.wait_event(theta_done)
                L = self.sctx.cholesky(self.S, info=self.info[1:2])
                self.Sinv = self.sctx.inverse_from_cholesky(L).contiguous()
                self.side.wait_event(theta_done)
                e = self.sctx.trace_prod(self.sctx.update_hb(self.S, self.theta), self.Sinv)
        else:
            L = ctx.cholesky(self.S)
            self.Sinv = ctx.inverse_from_cholesky(L).contiguous()
            e = ctx.trace_prod(H, self.Sinv)
            self.theta = ctx.theta(self.Sinv, H)
        Sinv = self.Sinv
        if lazy:
            ctx.normalize_scales(self.S, out=self.dscale)
        if not self.chunk:
            self._mark(timed, "residual")
            ctx.residual(psi, self.hpsi, self.theta, mode=self.gemm, apply_B=self.mehr,
                         work=self.corr, out=self.hpsi)
            self._mark(timed, "precond")
            if lazy:
                ctx.precond_update(self.hpsi, psi, self.alpha, self.lap_type, self.maxlevels,
                                   self.gamma, chunk=self.precond_chunk, work=self.corr,
                                   psi_scale=self.dscale)
                self._mark(timed, "update")
            elif self.use_learned:
                _, _, nfb = capi.precond_learned(ctx, self.learned, self.hpsi, self.lap_type,
                                                 self.maxlevels, self.gamma, self.tau,
                                                 mode=self.learned_mode,
                                                 chunk=self.precond_chunk, out=self.corr)
                self.fallbacks += nfb
                self._mark(timed, "update")
                if update:
                    self._update(psi, self.corr, Sinv, accelerate)
            else:
                ctx.precond_mg(self.hpsi, self.lap_type, self.maxlevels, self.gamma,
                               chunk=self.precond_chunk, out=self.corr)
                if self.on_pair is not None:
                    self.on_pair(self.hpsi, self.corr)
                self._mark(timed, "update")
                if update:
                    self._update(psi, self.corr, Sinv, accelerate)
        else:
            # theta.T is the column-major buffer: row j holds column j
            thc = self.theta.T
            for j0 in range(0, self.nfunc, self.chunk):
                j1 = min(self.nfunc, j0 + self.chunk)
                hc = self.hpsi[j0:j1]
                cb = self.corr[: j1 - j0]
                self._mark(timed, "residual")
                ctx.residual_cols(psi, hc, thc[j0:j1], mode=self.gemm, apply_B=self.mehr,
                                  work=self.work[: j1 - j0], out=hc)
                self._mark(timed, "precond")
                ctx.precond_mg(hc, self.lap_type, self.maxlevels, self.gamma,
                               chunk=self.precond_chunk, out=cb)
                hc.copy_(cb)
            self._mark(timed, "update")
            if update:
                self._update(psi, self.hpsi, Sinv, accelerate)
        if self.use_matb:
            torch.cuda.current_stream().wait_stream(self.side)
            if int(self.info.max()) != 0:
                which = "B" if int(self.info[0]) else "S"
                raise capi.MgxError(capi.MGX_NOT_SPD, f"Cholesky of {which}: leading minor "
                                    f"{int(self.info.max())} not positive")
        self._mark(timed)
        if timed:
            self.timed_runs += 1
        return e

    def _update(self, psi, corr, Sinv, accelerate):
        """psi += alpha corr, or the Anderson step with the residual alpha corr
        and the dot-product weights of S^-1 (AndersonMix<T>::update)."""
        if accelerate:
            if self.side is not None:
                torch.cuda.current_stream().wait_stream(self.side)
            self.last_mix = self.mixer.update(psi, corr, self.alpha, Sinv)
        else:
            capi.axpy(self.alpha, corr, psi)

    def restart_mixing(self):
        """AndersonMix<T>::restart (ABPG's restartMixing)."""
        if self.mixer is not None:
            self.mixer.restart()

    def correction(self):
        """P(res) of the last run (the block psi was moved along); not kept
        when the update is fused into the preconditioner."""
        if self.fuse_update:
            raise RuntimeError("the fused update does not keep P(res)")
        return self.hpsi if self.chunk else self.corr

    def phase_ms(self):
        """Average milliseconds per phase over the timed sweeps."""
        torch.cuda.synchronize()
        out = {p: 0.0 for p in self.PHASES}
        for phase, a, b in self.marks:
            out[phase] += a.elapsed_time(b)
        k = max(self.timed_runs, 1)
        return {p: v / k for p, v in out.items()}
