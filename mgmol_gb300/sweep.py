"""One orbital sweep of MGmol's hot path, composed from the C-ABI kernels.

A sweep over the N orbitals of a block Psi is one ABPG step
(ABPG<T>::updateWF / update_states, src/ABPG.cc:37-140):
  1. H psi       (Hamiltonian<T>::applyLocal, src/Hamiltonian.cc:85-159);
  2. S, H        (LocGridOrbitals::computeGram / Hamiltonian::addHlocalij,
                  src/LocGridOrbitals.cc:1504-1738, src/Hamiltonian.cc:227-239);
  3. Cholesky of S, S^-1, the energy trace tr(S^-1 H) and theta = S^-1 H in
     FP64 (GramMatrix::updateLS / computeInverse, src/GramMatrix.cc:75-191,
     ProjectedMatrices::getEigSum / updateTheta, src/ProjectedMatrices.cc:
     550-566, src/ProjectedMatrices.h:218-225);
  4. the residual res = B(psi) theta - H psi (MGmol::computeResidualUsingHPhi,
     src/MGmol.cc:1227-1290), written over H psi;
  5. one V-cycle preconditioner application on the residual
     (OrbitalsPreconditioning<T>::precond_mg, src/OrbitalsPreconditioning.cc:86-117);
  6. psi += alpha * P(res), alpha = 0.5 * precond_factor (the non-accelerated
     branch of ABPG<T>::update_states).
Every step runs on the GPU through mgmol_gb300.capi; the only host work is
the launch sequence and the Cholesky status read-back.

Two precision modes:
  "plain": FP64 orbitals, FP64 stencils, FP64 products, FP64 V-cycle;
  "mixed": FP32 orbitals and stencils with an FP32 potential, Gram / H and
           Psi Theta in the requested GEMM mode, FP32 V-cycle; FP64
           Cholesky / inverse / trace / theta in both.
"""
import torch

from . import capi


class OrbitalSweep:
    def __init__(self, ctx, V, nfunc, mode="mixed", gemm=None, lap_type=capi.LAP_MEHR4,
                 maxlevels=2, gamma=None, precond_chunk=0, precond_factor=1.0,
                 device="cuda"):
        self.ctx = ctx
        self.mode = mode
        self.lap_type = lap_type
        self.maxlevels = maxlevels
        self.nfunc = nfunc
        self.dtype = torch.float64 if mode == "plain" else torch.float32
        self.gemm = gemm if gemm is not None else (capi.GEMM_FP64 if mode == "plain" else capi.GEMM_FP32)
        self.V = V.to(device=device, dtype=self.dtype).contiguous()
        npts = ctx.npts
        self.hpsi = torch.empty((nfunc, npts), dtype=self.dtype, device=device)
        self.corr = torch.empty((nfunc, npts), dtype=self.dtype, device=device)
        self.S = torch.empty((nfunc, nfunc), dtype=torch.float64, device=device)
        self.Hm = torch.empty((nfunc, nfunc), dtype=torch.float64, device=device)
        self.precond_chunk = precond_chunk
        self.alpha = 0.5 * precond_factor
        self.theta = None
        if gamma is None:
            vmax = float(self.V.max())
            gamma = ctx.gamma(lap_type, maxlevels, vmax, float(self.V.min()))
        self.gamma = gamma
        self.events = {}

    def _ev(self, name):
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        self.events.setdefault(name, []).append(e)

    def run(self, psi, timed=False, update=True):
        """One sweep; psi is updated in place (unless update is False).
        Returns the device tensor holding tr(S^-1 H) (Ry)."""
        ctx = self.ctx
        if timed:
            self._ev("hpsi0")
        ctx.hpsi(psi, self.V, self.lap_type, True, out=self.hpsi)
        if timed:
            self._ev("gram0")
        ctx.gram_hmat(psi, self.hpsi, self.gemm, S=self.S, H=self.Hm)
        if timed:
            self._ev("dense0")
        L = ctx.cholesky(self.S)
        Sinv = ctx.inverse_from_cholesky(L)
        # Hm holds H column-major; the matrix calls want the row-major view
        e = ctx.trace_prod(self.Hm.T, Sinv.contiguous())
        self.theta = ctx.theta(Sinv, self.Hm.T)
        if timed:
            self._ev("residual0")
        ctx.residual(psi, self.hpsi, self.theta, mode=self.gemm,
                     apply_B=(self.lap_type == capi.LAP_MEHR4), work=self.corr, out=self.hpsi)
        if timed:
            self._ev("precond0")
        ctx.precond_mg(self.hpsi, self.lap_type, self.maxlevels, self.gamma,
                       chunk=self.precond_chunk, out=self.corr)
        if timed:
            self._ev("update0")
        if update:
            capi.axpy(self.alpha, self.corr, psi)
        if timed:
            self._ev("end")
        return e

    def phase_ms(self):
        """Average milliseconds per phase over the timed sweeps."""
        torch.cuda.synchronize()
        names = ["hpsi0", "gram0", "dense0", "residual0", "precond0", "update0", "end"]
        out = {}
        k = len(self.events.get("end", []))
        for a, b in zip(names[:-1], names[1:]):
            tot = sum(self.events[a][i].elapsed_time(self.events[b][i]) for i in range(k))
            out[a[:-1]] = tot / max(k, 1)
        return out
