/*
 * ORACLE PINNING DRIVER -- TEST INFRASTRUCTURE ONLY.
 *
 * Runs the reference's own AndersonMix<T>::update (src/AndersonMix.cc,
 * compiled unmodified by oracle/build_ref.sh with TESTING, once per storage
 * type, against the block type of oracle/shim_anderson/Solution.h) on a
 * given sequence of residual blocks, so that the oracle restatement in
 * oracle/mgx_oracle.cpp and the GPU implementation can be checked against
 * it.  Nothing here is part of the product.
 */
#include <algorithm>
#include <ostream>
#include <vector>

#include "AndersonMix.h"
#include "Solution.h"

namespace
{
/* nsteps updates of AndersonMix(m, beta, x) with residuals res_s =
 * fscale * f_s (the res.scal(alpha) of ABPG<T>::update_states); the
 * dot-product weights invS(k, k) of step s are invs[s * nfunc + k].
 * xs_out[s] receives x after update s. */
template <typename S, typename T>
int anderson_run(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const T* x0, int nsteps, const T* fseq, double fscale, T* xs_out)
{
    S::nfunc_ = nfunc;
    S::npts_  = npts;
    S::vel_   = vel;
    const size_t nb = (size_t)nfunc * npts;
    S x;
    std::copy(x0, x0 + nb, x.data());
    AndersonMix<S> mix(m, beta, x);
    S work;
    std::ostream quiet(nullptr);
    for (int s = 0; s < nsteps; s++)
    {
        S::invs_diag_.assign(invs + (size_t)s * nfunc, invs + (size_t)(s + 1) * nfunc);
        S f;
        std::copy(fseq + s * nb, fseq + (s + 1) * nb, f.data());
        f.scal(fscale);
        mix.update(f, work, quiet, false);
        std::copy(x.data(), x.data() + nb, xs_out + s * nb);
    }
    return 0;
}
} // namespace

extern "C" {
int ref_anderson_f(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const float* x0, int nsteps, const float* fseq, double fscale, float* xs_out)
{
    return anderson_run<SolutionF>(npts, nfunc, m, beta, vel, invs, x0, nsteps, fseq, fscale,
        xs_out);
}
int ref_anderson_d(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const double* x0, int nsteps, const double* fseq, double fscale, double* xs_out)
{
    return anderson_run<SolutionD>(npts, nfunc, m, beta, vel, invs, x0, nsteps, fseq, fscale,
        xs_out);
}
}
