// pb::Mgm / pb::Vcycle (src/pb/Mgm.h:20-112, src/pb/Vcycle.h:28-249): the
// multigrid Poisson solver on one field, one task, periodic boundaries.
//
// The cycle runs on the stencil engine and the transfer kernels of the
// orbital preconditioner:
//   - a Jacobi sweep is the OP_JACOBI plane kernel (x <- x - jf (A x - f),
//     ping-pong buffers); with jf = 0 the same kernel yields the residual
//     A x - f that Vcycle recomputes after pre-smoothing;
//   - restriction and prolongation-subtraction are restrict_kernel and
//     prolong_kernel (MODE 1);
//   - the residual norms Mgm tests (sqrt(sum r^2 * h^3), GridFunc::norm2,
//     src/pb/GridFunc.cc:2856-2861) are deterministic two-pass device
//     reductions read back once per outer iteration.
// Mgm feeds the cycle the residual rhs - A vh; this implementation passes
// its negative A vh - rhs (the kernel's natural output) and subtracts the
// correction instead of adding it.  Every operation of the cycle is linear
// and commutes exactly with negation, so the iterates are unchanged.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{
int restrict_launch(int, const Level&, const void*, size_t, void*, size_t, int,
    const MaskDev&, cudaStream_t);
int prolong_launch(int, int, const Level&, const void*, size_t, void*, size_t,
    int, const MaskDev&, cudaStream_t);

constexpr int NORM_BLOCKS = 512;

template <typename T>
__global__ void __launch_bounds__(256) sumsq_partial_kernel(const T* __restrict__ u,
    size_t n, double* __restrict__ partial)
{
    __shared__ double red[256];
    double acc = 0.;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const double v = (double)u[i];
        acc += v * v;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) sum_partials_kernel(const double* __restrict__ partial,
    int n, double* __restrict__ out)
{
    __shared__ double red[256];
    double acc = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        acc += partial[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

namespace
{
struct PoissonMG
{
    int dtype;
    int nu1, nu2;
    cudaStream_t s;
    std::vector<Level> lev;
    std::vector<int> op;      // operator per level
    std::vector<double> jf;   // Jacobi factor per level
    std::vector<void*> x0, x1, w, f;
    void* partial = nullptr;  // NORM_BLOCKS doubles + the result
    int* err      = nullptr;
    size_t es     = 8;

    int sweep(int l, const void* u, void* out, void* wout, double factor)
    {
        PlaneParams p;
        p.u   = u;
        p.ldu = lev[l].npts();
        p.f   = f[l];
        p.ldf = lev[l].npts();
        p.out = out;
        p.ldo = lev[l].npts();
        p.w   = wout;
        p.ldw = lev[l].npts();
        for (int i = 0; i < 3; i++)
            p.n[i] = lev[l].n[i];
        p.err = err;
        return stencil_launch(OP_JACOBI, op[l], dtype, dtype, p, lev[l], factor, 1, s);
    }

    // Vcycle at level l from x = 0; returns the buffer (0: x0, 1: x1) that
    // holds the result, or a negative status
    int cycle(int l)
    {
        const size_t bytes = lev[l].npts() * es;
        int st = cuda_check(cudaMemsetAsync(x0[l], 0, bytes, s), "mgm zero");
        if (st != MGX_OK) return -st - 1;
        int cur = 0;
        auto X  = [&](int b) { return b ? x1[l] : x0[l]; };
        for (int i = 0; i < nu1; i++)
        {
            st = sweep(l, X(cur), X(cur ^ 1), nullptr, jf[l]);
            if (st != MGX_OK) return -st - 1;
            cur ^= 1;
        }
        if (l + 1 < (int)lev.size())
        {
            // res = A x - rhs (src/pb/Vcycle.h:165-167): a sweep with factor 0
            // copies x to the other buffer and writes the residual to w
            st = sweep(l, X(cur), X(cur ^ 1), w[l], 0.);
            if (st != MGX_OK) return -st - 1;
            st = restrict_launch(dtype, lev[l], w[l], lev[l].npts(), f[l + 1],
                lev[l + 1].npts(), 1, MaskDev(), s);
            if (st != MGX_OK) return -st - 1;
            const int c = cycle(l + 1);
            if (c < 0) return c;
            // x -= extend(ucoarse) (src/pb/Vcycle.h:197-198)
            st = prolong_launch(dtype, 1, lev[l], c ? x1[l + 1] : x0[l + 1],
                lev[l + 1].npts(), X(cur), lev[l].npts(), 1, MaskDev(), s);
            if (st != MGX_OK) return -st - 1;
        }
        for (int i = 0; i < nu2; i++)
        {
            st = sweep(l, X(cur), X(cur ^ 1), nullptr, jf[l]);
            if (st != MGX_OK) return -st - 1;
            cur ^= 1;
        }
        return cur;
    }

    int norm(const void* u, size_t n, double vel, double* out)
    {
        double* part = (double*)partial;
        if (dtype == MGX_F64)
            sumsq_partial_kernel<double><<<NORM_BLOCKS, 256, 0, s>>>((const double*)u, n, part);
        else
            sumsq_partial_kernel<float><<<NORM_BLOCKS, 256, 0, s>>>((const float*)u, n, part);
        MGX_LAUNCH_CHECK("sumsq_partial_kernel");
        sum_partials_kernel<<<1, 256, 0, s>>>(part, NORM_BLOCKS, part + NORM_BLOCKS);
        MGX_LAUNCH_CHECK("sum_partials_kernel");
        double h = 0.;
        MGX_TRY(cuda_check(cudaMemcpyAsync(&h, part + NORM_BLOCKS, sizeof(double),
                               cudaMemcpyDeviceToHost, s),
            "norm read-back"));
        MGX_TRY(cuda_check(cudaStreamSynchronize(s), "norm sync"));
        *out = std::sqrt(h * vel);
        return MGX_OK;
    }
};
} // namespace

int mgm_solve(mgx_ctx* ctx, const mgx_mgm_params* P, int dtype, void* vh,
    const void* rho, mgx_mgm_result* R, cudaStream_t s)
{
    if (!P || !vh || !rho || !R) return fail(MGX_BAD_ARG, "mgm: null argument");
    if (vh == rho) return fail(MGX_BAD_ARG, "mgm: vh and rho alias");
    const int radius = lap_radius(P->lap_type);
    if (radius < 0) return fail(MGX_BAD_ARG, "lap_type %d", P->lap_type);
    if (P->nu1 < 0 || P->nu2 < 0 || P->max_sweeps < 0 || P->max_levels < 0)
        return fail(MGX_BAD_ARG, "mgm: negative count");
    const int g0 = P->ghosts > 0 ? P->ghosts : radius;
    if (g0 < radius) return fail(MGX_BAD_ARG, "ghost width %d below operator radius %d", g0, radius);

    PoissonMG M;
    M.dtype = dtype;
    M.nu1   = P->nu1;
    M.nu2   = P->nu2;
    M.s     = s;
    M.es    = dtype_size(dtype);
    // levels: coarsen while every dimension is even and at least twice the
    // ghost width of the level's function, at most max_levels times
    // (src/pb/Vcycle.h:52-60,154-188).  Each coarse level takes the lower-
    // order operator (Laph4M stays Laph4M; Laph8 -> Laph6 -> Laph4 -> Laph2,
    // src/pb/Laph8.h:79-87, Laph6.h:79-87, Laph4.h:75-83), whose grid has
    // that operator's minimum ghost width; the coarse function's ghost width
    // is max(ghosts of the finer operator's grid - 1, 1) (Vcycle.h:176-180),
    // with the caller's g0 on the fine level.
    static const int lower[5] = { 0, 1, 1, 2, 3 };
    int o = P->lap_type, ng = g0, op_ng = g0;
    for (int l = 0;; l++)
    {
        const Level L = make_level(ctx->grid, l);
        M.lev.push_back(L);
        M.op.push_back(o);
        M.jf.push_back(jacobi_factor(o, L.h));
        bool coarsen = (l < P->max_levels);
        for (int i = 0; i < 3; i++)
            if ((L.n[i] & 1) || L.n[i] < 2 * ng) coarsen = false;
        if (!coarsen) break;
        ng    = std::max(op_ng - 1, 1);
        o     = lower[o];
        op_ng = lap_radius(o);
    }
    const int nl = (int)M.lev.size();
    // workspace: per level x0, x1, w, f (the fine level's f holds the outer
    // residual), then rhs, a scratch copy of vh and the norm partials
    size_t total = 0;
    std::vector<size_t> off;
    auto take = [&](size_t bytes) {
        off.push_back(total);
        total += ((bytes + 255) / 256) * 256;
    };
    for (int l = 0; l < nl; l++)
        for (int k = 0; k < 4; k++)
            take(M.lev[l].npts() * M.es);
    take(M.lev[0].npts() * M.es); // rhs
    take(M.lev[0].npts() * M.es); // scratch copy of vh
    take((NORM_BLOCKS + 1) * sizeof(double));
    MGX_TRY(ctx->mgm.ensure(total));
    MGX_TRY(ctx->flag.ensure(16));
    char* base = (char*)ctx->mgm.ptr;
    for (int l = 0; l < nl; l++)
    {
        M.x0.push_back(base + off[4 * l + 0]);
        M.x1.push_back(base + off[4 * l + 1]);
        M.w.push_back(base + off[4 * l + 2]);
        M.f.push_back(base + off[4 * l + 3]);
    }
    void* rhs     = base + off[4 * nl];
    void* scratch = base + off[4 * nl + 1];
    M.partial     = base + off[4 * nl + 2];
    M.err         = (int*)ctx->flag.ptr;
    MGX_TRY(cuda_check(cudaMemsetAsync(M.err, 0, sizeof(int), s), "flag reset"));

    const Level& F  = M.lev[0];
    const size_t np = F.npts();
    const double vel = F.h[0] * F.h[1] * F.h[2];
    // rhs = A.rhs(rho): B rho for Mehrstellen, rho otherwise (src/pb/Mgm.h:36-41)
    if (P->lap_type == 0)
    {
        PlaneParams p;
        p.u   = rho;
        p.ldu = np;
        p.out = rhs;
        p.ldo = np;
        for (int i = 0; i < 3; i++)
            p.n[i] = F.n[i];
        MGX_TRY(stencil_launch(OP_RHS, 0, dtype, dtype, p, F, 0., 1, s));
    }
    else
        MGX_TRY(cuda_check(cudaMemcpyAsync(rhs, rho, np * M.es, cudaMemcpyDeviceToDevice, s),
            "rhs copy"));
    double rhs_norm = 0.;
    MGX_TRY(M.norm(rhs, np, vel, &rhs_norm));
    const double inv_rhs_norm = 1. / rhs_norm;

    // the outer residual A vh - rhs goes to r via a factor-0 sweep on the
    // fine level against rhs (its x output is a scratch copy); r is then the
    // fine-level right-hand side of the cycle
    void* r = M.f[0];
    auto residual = [&]() -> int {
        M.f[0] = rhs;
        const int st = M.sweep(0, vh, scratch, r, 0.);
        M.f[0] = r;
        return st;
    };
    double init = 1., res_norm = 0.;
    bool converged = false;
    int sweeps     = 0;
    R->final_residual = R->final_relative_residual = 0.;
    for (int i = 0; i < P->max_sweeps; i++)
    {
        MGX_TRY(residual());
        MGX_TRY(M.norm(r, np, vel, &res_norm));
        if (i == 0) init = res_norm;
        if (res_norm * inv_rhs_norm < P->tol)
        {
            R->final_residual          = res_norm;
            R->final_relative_residual = res_norm * inv_rhs_norm;
            converged                  = true;
            break;
        }
        const int c = M.cycle(0);
        if (c < 0) return -c - 1;
        sweeps++;
        // vh += work1, with work1 the cycle of the negated residual
        MGX_TRY(mgx_axpy(np, -1., (mgx_dtype)dtype, c ? M.x1[0] : M.x0[0], vh, s));
    }
    if (!converged)
    {
        MGX_TRY(residual());
        MGX_TRY(M.norm(r, np, vel, &res_norm));
        R->final_residual          = res_norm;
        R->final_relative_residual = res_norm * inv_rhs_norm;
    }
    int herr = 0;
    MGX_TRY(cuda_check(cudaMemcpyAsync(&herr, M.err, sizeof(int), cudaMemcpyDeviceToHost, s),
        "flag read-back"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "mgm sync"));
    if (herr) return fail(MGX_TIMEOUT, "stencil pipeline wait gave up");
    R->residual_reduction = R->final_residual / init;
    R->nb_sweeps          = sweeps;
    R->converged          = converged ? 1 : 0;
    R->levels             = nl;
    return MGX_OK;
}
} // namespace mgx
