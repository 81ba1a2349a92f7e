// The electronic density of a block of non-orthogonal orbitals on sm_103a:
// Rho<T>::computeRho with computeRhoSubdomainUsingBlas3 (src/Rho.cc:282-320,
// 359-450) and rescaleTotalCharge (:150-200).
//
//   rho(p) = sum_j (Psi X)_j(p) psi_j(p),   X the density matrix,
//
// the O(N^3) product of the reference followed by its O(N^2) reduction.  On
// the tensor cores the reduction is the epilogue of the product (each
// output tile is multiplied by the orbitals it belongs to and summed over
// its columns into rho), so the N x P product never reaches memory.  The
// CUDA-core modes form the product in column chunks and reduce each chunk.
// Then charge = vel sum_p rho(p) and rho *= nel / charge.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "mgx_internal.cuh"

namespace mgx
{
int psi_theta_cuda_cores(int, const void*, size_t, size_t, int, const double*, int, int,
    double, const void*, void*, cudaStream_t);
int psi_theta_tcgen05(mgx_ctx*, int, const float*, size_t, size_t, int, const double*, int,
    int, float, const float*, float*, cudaStream_t, double* rho);

// rho(p) += sum_j prod_j(p) psi_j(p) over the chunk's columns, j in order,
// each term formed in the orbital type (as the reference's product of two
// ORBDTYPE values) and added in FP64
template <typename T>
__global__ void __launch_bounds__(256) rho_chunk_kernel(const T* __restrict__ prod, size_t ldp,
    const T* __restrict__ psi, size_t ld, size_t npts, int nc, double* __restrict__ rho)
{
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
         p += (size_t)gridDim.x * blockDim.x)
    {
        double acc = rho[p];
        for (int j = 0; j < nc; j++)
            acc += (double)(prod[(size_t)j * ldp + p] * psi[(size_t)j * ld + p]);
        rho[p] = acc;
    }
}

constexpr int CHARGE_BLOCKS = 512;

__global__ void __launch_bounds__(256) charge_partial_kernel(const double* __restrict__ rho,
    size_t npts, double* __restrict__ part)
{
    __shared__ double red[256];
    double acc = 0.;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
         p += (size_t)gridDim.x * blockDim.x)
        acc += rho[p];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// one thread: the charge vel * sum of the partials (in order), the factor
// nel / charge and the flag of a factor off 1 by more than 0.02
__global__ void charge_finish_kernel(const double* __restrict__ part, int nb, double vel,
    double nel, double* __restrict__ out)
{
    double q = 0.;
    for (int b = 0; b < nb; b++)
        q += part[b];
    q *= vel;
    out[0]   = q;
    double t = 1.;
    if (nel > 0. && q > 0.) t = nel / q;
    out[1] = t;
    out[2] = (std::fabs(t - 1.) > 0.02) ? 1. : 0.;
}

// MPscal on the FP64 density, skipped when the factor is off
__global__ void __launch_bounds__(256) rho_scale_kernel(double* __restrict__ rho, size_t npts,
    const double* __restrict__ f)
{
    if (f[2] != 0.) return;
    const double t = f[1];
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
         p += (size_t)gridDim.x * blockDim.x)
        rho[p] *= t;
}
} // namespace mgx

using namespace mgx;

extern "C" {

int mgx_rho(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi, size_t ld, int nfunc,
    const double* dm, double nel, double* rho, double* charge, void* work, int work_funcs,
    void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    if (dtype != MGX_F64 && dtype != MGX_F32) return fail(MGX_BAD_ARG, "dtype %d", (int)dtype);
    if (!rho) return fail(MGX_BAD_ARG, "rho is NULL");
    if (nfunc < 0 || (nfunc > 0 && (!psi || !dm))) return fail(MGX_BAD_ARG, "psi or X is NULL");
    const Level L   = make_level(ctx->grid, 0);
    const size_t np = L.npts();
    if (nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, np);
    const size_t ldv = nfunc > 1 ? ld : np;
    cudaStream_t s   = (cudaStream_t)stream;
    MGX_TRY(cuda_check(cudaMemsetAsync(rho, 0, np * sizeof(double), s), "rho reset"));
    if (nfunc > 0)
    {
        if (mode == MGX_GEMM_TF32 || mode == MGX_GEMM_BF16X3 || mode == MGX_GEMM_FP16X3)
        {
            if (dtype != MGX_F32) return fail(MGX_BAD_ARG, "gemm mode %d needs FP32 orbitals", mode);
            MGX_TRY(psi_theta_tcgen05(ctx, mode, (const float*)psi, ldv, np, nfunc, dm, nfunc,
                nfunc, 0.f, nullptr, nullptr, s, rho));
        }
        else if (mode == MGX_GEMM_FP64 || mode == MGX_GEMM_FP32)
        {
            if (mode == MGX_GEMM_FP32 && dtype != MGX_F32)
                return fail(MGX_BAD_ARG, "gemm mode %d needs FP32 orbitals", mode);
            const size_t es = dtype_size(dtype);
            int wf          = work ? std::min(std::max(work_funcs, 1), nfunc) : std::min(nfunc, 256);
            if (!work)
            {
                MGX_TRY(ctx->resid.ensure((size_t)wf * ldv * es + 256));
                work = ctx->resid.ptr;
            }
            if (work == psi) return fail(MGX_BAD_ARG, "work aliases psi");
            const int kind = mode == MGX_GEMM_FP32 ? 2 : (dtype == MGX_F64 ? 0 : 1);
            const int nb   = (int)std::min<size_t>((np + 255) / 256, 16 * (size_t)ctx->sm_count);
            for (int j0 = 0; j0 < nfunc; j0 += wf)
            {
                const int nc = std::min(wf, nfunc - j0);
                MGX_TRY(psi_theta_cuda_cores(kind, psi, ldv, np, nfunc, dm + (size_t)j0 * nfunc,
                    nfunc, nc, 0., nullptr, work, s));
                if (dtype == MGX_F64)
                    rho_chunk_kernel<double><<<nb, 256, 0, s>>>((const double*)work, ldv,
                        (const double*)psi + (size_t)j0 * ldv, ldv, np, nc, rho);
                else
                    rho_chunk_kernel<float><<<nb, 256, 0, s>>>((const float*)work, ldv,
                        (const float*)psi + (size_t)j0 * ldv, ldv, np, nc, rho);
                MGX_LAUNCH_CHECK("rho_chunk_kernel");
            }
        }
        else
            return fail(MGX_BAD_ARG, "gemm mode %d", mode);
    }
    MGX_TRY(ctx->red.ensure((CHARGE_BLOCKS + 4) * sizeof(double)));
    double* part = (double*)ctx->red.ptr;
    double* fin  = part + CHARGE_BLOCKS;
    charge_partial_kernel<<<CHARGE_BLOCKS, 256, 0, s>>>(rho, np, part);
    MGX_LAUNCH_CHECK("charge_partial_kernel");
    charge_finish_kernel<<<1, 1, 0, s>>>(part, CHARGE_BLOCKS, L.h[0] * L.h[1] * L.h[2], nel, fin);
    MGX_LAUNCH_CHECK("charge_finish_kernel");
    const int nbs = (int)std::min<size_t>((np + 255) / 256, 16 * (size_t)ctx->sm_count);
    rho_scale_kernel<<<nbs, 256, 0, s>>>(rho, np, fin);
    MGX_LAUNCH_CHECK("rho_scale_kernel");
    double h[3];
    MGX_TRY(cuda_check(cudaMemcpyAsync(h, fin, sizeof(h), cudaMemcpyDeviceToHost, s),
        "charge read"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "rho sync"));
    if (charge) *charge = h[0];
    if (h[2] != 0.)
        return fail(MGX_BAD_ARG, "density charge %g differs from %g electrons by more than 2%%",
            h[0], nel);
    return MGX_OK;
}

} // extern "C"
