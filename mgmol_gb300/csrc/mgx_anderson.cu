// Anderson extrapolation of the orbital update on sm_103a: AndersonMix<T>
// (src/AndersonMix.cc:21-321), the accelerated branch of
// ABPG<T>::update_states (src/ABPG.cc:118-126).
//
// One update is three steps:
//  1. anderson_dots_kernel: for every function k, the FP64 dot products of
//     u_i = f' - f_i (i < mm, f' = fscale * f as res.scal(alpha) leaves it)
//     with each other and with f', where f_i are the stored residuals --
//     every pair of the reference's mat_ / rhs_ in one pass over f and the
//     history (the reference forms each difference block and takes one dot
//     product per pair);
//  2. anderson_reduce_kernel: the diagonal dot product of
//     LocGridOrbitals::dotProductDiagonal (src/LocGridOrbitals.cc:1783-1799,
//     1606-1630; GramMatrix::getTraceDiagProductWithInvS,
//     src/GramMatrix.cc:303-310): sum over k of vel * dot_k * (S^-1)(k, k),
//     then the mm x mm system is solved on the host with the reference's
//     safeguards (history shortened while the rescaled matrix has a
//     determinant below 0.01 or a coefficient leaves [-3, 0.5]);
//  3. anderson_update_kernel: x <- factor x + sum theta_j x_j + beta
//     (factor f' + sum theta_j f_j), with the old x and f' stored into the
//     history slots that the rotation frees, in one pass.
// The element operations repeat the reference's roundings (MPscal,
// MPaxpy, the storage-type difference), so only the order of the FP64 dot
// product sums differs from it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx
{
constexpr int AMAX       = MGX_ANDERSON_MAX_M;
constexpr int DOT_BLOCKS = 64;
constexpr int NPAIR_MAX  = AMAX * (AMAX + 1) / 2 + AMAX;

struct PtrSet
{
    const void* p[AMAX];
};

// pair index of (i, j), j <= i, then the rhs entries after the pairs
__host__ __device__ constexpr int pair_index(int i, int j) { return i * (i + 1) / 2 + j; }

template <typename T> struct Elem;
template <> struct Elem<float>
{
    // MPscal (src/linear_algebra/mputils.cc:61-80): (T)(alpha * (double)x)
    __device__ static float scal(double a, float x)
    {
        return a == 1. ? x : (a == 0. ? 0.f : __double2float_rn(__dmul_rn(a, (double)x)));
    }
    // MPaxpy (mputils.cc:233-244): y += (T)(alpha * (double)x)
    __device__ static float axpy(double a, float x, float y)
    {
        return __fadd_rn(y, __double2float_rn(__dmul_rn(a, (double)x)));
    }
    __device__ static float sub(float a, float b) { return __fsub_rn(a, b); }
};
template <> struct Elem<double>
{
    // DSCAL / DAXPY without fused multiply-add
    __device__ static double scal(double a, double x) { return a == 1. ? x : (a == 0. ? 0. : __dmul_rn(a, x)); }
    __device__ static double axpy(double a, double x, double y) { return __dadd_rn(y, __dmul_rn(a, x)); }
    __device__ static double sub(double a, double b) { return __dsub_rn(a, b); }
};

template <typename T, int MM>
__global__ void __launch_bounds__(256) anderson_dots_kernel(const T* __restrict__ f,
    double fscale, PtrSet fi, size_t ld, size_t npts, double* __restrict__ part)
{
    constexpr int NP = MM * (MM + 1) / 2 + MM;
    const int k      = blockIdx.y;
    const T* fk      = f + (size_t)k * ld;
    const T* hk[MM];
#pragma unroll
    for (int i = 0; i < MM; i++)
        hk[i] = reinterpret_cast<const T*>(fi.p[i]) + (size_t)k * ld;
    double acc[NP];
#pragma unroll
    for (int q = 0; q < NP; q++)
        acc[q] = 0.;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npts;
         p += (size_t)gridDim.x * blockDim.x)
    {
        const T fs = Elem<T>::scal(fscale, fk[p]);
        double u[MM];
#pragma unroll
        for (int i = 0; i < MM; i++)
            u[i] = (double)Elem<T>::sub(fs, hk[i][p]);
#pragma unroll
        for (int i = 0; i < MM; i++)
        {
#pragma unroll
            for (int j = 0; j <= i; j++)
                acc[pair_index(i, j)] += u[i] * u[j];
            acc[MM * (MM + 1) / 2 + i] += u[i] * (double)fs;
        }
    }
    __shared__ double red[8][NP];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < NP; q++)
    {
        double v = acc[q];
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    for (int q = threadIdx.x; q < NP; q += blockDim.x)
    {
        double v = 0.;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++)
            v += red[w][q];
        part[((size_t)k * gridDim.x + blockIdx.x) * NP + q] = v;
    }
}

// out[q] = sum_k (double)(vel * dot_k[q]) * invS(k, k), k in order (the
// trace of diag(ss) S^-1); dot_k[q] = sum of the block partials in order
__global__ void anderson_reduce_kernel(const double* __restrict__ part, int nblk, int np,
    int nfunc, double vel, const double* __restrict__ invS, double* __restrict__ out)
{
    const int q = threadIdx.x;
    if (q >= np) return;
    double tr = 0.;
    for (int k = 0; k < nfunc; k++)
    {
        double d = 0.;
        for (int b = 0; b < nblk; b++)
            d += part[((size_t)k * nblk + b) * np + q];
        tr += (d * vel) * invS[(size_t)k * nfunc + k];
    }
    out[q] = tr;
}

struct Coef
{
    double theta[AMAX];
};

template <typename T>
__global__ void __launch_bounds__(256) anderson_update_kernel(T* x, const T* f, double fscale,
    PtrSet xi, PtrSet fi, Coef c, int mm, double factor, double beta, T* slot_x, T* slot_f,
    T* fbar, size_t ld, size_t npts, int nfunc)
{
    const size_t total = (size_t)nfunc * npts;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
         e += (size_t)gridDim.x * blockDim.x)
    {
        const size_t k = e / npts, p = e % npts;
        const size_t o = k * ld + p;
        // every input of the point is read before any output is written:
        // the freed history slots may be the oldest x_j / f_j being read
        const T x0 = x[o];
        const T fs = Elem<T>::scal(fscale, f[o]);
        T hx[AMAX], hf[AMAX];
        for (int j = 0; j < mm; j++)
        {
            hx[j] = reinterpret_cast<const T*>(xi.p[j])[o];
            hf[j] = reinterpret_cast<const T*>(fi.p[j])[o];
        }
        T xs = x0, fb = fs;
        if (mm > 0)
        {
            xs = Elem<T>::scal(factor, xs);
            fb = Elem<T>::scal(factor, fb);
        }
        for (int j = 0; j < mm; j++)
            xs = Elem<T>::axpy(c.theta[j], hx[j], xs);
        for (int j = 0; j < mm; j++)
            fb = Elem<T>::axpy(c.theta[j], hf[j], fb);
        xs = Elem<T>::axpy(beta, fb, xs);
        if (slot_x) slot_x[o] = x0;
        if (slot_f) slot_f[o] = fs;
        if (fbar) fbar[o] = fb;
        x[o] = xs;
    }
}

/* ---------------- host algebra of the mm x mm system ---------------- */

/* eigenvalues of the symmetric n x n matrix whose lower triangle is in a
 * (column-major, leading dimension lda): cyclic Jacobi rotations */
static void sym_eigenvalues(const double* a, int n, int lda, double* w)
{
    std::vector<double> A((size_t)n * n);
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++)
            A[(size_t)j * n + i] = A[(size_t)i * n + j] = a[(size_t)j * lda + i];
    for (int sweep = 0; sweep < 100; sweep++)
    {
        double off = 0., tot = 0.;
        for (int j = 0; j < n; j++)
            for (int i = 0; i < n; i++)
            {
                tot += A[(size_t)j * n + i] * A[(size_t)j * n + i];
                if (i != j) off += A[(size_t)j * n + i] * A[(size_t)j * n + i];
            }
        if (off <= 1e-30 * tot || off == 0.) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++)
            {
                const double apq = A[(size_t)q * n + p];
                if (apq == 0.) continue;
                const double app = A[(size_t)p * n + p], aqq = A[(size_t)q * n + q];
                const double tau = (aqq - app) / (2. * apq);
                const double t   = (tau >= 0. ? 1. : -1.) / (std::fabs(tau) + std::sqrt(1. + tau * tau));
                const double cs = 1. / std::sqrt(1. + t * t), sn = t * cs;
                for (int r = 0; r < n; r++)
                {
                    const double arp = A[(size_t)p * n + r], arq = A[(size_t)q * n + r];
                    A[(size_t)p * n + r] = cs * arp - sn * arq;
                    A[(size_t)q * n + r] = sn * arp + cs * arq;
                }
                for (int r = 0; r < n; r++)
                {
                    const double apr = A[(size_t)r * n + p], aqr = A[(size_t)r * n + q];
                    A[(size_t)r * n + p] = cs * apr - sn * aqr;
                    A[(size_t)r * n + q] = sn * apr + cs * aqr;
                }
            }
    }
    for (int i = 0; i < n; i++)
        w[i] = A[(size_t)i * n + i];
    std::sort(w, w + n);
}

/* Cholesky solve of the n x n system whose lower triangle is in a (column-
 * major, leading dimension lda); b overwritten by the solution.  Returns 0,
 * or the 1-based index of a non-positive pivot. */
static int chol_solve(const double* a, int n, int lda, double* b)
{
    std::vector<double> L((size_t)n * n, 0.);
    for (int j = 0; j < n; j++)
    {
        double d = a[(size_t)j * lda + j];
        for (int k = 0; k < j; k++)
            d -= L[(size_t)k * n + j] * L[(size_t)k * n + j];
        if (!(d > 0.)) return j + 1;
        d = std::sqrt(d);
        L[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++)
        {
            double s = a[(size_t)j * lda + i];
            for (int k = 0; k < j; k++)
                s -= L[(size_t)k * n + i] * L[(size_t)k * n + j];
            L[(size_t)j * n + i] = s / d;
        }
    }
    for (int i = 0; i < n; i++)
    {
        double s = b[i];
        for (int k = 0; k < i; k++)
            s -= L[(size_t)k * n + i] * b[k];
        b[i] = s / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; i--)
    {
        double s = b[i];
        for (int k = i + 1; k < n; k++)
            s -= L[(size_t)i * n + k] * b[k];
        b[i] = s / L[(size_t)i * n + i];
    }
    return 0;
}

/* The coefficient logic of AndersonMix<T>::update (src/AndersonMix.cc:
 * 100-245): mat (m x m, lower triangle of the first mm rows and columns
 * valid) and rhs for the current mm; mm shortened while the matrix rescaled
 * to unit diagonal has a determinant (product of eigenvalues) below 0.01,
 * and whenever a coefficient leaves [min_theta, max_theta] with mm > 1; a
 * lone coefficient outside is reset (-0.5 above 1, 0 in (0.5, 1], -3 below
 * -3).  Returns MGX_NOT_SPD where the reference prints "dpotrs: info" and
 * exits. */
static int anderson_coefficients(const std::vector<double>& mat, const std::vector<double>& rhs,
    int m, int* mm_io, double* theta, int* reductions)
{
    const double min_det = 0.01, max_theta = 0.5, min_theta = -3.;
    int mm = *mm_io;
    bool again = true;
    while (again)
    {
        again = false;
        for (int i = 0; i < mm; i++)
            theta[i] = rhs[i];
        while (mm > 1)
        {
            std::vector<double> t(mat);
            for (int i = 0; i < mm; i++)
            {
                const double alpha = 1. / std::sqrt(t[(size_t)(m + 1) * i]);
                for (int j = 0; j <= i; j++)
                    t[(size_t)j * m + i] *= alpha;
                for (int j = i; j < mm; j++)
                    t[(size_t)i * m + j] *= alpha;
            }
            double w[AMAX];
            sym_eigenvalues(t.data(), mm, m, w);
            double det = 1.;
            for (int i = 0; i < mm; i++)
                det *= w[i];
            if (det < min_det)
            {
                mm--;
                (*reductions)++;
            }
            else
                break;
        }
        if (mm > 0)
        {
            for (int i = 0; i < mm; i++)
                theta[i] = rhs[i];
            if (chol_solve(mat.data(), mm, m, theta) != 0)
                return fail(MGX_NOT_SPD, "Anderson matrix not positive definite (mm = %d)", mm);
        }
        for (int j = 0; j < mm; j++)
        {
            if (theta[j] > max_theta)
            {
                if (mm > 1)
                {
                    mm--;
                    (*reductions)++;
                    again = true;
                    break;
                }
                theta[j] = theta[j] > 1. ? -0.5 : 0.;
            }
            else if (theta[j] < min_theta)
            {
                if (mm > 1)
                {
                    mm--;
                    (*reductions)++;
                    again = true;
                    break;
                }
                theta[j] = min_theta;
            }
        }
    }
    *mm_io = mm;
    return MGX_OK;
}
} // namespace mgx

/* the opaque handle of the C ABI: history blocks in rotation order */
struct mgx_anderson
{
    mgx_ctx* ctx = nullptr;
    int m = 0, mm = -1, dtype = 0, nfunc = 0;
    double beta = 1.;
    size_t ld = 0;
    std::vector<mgx::DeviceBuffer> blocks; // 2m blocks
    std::vector<int> xi, fi;               // block index of x_j / f_j, j < m
    mgx::DeviceBuffer part, out;
};

using namespace mgx;

extern "C" {

int mgx_anderson_create(mgx_ctx* ctx, int m, double beta, mgx_dtype dtype, size_t ld,
    int nfunc, mgx_anderson** mix)
{
    if (!ctx || !mix) return fail(MGX_BAD_ARG, "ctx or mix is NULL");
    if (m < 0 || m > AMAX) return fail(MGX_BAD_ARG, "history length %d outside [0, %d]", m, AMAX);
    if (dtype != MGX_F64 && dtype != MGX_F32) return fail(MGX_BAD_ARG, "dtype %d", (int)dtype);
    const size_t np = (size_t)ctx->grid.n[0] * ctx->grid.n[1] * ctx->grid.n[2];
    if (nfunc < 1 || nfunc > 65535) return fail(MGX_BAD_ARG, "nfunc %d", nfunc);
    if (nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, np);
    auto* a   = new mgx_anderson;
    a->ctx    = ctx;
    a->m      = m;
    a->beta   = beta;
    a->dtype  = dtype;
    a->nfunc  = nfunc;
    a->ld     = nfunc > 1 ? ld : np;
    a->blocks.resize(2 * m);
    const size_t bytes = (size_t)nfunc * a->ld * dtype_size(dtype);
    for (int i = 0; i < 2 * m; i++)
    {
        const int st = a->blocks[i].ensure(bytes);
        if (st != MGX_OK)
        {
            delete a;
            return st;
        }
    }
    for (int j = 0; j < m; j++)
    {
        a->xi.push_back(j);
        a->fi.push_back(m + j);
    }
    *mix = a;
    return MGX_OK;
}

int mgx_anderson_destroy(mgx_anderson* mix)
{
    delete mix;
    return MGX_OK;
}

int mgx_anderson_restart(mgx_anderson* mix)
{
    if (!mix) return fail(MGX_BAD_ARG, "mix is NULL");
    mix->mm = -1;
    return MGX_OK;
}

int mgx_anderson_update(mgx_anderson* a, void* x, const void* f, double fscale,
    const double* invS, void* fbar, mgx_anderson_info* info, void* stream)
{
    if (!a) return fail(MGX_BAD_ARG, "mix is NULL");
    if (!x || !f) return fail(MGX_BAD_ARG, "x or f is NULL");
    if (x == f) return fail(MGX_BAD_ARG, "x and f alias");
    cudaStream_t s  = (cudaStream_t)stream;
    const int m     = a->m;
    const size_t np = (size_t)a->ctx->grid.n[0] * a->ctx->grid.n[1] * a->ctx->grid.n[2];
    const Level L   = make_level(a->ctx->grid, 0);
    const double vel = L.h[0] * L.h[1] * L.h[2];
    // the history length of this update (committed to the handle only
    // once the update has been issued)
    int mm = a->mm < m ? a->mm + 1 : a->mm;
    int reductions = 0;
    double theta[AMAX] = {};
    if (mm > 0)
    {
        if (!invS) return fail(MGX_BAD_ARG, "invS is NULL");
        const int npair = mm * (mm + 1) / 2 + mm;
        MGX_TRY(a->part.ensure((size_t)a->nfunc * DOT_BLOCKS * NPAIR_MAX * sizeof(double)));
        MGX_TRY(a->out.ensure(NPAIR_MAX * sizeof(double)));
        PtrSet fi{};
        for (int i = 0; i < mm; i++)
            fi.p[i] = a->blocks[a->fi[i]].ptr;
        dim3 grid(DOT_BLOCKS, a->nfunc);
        double* part = (double*)a->part.ptr;
#define MGX_DOTS(T, MMV)                                                                      \
    case MMV:                                                                                 \
        anderson_dots_kernel<T, MMV><<<grid, 256, 0, s>>>((const T*)f, fscale, fi, a->ld, np, \
            part);                                                                            \
        break;
        if (a->dtype == MGX_F64)
        {
            switch (mm)
            {
                MGX_DOTS(double, 1) MGX_DOTS(double, 2) MGX_DOTS(double, 3) MGX_DOTS(double, 4)
                MGX_DOTS(double, 5) MGX_DOTS(double, 6) MGX_DOTS(double, 7) MGX_DOTS(double, 8)
            }
        }
        else
        {
            switch (mm)
            {
                MGX_DOTS(float, 1) MGX_DOTS(float, 2) MGX_DOTS(float, 3) MGX_DOTS(float, 4)
                MGX_DOTS(float, 5) MGX_DOTS(float, 6) MGX_DOTS(float, 7) MGX_DOTS(float, 8)
            }
        }
#undef MGX_DOTS
        MGX_LAUNCH_CHECK("anderson_dots_kernel");
        anderson_reduce_kernel<<<1, 64, 0, s>>>(part, DOT_BLOCKS, npair, a->nfunc, vel, invS,
            (double*)a->out.ptr);
        MGX_LAUNCH_CHECK("anderson_reduce_kernel");
        double h[NPAIR_MAX];
        MGX_TRY(cuda_check(cudaMemcpyAsync(h, a->out.ptr, npair * sizeof(double),
                               cudaMemcpyDeviceToHost, s),
            "Anderson products read"));
        MGX_TRY(cuda_check(cudaStreamSynchronize(s), "Anderson sync"));
        std::vector<double> mat((size_t)m * m, 0.), rhs(m, 0.);
        for (int i = 0; i < mm; i++)
        {
            for (int j = 0; j <= i; j++)
                mat[(size_t)j * m + i] = h[pair_index(i, j)];
            rhs[i] = h[mm * (mm + 1) / 2 + i];
        }
        MGX_TRY(anderson_coefficients(mat, rhs, m, &mm, theta, &reductions));
    }
    double factor = 1.;
    for (int j = 0; j < mm; j++)
        factor -= theta[j];
    PtrSet xi{}, fi{};
    for (int j = 0; j < mm; j++)
    {
        xi.p[j] = a->blocks[a->xi[j]].ptr;
        fi.p[j] = a->blocks[a->fi[j]].ptr;
    }
    Coef c{};
    for (int j = 0; j < mm; j++)
        c.theta[j] = theta[j];
    // the rotation frees the oldest slot, which receives the old x and f'
    void* slot_x = m > 0 ? a->blocks[a->xi[m - 1]].ptr : nullptr;
    void* slot_f = m > 0 ? a->blocks[a->fi[m - 1]].ptr : nullptr;
    const double beta = mm > 0 ? a->beta : 1.;
    const size_t total = (size_t)a->nfunc * np;
    const int nb = (int)std::min<size_t>((total + 255) / 256, 16 * (size_t)a->ctx->sm_count);
    if (a->dtype == MGX_F64)
        anderson_update_kernel<double><<<nb, 256, 0, s>>>((double*)x, (const double*)f, fscale,
            xi, fi, c, mm, factor, beta, (double*)slot_x, (double*)slot_f, (double*)fbar, a->ld,
            np, a->nfunc);
    else
        anderson_update_kernel<float><<<nb, 256, 0, s>>>((float*)x, (const float*)f, fscale, xi,
            fi, c, mm, factor, beta, (float*)slot_x, (float*)slot_f, (float*)fbar, a->ld, np,
            a->nfunc);
    MGX_LAUNCH_CHECK("anderson_update_kernel");
    a->mm = mm;
    if (m > 0)
    {
        std::rotate(a->xi.rbegin(), a->xi.rbegin() + 1, a->xi.rend());
        std::rotate(a->fi.rbegin(), a->fi.rbegin() + 1, a->fi.rend());
    }
    if (info)
    {
        info->mm         = mm;
        info->reductions = reductions;
        for (int j = 0; j < AMAX; j++)
            info->theta[j] = j < mm ? theta[j] : 0.;
    }
    return MGX_OK;
}

} // extern "C"
