// Gram / H-matrix contractions and the small dense FP64 algebra of the
// orbital hot path on sm_103a:
//  - S = Psi^T Psi * vel and H = Psi^T (H Psi) * vel as split-K tall-skinny
//    products on CUDA cores (FP64 data with FP64 FMA, or FP32 data with FP32
//    FMA in a three-level summation ending in double-float within the
//    K-slice),
//    FP64 atomics across slices, then the finishing pass
//    (scale by vel, the |x| > 1e-14 filter of
//    src/LocalMatrices2DistMatrix.cc:16,60, symmetric fill of S);
//  - GramMatrix::updateLS / computeInverse (src/GramMatrix.cc:75-191):
//    blocked right-looking Cholesky with inverted diagonal blocks, the
//    inverse factor, and S^-1 = L^-T L^-1, all FP64;
//  - ProjectedMatrices::getEigSum (src/ProjectedMatrices.cc:550-566):
//    tr(H S^-1) as a device reduction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{

/* ------------------------------------------------------------------ */
/* split-K Gram kernel: C[i][j] += sum_p A[i][p] B[j][p]                 */
/* A, B orbital-major (row i at A + i*ld), 64x64 output tiles.            */
/* ------------------------------------------------------------------ */
constexpr int GT  = 64; // output tile
constexpr int GKC = 32; // k chunk
// FP32 data: three-level summation.  FMAs chain over 8 k values; every 8
// k values that chain's sum is added to a second FP32 sum; every
// GKC * GRAM_F32_CHAIN = 128 k values the second sum goes into a
// double-float (hi + lo, two FP32) accumulator by an error-free two-sum.
// The rounding error then grows like 8 + 16 terms of FP32 rounding instead
// of the whole K slice's length, for one FP32 add per 8 FMAs and a two-sum
// per 128.
constexpr int GRAM_F32_CHAIN = 4;
constexpr int GRAM_F32_INNER = 8;

/* s + e = a + b exactly (Knuth's two-sum; no reassociation, no multiply to
 * contract) */
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s              = a + b;
    const float bb = s - a;
    e              = (a - (s - bb)) + (b - bb);
}

template <typename T>
__global__ void __launch_bounds__(256) gram_splitk_kernel(const T* __restrict__ A,
    const T* __restrict__ B, size_t ld, int n, int ncols, size_t K, size_t kslice,
    const int2* __restrict__ tiles, double* __restrict__ C)
{
    __shared__ T As[GKC][GT + 1];
    __shared__ T Bs[GKC][GT + 1];
    const int2 tile = tiles[blockIdx.x];
    const int i0 = tile.x * GT, j0 = tile.y * GT;
    const size_t k0 = (size_t)blockIdx.y * kslice;
    const size_t k1 = min(K, k0 + kslice);
    const int tid   = threadIdx.x;
    const int tx = tid % 16, ty = tid / 16; // 16 x 16 threads, 4x4 outputs each
    T acc[4][4];
    float mid[4][4];          // FP32 data: the sum of the 8-term chains
    float hi[4][4], lo[4][4]; // FP32 data: the double-float sum of the chains
#pragma unroll
    for (int a = 0; a < 4; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
        {
            acc[a][b] = (T)0;
            mid[a][b] = 0.f;
            hi[a][b]  = 0.f;
            lo[a][b]  = 0.f;
        }
    int chain = 0;
    for (size_t kc = k0; kc < k1; kc += GKC)
    {
        // 64 rows x 32 k for each operand: 2048 elements, 8 per thread
#pragma unroll
        for (int r = 0; r < 8; r++)
        {
            const int e   = tid + r * 256;
            const int row = e / GKC;
            const int kk  = e % GKC;
            const size_t k = kc + kk;
            T av = (T)0, bv = (T)0;
            if (k < k1)
            {
                if (i0 + row < n) av = A[(size_t)(i0 + row) * ld + k];
                if (j0 + row < ncols) bv = B[(size_t)(j0 + row) * ld + k];
            }
            As[kk][row] = av;
            Bs[kk][row] = bv;
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < GKC; kk++)
        {
            T a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    acc[p][q] += a[p] * b[q];
            if constexpr (sizeof(T) == 4)
            {
                if (kk % GRAM_F32_INNER == GRAM_F32_INNER - 1)
                {
#pragma unroll
                    for (int p = 0; p < 4; p++)
#pragma unroll
                        for (int q = 0; q < 4; q++)
                        {
                            mid[p][q] += (float)acc[p][q];
                            acc[p][q] = (T)0;
                        }
                }
            }
        }
        __syncthreads();
        if constexpr (sizeof(T) == 4)
        {
            if (++chain == GRAM_F32_CHAIN || kc + GKC >= k1)
            {
                chain = 0;
#pragma unroll
                for (int p = 0; p < 4; p++)
#pragma unroll
                    for (int q = 0; q < 4; q++)
                    {
                        float sum, err;
                        two_sum(hi[p][q], mid[p][q], sum, err);
                        hi[p][q] = sum;
                        lo[p][q] += err;
                        mid[p][q] = 0.f;
                    }
            }
        }
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
            const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            double v;
            if constexpr (sizeof(T) == 4)
                v = (double)hi[p][q] + (double)lo[p][q];
            else
                v = (double)acc[p][q];
            if (i < n && j < ncols) atomicAdd(&C[(size_t)j * n + i], v);
        }
}

/* S or H finishing: scale, filter, (S) mirror the lower triangle */
__global__ void gram_finish_kernel(double* C, int n, double vel, int symmetric)
{
    const size_t nn = (size_t)n * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const int i = (int)(t % n), j = (int)(t / n);
        if (symmetric && i < j) continue;
        double x = C[t] * vel;
        if (!(fabs(x) > 1.e-14)) x = 0.;
        C[t] = x;
        if (symmetric && i != j) C[(size_t)i * n + j] = x;
    }
}

int gram_cuda_cores(mgx_ctx* ctx, int dtype, const void* A, const void* B,
    size_t ld, size_t K, int n, double vel, int symmetric, double* C,
    cudaStream_t s)
{
    const int nt = (n + GT - 1) / GT;
    std::vector<int2> tiles;
    for (int j = 0; j < nt; j++)
        for (int i = 0; i < nt; i++)
            if (!symmetric || i >= j) tiles.push_back(make_int2(i, j));
    const int ntiles = (int)tiles.size();
    int ksplit       = std::max(1, (8 * ctx->sm_count + ntiles - 1) / ntiles);
    size_t kslice    = (K + ksplit - 1) / ksplit;
    kslice           = ((kslice + GKC - 1) / GKC) * GKC;
    ksplit           = (int)((K + kslice - 1) / kslice);
    if (ksplit > 65535) return fail(MGX_UNSUPPORTED, "K too large for split");
    MGX_TRY(ctx->gemm_ws.ensure(tiles.size() * sizeof(int2)));
    MGX_TRY(cuda_check(cudaMemcpyAsync(ctx->gemm_ws.ptr, tiles.data(),
                           tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, s),
        "gram tiles upload"));
    MGX_TRY(cuda_check(cudaMemsetAsync(C, 0, (size_t)n * n * sizeof(double), s),
        "gram zero"));
    dim3 grid(ntiles, ksplit);
    if (dtype == MGX_F64)
        gram_splitk_kernel<double><<<grid, 256, 0, s>>>((const double*)A,
            (const double*)B, ld, n, n, K, kslice, (const int2*)ctx->gemm_ws.ptr, C);
    else
        gram_splitk_kernel<float><<<grid, 256, 0, s>>>((const float*)A,
            (const float*)B, ld, n, n, K, kslice, (const int2*)ctx->gemm_ws.ptr, C);
    MGX_LAUNCH_CHECK("gram_splitk_kernel");
    // the tile list must stay alive until the kernel has read it
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "gram sync"));
    const int nb = (int)std::min<size_t>(((size_t)n * n + 255) / 256, 4096);
    gram_finish_kernel<<<nb, 256, 0, s>>>(C, n, vel, symmetric);
    MGX_LAUNCH_CHECK("gram_finish_kernel");
    return MGX_OK;
}

/* B = Psi^T (B Psi) * vel (LocGridOrbitals::computeMatB,
 * src/LocGridOrbitals.cc:1428-1487) on CUDA cores: B Psi is formed `wf`
 * functions at a time in `work` (leading dimension ld) by the Mehrstellen
 * right-hand-side stencil, and only output tiles that reach the lower
 * triangle are computed; the finishing pass mirrors the lower triangle. */
int matb_cuda_cores(mgx_ctx* ctx, int dtype, const void* psi, size_t ld, size_t K, int n,
    double vel, double* C, void* work, int wf, cudaStream_t s)
{
    if (wf <= 0) return fail(MGX_BAD_ARG, "matB: empty work block");
    const size_t es = dtype_size(dtype);
    const int nt    = (n + GT - 1) / GT;
    std::vector<int2> tiles;
    std::vector<size_t> first;
    for (int c0 = 0; c0 < n; c0 += wf)
    {
        const int nc = std::min(wf, n - c0);
        first.push_back(tiles.size());
        for (int j = 0; j < (nc + GT - 1) / GT; j++)
            for (int i = 0; i < nt; i++)
                if (i * GT + GT - 1 >= c0 + j * GT) tiles.push_back(make_int2(i, j));
    }
    first.push_back(tiles.size());
    const int nchunks = (int)first.size() - 1;
    const int avg     = std::max(1, (int)(tiles.size() / nchunks));
    int ksplit        = std::max(1, (8 * ctx->sm_count + avg - 1) / avg);
    size_t kslice     = (K + ksplit - 1) / ksplit;
    kslice            = ((kslice + GKC - 1) / GKC) * GKC;
    ksplit            = (int)((K + kslice - 1) / kslice);
    if (ksplit > 65535) return fail(MGX_UNSUPPORTED, "K too large for split");
    MGX_TRY(ctx->gemm_ws.ensure(tiles.size() * sizeof(int2)));
    const int2* dt = (const int2*)ctx->gemm_ws.ptr;
    MGX_TRY(cuda_check(cudaMemcpyAsync(ctx->gemm_ws.ptr, tiles.data(),
                           tiles.size() * sizeof(int2), cudaMemcpyHostToDevice, s),
        "matB tiles upload"));
    MGX_TRY(cuda_check(cudaMemsetAsync(C, 0, (size_t)n * n * sizeof(double), s), "matB zero"));
    for (int c = 0; c < nchunks; c++)
    {
        const int c0 = c * wf, nc = std::min(wf, n - c0);
        const int nct = (int)(first[c + 1] - first[c]);
        MGX_TRY(rhs_block(ctx->grid, dtype, (const char*)psi + (size_t)c0 * ld * es, ld, work,
            ld, nc, s));
        dim3 grid(nct, ksplit);
        if (dtype == MGX_F64)
            gram_splitk_kernel<double><<<grid, 256, 0, s>>>((const double*)psi,
                (const double*)work, ld, n, nc, K, kslice, dt + first[c], C + (size_t)c0 * n);
        else
            gram_splitk_kernel<float><<<grid, 256, 0, s>>>((const float*)psi,
                (const float*)work, ld, n, nc, K, kslice, dt + first[c], C + (size_t)c0 * n);
        MGX_LAUNCH_CHECK("gram_splitk_kernel");
    }
    // the tile list must stay alive until the kernels have read it
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "matB sync"));
    const int nb = (int)std::min<size_t>(((size_t)n * n + 255) / 256, 4096);
    gram_finish_kernel<<<nb, 256, 0, s>>>(C, n, vel, 1);
    MGX_LAUNCH_CHECK("gram_finish_kernel");
    return MGX_OK;
}

/* ------------------------------------------------------------------ */
/* generic FP64 GEMM, column-major: C = alpha op(A) op(B) + beta C        */
/* ------------------------------------------------------------------ */
// sym_a: A is symmetric and only its lower triangle is read (BLAS symm
// with side 'l', uplo 'l'); used without TA.
template <bool TA, bool TB>
__global__ void __launch_bounds__(256) dgemm_kernel(int m, int n, int k,
    double alpha, const double* __restrict__ A, int lda,
    const double* __restrict__ B, int ldb, double beta, double* C, int ldc,
    int lower_only, int sym_a)
{
    __shared__ double As[16][65];
    __shared__ double Bs[16][65];
    const int i0 = blockIdx.x * 64, j0 = blockIdx.y * 64;
    if (lower_only && i0 + 63 < j0) return;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    double acc[4][4] = {};
    for (int kc = 0; kc < k; kc += 16)
    {
#pragma unroll
        for (int r = 0; r < 4; r++)
        {
            const int e  = tid + r * 256;
            const int mm = e % 64, kk = e / 64;
            const int i = i0 + mm, j = j0 + mm, kq = kc + kk;
            double av = 0., bv = 0.;
            if (i < m && kq < k)
                av = (TA || (sym_a && kq > i)) ? A[(size_t)i * lda + kq] : A[(size_t)kq * lda + i];
            if (j < n && kq < k) bv = TB ? B[(size_t)kq * ldb + j] : B[(size_t)j * ldb + kq];
            As[kk][mm] = av;
            Bs[kk][mm] = bv;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++)
        {
            double a[4], b[4];
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                a[q] = As[kk][ty + 16 * q];
                b[q] = Bs[kk][tx + 16 * q];
            }
#pragma unroll
            for (int p = 0; p < 4; p++)
#pragma unroll
                for (int q = 0; q < 4; q++)
                    acc[p][q] = fma(a[p], b[q], acc[p][q]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int p = 0; p < 4; p++)
#pragma unroll
        for (int q = 0; q < 4; q++)
        {
            const int i = i0 + ty + 16 * p, j = j0 + tx + 16 * q;
            if (i < m && j < n && (!lower_only || i >= j))
            {
                double* c = C + (size_t)j * ldc + i;
                *c        = alpha * acc[p][q] + (beta == 0. ? 0. : beta * *c);
            }
        }
}

static int dgemm(bool ta, bool tb, int m, int n, int k, double alpha,
    const double* A, int lda, const double* B, int ldb, double beta, double* C,
    int ldc, int lower_only, cudaStream_t s, int sym_a = 0)
{
    if (m <= 0 || n <= 0) return MGX_OK;
    dim3 grid((m + 63) / 64, (n + 63) / 64);
    if (!ta && !tb)
        dgemm_kernel<false, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower_only, sym_a);
    else if (!ta && tb)
        dgemm_kernel<false, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower_only, sym_a);
    else if (ta && !tb)
        dgemm_kernel<true, false><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower_only, sym_a);
    else
        dgemm_kernel<true, true><<<grid, 256, 0, s>>>(m, n, k, alpha, A, lda, B, ldb, beta, C, ldc, lower_only, sym_a);
    MGX_LAUNCH_CHECK("dgemm_kernel");
    return MGX_OK;
}

/* ------------------------------------------------------------------ */
/* orbital block times a small FP64 matrix on CUDA cores (MPgemmNN,      */
/* src/linear_algebra/mputils.cc:719-760):                               */
/*   out_j[p] = sum_i psi_i[p] theta(i, j) + beta cin_j[p], j < ncols,   */
/*   theta column j at theta + j * ldt                                   */
/* ACC double: FP64 accumulation as the reference does for both orbital  */
/* types; ACC float: theta rounded to FP32 and FP32 FMA.  Tiles of 128   */
/* points x 64 functions, 8 x 4 results per thread.  cin may alias out.  */
/* ------------------------------------------------------------------ */
template <typename T, typename ACC>
__global__ void __launch_bounds__(256) psi_theta_kernel(size_t npts, int n,
    const T* __restrict__ psi, size_t ld, const double* __restrict__ theta, int ldt,
    int ncols, double beta, const T* cin, T* out)
{
    __shared__ ACC As[16][128];
    __shared__ ACC Bs[16][65];
    const size_t p0 = (size_t)blockIdx.x * 128;
    const int j0 = blockIdx.y * 64;
    const int tid = threadIdx.x, tx = tid % 16, ty = tid / 16;
    ACC acc[8][4];
#pragma unroll
    for (int a = 0; a < 8; a++)
#pragma unroll
        for (int b = 0; b < 4; b++)
            acc[a][b] = ACC(0);
    for (int kc = 0; kc < n; kc += 16)
    {
#pragma unroll
        for (int r = 0; r < 8; r++)
        {
            const int e = tid + r * 256;
            const int mm = e % 128, kk = e / 128;
            const size_t p = p0 + mm;
            const int i = kc + kk;
            As[kk][mm] = (p < npts && i < n) ? (ACC)psi[(size_t)i * ld + p] : ACC(0);
        }
#pragma unroll
        for (int r = 0; r < 4; r++)
        {
            const int e = tid + r * 256;
            const int kk = e % 16, jj = e / 16;
            const int i = kc + kk, j = j0 + jj;
            Bs[kk][jj] = (i < n && j < ncols) ? (ACC)theta[(size_t)j * ldt + i] : ACC(0);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; kk++)
        {
            ACC a[8], b[4];
#pragma unroll
            for (int q = 0; q < 8; q++) a[q] = As[kk][tx + 16 * q];
#pragma unroll
            for (int q = 0; q < 4; q++) b[q] = Bs[kk][ty + 16 * q];
#pragma unroll
            for (int u = 0; u < 8; u++)
#pragma unroll
                for (int v = 0; v < 4; v++)
                    acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int v = 0; v < 4; v++)
    {
        const int j = j0 + ty + 16 * v;
        if (j >= ncols) continue;
#pragma unroll
        for (int u = 0; u < 8; u++)
        {
            const size_t p = p0 + tx + 16 * u;
            if (p >= npts) continue;
            const size_t o = (size_t)j * ld + p;
            double r = (double)acc[u][v];
            if (beta != 0.) r += beta * (double)cin[o];
            out[o] = (T)r;
        }
    }
}

/* kind 0: FP64 orbitals; 1: FP32 orbitals, FP64 accumulation; 2: FP32
 * orbitals, FP32 accumulation */
int psi_theta_cuda_cores(int kind, const void* psi, size_t ld, size_t npts, int n,
    const double* theta, int ldt, int ncols, double beta, const void* cin, void* out,
    cudaStream_t s)
{
    if (n <= 0 || ncols <= 0 || npts == 0) return MGX_OK;
    dim3 grid((unsigned)((npts + 127) / 128), (unsigned)((ncols + 63) / 64));
    if (grid.y > 65535) return fail(MGX_UNSUPPORTED, "too many functions");
    if (kind == 0)
        psi_theta_kernel<double, double><<<grid, 256, 0, s>>>(npts, n, (const double*)psi, ld,
            theta, ldt, ncols, beta, (const double*)cin, (double*)out);
    else if (kind == 1)
        psi_theta_kernel<float, double><<<grid, 256, 0, s>>>(npts, n, (const float*)psi, ld,
            theta, ldt, ncols, beta, (const float*)cin, (float*)out);
    else
        psi_theta_kernel<float, float><<<grid, 256, 0, s>>>(npts, n, (const float*)psi, ld,
            theta, ldt, ncols, beta, (const float*)cin, (float*)out);
    MGX_LAUNCH_CHECK("psi_theta_kernel");
    return MGX_OK;
}

/* ProjectedMatrices::updateTheta (src/ProjectedMatrices.h:218-225):
 * theta = Sinv H with Sinv symmetric, read from its lower triangle. */
int theta_product(int n, const double* Sinv, const double* H, double* theta,
    cudaStream_t s)
{
    if (n <= 0 || !Sinv || !H || !theta) return fail(MGX_BAD_ARG, "theta: bad arguments");
    return dgemm(false, false, n, n, n, 1., Sinv, n, H, n, 0., theta, n, 0, s, 1);
}

/* ------------------------------------------------------------------ */
/* Cholesky                                                             */
/* ------------------------------------------------------------------ */
constexpr int NB        = 64;
constexpr int DIAG_SMEM = 2 * NB * (NB + 1) * sizeof(double);

/* Factor the diagonal block A[k0:k0+nb, k0:k0+nb] (lower), write L_kk in
 * place (upper part zeroed) and its inverse W (nb x nb, column-major, ld
 * NB) to `winv`.  Sets *info to the 1-based global pivot index on failure.
 * Right-looking by columns, the column scaled by the reciprocal of its
 * pivot (as LAPACK's dpotf2 scales); the trailing update has a thread per
 * column of the block and four row groups.  The inverse is formed row by
 * row, W(i, c) = -W(i, i) sum_{c <= q < i} L(i, q) W(q, c), four threads per
 * column summing a quarter of each dot product. */
__global__ void __launch_bounds__(256) potrf_diag_kernel(double* A, int n, int k0,
    int nb, double* winv, int* info)
{
    extern __shared__ double dsm[];
    double(*L)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dsm);
    double(*W)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dsm + NB * (NB + 1));
    __shared__ double rdiag[NB];
    __shared__ int bad;
    if (*info != 0) return;
    const int tid = threadIdx.x;
    for (int e = tid; e < NB * NB; e += blockDim.x)
    {
        const int i = e % NB, j = e / NB;
        L[i][j]     = (i >= j && i < nb && j < nb) ? A[(size_t)(k0 + j) * n + k0 + i] : 0.;
        W[i][j]     = 0.;
    }
    if (tid == 0) bad = 0;
    __syncthreads();
    const int cl = tid & 63, rg = tid >> 6;
    for (int j = 0; j < nb; j++)
    {
        if (tid == 0)
        {
            const double d = L[j][j];
            if (!(d > 0.) || !isfinite(d))
                bad = k0 + j + 1;
            else
            {
                const double sq = sqrt(d);
                L[j][j]         = sq;
                rdiag[j]        = 1. / sq;
            }
        }
        __syncthreads();
        if (bad) break;
        const double r = rdiag[j];
        for (int i = j + 1 + tid; i < nb; i += blockDim.x)
            L[i][j] *= r;
        __syncthreads();
        // trailing update of the block: column c, rows i >= c
        const int c = j + 1 + cl;
        if (c < nb)
        {
            const double lcj = L[c][j];
            for (int i = j + 1 + rg; i < nb; i += 4)
                if (i >= c) L[i][c] -= L[i][j] * lcj;
        }
        __syncthreads();
    }
    if (bad)
    {
        if (tid == 0) atomicCAS(info, 0, bad);
        return;
    }
    for (int i = tid; i < nb; i += blockDim.x)
        W[i][i] = rdiag[i];
    __syncthreads();
    {
        const int c = tid >> 2, part = tid & 3;
        for (int i = 1; i < nb; i++)
        {
            double sum = 0.;
            if (c < i)
                for (int q = c + part; q < i; q += 4)
                    sum += L[i][q] * W[q][c];
            sum += __shfl_xor_sync(0xffffffffu, sum, 1);
            sum += __shfl_xor_sync(0xffffffffu, sum, 2);
            if (c < i && part == 0) W[i][c] = -rdiag[i] * sum;
            __syncthreads();
        }
    }
    for (int e = tid; e < nb * nb; e += blockDim.x)
    {
        const int i = e % nb, j = e / nb;
        A[(size_t)(k0 + j) * n + k0 + i] = (i >= j) ? L[i][j] : 0.;
        winv[(size_t)j * NB + i]         = W[i][j];
    }
}

/* The panel of a Cholesky step in place: rows [k0 + nb, n) of columns
 * k0 .. k0+nb of A (column-major, leading dimension n) become
 * A_panel W^T, W = L_kk^-1 (lower, column-major, leading dimension NB):
 * the L_ik = A_ik L_kk^-T of the blocked algorithm.  16 rows per CTA. */
constexpr int PANEL_ROWS = 16;

__global__ void __launch_bounds__(256) panel_trsm_kernel(double* A, int n, int k0, int nb,
    const double* __restrict__ winv)
{
    __shared__ double Ws[NB][NB + 1];
    __shared__ double As[PANEL_ROWS][NB + 1];
    const int tid = threadIdx.x;
    const int r0  = k0 + nb + blockIdx.x * PANEL_ROWS;
    for (int e = tid; e < NB * NB; e += blockDim.x)
    {
        const int i = e % NB, j = e / NB;
        Ws[i][j]    = (i >= j && i < nb) ? winv[(size_t)j * NB + i] : 0.;
    }
    for (int e = tid; e < PANEL_ROWS * NB; e += blockDim.x)
    {
        const int rr = e % PANEL_ROWS, q = e / PANEL_ROWS;
        As[rr][q]    = (q < nb && r0 + rr < n) ? A[(size_t)(k0 + q) * n + r0 + rr] : 0.;
    }
    __syncthreads();
    const int rr = tid % PANEL_ROWS;
    for (int c = tid / PANEL_ROWS; c < nb; c += blockDim.x / PANEL_ROWS)
    {
        double acc = 0.;
        for (int q = 0; q <= c; q++)
            acc += As[rr][q] * Ws[c][q];
        if (r0 + rr < n) A[(size_t)(k0 + c) * n + r0 + rr] = acc;
    }
}

__global__ void copy_panel_kernel(const double* src, int lds, double* dst,
    int ldd, int m, int nb)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m * nb;
         e += gridDim.x * blockDim.x)
    {
        const int i = e % m, j = e / m;
        dst[(size_t)j * ldd + i] = src[(size_t)j * lds + i];
    }
}

__global__ void zero_upper_kernel(double* A, int n)
{
    const size_t nn = (size_t)n * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const int i = (int)(t % n), j = (int)(t / n);
        if (i < j) A[t] = 0.;
    }
}

/* workspace: diagonal inverses (nblocks x NB x NB) + panel (n x NB) + X */
static int dense_ws(mgx_ctx* ctx, int n, double** winv, double** panel,
    double** X, int** info)
{
    const int nbk = (n + NB - 1) / NB;
    const size_t b_w = (size_t)nbk * NB * NB * 8, b_p = (size_t)n * NB * 8,
                 b_x = (size_t)n * n * 8;
    MGX_TRY(ctx->dense_ws.ensure(b_w + b_p + b_x + 256));
    char* base = (char*)ctx->dense_ws.ptr;
    *winv      = (double*)base;
    *panel     = (double*)(base + b_w);
    *X         = (double*)(base + b_w + b_p);
    *info      = (int*)(base + b_w + b_p + b_x);
    return MGX_OK;
}

/* info_host set: synchronous, *info_host receives the pivot index; else
 * info_dev (device) receives it and nothing waits for the factorization */
int cholesky(mgx_ctx* ctx, int n, double* A, int* info_host, cudaStream_t s,
    int* info_dev = nullptr)
{
    if (n <= 0 || !A || (!info_host && !info_dev))
        return fail(MGX_BAD_ARG, "cholesky: bad arguments");
    double *winv, *panel, *X;
    int* dinfo;
    MGX_TRY(dense_ws(ctx, n, &winv, &panel, &X, &dinfo));
    if (info_dev) dinfo = info_dev;
    MGX_TRY(cuda_check(cudaMemsetAsync(dinfo, 0, sizeof(int), s), "info reset"));
    MGX_TRY(cuda_check(cudaFuncSetAttribute(potrf_diag_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM),
        "potrf smem attribute"));
    const int nbk = (n + NB - 1) / NB;
    for (int kb = 0; kb < nbk; kb++)
    {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        potrf_diag_kernel<<<1, 256, DIAG_SMEM, s>>>(A, n, k0, nb, winv + (size_t)kb * NB * NB, dinfo);
        MGX_LAUNCH_CHECK("potrf_diag_kernel");
        const int m = n - k0 - nb; // rows below the block
        if (m <= 0) continue;
        double* Ap = A + (size_t)k0 * n + k0 + nb; // panel A[k0+nb:, k0:k0+nb]
        // panel <- A_panel * W^T   (L_ik = A_ik L_kk^-T), in place
        panel_trsm_kernel<<<(m + PANEL_ROWS - 1) / PANEL_ROWS, 256, 0, s>>>(A, n, k0, nb,
            winv + (size_t)kb * NB * NB);
        MGX_LAUNCH_CHECK("panel_trsm_kernel");
        // trailing update A22 -= P P^T (lower)
        double* A22 = A + (size_t)(k0 + nb) * n + k0 + nb;
        MGX_TRY(dgemm(false, true, m, m, nb, -1., Ap, n, Ap, n, 1., A22, n, 1, s));
    }
    zero_upper_kernel<<<std::min<size_t>(((size_t)n * n + 255) / 256, 4096), 256, 0, s>>>(A, n);
    MGX_LAUNCH_CHECK("zero_upper_kernel");
    if (!info_host) return MGX_OK;
    int hinfo = 0;
    MGX_TRY(cuda_check(cudaMemcpyAsync(&hinfo, dinfo, sizeof(int), cudaMemcpyDeviceToHost, s),
        "info download"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "cholesky sync"));
    *info_host = hinfo;
    if (hinfo != 0) return fail(MGX_NOT_SPD, "Cholesky: leading minor %d not positive", hinfo);
    return MGX_OK;
}

/* inverse of a lower-triangular factor, blocked by rows:
 * X_ii = L_ii^-1 ; X_i,0:i = -X_ii (L_i,0:i X_0:i,0:i) */
__global__ void __launch_bounds__(256) trinv_diag_kernel(const double* L, int n,
    double* X)
{
    extern __shared__ double dsm[];
    double(*T)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dsm);
    double(*W)[NB + 1] = reinterpret_cast<double(*)[NB + 1]>(dsm + NB * (NB + 1));
    const int kb = blockIdx.x, k0 = kb * NB, nb = min(NB, n - k0);
    const int tid = threadIdx.x;
    for (int e = tid; e < nb * nb; e += blockDim.x)
    {
        const int i = e % nb, j = e / nb;
        T[i][j]     = (i >= j) ? L[(size_t)(k0 + j) * n + k0 + i] : 0.;
        W[i][j]     = 0.;
    }
    __syncthreads();
    // row by row as in potrf_diag_kernel: W(i, c) = -W(i, i) sum_{c <= q < i}
    // T(i, q) W(q, c), four threads per column
    for (int i = tid; i < nb; i += blockDim.x)
        W[i][i] = 1. / T[i][i];
    __syncthreads();
    {
        const int c = tid >> 2, part = tid & 3;
        for (int i = 1; i < nb; i++)
        {
            double sum = 0.;
            if (c < i)
                for (int q = c + part; q < i; q += 4)
                    sum += T[i][q] * W[q][c];
            sum += __shfl_xor_sync(0xffffffffu, sum, 1);
            sum += __shfl_xor_sync(0xffffffffu, sum, 2);
            if (c < i && part == 0) W[i][c] = -W[i][i] * sum;
            __syncthreads();
        }
    }
    for (int e = tid; e < nb * nb; e += blockDim.x)
    {
        const int i = e % nb, j = e / nb;
        X[(size_t)(k0 + j) * n + k0 + i] = W[i][j];
    }
}

/* forward substitution L Y = B in place on Y (n x ncols, leading dimension
 * n), with the inverses of L's diagonal blocks in the diagonal blocks of
 * X: per 64-row block, Y_k <- W_k Y_k through the panel, then the rows
 * below lose L[below, k] Y_k (one (n - k) x ncols x 64 product, parallel
 * over all of Y's columns) */
static int forward_subst(int n, const double* L, const double* X, double* Y, int ncols,
    double* panel, cudaStream_t s, bool lower_rhs = false)
{
    const int nbk = (n + NB - 1) / NB;
    for (int kb = 0; kb < nbk; kb++)
    {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        // a lower-triangular right-hand side (the identity) keeps Y lower
        // triangular: columns past this block row are still zero
        const int nc = lower_rhs ? std::min(ncols, k0 + nb) : ncols;
        MGX_TRY(dgemm(false, false, nb, nc, nb, 1., X + (size_t)k0 * n + k0, n, Y + k0, n,
            0., panel, NB, 0, s));
        copy_panel_kernel<<<std::min(1024, (nb * nc + 255) / 256), 256, 0, s>>>(panel, NB,
            Y + k0, n, nb, nc);
        MGX_LAUNCH_CHECK("copy_panel_kernel");
        const int m = n - k0 - nb;
        if (m > 0)
            MGX_TRY(dgemm(false, false, m, nc, nb, -1., L + (size_t)k0 * n + k0 + nb, n,
                Y + k0, n, 1., Y + k0 + nb, n, 0, s));
    }
    return MGX_OK;
}

// upper triangle <- lower triangle
__global__ void mirror_lower_kernel(double* A, int n)
{
    const size_t nn = (size_t)n * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t i = t % n, j = t / n;
        if (i < j) A[t] = A[i * n + j];
    }
}

__global__ void identity_kernel(double* X, int n)
{
    const size_t nn = (size_t)n * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
        X[t] = ((t % n) == (t / n)) ? 1. : 0.;
}

/* Sinv = (L L^T)^-1 = X^T X with X = L^-1 formed by forward substitution
 * on the identity (parallel over its n columns), then one product. */
int inverse_from_cholesky(mgx_ctx* ctx, int n, const double* L, double* Sinv,
    cudaStream_t s)
{
    if (n <= 0 || !L || !Sinv) return fail(MGX_BAD_ARG, "inverse: bad arguments");
    if (Sinv == L) return fail(MGX_BAD_ARG, "inverse: Sinv aliases L");
    double *winv, *panel, *X;
    int* dinfo;
    MGX_TRY(dense_ws(ctx, n, &winv, &panel, &X, &dinfo));
    const int nbk = (n + NB - 1) / NB;
    MGX_TRY(cuda_check(cudaFuncSetAttribute(trinv_diag_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM),
        "trinv smem attribute"));
    // inverses of the diagonal blocks into X, then Y = I in Sinv, solved
    trinv_diag_kernel<<<nbk, 256, DIAG_SMEM, s>>>(L, n, X);
    MGX_LAUNCH_CHECK("trinv_diag_kernel");
    const int nb = (int)std::min<size_t>(((size_t)n * n + 255) / 256, 4096);
    identity_kernel<<<nb, 256, 0, s>>>(Sinv, n);
    MGX_LAUNCH_CHECK("identity_kernel");
    MGX_TRY(forward_subst(n, L, X, Sinv, n, panel, s, true));
    // X <- L^-1, then the lower triangle of S^-1 = X^T X, mirrored
    MGX_TRY(cuda_check(cudaMemcpyAsync(X, Sinv, (size_t)n * n * 8, cudaMemcpyDeviceToDevice, s),
        "L^-1 copy"));
    MGX_TRY(dgemm(true, false, n, n, n, 1., X, n, X, n, 0., Sinv, n, 1, s));
    mirror_lower_kernel<<<nb, 256, 0, s>>>(Sinv, n);
    MGX_LAUNCH_CHECK("mirror_lower_kernel");
    return MGX_OK;
}

/* theta = S^-1 H = L^-T (L^-1 H) from the Cholesky factor L, without
 * forming S^-1: blocked forward substitution L Y = H and back substitution
 * L^T theta = Y with the n columns of H as right-hand sides.  The diagonal
 * blocks are applied through their inverses (trinv_diag_kernel); the
 * off-diagonal updates are (n - k) x n x 64 products with full-width
 * parallelism.  2 n^3 flop instead of the n^3 / 3 + 2 n^3 + 2 n^3 of
 * computeInverse followed by updateTheta (src/GramMatrix.cc:75-91,
 * src/ProjectedMatrices.h:218-225).  trace (device, may be NULL) receives
 * tr(theta) = tr(S^-1 H). */
__global__ void diag_sum_kernel(const double* __restrict__ A, int n, double* __restrict__ out)
{
    __shared__ double red[256];
    double acc = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        acc += A[(size_t)i * n + i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int theta_from_cholesky(mgx_ctx* ctx, int n, const double* L, const double* H,
    double* theta, double* trace, cudaStream_t s)
{
    if (n <= 0 || !L || !H || !theta) return fail(MGX_BAD_ARG, "theta: bad arguments");
    if (theta == H || theta == L) return fail(MGX_BAD_ARG, "theta aliases an input");
    double *winv, *panel, *X;
    int* dinfo;
    MGX_TRY(dense_ws(ctx, n, &winv, &panel, &X, &dinfo));
    const int nbk = (n + NB - 1) / NB;
    MGX_TRY(cuda_check(cudaFuncSetAttribute(trinv_diag_kernel,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, DIAG_SMEM),
        "trinv smem attribute"));
    trinv_diag_kernel<<<nbk, 256, DIAG_SMEM, s>>>(L, n, X);
    MGX_LAUNCH_CHECK("trinv_diag_kernel");
    MGX_TRY(cuda_check(cudaMemcpyAsync(theta, H, (size_t)n * n * 8, cudaMemcpyDeviceToDevice, s),
        "theta init"));
    auto apply_diag = [&](int k0, int nb, bool transpose) -> int {
        // rows k0..k0+nb of theta <- W^(T) * rows k0..k0+nb, through the panel
        MGX_TRY(dgemm(transpose, false, nb, n, nb, 1., X + (size_t)k0 * n + k0, n, theta + k0,
            n, 0., panel, NB, 0, s));
        copy_panel_kernel<<<std::min(1024, (nb * n + 255) / 256), 256, 0, s>>>(panel, NB,
            theta + k0, n, nb, n);
        MGX_LAUNCH_CHECK("copy_panel_kernel");
        return MGX_OK;
    };
    // forward: L Y = H
    MGX_TRY(forward_subst(n, L, X, theta, n, panel, s));
    // backward: L^T theta = Y
    for (int kb = nbk - 1; kb >= 0; kb--)
    {
        const int k0 = kb * NB, nb = std::min(NB, n - k0);
        MGX_TRY(apply_diag(k0, nb, true));
        if (k0 > 0)
            MGX_TRY(dgemm(true, false, k0, n, nb, -1., L + k0, n, theta + k0, n, 1., theta, n,
                0, s));
    }
    if (trace)
    {
        diag_sum_kernel<<<1, 256, 0, s>>>(theta, n, trace);
        MGX_LAUNCH_CHECK("diag_sum_kernel");
    }
    return MGX_OK;
}

/* tr(H Sinv) with both matrices symmetric and read from their lower
 * triangles: sum_k [H(k,k) S(k,k) + 2 sum_{i>k} H(i,k) S(i,k)], columns
 * spread over the blocks (coalesced column reads), one partial per block,
 * then a fixed-order sum of the partials. */
constexpr int TRACE_BLOCKS = 256;

__global__ void __launch_bounds__(256) trace_partial_kernel(const double* __restrict__ H,
    const double* __restrict__ Sinv, int n, double* __restrict__ part)
{
    __shared__ double red[256];
    double acc = 0.;
    for (int k = blockIdx.x; k < n; k += gridDim.x)
    {
        const double* h = H + (size_t)k * n;
        const double* q = Sinv + (size_t)k * n;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x)
            acc += (i == k ? 1. : 2.) * h[i] * q[i];
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void __launch_bounds__(256) trace_sum_kernel(const double* __restrict__ part, int n,
    double* __restrict__ out)
{
    __shared__ double red[256];
    double acc = 0.;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        acc += part[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = red[0];
}

int trace_prod(mgx_ctx* ctx, int n, const double* H, const double* Sinv, double* out,
    cudaStream_t s)
{
    if (n <= 0 || !H || !Sinv || !out) return fail(MGX_BAD_ARG, "trace: bad arguments");
    MGX_TRY(ctx->red.ensure(TRACE_BLOCKS * sizeof(double)));
    double* part = (double*)ctx->red.ptr;
    trace_partial_kernel<<<TRACE_BLOCKS, 256, 0, s>>>(H, Sinv, n, part);
    MGX_LAUNCH_CHECK("trace_partial_kernel");
    trace_sum_kernel<<<1, 256, 0, s>>>(part, TRACE_BLOCKS, out);
    MGX_LAUNCH_CHECK("trace_sum_kernel");
    return MGX_OK;
}

/* ProjectedMatricesMehrstellen::updateHB
 * (src/ProjectedMatricesMehrstellen.h:55-62): HB = S theta with S read as
 * symmetric from its lower triangle (symm 'l', 'l'), then
 * HB = 0.5 HB + 0.5 HB^T (the transpose(0.5, copy, 0.5) of the reference);
 * element (i, j) and (j, i) receive the same sum 0.5 a_ij + 0.5 a_ji. */
__global__ void sym_average_kernel(double* A, int n)
{
    const size_t nn = (size_t)n * n;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const int i = (int)(t % n), j = (int)(t / n);
        if (i <= j) continue;
        const double x = 0.5 * A[(size_t)j * n + i] + 0.5 * A[(size_t)i * n + j];
        A[(size_t)j * n + i] = x;
        A[(size_t)i * n + j] = x;
    }
}

int update_hb(int n, const double* S, const double* theta, double* HB, cudaStream_t s)
{
    if (n <= 0 || !S || !theta || !HB) return fail(MGX_BAD_ARG, "updateHB: bad arguments");
    if (HB == S || HB == theta) return fail(MGX_BAD_ARG, "HB aliases an input");
    MGX_TRY(dgemm(false, false, n, n, n, 1., S, n, theta, n, 0., HB, n, 0, s, 1));
    const int nb = (int)std::min<size_t>(((size_t)n * n + 255) / 256, 4096);
    sym_average_kernel<<<nb, 256, 0, s>>>(HB, n);
    MGX_LAUNCH_CHECK("sym_average_kernel");
    return MGX_OK;
}

/* LocGridOrbitals::normalize (src/LocGridOrbitals.cc:2230-2311, the branch
 * without short-sighted matrices): diagS_i = vel * psi_i . psi_i with FP64
 * accumulation (BlockVector::dot -> MPdot, src/linear_algebra/mputils.cc:
 * 145-166), then psi_i <- (T)(diagS_i^-1/2 * (double)psi_i) (MPscal,
 * mputils.cc:61-80).  The dot products are deterministic: NORM_BLOCKS
 * partial sums per function, then a fixed-order sum. */
constexpr int NORM_BLOCKS = 64;

template <typename T>
__global__ void __launch_bounds__(256) sumsq_partial_kernel(const T* __restrict__ psi,
    size_t ld, size_t npts, double* __restrict__ part)
{
    __shared__ double red[256];
    const int f    = blockIdx.y;
    const T* p     = psi + (size_t)f * ld;
    double acc     = 0.;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const double v = (double)p[i];
        acc += v * v;
    }
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[(size_t)f * gridDim.x + blockIdx.x] = red[0];
}

// one thread per function: diagS = vel * sum of the partials; alpha =
// 1 / sqrt(diagS); a diagS <= 1e-15 (the reference asserts) raises *bad
__global__ void norm_finish_kernel(const double* __restrict__ part, int nblk, int nfunc,
    double vel, double* __restrict__ diag, double* __restrict__ alpha, int* bad)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfunc) return;
    double acc = 0.;
    for (int b = 0; b < nblk; b++)
        acc += part[(size_t)f * nblk + b];
    const double d = vel * acc;
    if (diag) diag[f] = d;
    if (!(d > 1.e-15))
    {
        atomicExch(bad, 1);
        alpha[f] = 1.;
    }
    else
        alpha[f] = 1. / sqrt(d);
}

// psi_f <- (T)(alpha_f * (double)psi_f), skipped entirely when *bad is set
template <typename T>
__global__ void __launch_bounds__(256) scale_columns_kernel(T* __restrict__ psi, size_t ld,
    size_t npts, const double* __restrict__ alpha, const int* __restrict__ bad)
{
    if (bad && *bad) return;
    const int f    = blockIdx.y;
    const double a = alpha[f];
    T* p           = psi + (size_t)f * ld;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
        p[i] = (T)(a * (double)p[i]);
}

int normalize(mgx_ctx* ctx, int dtype, void* psi, size_t ld, size_t npts, int nfunc,
    double vel, double* diag, cudaStream_t s)
{
    if (nfunc <= 0) return MGX_OK;
    if (nfunc > 65535) return fail(MGX_UNSUPPORTED, "normalize: more than 65535 functions");
    const size_t part_bytes = (size_t)nfunc * NORM_BLOCKS * sizeof(double);
    MGX_TRY(ctx->red.ensure(part_bytes + (size_t)nfunc * sizeof(double) + 256));
    double* part  = (double*)ctx->red.ptr;
    double* alpha = part + (size_t)nfunc * NORM_BLOCKS;
    int* bad      = (int*)(alpha + nfunc);
    MGX_TRY(cuda_check(cudaMemsetAsync(bad, 0, sizeof(int), s), "normalize flag"));
    dim3 grid(NORM_BLOCKS, nfunc);
    if (dtype == MGX_F64)
        sumsq_partial_kernel<double><<<grid, 256, 0, s>>>((const double*)psi, ld, npts, part);
    else
        sumsq_partial_kernel<float><<<grid, 256, 0, s>>>((const float*)psi, ld, npts, part);
    MGX_LAUNCH_CHECK("sumsq_partial_kernel");
    norm_finish_kernel<<<(nfunc + 127) / 128, 128, 0, s>>>(part, NORM_BLOCKS, nfunc, vel, diag,
        alpha, bad);
    MGX_LAUNCH_CHECK("norm_finish_kernel");
    const int sblk = (int)std::min<size_t>((npts + 255) / 256, 256);
    dim3 sgrid(sblk, nfunc);
    if (dtype == MGX_F64)
        scale_columns_kernel<double><<<sgrid, 256, 0, s>>>((double*)psi, ld, npts, alpha, bad);
    else
        scale_columns_kernel<float><<<sgrid, 256, 0, s>>>((float*)psi, ld, npts, alpha, bad);
    MGX_LAUNCH_CHECK("scale_columns_kernel");
    int hbad = 0;
    MGX_TRY(cuda_check(cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s),
        "normalize flag read"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "normalize sync"));
    if (hbad) return fail(MGX_NOT_SPD, "normalize: a function with vel * |psi|^2 <= 1e-15");
    return MGX_OK;
}

/* d_i = 1 / sqrt(S(i, i)): the normalization factors of the functions
 * whose Gram matrix is S (LocGridOrbitals::normalize takes the same
 * diagonal from its own dot products) */
__global__ void diag_rsqrt_kernel(const double* __restrict__ S, int n, double* __restrict__ d)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) d[i] = 1. / sqrt(S[(size_t)i * n + i]);
}

int diag_rsqrt(mgx_ctx*, int n, const double* S, double* d, cudaStream_t s)
{
    if (n <= 0 || !S || !d) return fail(MGX_BAD_ARG, "diag_rsqrt: bad arguments");
    diag_rsqrt_kernel<<<(n + 255) / 256, 256, 0, s>>>(S, n, d);
    MGX_LAUNCH_CHECK("diag_rsqrt_kernel");
    return MGX_OK;
}

} // namespace mgx
