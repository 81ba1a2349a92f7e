// Centres and spreads of the orbitals (SpreadsAndCenters with
// SinCosOps::computeDiag, src/SpreadsAndCenters.cc:26-104,
// src/SinCosOps.cc:733-826): the diagonal matrix elements
//   a_k(i) = vel sum_p psi_i(p)^2 t_k(p),
// t = (cos x, sin x, cos y, sin y, cos z, sin z) scaled by L / (2 pi) per
// direction (pb::Grid::getSinCosFunctions, src/pb/Grid.cc:244-282), divided
// by the norm vel sum psi_i^2 unless the functions are normalized.  The
// centre of orbital i along x is L / (2 pi) atan2(a_1, a_0) mod L and its
// squared spread (L / (2 pi))^2 - a_0^2 - a_1^2.
//
// One pass over the block (the block is read once): warps take z rows of a
// function and accumulate the seven sums, FP32 orbitals in double-float
// arithmetic on the FP32 units (GB300's FP64 rate would bound a plain FP64
// loop far below HBM speed), FP64 orbitals in FP64; the per-block partials
// are summed in a fixed order, so the result is the same on every run.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx
{
namespace cen
{
constexpr int THREADS = 256;
constexpr int NSUM    = 7; // six trigonometric sums and the squared norm

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

/* partial[(f * nblk + b) * NSUM + k]: block b's sums of function f.  A
 * warp takes whole z rows (grid-stride over the rows of the function); the
 * x and y factors are constant along a row, so a row contributes
 * cos x * sum a, ..., sin y * sum a, sum a cos z, sum a sin z and sum a,
 * a = psi^2.  The tables are tab[0..nx) cos x, then sin x, cos y, sin y,
 * cos z, sin z. */
template <typename T>
__global__ void __launch_bounds__(THREADS) sincos_partial_kernel(const T* __restrict__ psi,
    size_t ld, int nx, int ny, int nz, const double* __restrict__ tab,
    double* __restrict__ partial)
{
    const int f    = blockIdx.y;
    const int nblk = gridDim.x;
    const T* p     = psi + (size_t)f * ld;
    const double *cx = tab, *sx = tab + nx, *cy = tab + 2 * nx, *sy = cy + ny,
                 *cz = tab + 2 * nx + 2 * ny, *sz = cz + nz;
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    constexpr int WPB = THREADS / 32;
    double acc[NSUM] = { 0., 0., 0., 0., 0., 0., 0. };
    const int nrows = nx * ny;
    for (int r = blockIdx.x * WPB + w; r < nrows; r += nblk * WPB)
    {
        const int ix = r / ny, iy = r - ix * ny;
        const T* row = p + (size_t)r * nz;
        double ra = 0., rc = 0., rs = 0.;
        for (int iz = l; iz < nz; iz += 32)
        {
            const double v = (double)row[iz];
            const double a = v * v;
            ra += a;
            rc += a * cz[iz];
            rs += a * sz[iz];
        }
        acc[0] += cx[ix] * ra;
        acc[1] += sx[ix] * ra;
        acc[2] += cy[iy] * ra;
        acc[3] += sy[iy] * ra;
        acc[4] += rc;
        acc[5] += rs;
        acc[6] += ra;
    }
    __shared__ double red[WPB][NSUM];
#pragma unroll
    for (int k = 0; k < NSUM; k++)
    {
        const double s = warp_sum(acc[k]);
        if (l == 0) red[w][k] = s;
    }
    __syncthreads();
    if (threadIdx.x < NSUM)
    {
        double s = 0.;
        for (int q = 0; q < WPB; q++)
            s += red[q][threadIdx.x];
        partial[((size_t)f * nblk + blockIdx.x) * NSUM + threadIdx.x] = s;
    }
}

/* s + e = a + b exactly (Knuth's two-sum; the _rn intrinsics are never
 * contracted into FMAs, which would break the identity) */
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e)
{
    s              = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e              = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

/* The FP32 form of the partial sums, at FP64 accuracy on the FP32 units:
 * psi^2 = ah + al exactly (al by an FMA); each lane keeps, for the z
 * indices it owns (l + 32 j, j < ZPL), the double-float sum over its rows
 * of psi^2 (the z profile) in registers, and the warp forms each row's
 * double-float total with a butterfly of two-sums, which lane 0 stores as
 * one FP64 value in rowsum (the x and y weights are applied to those by
 * sincos_rows_kernel, off this loop).  The z weights are applied to the z
 * profile at the end; the other sums of this kernel's partials are 0.
 * Needs nz <= 32 ZPL. */
constexpr int ZPL  = 8;
constexpr int MAXZ = 32 * ZPL;

__global__ void __launch_bounds__(THREADS) sincos_partial_f32_kernel(const float* __restrict__ psi,
    size_t ld, int nx, int ny, int nz, const double* __restrict__ tab,
    double* __restrict__ partial, double* __restrict__ rowsum)
{
    constexpr int WPB = THREADS / 32;
    const int f       = blockIdx.y;
    const int nblk    = gridDim.x;
    const float* p    = psi + (size_t)f * ld;
    const double *cz = tab + 2 * nx + 2 * ny, *sz = cz + nz;
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    float zh[ZPL], zl[ZPL];
#pragma unroll
    for (int j = 0; j < ZPL; j++)
        zh[j] = zl[j] = 0.f;
    const int nrows = nx * ny;
    for (int r = blockIdx.x * WPB + w; r < nrows; r += nblk * WPB)
    {
        const float* row = p + (size_t)r * nz;
        float rh = 0.f, rl = 0.f;
#pragma unroll
        for (int j = 0; j < ZPL; j++)
        {
            const int iz = l + 32 * j;
            if (iz < nz)
            {
                const float v  = row[iz];
                const float ah = __fmul_rn(v, v);
                const float al = fmaf(v, v, -ah);
                float s, e;
                two_sum(rh, ah, s, e);
                rh = s;
                rl += e + al;
                two_sum(zh[j], ah, s, e);
                zh[j] = s;
                zl[j] += e + al;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            const float oh = __shfl_xor_sync(0xffffffffu, rh, o);
            const float ol = __shfl_xor_sync(0xffffffffu, rl, o);
            float s, e;
            two_sum(rh, oh, s, e);
            rh = s;
            rl += ol + e;
        }
        if (l == 0) rowsum[(size_t)f * nrows + r] = (double)rh + (double)rl;
    }
    // the z weights on this lane's part of the z profile
    double c4 = 0., c5 = 0.;
#pragma unroll
    for (int j = 0; j < ZPL; j++)
    {
        const int iz = l + 32 * j;
        if (iz < nz)
        {
            const double z = (double)zh[j] + (double)zl[j];
            c4 += cz[iz] * z;
            c5 += sz[iz] * z;
        }
    }
    __shared__ double red[WPB][NSUM];
    const double vals[NSUM] = { 0., 0., 0., 0., c4, c5, 0. };
#pragma unroll
    for (int k = 0; k < NSUM; k++)
    {
        const double v = warp_sum(vals[k]);
        if (l == 0) red[w][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < NSUM)
    {
        double t = 0.;
        for (int q = 0; q < WPB; q++)
            t += red[q][threadIdx.x];
        partial[((size_t)f * nblk + blockIdx.x) * NSUM + threadIdx.x] = t;
    }
}

/* the x and y weights on the row totals of sincos_partial_f32_kernel, one
 * block per function, rows in a fixed order per thread and a fixed-order
 * block sum; added into block 0's partials of sums 0-3 and 6 */
__global__ void __launch_bounds__(THREADS) sincos_rows_kernel(const double* __restrict__ rowsum,
    int nx, int ny, const double* __restrict__ tab, int nblk, double* __restrict__ partial)
{
    const int f      = blockIdx.x;
    const int nrows  = nx * ny;
    const double* rs = rowsum + (size_t)f * nrows;
    const double *cx = tab, *sx = tab + nx, *cy = tab + 2 * nx, *sy = cy + ny;
    double acc[5] = { 0., 0., 0., 0., 0. };
    for (int r = threadIdx.x; r < nrows; r += THREADS)
    {
        const int ix = r / ny, iy = r - ix * ny;
        const double t = rs[r];
        acc[0] += cx[ix] * t;
        acc[1] += sx[ix] * t;
        acc[2] += cy[iy] * t;
        acc[3] += sy[iy] * t;
        acc[4] += t;
    }
    constexpr int WPB = THREADS / 32;
    __shared__ double red[WPB][5];
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
#pragma unroll
    for (int k = 0; k < 5; k++)
    {
        const double v = warp_sum(acc[k]);
        if (l == 0) red[w][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 5)
    {
        double t = 0.;
        for (int q = 0; q < WPB; q++)
            t += red[q][threadIdx.x];
        const int k = threadIdx.x < 4 ? threadIdx.x : 6;
        partial[(size_t)f * nblk * NSUM + k] += t;
    }
}

/* out[f * 6 + k] = vel * sum_b partial[f][b][k] (/ the norm unless the
 * functions are normalized), the partials of a function in block order */
__global__ void sincos_finish_kernel(const double* __restrict__ partial, int nblk, int nfunc,
    double vel, int normalized, double* __restrict__ out)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nfunc) return;
    double s[NSUM] = { 0., 0., 0., 0., 0., 0., 0. };
    for (int b = 0; b < nblk; b++)
        for (int k = 0; k < NSUM; k++)
            s[k] += partial[((size_t)f * nblk + b) * NSUM + k];
    // normalized: a = vel sum; else (vel sum) / (vel sum psi^2), as the
    // reference scales by 1 / diag(S) before its final scaling by vel
    const double scale = normalized ? vel : vel / (vel * s[6]);
    for (int k = 0; k < 6; k++)
        out[(size_t)f * 6 + k] = s[k] * scale;
}

} // namespace cen
} // namespace mgx

using namespace mgx;

extern "C" {

int mgx_sincos_diag(mgx_ctx* ctx, mgx_dtype dtype, const void* psi, size_t ld, int nfunc,
    int normalized, double* out, void* stream)
{
    if (!ctx || (nfunc > 0 && (!psi || !out)) || nfunc < 0)
        return fail(MGX_BAD_ARG, "sincos: NULL argument");
    if (dtype != MGX_F32 && dtype != MGX_F64) return fail(MGX_BAD_ARG, "sincos: dtype");
    const mgx_grid& g = ctx->grid;
    const size_t np   = (size_t)g.n[0] * g.n[1] * g.n[2];
    if (nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "sincos: ld %zu < %zu points", ld, np);
    if (nfunc == 0) return MGX_OK;
    if (ld == 0) ld = np;
    const cudaStream_t s = (cudaStream_t)stream;
    // the tables of pb::Grid::getSinCosFunctions, cos / sin (i 2 pi / n) L / (2 pi),
    // uploaded once per context
    const size_t ntab = 2 * ((size_t)g.n[0] + g.n[1] + g.n[2]);
    if (ctx->sincos.bytes < ntab * sizeof(double))
    {
        std::vector<double> tab(ntab);
        size_t o = 0;
        for (int d = 0; d < 3; d++)
        {
            const double alpha = g.ll[d] * (0.5 * M_1_PI);
            const double hh    = 2. * M_PI / (double)g.n[d];
            for (int i = 0; i < g.n[d]; i++)
                tab[o + i] = std::cos(double(i) * hh) * alpha;
            for (int i = 0; i < g.n[d]; i++)
                tab[o + g.n[d] + i] = std::sin(double(i) * hh) * alpha;
            o += 2 * (size_t)g.n[d];
        }
        MGX_TRY(ctx->sincos.ensure(ntab * sizeof(double)));
        MGX_TRY(cuda_check(cudaMemcpy(ctx->sincos.ptr, tab.data(), ntab * sizeof(double),
                               cudaMemcpyHostToDevice),
            "sincos tables"));
    }
    const double* dtab = (const double*)ctx->sincos.ptr;
    // about eight blocks per SM in all, at most one warp per z row
    const int nrows = g.n[0] * g.n[1];
    const int wpb   = cen::THREADS / 32;
    const int nblk  = std::max(1, std::min((nrows + wpb - 1) / wpb,
                                     (8 * ctx->sm_count + nfunc - 1) / nfunc));
    const size_t part_bytes = (size_t)nfunc * nblk * cen::NSUM * sizeof(double);
    const bool f32 = (dtype == MGX_F32 && g.n[2] <= cen::MAXZ);
    MGX_TRY(ctx->red.ensure(part_bytes + (f32 ? (size_t)nfunc * nrows * sizeof(double) : 0)));
    double* part   = (double*)ctx->red.ptr;
    double* rowsum = (double*)((char*)ctx->red.ptr + part_bytes);
    const dim3 grid(nblk, nfunc);
    if (f32)
    {
        cen::sincos_partial_f32_kernel<<<grid, cen::THREADS, 0, s>>>((const float*)psi, ld,
            g.n[0], g.n[1], g.n[2], dtab, part, rowsum);
        MGX_LAUNCH_CHECK("sincos_partial_f32_kernel");
        cen::sincos_rows_kernel<<<nfunc, cen::THREADS, 0, s>>>(rowsum, g.n[0], g.n[1], dtab, nblk,
            part);
        MGX_LAUNCH_CHECK("sincos_rows_kernel");
    }
    else
    {
        if (dtype == MGX_F64)
            cen::sincos_partial_kernel<double><<<grid, cen::THREADS, 0, s>>>((const double*)psi,
                ld, g.n[0], g.n[1], g.n[2], dtab, part);
        else
            cen::sincos_partial_kernel<float><<<grid, cen::THREADS, 0, s>>>((const float*)psi,
                ld, g.n[0], g.n[1], g.n[2], dtab, part);
        MGX_LAUNCH_CHECK("sincos_partial_kernel");
    }
    const double vel = (g.ll[0] / g.n[0]) * (g.ll[1] / g.n[1]) * (g.ll[2] / g.n[2]);
    cen::sincos_finish_kernel<<<(nfunc + 127) / 128, 128, 0, s>>>(part, nblk, nfunc, vel,
        normalized ? 1 : 0, out);
    MGX_LAUNCH_CHECK("sincos_finish_kernel");
    return MGX_OK;
}

} // extern "C"
