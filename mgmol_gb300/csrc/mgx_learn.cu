// Learned preconditioner of the orbital residual: a 3-level 3-D
// convolutional U-Net whose forward pass, backward pass and Adam update
// run as the kernels of this file, and its use as a correction of the
// residual with the plain V-cycle (mgx_mg.cu) as per-function fallback.
//
// Fields are the library's ghost-free periodic blocks: point (x, y, z) of
// an n0 x n1 x n2 level at (x * n1 + y) * n2 + z.  An activation block of
// nf functions and C channels is [f][c][points], so that its nf * C fields
// go through the V-cycle's restriction and prolongation unchanged.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{
int precond_mg(mgx_ctx*, const mgx_precond_params*, int, const void*, size_t, void*, int,
    const mgx_masks*, cudaStream_t, void*, double, const double*, bool);
int restrict_launch(int, const Level&, const void*, size_t, void*, size_t, int,
    const MaskDev&, cudaStream_t);
int prolong_launch(int, int, const Level&, const void*, size_t, void*, size_t, int,
    const MaskDev&, cudaStream_t);

namespace nn
{
constexpr int NLAYER = 6;
struct LayerDef
{
    int cin, cout, level;
};
// E0, E1, E2, D2, D1, D0
constexpr LayerDef LAYERS[NLAYER] = { { 1, 16, 0 }, { 16, 32, 1 }, { 32, 64, 2 },
    { 64, 32, 2 }, { 32, 16, 1 }, { 16, 1, 0 } };
constexpr size_t layer_size(int l) { return (size_t)LAYERS[l].cin * LAYERS[l].cout * 27; }
inline size_t layer_offset(int l)
{
    size_t o = 0;
    for (int i = 0; i < l; i++)
        o += layer_size(i);
    return o;
}
constexpr size_t NPARAM = 139104;
static_assert(NPARAM == MGX_UNET_PARAMS, "parameter count");

// output tile of a convolution block: TXP x TY x TZ points, one thread per
// (y, z) column computing TXP points along x
constexpr int TY = 8, TZ = 32, THREADS = TY * TZ;

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

/* stages the periodic halo tile (TXP + 2) x (TY + 2) x (TZ + 2) of CI
 * channels starting at channel c0 of function block x (channel stride
 * npts) into xs */
template <int CI, int TXP>
__device__ __forceinline__ void stage_halo(float* xs, const float* __restrict__ x, int c0,
    size_t npts, int nx, int ny, int nz, int x0, int y0, int z0)
{
    constexpr int HY = TY + 2, HZ = TZ + 2, HP = (TXP + 2) * HY * HZ;
    for (int c = 0; c < CI; c++)
    {
        const float* src = x + (size_t)(c0 + c) * npts;
        for (int h = threadIdx.x; h < HP; h += THREADS)
        {
            const int hz = h % HZ, r = h / HZ, hy = r % HY, hx = r / HY;
            const int gx = wrapi(x0 - 1 + hx, nx), gy = wrapi(y0 - 1 + hy, ny),
                      gz = wrapi(z0 - 1 + hz, nz);
            xs[c * HP + h] = src[((size_t)gx * ny + gy) * nz + gz];
        }
    }
}

/* y[f][co] = act(oscale[f] * sum_{ci, t} W[co][ci][t] x[f][ci][p + off(t)]),
 * a periodic 3x3x3 cross-correlation; CO output channels per block
 * (blockIdx.y = f * (cout / CO) + output block), CI input channels staged
 * at a time.  xf / yf: function strides of x and y. */
template <int CI, int CO, int TXP>
__global__ void __launch_bounds__(THREADS) conv_fwd_kernel(const float* __restrict__ x,
    size_t xf, int cin, const __nv_bfloat16* __restrict__ W, float* __restrict__ y, size_t yf,
    int cout, int nx, int ny, int nz, int relu, const float* __restrict__ oscale)
{
    constexpr int HY = TY + 2, HZ = TZ + 2, HP = (TXP + 2) * HY * HZ;
    extern __shared__ __align__(16) float smem[];
    float* xs = smem;           // CI * HP
    float* ws = smem + CI * HP; // [c][tap][co]
    const int ntz = (nz + TZ - 1) / TZ, nty = (ny + TY - 1) / TY;
    int t          = blockIdx.x;
    const int z0   = (t % ntz) * TZ;
    t /= ntz;
    const int y0   = (t % nty) * TY;
    const int x0   = (t / nty) * TXP;
    const int ncob = cout / CO;
    const int f    = blockIdx.y / ncob, cob = blockIdx.y % ncob;
    const size_t npts = (size_t)nx * ny * nz;
    const int ty = threadIdx.x / TZ, tz = threadIdx.x % TZ;
    const float* xb = x + (size_t)f * xf;

    float acc[TXP][CO];
#pragma unroll
    for (int p = 0; p < TXP; p++)
#pragma unroll
        for (int o = 0; o < CO; o++)
            acc[p][o] = 0.f;

    for (int ci0 = 0; ci0 < cin; ci0 += CI)
    {
        __syncthreads();
        stage_halo<CI, TXP>(xs, xb, ci0, npts, nx, ny, nz, x0, y0, z0);
        for (int i = threadIdx.x; i < CI * 27 * CO; i += THREADS)
        {
            const int o = i % CO, r = i / CO, tap = r % 27, c = r / 27;
            ws[i] = __bfloat162float(W[((size_t)(cob * CO + o) * cin + ci0 + c) * 27 + tap]);
        }
        __syncthreads();
#pragma unroll 1
        for (int c = 0; c < CI; c++)
        {
            const float* xt = xs + c * HP;
            const float* wc = ws + c * 27 * CO;
#pragma unroll
            for (int dy = 0; dy < 3; dy++)
#pragma unroll
                for (int dz = 0; dz < 3; dz++)
                {
                    float col[TXP + 2];
#pragma unroll
                    for (int i = 0; i < TXP + 2; i++)
                        col[i] = xt[(i * HY + ty + dy) * HZ + tz + dz];
#pragma unroll
                    for (int dx = 0; dx < 3; dx++)
                    {
                        const float* wv = wc + (dx * 9 + dy * 3 + dz) * CO;
                        if constexpr (CO % 4 == 0)
                        {
#pragma unroll
                            for (int q = 0; q < CO / 4; q++)
                            {
                                const float4 w4 = reinterpret_cast<const float4*>(wv)[q];
#pragma unroll
                                for (int p = 0; p < TXP; p++)
                                {
                                    const float v = col[p + dx];
                                    acc[p][4 * q + 0] = fmaf(w4.x, v, acc[p][4 * q + 0]);
                                    acc[p][4 * q + 1] = fmaf(w4.y, v, acc[p][4 * q + 1]);
                                    acc[p][4 * q + 2] = fmaf(w4.z, v, acc[p][4 * q + 2]);
                                    acc[p][4 * q + 3] = fmaf(w4.w, v, acc[p][4 * q + 3]);
                                }
                            }
                        }
                        else
                        {
#pragma unroll
                            for (int o = 0; o < CO; o++)
                            {
                                const float w = wv[o];
#pragma unroll
                                for (int p = 0; p < TXP; p++)
                                    acc[p][o] = fmaf(w, col[p + dx], acc[p][o]);
                            }
                        }
                    }
                }
        }
    }
    const float sc = oscale ? oscale[f] : 1.f;
    const int gy = y0 + ty, gz = z0 + tz;
    if (gy >= ny || gz >= nz) return;
    float* yb = y + (size_t)f * yf + (size_t)cob * CO * npts;
#pragma unroll
    for (int p = 0; p < TXP; p++)
    {
        const int gx = x0 + p;
        if (gx >= nx) break;
        const size_t idx = ((size_t)gx * ny + gy) * nz + gz;
#pragma unroll
        for (int o = 0; o < CO; o++)
        {
            float v = acc[p][o] * sc;
            if (relu) v = fmaxf(v, 0.f);
            yb[(size_t)o * npts + idx] = v;
        }
    }
}

/* dW[co][ci][t] += sum_{f, p} dy[f][co][p] x[f][ci][p + off(t)] over the
 * points of the blocks' tiles (TXW = 2 planes of x).  A thread owns one
 * (input channel, tap) pair and CO output channels; PS threads split the
 * points of a tile between them.  blockIdx.y = output block * (cin / CI)
 * + input block; blocks stride over (function, tile) items. */
constexpr int TXW = 2;
template <int CI, int CO, int PS>
__global__ void __launch_bounds__(THREADS) conv_wgrad_kernel(const float* __restrict__ x,
    int cin, const float* __restrict__ dy, int cout, float* __restrict__ dW, int nf, int nx,
    int ny, int nz)
{
    static_assert(CI * 27 * PS <= THREADS, "threads");
    constexpr int HY = TY + 2, HZ = TZ + 2, HP = (TXW + 2) * HY * HZ, NP = TXW * TY * TZ;
    extern __shared__ __align__(16) float smem[];
    float* xs  = smem;           // CI * HP
    float* dys = smem + CI * HP; // [p][co]
    const int ncib = cin / CI;
    const int cob = blockIdx.y / ncib, cib = blockIdx.y % ncib;
    const int q = threadIdx.x % (CI * 27), sp = threadIdx.x / (CI * 27);
    const bool active = sp < PS;
    const int c = q / 27, tap = q % 27;
    const int dx = tap / 9, dyy = (tap / 3) % 3, dz = tap % 3;
    const int ntz = (nz + TZ - 1) / TZ, nty = (ny + TY - 1) / TY, ntx = (nx + TXW - 1) / TXW;
    const int ntiles  = ntx * nty * ntz;
    const size_t npts = (size_t)nx * ny * nz;
    float acc[CO];
#pragma unroll
    for (int o = 0; o < CO; o++)
        acc[o] = 0.f;
    for (int item = blockIdx.x; item < nf * ntiles; item += gridDim.x)
    {
        const int f = item / ntiles;
        int t       = item % ntiles;
        const int z0 = (t % ntz) * TZ;
        t /= ntz;
        const int y0 = (t % nty) * TY;
        const int x0 = (t / nty) * TXW;
        __syncthreads();
        stage_halo<CI, TXW>(xs, x + (size_t)f * cin * npts, cib * CI, npts, nx, ny, nz, x0, y0,
            z0);
        for (int i = threadIdx.x; i < NP * CO; i += THREADS)
        {
            const int p = i % NP, o = i / NP;
            const int px = x0 + p / (TY * TZ), py = y0 + (p / TZ) % TY, pz = z0 + p % TZ;
            float v = 0.f;
            if (px < nx && py < ny && pz < nz)
                v = dy[((size_t)f * cout + cob * CO + o) * npts + ((size_t)px * ny + py) * nz + pz];
            dys[p * CO + o] = v;
        }
        __syncthreads();
        if (active)
        {
            const float* xt = xs + c * HP + (dx * HY + dyy) * HZ + dz;
            for (int p = sp; p < NP; p += PS)
            {
                const int px = p / (TY * TZ), py = (p / TZ) % TY, pz = p % TZ;
                const float xv = xt[(px * HY + py) * HZ + pz];
                const float* dv = dys + p * CO;
                if constexpr (CO % 4 == 0)
                {
#pragma unroll
                    for (int o4 = 0; o4 < CO / 4; o4++)
                    {
                        const float4 d4 = reinterpret_cast<const float4*>(dv)[o4];
                        acc[4 * o4 + 0] = fmaf(d4.x, xv, acc[4 * o4 + 0]);
                        acc[4 * o4 + 1] = fmaf(d4.y, xv, acc[4 * o4 + 1]);
                        acc[4 * o4 + 2] = fmaf(d4.z, xv, acc[4 * o4 + 2]);
                        acc[4 * o4 + 3] = fmaf(d4.w, xv, acc[4 * o4 + 3]);
                    }
                }
                else
                {
#pragma unroll
                    for (int o = 0; o < CO; o++)
                        acc[o] = fmaf(dv[o], xv, acc[o]);
                }
            }
        }
    }
    if (!active) return;
#pragma unroll
    for (int o = 0; o < CO; o++)
        atomicAdd(&dW[((size_t)(cob * CO + o) * cin + cib * CI + c) * 27 + tap], acc[o]);
}

/* ---------------- pointwise kernels ---------------- */
__device__ __forceinline__ double block_sum(double v)
{
    __shared__ double sh[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x / 32, l = threadIdx.x % 32;
    __syncthreads();
    if (l == 0) sh[w] = v;
    __syncthreads();
    v = (threadIdx.x < blockDim.x / 32) ? sh[threadIdx.x] : 0.;
    if (w == 0)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// acc[f] += sum_i x[f * ld + i]^2 (blockIdx.y = f)
__global__ void __launch_bounds__(256) sumsq_kernel(const float* __restrict__ x, size_t ld,
    size_t npts, double* acc)
{
    const float* xb = x + (size_t)blockIdx.y * ld;
    double s        = 0.;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const double v = xb[i];
        s += v * v;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) atomicAdd(&acc[blockIdx.y], s);
}

// s = RMS (1 for a zero field), inv = 1 / s
__global__ void rms_finish_kernel(const double* acc, size_t npts, int nf, float* s, float* inv)
{
    const int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= nf) return;
    const double r = acc[f] > 0. ? sqrt(acc[f] / (double)npts) : 1.;
    s[f]   = (float)r;
    inv[f] = (float)(1. / r);
}

// y[f * npts + i] = x[f * ld + i] * inv[f]
__global__ void __launch_bounds__(256) scale_in_kernel(const float* __restrict__ x, size_t ld,
    float* __restrict__ y, size_t npts, const float* __restrict__ inv)
{
    const int f   = blockIdx.y;
    const float a = inv[f];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
        y[(size_t)f * npts + i] = x[(size_t)f * ld + i] * a;
}

// a = relu(a + b)
__global__ void __launch_bounds__(256) add_relu_kernel(float* __restrict__ a,
    const float* __restrict__ b, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        a[i] = fmaxf(a[i] + b[i], 0.f);
}

// g = act > 0 ? g + alpha t : 0   (t may be NULL)
__global__ void __launch_bounds__(256) relu_grad_kernel(float* __restrict__ g,
    const float* __restrict__ t, float alpha, const float* __restrict__ act, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const float v = t ? fmaf(alpha, t[i], g[i]) : g[i];
        g[i]          = act[i] > 0.f ? v : 0.f;
    }
}

__global__ void __launch_bounds__(256) scale_inplace_kernel(float* __restrict__ a, float s,
    size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        a[i] *= s;
}

/* e = y - t inv; g = gscale e; loss += sum e^2 * lscale (blockIdx.y = f) */
__global__ void __launch_bounds__(256) loss_kernel(const float* __restrict__ y,
    const float* __restrict__ t, size_t ldt, const float* __restrict__ inv,
    float* __restrict__ g, size_t npts, float gscale, double lscale, double* loss)
{
    const int f   = blockIdx.y;
    const float a = inv[f];
    double s      = 0.;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const float e           = y[(size_t)f * npts + i] - t[(size_t)f * ldt + i] * a;
        g[(size_t)f * npts + i] = gscale * e;
        s += (double)e * e;
    }
    s = block_sum(s);
    if (threadIdx.x == 0) atomicAdd(loss, s * lscale);
}

// w = bf16(m); wt[ci][co][26 - t] = bf16(m[co][ci][t]) (the flipped,
// transposed kernel of the data gradient)
__global__ void __launch_bounds__(256) to_bf16_kernel(const float* __restrict__ m,
    __nv_bfloat16* __restrict__ w, __nv_bfloat16* __restrict__ wt, int cin, int cout)
{
    const int n = cin * cout * 27;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const int t = i % 27, r = i / 27, ci = r % cin, co = r / cin;
        const __nv_bfloat16 b = __float2bfloat16_rn(m[i]);
        w[i]                                     = b;
        wt[((size_t)ci * cout + co) * 27 + 26 - t] = b;
    }
}

__global__ void __launch_bounds__(256) adam_kernel(float* __restrict__ p, float* __restrict__ m,
    float* __restrict__ v, const float* __restrict__ g, int n, float lr, float b1, float b2,
    float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i]           = mi;
        v[i]           = vi;
        p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
    }
}

// num[f] += sum (Av - r)^2, den[f] += sum r^2
__global__ void __launch_bounds__(256) reduction_kernel(const float* __restrict__ Av,
    const float* __restrict__ r, size_t ldr, size_t npts, double* num, double* den)
{
    const int f = blockIdx.y;
    double a = 0., b = 0.;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const double rv = r[(size_t)f * ldr + i];
        const double d  = (double)Av[(size_t)f * npts + i] - rv;
        a += d * d;
        b += rv * rv;
    }
    a = block_sum(a);
    b = block_sum(b);
    if (threadIdx.x == 0)
    {
        atomicAdd(&num[f], a);
        atomicAdd(&den[f], b);
    }
}

inline dim3 pw_grid(size_t n, int rows = 1)
{
    return dim3((unsigned)std::min<size_t>((n + 255) / 256, 1024), rows);
}

/* ---------------- launchers ---------------- */
template <int CI, int CO, int TXP> constexpr size_t conv_smem()
{
    return (size_t)(CI * (TXP + 2) * (TY + 2) * (TZ + 2) + CI * 27 * CO) * sizeof(float);
}
template <int CI, int CO> constexpr size_t wgrad_smem()
{
    return (size_t)(CI * (TXW + 2) * (TY + 2) * (TZ + 2) + TXW * TY * TZ * CO) * sizeof(float);
}

template <int CI, int CO>
int conv_launch_t(const float* x, size_t xf, int cin, const __nv_bfloat16* W, float* y,
    size_t yf, int cout, const Level& L, int nf, bool relu, const float* oscale, cudaStream_t s)
{
    constexpr int TXP = 4;
    constexpr size_t sm = conv_smem<CI, CO, TXP>();
    static bool attr    = false;
    if (!attr)
    {
        MGX_TRY(cuda_check(cudaFuncSetAttribute(conv_fwd_kernel<CI, CO, TXP>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
            "conv smem"));
        attr = true;
    }
    const long tiles = (long)((L.n[0] + TXP - 1) / TXP) * ((L.n[1] + TY - 1) / TY)
        * ((L.n[2] + TZ - 1) / TZ);
    const long rows = (long)nf * (cout / CO);
    if (rows > 65535) return fail(MGX_BAD_ARG, "conv: %ld function-channel blocks", rows);
    conv_fwd_kernel<CI, CO, TXP><<<dim3((unsigned)tiles, (unsigned)rows), THREADS, sm, s>>>(x, xf,
        cin, W, y, yf, cout, L.n[0], L.n[1], L.n[2], relu ? 1 : 0, oscale);
    MGX_LAUNCH_CHECK("conv_fwd_kernel");
    return MGX_OK;
}

int conv_launch(const float* x, size_t xf, int cin, const __nv_bfloat16* W, float* y, size_t yf,
    int cout, const Level& L, int nf, bool relu, const float* oscale, cudaStream_t s)
{
    if (cin == 1 && cout % 16 == 0)
        return conv_launch_t<1, 16>(x, xf, cin, W, y, yf, cout, L, nf, relu, oscale, s);
    if (cin % 8 == 0 && cout % 16 == 0)
        return conv_launch_t<8, 16>(x, xf, cin, W, y, yf, cout, L, nf, relu, oscale, s);
    if (cin % 8 == 0 && cout == 1)
        return conv_launch_t<8, 1>(x, xf, cin, W, y, yf, cout, L, nf, relu, oscale, s);
    return fail(MGX_UNSUPPORTED, "conv %d -> %d channels", cin, cout);
}

template <int CI, int CO, int PS>
int wgrad_launch_t(const float* x, int cin, const float* dy, int cout, float* dW,
    const Level& L, int nf, int sms, cudaStream_t s)
{
    constexpr size_t sm = wgrad_smem<CI, CO>();
    static bool attr    = false;
    if (!attr)
    {
        MGX_TRY(cuda_check(cudaFuncSetAttribute(conv_wgrad_kernel<CI, CO, PS>,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm),
            "wgrad smem"));
        attr = true;
    }
    const long tiles = (long)((L.n[0] + TXW - 1) / TXW) * ((L.n[1] + TY - 1) / TY)
        * ((L.n[2] + TZ - 1) / TZ);
    const int rows   = (cout / CO) * (cin / CI);
    const long items = tiles * nf;
    const long want  = std::max<long>(1, (long)4 * sms / rows);
    const unsigned gx = (unsigned)std::min(items, want);
    conv_wgrad_kernel<CI, CO, PS><<<dim3(gx, rows), THREADS, sm, s>>>(x, cin, dy, cout, dW, nf,
        L.n[0], L.n[1], L.n[2]);
    MGX_LAUNCH_CHECK("conv_wgrad_kernel");
    return MGX_OK;
}

int wgrad_launch(const float* x, int cin, const float* dy, int cout, float* dW, const Level& L,
    int nf, int sms, cudaStream_t s)
{
    if (cin == 1 && cout % 16 == 0) return wgrad_launch_t<1, 16, 8>(x, cin, dy, cout, dW, L, nf, sms, s);
    if (cin % 8 == 0 && cout % 16 == 0)
        return wgrad_launch_t<8, 16, 1>(x, cin, dy, cout, dW, L, nf, sms, s);
    if (cin % 8 == 0 && cout == 1) return wgrad_launch_t<8, 1, 1>(x, cin, dy, cout, dW, L, nf, sms, s);
    return fail(MGX_UNSUPPORTED, "wgrad %d -> %d channels", cin, cout);
}

int relu_grad(float* g, const float* t, float alpha, const float* act, size_t n, cudaStream_t s)
{
    relu_grad_kernel<<<pw_grid(n), 256, 0, s>>>(g, t, alpha, act, n);
    MGX_LAUNCH_CHECK("relu_grad_kernel");
    return MGX_OK;
}
int add_relu(float* a, const float* b, size_t n, cudaStream_t s)
{
    add_relu_kernel<<<pw_grid(n), 256, 0, s>>>(a, b, n);
    MGX_LAUNCH_CHECK("add_relu_kernel");
    return MGX_OK;
}
int scale_inplace(float* a, float v, size_t n, cudaStream_t s)
{
    scale_inplace_kernel<<<pw_grid(n), 256, 0, s>>>(a, v, n);
    MGX_LAUNCH_CHECK("scale_inplace_kernel");
    return MGX_OK;
}

/* activation and gradient blocks of a chunk of nf functions */
struct Acts
{
    float *xh, *a0, *s0, *y;  // level 0: 1, 16, 16, 1 channels
    float *p1, *a1, *s1, *z1; // level 1: 16, 32, 32, 16
    float *p2, *a2, *z2;      // level 2: 32, 64, 32
    float *gy, *gs0, *gt0;    // level 0: 1, 16, 16
    float *gz1, *gs1, *gt1, *gp1; // level 1: 16, 32, 32, 16
    float *gz2, *ga2, *gp2;   // level 2: 32, 64, 32
};
constexpr size_t FWD_C0 = 34, FWD_C1 = 96, FWD_C2 = 128;
constexpr size_t BWD_C0 = 33, BWD_C1 = 96, BWD_C2 = 128;

} // namespace nn
} // namespace mgx

struct mgx_unet
{
    mgx_ctx* ctx = nullptr;
    mgx::Level lev[3];
    mgx::DeviceBuffer master, adam_m, adam_v, grad, wbf, wbft, act, red, scal, work;
    // the gathered residuals and V-cycle corrections of the fallback
    mgx::DeviceBuffer fallback;
    int step = 0;
};

namespace mgx
{
namespace nn
{
size_t npts(const mgx_unet* n, int l) { return n->lev[l].npts(); }

size_t per_func_floats(const mgx_unet* net, bool train)
{
    const size_t n0 = npts(net, 0), n1 = npts(net, 1), n2 = npts(net, 2);
    size_t f = FWD_C0 * n0 + FWD_C1 * n1 + FWD_C2 * n2;
    if (train) f += BWD_C0 * n0 + BWD_C1 * n1 + BWD_C2 * n2;
    return f;
}

/* functions per chunk: the activations of a chunk take at most 40 % of
 * the free device memory (plus what the net already holds) */
int chunk_funcs(mgx_unet* net, int nfunc, bool train)
{
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const size_t cap = (size_t)(0.4 * (double)(fr + net->act.bytes));
    const size_t pf  = per_func_floats(net, train) * sizeof(float);
    int c            = (int)std::max<size_t>(1, cap / pf);
    c                = std::min(c, nfunc);
    c                = std::min(c, 65535 / 64);
    return std::max(c, 1);
}

Acts carve(mgx_unet* net, int nf, bool train)
{
    const size_t n0 = npts(net, 0), n1 = npts(net, 1), n2 = npts(net, 2);
    float* p = (float*)net->act.ptr;
    auto take = [&](size_t c, size_t n) {
        float* r = p;
        p += c * n * nf;
        return r;
    };
    Acts A;
    A.xh = take(1, n0);
    A.a0 = take(16, n0);
    A.s0 = take(16, n0);
    A.y  = take(1, n0);
    A.p1 = take(16, n1);
    A.a1 = take(32, n1);
    A.s1 = take(32, n1);
    A.z1 = take(16, n1);
    A.p2 = take(32, n2);
    A.a2 = take(64, n2);
    A.z2 = take(32, n2);
    A.gy = A.gs0 = A.gt0 = A.gz1 = A.gs1 = A.gt1 = A.gp1 = A.gz2 = A.ga2 = A.gp2 = nullptr;
    if (train)
    {
        A.gy  = take(1, n0);
        A.gs0 = take(16, n0);
        A.gt0 = take(16, n0);
        A.gz1 = take(16, n1);
        A.gs1 = take(32, n1);
        A.gt1 = take(32, n1);
        A.gp1 = take(16, n1);
        A.gz2 = take(32, n2);
        A.ga2 = take(64, n2);
        A.gp2 = take(32, n2);
    }
    return A;
}

const __nv_bfloat16* W(const mgx_unet* net, int l)
{
    return (const __nv_bfloat16*)net->wbf.ptr + layer_offset(l);
}
const __nv_bfloat16* Wt(const mgx_unet* net, int l)
{
    return (const __nv_bfloat16*)net->wbft.ptr + layer_offset(l);
}

int refresh_bf16(mgx_unet* net, cudaStream_t s)
{
    for (int l = 0; l < NLAYER; l++)
    {
        const size_t o = layer_offset(l);
        to_bf16_kernel<<<pw_grid(layer_size(l)), 256, 0, s>>>((const float*)net->master.ptr + o,
            (__nv_bfloat16*)net->wbf.ptr + o, (__nv_bfloat16*)net->wbft.ptr + o, LAYERS[l].cin,
            LAYERS[l].cout);
        MGX_LAUNCH_CHECK("to_bf16_kernel");
    }
    return MGX_OK;
}

/* forward pass of nf functions (x with function stride ld); the output
 * goes to A.y (normalized units) or, with y, to y * s (stride ldy) */
int forward(mgx_unet* net, const Acts& A, const float* x, size_t ld, int nf, float* y,
    size_t ldy, cudaStream_t s)
{
    const Level *L = net->lev;
    const size_t n0 = L[0].npts(), n1 = L[1].npts(), n2 = L[2].npts();
    double* acc = (double*)net->red.ptr;
    float* sc   = (float*)net->scal.ptr; // s[nf], inv[nf]
    float* inv  = sc + nf;
    MGX_TRY(cuda_check(cudaMemsetAsync(acc, 0, nf * sizeof(double), s), "rms zero"));
    sumsq_kernel<<<pw_grid(n0, nf), 256, 0, s>>>(x, ld, n0, acc);
    MGX_LAUNCH_CHECK("sumsq_kernel");
    rms_finish_kernel<<<(nf + 127) / 128, 128, 0, s>>>(acc, n0, nf, sc, inv);
    MGX_LAUNCH_CHECK("rms_finish_kernel");
    scale_in_kernel<<<pw_grid(n0, nf), 256, 0, s>>>(x, ld, A.xh, n0, inv);
    MGX_LAUNCH_CHECK("scale_in_kernel");
    const MaskDev none;
    MGX_TRY(conv_launch(A.xh, n0, 1, W(net, 0), A.a0, 16 * n0, 16, L[0], nf, true, nullptr, s));
    MGX_TRY(restrict_launch(MGX_F32, L[0], A.a0, n0, A.p1, n1, nf * 16, none, s));
    MGX_TRY(conv_launch(A.p1, 16 * n1, 16, W(net, 1), A.a1, 32 * n1, 32, L[1], nf, true, nullptr, s));
    MGX_TRY(restrict_launch(MGX_F32, L[1], A.a1, n1, A.p2, n2, nf * 32, none, s));
    MGX_TRY(conv_launch(A.p2, 32 * n2, 32, W(net, 2), A.a2, 64 * n2, 64, L[2], nf, true, nullptr, s));
    MGX_TRY(conv_launch(A.a2, 64 * n2, 64, W(net, 3), A.z2, 32 * n2, 32, L[2], nf, false, nullptr, s));
    MGX_TRY(prolong_launch(MGX_F32, 0, L[1], A.z2, n2, A.s1, n1, nf * 32, none, s));
    MGX_TRY(add_relu(A.s1, A.a1, (size_t)nf * 32 * n1, s));
    MGX_TRY(conv_launch(A.s1, 32 * n1, 32, W(net, 4), A.z1, 16 * n1, 16, L[1], nf, false, nullptr, s));
    MGX_TRY(prolong_launch(MGX_F32, 0, L[0], A.z1, n1, A.s0, n0, nf * 16, none, s));
    MGX_TRY(add_relu(A.s0, A.a0, (size_t)nf * 16 * n0, s));
    if (y)
        return conv_launch(A.s0, 16 * n0, 16, W(net, 5), y, ldy, 1, L[0], nf, false, sc, s);
    return conv_launch(A.s0, 16 * n0, 16, W(net, 5), A.y, n0, 1, L[0], nf, false, nullptr, s);
}

/* backward pass after forward(..., y = NULL): A.gy holds d loss / d y;
 * the weight gradients are added to grad */
int backward(mgx_unet* net, const Acts& A, int nf, float* grad, cudaStream_t s)
{
    const Level* L  = net->lev;
    const size_t n0 = L[0].npts(), n1 = L[1].npts(), n2 = L[2].npts();
    const int sms   = net->ctx->sm_count;
    const MaskDev none;
    auto G = [&](int l) { return grad + layer_offset(l); };
    // D0
    MGX_TRY(wgrad_launch(A.s0, 16, A.gy, 1, G(5), L[0], nf, sms, s));
    MGX_TRY(conv_launch(A.gy, n0, 1, Wt(net, 5), A.gs0, 16 * n0, 16, L[0], nf, false, nullptr, s));
    MGX_TRY(relu_grad(A.gs0, nullptr, 0.f, A.s0, (size_t)nf * 16 * n0, s));
    // D1 (through the prolongation: P^T = 8 R)
    MGX_TRY(restrict_launch(MGX_F32, L[0], A.gs0, n0, A.gz1, n1, nf * 16, none, s));
    MGX_TRY(scale_inplace(A.gz1, 8.f, (size_t)nf * 16 * n1, s));
    MGX_TRY(wgrad_launch(A.s1, 32, A.gz1, 16, G(4), L[1], nf, sms, s));
    MGX_TRY(conv_launch(A.gz1, 16 * n1, 16, Wt(net, 4), A.gs1, 32 * n1, 32, L[1], nf, false, nullptr, s));
    MGX_TRY(relu_grad(A.gs1, nullptr, 0.f, A.s1, (size_t)nf * 32 * n1, s));
    // D2
    MGX_TRY(restrict_launch(MGX_F32, L[1], A.gs1, n1, A.gz2, n2, nf * 32, none, s));
    MGX_TRY(scale_inplace(A.gz2, 8.f, (size_t)nf * 32 * n2, s));
    MGX_TRY(wgrad_launch(A.a2, 64, A.gz2, 32, G(3), L[2], nf, sms, s));
    MGX_TRY(conv_launch(A.gz2, 32 * n2, 32, Wt(net, 3), A.ga2, 64 * n2, 64, L[2], nf, false, nullptr, s));
    MGX_TRY(relu_grad(A.ga2, nullptr, 0.f, A.a2, (size_t)nf * 64 * n2, s));
    // E2
    MGX_TRY(wgrad_launch(A.p2, 32, A.ga2, 64, G(2), L[2], nf, sms, s));
    MGX_TRY(conv_launch(A.ga2, 64 * n2, 64, Wt(net, 2), A.gp2, 32 * n2, 32, L[2], nf, false, nullptr, s));
    // through the restriction (R^T = P / 8) into the skip of level 1
    MGX_TRY(prolong_launch(MGX_F32, 0, L[1], A.gp2, n2, A.gt1, n1, nf * 32, none, s));
    MGX_TRY(relu_grad(A.gs1, A.gt1, 0.125f, A.a1, (size_t)nf * 32 * n1, s));
    // E1
    MGX_TRY(wgrad_launch(A.p1, 16, A.gs1, 32, G(1), L[1], nf, sms, s));
    MGX_TRY(conv_launch(A.gs1, 32 * n1, 32, Wt(net, 1), A.gp1, 16 * n1, 16, L[1], nf, false, nullptr, s));
    MGX_TRY(prolong_launch(MGX_F32, 0, L[0], A.gp1, n1, A.gt0, n0, nf * 16, none, s));
    MGX_TRY(relu_grad(A.gs0, A.gt0, 0.125f, A.a0, (size_t)nf * 16 * n0, s));
    // E0
    return wgrad_launch(A.xh, 1, A.gs0, 16, G(0), L[0], nf, sms, s);
}

int ensure_scratch(mgx_unet* net, int nf)
{
    MGX_TRY(net->red.ensure((size_t)2 * std::max(nf, 1) * sizeof(double) + 256));
    MGX_TRY(net->scal.ensure((size_t)2 * std::max(nf, 1) * sizeof(float) + 256));
    return MGX_OK;
}

int loss_grad(mgx_unet* net, const float* x, const float* t, size_t ld, int nfunc, float* grad,
    double* loss, cudaStream_t s)
{
    const size_t n0 = net->lev[0].npts();
    MGX_TRY(cuda_check(cudaMemsetAsync(grad, 0, NPARAM * sizeof(float), s), "grad zero"));
    MGX_TRY(cuda_check(cudaMemsetAsync(loss, 0, sizeof(double), s), "loss zero"));
    const int chunk = chunk_funcs(net, nfunc, true);
    MGX_TRY(net->act.ensure(per_func_floats(net, true) * sizeof(float) * chunk + 256));
    MGX_TRY(ensure_scratch(net, chunk));
    const double tot = (double)n0 * nfunc;
    for (int f0 = 0; f0 < nfunc; f0 += chunk)
    {
        const int nf = std::min(chunk, nfunc - f0);
        const Acts A = carve(net, nf, true);
        MGX_TRY(forward(net, A, x + (size_t)f0 * ld, ld, nf, nullptr, 0, s));
        const float* inv = (const float*)net->scal.ptr + nf;
        loss_kernel<<<pw_grid(n0, nf), 256, 0, s>>>(A.y, t + (size_t)f0 * ld, ld, inv, A.gy, n0,
            (float)(2. / tot), 1. / tot, loss);
        MGX_LAUNCH_CHECK("loss_kernel");
        MGX_TRY(backward(net, A, nf, grad, s));
    }
    return MGX_OK;
}

int adam(mgx_unet* net, const float* grad, const mgx_adam_params* p, cudaStream_t s)
{
    net->step++;
    const double c1 = 1. / (1. - std::pow((double)p->beta1, net->step));
    const double c2 = 1. / (1. - std::pow((double)p->beta2, net->step));
    adam_kernel<<<pw_grid(NPARAM), 256, 0, s>>>((float*)net->master.ptr, (float*)net->adam_m.ptr,
        (float*)net->adam_v.ptr, grad, (int)NPARAM, p->lr, p->beta1, p->beta2, p->eps, (float)c1,
        (float)c2);
    MGX_LAUNCH_CHECK("adam_kernel");
    return refresh_bf16(net, s);
}

/* reduction_j = |r_j - A v_j| / |r_j| for nf functions (host out) */
int reductions(mgx_ctx* ctx, mgx_unet* net, int lap_type, const float* r, size_t ldr,
    const float* v, size_t ldv, int nf, double* host, cudaStream_t s)
{
    const Level L0   = make_level(ctx->grid, 0);
    const size_t n0  = L0.npts();
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    const size_t cap = (size_t)(0.2 * (double)(fr + net->work.bytes));
    const int chunk  = (int)std::max<size_t>(1, std::min<size_t>(nf, cap / (n0 * sizeof(float))));
    MGX_TRY(net->work.ensure((size_t)chunk * n0 * sizeof(float) + 256));
    MGX_TRY(ensure_scratch(net, nf));
    double* num = (double*)net->red.ptr;
    double* den = num + nf;
    MGX_TRY(cuda_check(cudaMemsetAsync(num, 0, 2 * nf * sizeof(double), s), "reduction zero"));
    for (int f0 = 0; f0 < nf; f0 += chunk)
    {
        const int nc = std::min(chunk, nf - f0);
        PlaneParams p;
        for (int i = 0; i < 3; i++)
            p.n[i] = ctx->grid.n[i];
        p.u   = v + (size_t)f0 * ldv;
        p.ldu = ldv;
        p.out = net->work.ptr;
        p.ldo = n0;
        MGX_TRY(stencil_launch(OP_LAP, lap_type, MGX_F32, MGX_F32, p, L0, 0., nc, s));
        reduction_kernel<<<pw_grid(n0, nc), 256, 0, s>>>((const float*)net->work.ptr,
            r + (size_t)f0 * ldr, ldr, n0, num + f0, den + f0);
        MGX_LAUNCH_CHECK("reduction_kernel");
    }
    std::vector<double> h(2 * (size_t)nf);
    MGX_TRY(cuda_check(cudaMemcpyAsync(h.data(), num, 2 * nf * sizeof(double),
                           cudaMemcpyDeviceToHost, s),
        "reduction read"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "reduction sync"));
    for (int j = 0; j < nf; j++)
        host[j] = h[nf + j] > 0. ? std::sqrt(h[j] / h[nf + j]) : 0.;
    return MGX_OK;
}

} // namespace nn
} // namespace mgx

using namespace mgx;

static int check_net(const mgx_unet* net)
{
    if (!net || !net->ctx) return fail(MGX_BAD_ARG, "net is NULL");
    return MGX_OK;
}

extern "C" {

int mgx_unet_create(mgx_ctx* ctx, mgx_unet** out)
{
    if (!ctx || !out) return fail(MGX_BAD_ARG, "NULL argument");
    for (int i = 0; i < 3; i++)
        if (ctx->grid.n[i] % 4 || ctx->grid.n[i] < 4)
            return fail(MGX_BAD_ARG, "grid dimension %d (%d) not divisible by 4", i, ctx->grid.n[i]);
    auto net = std::make_unique<mgx_unet>();
    net->ctx = ctx;
    for (int l = 0; l < 3; l++)
        net->lev[l] = make_level(ctx->grid, l);
    const size_t pb = nn::NPARAM * sizeof(float);
    MGX_TRY(net->master.ensure(pb));
    MGX_TRY(net->adam_m.ensure(pb));
    MGX_TRY(net->adam_v.ensure(pb));
    MGX_TRY(net->grad.ensure(pb));
    MGX_TRY(net->wbf.ensure(nn::NPARAM * sizeof(__nv_bfloat16)));
    MGX_TRY(net->wbft.ensure(nn::NPARAM * sizeof(__nv_bfloat16)));
    MGX_TRY(cuda_check(cudaMemset(net->master.ptr, 0, pb), "net zero"));
    MGX_TRY(cuda_check(cudaMemset(net->adam_m.ptr, 0, pb), "net zero"));
    MGX_TRY(cuda_check(cudaMemset(net->adam_v.ptr, 0, pb), "net zero"));
    MGX_TRY(nn::refresh_bf16(net.get(), 0));
    MGX_TRY(cuda_check(cudaDeviceSynchronize(), "net create"));
    *out = net.release();
    return MGX_OK;
}

int mgx_unet_destroy(mgx_unet* net)
{
    delete net;
    return MGX_OK;
}

int mgx_unet_set_params(mgx_unet* net, const float* params, void* stream)
{
    MGX_TRY(check_net(net));
    if (!params) return fail(MGX_BAD_ARG, "params is NULL");
    const cudaStream_t s = (cudaStream_t)stream;
    const size_t pb      = nn::NPARAM * sizeof(float);
    MGX_TRY(cuda_check(cudaMemcpyAsync(net->master.ptr, params, pb, cudaMemcpyDeviceToDevice, s),
        "params copy"));
    MGX_TRY(cuda_check(cudaMemsetAsync(net->adam_m.ptr, 0, pb, s), "adam reset"));
    MGX_TRY(cuda_check(cudaMemsetAsync(net->adam_v.ptr, 0, pb, s), "adam reset"));
    net->step = 0;
    return nn::refresh_bf16(net, s);
}

int mgx_unet_get_params(mgx_unet* net, float* params, void* stream)
{
    MGX_TRY(check_net(net));
    if (!params) return fail(MGX_BAD_ARG, "params is NULL");
    return cuda_check(cudaMemcpyAsync(params, net->master.ptr, nn::NPARAM * sizeof(float),
                          cudaMemcpyDeviceToDevice, (cudaStream_t)stream),
        "params copy");
}

int mgx_unet_forward(mgx_unet* net, const float* x, size_t ld, float* y, int nfunc, void* stream)
{
    MGX_TRY(check_net(net));
    const size_t n0 = net->lev[0].npts();
    if (nfunc < 0 || (nfunc && (!x || !y))) return fail(MGX_BAD_ARG, "NULL block");
    if (nfunc > 1 && ld < n0) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, n0);
    if (x == y) return fail(MGX_BAD_ARG, "x and y alias");
    if (nfunc == 0) return MGX_OK;
    if (ld == 0) ld = n0;
    const cudaStream_t s = (cudaStream_t)stream;
    const int chunk      = nn::chunk_funcs(net, nfunc, false);
    MGX_TRY(net->act.ensure(nn::per_func_floats(net, false) * sizeof(float) * chunk + 256));
    MGX_TRY(nn::ensure_scratch(net, chunk));
    for (int f0 = 0; f0 < nfunc; f0 += chunk)
    {
        const int nf = std::min(chunk, nfunc - f0);
        MGX_TRY(nn::forward(net, nn::carve(net, nf, false), x + (size_t)f0 * ld, ld, nf,
            y + (size_t)f0 * ld, ld, s));
    }
    return MGX_OK;
}

int mgx_unet_loss_grad(mgx_unet* net, const float* x, const float* target, size_t ld,
    int nfunc, float* grad, double* loss, void* stream)
{
    MGX_TRY(check_net(net));
    const size_t n0 = net->lev[0].npts();
    if (nfunc <= 0 || !x || !target || !grad || !loss) return fail(MGX_BAD_ARG, "NULL argument");
    if (nfunc > 1 && ld < n0) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, n0);
    if (ld == 0) ld = n0;
    return nn::loss_grad(net, x, target, ld, nfunc, grad, loss, (cudaStream_t)stream);
}

int mgx_unet_adam(mgx_unet* net, const float* grad, const mgx_adam_params* p, void* stream)
{
    MGX_TRY(check_net(net));
    if (!grad || !p) return fail(MGX_BAD_ARG, "NULL argument");
    if (!(p->lr > 0.f) || !(p->beta1 >= 0.f && p->beta1 < 1.f) || !(p->beta2 >= 0.f && p->beta2 < 1.f)
        || !(p->eps > 0.f))
        return fail(MGX_BAD_ARG, "Adam parameters");
    return nn::adam(net, grad, p, (cudaStream_t)stream);
}

int mgx_unet_train_step(mgx_unet* net, const float* x, const float* target, size_t ld,
    int nfunc, const mgx_adam_params* p, double* loss, void* stream)
{
    MGX_TRY(check_net(net));
    MGX_TRY(mgx_unet_loss_grad(net, x, target, ld, nfunc, (float*)net->grad.ptr, loss, stream));
    return mgx_unet_adam(net, (const float*)net->grad.ptr, p, stream);
}

int mgx_precond_learned(mgx_ctx* ctx, mgx_unet* net, const mgx_precond_params* p,
    const float* res, size_t ld, float* out, int nfunc, int mode, double* tau,
    double* reduction, int* nfallback, void* stream)
{
    if (!ctx || !p) return fail(MGX_BAD_ARG, "NULL argument");
    MGX_TRY(check_net(net));
    if (net->ctx->grid.n[0] != ctx->grid.n[0] || net->ctx->grid.n[1] != ctx->grid.n[1]
        || net->ctx->grid.n[2] != ctx->grid.n[2])
        return fail(MGX_BAD_ARG, "net and context grids differ");
    if ((mode & ~3) != 0) return fail(MGX_BAD_ARG, "mode %d", mode);
    if (nfunc < 0 || (nfunc && (!res || !out || !tau))) return fail(MGX_BAD_ARG, "NULL argument");
    if (res == out) return fail(MGX_BAD_ARG, "res and out alias");
    const size_t n0 = net->lev[0].npts();
    if (nfunc > 1 && ld < n0) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, n0);
    if (nfallback) *nfallback = 0;
    if (nfunc == 0) return MGX_OK;
    if (ld == 0) ld = n0;
    const cudaStream_t s = (cudaStream_t)stream;
    // the learned correction
    MGX_TRY(mgx_unet_forward(net, res, ld, out, nfunc, stream));
    if (mode & MGX_LEARNED_WARM)
        MGX_TRY(precond_mg(ctx, p, MGX_F32, res, ld, out, nfunc, nullptr, s, nullptr, 0., nullptr,
            true));
    std::vector<double> rl(nfunc);
    MGX_TRY(nn::reductions(ctx, net, p->lap_type, res, ld, out, ld, nfunc, rl.data(), s));
    // the functions that take the plain V-cycle
    std::vector<int> run;
    for (int j = 0; j < nfunc; j++)
        if ((mode & MGX_LEARNED_REFRESH) || !(tau[j] > 0.) || rl[j] > tau[j]) run.push_back(j);
    int nfb = 0;
    if (!run.empty())
    {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        const int m = (int)run.size();
        int chunk   = (int)std::max<size_t>(1, std::min<size_t>(m,
                                             (size_t)(0.2 * (double)(fr + net->fallback.bytes))
                                                 / (2 * n0 * sizeof(float))));
        MGX_TRY(net->fallback.ensure((size_t)2 * chunk * n0 * sizeof(float) + 256));
        float* wres = (float*)net->fallback.ptr;
        float* wout = wres + (size_t)chunk * n0;
        std::vector<double> rv(chunk);
        for (int k0 = 0; k0 < m; k0 += chunk)
        {
            const int nc = std::min(chunk, m - k0);
            for (int k = 0; k < nc; k++)
                MGX_TRY(cuda_check(cudaMemcpyAsync(wres + (size_t)k * n0,
                                       res + (size_t)run[k0 + k] * ld, n0 * sizeof(float),
                                       cudaMemcpyDeviceToDevice, s),
                    "gather"));
            MGX_TRY(precond_mg(ctx, p, MGX_F32, wres, n0, wout, nc, nullptr, s, nullptr, 0.,
                nullptr, false));
            MGX_TRY(nn::reductions(ctx, net, p->lap_type, wres, n0, wout, n0, nc, rv.data(), s));
            for (int k = 0; k < nc; k++)
            {
                const int j = run[k0 + k];
                tau[j]      = rv[k];
                if (rv[k] < rl[j])
                {
                    MGX_TRY(cuda_check(cudaMemcpyAsync(out + (size_t)j * ld, wout + (size_t)k * n0,
                                           n0 * sizeof(float), cudaMemcpyDeviceToDevice, s),
                        "scatter"));
                    rl[j] = rv[k];
                    nfb++;
                }
            }
        }
        MGX_TRY(cuda_check(cudaStreamSynchronize(s), "fallback sync"));
    }
    if (reduction) std::memcpy(reduction, rl.data(), nfunc * sizeof(double));
    if (nfallback) *nfallback = nfb;
    return MGX_OK;
}

} // extern "C"
