// Multigrid transfers, localization masks and the block V-cycle of the
// orbital preconditioner on sm_103a.
//
//  - restriction: full weighting (8,4,2,1)/64 around fine point 2i
//    (pb::MGkernelRestrict3D, src/pb/MGkernels.cc:203-283), with the
//    coarse-level mask in the epilogue;
//  - prolongation: injection at even points and 1-D / 2-D / 3-D averages at
//    odd points (pb::MGkernelExtend3D, src/pb/MGkernels.cc:28-201), fused
//    with the fine-level mask and the correction v -= P e;
//  - masks: GridMask::init (src/GridMask.cc:120-264) evaluated on the device
//    over a periodic bounding box per orbital and level, with the per-axis
//    point coordinates formed on the host by the reference's repeated
//    addition so that membership tests are bit-identical;
//  - Preconditioning<T>::mg (src/Preconditioning.cc:155-216) driven from the
//    host: Jacobi sweeps (stencil engine, OP_JACOBI), restriction,
//    recursion with Laph2 on coarse grids, prolongation-correction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <memory>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{

/* ------------------------------------------------------------------ */
/* transfers                                                            */
/* ------------------------------------------------------------------ */
__device__ __forceinline__ int wrp(int i, int n)
{
    return i < 0 ? i + n : (i >= n ? i - n : i);
}

template <typename T>
__device__ __forceinline__ T mask_point(const MaskDev& m, int f, int x, int y,
    int z, T v)
{
    if (m.state == nullptr) return v;
    const int st = m.state[f];
    if (st == 1) return v;
    if (st <= 0) return (T)0;
    const int* b = m.box + 6 * f;
    int dx = x - b[0];
    if (dx < 0) dx += m.n[0];
    int dy = y - b[1];
    if (dy < 0) dy += m.n[1];
    int dz = z - b[2];
    if (dz < 0) dz += m.n[2];
    T mv = (T)0;
    if (dx < b[3] && dy < b[4] && dz < b[5])
        mv = reinterpret_cast<const T*>(m.values)[m.offset[f]
                                                  + ((size_t)dx * b[4] + dy) * b[5]
                                                  + dz];
    if (m.kind == 0)
    {
        if (v > mv) return mv;
        if (v < -mv) return -mv;
        return v;
    }
    return v * mv;
}

/* restriction of nfunc functions; accumulation type A (double for the FP64
 * path, as the reference; float for the FP32 path).  One block per pair of
 * coarse (i, j) lines (i and i + 1), threads along coarse z; blockIdx.y =
 * function.  A thread loads the 5 x 3 fine rows around its pair once (at
 * z - 1, z, z + 1; the plane x = 2i + 1 serves both) and forms each coarse
 * point with the grouping and order of src/pb/MGkernels.cc:249-270. */
template <typename T, typename A>
__global__ void restrict_kernel(const T* __restrict__ fine, size_t ldf,
    T* __restrict__ coarse, size_t ldc, int fx, int fy, int fz, MaskDev mask)
{
    const int cx = fx >> 1, cy = fy >> 1, cz = fz >> 1;
    const int f  = blockIdx.y;
    const int i0 = 2 * (blockIdx.x / cy), j = blockIdx.x - (blockIdx.x / cy) * cy;
    const T* u   = fine + (size_t)f * ldf;
    // rows[a][b]: fine row x = 2 i0 - 1 + a, y = 2 j - 1 + b
    const T* rows[5][3];
#pragma unroll
    for (int a = 0; a < 5; a++)
    {
        const int x = wrp(2 * i0 - 1 + a, fx);
#pragma unroll
        for (int b = 0; b < 3; b++)
            rows[a][b] = u + ((size_t)x * fy + wrp(2 * j - 1 + b, fy)) * fz;
    }
    const int npair = (i0 + 1 < cx) ? 2 : 1;
    for (int k = threadIdx.x; k < cz; k += blockDim.x)
    {
        const int z = 2 * k, zm = wrp(z - 1, fz), zp = wrp(z + 1, fz);
        A v[5][3][3];
#pragma unroll
        for (int a = 0; a < 5; a++)
#pragma unroll
            for (int b = 0; b < 3; b++)
            {
                v[a][b][0] = (A)rows[a][b][zm];
                v[a][b][1] = (A)rows[a][b][z];
                v[a][b][2] = (A)rows[a][b][zp];
            }
#pragma unroll
        for (int di = 0; di < 2; di++)
        {
            if (di >= npair) break;
            const int i  = i0 + di;
            const int ca = 2 * di + 1; // centre plane x = 2i
            const A* r00 = v[ca][1];
            const A* rp0 = v[ca + 1][1];
            const A* rm0 = v[ca - 1][1];
            const A* r0p = v[ca][2];
            const A* r0m = v[ca][0];
            const A* rpp = v[ca + 1][2];
            const A* rpm = v[ca + 1][0];
            const A* rmp = v[ca - 1][2];
            const A* rmm = v[ca - 1][0];
            const A face = rp0[1] + rm0[1] + r0p[1] + r0m[1] + r00[0] + r00[2];
            const A corner = rpp[0] + rpp[2] + rpm[0] + rpm[2] + rmp[0] + rmp[2] + rmm[0] + rmm[2];
            const A edge = r0p[0] + r0p[2] + r0m[0] + r0m[2] + rp0[0] + rp0[2] + rm0[0] + rm0[2]
                           + rmm[1] + rpm[1] + rmp[1] + rpp[1];
            const A r = (A)(1. / 64.) * ((A)8. * r00[1] + (A)4. * face + (A)2. * edge + corner);
            coarse[(size_t)f * ldc + ((size_t)i * cy + j) * cz + k]
                = mask_point<T>(mask, f, i, j, k, (T)r);
        }
    }
}

/* trilinear prolongation; MODE 0: out = P e; MODE 1: out -= mask(P e).
 * One block per fine x plane and band of PROLONG_CROWS coarse y rows.  A
 * thread owns coarse point (j, k) of the band and writes the 2 x 2 fine
 * points (2j + b, 2k + c) of its x plane: it loads the coarse values at
 * k and k + 1 of rows j and j + 1 (and of plane i + 1 for odd x) once and
 * forms every output with the operation order of src/pb/MGkernels.cc:84-197.
 * VEC2: the two z neighbours are stored (and, MODE 1, read) as one pair. */
constexpr int PROLONG_CROWS = 4;

template <typename T> struct Pair;
template <> struct Pair<float> { using type = float2; };
template <> struct Pair<double> { using type = double2; };

template <typename T, int MODE, bool VEC2>
__global__ void __launch_bounds__(256) prolong_kernel(const T* __restrict__ coarse,
    size_t ldc, T* __restrict__ out, size_t ldo, int fx, int fy, int fz, MaskDev mask)
{
    using P2 = typename Pair<T>::type;
    const int cx = fx >> 1, cy = fy >> 1, cz = fz >> 1;
    const int f      = blockIdx.y;
    const int bands  = (cy + PROLONG_CROWS - 1) / PROLONG_CROWS;
    const int x      = blockIdx.x / bands;
    const int jb     = (blockIdx.x - x * bands) * PROLONG_CROWS;
    const T* e       = coarse + (size_t)f * ldc;
    const int i = x >> 1, a = x & 1, i1 = wrp(i + 1, cx);
    for (int t = threadIdx.x; t < PROLONG_CROWS * cz; t += blockDim.x)
    {
        const int r = t / cz, k = t - (t / cz) * cz;
        const int j = jb + r;
        if (j >= cy) break;
        const int j1 = wrp(j + 1, cy), k1 = wrp(k + 1, cz);
        const T* c00 = e + ((size_t)i * cy + j) * cz;
        const T* c01 = e + ((size_t)i * cy + j1) * cz;
        const T a0 = c00[k], a1 = c00[k1], b0 = c01[k], b1 = c01[k1];
        T v[2][2]; // [y parity][z parity]
        if (!a)
        {
            v[0][0] = a0;
            v[0][1] = (T)0.5 * (a0 + a1);
            v[1][0] = (T)0.5 * (b0 + a0);
            v[1][1] = (T)0.25 * (b1 + a1 + b0 + a0);
        }
        else
        {
            const T* c10 = e + ((size_t)i1 * cy + j) * cz;
            const T* c11 = e + ((size_t)i1 * cy + j1) * cz;
            const T d0 = c10[k], d1 = c10[k1], g0 = c11[k], g1 = c11[k1];
            v[0][0] = (T)0.5 * (d0 + a0);
            v[0][1] = (T)0.25 * (d1 + d0 + a1 + a0);
            v[1][0] = (T)0.25 * (g0 + d0 + b0 + a0);
            v[1][1] = (T)0.125 * (g1 + g0 + d1 + d0 + b1 + b0 + a1 + a0);
        }
#pragma unroll
        for (int b = 0; b < 2; b++)
        {
            const int y = 2 * j + b;
            T* o = out + (size_t)f * ldo + ((size_t)x * fy + y) * fz + 2 * k;
            T w0 = v[b][0], w1 = v[b][1];
            if (MODE == 1)
            {
                w0 = mask_point<T>(mask, f, x, y, 2 * k, w0);
                w1 = mask_point<T>(mask, f, x, y, 2 * k + 1, w1);
            }
            if (VEC2)
            {
                P2 q;
                if (MODE == 1)
                {
                    q = *reinterpret_cast<const P2*>(o);
                    q.x = q.x - w0;
                    q.y = q.y - w1;
                }
                else
                {
                    q.x = w0;
                    q.y = w1;
                }
                *reinterpret_cast<P2*>(o) = q;
            }
            else if (MODE == 1)
            {
                o[0] = o[0] - w0;
                o[1] = o[1] - w1;
            }
            else
            {
                o[0] = w0;
                o[1] = w1;
            }
        }
    }
}

/* The FP32 prolongation with four fine z points per thread and y parity:
 * a thread owns coarse points (j, 2m) and (j, 2m + 1) and writes the 2 x 4
 * fine points (2j + b, 4m + c) of its x plane as two 16-byte stores (MODE
 * 1: read-modify-write), which keeps twice the bytes in flight of the
 * pair form.  Every output has the operation order of prolong_kernel.
 * Needs fz % 4 == 0 and 16-byte aligned fine rows. */
constexpr int PROLONG4_CROWS = 16;

template <int MODE>
__global__ void __launch_bounds__(256) prolong4_kernel(const float* __restrict__ coarse,
    size_t ldc, float* __restrict__ out, size_t ldo, int fx, int fy, int fz, MaskDev mask)
{
    const int cx = fx >> 1, cy = fy >> 1, cz = fz >> 1, hz = cz >> 1;
    const int f      = blockIdx.y;
    const int bands  = (cy + PROLONG4_CROWS - 1) / PROLONG4_CROWS;
    const int x      = blockIdx.x / bands;
    const int jb     = (blockIdx.x - x * bands) * PROLONG4_CROWS;
    const float* e   = coarse + (size_t)f * ldc;
    const int i = x >> 1, a = x & 1, i1 = wrp(i + 1, cx);
    for (int t = threadIdx.x; t < PROLONG4_CROWS * hz; t += blockDim.x)
    {
        const int r = t / hz, m = t - r * hz;
        const int j = jb + r;
        if (j >= cy) break;
        const int j1 = wrp(j + 1, cy);
        const int k = 2 * m, k1 = k + 1, k2 = wrp(k + 2, cz);
        const float* c00 = e + ((size_t)i * cy + j) * cz;
        const float* c01 = e + ((size_t)i * cy + j1) * cz;
        const float a0 = c00[k], a1 = c00[k1], a2 = c00[k2];
        const float b0 = c01[k], b1 = c01[k1], b2 = c01[k2];
        float v[2][4]; // [y parity][fine z - 4m]
        if (!a)
        {
            v[0][0] = a0;
            v[0][1] = 0.5f * (a0 + a1);
            v[0][2] = a1;
            v[0][3] = 0.5f * (a1 + a2);
            v[1][0] = 0.5f * (b0 + a0);
            v[1][1] = 0.25f * (b1 + a1 + b0 + a0);
            v[1][2] = 0.5f * (b1 + a1);
            v[1][3] = 0.25f * (b2 + a2 + b1 + a1);
        }
        else
        {
            const float* c10 = e + ((size_t)i1 * cy + j) * cz;
            const float* c11 = e + ((size_t)i1 * cy + j1) * cz;
            const float d0 = c10[k], d1 = c10[k1], d2 = c10[k2];
            const float g0 = c11[k], g1 = c11[k1], g2 = c11[k2];
            v[0][0] = 0.5f * (d0 + a0);
            v[0][1] = 0.25f * (d1 + d0 + a1 + a0);
            v[0][2] = 0.5f * (d1 + a1);
            v[0][3] = 0.25f * (d2 + d1 + a2 + a1);
            v[1][0] = 0.25f * (g0 + d0 + b0 + a0);
            v[1][1] = 0.125f * (g1 + g0 + d1 + d0 + b1 + b0 + a1 + a0);
            v[1][2] = 0.25f * (g1 + d1 + b1 + a1);
            v[1][3] = 0.125f * (g2 + g1 + d2 + d1 + b2 + b1 + a2 + a1);
        }
#pragma unroll
        for (int b = 0; b < 2; b++)
        {
            const int y = 2 * j + b;
            float4* o = reinterpret_cast<float4*>(out + (size_t)f * ldo + ((size_t)x * fy + y) * fz
                                                  + 4 * m);
            float w[4];
#pragma unroll
            for (int c = 0; c < 4; c++)
                w[c] = MODE == 1 ? mask_point<float>(mask, f, x, y, 4 * m + c, v[b][c]) : v[b][c];
            float4 q;
            if (MODE == 1)
            {
                q = *o;
                q.x = q.x - w[0];
                q.y = q.y - w[1];
                q.z = q.z - w[2];
                q.w = q.w - w[3];
            }
            else
                q = make_float4(w[0], w[1], w[2], w[3]);
            *o = q;
        }
    }
}

template <typename T>
__global__ void scale_kernel(const T* in, size_t ldi, T* out, size_t ldo,
    size_t npts, T alpha)
{
    const int f = blockIdx.y;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < npts;
         i += (size_t)gridDim.x * blockDim.x)
        out[(size_t)f * ldo + i] = alpha * in[(size_t)f * ldi + i];
}

template <typename T>
__global__ void mask_apply_kernel(T* u, size_t ld, int nx, int ny, int nz,
    MaskDev mask)
{
    const int f       = blockIdx.y;
    const size_t npts = (size_t)nx * ny * nz;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
         idx += (size_t)gridDim.x * blockDim.x)
    {
        const int z = (int)(idx % nz);
        const int y = (int)((idx / nz) % ny);
        const int x = (int)(idx / ((size_t)nz * ny));
        T* p        = u + (size_t)f * ld + idx;
        *p          = mask_point<T>(mask, f, x, y, z, *p);
    }
}

static dim3 grid_for(size_t npts, int nfunc)
{
    const int bx = (int)std::min<size_t>((npts + 255) / 256, 2048);
    return dim3(bx, nfunc);
}

int restrict_launch(int dtype, const Level& fine, const void* f, size_t ldf,
    void* c, size_t ldc, int nfunc, const MaskDev& mask, cudaStream_t s)
{
    const dim3 g((((fine.n[0] / 2) + 1) / 2) * (fine.n[1] / 2), nfunc);
    const int nt = std::min(256, std::max(32, ((fine.n[2] / 2 + 31) / 32) * 32));
    if (dtype == MGX_F64)
        restrict_kernel<double, double><<<g, nt, 0, s>>>((const double*)f, ldf,
            (double*)c, ldc, fine.n[0], fine.n[1], fine.n[2], mask);
    else
        restrict_kernel<float, float><<<g, nt, 0, s>>>((const float*)f, ldf,
            (float*)c, ldc, fine.n[0], fine.n[1], fine.n[2], mask);
    MGX_LAUNCH_CHECK("restrict_kernel");
    return MGX_OK;
}

/* MGX_PROLONG4=0 keeps the pair form for FP32 (the same bits) */
static bool prolong4_on()
{
    static const bool on = [] {
        const char* e = getenv("MGX_PROLONG4");
        return !(e && e[0] == '0');
    }();
    return on;
}

int prolong_launch(int dtype, int mode, const Level& fine, const void* c,
    size_t ldc, void* out, size_t ldo, int nfunc, const MaskDev& mask,
    cudaStream_t s)
{
    if (dtype == MGX_F32 && (fine.n[2] % 4) == 0 && (ldo % 4) == 0
        && ((uintptr_t)out % 16) == 0 && prolong4_on())
    {
        const int bands4 = ((fine.n[1] / 2) + PROLONG4_CROWS - 1) / PROLONG4_CROWS;
        const dim3 g4(fine.n[0] * bands4, nfunc);
        if (mode == 0)
            prolong4_kernel<0><<<g4, 256, 0, s>>>((const float*)c, ldc, (float*)out, ldo,
                fine.n[0], fine.n[1], fine.n[2], mask);
        else
            prolong4_kernel<1><<<g4, 256, 0, s>>>((const float*)c, ldc, (float*)out, ldo,
                fine.n[0], fine.n[1], fine.n[2], mask);
        MGX_LAUNCH_CHECK("prolong4_kernel");
        return MGX_OK;
    }
    const int bands = ((fine.n[1] / 2) + PROLONG_CROWS - 1) / PROLONG_CROWS;
    const dim3 g(fine.n[0] * bands, nfunc);
    const int nt = 256;
    const size_t es = dtype_size(dtype);
    const bool v2   = ((ldo % 2) == 0) && ((uintptr_t)out % (2 * es) == 0);
#define MGX_PROLONG(T, M, V)                                                                 \
    prolong_kernel<T, M, V><<<g, nt, 0, s>>>((const T*)c, ldc, (T*)out, ldo, fine.n[0],     \
        fine.n[1], fine.n[2], mask)
    if (dtype == MGX_F64)
    {
        if (mode == 0)
            v2 ? MGX_PROLONG(double, 0, true) : MGX_PROLONG(double, 0, false);
        else
            v2 ? MGX_PROLONG(double, 1, true) : MGX_PROLONG(double, 1, false);
    }
    else
    {
        if (mode == 0)
            v2 ? MGX_PROLONG(float, 0, true) : MGX_PROLONG(float, 0, false);
        else
            v2 ? MGX_PROLONG(float, 1, true) : MGX_PROLONG(float, 1, false);
    }
#undef MGX_PROLONG
    MGX_LAUNCH_CHECK("prolong_kernel");
    return MGX_OK;
}

int scale_launch(int dtype, const void* in, size_t ldi, void* out, size_t ldo,
    size_t npts, int nfunc, double alpha, cudaStream_t s)
{
    const dim3 g = grid_for(npts, nfunc);
    if (dtype == MGX_F64)
        scale_kernel<double><<<g, 256, 0, s>>>((const double*)in, ldi,
            (double*)out, ldo, npts, alpha);
    else
        scale_kernel<float><<<g, 256, 0, s>>>((const float*)in, ldi,
            (float*)out, ldo, npts, (float)alpha);
    MGX_LAUNCH_CHECK("scale_kernel");
    return MGX_OK;
}

/* ------------------------------------------------------------------ */
/* masks                                                                */
/* ------------------------------------------------------------------ */
struct MaskJob
{
    double center[3];
    double rcut;
    double rc_inv;
    double overlap_radius;
    int box[6];
    size_t offset;
    int func;
};

/* GridMask::init over the box of one (orbital, level) job; grid-stride
 * over the box points of all jobs of the level. */
template <typename M>
__global__ void mask_values_kernel(const MaskJob* jobs, int njobs,
    const double* cx, const double* cy, const double* cz, int nx, int ny,
    int nz, double llx, double lly, double llz, double exp2_rc,
    double exp2_coeff, M* values, unsigned long long* counts)
{
    const int j = blockIdx.y;
    if (j >= njobs) return;
    const MaskJob& J = jobs[j];
    const size_t nb  = (size_t)J.box[3] * J.box[4] * J.box[5];
    unsigned long long ni = 0, nc = 0;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nb;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const int dz = (int)(t % J.box[5]);
        const int dy = (int)((t / J.box[5]) % J.box[4]);
        const int dx = (int)(t / ((size_t)J.box[5] * J.box[4]));
        int x = J.box[0] + dx;
        if (x >= nx) x -= nx;
        int y = J.box[1] + dy;
        if (y >= ny) y -= ny;
        int z = J.box[2] + dz;
        if (z >= nz) z -= nz;
        // Vector3D::minimage (src/tools/Vector3D.cc:13-30), no contraction
        const double d0 = remainder(__dsub_rn(cx[x], J.center[0]), llx);
        const double d1 = remainder(__dsub_rn(cy[y], J.center[1]), lly);
        const double d2 = remainder(__dsub_rn(cz[z], J.center[2]), llz);
        const double r
            = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)),
                __dmul_rn(d2, d2)));
        M val = (M)0;
        if (r < J.overlap_radius)
        {
            ni++;
            if (r <= J.rcut)
            {
                nc++;
                const double rr = __dmul_rn(r, J.rc_inv);
                if (J.func == 0)
                {
                    // gaussianDecay, src/MasksSet.cc:37-48
                    float fv = 1.f;
                    if (rr > 0.75)
                    {
                        const double t1 = __dsub_rn(rr, 0.75);
                        const double ex = exp(__dmul_rn(__dmul_rn(-32., t1), t1));
                        fv              = (float)__dmul_rn(__dsub_rn(ex, exp2_rc),
                            exp2_coeff);
                    }
                    val = (M)fv;
                }
                else
                {
                    // one, src/MasksSet.cc:26-35
                    if (rr < 0.99999)
                        val = (M)1.;
                    else
                        val = (M)__dmul_rn(__dsub_rn(1., rr), 1. / (1. - 0.99999));
                }
            }
        }
        values[J.offset + t] = val;
    }
    // warp reduction of the counts
    for (int o = 16; o > 0; o >>= 1)
    {
        ni += __shfl_down_sync(0xffffffffu, ni, o);
        nc += __shfl_down_sync(0xffffffffu, nc, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        atomicAdd(counts + 2 * j, ni);
        atomicAdd(counts + 2 * j + 1, nc);
    }
}

/* SubCell::spherePossibleOverlap for the single subdomain of a level
 * (src/SubCell.cc:14-95) */
static bool sphere_overlap(const double center[3], double radius,
    const double ll[3], const int dims[3], const double hs[3])
{
    double vd[3];
    for (int i = 0; i < 3; i++)
    {
        const double subdim = (dims[i] - 1) * hs[i];
        const double cc     = 0. + 0.5 * subdim;
        const double d      = cc - center[i];
        double r            = fmod(d, ll[i]);
        const double ax2    = 0.5 * ll[i];
        if (r > ax2)
            r -= ll[i];
        else if (r < -ax2)
            r += ll[i];
        const double vc = r < 0. ? std::max(-0.5 * subdim, r) : std::min(0.5 * subdim, r);
        vd[i]           = r - vc;
    }
    const double dc = sqrt(vd[0] * vd[0] + vd[1] * vd[1] + vd[2] * vd[2]);
    return dc <= radius;
}

int masks_create(mgx_ctx* ctx, int nlevels, int nfunc, const double* centers,
    const double* radii, int func, int kind, int mesh_ghosts, int dtype,
    mgx_masks** out, cudaStream_t s)
{
    if (nlevels < 1 || nlevels > 8 || nfunc < 1 || !centers || !radii || !out)
        return fail(MGX_BAD_ARG, "masks_create: bad arguments");
    if (func != 0 && func != 1) return fail(MGX_BAD_ARG, "mask func %d", func);
    if (kind != 0 && kind != 1) return fail(MGX_BAD_ARG, "mask kind %d", kind);
    const mgx_grid& g = ctx->grid;
    std::unique_ptr<mgx_masks> M(new mgx_masks);
    M->nlevels     = nlevels;
    M->nfunc       = nfunc;
    M->kind        = kind;
    M->dtype       = dtype;
    M->func        = func;
    M->mesh_ghosts = mesh_ghosts;
    for (int i = 0; i < 3; i++)
        M->n[i] = g.n[i];
    M->state.resize(nlevels);
    M->box.resize(nlevels);
    M->offset.resize(nlevels);
    M->values.resize(nlevels);
    M->h_state.resize(nlevels);
    M->h_box.resize(nlevels);
    M->dev.resize(nlevels);

    const double h[3] = { g.ll[0] / g.n[0], g.ll[1] / g.n[1], g.ll[2] / g.n[2] };
    const double exp2_rc    = exp(-32. * (1. - 0.75) * (1. - 0.75));
    const double exp2_coeff = 1. / (1. - exp2_rc);
    const size_t esz        = dtype_size(dtype);
    DeviceBuffer d_coords, d_jobs, d_counts;

    for (int l = 0; l < nlevels; l++)
    {
        const int nl[3] = { g.n[0] >> l, g.n[1] >> l, g.n[2] >> l };
        double delta = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) + 1.e-8;
        delta *= (double)mesh_ghosts;
        for (int k = 0; k < l; k++)
            delta *= 2.;
        double hs[3] = { h[0], h[1], h[2] };
        for (int k = 0; k < l; k++)
            for (int i = 0; i < 3; i++)
                hs[i] *= 2.;
        const double hl[3] = { h[0] * (1 << l), h[1] * (1 << l), h[2] * (1 << l) };
        // per-axis coordinates by repeated addition (src/GridMask.cc:190-234)
        std::vector<double> coords(nl[0] + nl[1] + nl[2]);
        {
            size_t o = 0;
            for (int i = 0; i < 3; i++)
            {
                double xc = 0.;
                for (int k = 0; k < nl[i]; k++)
                {
                    coords[o++] = xc;
                    xc += hl[i];
                }
            }
        }
        std::vector<int>& st = M->h_state[l];
        std::vector<int>& bx = M->h_box[l];
        st.assign(nfunc, 0);
        bx.assign(6 * (size_t)nfunc, 0);
        std::vector<size_t> offs(nfunc, 0);
        std::vector<MaskJob> jobs;
        size_t total = 0;
        for (int f = 0; f < nfunc; f++)
        {
            const double* c  = centers + 3 * f;
            const double rc  = radii[f];
            const double ovr = rc + delta;
            if (!(rc > 0.001)) return fail(MGX_BAD_ARG, "mask radius %g too small", rc);
            if (!sphere_overlap(c, ovr, g.ll, nl, hs))
            {
                st[f] = -1;
                continue;
            }
            if (100. < rc)
            {
                st[f] = 1;
                continue;
            }
            MaskJob J;
            for (int i = 0; i < 3; i++)
                J.center[i] = c[i];
            J.rcut           = rc;
            J.rc_inv         = 1. / rc;
            J.overlap_radius = ovr;
            J.func           = func;
            for (int i = 0; i < 3; i++)
            {
                const int k   = (int)ceil(ovr / hl[i]) + 2;
                const int ext = 2 * k + 1;
                if (ext >= nl[i])
                {
                    J.box[i]     = 0;
                    J.box[3 + i] = nl[i];
                }
                else
                {
                    int ci = (int)floor(c[i] / hl[i]);
                    int b0 = ci - k;
                    b0 %= nl[i];
                    if (b0 < 0) b0 += nl[i];
                    J.box[i]     = b0;
                    J.box[3 + i] = ext;
                }
            }
            J.offset = total;
            offs[f]  = total;
            total += (size_t)J.box[3] * J.box[4] * J.box[5];
            for (int i = 0; i < 6; i++)
                bx[6 * f + i] = J.box[i];
            st[f] = 2; // provisional, fixed from the counts below
            jobs.push_back(J);
        }
        MGX_TRY(M->values[l].ensure(std::max<size_t>(total, 1) * esz));
        if (!jobs.empty())
        {
            MGX_TRY(d_coords.ensure(coords.size() * sizeof(double)));
            MGX_TRY(d_jobs.ensure(jobs.size() * sizeof(MaskJob)));
            MGX_TRY(d_counts.ensure(jobs.size() * 2 * sizeof(unsigned long long)));
            MGX_TRY(cuda_check(cudaMemcpyAsync(d_coords.ptr, coords.data(),
                                   coords.size() * sizeof(double),
                                   cudaMemcpyHostToDevice, s),
                "mask coords upload"));
            MGX_TRY(cuda_check(cudaMemcpyAsync(d_jobs.ptr, jobs.data(),
                                   jobs.size() * sizeof(MaskJob),
                                   cudaMemcpyHostToDevice, s),
                "mask jobs upload"));
            MGX_TRY(cuda_check(cudaMemsetAsync(d_counts.ptr, 0,
                                   jobs.size() * 2 * sizeof(unsigned long long), s),
                "mask counts"));
            const double* dc = (const double*)d_coords.ptr;
            size_t maxbox    = 0;
            for (auto& J : jobs)
                maxbox = std::max(maxbox, (size_t)J.box[3] * J.box[4] * J.box[5]);
            // one grid row per job (jobs are processed in slices of 65535)
            for (size_t j0 = 0; j0 < jobs.size(); j0 += 65535)
            {
                const int nj = (int)std::min<size_t>(65535, jobs.size() - j0);
                dim3 grid((unsigned)std::min<size_t>((maxbox + 255) / 256, 256), nj);
                const MaskJob* dj = (const MaskJob*)d_jobs.ptr + j0;
                unsigned long long* cnt = (unsigned long long*)d_counts.ptr + 2 * j0;
                if (dtype == MGX_F64)
                    mask_values_kernel<double><<<grid, 256, 0, s>>>(dj, nj, dc,
                        dc + nl[0], dc + nl[0] + nl[1], nl[0], nl[1], nl[2], g.ll[0],
                        g.ll[1], g.ll[2], exp2_rc, exp2_coeff,
                        (double*)M->values[l].ptr, cnt);
                else
                    mask_values_kernel<float><<<grid, 256, 0, s>>>(dj, nj, dc,
                        dc + nl[0], dc + nl[0] + nl[1], nl[0], nl[1], nl[2], g.ll[0],
                        g.ll[1], g.ll[2], exp2_rc, exp2_coeff,
                        (float*)M->values[l].ptr, cnt);
                MGX_LAUNCH_CHECK("mask_values_kernel");
            }
            std::vector<unsigned long long> counts(jobs.size() * 2);
            MGX_TRY(cuda_check(cudaMemcpyAsync(counts.data(), d_counts.ptr,
                                   counts.size() * sizeof(unsigned long long),
                                   cudaMemcpyDeviceToHost, s),
                "mask counts download"));
            MGX_TRY(cuda_check(cudaStreamSynchronize(s), "mask build sync"));
            // GridMask::assign (src/GridMask.cc:311-339) from the counts
            size_t jj = 0;
            for (int f = 0; f < nfunc; f++)
            {
                if (st[f] != 2) continue;
                unsigned long long icount = counts[2 * jj], ncount = counts[2 * jj + 1];
                jj++;
                if (l == 0 && icount < 1) icount = 1;
                if (ncount == 0 && icount == 0)
                    st[f] = -1;
                else if (ncount == 0)
                    st[f] = 0;
                else
                    st[f] = 2;
            }
        }
        MGX_TRY(M->state[l].ensure(nfunc * sizeof(int)));
        MGX_TRY(M->box[l].ensure(6 * (size_t)nfunc * sizeof(int)));
        MGX_TRY(M->offset[l].ensure(nfunc * sizeof(size_t)));
        MGX_TRY(cuda_check(cudaMemcpyAsync(M->state[l].ptr, st.data(),
                               nfunc * sizeof(int), cudaMemcpyHostToDevice, s),
            "mask state upload"));
        MGX_TRY(cuda_check(cudaMemcpyAsync(M->box[l].ptr, bx.data(),
                               bx.size() * sizeof(int), cudaMemcpyHostToDevice, s),
            "mask box upload"));
        MGX_TRY(cuda_check(cudaMemcpyAsync(M->offset[l].ptr, offs.data(),
                               nfunc * sizeof(size_t), cudaMemcpyHostToDevice, s),
            "mask offset upload"));
        MGX_TRY(cuda_check(cudaStreamSynchronize(s), "mask upload sync"));
        MaskDev& D = M->dev[l];
        D.state    = (const int*)M->state[l].ptr;
        D.box      = (const int*)M->box[l].ptr;
        D.offset   = (const size_t*)M->offset[l].ptr;
        D.values   = M->values[l].ptr;
        for (int i = 0; i < 3; i++)
            D.n[i] = nl[i];
        D.kind = kind;
    }
    *out = M.release();
    return MGX_OK;
}

/* MasksSet::update (src/MasksSet.cc:208-218): the set rebuilt for moved
 * centres or new radii, with its levels, functions, profile and kind; the
 * handle keeps its address, so calls holding it see the new masks */
int masks_update(mgx_ctx* ctx, mgx_masks* M, const double* centers, const double* radii,
    cudaStream_t s)
{
    if (!M || !centers || !radii) return fail(MGX_BAD_ARG, "masks_update: bad arguments");
    mgx_masks* T = nullptr;
    MGX_TRY(masks_create(ctx, M->nlevels, M->nfunc, centers, radii, M->func, M->kind,
        M->mesh_ghosts, M->dtype, &T, s));
    std::swap(*M, *T);
    delete T;
    return MGX_OK;
}

/* masks of functions [f0, f0 + nf) at level l, as seen by a launch whose
 * blockIdx.y runs over those functions */
MaskDev mask_slice(const mgx_masks* M, int level, int f0)
{
    MaskDev D;
    if (M == nullptr || level >= M->nlevels) return D;
    D = M->dev[level];
    D.state += f0;
    D.box += 6 * (size_t)f0;
    D.offset += f0;
    return D;
}

int masks_apply(mgx_ctx* ctx, const mgx_masks* M, int level, void* u, size_t ld,
    int nfunc, cudaStream_t s)
{
    if (!M || level < 0 || level >= M->nlevels || nfunc > M->nfunc)
        return fail(MGX_BAD_ARG, "masks_apply: bad level or nfunc");
    const Level L = make_level(ctx->grid, level);
    const MaskDev D = mask_slice(M, level, 0);
    const dim3 g    = grid_for(L.npts(), nfunc);
    if (M->dtype == MGX_F64)
        mask_apply_kernel<double><<<g, 256, 0, s>>>((double*)u, ld, L.n[0], L.n[1], L.n[2], D);
    else
        mask_apply_kernel<float><<<g, 256, 0, s>>>((float*)u, ld, L.n[0], L.n[1], L.n[2], D);
    MGX_LAUNCH_CHECK("mask_apply_kernel");
    return MGX_OK;
}

template <typename T>
__global__ void mask_expand_kernel(T* dense, int nx, int ny, int nz, MaskDev m)
{
    const int f       = blockIdx.y;
    const size_t npts = (size_t)nx * ny * nz;
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
         idx += (size_t)gridDim.x * blockDim.x)
    {
        const int z = (int)(idx % nz);
        const int y = (int)((idx / nz) % ny);
        const int x = (int)(idx / ((size_t)nz * ny));
        const int st = m.state[f];
        T v          = (T)0;
        if (st == 1)
            v = (T)1;
        else if (st == 2)
        {
            const int* b = m.box + 6 * f;
            int dx = x - b[0], dy = y - b[1], dz = z - b[2];
            if (dx < 0) dx += nx;
            if (dy < 0) dy += ny;
            if (dz < 0) dz += nz;
            if (dx < b[3] && dy < b[4] && dz < b[5])
                v = reinterpret_cast<const T*>(m.values)[m.offset[f]
                                                         + ((size_t)dx * b[4] + dy) * b[5]
                                                         + dz];
        }
        dense[(size_t)f * npts + idx] = v;
    }
}

int masks_expand(const mgx_masks* M, int level, void* dense, int* host_state,
    cudaStream_t s)
{
    if (!M || level < 0 || level >= M->nlevels)
        return fail(MGX_BAD_ARG, "masks_expand: bad level");
    const MaskDev D = M->dev[level];
    const size_t np = (size_t)D.n[0] * D.n[1] * D.n[2];
    const dim3 g    = grid_for(np, M->nfunc);
    if (M->dtype == MGX_F64)
        mask_expand_kernel<double><<<g, 256, 0, s>>>((double*)dense, D.n[0], D.n[1], D.n[2], D);
    else
        mask_expand_kernel<float><<<g, 256, 0, s>>>((float*)dense, D.n[0], D.n[1], D.n[2], D);
    MGX_LAUNCH_CHECK("mask_expand_kernel");
    if (host_state)
        std::memcpy(host_state, M->h_state[level].data(), M->nfunc * sizeof(int));
    return MGX_OK;
}

/* ------------------------------------------------------------------ */
/* the V-cycle                                                          */
/* ------------------------------------------------------------------ */
/* The second pre-sweep of a level restricts its residual in the same kernel
 * (OP_JACOBI_RST) unless MGX_FUSED_RESTRICT=0: the residual block is then
 * neither written nor read again.  The results are the same bits either
 * way (the restriction keeps restrict_kernel's operation order). */
static bool fused_restrict()
{
    static const bool on = [] {
        const char* e = getenv("MGX_FUSED_RESTRICT");
        return !(e && e[0] == '0');
    }();
    return on;
}

/* Both post-sweeps of a level in one kernel, and both pre-sweeps where the
 * pair pays (jacobi2_launch: the first sweep's iterate stays on chip),
 * unless MGX_TWO_SWEEPS=0.  The results are the same bits either way. */
static bool two_sweeps()
{
    static const bool on = [] {
        const char* e = getenv("MGX_TWO_SWEEPS");
        return !(e && e[0] == '0');
    }();
    return on;
}

/* The pre-sweep pair forms its first sweep on two more rows than the tile
 * and its second sweep's residual on one more, so it re-does more work the
 * lower the tile: it runs when the tile holds at least JJ_PAIR_MIN_ROWS
 * rows (at most a quarter more first-sweep rows).  On 192^3 FP32 a
 * 256-thread tile holds 6 rows and the pair ran 23.2 ms per 512 orbitals
 * against 20.7 ms for the two single kernels; a 512-thread tile holds 16
 * and it ran 19.6 ms.  MGX_PRE_PAIR=1 runs it whenever the kernel can, 0
 * never. */
static int pre_pair_policy()
{
    static const int v = [] {
        const char* e = getenv("MGX_PRE_PAIR");
        return e ? (e[0] == '0' ? 0 : 1) : -1;
    }();
    return v;
}

/* The post-sweep pair starts from u - P e formed on chip (the coarse-grid
 * correction folded into it, JJ_PRO) when MGX_PAIR_PROLONG=1; by default the
 * prolongation kernel runs first: the folded correction runs between the
 * planes' barriers and made the V-cycle of 512 orbitals on 192^3 16 %
 * slower (52.0 against 44.9 ms).  The same bits either way. */
static bool pair_prolong()
{
    static const bool on = [] {
        const char* e = getenv("MGX_PAIR_PROLONG");
        return e && e[0] == '1';
    }();
    return on;
}

struct VCycle
{
    mgx_ctx* ctx;
    int dtype;
    int lap_type;
    int L; // maxlevels
    int nf;
    int f0;
    const mgx_masks* masks;
    cudaStream_t s;
    std::vector<Level> lev;
    std::vector<double> jf;
    // per level: v[2], w, f  (level 0: v[0] = caller out, f = caller res)
    std::vector<void*> v0, v1, w, f;
    std::vector<size_t> ld;
    int* err;

    double gamma = 0.;
    bool pending_scale = false; // level-0 iterate still to be set to gamma*f
    // fused update: the last level-0 sweep adds upd_alpha * v to upd0
    // (chunk base) instead of storing v
    void* upd0       = nullptr;
    double upd_alpha = 0.;
    const double* upd_scale0 = nullptr; // per-function scale of the update (chunk base)

    // with restricted set, a sweep that writes w may restrict it in the same
    // kernel into the next level's right-hand side (f[l + 1]) instead of
    // storing it; *restricted tells the caller that it did
    int jacobi(int l, int cur, bool write_w, bool last = false, bool* restricted = nullptr)
    {
        PlaneParams p;
        if (last && l == 0 && upd0)
        {
            p.upd       = upd0;
            p.ldupd     = ld[0];
            p.upd_alpha = upd_alpha;
            p.upd_scale = upd_scale0;
        }
        if (l == 0 && pending_scale)
        {
            // first sweep straight from f with u = gamma f
            p.gamma_in = gamma;
            p.u        = f[0];
            p.ldu      = ld[0];
            p.f        = f[0];
            p.ldf      = ld[0];
            p.out      = cur ? v0[0] : v1[0];
            p.ldo      = ld[0];
            p.w        = write_w ? w[0] : nullptr;
            p.ldw      = ld[0];
            for (int i = 0; i < 3; i++)
                p.n[i] = lev[0].n[i];
            p.mask = mask_slice(masks, 0, f0);
            p.err  = err;
            int st = stencil_launch(OP_JACOBI, lap_type, dtype, dtype, p, lev[0], jf[0], nf, s);
            if (st == MGX_UNSUPPORTED)
            {
                // v = gamma * res (src/OrbitalsPreconditioning.cc:102-107), then a plain sweep
                st = scale_launch(dtype, f[0], ld[0], cur ? v1[0] : v0[0], ld[0],
                    lev[0].npts(), nf, gamma, s);
                if (st != MGX_OK) return st;
                pending_scale = false;
                return jacobi(l, cur, write_w);
            }
            pending_scale = false;
            return st;
        }
        p.u   = cur ? v1[l] : v0[l];
        p.ldu = ld[l];
        p.f   = f[l];
        p.ldf = ld[l];
        p.out = cur ? v0[l] : v1[l];
        p.ldo = ld[l];
        p.w   = write_w ? w[l] : nullptr;
        p.ldw = ld[l];
        for (int i = 0; i < 3; i++)
            p.n[i] = lev[l].n[i];
        p.mask = mask_slice(masks, l, f0);
        p.err  = err;
        if (restricted && write_w && !p.upd && masks == nullptr && l < L && fused_restrict())
        {
            PlaneParams q = p;
            q.w           = nullptr;
            q.coarse      = f[l + 1];
            q.ldc         = ld[l + 1];
            const int st  = stencil_launch(OP_JACOBI_RST, l == 0 ? lap_type : 1, dtype, dtype, q,
                lev[l], jf[l], nf, s);
            if (st != MGX_UNSUPPORTED)
            {
                *restricted = (st == MGX_OK);
                return st;
            }
        }
        return stencil_launch(p.upd ? OP_JACOBI_UPD : OP_JACOBI, l == 0 ? lap_type : 1, dtype,
            dtype, p, lev[l], jf[l], nf, s);
    }

    // both sweeps of a level's pre-smoothing (pre: the second one's
    // residual restricted into f[l + 1]) or post-smoothing (the last one
    // with the fused update at level 0; pro: from u - P pro, pro the next
    // level's correction) in one kernel, from buffer cur into the other
    // one; dry: only whether the kernel runs the block
    int jacobi2(int l, int cur, bool pre, bool dry, const void* pro = nullptr, int* ty = nullptr)
    {
        PlaneParams p;
        p.u   = cur ? v1[l] : v0[l];
        p.ldu = ld[l];
        p.f   = f[l];
        p.ldf = ld[l];
        p.out = cur ? v0[l] : v1[l];
        p.ldo = ld[l];
        for (int i = 0; i < 3; i++)
            p.n[i] = lev[l].n[i];
        p.err    = err;
        int mode = JJ_STORE;
        if (pre)
        {
            if (l == 0 && pending_scale)
            {
                // first sweep straight from f with u = gamma f
                p.gamma_in = gamma;
                p.u        = f[0];
                p.ldu      = ld[0];
            }
            p.coarse = f[l + 1];
            p.ldc    = ld[l + 1];
            mode     = JJ_RST;
        }
        else if (l == 0 && upd0)
        {
            p.upd       = upd0;
            p.ldupd     = ld[0];
            p.upd_alpha = upd_alpha;
            p.upd_scale = upd_scale0;
            mode        = JJ_UPD;
        }
        if (!pre && pro)
        {
            p.pro   = pro;
            p.ldpro = ld[l + 1];
            mode |= JJ_PRO;
        }
        const int st = jacobi2_launch(mode, l == 0 ? lap_type : 1, dtype, p, lev[l], jf[l], nf, s,
            dry, ty);
        if (!dry && pre && st == MGX_OK && l == 0) pending_scale = false;
        return st;
    }

    // returns the buffer index holding the result at level l
    int mg(int l)
    {
        int cur         = 0;
        const int ncycl = (l == L) ? 4 : 2;
        bool restricted = false;
        // the coarsest level's four sweeps as two pairs (an even count of
        // buffer moves either way); level 0 without coarse levels keeps its
        // single sweeps, whose last one may carry the update
        if (l == L && l > 0 && two_sweeps() && masks == nullptr
            && jacobi2(l, 0, false, true) == MGX_OK)
        {
            for (int it = 0; it < 2; it++)
            {
                const int st = jacobi2(l, cur, false, false);
                if (st != MGX_OK) return -st - 1;
                cur ^= 1;
            }
            return cur;
        }
        const bool can = l < L && two_sweeps() && masks == nullptr;
        int ty_pre      = 0;
        bool pre_pair   = can && fused_restrict() && pre_pair_policy() != 0
                        && jacobi2(l, 0, true, true, nullptr, &ty_pre) == MGX_OK
                        && (pre_pair_policy() == 1 || ty_pre >= JJ_PAIR_MIN_ROWS);
        bool post_pair = can && jacobi2(l, 1, false, true) == MGX_OK;
        // a pair moves the iterate to the other buffer once where two single
        // sweeps move it twice.  Level 0 must end in buffer 0 (the caller's
        // block): with an odd count the first sweep, which reads only f when
        // it starts from gamma f, writes into buffer 0 instead of 1; a warm
        // start reads buffer 0, so it runs both pairs or neither
        if (l == 0 && ((pre_pair ? 1 : 2) + (post_pair ? 1 : 2)) % 2)
        {
            if (pending_scale)
                cur = 1;
            else
                pre_pair = post_pair = false;
        }
        // the correction folded into the post-sweep pair (checked with a
        // stand-in block: the coarse result's buffer is known only later)
        const bool pair_pro = post_pair && pair_prolong()
                              && jacobi2(l, cur ^ 1, false, true, v0[l + 1]) == MGX_OK;
        if (pre_pair)
        {
            const int st = jacobi2(l, cur, true, false);
            if (st != MGX_OK) return -st - 1;
            cur ^= 1;
            restricted = true;
        }
        else
            for (int it = 0; it < ncycl; it++)
            {
                // without coarse levels the last of these sweeps is the final one
                const int st = jacobi(l, cur, (it == ncycl - 1) && (l < L),
                    (l == L) && (it == ncycl - 1), &restricted);
                if (st != MGX_OK) return -st - 1;
                cur ^= 1;
            }
        if (l == L) return cur;
        int st = MGX_OK;
        if (!restricted)
            st = restrict_launch(dtype, lev[l], w[l], ld[l], f[l + 1], ld[l + 1], nf,
                mask_slice(masks, l + 1, f0), s);
        if (st != MGX_OK) return -st - 1;
        st = cuda_check(cudaMemsetAsync(v0[l + 1], 0,
                            ld[l + 1] * nf * dtype_size(dtype), s),
            "coarse zero");
        if (st != MGX_OK) return -st - 1;
        const int c1 = mg(l + 1);
        if (c1 < 0) return c1;
        if (pair_pro)
        {
            st = jacobi2(l, cur, false, false, c1 ? v1[l + 1] : v0[l + 1]);
            if (st != MGX_OK) return -st - 1;
            return cur ^ 1;
        }
        st = prolong_launch(dtype, 1, lev[l], c1 ? v1[l + 1] : v0[l + 1],
            ld[l + 1], cur ? v1[l] : v0[l], ld[l], nf, mask_slice(masks, l, f0), s);
        if (st != MGX_OK) return -st - 1;
        if (post_pair)
        {
            st = jacobi2(l, cur, false, false);
            if (st != MGX_OK) return -st - 1;
            return cur ^ 1;
        }
        for (int it = 0; it < 2; it++)
        {
            st = jacobi(l, cur, false, it == 1);
            if (st != MGX_OK) return -st - 1;
            cur ^= 1;
        }
        return cur;
    }
};

/* out = V-cycle(res); or, with upd set, upd += alpha * V-cycle(res)
 * through the last fine-level sweep (upd_j = scale_j (upd_j + alpha
 * V-cycle(res)_j) when scale is given), and out (nfunc x ld, may be NULL)
 * is only scratch for the fine-level iterate.  warm: the V-cycle starts
 * from the iterate that out holds on entry instead of gamma * res. */
int precond_mg(mgx_ctx* ctx, const mgx_precond_params* P, int dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks,
    cudaStream_t s, void* upd = nullptr, double alpha = 0., const double* scale = nullptr,
    bool warm = false)
{
    if (!P || !res || (!out && !upd) || nfunc < 0)
        return fail(MGX_BAD_ARG, "precond_mg: null argument");
    if (warm && (!out || upd))
        return fail(MGX_BAD_ARG, "precond_mg: a warm start needs out and no update block");
    if (res == out || res == upd || (upd && upd == out))
        return fail(MGX_BAD_ARG, "precond_mg: res, out and the update block alias");
    if (P->lap_type < 0 || P->lap_type > 4) return fail(MGX_BAD_ARG, "lap_type %d", P->lap_type);
    const int L = P->maxlevels;
    if (L < 0 || L > 6) return fail(MGX_BAD_ARG, "maxlevels %d", L);
    const mgx_grid& g = ctx->grid;
    for (int l = 0; l < L; l++)
        for (int i = 0; i < 3; i++)
            if ((g.n[i] >> l) % 2)
                return fail(MGX_BAD_ARG, "grid dimension %d not divisible by 2^%d", i, L);
    if (masks && (masks->nlevels < L + 1 || masks->nfunc < nfunc))
        return fail(MGX_BAD_ARG, "masks cover %d levels / %d functions", masks->nlevels, masks->nfunc);
    if (nfunc == 0) return MGX_OK;
    const size_t es = dtype_size(dtype);

    VCycle V;
    V.ctx      = ctx;
    V.dtype    = dtype;
    V.lap_type = P->lap_type;
    V.L        = L;
    V.masks    = masks;
    V.s        = s;
    for (int l = 0; l <= L; l++)
    {
        V.lev.push_back(make_level(g, l));
        V.jf.push_back(jacobi_factor(l == 0 ? P->lap_type : 1, V.lev[l].h));
    }
    // workspace per function: level 0: v1 + w (+ v0 when the update is
    // fused and the caller gave no scratch block), each with the caller's
    // leading dimension ld, as every level-0 array is addressed with it;
    // level l>0: v0, v1, w, f
    const bool own_v0 = upd && !out;
    size_t per_func   = (own_v0 ? 3 : 2) * ld;
    for (int l = 1; l <= L; l++)
        per_func += 4 * V.lev[l].npts();
    per_func *= es;
    int chunk = P->chunk > 0 ? P->chunk : nfunc;
    if (P->chunk <= 0)
    {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        const size_t cap = (size_t)(0.4 * (double)(fr + ctx->vc.bytes));
        if (per_func * (size_t)chunk > cap)
            chunk = (int)std::max<size_t>(1, cap / per_func);
    }
    chunk = std::min(chunk, 65535);
    chunk = std::min(chunk, nfunc);
    MGX_TRY(ctx->vc.ensure(per_func * chunk + 256));
    MGX_TRY(ctx->flag.ensure(256));
    V.err = (int*)ctx->flag.ptr;
    MGX_TRY(cuda_check(cudaMemsetAsync(V.err, 0, sizeof(int), s), "flag reset"));

    for (int f0 = 0; f0 < nfunc; f0 += chunk)
    {
        const int nf = std::min(chunk, nfunc - f0);
        V.nf = nf;
        V.f0 = f0;
        V.v0.assign(L + 1, nullptr);
        V.v1.assign(L + 1, nullptr);
        V.w.assign(L + 1, nullptr);
        V.f.assign(L + 1, nullptr);
        V.ld.assign(L + 1, 0);
        char* base = (char*)ctx->vc.ptr;
        V.ld[0]    = ld;
        V.f[0]     = (void*)((const char*)res + (size_t)f0 * ld * es);
        if (own_v0)
        {
            V.v0[0] = base;
            base += (size_t)nf * ld * es;
        }
        else
            V.v0[0] = (char*)out + (size_t)f0 * ld * es;
        if (upd)
        {
            V.upd0       = (char*)upd + (size_t)f0 * ld * es;
            V.upd_alpha  = alpha;
            V.upd_scale0 = scale ? scale + f0 : nullptr;
        }
        V.v1[0]    = base;
        base += (size_t)nf * ld * es;
        V.w[0] = base;
        base += (size_t)nf * ld * es;
        for (int l = 1; l <= L; l++)
        {
            const size_t pl = V.lev[l].npts();
            V.ld[l]         = pl;
            V.v0[l]         = base;
            base += (size_t)nf * pl * es;
            V.v1[l] = base;
            base += (size_t)nf * pl * es;
            V.w[l] = base;
            base += (size_t)nf * pl * es;
            V.f[l] = base;
            base += (size_t)nf * pl * es;
        }
        // v = gamma * res (src/OrbitalsPreconditioning.cc:102-107), or, for
        // a warm start, the iterate the caller left in out
        V.gamma         = P->gamma;
        V.pending_scale = !warm;
        const int c = V.mg(0);
        if (c < 0) return -(c + 1);
        if (c != 0) return fail(MGX_UNSUPPORTED, "V-cycle ended in the work buffer");
    }
    return MGX_OK;
}

/* ------------------------------------------------------------------ */
/* Allocation-free V-cycle                                              */
/* ------------------------------------------------------------------ */
// For callers that cannot allocate device memory at all: host programs
// whose device memory is owned by a pool they do not control (an
// application that reserves the GPU's memory up front and hands out slices
// of it), or plug-ins loaded into a process that forbids device allocations
// after start-up (cudaMalloc may synchronize the device and stall every
// other stream of the process).  The V-cycle's level buffers and status
// word then live in this file-scope device array instead of the context
// workspace.  The array is part of the library's device image: every GPU
// that loads the library holds these 64 MiB until the process exits.
constexpr size_t STATIC_VCYCLE_SCRATCH_BYTES = size_t(64) << 20;
constexpr size_t STATIC_VCYCLE_STATUS_BYTES  = 256;
static __device__ __align__(256) unsigned char g_vcycle_scratch[STATIC_VCYCLE_SCRATCH_BYTES];

namespace
{
constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mutex;
void* g_scratch_address[MAX_DEVICES] = {};

/* Device address of the static scratch on the current device.  The host
 * symbol g_vcycle_scratch is only a stand-in for the device array; its
 * device address is looked up once per device, with that device current,
 * on the first call that needs it.  The cached address belongs to the device's primary
 * context as it was at that first call: it assumes that context lives as
 * long as the process (no cudaDeviceReset in between). */
int static_scratch_address(void** ptr)
{
    int dev = 0;
    MGX_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
    if (dev < 0 || dev >= MAX_DEVICES)
        return fail(MGX_UNSUPPORTED, "device index %d beyond %d", dev, MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_scratch_mutex);
    if (g_scratch_address[dev] == nullptr)
    {
        void* p       = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_vcycle_scratch);
        if (e != cudaSuccess) return cuda_check(e, "cudaGetSymbolAddress of the V-cycle scratch");
        g_scratch_address[dev] = p;
    }
    *ptr = g_scratch_address[dev];
    return MGX_OK;
}
} // namespace

int precond_mg_static(mgx_ctx* ctx, const mgx_precond_params* P, int dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks,
    cudaStream_t s)
{
    if (!P || !res || !out || nfunc < 0) return fail(MGX_BAD_ARG, "precond_mg: null argument");
    if (res == out) return fail(MGX_BAD_ARG, "precond_mg: res and out alias");
    if (P->lap_type < 0 || P->lap_type > 4) return fail(MGX_BAD_ARG, "lap_type %d", P->lap_type);
    const int L = P->maxlevels;
    if (L < 0 || L > 6) return fail(MGX_BAD_ARG, "maxlevels %d", L);
    const mgx_grid& g = ctx->grid;
    for (int l = 0; l < L; l++)
        for (int i = 0; i < 3; i++)
            if ((g.n[i] >> l) % 2)
                return fail(MGX_BAD_ARG, "grid dimension %d not divisible by 2^%d", i, L);
    if (masks && (masks->nlevels < L + 1 || masks->nfunc < nfunc))
        return fail(MGX_BAD_ARG, "masks cover %d levels / %d functions", masks->nlevels, masks->nfunc);
    const size_t es = dtype_size(dtype);

    VCycle V;
    V.ctx      = ctx;
    V.dtype    = dtype;
    V.lap_type = P->lap_type;
    V.L        = L;
    V.masks    = masks;
    V.s        = s;
    for (int l = 0; l <= L; l++)
    {
        V.lev.push_back(make_level(g, l));
        V.jf.push_back(jacobi_factor(l == 0 ? P->lap_type : 1, V.lev[l].h));
    }
    // level-0 arrays are addressed with the caller's leading dimension ld
    size_t per_func = 2 * ld;
    for (int l = 1; l <= L; l++)
        per_func += 4 * V.lev[l].npts();
    per_func *= es;
    const size_t avail = STATIC_VCYCLE_SCRATCH_BYTES - STATIC_VCYCLE_STATUS_BYTES;
    if (per_func > avail)
        return fail(MGX_BAD_ARG,
            "one function needs %zu bytes of V-cycle scratch; the static scratch holds %zu",
            per_func, avail);
    if (nfunc == 0) return MGX_OK;
    size_t chunk = avail / per_func;
    if (P->chunk > 0) chunk = std::min(chunk, (size_t)P->chunk);
    chunk = std::min(chunk, (size_t)65535);
    chunk = std::min(chunk, (size_t)nfunc);

    void* scratch = nullptr;
    MGX_TRY(static_scratch_address(&scratch));
    // the status word starts at zero; every other scratch byte is written
    // before it is read within a call
    V.err = (int*)scratch;
    MGX_TRY(cuda_check(cudaMemsetAsync(scratch, 0, STATIC_VCYCLE_STATUS_BYTES, s), "status reset"));

    for (int f0 = 0; f0 < nfunc; f0 += (int)chunk)
    {
        const int nf = (int)std::min(chunk, (size_t)(nfunc - f0));
        V.nf = nf;
        V.f0 = f0;
        V.v0.assign(L + 1, nullptr);
        V.v1.assign(L + 1, nullptr);
        V.w.assign(L + 1, nullptr);
        V.f.assign(L + 1, nullptr);
        V.ld.assign(L + 1, 0);
        char* base = (char*)scratch + STATIC_VCYCLE_STATUS_BYTES;
        V.ld[0]    = ld;
        V.v0[0]    = (char*)out + (size_t)f0 * ld * es;
        V.f[0]     = (void*)((const char*)res + (size_t)f0 * ld * es);
        V.v1[0]    = base;
        base += (size_t)nf * ld * es;
        V.w[0] = base;
        base += (size_t)nf * ld * es;
        for (int l = 1; l <= L; l++)
        {
            const size_t pl = V.lev[l].npts();
            V.ld[l]         = pl;
            V.v0[l]         = base;
            base += (size_t)nf * pl * es;
            V.v1[l] = base;
            base += (size_t)nf * pl * es;
            V.w[l] = base;
            base += (size_t)nf * pl * es;
            V.f[l] = base;
            base += (size_t)nf * pl * es;
        }
        V.gamma         = P->gamma;
        V.pending_scale = true;
        const int c = V.mg(0);
        if (c < 0) return -(c + 1);
        if (c != 0) return fail(MGX_UNSUPPORTED, "V-cycle ended in the work buffer");
    }
    int status = 0;
    MGX_TRY(cuda_check(cudaMemcpyAsync(&status, scratch, sizeof(int), cudaMemcpyDeviceToHost, s),
        "status read"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "static V-cycle sync"));
    if (status != 0) return fail(MGX_TIMEOUT, "a bounded wait in the V-cycle gave up");
    return MGX_OK;
}

} // namespace mgx

extern "C" int mgx_precond_mg_static(mgx_ctx* ctx, const mgx_precond_params* p,
    mgx_dtype dtype, const void* res, size_t ld, void* out, int nfunc,
    const mgx_masks* masks, void* stream)
{
    using namespace mgx;
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    if (dtype != MGX_F64 && dtype != MGX_F32) return fail(MGX_BAD_ARG, "dtype %d invalid", (int)dtype);
    const size_t np = (size_t)ctx->grid.n[0] * ctx->grid.n[1] * ctx->grid.n[2];
    if (nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, np);
    if (masks && masks->dtype != dtype)
        return fail(MGX_BAD_ARG, "mask value type differs from the orbital type");
    return precond_mg_static(ctx, p, dtype, res, nfunc > 1 ? ld : (ld ? ld : np), out, nfunc,
        masks, (cudaStream_t)stream);
}
