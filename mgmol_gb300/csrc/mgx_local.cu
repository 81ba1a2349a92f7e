// Localized orbitals: box-local storage and one persistent fused kernel for
// the fine-level work of an orbital iteration on uneven mask boxes.
//
// Orbital j lives on the level-0 box of its localization mask (origin o_j,
// extents e_j, the box form of mgx_masks: point b of the box is grid point
// (o_j + b) mod n, z fastest), packed one box after another.  Outside its
// box an orbital is zero, which is what the masks make of it on the whole
// grid: the mask values are zero there (src/GridMask.cc:120-264).
//
// The fused step, per orbital (FP32, the reference's operators):
//   r  = Mc (B(phi - V psi) + Delta_M psi)       = Mc (B phi - H psi)
//   u0 = gamma r
//   u1 = M(u0 - jf (A u0 - r))                    first Jacobi sweep
//   u2 = M(u1 - jf (A u1 - r)),  w = M(A u1 - r)  second sweep
// with H psi = -Delta_M psi + B(V psi) (Hamiltonian::applyLocal,
// src/Hamiltonian.cc:106-132), phi the column of Psi Theta (the residual of
// MGmol::computeResidualUsingHPhi, src/MGmol.cc:1227-1290, with the
// correction mask Mc of LocGridOrbitals::applyCorrMask), A = -Delta_M and
// the orbital mask M (GridMaskMax) of the V-cycle's fine-level pre-sweeps
// (Preconditioning<T>::mg, src/Preconditioning.cc:170-178).  u2 and w are
// what the V-cycle restricts next.
//
// One CTA takes (orbital, column) items from a work list until it is empty
// (largest boxes first); a column is a TY x TZ window of the box marched
// along x, each stage keeping three planes in shared memory, so the
// orbital block is read once (plus the y / z halo) and u2, w written once.
// The column shape and the CTAs per SM are chosen by timing
// (mgx_local_tune); the launch can be a CUDA graph.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{
namespace loc
{
constexpr int THREADS = 256;
constexpr int HALO    = 3;

struct StepParams
{
    const float* psi;
    const float* phi;
    const float* V; // FP32 potential on the whole grid
    float* u;
    float* w;
    const int* box;       // 6 per orbital: origin, extents
    const size_t* off;    // packed offset of each orbital
    const float* mvals;   // orbital mask values, box-local
    const size_t* moff;
    const float* cvals;   // correction mask values, box-local
    const size_t* coff;
    const int4* items;    // (orbital, 0, column origin y, z)
    int nitems;
    int* counter;
    int n[3];
    float c0, cx, cy, cz, cxy, cyz, cxz; // -Delta_M
    float gamma, jf;
};

__device__ __forceinline__ int wrapi(int i, int n)
{
    i %= n;
    return i < 0 ? i + n : i;
}

__device__ __forceinline__ float clampm(float v, float m)
{
    if (v > m) return m;
    if (v < -m) return -m;
    return v;
}

/* -Delta_M at index i of plane C, with the x neighbours in planes M and P
 * (plane stride sy along y, 1 along z) */
__device__ __forceinline__ float lap_m(const float* M, const float* C, const float* Pn, int i,
    int sy, const StepParams& P)
{
    const float faces = P.cx * (M[i] + Pn[i]) + P.cy * (C[i - sy] + C[i + sy])
        + P.cz * (C[i - 1] + C[i + 1]);
    const float exy = M[i - sy] + M[i + sy] + Pn[i - sy] + Pn[i + sy];
    const float eyz = C[i - sy - 1] + C[i - sy + 1] + C[i + sy - 1] + C[i + sy + 1];
    const float exz = M[i - 1] + M[i + 1] + Pn[i - 1] + Pn[i + 1];
    return P.c0 * C[i] + faces + P.cxy * exy + P.cyz * eyz + P.cxz * exz;
}

/* B = 1/2 + (1/12) sum of the six faces (FDkernelRHS_4th_Mehr1) */
__device__ __forceinline__ float rhs_b(const float* M, const float* C, const float* Pn, int i,
    int sy)
{
    const float s = (M[i] + Pn[i]) + (C[i - sy] + C[i + sy]) + (C[i - 1] + C[i + 1]);
    return 0.5f * C[i] + (1.f / 12.f) * s;
}

/* values at z - 1, z, z + 1, z + 2 of a plane column, i the (odd) index of
 * z: two 8-byte loads */
struct Col4
{
    float a, b, c, d;
};
__device__ __forceinline__ Col4 col4(const float* A, int i)
{
    const float2 lo = *reinterpret_cast<const float2*>(A + i - 1);
    const float2 hi = *reinterpret_cast<const float2*>(A + i + 1);
    return { lo.x, lo.y, hi.x, hi.y };
}

/* lap_m at the z pair (i, i + 1), i odd; the same operation order as lap_m */
__device__ __forceinline__ void lap_m2(const float* M, const float* C, const float* Pn, int i,
    int sy, const StepParams& P, float& o0, float& o1)
{
    const Col4 c = col4(C, i), m = col4(M, i), p = col4(Pn, i);
    const Col4 ym = col4(C, i - sy), yp = col4(C, i + sy);
    const Col4 mym = col4(M, i - sy), myp = col4(M, i + sy);
    const Col4 pym = col4(Pn, i - sy), pyp = col4(Pn, i + sy);
    {
        const float faces = P.cx * (m.b + p.b) + P.cy * (ym.b + yp.b) + P.cz * (c.a + c.c);
        const float exy   = mym.b + myp.b + pym.b + pyp.b;
        const float eyz   = ym.a + ym.c + yp.a + yp.c;
        const float exz   = m.a + m.c + p.a + p.c;
        o0 = P.c0 * c.b + faces + P.cxy * exy + P.cyz * eyz + P.cxz * exz;
    }
    {
        const float faces = P.cx * (m.c + p.c) + P.cy * (ym.c + yp.c) + P.cz * (c.b + c.d);
        const float exy   = mym.c + myp.c + pym.c + pyp.c;
        const float eyz   = ym.b + ym.d + yp.b + yp.d;
        const float exz   = m.b + m.d + p.b + p.d;
        o1 = P.c0 * c.c + faces + P.cxy * exy + P.cyz * eyz + P.cxz * exz;
    }
}

/* rhs_b at the z pair (i, i + 1), i odd; the same operation order */
__device__ __forceinline__ void rhs_b2(const float* M, const float* C, const float* Pn, int i,
    int sy, float& o0, float& o1)
{
    const Col4 c = col4(C, i);
    const float2 m  = *reinterpret_cast<const float2*>(M + i - 1);
    const float2 m2 = *reinterpret_cast<const float2*>(M + i + 1);
    const float2 p  = *reinterpret_cast<const float2*>(Pn + i - 1);
    const float2 p2 = *reinterpret_cast<const float2*>(Pn + i + 1);
    const Col4 ym = col4(C, i - sy), yp = col4(C, i + sy);
    const float s0 = (m.y + p.y) + (ym.b + yp.b) + (c.a + c.c);
    const float s1 = (m2.x + p2.x) + (ym.c + yp.c) + (c.b + c.d);
    o0 = 0.5f * c.b + (1.f / 12.f) * s0;
    o1 = 0.5f * c.c + (1.f / 12.f) * s1;
}

/* q / d for 0 <= q < 4096 and 1 <= d <= 64 with inv = 1/d rounded to FP32:
 * (q + 1/2) / d lies at least 1/(2d) from an integer, far more than the
 * 2^-23 relative error of the product, so the truncation is exact */
__device__ __forceinline__ int divq(int q, float inv)
{
    return __float2int_rz(((float)q + 0.5f) * inv);
}

/* one periodic coordinate of a box point: b in [-3, e + 3) with e + 6 <= n */
__device__ __forceinline__ int wrap1(int g, int n)
{
    return g < 0 ? g + n : (g >= n ? g - n : g);
}

/* A CTA owns a ty x tz column of an orbital's box and marches along x,
 * PPS planes per step.  The column is fitted to the box: the box's y
 * extent is cut into ceil(e1 / TY) equal columns, its z extent into
 * ceil(e2 / TZ) (tz rounded up to even), so that a box a little wider than
 * TY or TZ does not pay for a second, mostly empty column; TY x TZ bounds
 * the shared-memory planes.  Plane regions shrink by one point per stage
 * in y and z: stage 0 (psi and phi - V psi) on (ty + 6) x (tz + 6), stage 1
 * (r) on (ty + 4) x (tz + 4), stage 2 (u1) on (ty + 2) x (tz + 2), stage 3
 * (u, w) on ty x tz.  Stage k makes planes PPS t + j - 3 - k (j < PPS,
 * box-local x) at step t, within [k - 3, e0 - 1 + 3 - k]; a plane needs
 * the planes p - 1 .. p + 1 of the stage before, made at this step or the
 * one before, so each stage keeps a ring of PPS + 2 planes.  Three
 * barriers per step. */
template <int TY, int TZ, int PPS> struct Cols
{
    static constexpr int RING = PPS + 2;
    static constexpr int Y3 = TY + 6, Z3 = TZ + 6, N3 = Y3 * Z3;
    static constexpr int Y2 = TY + 4, Z2 = TZ + 4, N2 = Y2 * Z2;
    static constexpr int Y1 = TY + 2, Z1 = TZ + 2, N1 = Y1 * Z1;
    static constexpr int N0 = TY * TZ;
    static constexpr size_t SMEM = (size_t)(RING * (2 * N3 + N2 + N1)) * sizeof(float);
    // ring slot of plane p >= -3
    static __device__ __forceinline__ int slot(int p) { return (p + 3 * RING) % RING; }
    // resident CTAs per SM the shared memory allows (the register cap of
    // the launch bounds follows it)
    static constexpr int MINB = (int)(227 * 1024 / (SMEM + 1024)) < 4
                                    ? (int)(227 * 1024 / (SMEM + 1024))
                                    : 4;
};

template <int TY, int TZ, int PPS>
__global__ void __launch_bounds__(THREADS, Cols<TY, TZ, PPS>::MINB) local_step_kernel(StepParams P)
{
    using C = Cols<TY, TZ, PPS>;
    extern __shared__ __align__(16) float sm[];
    float* s_psi = sm;                      // RING x N3
    float* s_d   = s_psi + C::RING * C::N3; // RING x N3: phi - V psi
    float* s_r   = s_d + C::RING * C::N3;   // RING x N2
    float* s_u   = s_r + C::RING * C::N2;   // RING x N1
    __shared__ int s_item;
    const int tid = threadIdx.x;
    for (;;)
    {
        __syncthreads();
        if (tid == 0) s_item = atomicAdd(P.counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= P.nitems) break;
        const int4 W = P.items[it]; // (orbital, ty | tz << 16, y0, z0)
        const int f  = W.x;
        const int ty = W.y & 0xffff, tz = W.y >> 16;
        // the column's plane regions of each stage (row pitch z_k, pairs
        // per row p_k) and the reciprocals of the divisors
        const int z3 = tz + 6, n3 = (ty + 6) * z3;
        const int z2 = tz + 4, n2 = (ty + 4) * z2, p2 = z2 / 2;
        const int z1 = tz + 2, n1 = (ty + 2) * z1, p1 = z1 / 2;
        const int n0 = ty * tz, p0 = tz / 2;
        const float i3 = 1.f / (float)z3, ip2 = 1.f / (float)p2, ip1 = 1.f / (float)p1,
                    ip0 = 1.f / (float)p0;
        const int* b = P.box + 6 * f;
        const int o0 = b[0], o1 = b[1], o2 = b[2], e0 = b[3], e1 = b[4], e2 = b[5];
        const int y0 = W.z, z0 = W.w;
        const size_t ex = (size_t)e1 * e2;
        const float* psi = P.psi + P.off[f];
        const float* phi = P.phi + P.off[f];
        const float* mo  = P.mvals + P.moff[f];
        const float* mc  = P.cvals + P.coff[f];
        // stage 0 inputs of the next PPS planes, loaded into registers one
        // march step ahead so that their latency overlaps stages 1 to 3
        constexpr int NQ = (C::N3 + THREADS - 1) / THREADS;
        float rps[PPS][NQ], rph[PPS][NQ], rv[PPS][NQ];
        auto load_plane = [&](int p, int j) {
            const bool in = (p >= 0 && p < e0);
            const int gx  = wrap1(o0 + (in ? p : 0), P.n[0]);
#pragma unroll
            for (int k = 0; k < NQ; k++)
            {
                const int q  = tid + k * THREADS;
                const int qy = divq(q, i3), qz = q - qy * z3;
                const int by = y0 + qy - 3, bz = z0 + qz - 3;
                float ps = 0.f, ph = 0.f, v = 0.f;
                if (q < n3 && in && by >= 0 && by < e1 && bz >= 0 && bz < e2)
                {
                    const size_t li = (size_t)p * ex + (size_t)by * e2 + bz;
                    ps              = psi[li];
                    ph              = phi[li];
                    const int gy = wrap1(o1 + by, P.n[1]), gz = wrap1(o2 + bz, P.n[2]);
                    v = P.V[((size_t)gx * P.n[1] + gy) * P.n[2] + gz];
                }
                rps[j][k] = ps;
                rph[j][k] = ph;
                rv[j][k]  = v;
            }
        };
#pragma unroll
        for (int j = 0; j < PPS; j++)
            load_plane(j - 3, j);
        for (int t = 0; PPS * t - 6 < e0; t++)
        {
            // stage 0: psi and phi - V psi, from the registers; then the
            // loads of the planes of the next step
#pragma unroll
            for (int j = 0; j < PPS; j++)
            {
                const int p = PPS * t + j - 3;
                if (p <= e0 + 2)
                {
                    float* dp = s_psi + C::slot(p) * C::N3;
                    float* dd = s_d + C::slot(p) * C::N3;
#pragma unroll
                    for (int k = 0; k < NQ; k++)
                    {
                        const int q = tid + k * THREADS;
                        if (q < n3)
                        {
                            dp[q] = rps[j][k];
                            dd[q] = rph[j][k] - rv[j][k] * rps[j][k];
                        }
                    }
                }
                load_plane(p + PPS, j);
            }
            __syncthreads();
            // stage 1: r = Mc (B(phi - V psi) + Delta_M psi), z pairs
#pragma unroll
            for (int j = 0; j < PPS; j++)
            {
                const int p = PPS * t + j - 4;
                if (p < -2 || p > e0 + 1) continue;
                const float* M  = s_psi + C::slot(p - 1) * C::N3;
                const float* X  = s_psi + C::slot(p) * C::N3;
                const float* N  = s_psi + C::slot(p + 1) * C::N3;
                const float* dM = s_d + C::slot(p - 1) * C::N3;
                const float* dX = s_d + C::slot(p) * C::N3;
                const float* dN = s_d + C::slot(p + 1) * C::N3;
                float* out      = s_r + C::slot(p) * C::N2;
                const bool in   = (p >= 0 && p < e0);
                for (int q = tid; q < n2 / 2; q += THREADS)
                {
                    const int qy = divq(q, ip2), qz = 2 * (q - qy * p2);
                    const int by = y0 + qy - 2, bz = z0 + qz - 2;
                    float m0 = 0.f, m1 = 0.f;
                    if (in && by >= 0 && by < e1)
                    {
                        const float* mrow = mc + (size_t)p * ex + (size_t)by * e2;
                        if (bz >= 0 && bz < e2) m0 = mrow[bz];
                        if (bz + 1 >= 0 && bz + 1 < e2) m1 = mrow[bz + 1];
                    }
                    float r0 = 0.f, r1 = 0.f;
                    if (m0 != 0.f || m1 != 0.f)
                    {
                        const int i = (qy + 1) * z3 + qz + 1;
                        float b0, b1, l0, l1;
                        rhs_b2(dM, dX, dN, i, z3, b0, b1);
                        lap_m2(M, X, N, i, z3, P, l0, l1);
                        r0 = m0 * (b0 - l0);
                        r1 = m1 * (b1 - l1);
                    }
                    *reinterpret_cast<float2*>(out + qy * z2 + qz) = make_float2(r0, r1);
                }
            }
            __syncthreads();
            // stage 2: the first sweep u1, from u0 = gamma r, z pairs
#pragma unroll
            for (int j = 0; j < PPS; j++)
            {
                const int p = PPS * t + j - 5;
                if (p < -1 || p > e0) continue;
                const float* M = s_r + C::slot(p - 1) * C::N2;
                const float* X = s_r + C::slot(p) * C::N2;
                const float* N = s_r + C::slot(p + 1) * C::N2;
                float* out     = s_u + C::slot(p) * C::N1;
                const bool in  = (p >= 0 && p < e0);
                for (int q = tid; q < n1 / 2; q += THREADS)
                {
                    const int qy = divq(q, ip1), qz = 2 * (q - qy * p1);
                    const int by = y0 + qy - 1, bz = z0 + qz - 1;
                    float m0 = 0.f, m1 = 0.f;
                    if (in && by >= 0 && by < e1)
                    {
                        const float* mrow = mo + (size_t)p * ex + (size_t)by * e2;
                        if (bz >= 0 && bz < e2) m0 = mrow[bz];
                        if (bz + 1 >= 0 && bz + 1 < e2) m1 = mrow[bz + 1];
                    }
                    const int i = (qy + 1) * z2 + qz + 1;
                    // outside the orbital's mask the sweep clamps to zero
                    // whatever the stencil gives: skip the stencil there
                    float l0 = 0.f, l1 = 0.f;
                    if (m0 != 0.f || m1 != 0.f) lap_m2(M, X, N, i, z2, P, l0, l1);
                    const float2 r  = make_float2(X[i], X[i + 1]);
                    const float w0  = P.gamma * l0 - r.x;
                    const float w1  = P.gamma * l1 - r.y;
                    *reinterpret_cast<float2*>(out + qy * z1 + qz)
                        = make_float2(clampm(P.gamma * r.x - P.jf * w0, m0),
                            clampm(P.gamma * r.y - P.jf * w1, m1));
                }
            }
            __syncthreads();
            // stage 3: the second sweep, stored inside the box, z pairs
#pragma unroll
            for (int j = 0; j < PPS; j++)
            {
                const int p = PPS * t + j - 6;
                if (p < 0 || p >= e0) continue;
                const float* M = s_u + C::slot(p - 1) * C::N1;
                const float* X = s_u + C::slot(p) * C::N1;
                const float* N = s_u + C::slot(p + 1) * C::N1;
                const float* R = s_r + C::slot(p) * C::N2;
                for (int q = tid; q < n0 / 2; q += THREADS)
                {
                    const int qy = divq(q, ip0), qz = 2 * (q - qy * p0);
                    const int by = y0 + qy, bz = z0 + qz;
                    if (by >= e1 || bz >= e2) continue;
                    const size_t li = (size_t)p * ex + (size_t)by * e2 + bz;
                    const int i     = (qy + 1) * z1 + qz + 1;
                    const float m0  = mo[li];
                    const float m1  = (bz + 1 < e2) ? mo[li + 1] : 0.f;
                    // the stencil only where the mask keeps something
                    float l0 = 0.f, l1 = 0.f;
                    if (m0 != 0.f || m1 != 0.f) lap_m2(M, X, N, i, z1, P, l0, l1);
                    const int ir    = (qy + 2) * z2 + qz + 2;
                    const float w0  = l0 - R[ir];
                    P.u[P.off[f] + li] = clampm(X[i] - P.jf * w0, m0);
                    P.w[P.off[f] + li] = clampm(w0, m0);
                    if (bz + 1 < e2)
                    {
                        const float w1 = l1 - R[ir + 1];
                        P.u[P.off[f] + li + 1] = clampm(X[i + 1] - P.jf * w1, m1);
                        P.w[P.off[f] + li + 1] = clampm(w1, m1);
                    }
                }
            }
        }
    }
}

/* packed box-local <-> whole-grid copies (blockIdx.y = orbital) */
__global__ void __launch_bounds__(256) gather_kernel(const float* __restrict__ full, size_t ld,
    float* __restrict__ packed, const int* __restrict__ box, const size_t* __restrict__ off,
    int n0, int n1, int n2)
{
    const int f  = blockIdx.y;
    const int* b = box + 6 * f;
    const size_t vol = (size_t)b[3] * b[4] * b[5];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < vol;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const int bz = (int)(i % b[5]), by = (int)((i / b[5]) % b[4]), bx = (int)(i / ((size_t)b[5] * b[4]));
        const int gx = wrapi(b[0] + bx, n0), gy = wrapi(b[1] + by, n1), gz = wrapi(b[2] + bz, n2);
        packed[off[f] + i] = full[(size_t)f * ld + ((size_t)gx * n1 + gy) * n2 + gz];
    }
}

__global__ void __launch_bounds__(256) scatter_kernel(const float* __restrict__ packed,
    float* __restrict__ full, size_t ld, const int* __restrict__ box,
    const size_t* __restrict__ off, int n0, int n1, int n2)
{
    const int f  = blockIdx.y;
    const int* b = box + 6 * f;
    const size_t vol = (size_t)b[3] * b[4] * b[5];
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < vol;
         i += (size_t)gridDim.x * blockDim.x)
    {
        const int bz = (int)(i % b[5]), by = (int)((i / b[5]) % b[4]), bx = (int)(i / ((size_t)b[5] * b[4]));
        const int gx = wrapi(b[0] + bx, n0), gy = wrapi(b[1] + by, n1), gz = wrapi(b[2] + bz, n2);
        full[(size_t)f * ld + ((size_t)gx * n1 + gy) * n2 + gz] = packed[off[f] + i];
    }
}

/* the kernel variants the tuner chooses from: largest column TY x TZ and
 * planes per march step */
struct Shape
{
    int ty, tz, pps;
};
constexpr int NSHAPE           = 6;
constexpr Shape SHAPES[NSHAPE] = { { 24, 32, 1 }, { 16, 32, 1 }, { 32, 32, 1 }, { 24, 32, 2 },
    { 16, 32, 2 }, { 32, 32, 2 } };

/* kernel and dynamic shared memory of a variant */
template <int TY, int TZ, int PPS> struct Variant
{
    static constexpr auto kernel() { return &local_step_kernel<TY, TZ, PPS>; }
    static constexpr size_t smem = Cols<TY, TZ, PPS>::SMEM;
};

template <int TY, int TZ, int PPS> int set_attr()
{
    static bool done = false;
    if (!done)
    {
        MGX_TRY(cuda_check(cudaFuncSetAttribute(Variant<TY, TZ, PPS>::kernel(),
                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)Variant<TY, TZ, PPS>::smem),
            "local smem"));
        done = true;
    }
    return MGX_OK;
}

template <int TY, int TZ, int PPS> int occupancy()
{
    if (set_attr<TY, TZ, PPS>() != MGX_OK) return 1;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, Variant<TY, TZ, PPS>::kernel(),
            THREADS, Variant<TY, TZ, PPS>::smem)
        != cudaSuccess)
    {
        cudaGetLastError();
        return 1;
    }
    return std::max(n, 1);
}

/* resident CTAs per SM of variant s (also sets its shared-memory limit) */
int max_ctas_per_sm(int s)
{
    switch (s)
    {
        case 0: return occupancy<24, 32, 1>();
        case 1: return occupancy<16, 32, 1>();
        case 2: return occupancy<32, 32, 1>();
        case 3: return occupancy<24, 32, 2>();
        case 4: return occupancy<16, 32, 2>();
        default: return occupancy<32, 32, 2>();
    }
}

template <int TY, int TZ, int PPS> int launch_shape(const StepParams& P, int ctas, cudaStream_t s)
{
    Variant<TY, TZ, PPS>::kernel()<<<ctas, THREADS, Variant<TY, TZ, PPS>::smem, s>>>(P);
    MGX_LAUNCH_CHECK("local_step_kernel");
    return MGX_OK;
}

} // namespace loc
} // namespace mgx

struct mgx_local
{
    mgx_ctx* ctx       = nullptr;
    int nfunc          = 0;
    size_t total       = 0;
    std::vector<int> h_box;      // 6 per orbital
    std::vector<size_t> h_off;   // nfunc + 1
    mgx::DeviceBuffer box, off, counter;
    mgx::DeviceBuffer items[mgx::loc::NSHAPE];
    int nitems[mgx::loc::NSHAPE] = {};
    const mgx_masks* masks = nullptr;
    const mgx_masks* corr  = nullptr;
    // chosen configuration
    int shape = 1, ctas_per_sm = 2, use_graph = 1;
    // the captured step, valid for the arguments it was captured with
    cudaGraphExec_t exec = nullptr;
    cudaGraph_t graph    = nullptr;
    const void* key[5]   = { nullptr, nullptr, nullptr, nullptr, nullptr };
    double key_gamma     = 0.;
    int key_shape = -1, key_ctas = -1;
    ~mgx_local()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
    }
};

namespace mgx
{
namespace loc
{
int build_items(mgx_local* L, int s)
{
    const Shape S = SHAPES[s];
    std::vector<int4> it;
    std::vector<std::pair<size_t, int>> order; // largest box first
    for (int f = 0; f < L->nfunc; f++)
        order.push_back({ (size_t)L->h_box[6 * f + 3] * L->h_box[6 * f + 4] * L->h_box[6 * f + 5], f });
    std::stable_sort(order.begin(), order.end(),
        [](const std::pair<size_t, int>& a, const std::pair<size_t, int>& b) { return a.first > b.first; });
    for (const auto& pr : order)
    {
        const int f  = pr.second;
        const int* e = &L->h_box[6 * f + 3];
        // columns fitted to the box: equal cuts of each extent, at most
        // S.ty x S.tz, tz even (the kernel works on z pairs)
        const int ny = (e[1] + S.ty - 1) / S.ty, nz = (e[2] + S.tz - 1) / S.tz;
        const int ty = (e[1] + ny - 1) / ny;
        const int tz = (((e[2] + nz - 1) / nz) + 1) & ~1;
        for (int y = 0; y < e[1]; y += ty)
            for (int z = 0; z < e[2]; z += tz)
                it.push_back(make_int4(f, ty | (tz << 16), y, z));
    }
    L->nitems[s] = (int)it.size();
    MGX_TRY(L->items[s].ensure(std::max<size_t>(it.size(), 1) * sizeof(int4)));
    if (!it.empty())
        MGX_TRY(cuda_check(cudaMemcpy(L->items[s].ptr, it.data(), it.size() * sizeof(int4),
                               cudaMemcpyHostToDevice),
            "items upload"));
    return MGX_OK;
}

StepParams params(mgx_local* L, int s, const float* psi, const float* phi, const float* V,
    double gamma, float* u, float* w)
{
    StepParams P;
    P.psi   = psi;
    P.phi   = phi;
    P.V     = V;
    P.u     = u;
    P.w     = w;
    P.box   = (const int*)L->box.ptr;
    P.off   = (const size_t*)L->off.ptr;
    P.mvals = (const float*)L->masks->values[0].ptr;
    P.moff  = (const size_t*)L->masks->offset[0].ptr;
    P.cvals = (const float*)L->corr->values[0].ptr;
    P.coff  = (const size_t*)L->corr->offset[0].ptr;
    P.items   = (const int4*)L->items[s].ptr;
    P.nitems  = L->nitems[s];
    P.counter = (int*)L->counter.ptr;
    const mgx_grid& g = L->ctx->grid;
    for (int i = 0; i < 3; i++)
        P.n[i] = g.n[i];
    const Level L0        = make_level(g, 0);
    const StencilCoeffs c = stencil_coeffs(0, L0.h);
    P.c0    = (float)c.c0;
    P.cx    = (float)c.cx[0];
    P.cy    = (float)c.cy[0];
    P.cz    = (float)c.cz[0];
    P.cxy   = (float)c.cxy;
    P.cyz   = (float)c.cyz;
    P.cxz   = (float)c.cxz;
    P.gamma = (float)gamma;
    P.jf    = (float)jacobi_factor(0, L0.h);
    return P;
}

/* persistent grid of shape s: ctas_per_sm per SM, at most what is resident */
int grid_ctas(mgx_local* L, int s, int ctas_per_sm)
{
    return L->ctx->sm_count * std::max(1, std::min(ctas_per_sm, max_ctas_per_sm(s)));
}

int enqueue(mgx_local* L, int s, int ctas, const StepParams& P, cudaStream_t st)
{
    MGX_TRY(cuda_check(cudaMemsetAsync(L->counter.ptr, 0, sizeof(int), st), "counter reset"));
    switch (s)
    {
        case 0: return launch_shape<24, 32, 1>(P, ctas, st);
        case 1: return launch_shape<16, 32, 1>(P, ctas, st);
        case 2: return launch_shape<32, 32, 1>(P, ctas, st);
        case 3: return launch_shape<24, 32, 2>(P, ctas, st);
        case 4: return launch_shape<16, 32, 2>(P, ctas, st);
        default: return launch_shape<32, 32, 2>(P, ctas, st);
    }
}

int step(mgx_local* L, const float* psi, const float* phi, const float* V, double gamma, float* u,
    float* w, cudaStream_t st)
{
    const int s         = L->shape;
    const StepParams P  = params(L, s, psi, phi, V, gamma, u, w);
    const int ctas      = grid_ctas(L, s, L->ctas_per_sm);
    if (!L->use_graph) return enqueue(L, s, ctas, P, st);
    const void* key[5] = { psi, phi, V, u, w };
    bool same = L->exec && L->key_gamma == gamma && L->key_shape == s && L->key_ctas == L->ctas_per_sm;
    for (int i = 0; i < 5 && same; i++)
        same = (key[i] == L->key[i]);
    if (!same)
    {
        if (L->exec) cudaGraphExecDestroy(L->exec);
        if (L->graph) cudaGraphDestroy(L->graph);
        L->exec  = nullptr;
        L->graph = nullptr;
        // capture on a private stream (the caller's may be the legacy stream)
        cudaStream_t cs = nullptr;
        MGX_TRY(cuda_check(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "capture stream"));
        // (the kernel's attributes were set by grid_ctas, before the capture)
        int rc = cuda_check(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal), "begin capture");
        if (rc == MGX_OK)
        {
            const int e1 = enqueue(L, s, ctas, P, cs);
            cudaGraph_t g  = nullptr;
            const int e2   = cuda_check(cudaStreamEndCapture(cs, &g), "end capture");
            rc             = e1 != MGX_OK ? e1 : e2;
            if (rc == MGX_OK)
            {
                rc = cuda_check(cudaGraphInstantiate(&L->exec, g, 0), "graph instantiate");
                L->graph = g;
            }
            else if (g)
                cudaGraphDestroy(g);
        }
        cudaStreamDestroy(cs);
        MGX_TRY(rc);
        for (int i = 0; i < 5; i++)
            L->key[i] = key[i];
        L->key_gamma = gamma;
        L->key_shape = s;
        L->key_ctas  = L->ctas_per_sm;
    }
    count_launch();
    return cuda_check(cudaGraphLaunch(L->exec, st), "graph launch");
}

} // namespace loc
} // namespace mgx

using namespace mgx;

extern "C" {

int mgx_local_create(mgx_ctx* ctx, const mgx_masks* masks, const mgx_masks* corr,
    mgx_local** out)
{
    if (!ctx || !masks || !corr || !out) return fail(MGX_BAD_ARG, "NULL argument");
    if (masks->dtype != MGX_F32 || corr->dtype != MGX_F32)
        return fail(MGX_BAD_ARG, "localized orbitals need FP32 masks");
    if (masks->nfunc != corr->nfunc) return fail(MGX_BAD_ARG, "mask sets of different sizes");
    if (masks->kind != 0 || corr->kind != 1)
        return fail(MGX_BAD_ARG, "orbital masks must clamp (GridMaskMax), correction masks multiply");
    const mgx_grid& g = ctx->grid;
    for (int i = 0; i < 3; i++)
        if (masks->n[i] != g.n[i] || corr->n[i] != g.n[i])
            return fail(MGX_BAD_ARG, "masks of another grid");
    auto L   = std::make_unique<mgx_local>();
    L->ctx   = ctx;
    L->nfunc = masks->nfunc;
    L->masks = masks;
    L->corr  = corr;
    L->h_box.resize(6 * (size_t)L->nfunc);
    L->h_off.resize(L->nfunc + 1);
    size_t tot = 0;
    for (int f = 0; f < L->nfunc; f++)
    {
        if (masks->h_state[0][f] != 2 || corr->h_state[0][f] != 2)
            return fail(MGX_UNSUPPORTED, "orbital %d: mask without a box of values", f);
        for (int k = 0; k < 6; k++)
        {
            const int v = masks->h_box[0][6 * f + k];
            if (corr->h_box[0][6 * f + k] != v)
                return fail(MGX_UNSUPPORTED, "orbital %d: correction box differs from the mask box", f);
            L->h_box[6 * f + k] = v;
        }
        for (int k = 0; k < 3; k++)
            if (L->h_box[6 * f + 3 + k] + 2 * loc::HALO > g.n[k])
                return fail(MGX_UNSUPPORTED, "orbital %d: box wider than the grid less the halo", f);
        L->h_off[f] = tot;
        tot += (size_t)L->h_box[6 * f + 3] * L->h_box[6 * f + 4] * L->h_box[6 * f + 5];
    }
    L->h_off[L->nfunc] = tot;
    L->total           = tot;
    MGX_TRY(L->box.ensure(std::max<size_t>(L->h_box.size(), 1) * sizeof(int)));
    MGX_TRY(L->off.ensure(L->h_off.size() * sizeof(size_t)));
    MGX_TRY(L->counter.ensure(256));
    if (L->nfunc)
    {
        MGX_TRY(cuda_check(cudaMemcpy(L->box.ptr, L->h_box.data(), L->h_box.size() * sizeof(int),
                               cudaMemcpyHostToDevice),
            "box upload"));
        MGX_TRY(cuda_check(cudaMemcpy(L->off.ptr, L->h_off.data(), L->h_off.size() * sizeof(size_t),
                               cudaMemcpyHostToDevice),
            "offset upload"));
    }
    for (int s = 0; s < loc::NSHAPE; s++)
        MGX_TRY(loc::build_items(L.get(), s));
    *out = L.release();
    return MGX_OK;
}

int mgx_local_destroy(mgx_local* L)
{
    delete L;
    return MGX_OK;
}

int mgx_local_layout(const mgx_local* L, size_t* total, size_t* offsets, int* boxes)
{
    if (!L) return fail(MGX_BAD_ARG, "NULL argument");
    if (total) *total = L->total;
    if (offsets) std::memcpy(offsets, L->h_off.data(), L->h_off.size() * sizeof(size_t));
    if (boxes) std::memcpy(boxes, L->h_box.data(), L->h_box.size() * sizeof(int));
    return MGX_OK;
}

int mgx_local_gather(mgx_local* L, const float* full, size_t ld, float* packed, void* stream)
{
    if (!L || (L->nfunc && (!full || !packed))) return fail(MGX_BAD_ARG, "NULL argument");
    const mgx_grid& g = L->ctx->grid;
    const size_t np   = (size_t)g.n[0] * g.n[1] * g.n[2];
    if (L->nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, np);
    if (L->nfunc == 0) return MGX_OK;
    loc::gather_kernel<<<dim3(64, L->nfunc), 256, 0, (cudaStream_t)stream>>>(full, ld ? ld : np,
        packed, (const int*)L->box.ptr, (const size_t*)L->off.ptr, g.n[0], g.n[1], g.n[2]);
    MGX_LAUNCH_CHECK("gather_kernel");
    return MGX_OK;
}

int mgx_local_scatter(mgx_local* L, const float* packed, float* full, size_t ld, void* stream)
{
    if (!L || (L->nfunc && (!full || !packed))) return fail(MGX_BAD_ARG, "NULL argument");
    const mgx_grid& g = L->ctx->grid;
    const size_t np   = (size_t)g.n[0] * g.n[1] * g.n[2];
    if (L->nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "ld %zu < %zu points", ld, np);
    if (L->nfunc == 0) return MGX_OK;
    loc::scatter_kernel<<<dim3(64, L->nfunc), 256, 0, (cudaStream_t)stream>>>(packed, full,
        ld ? ld : np, (const int*)L->box.ptr, (const size_t*)L->off.ptr, g.n[0], g.n[1], g.n[2]);
    MGX_LAUNCH_CHECK("scatter_kernel");
    return MGX_OK;
}

int mgx_local_set_config(mgx_local* L, int shape, int ctas_per_sm, int use_graph)
{
    if (!L) return fail(MGX_BAD_ARG, "NULL argument");
    if (shape < 0 || shape >= loc::NSHAPE) return fail(MGX_BAD_ARG, "shape %d", shape);
    if (ctas_per_sm < 1 || ctas_per_sm > 8) return fail(MGX_BAD_ARG, "ctas_per_sm %d", ctas_per_sm);
    L->shape       = shape;
    L->ctas_per_sm = ctas_per_sm;
    L->use_graph   = use_graph ? 1 : 0;
    return MGX_OK;
}

int mgx_local_get_config(const mgx_local* L, int* shape, int* ctas_per_sm, int* use_graph)
{
    if (!L) return fail(MGX_BAD_ARG, "NULL argument");
    if (shape) *shape = L->shape;
    if (ctas_per_sm) *ctas_per_sm = L->ctas_per_sm;
    if (use_graph) *use_graph = L->use_graph;
    return MGX_OK;
}

int mgx_local_step(mgx_local* L, const float* psi, const float* phi, const float* V,
    double gamma, float* u, float* w, void* stream)
{
    if (!L) return fail(MGX_BAD_ARG, "NULL argument");
    if (L->total && (!psi || !phi || !V || !u || !w)) return fail(MGX_BAD_ARG, "NULL block");
    if (u == w || u == psi || u == phi || w == psi || w == phi)
        return fail(MGX_BAD_ARG, "outputs alias the inputs or each other");
    if (L->total == 0) return MGX_OK;
    return loc::step(L, psi, phi, V, gamma, u, w, (cudaStream_t)stream);
}

int mgx_local_tune(mgx_local* L, const float* psi, const float* phi, const float* V,
    double gamma, float* u, float* w, double* ms, int* ncand, void* stream)
{
    if (!L) return fail(MGX_BAD_ARG, "NULL argument");
    if (L->total == 0) return MGX_OK;
    if (!psi || !phi || !V || !u || !w) return fail(MGX_BAD_ARG, "NULL block");
    const cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    MGX_TRY(cuda_check(cudaEventCreate(&e0), "event"));
    MGX_TRY(cuda_check(cudaEventCreate(&e1), "event"));
    int best_s = L->shape, best_c = L->ctas_per_sm, k = 0;
    double best = 1e300;
    int rc = MGX_OK;
    for (int s = 0; s < loc::NSHAPE && rc == MGX_OK; s++)
    {
        const int cmax = loc::max_ctas_per_sm(s);
        for (int ci = 0; ci < 4 && rc == MGX_OK; ci++)
        {
            const int c = ci + 1; // 1 to 4 resident CTAs per SM
            double t = 1e300;
            if (c <= cmax)
            {
                const loc::StepParams P = loc::params(L, s, psi, phi, V, gamma, u, w);
                const int ctas          = loc::grid_ctas(L, s, c);
                rc = loc::enqueue(L, s, ctas, P, st); // warm-up
                if (rc == MGX_OK) rc = cuda_check(cudaEventRecord(e0, st), "event");
                for (int r = 0; r < 3 && rc == MGX_OK; r++)
                    rc = loc::enqueue(L, s, ctas, P, st);
                if (rc == MGX_OK) rc = cuda_check(cudaEventRecord(e1, st), "event");
                if (rc == MGX_OK) rc = cuda_check(cudaEventSynchronize(e1), "event");
                float f = 0.f;
                if (rc == MGX_OK) rc = cuda_check(cudaEventElapsedTime(&f, e0, e1), "event");
                t = f / 3.;
                if (t < best)
                {
                    best   = t;
                    best_s = s;
                    best_c = c;
                }
            }
            if (ms && ncand && k < *ncand) ms[k] = t < 1e299 ? t : -1.;
            k++;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    MGX_TRY(rc);
    if (ncand) *ncand = k;
    L->shape       = best_s;
    L->ctas_per_sm = best_c;
    return MGX_OK;
}

} // extern "C"
