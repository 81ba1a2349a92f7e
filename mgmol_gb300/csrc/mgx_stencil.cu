// Finite-difference stencils of MGmol's orbital hot path on sm_103a.
//
// Fused path (ghost-free blocks, periodic): a plane-marching engine.  Each
// CTA owns one function, a band of TY y-rows and a chunk of x-planes.  The
// tile of every plane (TY + 2R rows, whole z lines, the periodic y wrap
// split into at most two contiguous runs) is fetched with 1-D bulk copies
// (cp.async.bulk) into a ring of S shared-memory stages completed on
// mbarriers, so that S - 2R - 1 planes are in flight while one is computed.
// z neighbours wrap inside the staged line; x neighbours come from the other
// stages.  One template serves -Lap, the Hamiltonian (with B(V psi) or
// V psi), the Mehrstellen B operator and the Jacobi sweep of the V-cycle
// (residual, update, localization mask in the epilogue).
//
// Coefficients follow src/pb/FDkernels.cc (del2 2nd/4th/6th/8th and
// Mehrstellen) and src/pb/Laph*.h (diagonals and Jacobi factors).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{

int lap_radius(int lap_type)
{
    switch (lap_type)
    {
        case 0: return 1;
        case 1: return 1;
        case 2: return 2;
        case 3: return 3;
        case 4: return 4;
    }
    return -1;
}

StencilCoeffs stencil_coeffs(int lap_type, const double h[3])
{
    StencilCoeffs c = {};
    const double ih[3] = { 1. / (h[0] * h[0]), 1. / (h[1] * h[1]),
        1. / (h[2] * h[2]) };
    const double inv12 = 1. / 12.;
    c.radius           = lap_radius(lap_type);
    switch (lap_type)
    {
        case 0: // FDkernelDel2_4th_Mehr, src/pb/FDkernels.cc:453-463
        {
            c.c0    = 16. * inv12 * (ih[0] + ih[1] + ih[2]);
            c.cx[0] = -10. * inv12 * ih[0] + 0.125 * c.c0;
            c.cy[0] = -10. * inv12 * ih[1] + 0.125 * c.c0;
            c.cz[0] = -10. * inv12 * ih[2] + 0.125 * c.c0;
            c.cxy   = -inv12 * (ih[0] + ih[1]);
            c.cyz   = -inv12 * (ih[2] + ih[1]);
            c.cxz   = -inv12 * (ih[0] + ih[2]);
            break;
        }
        case 1: // FDkernelDel2_2nd, src/pb/FDkernels.cc:28-42
            c.cx[0] = -ih[0];
            c.cy[0] = -ih[1];
            c.cz[0] = -ih[2];
            c.c0    = -2. * (c.cx[0] + c.cy[0] + c.cz[0]);
            break;
        case 2: // FDkernelDel2_4th, src/pb/FDkernels.cc:86-104
        {
            const double w[2] = { -16., 1. };
            double s = 0.;
            for (int k = 0; k < 2; k++)
            {
                c.cx[k] = w[k] * (inv12 * ih[0]);
                c.cy[k] = w[k] * (inv12 * ih[1]);
                c.cz[k] = w[k] * (inv12 * ih[2]);
            }
            s    = c.cx[0] + c.cx[1] + c.cy[0] + c.cy[1] + c.cz[0] + c.cz[1];
            c.c0 = -2. * s;
            break;
        }
        case 3: // FDkernelDel2_6th, src/pb/FDkernels.cc:261-281
        {
            const double w[3] = { -270., 27., -2. };
            for (int k = 0; k < 3; k++)
            {
                c.cx[k] = w[k] * ((1. / 180.) * ih[0]);
                c.cy[k] = w[k] * ((1. / 180.) * ih[1]);
                c.cz[k] = w[k] * ((1. / 180.) * ih[2]);
            }
            c.c0 = -2.
                   * (c.cx[0] + c.cx[1] + c.cx[2] + c.cy[0] + c.cy[1] + c.cy[2]
                       + c.cz[0] + c.cz[1] + c.cz[2]);
            break;
        }
        case 4: // FDkernelDel2_8th, src/pb/FDkernels.cc:350-374
        {
            const double w[4] = { -8064., 1008., -128., 9. };
            for (int k = 0; k < 4; k++)
            {
                c.cx[k] = w[k] * ((1. / 5040.) * ih[0]);
                c.cy[k] = w[k] * ((1. / 5040.) * ih[1]);
                c.cz[k] = w[k] * ((1. / 5040.) * ih[2]);
            }
            c.c0 = -2.
                   * (c.cx[0] + c.cx[1] + c.cx[2] + c.cx[3] + c.cy[0] + c.cy[1]
                       + c.cy[2] + c.cy[3] + c.cz[0] + c.cz[1] + c.cz[2]
                       + c.cz[3]);
            break;
        }
    }
    return c;
}

double jacobi_factor(int lap_type, const double h[3])
{
    const double s = 1. / (h[0] * h[0]) + 1. / (h[1] * h[1]) + 1. / (h[2] * h[2]);
    switch (lap_type)
    {
        case 0: return 1. / ((4. / 3.) * s);                   // Laph4M.h:29-31,80
        case 1: return 6. * (1. / (2. * s)) / 7.;              // Laph2.h:32-34,95
        case 2: return (1. / (2.5 * s)) / 1.5;                 // Laph4.h:35,106
        case 3: return (1. / ((49. / 18.) * s)) / 1.5;         // Laph6.h:40,101
        case 4: return (1. / ((1435. / 504.) * s)) / 1.5;      // Laph8.h:40-42,100
    }
    return 0.;
}

/* ------------------------------------------------------------------ */
/* device helpers                                                       */
/* ------------------------------------------------------------------ */
template <typename T>
struct DevCoef
{
    T c0;
    T cx[4], cy[4], cz[4];
    T cxy, cyz, cxz;
    T jf;
};

template <typename T>
DevCoef<T> to_dev(const StencilCoeffs& c, double jf)
{
    DevCoef<T> d;
    d.c0 = (T)c.c0;
    for (int k = 0; k < 4; k++)
    {
        d.cx[k] = (T)c.cx[k];
        d.cy[k] = (T)c.cy[k];
        d.cz[k] = (T)c.cz[k];
    }
    d.cxy = (T)c.cxy;
    d.cyz = (T)c.cyz;
    d.cxz = (T)c.cxz;
    d.jf  = (T)jf;
    return d;
}

/* Operations rounded once each, that the compiler may neither fuse nor
 * split: the stencil kernels that must give the same bits as one another
 * (single and paired sweeps) form every sum and product of a point with
 * these, since whether a plain a * b + c becomes one FMA depends on the
 * code around it. */
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

__device__ __forceinline__ int wrap(int i, int n)
{
    return i < 0 ? i + n : (i >= n ? i - n : i);
}

/* localization mask of one function at one level (box representation) */
template <typename T>
__device__ __forceinline__ T apply_mask(const MaskDev& m, int f, int x, int y,
    int z, T v)
{
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

/* Per-point operator evaluation shared by the staged and direct kernels.
 * `at(dx, dy, dz)` returns u at the offset; `vat` returns V. */
template <typename T, int LAP, int R, typename UA>
__device__ __forceinline__ T eval_lap(const DevCoef<T>& c, UA at)
{
    if (LAP == 0)
    {
        const T u0 = at(0, 0, 0);
        T r        = c.c0 * u0;
        r += c.cz[0] * (at(0, 0, -1) + at(0, 0, 1));
        r += c.cy[0] * (at(0, -1, 0) + at(0, 1, 0));
        r += c.cx[0] * (at(-1, 0, 0) + at(1, 0, 0));
        r += c.cxz * (at(-1, 0, -1) + at(-1, 0, 1) + at(1, 0, -1) + at(1, 0, 1));
        r += c.cyz * (at(0, -1, -1) + at(0, -1, 1) + at(0, 1, -1) + at(0, 1, 1));
        r += c.cxy * (at(-1, -1, 0) + at(1, -1, 0) + at(-1, 1, 0) + at(1, 1, 0));
        return r;
    }
    T r = c.c0 * at(0, 0, 0);
#pragma unroll
    for (int k = 1; k <= R; k++)
    {
        r += c.cx[k - 1] * (at(-k, 0, 0) + at(k, 0, 0));
        r += c.cy[k - 1] * (at(0, -k, 0) + at(0, k, 0));
        r += c.cz[k - 1] * (at(0, 0, -k) + at(0, 0, k));
    }
    return r;
}

/* B w = 1/2 w + 1/12 (sum of the 6 face neighbours), FDkernelRHS_4th_Mehr1 */
template <typename T, typename WA>
__device__ __forceinline__ T eval_rhs(WA w)
{
    const T c0 = (T)0.5, c1 = (T)(1. / 12.);
    return c0 * w(0, 0, 0)
           + c1 * (w(-1, 0, 0) + w(1, 0, 0) + w(0, -1, 0) + w(0, 1, 0)
                   + w(0, 0, -1) + w(0, 0, 1));
}

template <typename T, typename TV, int LAP, int OP, int R>
struct PointOp
{
    /* returns the value written to `out`; writes *wres for OP_JACOBI */
    template <typename UA, typename VA>
    __device__ __forceinline__ static T apply(const PlaneParams& p,
        const DevCoef<T>& c, UA at, VA vat, int f, size_t idx, T* wres)
    {
        if (OP == OP_RHS)
        {
            return eval_rhs<T>(at);
        }
        if (OP == OP_RHS_SUB)
            return eval_rhs<T>(at) - reinterpret_cast<const T*>(p.f)[(size_t)f * p.ldf + idx];
        const T lap = eval_lap<T, LAP, R>(c, at);
        if (OP == OP_LAP) return lap;
        if (OP == OP_HPSI_B)
        {
            auto w = [&](int dx, int dy, int dz) -> T {
                return (T)((TV)at(dx, dy, dz) * vat(dx, dy, dz));
            };
            // reference order: B(V psi) first, then += -Lap psi
            return eval_rhs<T>(w) + lap;
        }
        if (OP == OP_HPSI_V)
        {
            return lap + (T)((TV)at(0, 0, 0) * vat(0, 0, 0));
        }
        // OP_JACOBI: w = A v - f ; v -= jf w
        const T fv = reinterpret_cast<const T*>(p.f)[(size_t)f * p.ldf + idx];
        const T w  = lap - fv;
        *wres      = w;
        return at(0, 0, 0) - c.jf * w;
    }
};

/* ------------------------------------------------------------------ */
/* staged, register-pipelined plane kernel                              */
/* ------------------------------------------------------------------ */
// Each thread owns up to NP points (y, z) of the CTA's y-band and marches
// with them through the x-planes of its chunk.  Planes arrive in a ring of
// S shared-memory stages (1-D bulk copies of TY + 2RR whole z lines).
//  - Radius-1 "Mehrstellen-like" operators (LAP 0 and the B operator)
//    fold plane p, as soon as it lands, into a(p) (the part of the output at
//    p that lives in plane p) and b(p) (what plane p adds to its two x
//    neighbours): out(x) = a(x) + b(x-1) + b(x+1).  One plane is read per
//    point and step (9 values, plus 5 of V for B(V psi)).
//  - Axis stencils of radius R keep the centre column u(x-R..x+R) in a
//    register queue and read the y/z neighbours of plane x from the stage
//    still resident when plane x+R lands (4R + 1 values per point).
template <typename T, typename TV, int LAP, int OP, int R, int S, int NP>
__global__ void __launch_bounds__(256) plane_kernel(PlaneParams p, DevCoef<T> c)
{
    constexpr bool MEHRLIKE = (LAP == 0) || is_rhs_op(OP);
    constexpr int RR        = MEHRLIKE ? 1 : R; // halo rows staged
    constexpr int HOLD      = MEHRLIKE ? 0 : R; // stages kept behind the newest
    constexpr bool STAGE_V  = (OP == OP_HPSI_B);
    constexpr int QL        = MEHRLIKE ? 1 : 2 * R + 1;
    extern __shared__ __align__(128) unsigned char smem_raw[];

    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const int TY      = p.ty;
    const int rows    = TY + 2 * RR;
    const int tile_y  = blockIdx.x % p.ntile_y;
    const int tile_x  = blockIdx.x / p.ntile_y;
    const int f       = blockIdx.y;
    const int y0      = tile_y * TY;
    const int x0      = tile_x * p.xc;
    const int xcount  = min(p.xc, nx - x0);
    const int nplanes = xcount + 2 * R;

    const size_t stage_elems = (size_t)rows * nz;
    T* stages                = reinterpret_cast<T*>(smem_raw);
    TV* vstages = reinterpret_cast<TV*>(smem_raw + S * stage_elems * sizeof(T));
    uint64_t* bars = reinterpret_cast<uint64_t*>(
        smem_raw + S * stage_elems * (sizeof(T) + (STAGE_V ? sizeof(TV) : 0)));

    const T* ubase  = reinterpret_cast<const T*>(p.u) + (size_t)f * p.ldu;
    const TV* vbase = reinterpret_cast<const TV*>(p.V);

    // staged rows y0-RR .. y0+TY+RR-1 (mod ny) as at most two runs
    int ya = y0 - RR, na, nb;
    if (ya < 0)
    {
        na = -ya;
        ya += ny;
        nb = rows - na;
    }
    else if (ya + rows > ny)
    {
        na = ny - ya;
        nb = rows - na;
    }
    else
    {
        na = rows;
        nb = 0;
    }
    const uint32_t bytes_u = (uint32_t)(stage_elems * sizeof(T));
    const uint32_t bytes_v = STAGE_V ? (uint32_t)(stage_elems * sizeof(TV)) : 0u;

    auto issue = [&](int i) {
        const int slot = i % S;
        const int x    = wrap(x0 - R + i, nx);
        uint64_t* bar  = bars + slot;
        mbar_arrive_expect_tx(bar, bytes_u + bytes_v);
        T* dst       = stages + slot * stage_elems;
        const T* src = ubase + (size_t)x * ny * nz;
        bulk_g2s(dst, src + (size_t)ya * nz, (uint32_t)(na * nz * sizeof(T)), bar);
        if (nb > 0)
            bulk_g2s(dst + (size_t)na * nz, src, (uint32_t)(nb * nz * sizeof(T)), bar);
        if (STAGE_V)
        {
            TV* vdst       = vstages + slot * stage_elems;
            const TV* vsrc = vbase + (size_t)x * ny * nz;
            bulk_g2s(vdst, vsrc + (size_t)ya * nz, (uint32_t)(na * nz * sizeof(TV)), bar);
            if (nb > 0)
                bulk_g2s(vdst + (size_t)na * nz, vsrc, (uint32_t)(nb * nz * sizeof(TV)), bar);
        }
    };

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
            mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = min(S, nplanes) - 1;
    if (threadIdx.x == 0)
        for (int i = 0; i <= issued; i++)
            issue(i);

    // per-point geometry, fixed for the whole march
    const int npts = TY * nz;
    int oc[NP], ozm[NP], ozp[NP], zz[NP], yy[NP];
    bool val[NP];
#pragma unroll
    for (int k = 0; k < NP; k++)
    {
        const int pt = threadIdx.x + k * 256;
        const int y  = pt / nz;
        const int z  = pt - y * nz;
        val[k]       = (pt < npts) && (y0 + y < ny);
        yy[k]        = y;
        zz[k]        = z;
        oc[k]        = (y + RR) * nz + z;
        ozm[k]       = oc[k] + (z > 0 ? -1 : nz - 1);
        ozp[k]       = oc[k] + (z < nz - 1 ? 1 : 1 - nz);
    }
    T A1[NP], B1[NP], B2[NP], U1[NP];
    T q[NP][QL];
#pragma unroll
    for (int k = 0; k < NP; k++)
    {
        A1[k] = B1[k] = B2[k] = U1[k] = (T)0;
#pragma unroll
        for (int j = 0; j < QL; j++)
            q[k][j] = (T)0;
    }

    T* __restrict__ outp     = reinterpret_cast<T*>(p.out) + (size_t)f * p.ldo;
    T* __restrict__ updp     = (OP == OP_JACOBI_UPD)
                                   ? reinterpret_cast<T*>(p.upd) + (size_t)f * p.ldupd
                                   : nullptr;
    const T ualpha           = (T)p.upd_alpha;
    const T uscale           = (OP == OP_JACOBI_UPD && p.upd_scale) ? (T)p.upd_scale[f] : (T)1;
    T* __restrict__ wp       = p.w ? reinterpret_cast<T*>(p.w) + (size_t)f * p.ldw : nullptr;
    const T* __restrict__ fp = p.f ? reinterpret_cast<const T*>(p.f) + (size_t)f * p.ldf : nullptr;
    constexpr bool POINTWISE = is_jacobi(OP) || (OP == OP_HPSI_V) || (OP == OP_RHS_SUB);

    // pv: the pointwise operand at the emitted point (f for Jacobi, V for
    // V psi, g for B u - g), loaded before the plane wait so that its
    // latency overlaps it
    auto finish = [&](int k, int x, T lap, T ucen, T pv) {
        const int y      = y0 + yy[k];
        const int z      = zz[k];
        const size_t idx = ((size_t)x * ny + y) * nz + z;
        T r              = lap;
        if (OP == OP_HPSI_V) r = lap + (T)((TV)ucen * (TV)pv);
        if (OP == OP_RHS_SUB) r = lap - pv;
        if (is_jacobi(OP))
        {
            T w = lap - pv;
            r   = ucen - c.jf * w;
            if (p.mask.state != nullptr)
            {
                r = apply_mask<T>(p.mask, f, x, y, z, r);
                if (wp != nullptr) w = apply_mask<T>(p.mask, f, x, y, z, w);
            }
            if (wp != nullptr) wp[idx] = w;
        }
        if (OP == OP_JACOBI_UPD)
            updp[idx] = uscale * (updp[idx] + ualpha * r);
        else
            outp[idx] = r;
    };

    bool ok    = true;
    int waited = -1;
    for (int i = 0; i < nplanes; i++)
    {
        T pv[NP];
        if (POINTWISE)
        {
            const int xe = MEHRLIKE ? x0 + i - 2 : x0 + i - 2 * R;
            if (xe >= x0)
            {
#pragma unroll
                for (int k = 0; k < NP; k++)
                {
                    const size_t idx = ((size_t)xe * ny + y0 + yy[k]) * nz + zz[k];
                    pv[k]            = (T)0;
                    if (val[k]) pv[k] = (OP != OP_HPSI_V) ? fp[idx] : (T)vbase[idx];
                }
            }
        }
        ok = ok && mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
        if (ok) waited = i;
        const T* st = stages + (i % S) * stage_elems;
        if (MEHRLIKE)
        {
            const TV* vs = vstages + (i % S) * stage_elems;
            const bool emit = (i >= 2);
            const int x     = x0 + i - 2;
#pragma unroll
            for (int k = 0; k < NP; k++)
            {
                if (!val[k]) continue;
                const T u = st[oc[k]], uzm = st[ozm[k]], uzp = st[ozp[k]];
                const T uym = st[oc[k] - nz], uyp = st[oc[k] + nz];
                T a, b;
                if (is_rhs_op(OP))
                {
                    a = (T)0.5 * u + (T)(1. / 12.) * (uym + uyp + uzm + uzp);
                    b = (T)(1. / 12.) * u;
                }
                else
                {
                    const T sz = uzm + uzp, sy = uym + uyp;
                    const T corners = st[ozm[k] - nz] + st[ozp[k] - nz] + st[ozm[k] + nz]
                                      + st[ozp[k] + nz];
                    a = c.c0 * u + c.cz[0] * sz + c.cy[0] * sy + c.cyz * corners;
                    b = c.cx[0] * u + c.cxz * sz + c.cxy * sy;
                    if (STAGE_V)
                    {
                        const T wc = (T)((TV)u * vs[oc[k]]);
                        const T wf = (T)((TV)uzm * vs[ozm[k]]) + (T)((TV)uzp * vs[ozp[k]])
                                     + (T)((TV)uym * vs[oc[k] - nz])
                                     + (T)((TV)uyp * vs[oc[k] + nz]);
                        a += (T)0.5 * wc + (T)(1. / 12.) * wf;
                        b += (T)(1. / 12.) * wc;
                    }
                }
                if (emit) finish(k, x, A1[k] + B2[k] + b, U1[k], POINTWISE ? pv[k] : (T)0);
                B2[k] = B1[k];
                B1[k] = b;
                A1[k] = a;
                U1[k] = u;
            }
        }
        else
        {
            const bool emit = (i >= 2 * R);
            const int x     = x0 + i - 2 * R;
            const T* sc     = stages + ((i - R + S) % S) * stage_elems; // plane x
#pragma unroll
            for (int k = 0; k < NP; k++)
            {
                if (!val[k]) continue;
#pragma unroll
                for (int j = 0; j < QL - 1; j++)
                    q[k][j] = q[k][j + 1];
                q[k][QL - 1] = st[oc[k]];
                if (emit)
                {
                    const int z = zz[k];
                    T r         = c.c0 * q[k][R];
#pragma unroll
                    for (int d = 1; d <= R; d++)
                    {
                        const int zp = (z + d < nz) ? d : d - nz;
                        const int zm = (z - d >= 0) ? -d : nz - d;
                        r += c.cx[d - 1] * (q[k][R - d] + q[k][R + d]);
                        r += c.cy[d - 1] * (sc[oc[k] - d * nz] + sc[oc[k] + d * nz]);
                        r += c.cz[d - 1] * (sc[oc[k] + zm] + sc[oc[k] + zp]);
                    }
                    finish(k, x, r, q[k][R], POINTWISE ? pv[k] : (T)0);
                }
            }
        }
        __syncthreads();
        const int nxt = i - HOLD + S;
        if (nxt < nplanes && nxt > issued)
        {
            if (threadIdx.x == 0)
            {
                fence_proxy_async_smem();
                issue(nxt);
            }
            issued = nxt;
        }
    }
    if (!ok && threadIdx.x == 0)
    {
        if (p.err != nullptr) atomicExch(p.err, MGX_TIMEOUT);
        for (int i = waited + 1; i <= issued; i++)
            mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
    }
}

/* ------------------------------------------------------------------ */
/* vectorised radius-1 plane kernel                                     */
/* ------------------------------------------------------------------ */
// The radius-1 operators (Mehrstellen -Lap_M with or without B(V psi), the
// B operator, and the 2nd-order operator of the coarse levels) on groups of
// VEC = 16 / sizeof(T) consecutive z points: every shared-memory row access
// is one 16-byte vector plus the two z neighbours at the group ends, and the
// outputs leave as 16-byte stores.  The plane recurrence is the one of
// plane_kernel: out(x) = a(x) + b(x-1) + b(x+1).
template <typename T>
struct Vec16;
template <>
struct Vec16<float>
{
    using type = float4;
    static constexpr int N = 4;
    __device__ static float get(const float4& v, int i)
    {
        return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
    }
    __device__ static void set(float4& v, int i, float x)
    {
        if (i == 0) v.x = x;
        else if (i == 1) v.y = x;
        else if (i == 2) v.z = x;
        else v.w = x;
    }
};
template <>
struct Vec16<double>
{
    using type = double2;
    static constexpr int N = 2;
    __device__ static double get(const double2& v, int i) { return i == 0 ? v.x : v.y; }
    __device__ static void set(double2& v, int i, double x)
    {
        if (i == 0) v.x = x;
        else v.y = x;
    }
};

constexpr int JJ_CS = 4; // coarse-plane slots of the folded prolongation

/* In-plane part a and neighbour-plane part b of a radius-1 operator at the
 * VEC points of a group along z: centre row c0v with its z neighbours zl /
 * zr, rows y - 1 / y + 1 cmv / cpv and, for the Mehrstellen edges (EDGES),
 * their z neighbours ml, mr / pl, pr.  The y sum of each z column is formed
 * once and serves the column's own term and the edge terms of the columns
 * beside it.  Every stencil kernel that must give the same bits as another
 * forms a and b here. */
template <typename T, typename VH, bool EDGES>
__device__ __forceinline__ void vec_terms(const DevCoef<T>& c, const typename VH::type& c0v,
    const typename VH::type& cmv, const typename VH::type& cpv, T zl, T zr, T ml, T mr, T pl,
    T pr, T* a, T* b, T* u)
{
    constexpr int VEC = VH::N;
    T sy[VEC + 2];
#pragma unroll
    for (int v = 0; v < VEC; v++)
        sy[v + 1] = add_rn(VH::get(cmv, v), VH::get(cpv, v));
    if (EDGES)
    {
        sy[0]       = add_rn(ml, pl);
        sy[VEC + 1] = add_rn(mr, pr);
    }
#pragma unroll
    for (int v = 0; v < VEC; v++)
    {
        const T uc  = VH::get(c0v, v);
        const T uzm = v == 0 ? zl : VH::get(c0v, v - 1);
        const T uzp = v == VEC - 1 ? zr : VH::get(c0v, v + 1);
        const T sz  = add_rn(uzm, uzp);
        T aa        = fma_rn(c.cy[0], sy[v + 1], fma_rn(c.cz[0], sz, mul_rn(c.c0, uc)));
        T bb;
        if (EDGES)
        {
            aa = fma_rn(c.cyz, add_rn(sy[v], sy[v + 2]), aa);
            bb = fma_rn(c.cxy, sy[v + 1], fma_rn(c.cxz, sz, mul_rn(c.cx[0], uc)));
        }
        else
            bb = mul_rn(c.cx[0], uc);
        a[v] = aa;
        b[v] = bb;
        u[v] = uc;
    }
}

/* One Jacobi point: w = lap - f and the result ucen - jf w; scaled (the
 * first sweep from gamma f, with the staged f as input): lap and ucen are
 * gamma times the staged operator and centre, f the staged centre. */
template <typename T>
__device__ __forceinline__ T jacobi_point(T lap, T ucen, T fv, T jf, bool scaled, T gam, T& w)
{
    if (scaled)
    {
        fv   = ucen;
        lap  = mul_rn(gam, lap);
        ucen = mul_rn(gam, ucen);
    }
    w = sub_rn(lap, fv);
    return fma_rn(-jf, w, ucen);
}

/* The ABPG update of one point: scale (q + alpha r). */
template <typename T>
__device__ __forceinline__ T update_point(T q, T r, T alpha, T scale)
{
    return mul_rn(scale, fma_rn(alpha, r, q));
}

template <typename T> struct Vec8;
template <> struct Vec8<float> { using type = float2; };
template <> struct Vec8<double> { using type = double2; };

template <typename T, int LAP, int OP, int S, int NG>
__global__ void __launch_bounds__(256, 2) plane_vec_kernel(PlaneParams p, DevCoef<T> c)
{
    using V4          = typename Vec16<T>::type;
    using VH          = Vec16<T>;
    constexpr int VEC = VH::N;
    constexpr bool EDGES   = (LAP == 0) && !is_rhs_op(OP);
    constexpr bool STAGE_V = (OP == OP_HPSI_B);
    // OP_JACOBI_RST: the sweep also forms w on the row y0 - 1 and the plane
    // x0 - 1 (one more staged row and plane), keeps the last four w planes
    // in a ring and restricts three of them after each odd plane
    constexpr bool RST = (OP == OP_JACOBI_RST);
    constexpr int YO   = RST ? 1 : 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];

    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const int TY      = p.ty;
    const int rows    = TY + 2 + YO;
    const int tile_y  = blockIdx.x % p.ntile_y;
    const int tile_x  = blockIdx.x / p.ntile_y;
    const int f       = blockIdx.y;
    const int y0      = tile_y * TY;
    const int x0      = tile_x * p.xc;
    const int xcount  = min(p.xc, nx - x0);
    const int nplanes = xcount + 2 + YO;
    const bool scaled = is_jacobi(OP) && (p.gamma_in != 0.);
    const T gam       = (T)p.gamma_in;

    const size_t stage_elems = (size_t)rows * nz;
    T* stages                = reinterpret_cast<T*>(smem_raw);
    T* vstages = reinterpret_cast<T*>(smem_raw + S * stage_elems * sizeof(T));
    const size_t ring_elems = RST ? (size_t)(TY + 1) * nz : 0;
    T* wring = reinterpret_cast<T*>(smem_raw + S * stage_elems * sizeof(T) * (STAGE_V ? 2 : 1));
    uint64_t* bars = reinterpret_cast<uint64_t*>(
        smem_raw + S * stage_elems * sizeof(T) * (STAGE_V ? 2 : 1) + 4 * ring_elems * sizeof(T));

    const T* ubase = reinterpret_cast<const T*>(scaled ? p.f : p.u)
                     + (size_t)f * (scaled ? p.ldf : p.ldu);
    const T* vbase = reinterpret_cast<const T*>(p.V);

    int ya = y0 - 1 - YO, na, nb;
    if (ya < 0)
    {
        na = -ya;
        ya += ny;
        nb = rows - na;
    }
    else if (ya + rows > ny)
    {
        na = ny - ya;
        nb = rows - na;
    }
    else
    {
        na = rows;
        nb = 0;
    }
    const uint32_t bytes = (uint32_t)(stage_elems * sizeof(T)) * (STAGE_V ? 2u : 1u);

    auto issue = [&](int i) {
        const int slot = i % S;
        const int x    = wrap(x0 - 1 - YO + i, nx);
        uint64_t* bar  = bars + slot;
        mbar_arrive_expect_tx(bar, bytes);
        T* dst       = stages + slot * stage_elems;
        const T* src = ubase + (size_t)x * ny * nz;
        bulk_g2s(dst, src + (size_t)ya * nz, (uint32_t)(na * nz * sizeof(T)), bar);
        if (nb > 0) bulk_g2s(dst + (size_t)na * nz, src, (uint32_t)(nb * nz * sizeof(T)), bar);
        if (STAGE_V)
        {
            T* vdst       = vstages + slot * stage_elems;
            const T* vsrc = vbase + (size_t)x * ny * nz;
            bulk_g2s(vdst, vsrc + (size_t)ya * nz, (uint32_t)(na * nz * sizeof(T)), bar);
            if (nb > 0)
                bulk_g2s(vdst + (size_t)na * nz, vsrc, (uint32_t)(nb * nz * sizeof(T)), bar);
        }
    };

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
            mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = min(S, nplanes) - 1;
    if (threadIdx.x == 0)
        for (int i = 0; i <= issued; i++)
            issue(i);

    // group geometry
    const int gpr  = nz / VEC; // groups per row
    const int ngrp = (TY + YO) * gpr;
    int oc[NG], om[NG], op[NG], goff[NG], gy[NG], gz[NG];
    bool val[NG];
#pragma unroll
    for (int k = 0; k < NG; k++)
    {
        const int g  = threadIdx.x + k * 256;
        const int y  = g / gpr;
        const int z0 = (g - y * gpr) * VEC;
        val[k]       = (g < ngrp) && (y0 - YO + y < ny);
        gy[k]        = y;
        gz[k]        = z0;
        oc[k]        = (y + 1) * nz + z0;
        om[k]        = (y + 1) * nz + (z0 > 0 ? z0 - 1 : nz - 1);
        op[k]        = (y + 1) * nz + (z0 + VEC < nz ? z0 + VEC : 0);
        const int yr = y0 - YO + y; // row y0 - 1 of the first tile wraps
        goff[k]      = (yr < 0 ? yr + ny : yr) * nz + z0; // point offset within an x-plane
    }
    T A1[NG][VEC], B1[NG][VEC], B2[NG][VEC], U1[NG][VEC];
#pragma unroll
    for (int k = 0; k < NG; k++)
#pragma unroll
        for (int v = 0; v < VEC; v++)
            A1[k][v] = B1[k][v] = B2[k][v] = U1[k][v] = (T)0;

    T* __restrict__ outp     = reinterpret_cast<T*>(p.out) + (size_t)f * p.ldo;
    T* __restrict__ updp     = (OP == OP_JACOBI_UPD)
                                   ? reinterpret_cast<T*>(p.upd) + (size_t)f * p.ldupd
                                   : nullptr;
    const T ualpha           = (T)p.upd_alpha;
    const T uscale           = (OP == OP_JACOBI_UPD && p.upd_scale) ? (T)p.upd_scale[f] : (T)1;
    T* __restrict__ wp       = p.w ? reinterpret_cast<T*>(p.w) + (size_t)f * p.ldw : nullptr;
    const T* __restrict__ fp = p.f ? reinterpret_cast<const T*>(p.f) + (size_t)f * p.ldf : nullptr;
    constexpr bool POINTWISE = is_jacobi(OP) || (OP == OP_HPSI_V) || (OP == OP_RHS_SUB);
    const T c12 = (T)(1. / 12.), c05 = (T)0.5;
    // the result of 4 consecutive points (never across a 64-point block) as
    // bf16 hi = rn(r), lo = rn(r - hi) in the K-blocked operand planes, the
    // split of the tensor-core products
    auto store_split = [&](const size_t pt, const V4& res) {
        if constexpr (sizeof(T) == 4 && VEC == 4)
        {
            const size_t o = ((pt / 64) * (size_t)p.split_rows + f) * 64 + pt % 64;
            __align__(8) __nv_bfloat16 h[4], l[4];
#pragma unroll
            for (int v = 0; v < 4; v++)
            {
                const float x = VH::get(res, v);
                h[v]          = __float2bfloat16_rn(x);
                l[v]          = __float2bfloat16_rn(x - __bfloat162float(h[v]));
            }
            *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p.split_hi) + o)
                = *reinterpret_cast<const uint2*>(h);
            *reinterpret_cast<uint2*>(reinterpret_cast<__nv_bfloat16*>(p.split_lo) + o)
                = *reinterpret_cast<const uint2*>(l);
        }
    };

    // OP_JACOBI_RST: coarse plane X = (xe - 1) / 2 from the w planes xe - 2
    // .. xe, rows y0 - 1 .. y0 + TY - 1 of the ring; the grouping and order
    // of restrict_kernel (src/pb/MGkernels.cc:249-270).  Run after the
    // barrier that ends plane xe, beside the next plane's stencil (the ring
    // holds four planes, so that plane's w stores go to the fourth slot)
    auto restrict_plane = [&](const int xe) {
        const int cy = ny >> 1, cz = nz >> 1;
        const int X  = (xe - 1) >> 1;
        const int nyc = min(TY, ny - y0) >> 1;
        const T* Wm   = wring + (size_t)((xe - x0 - 1) & 3) * ring_elems; // plane 2X - 1
        const T* W0   = wring + (size_t)((xe - x0) & 3) * ring_elems;     // plane 2X
        const T* Wp   = wring + (size_t)((xe - x0 + 1) & 3) * ring_elems; // plane 2X + 1
        T* cp         = reinterpret_cast<T*>(p.coarse) + (size_t)f * p.ldc;
        // a thread forms the coarse pair (Z, Z + 1), Z even: fine z - 1
        // (one load) and z .. z + 3 (16-byte loads) of each of the nine
        // rows, z = 2 Z a multiple of 4
        const int hz = cz >> 1;
        for (int t = threadIdx.x; t < nyc * hz; t += 256)
        {
            const int yl = t / hz, Z = 2 * (t - (t / hz) * hz);
            const int z = 2 * Z, zm = z > 0 ? z - 1 : nz - 1;
            const int r = 2 * yl + 1; // ring row of fine y = y0 + 2 yl
            // v6[0..4]: fine z - 1 .. z + 3 of one row
            auto row = [&](const T* P, int dy, T* v6) {
                const T* q = P + (size_t)(r + dy) * nz;
                v6[0]      = q[zm];
#pragma unroll
                for (int h = 0; h < 4 / VEC; h++)
                {
                    const V4 c = *reinterpret_cast<const V4*>(q + z + h * VEC);
#pragma unroll
                    for (int v = 0; v < VEC; v++)
                        v6[1 + h * VEC + v] = VH::get(c, v);
                }
            };
            T r00[5], rp0[5], rm0[5], r0p[5], r0m[5], rpp[5], rpm[5], rmp[5], rmm[5];
            row(W0, 0, r00);
            row(Wp, 0, rp0);
            row(Wm, 0, rm0);
            row(W0, 1, r0p);
            row(W0, -1, r0m);
            row(Wp, 1, rpp);
            row(Wp, -1, rpm);
            row(Wm, 1, rmp);
            row(Wm, -1, rmm);
#pragma unroll
            for (int c2 = 0; c2 < 2; c2++)
            {
                // the three fine z of coarse Z + c2 start at index 2 c2
                const int o    = 2 * c2;
                const T face   = rp0[o + 1] + rm0[o + 1] + r0p[o + 1] + r0m[o + 1] + r00[o]
                               + r00[o + 2];
                const T corner = rpp[o] + rpp[o + 2] + rpm[o] + rpm[o + 2] + rmp[o] + rmp[o + 2]
                                 + rmm[o] + rmm[o + 2];
                const T edge   = r0p[o] + r0p[o + 2] + r0m[o] + r0m[o + 2] + rp0[o] + rp0[o + 2]
                               + rm0[o] + rm0[o + 2] + rmm[o + 1] + rpm[o + 1] + rmp[o + 1]
                               + rpp[o + 1];
                cp[((size_t)X * cy + (y0 >> 1) + yl) * cz + Z + c2]
                    = (T)(1. / 64.) * ((T)8. * r00[o + 1] + (T)4. * face + (T)2. * edge + corner);
            }
        }
    };
    int pend = -1; // the plane whose restriction is due

    bool ok    = true;
    int waited = -1;
    for (int i = 0; i < nplanes; i++)
    {
        if (RST && pend >= 0)
        {
            restrict_plane(pend);
            pend = -1;
        }
        const int xe    = x0 + i - 2 - YO;
        const bool emit = (i >= 2);
        const size_t xoff = (size_t)(emit ? (xe < 0 ? xe + nx : xe) : 0) * ny * nz;
        V4 pv[NG];
        V4 uv[NG]; // OP_JACOBI_UPD: the block being updated, fetched with pv
        if (POINTWISE && emit && !scaled)
        {
#pragma unroll
            for (int k = 0; k < NG; k++)
                if (val[k])
                {
                    pv[k] = *reinterpret_cast<const V4*>(
                        (OP != OP_HPSI_V ? fp : vbase) + xoff + goff[k]);
                    if (OP == OP_JACOBI_UPD)
                        uv[k] = *reinterpret_cast<const V4*>(updp + xoff + goff[k]);
                }
        }
        ok = ok && mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
        if (ok) waited = i;
        const T* st = stages + (i % S) * stage_elems;
        const T* vs = vstages + (i % S) * stage_elems;
#pragma unroll
        for (int k = 0; k < NG; k++)
        {
            if (!val[k]) continue;
            const V4 c0v = *reinterpret_cast<const V4*>(st + oc[k]);
            const V4 cmv = *reinterpret_cast<const V4*>(st + oc[k] - nz);
            const V4 cpv = *reinterpret_cast<const V4*>(st + oc[k] + nz);
            const T zl = st[om[k]], zr = st[op[k]];
            T ml = 0, mr = 0, pl = 0, pr = 0;
            if (EDGES)
            {
                ml = st[om[k] - nz];
                mr = st[op[k] - nz];
                pl = st[om[k] + nz];
                pr = st[op[k] + nz];
            }
            V4 vcv, vmv, vpv;
            T vzl = 0, vzr = 0;
            if (STAGE_V)
            {
                vcv = *reinterpret_cast<const V4*>(vs + oc[k]);
                vmv = *reinterpret_cast<const V4*>(vs + oc[k] - nz);
                vpv = *reinterpret_cast<const V4*>(vs + oc[k] + nz);
                vzl = vs[om[k]];
                vzr = vs[op[k]];
            }
            V4 res;
            V4 wres;
            T ta[VEC], tb[VEC], tu[VEC];
            if (!is_rhs_op(OP)) vec_terms<T, VH, EDGES>(c, c0v, cmv, cpv, zl, zr, ml, mr, pl, pr, ta, tb, tu);
#pragma unroll
            for (int v = 0; v < VEC; v++)
            {
                T u         = VH::get(c0v, v);
                T uzm       = v == 0 ? zl : VH::get(c0v, v - 1);
                T uzp       = v == VEC - 1 ? zr : VH::get(c0v, v + 1);
                T uym       = VH::get(cmv, v);
                T uyp       = VH::get(cpv, v);
                T a, b;
                if (is_rhs_op(OP))
                {
                    a = c05 * u + c12 * (uym + uyp + uzm + uzp);
                    b = c12 * u;
                }
                else
                {
                    a = ta[v];
                    b = tb[v];
                    if (STAGE_V)
                    {
                        const T vc  = VH::get(vcv, v);
                        const T vzm = v == 0 ? vzl : VH::get(vcv, v - 1);
                        const T vzp = v == VEC - 1 ? vzr : VH::get(vcv, v + 1);
                        const T wc  = u * vc;
                        const T wf  = uzm * vzm + uzp * vzp + uym * VH::get(vmv, v)
                                     + uyp * VH::get(vpv, v);
                        a += c05 * wc + c12 * wf;
                        b += c12 * wc;
                    }
                }
                if (emit)
                {
                    T lap = add_rn(add_rn(A1[k][v], B2[k][v]), b);
                    T ucen = U1[k][v];
                    T r    = lap;
                    if (OP == OP_HPSI_V) r = lap + ucen * VH::get(pv[k], v);
                    if (OP == OP_RHS_SUB) r = lap - VH::get(pv[k], v);
                    if (is_jacobi(OP))
                    {
                        // scaled: staged f, u = gamma f, -Lap u = gamma (-Lap f)
                        T w;
                        r = jacobi_point<T>(lap, ucen, scaled ? (T)0 : VH::get(pv[k], v), c.jf,
                            scaled, gam, w);
                        if (p.mask.state != nullptr)
                        {
                            const int y = y0 + gy[k], z = gz[k] + v;
                            r           = apply_mask<T>(p.mask, f, xe, y, z, r);
                            w           = apply_mask<T>(p.mask, f, xe, y, z, w);
                        }
                        VH::set(wres, v, w);
                    }
                    VH::set(res, v, r);
                }
                B2[k][v] = B1[k][v];
                B1[k][v] = b;
                A1[k][v] = a;
                U1[k][v] = u;
            }
            if (emit)
            {
                if (OP == OP_JACOBI_UPD)
                {
                    // the sweep that starts from gamma f (scaled) is never the
                    // last one, so uv was fetched above
                    V4 q = uv[k];
#pragma unroll
                    for (int v = 0; v < VEC; v++)
                        VH::set(q, v, update_point<T>(VH::get(q, v), VH::get(res, v), ualpha, uscale));
                    *reinterpret_cast<V4*>(updp + xoff + goff[k]) = q;
                }
                else if (OP == OP_RHS_SPLIT)
                    store_split(xoff + goff[k], res);
                else if (!RST || (gy[k] >= YO && xe >= x0))
                {
                    *reinterpret_cast<V4*>(outp + xoff + goff[k]) = res;
                    // H psi also written as the tensor-core operand planes
                    if (OP == OP_HPSI_B && p.split_hi != nullptr) store_split(xoff + goff[k], res);
                }
                if (RST)
                    *reinterpret_cast<V4*>(wring + (size_t)((xe - x0 + 1) & 3) * ring_elems
                                           + (size_t)gy[k] * nz + gz[k]) = wres;
                else if (is_jacobi(OP) && wp != nullptr)
                    *reinterpret_cast<V4*>(wp + xoff + goff[k]) = wres;
            }
        }
        if (RST && emit && xe > x0 && ((xe - x0) & 1)) pend = xe;
        __syncthreads();
        const int nxt = i + S;
        if (nxt < nplanes && nxt > issued)
        {
            if (threadIdx.x == 0)
            {
                fence_proxy_async_smem();
                issue(nxt);
            }
            issued = nxt;
        }
    }
    if (RST && pend >= 0) restrict_plane(pend);
    if (!ok && threadIdx.x == 0)
    {
        if (p.err != nullptr) atomicExch(p.err, MGX_TIMEOUT);
        for (int i = waited + 1; i <= issued; i++)
            mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
    }
}

/* ------------------------------------------------------------------ */
/* two Jacobi sweeps in one plane march                                 */
/* ------------------------------------------------------------------ */
// Two consecutive Jacobi sweeps of one level, u1 = u - jf (A u - f) and
// u2 = u1 - jf (A u1 - f), in one launch.  The staged input is folded into
// u1 as in plane_vec_kernel; each plane of u1 goes to a two-plane buffer in
// shared memory, and a second set of partial sums folds it into u2 one
// plane behind.  u1 is formed on the tile's rows and planes and one more on
// each side, so a tile needs no other tile's u1: the input and f cross DRAM
// once and u1 never does.  Each point keeps the operation order of two
// plane_vec_kernel sweeps (the first one scaled when gamma_in is set), so
// the results are the same bits.  The running sums keep A(x - 1) + B(x - 2)
// as one value, the first addition of plane_vec_kernel's A1 + B2 + b, and
// both kernels form every sum and product of a point with explicitly
// rounded operations (vec_terms, jacobi_point, update_point, add_rn).
// MODE JJ_STORE stores u2 to out; JJ_UPD adds it into the update block as
// OP_JACOBI_UPD does; JJ_RST stores it and restricts the second sweep's
// residual into the next level's right-hand side as OP_JACOBI_RST does
// (w on one more row and plane, kept in a four-plane ring).
template <typename T, int LAP, int MODE, int S, int NG1, int NG2, int NT>
__global__ void __launch_bounds__(NT, 512 / NT) plane_jj_kernel(PlaneParams p, DevCoef<T> c)
{
    using V4             = typename Vec16<T>::type;
    using VH             = Vec16<T>;
    using T2             = typename Vec8<T>::type;
    constexpr int VEC    = VH::N;
    constexpr bool EDGES = (LAP == 0);
    constexpr bool PRO   = (MODE & JJ_PRO) != 0;
    constexpr bool RST   = ((MODE & 3) == JJ_RST);
    constexpr bool UPD   = ((MODE & 3) == JJ_UPD);
    constexpr int YO     = RST ? 1 : 0;
    extern __shared__ __align__(128) unsigned char smem_raw[];

    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const int TY      = p.ty;
    const int rows2   = TY + YO;   // second sweep: rows y0 - YO .. y0 + TY - 1
    const int rows1   = rows2 + 2; // first sweep: one row more on each side
    const int rows_s  = rows1 + 2; // staged input
    const int tile_y  = blockIdx.x % p.ntile_y;
    const int tile_x  = blockIdx.x / p.ntile_y;
    const int f       = blockIdx.y;
    const int y0      = tile_y * TY;
    const int x0      = tile_x * p.xc;
    const int xcount  = min(p.xc, nx - x0);
    const int nplanes = xcount + YO + 4; // staged planes x0 - YO - 2 .. x0 + xcount + 1
    const bool scaled = (p.gamma_in != 0.);
    const T gam       = (T)p.gamma_in;

    const size_t stage_elems = (size_t)rows_s * nz;
    const size_t u1_elems    = (size_t)rows1 * nz;
    const size_t ring_elems  = RST ? (size_t)(TY + 1) * nz : 0;
    // JJ_PRO: coarse rows jlo .. jlo + CROWS - 1 of the correction e, one
    // coarse plane per slot of a JJ_CS-slot ring; coarse plane q (from
    // (x0 - 2) / 2) rides on the mbarrier of fine stage 0 (q = 0) or
    // 2q - 1, and fine stage i reads planes i / 2 and, odd, i / 2 + 1
    const int cz         = nz >> 1;
    const int crows      = PRO ? (TY + 7) / 2 : 0;
    const int jlo        = (y0 - 2) >> 1;
    const size_t c_elems = (size_t)crows * cz;
    T* stages      = reinterpret_cast<T*>(smem_raw);
    T* u1buf       = stages + S * stage_elems;
    T* wring       = u1buf + 2 * u1_elems;
    T* cring       = wring + 4 * ring_elems;
    uint64_t* bars = reinterpret_cast<uint64_t*>(cring + JJ_CS * c_elems);

    const T* ubase = reinterpret_cast<const T*>(scaled ? p.f : p.u)
                     + (size_t)f * (scaled ? p.ldf : p.ldu);
    // the staged rows y0 - YO - 2 .. y0 + TY + 1 in at most two pieces
    int ya = y0 - YO - 2, na, nb;
    if (ya < 0)
    {
        na = -ya;
        ya += ny;
        nb = rows_s - na;
    }
    else if (ya + rows_s > ny)
    {
        na = ny - ya;
        nb = rows_s - na;
    }
    else
    {
        na = rows_s;
        nb = 0;
    }
    const uint32_t bytes = (uint32_t)(stage_elems * sizeof(T));
    // JJ_PRO: the coarse rows in at most two pieces
    const int cy = ny >> 1, cx = nx >> 1;
    int cja = jlo < 0 ? jlo + cy : jlo, cna = crows, cnb = 0;
    if (PRO && cja + crows > cy)
    {
        cna = cy - cja;
        cnb = crows - cna;
    }
    const T* epb = PRO ? reinterpret_cast<const T*>(p.pro) + (size_t)f * p.ldpro : nullptr;
    auto issue = [&](int i) {
        const int slot = i % S;
        const int x    = wrap(x0 - YO - 2 + i, nx);
        uint64_t* bar  = bars + slot;
        const bool cpl = PRO && (i == 0 || (i & 1));
        mbar_arrive_expect_tx(bar, bytes + (cpl ? (uint32_t)(c_elems * sizeof(T)) : 0u));
        T* dst       = stages + slot * stage_elems;
        const T* src = ubase + (size_t)x * ny * nz;
        bulk_g2s(dst, src + (size_t)ya * nz, (uint32_t)(na * nz * sizeof(T)), bar);
        if (nb > 0) bulk_g2s(dst + (size_t)na * nz, src, (uint32_t)(nb * nz * sizeof(T)), bar);
        if (cpl)
        {
            const int q  = (i + 1) >> 1;
            const int xc = wrap(((x0 - 2) >> 1) + q, cx);
            T* cdst       = cring + (size_t)(q % JJ_CS) * c_elems;
            const T* csrc = epb + (size_t)xc * cy * cz;
            bulk_g2s(cdst, csrc + (size_t)cja * cz, (uint32_t)(cna * cz * sizeof(T)), bar);
            if (cnb > 0)
                bulk_g2s(cdst + (size_t)cna * cz, csrc, (uint32_t)(cnb * cz * sizeof(T)), bar);
        }
    };

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < S; s++)
            mbar_init(bars + s, 1);
        fence_mbar_init();
    }
    __syncthreads();
    int issued = min(S, nplanes) - 1;
    if (threadIdx.x == 0)
        for (int i = 0; i <= issued; i++)
            issue(i);

    // groups of VEC points along z: the first sweep's on rows1 rows (centre
    // in stage row r + 1, u1 row r), the second sweep's on rows2 rows
    // (centre in u1 row r + 1)
    const int gpr = nz / VEC;
    int o1[NG1], m1[NG1], p1[NG1], g1[NG1];
    bool ok1[NG1];
#pragma unroll
    for (int k = 0; k < NG1; k++)
    {
        const int g  = threadIdx.x + k * NT;
        const int r  = g / gpr;
        const int z0 = (g - r * gpr) * VEC;
        ok1[k]       = g < rows1 * gpr;
        o1[k]        = (r + 1) * nz + z0;
        m1[k]        = (r + 1) * nz + (z0 > 0 ? z0 - 1 : nz - 1);
        p1[k]        = (r + 1) * nz + (z0 + VEC < nz ? z0 + VEC : 0);
        const int yr = y0 - YO - 1 + r;
        g1[k]        = (yr < 0 ? yr + ny : (yr >= ny ? yr - ny : yr)) * nz + z0;
    }
    int o2[NG2], m2[NG2], p2[NG2], g2[NG2], r2[NG2];
    bool ok2[NG2];
#pragma unroll
    for (int k = 0; k < NG2; k++)
    {
        const int g  = threadIdx.x + k * NT;
        const int r  = g / gpr;
        const int z0 = (g - r * gpr) * VEC;
        ok2[k]       = g < rows2 * gpr;
        r2[k]        = r;
        o2[k]        = (r + 1) * nz + z0;
        m2[k]        = (r + 1) * nz + (z0 > 0 ? z0 - 1 : nz - 1);
        p2[k]        = (r + 1) * nz + (z0 + VEC < nz ? z0 + VEC : 0);
        const int yr = y0 - YO + r;
        g2[k]        = (yr < 0 ? yr + ny : yr) * nz + z0;
    }
    bool ok    = true;
    int waited = -1;
    // running sums: P = A(x - 1) + B(x - 2), Q = B(x - 1), C = u(x - 1)
    T P1[NG1][VEC], Q1[NG1][VEC], C1[NG1][VEC];
    T P2[NG2][VEC], Q2[NG2][VEC], C2[NG2][VEC];
#pragma unroll
    for (int k = 0; k < NG1; k++)
#pragma unroll
        for (int v = 0; v < VEC; v++)
            P1[k][v] = Q1[k][v] = C1[k][v] = (T)0;
#pragma unroll
    for (int k = 0; k < NG2; k++)
#pragma unroll
        for (int v = 0; v < VEC; v++)
            P2[k][v] = Q2[k][v] = C2[k][v] = (T)0;

    T* __restrict__ outp     = reinterpret_cast<T*>(p.out) + (size_t)f * p.ldo;
    T* __restrict__ updp     = UPD ? reinterpret_cast<T*>(p.upd) + (size_t)f * p.ldupd : nullptr;
    const T ualpha           = (T)p.upd_alpha;
    const T uscale           = (UPD && p.upd_scale) ? (T)p.upd_scale[f] : (T)1;
    const T* __restrict__ fp = reinterpret_cast<const T*>(p.f) + (size_t)f * p.ldf;

    // JJ_PRO: the staged plane i becomes u - P e before the first sweep
    // reads it; each thread takes fine z pairs (2k, 2k + 1) of the staged
    // rows, with prolong_kernel's arithmetic for every point
    // the staged coarse rows of fine stage i: plane i / 2 (and i / 2 + 1);
    // fine row y0 - 2 + rs reads coarse rows jr and jr + 1 of them
    auto correct = [&](int i) {
        const int a = i & 1; // parity of the fine plane (x0 is even)
        const T* ca = cring + (size_t)((i >> 1) % JJ_CS) * c_elems;
        const T* cb = cring + (size_t)(((i >> 1) + 1) % JJ_CS) * c_elems;
        T* stp      = stages + (size_t)(i % S) * stage_elems;
        for (int t = threadIdx.x; t < rows_s * cz; t += NT)
        {
            const int rs = t / cz, k = t - rs * cz;
            const int yu = y0 - 2 + rs;
            const int jr = (yu >> 1) - jlo, b = yu & 1;
            const int k1 = k + 1 < cz ? k + 1 : 0;
            const T* c00 = ca + (size_t)jr * cz;
            const T a0 = c00[k], a1 = c00[k1];
            T v0, v1;
            if (!a)
            {
                if (!b)
                {
                    v0 = a0;
                    v1 = (T)0.5 * (a0 + a1);
                }
                else
                {
                    const T* c01 = c00 + cz;
                    const T b0 = c01[k], b1 = c01[k1];
                    v0 = (T)0.5 * (b0 + a0);
                    v1 = (T)0.25 * (b1 + a1 + b0 + a0);
                }
            }
            else
            {
                const T* c10 = cb + (size_t)jr * cz;
                const T d0 = c10[k], d1 = c10[k1];
                if (!b)
                {
                    v0 = (T)0.5 * (d0 + a0);
                    v1 = (T)0.25 * (d1 + d0 + a1 + a0);
                }
                else
                {
                    const T* c01 = c00 + cz;
                    const T* c11 = c10 + cz;
                    const T b0 = c01[k], b1 = c01[k1], g0 = c11[k], g1 = c11[k1];
                    v0 = (T)0.25 * (g0 + d0 + b0 + a0);
                    v1 = (T)0.125 * (g1 + g0 + d1 + d0 + b1 + b0 + a1 + a0);
                }
            }
            T2* q = reinterpret_cast<T2*>(stp + (size_t)rs * nz + 2 * k);
            T2 uu = *q;
            uu.x  = uu.x - v0;
            uu.y  = uu.y - v1;
            *q    = uu;
        }
    };
    if (PRO)
    {
        ok = mbar_wait(bars, 0u);
        if (ok) waited = 0;
        if (ok) correct(0);
        __syncthreads();
    }

    // in-plane part a and neighbour-plane part b of the operator at the
    // group's VEC points (vec_terms, as in plane_vec_kernel)
    auto terms = [&](const T* q, int oc, int om, int op, T (&a)[VEC], T (&b)[VEC], T (&u)[VEC]) {
        const V4 c0v = *reinterpret_cast<const V4*>(q + oc);
        const V4 cmv = *reinterpret_cast<const V4*>(q + oc - nz);
        const V4 cpv = *reinterpret_cast<const V4*>(q + oc + nz);
        const T zl = q[om], zr = q[op];
        T ml = 0, mr = 0, pl = 0, pr = 0;
        if (EDGES)
        {
            ml = q[om - nz];
            mr = q[op - nz];
            pl = q[om + nz];
            pr = q[op + nz];
        }
        vec_terms<T, VH, EDGES>(c, c0v, cmv, cpv, zl, zr, ml, mr, pl, pr, a, b, u);
    };

    // OP_JACOBI_RST's restriction of the fine plane xe (odd from x0) and the
    // two before it (plane_vec_kernel's restrict_plane)
    auto restrict_plane = [&](const int xe) {
        const int X   = (xe - 1) >> 1;
        const int nyc = TY >> 1;
        const T* Wm   = wring + (size_t)((xe - x0 - 1) & 3) * ring_elems; // plane 2X - 1
        const T* W0   = wring + (size_t)((xe - x0) & 3) * ring_elems;     // plane 2X
        const T* Wp   = wring + (size_t)((xe - x0 + 1) & 3) * ring_elems; // plane 2X + 1
        T* cp         = reinterpret_cast<T*>(p.coarse) + (size_t)f * p.ldc;
        const int hz  = cz >> 1;
        // from the last threads, which hold one second-sweep group fewer
        for (int t = NT - 1 - threadIdx.x; t < nyc * hz; t += NT)
        {
            const int yl = t / hz, Z = 2 * (t - (t / hz) * hz);
            const int z = 2 * Z, zm = z > 0 ? z - 1 : nz - 1;
            const int r = 2 * yl + 1; // ring row of fine y = y0 + 2 yl
            auto row = [&](const T* P, int dy, T* v6) {
                const T* q = P + (size_t)(r + dy) * nz;
                v6[0]      = q[zm];
#pragma unroll
                for (int h = 0; h < 4 / VEC; h++)
                {
                    const V4 cc = *reinterpret_cast<const V4*>(q + z + h * VEC);
#pragma unroll
                    for (int v = 0; v < VEC; v++)
                        v6[1 + h * VEC + v] = VH::get(cc, v);
                }
            };
            T r00[5], rp0[5], rm0[5], r0p[5], r0m[5], rpp[5], rpm[5], rmp[5], rmm[5];
            row(W0, 0, r00);
            row(Wp, 0, rp0);
            row(Wm, 0, rm0);
            row(W0, 1, r0p);
            row(W0, -1, r0m);
            row(Wp, 1, rpp);
            row(Wp, -1, rpm);
            row(Wm, 1, rmp);
            row(Wm, -1, rmm);
#pragma unroll
            for (int c2 = 0; c2 < 2; c2++)
            {
                const int o    = 2 * c2;
                const T face   = rp0[o + 1] + rm0[o + 1] + r0p[o + 1] + r0m[o + 1] + r00[o]
                               + r00[o + 2];
                const T corner = rpp[o] + rpp[o + 2] + rpm[o] + rpm[o + 2] + rmp[o] + rmp[o + 2]
                                 + rmm[o] + rmm[o + 2];
                const T edge   = r0p[o] + r0p[o + 2] + r0m[o] + r0m[o + 2] + rp0[o] + rp0[o + 2]
                               + rm0[o] + rm0[o + 2] + rmm[o + 1] + rpm[o + 1] + rmp[o + 1]
                               + rpp[o + 1];
                cp[((size_t)X * cy + (y0 >> 1) + yl) * cz + Z + c2]
                    = (T)(1. / 64.) * ((T)8. * r00[o + 1] + (T)4. * face + (T)2. * edge + corner);
            }
        }
    };
    int pend = -1; // the w plane whose restriction is due after the next barrier

    for (int i = 0; i < nplanes; i++)
    {
        const int xs     = x0 - YO - 2 + i; // staged plane
        const bool emit1 = (i >= 2);        // u1 of plane xs - 1
        const bool emit2 = (i >= 4);        // u2 of plane xs - 2
        const int e2     = xs - 2;
        const size_t xo1 = (size_t)(emit1 ? wrap(xs - 1, nx) : 0) * ny * nz;
        const size_t xo2 = (size_t)(emit2 ? wrap(e2, nx) : 0) * ny * nz;
        V4 fa[NG1], fb[NG2], ub[NG2];
        if (emit1 && !scaled)
        {
#pragma unroll
            for (int k = 0; k < NG1; k++)
                if (ok1[k]) fa[k] = *reinterpret_cast<const V4*>(fp + xo1 + g1[k]);
        }
        // the second sweep's f (and update block), fetched here or, with
        // JJ_PRO, after the correction (fewer values live across it)
        auto fetch2 = [&]() {
            if (!emit2) return;
#pragma unroll
            for (int k = 0; k < NG2; k++)
                if (ok2[k])
                {
                    fb[k] = *reinterpret_cast<const V4*>(fp + xo2 + g2[k]);
                    if (UPD) ub[k] = *reinterpret_cast<const V4*>(updp + xo2 + g2[k]);
                }
        };
        if (!PRO) fetch2();
        ok = ok && mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
        if (ok) waited = i;
        const T* st = stages + (i % S) * stage_elems;
        T* u1p      = u1buf + (size_t)(i & 1) * u1_elems;
        // first sweep
#pragma unroll
        for (int k = 0; k < NG1; k++)
        {
            if (!ok1[k]) continue;
            T a[VEC], b[VEC], u[VEC];
            terms(st, o1[k], m1[k], p1[k], a, b, u);
            V4 res;
#pragma unroll
            for (int v = 0; v < VEC; v++)
            {
                if (emit1)
                {
                    T w;
                    VH::set(res, v, jacobi_point<T>(add_rn(P1[k][v], b[v]), C1[k][v],
                                        scaled ? (T)0 : VH::get(fa[k], v), c.jf, scaled, gam, w));
                }
                P1[k][v] = add_rn(a[v], Q1[k][v]);
                Q1[k][v] = b[v];
                C1[k][v] = u[v];
            }
            if (emit1) *reinterpret_cast<V4*>(u1p + o1[k] - nz) = res;
        }
        // JJ_PRO: the next staged plane, read after the barrier below
        if (PRO)
        {
            if (i + 1 < nplanes)
            {
                ok = ok && mbar_wait(bars + ((i + 1) % S), (uint32_t)(((i + 1) / S) & 1));
                if (ok) correct(i + 1);
            }
            fetch2();
        }
        __syncthreads();
        const int nxt = i + S;
        if (nxt < nplanes && nxt > issued)
        {
            if (threadIdx.x == 0)
            {
                fence_proxy_async_smem();
                issue(nxt);
            }
            issued = nxt;
        }
        if (RST && pend >= 0)
        {
            restrict_plane(pend);
            pend = -1;
        }
        if (!emit1) continue;
        // second sweep, folding the u1 plane xs - 1 written above
#pragma unroll
        for (int k = 0; k < NG2; k++)
        {
            if (!ok2[k]) continue;
            T a[VEC], b[VEC], u[VEC];
            terms(u1p, o2[k], m2[k], p2[k], a, b, u);
            V4 res, wres;
#pragma unroll
            for (int v = 0; v < VEC; v++)
            {
                if (emit2)
                {
                    T w;
                    VH::set(res, v, jacobi_point<T>(add_rn(P2[k][v], b[v]), C2[k][v],
                                        VH::get(fb[k], v), c.jf, false, (T)0, w));
                    VH::set(wres, v, w);
                }
                P2[k][v] = add_rn(a[v], Q2[k][v]);
                Q2[k][v] = b[v];
                C2[k][v] = u[v];
            }
            if (!emit2) continue;
            if (UPD)
            {
                V4 q = ub[k];
#pragma unroll
                for (int v = 0; v < VEC; v++)
                    VH::set(q, v, update_point<T>(VH::get(q, v), VH::get(res, v), ualpha, uscale));
                *reinterpret_cast<V4*>(updp + xo2 + g2[k]) = q;
            }
            else if (!RST || (r2[k] >= YO && e2 >= x0))
                *reinterpret_cast<V4*>(outp + xo2 + g2[k]) = res;
            if (RST)
                *reinterpret_cast<V4*>(wring + (size_t)((e2 - x0 + 1) & 3) * ring_elems
                                       + (size_t)(o2[k] - nz)) = wres;
        }
        if (RST && emit2 && e2 > x0 && ((e2 - x0) & 1)) pend = e2;
    }
    if (RST && pend >= 0)
    {
        __syncthreads();
        restrict_plane(pend);
    }
    if (!ok && threadIdx.x == 0)
    {
        if (p.err != nullptr) atomicExch(p.err, MGX_TIMEOUT);
        for (int i = waited + 1; i <= issued; i++)
            mbar_wait(bars + (i % S), (uint32_t)((i / S) & 1));
    }
}

/* ------------------------------------------------------------------ */
/* direct kernel (global loads with wrap), for small / unaligned cases  */
/* ------------------------------------------------------------------ */
template <typename T, typename TV, int LAP, int OP, int R>
__global__ void __launch_bounds__(256) direct_kernel(PlaneParams p, DevCoef<T> c)
{
    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const size_t npts = (size_t)nx * ny * nz;
    const int f       = blockIdx.y;
    const T* ub       = reinterpret_cast<const T*>(p.u) + (size_t)f * p.ldu;
    const TV* vb      = reinterpret_cast<const TV*>(p.V);
    for (size_t idx = (size_t)blockIdx.x * blockDim.x + threadIdx.x; idx < npts;
         idx += (size_t)gridDim.x * blockDim.x)
    {
        const int z = (int)(idx % nz);
        const int y = (int)((idx / nz) % ny);
        const int x = (int)(idx / ((size_t)nz * ny));
        auto at     = [&](int dx, int dy, int dz) -> T {
            return ub[((size_t)wrap(x + dx, nx) * ny + wrap(y + dy, ny)) * nz
                      + wrap(z + dz, nz)];
        };
        auto vat = [&](int dx, int dy, int dz) -> TV {
            return vb[((size_t)wrap(x + dx, nx) * ny + wrap(y + dy, ny)) * nz
                      + wrap(z + dz, nz)];
        };
        T wres = (T)0;
        T r    = PointOp<T, TV, LAP, OP, R>::apply(p, c, at, vat, f, idx, &wres);
        if (is_jacobi(OP))
        {
            if (p.mask.state != nullptr)
            {
                r = apply_mask<T>(p.mask, f, x, y, z, r);
                if (p.w != nullptr) wres = apply_mask<T>(p.mask, f, x, y, z, wres);
            }
            if (p.w != nullptr)
                reinterpret_cast<T*>(p.w)[(size_t)f * p.ldw + idx] = wres;
        }
        if (OP == OP_JACOBI_UPD)
        {
            T* u = reinterpret_cast<T*>(p.upd) + (size_t)f * p.ldupd + idx;
            *u   = (p.upd_scale ? (T)p.upd_scale[f] : (T)1) * (*u + (T)p.upd_alpha * r);
        }
        else
            reinterpret_cast<T*>(p.out)[(size_t)f * p.ldo + idx] = r;
    }
}

/* ------------------------------------------------------------------ */
/* launcher                                                             */
/* ------------------------------------------------------------------ */
constexpr int PLANE_NP = 8; // points per thread (TY * nz <= 2048)

template <int LAP, int OP, int R>
constexpr int stages_for()
{
    // ring depth: planes held behind the newest + 3 in flight
    return ((LAP == 0) || is_rhs_op(OP)) ? 4 : R + 4;
}

/* Can the vectorised radius-1 kernel run this launch?  It needs the
 * operator to be radius 1 with a uniform element type, and every block it
 * touches 16-byte aligned with rows of whole vectors. */
template <typename T, typename TV, int LAP, int OP, int R>
static bool vec_ok(const PlaneParams& p, int force_direct)
{
    if (force_direct || R != 1) return false;
    if (!(LAP == 0 || LAP == 1 || is_rhs_op(OP))) return false;
    if ((OP == OP_HPSI_B || OP == OP_HPSI_V) && sizeof(T) != sizeof(TV)) return false;
    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    auto al = [](const void* q, size_t ld) {
        return q == nullptr || (((uintptr_t)q % 16) == 0 && (ld * sizeof(T)) % 16 == 0);
    };
    if ((nz * sizeof(T)) % 16) return false;
    if (!al(p.u, p.ldu) || !al(p.out, p.ldo) || !al(p.w, p.ldw) || !al(p.f, p.ldf)
        || !al(p.upd, p.ldupd))
        return false;
    if (p.V && ((uintptr_t)p.V % 16)) return false;
    if (ny < 3 || nx < 1 || nz > 256 * 2 * (16 / (int)sizeof(T))) return false;
    return true;
}

template <typename T, typename TV, int LAP, int OP, int R>
static int launch_vec(const PlaneParams& p0, const DevCoef<T>& c, int nfunc,
    cudaStream_t stream)
{
    constexpr int S   = 4;
    constexpr int NG  = 2;
    constexpr int VEC = 16 / sizeof(T);
    constexpr bool STAGE_V = (OP == OP_HPSI_B);
    PlaneParams p = p0;
    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const size_t esz = sizeof(T) * (STAGE_V ? 2 : 1);
    const size_t smem_cap = 110 * 1024;
    // OP_JACOBI_RST: one more row of groups (y0 - 1), an even tile height,
    // and three planes of TY + 1 rows of w for the restriction
    constexpr bool RST = (OP == OP_JACOBI_RST);
    constexpr int YO   = RST ? 1 : 0;
    if (RST && (((nx | ny) & 1) || (nz % 4)))
        return fail(MGX_UNSUPPORTED, "the fused restriction needs even x, y and z % 4 == 0");
    auto smem_for = [&](int t) {
        return (size_t)S * (t + 2 + YO) * nz * esz + (RST ? 4 * (size_t)(t + 1) * nz * sizeof(T) : 0)
               + S * 8;
    };
    int ty = std::min(32, (256 * NG * VEC) / nz - YO);
    ty     = std::min(ty, ny - 2 - YO);
    if (RST) ty &= ~1;
    for (; ty >= 1; ty -= RST ? 2 : 1)
        if (smem_for(ty) <= smem_cap) break;
    if (ty < 1) return fail(MGX_UNSUPPORTED, "plane too large for the vector kernel");
    p.ty      = ty;
    p.ntile_y = (ny + ty - 1) / ty;
    int xc = 32;
    while (xc > 4 && (size_t)p.ntile_y * ((nx + xc - 1) / xc) * nfunc < 4 * 152)
        xc /= 2;
    if (xc > nx) xc = nx;
    p.xc       = xc;
    p.ntile_x  = (nx + xc - 1) / xc;
    const size_t smem = smem_for(ty);
    auto kern         = plane_vec_kernel<T, LAP == 1 ? 1 : 0, OP, S, NG>;
    cudaError_t e     = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
        (int)smem);
    if (e != cudaSuccess) return cuda_check(e, "plane_vec_kernel smem attribute");
    dim3 grid(p.ntile_y * p.ntile_x, nfunc);
    kern<<<grid, 256, smem, stream>>>(p, c);
    MGX_LAUNCH_CHECK("plane_vec_kernel");
    return MGX_OK;
}

template <typename T, typename TV, int LAP, int OP, int R>
static int launch_t(const PlaneParams& p0, const DevCoef<T>& c, int nfunc,
    cudaStream_t stream, int force_direct)
{
    if (vec_ok<T, TV, LAP, OP, R>(p0, force_direct) && (OP != OP_JACOBI_RST || !p0.mask.state))
        return launch_vec<T, TV, LAP, OP, R>(p0, c, nfunc, stream);
    if (OP == OP_JACOBI_RST)
        return fail(MGX_UNSUPPORTED, "the fused restriction needs the vector kernel, no masks");
    if (p0.gamma_in != 0.)
        return fail(MGX_UNSUPPORTED, "scaled first sweep needs the vector kernel");
    PlaneParams p = p0;
    constexpr int S  = stages_for<LAP, OP, R>();
    constexpr int RR = ((LAP == 0) || is_rhs_op(OP)) ? 1 : R;
    constexpr bool STAGE_V = (OP == OP_HPSI_B);
    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    const size_t esz = sizeof(T) + (STAGE_V ? sizeof(TV) : 0);

    bool staged = !force_direct;
    // bulk copies need 16-byte aligned rows and bases
    if ((nz * sizeof(T)) % 16 || (p.ldu * sizeof(T)) % 16
        || ((uintptr_t)p.u % 16))
        staged = false;
    if (STAGE_V && ((nz * sizeof(TV)) % 16 || ((uintptr_t)p.V % 16)))
        staged = false;
    if (nz < 2 * RR + 1 || nx < R) staged = false;
    // rows per tile: as many as the per-thread point budget allows, room for
    // the halo (one wrap at most), shared memory within ~110 KB
    int ty = 0;
    if (staged)
    {
        const size_t smem_cap = 110 * 1024;
        int cand = std::min(32, (256 * PLANE_NP) / nz);
        cand     = std::min(cand, ny - 2 * RR);
        for (; cand >= 1; cand--)
        {
            const size_t sm = (size_t)S * (cand + 2 * RR) * nz * esz + S * 8;
            if (sm <= smem_cap) break;
        }
        ty = cand;
        if (ty < 1 || nz > 256 * PLANE_NP) staged = false;
    }
    if (staged)
    {
        p.ty      = ty;
        p.ntile_y = (ny + ty - 1) / ty;
        // x chunk: enough CTAs to fill the GPU, little halo re-read
        int xc = 32;
        while (xc > 4 && (size_t)p.ntile_y * ((nx + xc - 1) / xc) * nfunc < 4 * 152)
            xc /= 2;
        if (xc > nx) xc = nx;
        p.xc       = xc;
        p.ntile_x  = (nx + xc - 1) / xc;
        const size_t smem = (size_t)S * (ty + 2 * RR) * nz * esz + S * 8;
        auto kern         = plane_kernel<T, TV, LAP, OP, R, S, PLANE_NP>;
        cudaError_t e     = cudaFuncSetAttribute(
            kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return cuda_check(e, "plane_kernel smem attribute");
        dim3 grid(p.ntile_y * p.ntile_x, nfunc);
        kern<<<grid, 256, smem, stream>>>(p, c);
        MGX_LAUNCH_CHECK("plane_kernel");
        return MGX_OK;
    }
    const size_t npts = (size_t)nx * ny * nz;
    int bx            = (int)std::min<size_t>((npts + 255) / 256, 4096);
    dim3 grid(bx, nfunc);
    direct_kernel<T, TV, LAP, OP, R><<<grid, 256, 0, stream>>>(p, c);
    MGX_LAUNCH_CHECK("direct_kernel");
    return MGX_OK;
}

template <typename T, typename TV, int OP>
static int dispatch_lap(int lap_type, const PlaneParams& p, const DevCoef<T>& c,
    int nfunc, cudaStream_t s, int force_direct)
{
    switch (lap_type)
    {
        case 0: return launch_t<T, TV, 0, OP, 1>(p, c, nfunc, s, force_direct);
        case 1: return launch_t<T, TV, 1, OP, 1>(p, c, nfunc, s, force_direct);
        case 2: return launch_t<T, TV, 2, OP, 2>(p, c, nfunc, s, force_direct);
        case 3: return launch_t<T, TV, 3, OP, 3>(p, c, nfunc, s, force_direct);
        case 4: return launch_t<T, TV, 4, OP, 4>(p, c, nfunc, s, force_direct);
    }
    return fail(MGX_BAD_ARG, "lap_type %d invalid", lap_type);
}

int stencil_launch(int op, int lap_type, int dtype, int v_dtype,
    const PlaneParams& p, const Level& L, double jf, int nfunc,
    cudaStream_t stream, int force_direct)
{
    if (nfunc <= 0) return MGX_OK;
    if (nfunc > 65535) return fail(MGX_BAD_ARG, "nfunc %d > 65535 per launch", nfunc);
    {
        const int R = is_rhs_op(op) ? 1 : lap_radius(lap_type);
        for (int i = 0; i < 3; i++)
            if (p.n[i] < R)
                return fail(MGX_BAD_ARG, "grid dimension %d = %d below stencil radius %d",
                    i, p.n[i], R);
    }
    const StencilCoeffs sc = stencil_coeffs(is_rhs_op(op) ? 1 : lap_type, L.h);
    if (op == OP_RHS)
    {
        if (dtype == MGX_F64)
            return launch_t<double, double, 0, OP_RHS, 1>(
                p, to_dev<double>(sc, jf), nfunc, stream, force_direct);
        return launch_t<float, float, 0, OP_RHS, 1>(
            p, to_dev<float>(sc, jf), nfunc, stream, force_direct);
    }
    if (op == OP_RHS_SPLIT)
    {
        // float blocks through the vector kernel only
        if (dtype != MGX_F32 || !vec_ok<float, float, 0, OP_RHS_SPLIT, 1>(p, force_direct)
            || (L.npts() % 64) != 0)
            return fail(MGX_UNSUPPORTED, "split right-hand side needs the vector kernel");
        return launch_vec<float, float, 0, OP_RHS_SPLIT, 1>(p, to_dev<float>(sc, jf), nfunc,
            stream);
    }
    if (op == OP_RHS_SUB)
    {
        if (dtype == MGX_F64)
            return launch_t<double, double, 0, OP_RHS_SUB, 1>(
                p, to_dev<double>(sc, jf), nfunc, stream, force_direct);
        return launch_t<float, float, 0, OP_RHS_SUB, 1>(
            p, to_dev<float>(sc, jf), nfunc, stream, force_direct);
    }
    if (dtype == MGX_F64)
    {
        const DevCoef<double> c = to_dev<double>(sc, jf);
        switch (op)
        {
            case OP_LAP:
                return dispatch_lap<double, double, OP_LAP>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI:
                return dispatch_lap<double, double, OP_JACOBI>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI_UPD:
                return dispatch_lap<double, double, OP_JACOBI_UPD>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI_RST:
                return dispatch_lap<double, double, OP_JACOBI_RST>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_HPSI_B:
                if (p.split_hi != nullptr) return fail(MGX_UNSUPPORTED, "split H psi is FP32 only");
                if (v_dtype == MGX_F64)
                    return launch_t<double, double, 0, OP_HPSI_B, 1>(p, c, nfunc, stream, force_direct);
                return launch_t<double, float, 0, OP_HPSI_B, 1>(p, c, nfunc, stream, force_direct);
            case OP_HPSI_V:
                if (v_dtype == MGX_F64)
                    return dispatch_lap<double, double, OP_HPSI_V>(lap_type, p, c, nfunc, stream, force_direct);
                return dispatch_lap<double, float, OP_HPSI_V>(lap_type, p, c, nfunc, stream, force_direct);
        }
    }
    else
    {
        const DevCoef<float> c = to_dev<float>(sc, jf);
        switch (op)
        {
            case OP_LAP:
                return dispatch_lap<float, float, OP_LAP>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI:
                return dispatch_lap<float, float, OP_JACOBI>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI_UPD:
                return dispatch_lap<float, float, OP_JACOBI_UPD>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_JACOBI_RST:
                return dispatch_lap<float, float, OP_JACOBI_RST>(lap_type, p, c, nfunc, stream, force_direct);
            case OP_HPSI_B:
                if (p.split_hi != nullptr)
                {
                    // the operand planes are written by the vector kernel only
                    if (v_dtype != MGX_F32 || !vec_ok<float, float, 0, OP_HPSI_B, 1>(p, force_direct)
                        || (L.npts() % 64) != 0)
                        return fail(MGX_UNSUPPORTED, "split H psi needs the vector kernel");
                    return launch_vec<float, float, 0, OP_HPSI_B, 1>(p, c, nfunc, stream);
                }
                if (v_dtype == MGX_F64)
                    return launch_t<float, double, 0, OP_HPSI_B, 1>(p, c, nfunc, stream, force_direct);
                return launch_t<float, float, 0, OP_HPSI_B, 1>(p, c, nfunc, stream, force_direct);
            case OP_HPSI_V:
                if (v_dtype == MGX_F64)
                    return dispatch_lap<float, double, OP_HPSI_V>(lap_type, p, c, nfunc, stream, force_direct);
                return dispatch_lap<float, float, OP_HPSI_V>(lap_type, p, c, nfunc, stream, force_direct);
        }
    }
    return fail(MGX_BAD_ARG, "stencil op %d invalid", op);
}

/* ------------------------------------------------------------------ */
/* two Jacobi sweeps in one launch                                      */
/* ------------------------------------------------------------------ */
/* Threads per block of the two-sweep kernel: 256 (two blocks per SM), or
 * 512 (one block per SM, tiles twice as high, so less of the first sweep
 * is re-done on the halo rows) for the pre-sweep pair when 256 threads
 * cannot hold JJ_PAIR_MIN_ROWS rows.  On 192^3 FP32 that pair ran 19.6 ms
 * per 512 orbitals with 512 threads (16 rows) against 23.2 ms with 256 (6
 * rows); the post-sweep pair ran 15.6 against 14.3 ms, so it keeps 256.
 * MGX_JJ_THREADS=256 or 512 sets every launch. */
static int jj_threads()
{
    static const int v = [] {
        const char* e = getenv("MGX_JJ_THREADS");
        const int n   = e ? atoi(e) : 0;
        return (n == 256 || n == 512) ? n : 0;
    }();
    return v;
}

template <typename T, int LAP, int MODE, int NT>
static int launch_jj_nt(const PlaneParams& p0, const DevCoef<T>& c, int nfunc, cudaStream_t stream,
    bool dry, int* tile_rows)
{
    constexpr int S   = 4;
    constexpr int NG1 = 2;
    constexpr int NG2 = 2;
    constexpr int VEC = 16 / sizeof(T);
    constexpr bool RST = ((MODE & 3) == JJ_RST);
    constexpr bool UPD = ((MODE & 3) == JJ_UPD);
    constexpr bool PRO = (MODE & JJ_PRO) != 0;
    constexpr int YO   = RST ? 1 : 0;
    PlaneParams p = p0;
    const int nx = p.n[0], ny = p.n[1], nz = p.n[2];
    if (p.mask.state != nullptr) return fail(MGX_UNSUPPORTED, "two-sweep kernel: masks");
    const bool scaled = (p.gamma_in != 0.);
    if (!p.f || (!scaled && !p.u) || (UPD ? !p.upd : !p.out) || (RST && !p.coarse)
        || (PRO && (!p.pro || scaled)))
        return fail(MGX_BAD_ARG, "two-sweep kernel: null block");
    if (!UPD && (p.out == p.u || p.out == p.f))
        return fail(MGX_BAD_ARG, "two-sweep kernel: out aliases its input");
    if (PRO && ((nx | ny | nz) & 1))
        return fail(MGX_UNSUPPORTED, "the folded prolongation needs even dimensions");
    auto al = [](const void* q, size_t ld) {
        return q == nullptr || (((uintptr_t)q % 16) == 0 && (ld * sizeof(T)) % 16 == 0);
    };
    if ((nz * sizeof(T)) % 16 || !al(p.u, p.ldu) || !al(p.f, p.ldf) || !al(p.out, p.ldo)
        || !al(p.upd, p.ldupd))
        return fail(MGX_UNSUPPORTED, "two-sweep kernel: unaligned block");
    if (RST && (((nx | ny) & 1) || (nz % 4)))
        return fail(MGX_UNSUPPORTED, "the fused restriction needs even x, y and z % 4 == 0");
    if (nx < 3) return fail(MGX_UNSUPPORTED, "two-sweep kernel: nx < 3");
    const int gpr = nz / VEC;
    if (PRO
        && (((nz / 2) * sizeof(T)) % 16 || ((uintptr_t)p.pro % 16) || (p.ldpro * sizeof(T)) % 16))
        return fail(MGX_UNSUPPORTED, "the folded prolongation needs 16-byte coarse rows");
    auto smem_for = [&](int t) {
        return (size_t)S * (t + YO + 4) * nz * sizeof(T) + 2 * (size_t)(t + YO + 2) * nz * sizeof(T)
               + (RST ? 4 * (size_t)(t + 1) * nz * sizeof(T) : 0)
               + (PRO ? (size_t)JJ_CS * ((t + 7) / 2) * (nz / 2) * sizeof(T) : 0) + S * 8;
    };
    // rows per tile: the first sweep's TY + YO + 2 rows and the second's
    // TY + YO within the threads' groups, TY dividing ny (even with the
    // restriction), the staged rows within the grid, shared memory within
    // ~110 KB per block (220 KB for one 512-thread block per SM)
    const size_t smem_cap = NT == 512 ? 220 * 1024 : 110 * 1024;
    int ty = std::min(NG1 * NT / gpr - YO - 2, NG2 * NT / gpr - YO);
    ty     = std::min(ty, ny - YO - 4);
    for (; ty >= 1; ty--)
        if (ny % ty == 0 && (!RST || ty % 2 == 0) && (!PRO || (ty + 7) / 2 <= ny / 2)
            && smem_for(ty) <= smem_cap)
            break;
    if (ty < 1) return fail(MGX_UNSUPPORTED, "two-sweep kernel: no tile height fits");
    if (tile_rows) *tile_rows = ty;
    if (dry) return MGX_OK;
    p.ty      = ty;
    p.ntile_y = ny / ty;
    int xc    = 32;
    while (xc > 4 && (size_t)p.ntile_y * ((nx + xc - 1) / xc) * nfunc < 4 * 152)
        xc /= 2;
    if (xc > nx) xc = nx;
    p.xc      = xc;
    p.ntile_x = (nx + xc - 1) / xc;
    const size_t smem = smem_for(ty);
    auto kern         = plane_jj_kernel<T, LAP, MODE, S, NG1, NG2, NT>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return cuda_check(e, "plane_jj_kernel smem attribute");
    dim3 grid(p.ntile_y * p.ntile_x, nfunc);
    kern<<<grid, NT, smem, stream>>>(p, c);
    MGX_LAUNCH_CHECK("plane_jj_kernel");
    return MGX_OK;
}

template <typename T, int LAP, int MODE>
static int launch_jj(const PlaneParams& p, const DevCoef<T>& c, int nfunc, cudaStream_t stream,
    bool dry, int* tile_rows)
{
    int nt = jj_threads();
    if (nt == 0)
    {
        nt = 256;
        int ty = 0;
        if ((MODE & 3) == JJ_RST
            && launch_jj_nt<T, LAP, MODE, 256>(p, c, nfunc, stream, true, &ty) == MGX_OK
            && ty < JJ_PAIR_MIN_ROWS)
            nt = 512;
    }
    if (nt == 512) return launch_jj_nt<T, LAP, MODE, 512>(p, c, nfunc, stream, dry, tile_rows);
    return launch_jj_nt<T, LAP, MODE, 256>(p, c, nfunc, stream, dry, tile_rows);
}

template <typename T, int LAP>
static int jj_mode(int mode, const PlaneParams& p, const DevCoef<T>& c, int nfunc, cudaStream_t s,
    bool dry, int* ty)
{
    switch (mode)
    {
        case JJ_STORE: return launch_jj<T, LAP, JJ_STORE>(p, c, nfunc, s, dry, ty);
        case JJ_UPD: return launch_jj<T, LAP, JJ_UPD>(p, c, nfunc, s, dry, ty);
        case JJ_RST: return launch_jj<T, LAP, JJ_RST>(p, c, nfunc, s, dry, ty);
        case JJ_STORE | JJ_PRO: return launch_jj<T, LAP, JJ_STORE | JJ_PRO>(p, c, nfunc, s, dry, ty);
        case JJ_UPD | JJ_PRO: return launch_jj<T, LAP, JJ_UPD | JJ_PRO>(p, c, nfunc, s, dry, ty);
    }
    return fail(MGX_BAD_ARG, "two-sweep mode %d", mode);
}

int jacobi2_launch(int mode, int lap_type, int dtype, const PlaneParams& p, const Level& L,
    double jf, int nfunc, cudaStream_t s, bool dry, int* tile_rows)
{
    if (nfunc <= 0) return MGX_OK;
    if (nfunc > 65535) return fail(MGX_BAD_ARG, "nfunc %d > 65535 per launch", nfunc);
    if (lap_type != 0 && lap_type != 1)
        return fail(MGX_UNSUPPORTED, "two-sweep kernel: radius-1 operators only");
    const StencilCoeffs sc = stencil_coeffs(lap_type, L.h);
    if (dtype == MGX_F64)
    {
        const DevCoef<double> c = to_dev<double>(sc, jf);
        return lap_type == 0 ? jj_mode<double, 0>(mode, p, c, nfunc, s, dry, tile_rows)
                             : jj_mode<double, 1>(mode, p, c, nfunc, s, dry, tile_rows);
    }
    if (dtype != MGX_F32) return fail(MGX_BAD_ARG, "two-sweep kernel: dtype %d", dtype);
    const DevCoef<float> c = to_dev<float>(sc, jf);
    return lap_type == 0 ? jj_mode<float, 0>(mode, p, c, nfunc, s, dry, tile_rows)
                         : jj_mode<float, 1>(mode, p, c, nfunc, s, dry, tile_rows);
}

/* ------------------------------------------------------------------ */
/* ghosted drop-in kernels (src/pb/FDkernels.cc, src/pb/MGkernels.cc)   */
/* ------------------------------------------------------------------ */
struct GhostGeom
{
    int n[3];
    int g;
    int incx, incy;
    size_t sizeg;
};

inline GhostGeom ghost_geom(const int n[3], int g)
{
    GhostGeom G;
    for (int i = 0; i < 3; i++)
        G.n[i] = n[i];
    G.g     = g;
    G.incy  = n[2] + 2 * g;
    G.incx  = (n[1] + 2 * g) * G.incy;
    G.sizeg = (size_t)(n[0] + 2 * g) * G.incx;
    return G;
}

template <typename T, int LAP, int R>
__global__ void ghosted_del2_kernel(GhostGeom G, DevCoef<T> c, const T* v, T* b,
    size_t nfunc)
{
    const size_t npts  = (size_t)G.n[0] * G.n[1] * G.n[2];
    const size_t total = npts * nfunc;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t f   = t / npts;
        const size_t idx = t - f * npts;
        const int z      = (int)(idx % G.n[2]);
        const int y      = (int)((idx / G.n[2]) % G.n[1]);
        const int x      = (int)(idx / ((size_t)G.n[2] * G.n[1]));
        const size_t i0  = f * G.sizeg + (size_t)(x + G.g) * G.incx
                          + (size_t)(y + G.g) * G.incy + z + G.g;
        auto at = [&](int dx, int dy, int dz) -> T {
            return v[i0 + (ptrdiff_t)dx * G.incx + (ptrdiff_t)dy * G.incy + dz];
        };
        b[i0] = eval_lap<T, LAP, R>(c, at);
    }
}

template <typename T>
__global__ void ghosted_rhs_kernel(GhostGeom G, GhostGeom O, const T* v, T* rhs,
    size_t nfunc)
{
    const size_t npts  = (size_t)G.n[0] * G.n[1] * G.n[2];
    const size_t total = npts * nfunc;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t f   = t / npts;
        const size_t idx = t - f * npts;
        const int z      = (int)(idx % G.n[2]);
        const int y      = (int)((idx / G.n[2]) % G.n[1]);
        const int x      = (int)(idx / ((size_t)G.n[2] * G.n[1]));
        const size_t i0  = f * G.sizeg + (size_t)(x + G.g) * G.incx
                          + (size_t)(y + G.g) * G.incy + z + G.g;
        auto at = [&](int dx, int dy, int dz) -> T {
            return v[i0 + (ptrdiff_t)dx * G.incx + (ptrdiff_t)dy * G.incy + dz];
        };
        const size_t o0 = f * O.sizeg + (size_t)(x + O.g) * O.incx
                          + (size_t)(y + O.g) * O.incy + z + O.g;
        rhs[o0] = eval_rhs<T>(at);
    }
}

/* periodic ghost fill: every ghost point takes its periodic image */
template <typename T>
__global__ void trade_kernel(GhostGeom G, T* u, size_t nfunc)
{
    const int ex = G.n[0] + 2 * G.g, ey = G.n[1] + 2 * G.g, ez = G.n[2] + 2 * G.g;
    const size_t total = G.sizeg * nfunc;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t f   = t / G.sizeg;
        const size_t idx = t - f * G.sizeg;
        const int z      = (int)(idx % ez);
        const int y      = (int)((idx / ez) % ey);
        const int x      = (int)(idx / ((size_t)ez * ey));
        const int ix = x - G.g, iy = y - G.g, iz = z - G.g;
        if (ix >= 0 && ix < G.n[0] && iy >= 0 && iy < G.n[1] && iz >= 0
            && iz < G.n[2])
            continue;
        const int sx = (ix % G.n[0] + G.n[0]) % G.n[0] + G.g;
        const int sy = (iy % G.n[1] + G.n[1]) % G.n[1] + G.g;
        const int sz = (iz % G.n[2] + G.n[2]) % G.n[2] + G.g;
        u[f * G.sizeg + idx]
            = u[f * G.sizeg + (size_t)sx * G.incx + (size_t)sy * G.incy + sz];
    }
}

static int grid_blocks(size_t total)
{
    return (int)std::min<size_t>((total + 255) / 256, 1u << 20);
}

template <typename T>
static int ghosted_del2_t(const GhostGeom& G, const StencilCoeffs& sc, int lap,
    const void* v, void* b, size_t nfunc, cudaStream_t s)
{
    const DevCoef<T> c = to_dev<T>(sc, 0.);
    const int nb = grid_blocks((size_t)G.n[0] * G.n[1] * G.n[2] * nfunc);
    const T* vv  = (const T*)v;
    T* bb        = (T*)b;
    switch (lap)
    {
        case 0: ghosted_del2_kernel<T, 0, 1><<<nb, 256, 0, s>>>(G, c, vv, bb, nfunc); break;
        case 1: ghosted_del2_kernel<T, 1, 1><<<nb, 256, 0, s>>>(G, c, vv, bb, nfunc); break;
        case 2: ghosted_del2_kernel<T, 2, 2><<<nb, 256, 0, s>>>(G, c, vv, bb, nfunc); break;
        case 3: ghosted_del2_kernel<T, 3, 3><<<nb, 256, 0, s>>>(G, c, vv, bb, nfunc); break;
        case 4: ghosted_del2_kernel<T, 4, 4><<<nb, 256, 0, s>>>(G, c, vv, bb, nfunc); break;
    }
    MGX_LAUNCH_CHECK("ghosted_del2_kernel");
    return MGX_OK;
}

int ghosted_del2(const mgx_grid& g, int ghosts, int lap_type, int dtype,
    const void* v, void* b, size_t nfunc, cudaStream_t s)
{
    const int R = lap_radius(lap_type);
    if (R < 0) return fail(MGX_BAD_ARG, "lap_type %d invalid", lap_type);
    if (ghosts < R)
        return fail(MGX_BAD_ARG, "ghost width %d below operator radius %d", ghosts, R);
    const Level L = make_level(g, 0);
    const StencilCoeffs sc = stencil_coeffs(lap_type, L.h);
    const GhostGeom G = ghost_geom(g.n, ghosts);
    if (dtype == MGX_F64) return ghosted_del2_t<double>(G, sc, lap_type, v, b, nfunc, s);
    return ghosted_del2_t<float>(G, sc, lap_type, v, b, nfunc, s);
}

int ghosted_rhs(const mgx_grid& g, int ghosts, int dtype, const void* v, void* rhs,
    int rhs_ghosts, size_t nfunc, cudaStream_t s)
{
    if (ghosts < 1) return fail(MGX_BAD_ARG, "ghost width must be >= 1");
    if (rhs_ghosts < 0) return fail(MGX_BAD_ARG, "rhs_ghosts < 0");
    const GhostGeom G = ghost_geom(g.n, ghosts), O = ghost_geom(g.n, rhs_ghosts);
    const int nb = grid_blocks((size_t)g.n[0] * g.n[1] * g.n[2] * nfunc);
    if (dtype == MGX_F64)
        ghosted_rhs_kernel<double><<<nb, 256, 0, s>>>(G, O, (const double*)v, (double*)rhs, nfunc);
    else
        ghosted_rhs_kernel<float><<<nb, 256, 0, s>>>(G, O, (const float*)v, (float*)rhs, nfunc);
    MGX_LAUNCH_CHECK("ghosted_rhs_kernel");
    return MGX_OK;
}

int ghosted_trade(const mgx_grid& g, int ghosts, int dtype, void* u, size_t nfunc,
    cudaStream_t s)
{
    if (ghosts < 1) return MGX_OK;
    for (int i = 0; i < 3; i++)
        if (g.n[i] < ghosts)
            return fail(MGX_BAD_ARG, "dimension %d smaller than ghost width", i);
    const GhostGeom G = ghost_geom(g.n, ghosts);
    const int nb      = grid_blocks(G.sizeg * nfunc);
    if (dtype == MGX_F64)
        trade_kernel<double><<<nb, 256, 0, s>>>(G, (double*)u, nfunc);
    else
        trade_kernel<float><<<nb, 256, 0, s>>>(G, (float*)u, nfunc);
    MGX_LAUNCH_CHECK("trade_kernel");
    return MGX_OK;
}

} // namespace mgx
