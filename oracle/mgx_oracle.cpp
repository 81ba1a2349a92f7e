/*
 * ORACLE -- TEST INFRASTRUCTURE ONLY.
 *
 * A CPU restatement, in plain C++ loops, of the MGmol orbital hot path:
 * finite-difference stencils, multigrid transfers, the block V-cycle used as
 * the orbital preconditioner, the local Hamiltonian, localization masks and
 * the Gram / H-matrix contractions with their FP64 Cholesky, inverse and trace.
 *
 * It is the checker for the CUDA product in mgmol_gb300/csrc.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.  The
 * product never calls it and has no CPU fallback.
 *
 * Every routine cites the reference file:line whose behaviour it restates
 * (paths relative to the MGmol source tree).  The restatement keeps the
 * reference's operation order (double accumulation of float data, sums of
 * pairs formed in the storage type, casts at the same places) so that the
 * float instantiation matches the reference bit-for-bit when both are built
 * with -ffp-contract=off.  Pinning: oracle/build_ref.sh compiles the
 * reference's own translation units against single-rank shims into
 * oracle/_ref/, and tests/golden/make_golden.py records their outputs as
 * fixtures that tests/test_oracle.py compares this file against.
 *
 * Scope: periodic boundary conditions in all three directions, one MPI task,
 * one x-subdomain (subdivx = 1), each orbital its own colour.
 */
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace orc
{

/* Grid geometry: n interior points per direction, ll the domain lengths,
 * ng ghost layers.  h = ll / n, as pb::Grid::Grid (src/pb/Grid.cc:72-76).
 * Ghosted storage is x-slowest, z-fastest (src/pb/Grid.cc:80-82). */
struct Grid
{
    int n[3];
    double ll[3];
    int ng;

    double h(int i) const { return ll[i] / (double)n[i]; }
    int incy() const { return n[2] + 2 * ng; }
    int incx() const { return (n[1] + 2 * ng) * (n[2] + 2 * ng); }
    size_t sizeg() const { return (size_t)(n[0] + 2 * ng) * (size_t)incx(); }
    size_t size() const { return (size_t)n[0] * n[1] * n[2]; }
    double vel() const { return h(0) * h(1) * h(2); }
    /* pb::Grid::coarse_grid (src/pb/Grid.cc:214-231): half the points, same
     * lattice, same ghost count. */
    Grid coarse() const
    {
        Grid c = *this;
        for (int i = 0; i < 3; i++)
            c.n[i] = n[i] / 2;
        return c;
    }
    Grid with_ghosts(int g) const
    {
        Grid c = *this;
        c.ng   = g;
        return c;
    }
};

static const double inv12 = 1. / 12.;
static const double inv64 = 1. / 64.;

/* Ghost width per operator, src/GridFactory.h:19-51. */
static int ghosts_for(int lap_type)
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

/* ------------------------------------------------------------------ */
/* Ghost fill, one task, periodic: GridFuncVector::trade_boundaries     */
/* (src/pb/GridFuncVector.cc:1543-1621) with the single-task wraps of   */
/* finishNorthSouthComm (:586-604, Y: interior x, interior z),          */
/* finishUpDownComm (:1052-1068, Z: interior x, all y) and              */
/* finishEastWestComm (:1423-1437, X: whole planes).                    */
/* ------------------------------------------------------------------ */
template <typename T>
void trade(const Grid& g, T* u, int nfunc)
{
    const int ng = g.ng, nx = g.n[0], ny = g.n[1], nz = g.n[2];
    const int incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
    for (int f = 0; f < nfunc; f++)
    {
        T* pu = u + (size_t)f * sg;
        for (int ix = ng; ix < nx + ng; ix++)
            for (int j = 0; j < ng; j++)
            {
                memcpy(&pu[ix * incx + j * incy + ng],
                    &pu[ix * incx + (j + ny) * incy + ng], nz * sizeof(T));
                memcpy(&pu[ix * incx + (ny + ng + j) * incy + ng],
                    &pu[ix * incx + (ng + j) * incy + ng], nz * sizeof(T));
            }
        for (int ix = ng; ix < nx + ng; ix++)
            for (int iy = 0; iy < ny + 2 * ng; iy++)
            {
                T* row = &pu[ix * incx + iy * incy];
                for (int j = 0; j < ng; j++)
                {
                    row[j]           = row[j + nz];
                    row[nz + ng + j] = row[ng + j];
                }
            }
        for (int j = 0; j < ng; j++)
        {
            memcpy(&pu[j * incx], &pu[(j + nx) * incx], incx * sizeof(T));
            memcpy(&pu[(nx + ng + j) * incx], &pu[(ng + j) * incx],
                incx * sizeof(T));
        }
    }
}

/* ------------------------------------------------------------------ */
/* FD kernels on ghosted blocks, src/pb/FDkernels.cc                    */
/* ------------------------------------------------------------------ */

/* FDkernelDel2_2nd, src/pb/FDkernels.cc:18-75 */
template <typename T>
void del2_2nd(const Grid& g, const T* v, T* b, int nfunc)
{
    const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
        1. / (g.h(2) * g.h(2)) };
    const double c1x = -ih[0], c1y = -ih[1], c1z = -ih[2];
    const double c0  = -2. * (c1x + c1y + c1z);
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                {
                    size_t i = f * sg + (size_t)((ix + ng) * incx
                                                 + (iy + ng) * incy + iz + ng);
                    b[i] = c0 * v[i] + c1x * (v[i - incx] + v[i + incx])
                           + c1y * (v[i - incy] + v[i + incy])
                           + c1z * (v[i - 1] + v[i + 1]);
                }
}

/* FDkernelDel2_4th, src/pb/FDkernels.cc:77-162 */
template <typename T>
void del2_4th(const Grid& g, const T* A, T* B, int nfunc)
{
    const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
        1. / (g.h(2) * g.h(2)) };
    const double cc0 = inv12 * ih[0], c1x = -16. * cc0, c2x = 1. * cc0;
    const double cc1 = inv12 * ih[1], c1y = -16. * cc1, c2y = 1. * cc1;
    const double cc2 = inv12 * ih[2], c1z = -16. * cc2, c2z = 1. * cc2;
    const double c0  = -2. * (c1x + c2x + c1y + c2y + c1z + c2z);
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const int incx2 = 2 * incx, incy2 = 2 * incy;
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                {
                    const T* v = A + f * sg
                                 + (size_t)((ix + ng) * incx + (iy + ng) * incy
                                            + iz + ng);
                    B[v - A] = c0 * (double)v[0]
                               + c1x * ((double)v[-incx] + (double)v[incx])
                               + c1y * ((double)v[-incy] + (double)v[incy])
                               + c1z * ((double)v[-1] + (double)v[1])
                               + c2x * ((double)v[-incx2] + (double)v[incx2])
                               + c2y * ((double)v[-incy2] + (double)v[incy2])
                               + c2z * ((double)v[-2] + (double)v[2]);
                }
}

/* FDkernelDel2_6th, src/pb/FDkernels.cc:255-344 */
template <typename T>
void del2_6th(const Grid& g, const T* v, T* u, int nfunc)
{
    const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
        1. / (g.h(2) * g.h(2)) };
    double cc        = (1. / 180.) * ih[0];
    const double c1x = -270. * cc, c2x = 27. * cc, c3x = -2. * cc;
    cc               = (1. / 180.) * ih[1];
    const double c1y = -270. * cc, c2y = 27. * cc, c3y = -2. * cc;
    cc               = (1. / 180.) * ih[2];
    const double c1z = -270. * cc, c2z = 27. * cc, c3z = -2. * cc;
    const double c0
        = -2. * (c1x + c2x + c3x + c1y + c2y + c3y + c1z + c2z + c3z);
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                {
                    size_t i = f * sg + (size_t)((ix + ng) * incx
                                                 + (iy + ng) * incy + iz + ng);
                    u[i] = (T)(c0 * (double)v[i]
                               + c1x * ((double)v[i - incx] + (double)v[i + incx])
                               + c1y * ((double)v[i - incy] + (double)v[i + incy])
                               + c1z * ((double)v[i - 1] + (double)v[i + 1])
                               + c2x * ((double)v[i - 2 * incx]
                                          + (double)v[i + 2 * incx])
                               + c2y * ((double)v[i - 2 * incy]
                                          + (double)v[i + 2 * incy])
                               + c2z * ((double)v[i - 2] + (double)v[i + 2])
                               + c3x * ((double)v[i - 3 * incx]
                                          + (double)v[i + 3 * incx])
                               + c3y * ((double)v[i - 3 * incy]
                                          + (double)v[i + 3 * incy])
                               + c3z * ((double)v[i - 3] + (double)v[i + 3]));
                }
}

/* FDkernelDel2_8th, src/pb/FDkernels.cc:346-445 */
template <typename T>
void del2_8th(const Grid& g, const T* v, T* u, int nfunc)
{
    const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
        1. / (g.h(2) * g.h(2)) };
    double cc        = (1. / 5040.) * ih[0];
    const double c1x = -8064. * cc, c2x = 1008. * cc, c3x = -128. * cc,
                 c4x = 9. * cc;
    cc               = (1. / 5040.) * ih[1];
    const double c1y = -8064. * cc, c2y = 1008. * cc, c3y = -128. * cc,
                 c4y = 9. * cc;
    cc               = (1. / 5040.) * ih[2];
    const double c1z = -8064. * cc, c2z = 1008. * cc, c3z = -128. * cc,
                 c4z = 9. * cc;
    const double c0 = -2.
                      * (c1x + c2x + c3x + c4x + c1y + c2y + c3y + c4y + c1z
                          + c2z + c3z + c4z);
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                {
                    size_t i = f * sg + (size_t)((ix + ng) * incx
                                                 + (iy + ng) * incy + iz + ng);
                    u[i] = (T)(c0 * (double)v[i]
                               + c1x * ((double)v[i - incx] + (double)v[i + incx])
                               + c1y * ((double)v[i - incy] + (double)v[i + incy])
                               + c1z * ((double)v[i - 1] + (double)v[i + 1])
                               + c2x * ((double)v[i - 2 * incx]
                                          + (double)v[i + 2 * incx])
                               + c2y * ((double)v[i - 2 * incy]
                                          + (double)v[i + 2 * incy])
                               + c2z * ((double)v[i - 2] + (double)v[i + 2])
                               + c3x * ((double)v[i - 3 * incx]
                                          + (double)v[i + 3 * incx])
                               + c3y * ((double)v[i - 3 * incy]
                                          + (double)v[i + 3 * incy])
                               + c3z * ((double)v[i - 3] + (double)v[i + 3])
                               + c4x * ((double)v[i - 4 * incx]
                                          + (double)v[i + 4 * incx])
                               + c4y * ((double)v[i - 4 * incy]
                                          + (double)v[i + 4 * incy])
                               + c4z * ((double)v[i - 4] + (double)v[i + 4]));
                }
}

/* FDkernelDel2_4th_Mehr, src/pb/FDkernels.cc:447-520 */
template <typename T>
void del2_mehr(const Grid& g, const T* v, T* u, int nfunc)
{
    const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
        1. / (g.h(2) * g.h(2)) };
    const double c0  = 16. * inv12 * (ih[0] + ih[1] + ih[2]);
    const double cx  = -10. * inv12 * ih[0] + 0.125 * c0;
    const double cy  = -10. * inv12 * ih[1] + 0.125 * c0;
    const double cz  = -10. * inv12 * ih[2] + 0.125 * c0;
    const double cxy = -inv12 * (ih[0] + ih[1]);
    const double cyz = -inv12 * (ih[2] + ih[1]);
    const double cxz = -inv12 * (ih[0] + ih[2]);
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
            {
                const size_t i0 = f * sg
                                  + (size_t)((ix + ng) * incx + (iy + ng) * incy
                                             + ng);
                T* u0          = u + i0;
                const T* v0    = v + i0;
                const T* vmx   = v0 - incx;
                const T* vpx   = v0 + incx;
                const T* vmxmy = vmx - incy;
                const T* vpxmy = vpx - incy;
                const T* vmy   = v0 - incy;
                const T* vpy   = v0 + incy;
                const T* vmxpy = vmx + incy;
                const T* vpxpy = vpx + incy;
                for (int iz = 0; iz < g.n[2]; iz++)
                {
                    u0[iz] = (T)(c0 * (double)v0[iz]
                                 + cz * (double)(v0[iz - 1] + v0[iz + 1])
                                 + cy * (double)(vmy[iz] + vpy[iz])
                                 + cx * (double)(vmx[iz] + vpx[iz])
                                 + cxz
                                       * (double)(vmx[iz - 1] + vmx[iz + 1]
                                                  + vpx[iz - 1] + vpx[iz + 1])
                                 + cyz
                                       * (double)(vmy[iz - 1] + vmy[iz + 1]
                                                  + vpy[iz - 1] + vpy[iz + 1])
                                 + cxy
                                       * (double)(vmxmy[iz] + vpxmy[iz]
                                                  + vmxpy[iz] + vpxpy[iz]));
                }
            }
}

/* FDkernelRHS_4th_Mehr1, src/pb/FDkernels.cc:522-584, output ghosted with
 * the same ghost width as the input (GridFuncVector::rhs_4th_Mehr1,
 * src/pb/GridFuncVector.h:331-339). */
template <typename T>
void rhs_mehr1(const Grid& g, const T* v, T* rhs, int nfunc)
{
    const double c0 = 0.5, c1 = inv12;
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    const size_t sg = g.sizeg();
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
            {
                const size_t i0 = f * sg
                                  + (size_t)((ix + ng) * incx + (iy + ng) * incy
                                             + ng);
                T* u0         = rhs + i0;
                const T* v0   = v + i0;
                const T* vmx  = v0 - incx;
                const T* vpx  = v0 + incx;
                const T* vmy  = v0 - incy;
                const T* vpy  = v0 + incy;
                for (int iz = 0; iz < g.n[2]; iz++)
                    u0[iz] = (T)(c0 * (double)v0[iz]
                                 + c1
                                       * (double)(vmx[iz] + vpx[iz] + vmy[iz]
                                                  + vpy[iz] + v0[iz - 1]
                                                  + v0[iz + 1]));
            }
}

/* GridFuncVector::applyLap dispatch, src/pb/GridFuncVector.cc:2369-2397 */
template <typename T>
void apply_lap(int type, const Grid& g, const T* v, T* out, int nfunc)
{
    switch (type)
    {
        case 0: del2_mehr(g, v, out, nfunc); break;
        case 1: del2_2nd(g, v, out, nfunc); break;
        case 2: del2_4th(g, v, out, nfunc); break;
        case 3: del2_6th(g, v, out, nfunc); break;
        case 4: del2_8th(g, v, out, nfunc); break;
        default: abort();
    }
}

/* ------------------------------------------------------------------ */
/* MG transfer kernels, src/pb/MGkernels.cc                             */
/* ------------------------------------------------------------------ */

/* MGkernelRestrict3D, src/pb/MGkernels.cc:203-283 */
template <typename T>
void restrict3d(const Grid& fg, const T* fine, const Grid& cg, T* coarse,
    int nfunc)
{
    const int incxf = fg.incx(), incyf = fg.incy();
    const int incxc = cg.incx(), incyc = cg.incy();
    const int ngf = fg.ng, ngc = cg.ng;
#pragma omp parallel for collapse(2)
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < cg.n[0]; ix++)
            for (int iy = 0; iy < cg.n[1]; iy++)
            {
                const T* u0 = fine + f * fg.sizeg()
                              + (size_t)((ngf + 2 * ix) * incxf
                                         + (ngf + 2 * iy) * incyf + ngf);
                const T* umx   = u0 - incxf;
                const T* upx   = u0 + incxf;
                const T* umy   = u0 - incyf;
                const T* upy   = u0 + incyf;
                const T* umxpy = u0 - incxf + incyf;
                const T* upxpy = u0 + incxf + incyf;
                const T* umxmy = u0 - incxf - incyf;
                const T* upxmy = u0 + incxf - incyf;
                T* c           = coarse + f * cg.sizeg()
                       + (size_t)((ngc + ix) * incxc + (ngc + iy) * incyc + ngc);
                for (int iz = 0; iz < cg.n[2]; iz++)
                {
                    const int t = 2 * iz;
                    double face = (double)upx[t] + (double)umx[t]
                                  + (double)upy[t] + (double)umy[t]
                                  + (double)u0[t - 1] + (double)u0[t + 1];
                    double corner = (double)upxpy[t - 1] + (double)upxpy[t + 1]
                                    + (double)upxmy[t - 1] + (double)upxmy[t + 1]
                                    + (double)umxpy[t - 1] + (double)umxpy[t + 1]
                                    + (double)umxmy[t - 1]
                                    + (double)umxmy[t + 1];
                    double edge = (double)upy[t - 1] + (double)upy[t + 1]
                                  + (double)umy[t - 1] + (double)umy[t + 1]
                                  + (double)upx[t - 1] + (double)upx[t + 1]
                                  + (double)umx[t - 1] + (double)umx[t + 1]
                                  + (double)umxmy[t] + (double)upxmy[t]
                                  + (double)umxpy[t] + (double)upxpy[t];
                    c[iz] = (T)(inv64
                                * (8. * u0[t] + 4. * face + 2. * edge + corner));
                }
            }
}

/* MGkernelExtend3D, src/pb/MGkernels.cc:28-201: injection of the coarse
 * values (first high-side ghost included) at even fine points, then the
 * 1-D, 2-D and 3-D averages at odd points. */
template <typename T>
void extend3d(const Grid& cg, const T* coarse, const Grid& fg, T* fine,
    int nfunc)
{
    const int incxf = fg.incx(), incyf = fg.incy();
    const int incxc = cg.incx(), incyc = cg.incy();
    const int ngf = fg.ng, ngc = cg.ng;
    const int dimx = fg.n[0], dimy = fg.n[1], dimz = fg.n[2];
    for (int f = 0; f < nfunc; f++)
    {
        T* fd       = fine + f * fg.sizeg();
        const T* cd = coarse + f * cg.sizeg();
        for (int ix = 0; ix <= cg.n[0]; ix++)
            for (int iy = 0; iy <= cg.n[1]; iy++)
                for (int iz = 0; iz <= cg.n[2]; iz++)
                    fd[incxf * (2 * ix + ngf) + incyf * (2 * iy + ngf) + ngf
                        + 2 * iz]
                        = cd[incxc * (ix + ngc) + incyc * (iy + ngc) + ngc + iz];
        for (int ix = ngf; ix < dimx + ngf; ix += 2)
        {
            const int ifx = incxf * ix;
            for (int iy = ngf; iy < dimy + ngf; iy += 2)
            {
                const int ify = ifx + incyf * iy;
                for (int iz = ngf + 1; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i]       = 0.5 * (fd[i - 1] + fd[i + 1]);
                }
            }
            for (int iy = ngf + 1; iy < dimy + ngf; iy += 2)
            {
                const int ify = ifx + incyf * iy;
                for (int iz = ngf; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i]       = 0.5 * (fd[i + incyf] + fd[i - incyf]);
                }
                for (int iz = ngf + 1; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i] = 0.25
                            * (fd[i + 1 + incyf] + fd[i + 1 - incyf]
                                + fd[i - 1 + incyf] + fd[i - 1 - incyf]);
                }
            }
        }
        for (int ix = ngf + 1; ix < dimx + ngf; ix += 2)
        {
            const int ifx = incxf * ix;
            for (int iy = ngf; iy < dimy + ngf; iy += 2)
            {
                const int ify = ifx + incyf * iy;
                for (int iz = ngf + 1; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i] = 0.25
                            * (fd[i + incxf + 1] + fd[i + incxf - 1]
                                + fd[i - incxf + 1] + fd[i - incxf - 1]);
                }
                for (int iz = ngf; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i]       = 0.5 * (fd[i + incxf] + fd[i - incxf]);
                }
            }
            for (int iy = ngf + 1; iy < dimy + ngf; iy += 2)
            {
                const int ify = ifx + incyf * iy;
                for (int iz = ngf + 1; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i]       = 0.125
                            * (fd[i + incxf + incyf + 1] + fd[i + incxf + incyf - 1]
                                + fd[i + incxf - incyf + 1]
                                + fd[i + incxf - incyf - 1]
                                + fd[i - incxf + incyf + 1]
                                + fd[i - incxf + incyf - 1]
                                + fd[i - incxf - incyf + 1]
                                + fd[i - incxf - incyf - 1]);
                }
                for (int iz = ngf; iz < dimz + ngf; iz += 2)
                {
                    const int i = ify + iz;
                    fd[i]       = 0.25
                            * (fd[i + incxf + incyf] + fd[i + incxf - incyf]
                                + fd[i - incxf + incyf] + fd[i - incxf - incyf]);
                }
            }
        }
    }
}

/* LinearAlgebraUtils<Host>::MPaxpy, src/linear_algebra/mputils.cc:222-244:
 * y += (T)(alpha * (double)x) over n entries. */
template <typename T>
void mpaxpy(size_t n, double alpha, const T* x, T* y)
{
#pragma omp parallel for
    for (long k = 0; k < (long)n; k++)
        y[k] += static_cast<T>(alpha * static_cast<double>(x[k]));
}

/* ------------------------------------------------------------------ */
/* Localization masks: GridMask::init (src/GridMask.cc:120-264),        */
/* SubCell::spherePossibleOverlap (src/SubCell.cc:74-95),               */
/* Vector3D::minimage / vminimage (src/tools/Vector3D.cc:13-60),        */
/* MasksSet mask functions (src/MasksSet.cc:16-48).                     */
/* ------------------------------------------------------------------ */
static const double r1               = 0.99999;
static const double inv_one_minus_r1 = 1. / (1. - r1);
static const double rc_exp2          = 0.75;
static const double fac_exp2 = 2. * (1. / (1. - rc_exp2)) * (1. / (1. - rc_exp2));

template <typename M>
M mask_one(const double r)
{
    if (r < r1) return 1.;
    return (M)((1. - r) * inv_one_minus_r1);
}

template <typename M>
M mask_gaussian_decay(const double r)
{
    const double exp2_rc    = exp(-fac_exp2 * (1. - rc_exp2) * (1. - rc_exp2));
    const double exp2_coeff = 1. / (1. - exp2_rc);
    float val               = 1.;
    if (r > rc_exp2)
        val = (exp(-fac_exp2 * (r - rc_exp2) * (r - rc_exp2)) - exp2_rc)
              * exp2_coeff;
    return (M)val;
}

static double minimage(const double x[3], const double c[3], const double l[3])
{
    double d[3];
    for (int i = 0; i < 3; i++)
        d[i] = x[i] - c[i];
    for (int i = 0; i < 3; i++)
        d[i] = remainder(d[i], l[i]);
    return sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
}

/* Per-level point coordinates along one axis, formed by repeated addition
 * of the level spacing as GridMask::init does (src/GridMask.cc:190-234). */
static void level_coords(double start, double hl, int n, double* out)
{
    double xc = start;
    for (int i = 0; i < n; i++)
    {
        out[i] = xc;
        xc += hl;
    }
}

/* GridMask::init for iloc = 0 (one subdomain), periodic bcPoisson.
 * fine: the mesh grid (its ghost count enters delta, src/GridMask.cc:42-45).
 * Writes the level's mask values (x-slowest, z-fastest) and returns the
 * subdomain state of src/GridMask.h:47-52: -1 void, 0 all zero, 1 all one,
 * 2 values. */
template <typename M>
int mask_init(const Grid& fine, int level, const double center[3], double rcut,
    int func, M* out)
{
    const int nx = fine.n[0] >> level, ny = fine.n[1] >> level,
              nz = fine.n[2] >> level;
    const size_t size = (size_t)nx * ny * nz;
    for (size_t i = 0; i < size; i++)
        out[i] = 0;
    const double h[3] = { fine.h(0), fine.h(1), fine.h(2) };
    double delta      = sqrt(h[0] * h[0] + h[1] * h[1] + h[2] * h[2]) + 1.e-8;
    delta *= (double)fine.ng;
    for (int l = 0; l < level; l++)
        delta *= 2.;
    const double overlap_radius = rcut + delta;

    /* SubCell of this level (src/SubCell.cc:14-72) and its overlap test */
    double hs[3] = { h[0], h[1], h[2] };
    for (int l = 0; l < level; l++)
        for (int i = 0; i < 3; i++)
            hs[i] *= 2.;
    const double start[3] = { 0., 0., 0. };
    const int dims[3]     = { nx, ny, nz };
    double subdim[3], cell_center[3];
    for (int i = 0; i < 3; i++)
    {
        subdim[i]      = (dims[i] - 1) * hs[i];
        cell_center[i] = start[i] + 0.5 * subdim[i];
    }
    cell_center[0] += 0 * dims[0] * hs[0];
    {
        double vd[3];
        for (int i = 0; i < 3; i++)
        {
            const double d = cell_center[i] - center[i];
            double r       = fmod(d, fine.ll[i]);
            const double ax2 = 0.5 * fine.ll[i];
            if (r > ax2)
                r -= fine.ll[i];
            else if (r < -ax2)
                r += fine.ll[i];
            vd[i] = r;
        }
        for (int i = 0; i < 3; i++)
        {
            const double vc = vd[i] < 0. ? std::max(-0.5 * subdim[i], vd[i])
                                         : std::min(0.5 * subdim[i], vd[i]);
            vd[i] -= vc;
        }
        const double dcenter = sqrt(vd[0] * vd[0] + vd[1] * vd[1] + vd[2] * vd[2]);
        if (!(dcenter <= overlap_radius)) return -1;
    }
    if (100. < rcut) return 1;

    const double rc_inv   = 1. / rcut;
    const double hl[3]    = { fine.h(0) * (1 << level), fine.h(1) * (1 << level),
        fine.h(2) * (1 << level) };
    std::vector<double> cx(nx), cy(ny), cz(nz);
    level_coords(start[0] + 0 * nx * hl[0], hl[0], nx, cx.data());
    level_coords(start[1], hl[1], ny, cy.data());
    level_coords(start[2], hl[2], nz, cz.data());
    long icount = 0, ncount = 0;
    M* pmask    = out;
    for (int ix = 0; ix < nx; ix++)
        for (int iy = 0; iy < ny; iy++)
            for (int iz = 0; iz < nz; iz++)
            {
                const double xc[3] = { cx[ix], cy[iy], cz[iz] };
                const double r     = minimage(xc, center, fine.ll);
                if (r < overlap_radius)
                {
                    icount++;
                    if (r <= rcut)
                    {
                        *pmask = func == 0 ? mask_gaussian_decay<M>(r * rc_inv)
                                           : mask_one<M>(r * rc_inv);
                        ncount++;
                    }
                    else
                        *pmask = 0;
                }
                pmask++;
            }
    if (level == 0) icount = std::max(1L, icount);
    if (ncount == 0 && icount == 0) return -1;
    if (ncount == 0) return 0;
    return 2;
}

/* GridMaskMax::applyPrivate (src/GridMaskMax.cc:33-87) and
 * GridMaskMult::applyPrivate (src/GridMaskMult.cc:31-89) on the interior
 * of one ghosted function.  kind 0 = Max (clamp), 1 = Mult. */
template <typename T, typename M>
void mask_apply(const Grid& g, T* u, int state, const M* mask, int kind)
{
    if (state == 1) return;
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    for (int ix = 0; ix < g.n[0]; ix++)
        for (int iy = 0; iy < g.n[1]; iy++)
        {
            T* pu      = u + (ix + ng) * incx + (iy + ng) * incy + ng;
            const M* m = mask + ((size_t)ix * g.n[1] + iy) * g.n[2];
            for (int iz = 0; iz < g.n[2]; iz++)
            {
                if (state <= 0)
                    pu[iz] = 0;
                else if (kind == 0)
                {
                    const T uu = pu[iz];
                    const M mm = m[iz];
                    if (uu > mm)
                        pu[iz] = (T)mm;
                    else if (uu < -mm)
                        pu[iz] = -(T)mm;
                }
                else
                    pu[iz] *= (T)m[iz];
            }
        }
}

/* Masks for every orbital and level, applied like GridFuncVector::app_mask
 * (src/pb/GridFuncVector.cc:2427-2438) through Map2Masks::apply
 * (src/Map2Masks.cc:26-61). */
template <typename M>
struct MaskSet
{
    int nlevels = 0;
    int kind    = 0;
    std::vector<std::vector<int>> state; // [level][orbital]
    std::vector<std::vector<std::vector<M>>> values; // [level][orbital][pt]
};

template <typename T, typename M>
void app_mask(const Grid& g, T* u, int nfunc, const MaskSet<M>* ms, int level)
{
    if (ms == nullptr) return;
#pragma omp parallel for
    for (int f = 0; f < nfunc; f++)
        mask_apply(g, u + (size_t)f * g.sizeg(), ms->state[level][f],
            ms->values[level][f].data(), ms->kind);
}

/* ------------------------------------------------------------------ */
/* Block V-cycle, Preconditioning<T>::mg (src/Preconditioning.cc:155-216) */
/* with GridFuncVector::jacobi (src/pb/GridFuncVector.cc:2415-2425).    */
/* ------------------------------------------------------------------ */
template <typename T, typename M>
struct Precond
{
    int maxlevels;
    std::vector<Grid> grids;
    std::vector<double> jf;
    std::vector<std::vector<T>> work, rcoarse, newv;
    const MaskSet<M>* masks = nullptr;
    int nfunc;

    /* Preconditioning::Preconditioning + setup (src/Preconditioning.cc:15-28,
     * 98-151): fine-level factor from the fine operator, Laph2 factors on the
     * coarse grids, coarse grids keep the fine ghost count. */
    Precond(const Grid& fine, int lap_type, int maxl, int nf)
        : maxlevels(maxl), nfunc(nf)
    {
        grids.push_back(fine);
        jf.push_back(jacobi_factor(lap_type, fine));
        for (int l = 1; l <= maxl; l++)
        {
            grids.push_back(grids.back().coarse());
            jf.push_back(jacobi_factor(1, grids.back()));
        }
        for (int l = 0; l <= maxl; l++)
        {
            work.emplace_back((size_t)nf * grids[l].sizeg(), (T)0);
            if (l < maxl)
            {
                rcoarse.emplace_back((size_t)nf * grids[l + 1].sizeg(), (T)0);
                newv.emplace_back((size_t)nf * grids[l + 1].sizeg(), (T)0);
            }
        }
    }

    /* jacobiFactor() of Laph4M / Laph2 / Laph4 / Laph6 / Laph8
     * (src/pb/Laph4M.h:29-31,80; Laph2.h:32-34,95; Laph4.h:35,106;
     * Laph6.h:40,101; Laph8.h:40-42,100), FDoper inv_h2 from
     * src/pb/FDoper.cc:60. */
    static double jacobi_factor(int lap_type, const Grid& g)
    {
        double s = 0.;
        for (int i = 0; i < 3; i++)
            s += 1. / (g.h(i) * g.h(i));
        const double ih0 = 1. / (g.h(0) * g.h(0)), ih1 = 1. / (g.h(1) * g.h(1)),
                     ih2 = 1. / (g.h(2) * g.h(2));
        switch (lap_type)
        {
            case 0: return 1. / ((4. / 3.) * (ih0 + ih1 + ih2));
            case 1: return 6. * (1. / (2. * (ih0 + ih1 + ih2))) / 7.;
            case 2: return (1. / (2.5 * (ih0 + ih1 + ih2))) / 1.5;
            case 3: return (1. / ((49. / 18.) * (ih0 + ih1 + ih2))) / 1.5;
            case 4: return (1. / ((1435. / 504.) * (ih0 + ih1 + ih2))) / 1.5;
        }
        (void)s;
        return 0.;
    }

    void jacobi(int type, int level, T* v, const T* f, T* w)
    {
        const Grid& g = grids[level];
        trade(g, v, nfunc);
        apply_lap(type, g, v, w, nfunc);
        const size_t n = (size_t)nfunc * g.sizeg();
        mpaxpy(n, -1., f, w);
        mpaxpy(n, -1. * jf[level], w, v);
    }

    void mg(T* v, const T* f, int lap_type, int level)
    {
        const Grid& g = grids[level];
        const int ncycl = (level == maxlevels) ? 4 : 2;
        T* w = work[level].data();
        for (int it = 0; it < ncycl; it++)
        {
            jacobi(lap_type, level, v, f, w);
            app_mask(g, v, nfunc, masks, level);
        }
        if (level == maxlevels) return;
        app_mask(g, w, nfunc, masks, level);
        T* rc = rcoarse[level].data();
        trade(g, w, nfunc);
        restrict3d(g, w, grids[level + 1], rc, nfunc);
        app_mask(grids[level + 1], rc, nfunc, masks, level + 1);
        T* nv = newv[level].data();
        std::fill(newv[level].begin(), newv[level].end(), (T)0);
        mg(nv, rc, 1, level + 1);
        trade(grids[level + 1], nv, nfunc);
        extend3d(grids[level + 1], nv, g, w, nfunc);
        app_mask(g, w, nfunc, masks, level);
        mpaxpy((size_t)nfunc * g.sizeg(), -1., w, v);
        for (int it = 0; it < 2; it++)
        {
            jacobi(lap_type, level, v, f, w);
            app_mask(g, v, nfunc, masks, level);
        }
    }
};

/* ghost-free (x-slowest, z-fastest, leading dimension ld) <-> ghosted */
template <typename S, typename T>
void to_ghosted(const Grid& g, const S* src, size_t ld, T* dst, int nfunc)
{
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                    dst[f * g.sizeg() + (ix + ng) * incx + (iy + ng) * incy + iz
                        + ng]
                        = (T)src[f * ld + ((size_t)ix * g.n[1] + iy) * g.n[2]
                                 + iz];
}
template <typename S, typename T>
void from_ghosted(const Grid& g, const S* src, T* dst, size_t ld, int nfunc)
{
    const int ng = g.ng, incx = g.incx(), incy = g.incy();
    for (int f = 0; f < nfunc; f++)
        for (int ix = 0; ix < g.n[0]; ix++)
            for (int iy = 0; iy < g.n[1]; iy++)
                for (int iz = 0; iz < g.n[2]; iz++)
                    dst[f * ld + ((size_t)ix * g.n[1] + iy) * g.n[2] + iz]
                        = (T)src[f * g.sizeg() + (ix + ng) * incx
                                 + (iy + ng) * incy + iz + ng];
}

} // namespace orc

using namespace orc;

static Grid make_grid(const int n[3], const double ll[3], int ng)
{
    Grid g;
    for (int i = 0; i < 3; i++)
    {
        g.n[i]  = n[i];
        g.ll[i] = ll[i];
    }
    g.ng = ng;
    return g;
}

/* ------------------------------------------------------------------ */
/* Ghost-free entry points for tests (ctypes).                          */
/* ------------------------------------------------------------------ */
template <typename T>
static int fd_apply_t(const int n[3], const double ll[3], int lap_type,
    int nfunc, const T* u, T* out)
{
    const int ng = ghosts_for(lap_type);
    if (ng < 0) return 1;
    Grid g = make_grid(n, ll, ng);
    std::vector<T> a((size_t)nfunc * g.sizeg(), (T)0), b(a.size(), (T)0);
    to_ghosted(g, u, g.size(), a.data(), nfunc);
    trade(g, a.data(), nfunc);
    apply_lap(lap_type, g, a.data(), b.data(), nfunc);
    from_ghosted(g, b.data(), out, g.size(), nfunc);
    return 0;
}

template <typename T>
static int rhs_mehr_t(const int n[3], const double ll[3], int nfunc, const T* u,
    T* out)
{
    Grid g = make_grid(n, ll, 1);
    std::vector<T> a((size_t)nfunc * g.sizeg(), (T)0), b(a.size(), (T)0);
    to_ghosted(g, u, g.size(), a.data(), nfunc);
    trade(g, a.data(), nfunc);
    rhs_mehr1(g, a.data(), b.data(), nfunc);
    from_ghosted(g, b.data(), out, g.size(), nfunc);
    return 0;
}

/* Hamiltonian<T>::applyLocal, src/Hamiltonian.cc:85-159.
 * lap_type 0 (Mehrstellen), apply_B 1: -Lap_M psi + B(V psi)
 *   (pointwiseProduct over ghosted points, rhs_4th_Mehr1, del2_4th_Mehr,
 *   axpy, src/Hamiltonian.cc:106-132 and src/pb/GridFuncVector.cc:88-136);
 * lap_type 0, apply_B 0: -Lap_M psi + V psi (the B-less variant);
 * lap_type 2: FDoper::del2_4th_withPot (src/pb/FDoper.cc:321-399);
 * lap_type 1/3/4: FDkernelDel2_* plus V psi (no reference Hamiltonian path
 *   exists for these, src/pb/Lap.h:35-39; the sum is -Lap psi + V psi). */
template <typename T>
static int hpsi_t(const int n[3], const double ll[3], int lap_type, int apply_B,
    int nfunc, const T* psi, const double* V, T* hpsi)
{
    const int ng = ghosts_for(lap_type);
    if (ng < 0) return 1;
    Grid g = make_grid(n, ll, ng);
    const size_t sg = g.sizeg();
    std::vector<T> phi((size_t)nfunc * sg, (T)0);
    to_ghosted(g, psi, g.size(), phi.data(), nfunc);
    trade(g, phi.data(), nfunc);
    if (lap_type == 0 && apply_B)
    {
        std::vector<double> pot(sg, 0.);
        to_ghosted(g, V, g.size(), pot.data(), 1);
        trade(g, pot.data(), 1);
        std::vector<T> w1((size_t)nfunc * sg, (T)0), work1(w1.size(), (T)0);
        for (int f = 0; f < nfunc; f++)
            for (size_t i = 0; i < sg; i++)
                w1[f * sg + i] = (T)(phi[f * sg + i] * pot[i]);
        rhs_mehr1(g, w1.data(), work1.data(), nfunc);
        del2_mehr(g, phi.data(), w1.data(), nfunc);
        mpaxpy(w1.size(), 1., w1.data(), work1.data());
        from_ghosted(g, work1.data(), hpsi, g.size(), nfunc);
        return 0;
    }
    if (lap_type == 2)
    {
        const double ih[3] = { 1. / (g.h(0) * g.h(0)), 1. / (g.h(1) * g.h(1)),
            1. / (g.h(2) * g.h(2)) };
        const double cc0 = inv12 * ih[0], c1x = -16. * cc0, c2x = 1. * cc0;
        const double cc1 = inv12 * ih[1], c1y = -16. * cc1, c2y = 1. * cc1;
        const double cc2 = inv12 * ih[2], c1z = -16. * cc2, c2z = 1. * cc2;
        const double c0  = -2. * (c1x + c2x + c1y + c2y + c1z + c2z);
        const int incx = g.incx(), incy = g.incy();
        for (int f = 0; f < nfunc; f++)
        {
            size_t ipx = 0;
            for (int ix = 0; ix < n[0]; ix++)
                for (int iy = 0; iy < n[1]; iy++)
                    for (int iz = 0; iz < n[2]; iz++)
                    {
                        const T* v0 = phi.data() + f * sg
                                      + (size_t)((ix + ng) * incx
                                                 + (iy + ng) * incy + iz + ng);
                        hpsi[f * g.size() + ipx]
                            = ((c0 + V[ipx]) * (double)v0[0]
                                + c1x * ((double)v0[-incx] + (double)v0[incx])
                                + c1y * ((double)v0[-incy] + (double)v0[incy])
                                + c1z * ((double)v0[-1] + (double)v0[1])
                                + c2x
                                      * ((double)v0[-2 * incx]
                                          + (double)v0[2 * incx])
                                + c2y
                                      * ((double)v0[-2 * incy]
                                          + (double)v0[2 * incy])
                                + c2z * ((double)v0[-2] + (double)v0[2]));
                        ipx++;
                    }
        }
        return 0;
    }
    std::vector<T> lap((size_t)nfunc * sg, (T)0);
    apply_lap(lap_type, g, phi.data(), lap.data(), nfunc);
    std::vector<T> tmp((size_t)nfunc * g.size());
    from_ghosted(g, lap.data(), tmp.data(), g.size(), nfunc);
    for (int f = 0; f < nfunc; f++)
        for (size_t i = 0; i < g.size(); i++)
            hpsi[f * g.size() + i] = (T)((double)tmp[f * g.size() + i]
                                         + (double)psi[f * g.size() + i] * V[i]);
    return 0;
}

template <typename T>
static int restrict_t(const int n[3], const double ll[3], int nfunc,
    const T* fine, T* coarse)
{
    Grid fg = make_grid(n, ll, 1), cg = fg.coarse();
    std::vector<T> a((size_t)nfunc * fg.sizeg(), (T)0),
        b((size_t)nfunc * cg.sizeg(), (T)0);
    to_ghosted(fg, fine, fg.size(), a.data(), nfunc);
    trade(fg, a.data(), nfunc);
    restrict3d(fg, a.data(), cg, b.data(), nfunc);
    from_ghosted(cg, b.data(), coarse, cg.size(), nfunc);
    return 0;
}

template <typename T>
static int extend_t(const int n[3], const double ll[3], int nfunc,
    const T* coarse, T* fine)
{
    Grid fg = make_grid(n, ll, 1), cg = fg.coarse();
    std::vector<T> a((size_t)nfunc * fg.sizeg(), (T)0),
        b((size_t)nfunc * cg.sizeg(), (T)0);
    to_ghosted(cg, coarse, cg.size(), b.data(), nfunc);
    trade(cg, b.data(), nfunc);
    extend3d(cg, b.data(), fg, a.data(), nfunc);
    from_ghosted(fg, a.data(), fine, fg.size(), nfunc);
    return 0;
}

/* OrbitalsPreconditioning<T>::precond_mg (src/OrbitalsPreconditioning.cc:86-117):
 * v = 0; f = res; v += gamma f; Preconditioning::mg(v, f, lap_type, 0);
 * out = v.  Masks (optional) are those of a MaskSet built by mask_build. */
template <typename T>
static int precond_t(const int n[3], const double ll[3], int lap_type,
    int maxlevels, double gamma, int nfunc, const T* res, T* out,
    const MaskSet<T>* masks)
{
    const int ng = ghosts_for(lap_type);
    if (ng < 0) return 1;
    Grid g = make_grid(n, ll, ng);
    for (int l = 0; l < maxlevels; l++)
        for (int i = 0; i < 3; i++)
            if ((n[i] >> l) % 2) return 2;
    Precond<T, T> P(g, lap_type, maxlevels, nfunc);
    P.masks = masks;
    std::vector<T> v((size_t)nfunc * g.sizeg(), (T)0), f(v.size(), (T)0);
    to_ghosted(g, res, g.size(), f.data(), nfunc);
    mpaxpy(v.size(), gamma, f.data(), v.data());
    P.mg(v.data(), f.data(), lap_type, 0);
    from_ghosted(g, v.data(), out, g.size(), nfunc);
    return 0;
}

/* ------------------------------------------------------------------ */
/* Poisson multigrid on one field: pb::Vcycle (src/pb/Vcycle.h:28-249)  */
/* and pb::Mgm (src/pb/Mgm.h:20-112), one task, periodic.               */
/* ------------------------------------------------------------------ */

/* BLAS-style y += alpha x in the element type (GridFunc::operator-= and
 * operator+=, src/pb/GridFunc.cc:306-319,497-505). */
template <typename T>
void taxpy(size_t n, T alpha, const T* x, T* y)
{
    for (size_t k = 0; k < n; k++)
        y[k] += alpha * x[k];
}

/* GridFunc::norm2 (src/pb/GridFunc.cc:2745-2800,2856-2861): interior sum
 * of squares in double, one partial dot per z line (MPdot) added in x, y
 * order, times the volume element, square root. */
template <typename T>
double gf_norm(const Grid& g, const T* u)
{
    double d = 0.;
    for (int ix = 0; ix < g.n[0]; ix++)
        for (int iy = 0; iy < g.n[1]; iy++)
        {
            const T* line = u + (size_t)(ix + g.ng) * g.incx() + (iy + g.ng) * g.incy() + g.ng;
            double t = 0.;
            for (int iz = 0; iz < g.n[2]; iz++)
                t += (double)line[iz] * (double)line[iz];
            d += t;
        }
    return std::sqrt(d * g.vel());
}

/* Lap::jacobi (src/pb/Lap.cc:27-37): W = A x - B; x += -jf W. */
template <typename T>
void gf_jacobi(int op, const Grid& g, double jf, T* x, const T* b, T* w)
{
    const size_t n = g.sizeg();
    trade(g, x, 1);
    apply_lap(op, g, x, w, 1);
    taxpy(n, (T)-1, b, w);
    mpaxpy(n, -1. * jf, w, x);
}

/* getLowerOrderOp of each operator: Laph4M stays Laph4M (src/pb/Laph4M.h:57),
 * Laph8 -> Laph6 -> Laph4 -> Laph2 -> Laph2 (src/pb/Laph8.h:79-87,
 * Laph6.h:79-87, Laph4.h:75-83, Laph2.h:71-79). */
static int lower_order(int op)
{
    switch (op)
    {
        case 0: return 0;
        case 1: return 1;
        case 2: return 1;
        case 3: return 2;
        case 4: return 3;
    }
    return -1;
}

/* Vcycle from x = 0.  op_ng: ghost width of the level operator's grid
 * (the caller's on the fine level; below, the lower-order grid built with
 * the lower operator's minimum ghost width), which sets the coarse
 * function's ghost width max(op_ng - 1, 1) (src/pb/Vcycle.h:176-180). */
template <typename T>
void vcycle(int op, const Grid& g, int op_ng, int level, T* x, const T* rhs, int cogr,
    int nu1, int nu2)
{
    const double jf = Precond<T, T>::jacobi_factor(op, g);
    const size_t n  = g.sizeg();
    std::vector<T> res(n, (T)0);
    bool coarsen = true;
    for (int i = 0; i < 3; i++)
        if ((g.n[i] & 1) || g.n[i] < 2 * g.ng) coarsen = false;
    for (int i = 0; i < nu1; i++)
        gf_jacobi(op, g, jf, x, rhs, res.data());
    if (level > -cogr && coarsen)
    {
        trade(g, x, 1);
        apply_lap(op, g, x, res.data(), 1);
        taxpy(n, (T)-1, rhs, res.data());
        const Grid cg = g.coarse().with_ghosts(std::max(op_ng - 1, 1));
        std::vector<T> rc(cg.sizeg(), (T)0), uc(cg.sizeg(), (T)0);
        trade(g, res.data(), 1);
        restrict3d(g, res.data(), cg, rc.data(), 1);
        const int lop = lower_order(op);
        vcycle(lop, cg, ghosts_for(lop), level - 1, uc.data(), rc.data(), cogr, nu1, nu2);
        trade(cg, uc.data(), 1);
        extend3d(cg, uc.data(), g, res.data(), 1);
        taxpy(n, (T)-1, res.data(), x);
    }
    for (int i = 0; i < nu2; i++)
        gf_jacobi(op, g, jf, x, rhs, res.data());
}

/* Mgm: rhs = A.rhs(rho) (B rho for Laph4M, rho otherwise); up to
 * max_sweeps times: res = rhs - A vh, stop when |res| < tol |rhs|, else
 * vh += Vcycle(res).  out = final residual, final relative residual,
 * residual reduction, sweeps, converged, levels used. */
template <typename T>
static int mgm_t(const int n[3], const double ll[3], int lap_type, int ng, int cogr,
    int max_sweeps, double tol, int nu1, int nu2, T* vh_io, const T* rho, double* out)
{
    if (ghosts_for(lap_type) < 0 || ng < ghosts_for(lap_type)) return 1;
    const Grid g   = make_grid(n, ll, ng);
    const size_t s = g.sizeg();
    std::vector<T> vh(s, (T)0), rhs(s, (T)0), res(s, (T)0), lhs(s, (T)0), work(s, (T)0);
    to_ghosted(g, vh_io, g.size(), vh.data(), 1);
    to_ghosted(g, rho, g.size(), res.data(), 1);
    if (lap_type == 0)
    {
        trade(g, res.data(), 1);
        rhs_mehr1(g, res.data(), rhs.data(), 1);
    }
    else
        rhs = res;
    const double inv_rhs_norm = 1. / gf_norm(g, rhs.data());
    double init = 1., fr = 0., frr = 0.;
    bool conv = false;
    int nb    = 0;
    for (int i = 0; i < max_sweeps; i++)
    {
        trade(g, vh.data(), 1);
        apply_lap(lap_type, g, vh.data(), lhs.data(), 1);
        for (size_t k = 0; k < s; k++)
            res[k] = rhs[k] - lhs[k];
        const double rn = gf_norm(g, res.data());
        if (i == 0) init = rn;
        if (rn * inv_rhs_norm < tol)
        {
            fr   = rn;
            frr  = rn * inv_rhs_norm;
            conv = true;
            break;
        }
        std::fill(work.begin(), work.end(), (T)0);
        vcycle(lap_type, g, ng, 0, work.data(), res.data(), cogr, nu1, nu2);
        nb++;
        taxpy(s, (T)1, work.data(), vh.data());
    }
    if (!conv)
    {
        trade(g, vh.data(), 1);
        apply_lap(lap_type, g, vh.data(), lhs.data(), 1);
        taxpy(s, (T)-1, rhs.data(), lhs.data());
        fr  = gf_norm(g, lhs.data());
        frr = fr * inv_rhs_norm;
    }
    from_ghosted(g, vh.data(), vh_io, g.size(), 1);
    // grids the cycle visits
    int levels = 1;
    {
        Grid c  = g;
        int cng = ng, op = lap_type;
        for (int l = 0; l < cogr; l++)
        {
            bool ok = true;
            for (int i = 0; i < 3; i++)
                if ((c.n[i] & 1) || c.n[i] < 2 * c.ng) ok = false;
            if (!ok) break;
            c   = c.coarse().with_ghosts(std::max(cng - 1, 1));
            op  = lower_order(op);
            cng = ghosts_for(op);
            levels++;
        }
    }
    out[0] = fr;
    out[1] = frr;
    out[2] = fr / init;
    out[3] = nb;
    out[4] = conv ? 1. : 0.;
    out[5] = levels;
    return 0;
}

/* OrbitalsPreconditioning<T>::setGamma, src/OrbitalsPreconditioning.cc:119-145 */
static double set_gamma(double inv_diag, int mg_levels, double vmax, double small_eig)
{
    double gamma = inv_diag;
    for (int ln = 0; ln <= mg_levels; ln++)
        gamma *= 4.;
    return 1.0 / (2.0 / gamma + fabs(vmax - small_eig));
}

extern "C" {

int orc_fd_apply_d(const int* n, const double* ll, int lap_type, int nfunc,
    const double* u, double* out)
{
    return fd_apply_t(n, ll, lap_type, nfunc, u, out);
}
int orc_fd_apply_f(const int* n, const double* ll, int lap_type, int nfunc,
    const float* u, float* out)
{
    return fd_apply_t(n, ll, lap_type, nfunc, u, out);
}
int orc_rhs_mehr_d(const int* n, const double* ll, int nfunc, const double* u,
    double* out)
{
    return rhs_mehr_t(n, ll, nfunc, u, out);
}
int orc_rhs_mehr_f(const int* n, const double* ll, int nfunc, const float* u,
    float* out)
{
    return rhs_mehr_t(n, ll, nfunc, u, out);
}
int orc_hpsi_d(const int* n, const double* ll, int lap_type, int apply_B,
    int nfunc, const double* psi, const double* V, double* hpsi)
{
    return hpsi_t(n, ll, lap_type, apply_B, nfunc, psi, V, hpsi);
}
int orc_hpsi_f(const int* n, const double* ll, int lap_type, int apply_B,
    int nfunc, const float* psi, const double* V, float* hpsi)
{
    return hpsi_t(n, ll, lap_type, apply_B, nfunc, psi, V, hpsi);
}
int orc_restrict_d(const int* n, const double* ll, int nfunc, const double* f,
    double* c)
{
    return restrict_t(n, ll, nfunc, f, c);
}
int orc_restrict_f(const int* n, const double* ll, int nfunc, const float* f,
    float* c)
{
    return restrict_t(n, ll, nfunc, f, c);
}
int orc_extend_d(const int* n, const double* ll, int nfunc, const double* c,
    double* f)
{
    return extend_t(n, ll, nfunc, c, f);
}
int orc_extend_f(const int* n, const double* ll, int nfunc, const float* c,
    float* f)
{
    return extend_t(n, ll, nfunc, c, f);
}

double orc_set_gamma(double inv_diag, int mg_levels, double vmax, double small_eig)
{
    return set_gamma(inv_diag, mg_levels, vmax, small_eig);
}
double orc_jacobi_factor(const int* n, const double* ll, int lap_type)
{
    Grid g = make_grid(n, ll, 1);
    return Precond<double, double>::jacobi_factor(lap_type, g);
}

/* Masks.  mask_build_* fills, for nfunc orbitals with centres (nfunc x 3)
 * and radii, the state of every level 0..nlevels-1 (state[l*nfunc+f]) and
 * the values (values[(l*nfunc+f)*level_size(l) + pt]).  ng is the ghost
 * count of the mesh grid (1 Mehrstellen, 4 8th order). */
} // extern "C"

template <typename M>
static int mask_build_t(const int* n, const double* ll, int ng, int nlevels,
    int nfunc, const double* centers, const double* radii, int func,
    int* state, M* values)
{
    Grid g      = make_grid(n, ll, ng);
    size_t off  = 0;
    for (int l = 0; l < nlevels; l++)
    {
        const size_t ls = (size_t)(n[0] >> l) * (n[1] >> l) * (n[2] >> l);
#pragma omp parallel for
        for (int f = 0; f < nfunc; f++)
            state[l * nfunc + f] = mask_init(g, l, centers + 3 * f, radii[f],
                func, values + off + (size_t)f * ls);
        off += (size_t)nfunc * ls;
    }
    return 0;
}
extern "C" {
int orc_mask_build_d(const int* n, const double* ll, int ng, int nlevels,
    int nfunc, const double* centers, const double* radii, int func,
    int* state, double* values)
{
    return mask_build_t(n, ll, ng, nlevels, nfunc, centers, radii, func, state,
        values);
}
int orc_mask_build_f(const int* n, const double* ll, int ng, int nlevels,
    int nfunc, const double* centers, const double* radii, int func,
    int* state, float* values)
{
    return mask_build_t(n, ll, ng, nlevels, nfunc, centers, radii, func, state,
        values);
}

} // extern "C"

template <typename T>
static MaskSet<T> wrap_masks(const int* n, int nlevels, int nfunc, int kind,
    const int* state, const T* values)
{
    MaskSet<T> ms;
    ms.nlevels = nlevels;
    ms.kind    = kind;
    size_t off = 0;
    for (int l = 0; l < nlevels; l++)
    {
        const size_t ls = (size_t)(n[0] >> l) * (n[1] >> l) * (n[2] >> l);
        ms.state.emplace_back(state + l * nfunc, state + (l + 1) * nfunc);
        ms.values.emplace_back();
        for (int f = 0; f < nfunc; f++)
            ms.values.back().emplace_back(values + off + f * ls,
                values + off + (f + 1) * ls);
        off += (size_t)nfunc * ls;
    }
    return ms;
}

/* mask apply on ghost-free data at one level */
template <typename T>
static int mask_apply_t(const int* n, int level, int nlevels, int nfunc, int kind,
    const int* state, const T* values, T* u)
{
    int nl[3] = { n[0] >> level, n[1] >> level, n[2] >> level };
    double ll[3] = { 1., 1., 1. };
    Grid g = make_grid(nl, ll, 1);
    MaskSet<T> ms = wrap_masks(n, nlevels, nfunc, kind, state, values);
    std::vector<T> a((size_t)nfunc * g.sizeg(), (T)0);
    to_ghosted(g, u, g.size(), a.data(), nfunc);
    app_mask(g, a.data(), nfunc, &ms, level);
    from_ghosted(g, a.data(), u, g.size(), nfunc);
    return 0;
}
extern "C" {
int orc_mask_apply_d(const int* n, int level, int nlevels, int nfunc, int kind,
    const int* state, const double* values, double* u)
{
    return mask_apply_t(n, level, nlevels, nfunc, kind, state, values, u);
}
int orc_mask_apply_f(const int* n, int level, int nlevels, int nfunc, int kind,
    const int* state, const float* values, float* u)
{
    return mask_apply_t(n, level, nlevels, nfunc, kind, state, values, u);
}

/* precond with optional masks (state == NULL: no masks) */
int orc_precond_d(const int* n, const double* ll, int lap_type, int maxlevels,
    double gamma, int nfunc, const double* res, double* out, int kind,
    const int* state, const double* values)
{
    if (state == nullptr)
        return precond_t<double>(n, ll, lap_type, maxlevels, gamma, nfunc, res,
            out, nullptr);
    MaskSet<double> ms
        = wrap_masks(n, maxlevels + 1, nfunc, kind, state, values);
    return precond_t<double>(n, ll, lap_type, maxlevels, gamma, nfunc, res, out,
        &ms);
}
int orc_precond_f(const int* n, const double* ll, int lap_type, int maxlevels,
    double gamma, int nfunc, const float* res, float* out, int kind,
    const int* state, const float* values)
{
    if (state == nullptr)
        return precond_t<float>(n, ll, lap_type, maxlevels, gamma, nfunc, res,
            out, nullptr);
    MaskSet<float> ms = wrap_masks(n, maxlevels + 1, nfunc, kind, state, values);
    return precond_t<float>(n, ll, lap_type, maxlevels, gamma, nfunc, res, out,
        &ms);
}

/* ------------------------------------------------------------------ */
/* Gram and H matrices.                                                 */
/* ------------------------------------------------------------------ */

/* LocGridOrbitals::getLocalOverlap (src/LocGridOrbitals.cc:1504-1530) with
 * a reference-BLAS DSYRK('l','t') (sequential dot per entry), then
 * fillUpperWithLower, scal(vel), and the |x| > 1e-14 filter of
 * LocalMatrices2DistMatrix::convert (src/LocalMatrices2DistMatrix.cc:16,60).
 * psi: nfunc columns of numpt points, leading dimension ld. */
int orc_gram_d(const double* psi, long ld, int nfunc, long numpt, double vel,
    double* S)
{
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = j; i < nfunc; i++)
        {
            double t = 0.;
            const double* a = psi + (size_t)i * ld;
            const double* b = psi + (size_t)j * ld;
            for (long k = 0; k < numpt; k++)
                t = t + a[k] * b[k];
            S[(size_t)j * nfunc + i] = t;
        }
    for (int j = 0; j < nfunc; j++)
        for (int i = j; i < nfunc; i++)
        {
            double x = S[(size_t)j * nfunc + i] * vel;
            if (!(std::fabs(x) > 1.e-14)) x = 0.;
            S[(size_t)j * nfunc + i] = x;
            S[(size_t)i * nfunc + j] = x;
        }
    return 0;
}

/* FP32 orbitals: LAU_H::MPdot-style FP64 accumulation of FP32 products
 * (src/linear_algebra/mputils.cc:147-165) for every entry, result kept in
 * FP64 (the FP64 reference the mixed path is measured against). */
int orc_gram_f(const float* psi, long ld, int nfunc, long numpt, double vel,
    double* S)
{
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = j; i < nfunc; i++)
        {
            double t = 0.;
            const float* a = psi + (size_t)i * ld;
            const float* b = psi + (size_t)j * ld;
            for (long k = 0; k < numpt; k++)
                t += (double)a[k] * (double)b[k];
            double x = t * vel;
            if (!(std::fabs(x) > 1.e-14)) x = 0.;
            S[(size_t)j * nfunc + i] = x;
            S[(size_t)i * nfunc + j] = x;
        }
    return 0;
}

/* The reference's mixed-precision (USE_MP) build forms S and H of FP32
 * orbitals in a float local matrix: LocalMatrices<float>::gemm (MPgemm 't',
 * 'n': each entry the FP64 MPdot rounded to float), copied to double and
 * scaled by vel (src/LocGridOrbitals.cc:1584-1602), then the 1e-14 filter.
 * b is psi for S and hpsi for H; out column-major (j * nfunc + i). */
int orc_product_f_usemp(const float* psi, const float* b, long ld, int nfunc,
    long numpt, double vel, double* out)
{
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = 0; i < nfunc; i++)
        {
            double t = 0.;
            const float* x = psi + (size_t)i * ld;
            const float* y = b + (size_t)j * ld;
            for (long k = 0; k < numpt; k++)
                t += (double)x[k] * (double)y[k];
            double v = (double)(float)t * vel;
            if (!(std::fabs(v) > 1.e-14)) v = 0.;
            out[(size_t)j * nfunc + i] = v;
        }
    return 0;
}

/* Hamiltonian::addHlocalij -> LocGridOrbitals::computeLocalProduct
 * (src/LocGridOrbitals.cc:1554-1604): reference-BLAS DGEMM('t','n'),
 * H(i,j) = <psi_i, hpsi_j> * vel, same 1e-14 filter on accumulation. */
int orc_hmat_d(const double* psi, const double* hpsi, long ld, int nfunc,
    long numpt, double vel, double* H)
{
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = 0; i < nfunc; i++)
        {
            double t = 0.;
            const double* a = psi + (size_t)i * ld;
            const double* b = hpsi + (size_t)j * ld;
            for (long k = 0; k < numpt; k++)
                t = t + a[k] * b[k];
            double x = t * vel;
            if (!(std::fabs(x) > 1.e-14)) x = 0.;
            H[(size_t)j * nfunc + i] = x;
        }
    return 0;
}
int orc_hmat_f(const float* psi, const float* hpsi, long ld, int nfunc,
    long numpt, double vel, double* H)
{
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = 0; i < nfunc; i++)
        {
            double t = 0.;
            const float* a = psi + (size_t)i * ld;
            const float* b = hpsi + (size_t)j * ld;
            for (long k = 0; k < numpt; k++)
                t += (double)a[k] * (double)b[k];
            double x = t * vel;
            if (!(std::fabs(x) > 1.e-14)) x = 0.;
            H[(size_t)j * nfunc + i] = x;
        }
    return 0;
}

/* GramMatrix::updateLS (src/GramMatrix.cc:180-191): Cholesky S = L L^T,
 * lower, column-major n x n, returns LAPACK-style info (0 ok, k>0 if the
 * leading minor k is not positive). */
int orc_potrf(int n, double* A)
{
    for (int j = 0; j < n; j++)
    {
        double d = A[(size_t)j * n + j];
        for (int k = 0; k < j; k++)
            d -= A[(size_t)k * n + j] * A[(size_t)k * n + j];
        if (!(d > 0.)) return j + 1;
        d                    = sqrt(d);
        A[(size_t)j * n + j] = d;
        for (int i = j + 1; i < n; i++)
        {
            double s = A[(size_t)j * n + i];
            for (int k = 0; k < j; k++)
                s -= A[(size_t)k * n + i] * A[(size_t)k * n + j];
            A[(size_t)j * n + i] = s / d;
        }
    }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < j; i++)
            A[(size_t)j * n + i] = 0.;
    return 0;
}

/* GramMatrix::computeInverse (src/GramMatrix.cc:75-91): potri on the factor,
 * then the full symmetric inverse.  Computed here as L^{-T} L^{-1}. */
int orc_inverse_from_chol(int n, const double* L, double* Sinv)
{
    std::vector<double> Li((size_t)n * n, 0.);
    for (int j = 0; j < n; j++)
    {
        Li[(size_t)j * n + j] = 1. / L[(size_t)j * n + j];
        for (int i = j + 1; i < n; i++)
        {
            double s = 0.;
            for (int k = j; k < i; k++)
                s -= L[(size_t)k * n + i] * Li[(size_t)j * n + k];
            Li[(size_t)j * n + i] = s / L[(size_t)i * n + i];
        }
    }
#pragma omp parallel for
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
        {
            double s = 0.;
            const int k0 = std::max(i, j);
            for (int k = k0; k < n; k++)
                s += Li[(size_t)i * n + k] * Li[(size_t)j * n + k];
            Sinv[(size_t)j * n + i] = s;
        }
    return 0;
}

/* ProjectedMatrices::getEigSum (src/ProjectedMatrices.cc:550-566):
 * tr(H S^-1) with H used as a symmetric matrix (lower triangle). */
double orc_trace_prod(int n, const double* H, const double* Sinv)
{
    double tr = 0.;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < n; k++)
        {
            const double h = (i >= k) ? H[(size_t)k * n + i] : H[(size_t)i * n + k];
            tr += h * Sinv[(size_t)i * n + k];
        }
    return tr;
}

} // extern "C"

/* ------------------------------------------------------------------ */
/* Residual and update of the block preconditioned-gradient step.       */
/* ------------------------------------------------------------------ */
extern "C" {

/* ProjectedMatrices::updateTheta (src/ProjectedMatrices.h:218-225):
 * theta = S^-1 H with S^-1 used as symmetric (lower part), column-major. */
int orc_theta(int n, const double* Sinv, const double* H, double* theta)
{
#pragma omp parallel for
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
        {
            double s = 0.;
            for (int k = 0; k < n; k++)
            {
                const double a = (i >= k) ? Sinv[(size_t)k * n + i] : Sinv[(size_t)i * n + k];
                s += a * H[(size_t)j * n + k];
            }
            theta[(size_t)j * n + i] = s;
        }
    return 0;
}

/* LocGridOrbitals::multiplyByMatrix (src/LocGridOrbitals.cc:793-830), one
 * subdomain: out_j = sum_i psi_i theta(i, j), FP64 accumulation. */
int orc_mult_matrix_d(const double* psi, long ld, int nfunc, long numpt,
    const double* theta, double* out)
{
#pragma omp parallel for
    for (long p = 0; p < numpt; p++)
        for (int j = 0; j < nfunc; j++)
        {
            double s = 0.;
            for (int i = 0; i < nfunc; i++)
                s += psi[(size_t)i * ld + p] * theta[(size_t)j * nfunc + i];
            out[(size_t)j * ld + p] = s;
        }
    return 0;
}
int orc_mult_matrix_f(const float* psi, long ld, int nfunc, long numpt,
    const double* theta, float* out)
{
#pragma omp parallel for
    for (long p = 0; p < numpt; p++)
        for (int j = 0; j < nfunc; j++)
        {
            double s = 0.;
            for (int i = 0; i < nfunc; i++)
                s += (double)psi[(size_t)i * ld + p] * theta[(size_t)j * nfunc + i];
            out[(size_t)j * ld + p] = (float)s;
        }
    return 0;
}
}

/* MGmol::computeResidualUsingHPhi (src/MGmol.cc:1227-1290): with applyB,
 * tmp = B psi for every function (Lap::rhs), then res = tmp theta - hpsi;
 * without, res = psi theta - hpsi.  Rydberg units. */
template <typename T>
static int residual_t(const int* n, const double* ll, int apply_B, int nfunc,
    const T* psi, const T* hpsi, const double* theta, T* res)
{
    const size_t np = (size_t)n[0] * n[1] * n[2];
    std::vector<T> tmp(np * nfunc);
    if (apply_B)
        rhs_mehr_t(n, ll, nfunc, psi, tmp.data());
    else
        std::copy(psi, psi + np * nfunc, tmp.begin());
    std::vector<T> prod(np * nfunc);
#pragma omp parallel for
    for (long p = 0; p < (long)np; p++)
        for (int j = 0; j < nfunc; j++)
        {
            double s = 0.;
            for (int i = 0; i < nfunc; i++)
                s += (double)tmp[(size_t)i * np + p] * theta[(size_t)j * nfunc + i];
            prod[(size_t)j * np + p] = (T)s;
        }
    // res.axpy(-1., hphi)
    for (size_t k = 0; k < np * nfunc; k++)
        res[k] = prod[k] + static_cast<T>(-1. * static_cast<double>(hpsi[k]));
    return 0;
}

extern "C" {
int orc_residual_d(const int* n, const double* ll, int apply_B, int nfunc,
    const double* psi, const double* hpsi, const double* theta, double* res)
{
    return residual_t(n, ll, apply_B, nfunc, psi, hpsi, theta, res);
}
int orc_residual_f(const int* n, const double* ll, int apply_B, int nfunc,
    const float* psi, const float* hpsi, const double* theta, float* res)
{
    return residual_t(n, ll, apply_B, nfunc, psi, hpsi, theta, res);
}

int orc_mgm_d(const int* n, const double* ll, int lap_type, int ng, int cogr,
    int max_sweeps, double tol, int nu1, int nu2, double* vh, const double* rho,
    double* out)
{
    return mgm_t(n, ll, lap_type, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
}
int orc_mgm_f(const int* n, const double* ll, int lap_type, int ng, int cogr,
    int max_sweeps, double tol, int nu1, int nu2, float* vh, const float* rho,
    double* out)
{
    return mgm_t(n, ll, lap_type, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
}
}

/* ------------------------------------------------------------------ */
/* Mehrstellen projected matrices and the normalization.               */
/* ------------------------------------------------------------------ */

/* LocGridOrbitals::computeMatB (src/LocGridOrbitals.cc:1428-1487): work_i =
 * B psi_i (LapOper.rhs, the Mehrstellen right-hand side), ss = psi^T work
 * (MPgemmTN: float input, FP64 accumulation; src/linear_algebra/
 * mputils.cc:1035-1054), ss.scal(vel), then the |x| > 1e-14 filter of the
 * conversion to the distributed matrix (ProjectedMatricesMehrstellen::
 * initializeMatB -> LocalMatrices2DistMatrix::accumulate).  Both triangles
 * are formed, as the reference does. */
template <typename T>
static int matb_t(const int* n, const double* ll, int nfunc, const T* psi, double* B)
{
    const size_t np = (size_t)n[0] * n[1] * n[2];
    std::vector<T> w(np * nfunc);
    rhs_mehr_t(n, ll, nfunc, psi, w.data());
    const double vel = (ll[0] / n[0]) * (ll[1] / n[1]) * (ll[2] / n[2]);
#pragma omp parallel for schedule(dynamic)
    for (int j = 0; j < nfunc; j++)
        for (int i = 0; i < nfunc; i++)
        {
            double t = 0.;
            const T* a = psi + (size_t)i * np;
            const T* b = w.data() + (size_t)j * np;
            for (size_t k = 0; k < np; k++)
                t += (double)a[k] * (double)b[k];
            double x = t * vel;
            if (!(std::fabs(x) > 1.e-14)) x = 0.;
            B[(size_t)j * nfunc + i] = x;
        }
    return 0;
}

/* LocGridOrbitals::normalize (src/LocGridOrbitals.cc:2230-2311, the branch
 * without short-sighted matrices): diagS_i = vel * BlockVector::dot(i, i)
 * (MPdot, FP64 accumulation, src/linear_algebra/mputils.cc:145-166), then
 * BlockVector::scal(1 / sqrt(diagS_i)) (MPscal: (T)(alpha * (double)x),
 * mputils.cc:53-80).  Returns 1 (psi unchanged) when a diagS_i <= 1e-15,
 * which the reference asserts against. */
template <typename T>
static int normalize_t(const int* n, const double* ll, int nfunc, T* psi, double* diag)
{
    const size_t np  = (size_t)n[0] * n[1] * n[2];
    const double vel = (ll[0] / n[0]) * (ll[1] / n[1]) * (ll[2] / n[2]);
    for (int i = 0; i < nfunc; i++)
    {
        double d = 0.;
        const T* p = psi + (size_t)i * np;
        for (size_t k = 0; k < np; k++)
            d += (double)p[k] * (double)p[k];
        diag[i] = vel * d;
        if (!(diag[i] > 1.e-15)) return 1;
    }
    for (int i = 0; i < nfunc; i++)
    {
        const double alpha = 1. / std::sqrt(diag[i]);
        T* p = psi + (size_t)i * np;
        for (size_t k = 0; k < np; k++)
            p[k] = (T)(alpha * (double)p[k]);
    }
    return 0;
}

extern "C" {
int orc_matb_d(const int* n, const double* ll, int nfunc, const double* psi, double* B)
{
    return matb_t(n, ll, nfunc, psi, B);
}
int orc_matb_f(const int* n, const double* ll, int nfunc, const float* psi, double* B)
{
    return matb_t(n, ll, nfunc, psi, B);
}
int orc_normalize_d(const int* n, const double* ll, int nfunc, double* psi, double* diag)
{
    return normalize_t(n, ll, nfunc, psi, diag);
}
int orc_normalize_f(const int* n, const double* ll, int nfunc, float* psi, double* diag)
{
    return normalize_t(n, ll, nfunc, psi, diag);
}

/* ProjectedMatricesMehrstellen::updateHB (src/ProjectedMatricesMehrstellen.h:
 * 55-62): HB = symm('l', 'l', S, theta) (S read from its lower triangle),
 * then transpose(0.5, copy, 0.5): HB(i, j) = 0.5 HB(i, j) + 0.5 HB(j, i).
 * Column-major n x n. */
int orc_update_hb(int n, const double* S, const double* theta, double* HB)
{
    std::vector<double> t((size_t)n * n);
#pragma omp parallel for
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
        {
            double s = 0.;
            for (int k = 0; k < n; k++)
            {
                const double a = (i >= k) ? S[(size_t)k * n + i] : S[(size_t)i * n + k];
                s += a * theta[(size_t)j * n + k];
            }
            t[(size_t)j * n + i] = s;
        }
    for (int j = 0; j < n; j++)
        for (int i = 0; i < n; i++)
            HB[(size_t)j * n + i] = 0.5 * t[(size_t)j * n + i] + 0.5 * t[(size_t)i * n + j];
    return 0;
}
}

/* ------------------------------------------------------------------ */
/* Anderson extrapolation (AndersonMix<T>::update).                     */
/* ------------------------------------------------------------------ */

/* eigenvalues (ascending) of the symmetric n x n matrix in the lower
 * triangle of a (column-major, leading dimension lda), cyclic Jacobi: the
 * DSYEV('N', 'l') of src/AndersonMix.cc:138 */
static void orc_sym_eig(const double* a, int n, int lda, double* w)
{
    std::vector<double> A((size_t)n * n);
    for (int j = 0; j < n; j++)
        for (int i = j; i < n; i++)
            A[i + (size_t)j * n] = A[j + (size_t)i * n] = a[i + (size_t)j * lda];
    for (int sweep = 0; sweep < 100; sweep++)
    {
        double off = 0., tot = 0.;
        for (size_t t = 0; t < A.size(); t++)
        {
            tot += A[t] * A[t];
            if (t % n != t / n) off += A[t] * A[t];
        }
        if (off == 0. || off <= 1e-30 * tot) break;
        for (int p = 0; p < n - 1; p++)
            for (int q = p + 1; q < n; q++)
            {
                const double apq = A[p + (size_t)q * n];
                if (apq == 0.) continue;
                const double tau = (A[q + (size_t)q * n] - A[p + (size_t)p * n]) / (2. * apq);
                const double t = (tau >= 0. ? 1. : -1.) / (std::fabs(tau) + std::sqrt(1. + tau * tau));
                const double c = 1. / std::sqrt(1. + t * t), s = t * c;
                for (int r = 0; r < n; r++)
                {
                    const double x = A[r + (size_t)p * n], y = A[r + (size_t)q * n];
                    A[r + (size_t)p * n] = c * x - s * y;
                    A[r + (size_t)q * n] = s * x + c * y;
                }
                for (int r = 0; r < n; r++)
                {
                    const double x = A[p + (size_t)r * n], y = A[q + (size_t)r * n];
                    A[p + (size_t)r * n] = c * x - s * y;
                    A[q + (size_t)r * n] = s * x + c * y;
                }
            }
    }
    for (int i = 0; i < n; i++)
        w[i] = A[i + (size_t)i * n];
    std::sort(w, w + n);
}

/* DPOTRF + DPOTRS with uplo 'l' on the leading n x n block (leading
 * dimension lda) of a copy of a; b overwritten; returns the DPOTRF info */
static int orc_chol_solve(const double* a0, int n, int lda, double* b)
{
    std::vector<double> a(a0, a0 + (size_t)lda * n);
    for (int j = 0; j < n; j++)
    {
        double d = a[j + (size_t)j * lda];
        for (int k = 0; k < j; k++)
            d -= a[j + (size_t)k * lda] * a[j + (size_t)k * lda];
        if (!(d > 0.)) return j + 1;
        d = std::sqrt(d);
        a[j + (size_t)j * lda] = d;
        for (int i = j + 1; i < n; i++)
        {
            double t = a[i + (size_t)j * lda];
            for (int k = 0; k < j; k++)
                t -= a[i + (size_t)k * lda] * a[j + (size_t)k * lda];
            a[i + (size_t)j * lda] = t / d;
        }
    }
    for (int i = 0; i < n; i++)
    {
        double t = b[i];
        for (int k = 0; k < i; k++)
            t -= a[i + (size_t)k * lda] * b[k];
        b[i] = t / a[i + (size_t)i * lda];
    }
    for (int i = n - 1; i >= 0; i--)
    {
        double t = b[i];
        for (int k = i + 1; k < n; k++)
            t -= a[k + (size_t)i * lda] * b[k];
        b[i] = t / a[i + (size_t)i * lda];
    }
    return 0;
}

/* the orbital block arithmetic the update uses (LocGridOrbitals over
 * BlockVector and mputils): MPscal, MPaxpy, v -= s in the storage type, and
 * the diagonal dot product sum_k (double)(MPdot_k * vel) * invS(k, k) */
template <typename T>
struct OrcBlocks
{
    int nfunc;
    size_t npts;
    double vel;
    const double* invs;
    static void scal(std::vector<T>& u, double a)
    {
        if (a == 1.) return;
        for (auto& v : u)
            v = (a == 0.) ? (T)0 : (T)(a * (double)v);
    }
    static void axpy(std::vector<T>& y, double a, const std::vector<T>& x)
    {
        for (size_t i = 0; i < y.size(); i++)
            y[i] += (T)(a * (double)x[i]);
    }
    static void sub(std::vector<T>& v, const std::vector<T>& s)
    {
        for (size_t i = 0; i < v.size(); i++)
            v[i] -= s[i];
    }
    double dot(const std::vector<T>& a, const std::vector<T>& b) const
    {
        double tr = 0.;
        std::vector<double> ss(nfunc);
        for (int k = 0; k < nfunc; k++)
        {
            double d = 0.;
            for (size_t p = 0; p < npts; p++)
                d += (double)a[k * npts + p] * (double)b[k * npts + p];
            ss[k] = d * vel;
        }
        for (int k = 0; k < nfunc; k++)
            tr += ss[k] * invs[k];
        return tr;
    }
};

/* AndersonMix<T>::update (src/AndersonMix.cc:63-321) for nsteps residuals
 * res_s = fscale * f_s: history of m pairs, mm grown by one per call up to
 * m; mat / rhs from the differences f - f_i; mm shortened while the
 * matrix rescaled to unit diagonal has a determinant (product of its
 * eigenvalues) below 0.01 and whenever a coefficient leaves [-3, 0.5] with
 * mm > 1; a lone coefficient outside is reset; then x and f are mixed and
 * the old x and f enter the history.  invs: nsteps x nfunc weights
 * (S^-1)(k, k).  xs_out[s]: x after update s.  Returns 1 where the
 * reference's factorization fails. */
template <typename T>
struct OrcAnderson
{
    int m, mm = -1;
    double beta;
    std::vector<std::vector<T>> xi, fi;
    std::vector<double> mat, rhs, theta;
    OrcAnderson(int m_, double b, size_t nb)
        : m(m_), beta(b), xi(m_, std::vector<T>(nb)), fi(m_, std::vector<T>(nb)),
          mat((size_t)m_ * m_), rhs(m_), theta(m_)
    {
    }

    /* one update of x with the residual f (already scaled); returns 1 where
     * the reference's factorization fails */
    int update(std::vector<T>& x, std::vector<T>& f, const OrcBlocks<T>& B)
    {
        const double min_det = 0.01, max_theta = 0.5, min_theta = -3.;
        if (mm < m) mm++;
        if (mm > 0)
        {
            std::vector<std::vector<T>> u(mm, f);
            for (int i = 0; i < mm; i++)
                OrcBlocks<T>::sub(u[i], fi[i]);
            for (int i = 0; i < mm; i++)
            {
                mat[(size_t)i * m + i] = B.dot(u[i], u[i]);
                rhs[i]                 = B.dot(u[i], f);
                for (int j = 0; j < i; j++)
                    mat[(size_t)j * m + i] = B.dot(u[i], u[j]);
            }
            bool flag = true;
            while (flag)
            {
                flag = false;
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
                    std::vector<double> w(mm);
                    orc_sym_eig(t.data(), mm, m, w.data());
                    double det = 1.;
                    for (int i = 0; i < mm; i++)
                        det *= w[i];
                    if (det < min_det)
                        mm--;
                    else
                        break;
                }
                if (orc_chol_solve(mat.data(), mm, m, theta.data()) != 0) return 1;
                for (int j = 0; j < mm; j++)
                {
                    if (theta[j] > max_theta)
                    {
                        if (mm > 1)
                        {
                            mm--;
                            flag = true;
                            break;
                        }
                        theta[j] = theta[j] > 1. ? -0.5 : 0.;
                    }
                    else if (theta[j] < min_theta)
                    {
                        if (mm > 1)
                        {
                            mm--;
                            flag = true;
                            break;
                        }
                        theta[j] = min_theta;
                    }
                }
            }
        }
        double factor = 1.;
        for (int j = 0; j < mm; j++)
            factor -= theta[j];
        if (m > 0)
        {
            std::vector<T> xold(x);
            if (mm > 0) OrcBlocks<T>::scal(x, factor);
            for (int j = 0; j < mm; j++)
                OrcBlocks<T>::axpy(x, theta[j], xi[j]);
            std::rotate(xi.rbegin(), xi.rbegin() + 1, xi.rend());
            xi[0] = xold;
            std::vector<T> fold(f);
            if (mm > 0) OrcBlocks<T>::scal(f, factor);
            for (int j = 0; j < mm; j++)
                OrcBlocks<T>::axpy(f, theta[j], fi[j]);
            std::rotate(fi.rbegin(), fi.rbegin() + 1, fi.rend());
            fi[0] = fold;
        }
        OrcBlocks<T>::axpy(x, mm > 0 ? beta : 1., f);
        return 0;
    }
};

/* AndersonMix<T>::update (src/AndersonMix.cc:63-321) for nsteps residuals
 * res_s = fscale * f_s: history of m pairs, mm grown by one per call up to
 * m; mat / rhs from the differences f - f_i; mm shortened while the
 * matrix rescaled to unit diagonal has a determinant (product of its
 * eigenvalues) below 0.01 and whenever a coefficient leaves [-3, 0.5] with
 * mm > 1; a lone coefficient outside is reset; then x and f are mixed and
 * the old x and f enter the history.  invs: nsteps x nfunc weights
 * (S^-1)(k, k).  xs_out[s]: x after update s.  Returns 1 where the
 * reference's factorization fails. */
template <typename T>
static int anderson_t(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const T* x0, int nsteps, const T* fseq, double fscale, T* xs_out)
{
    const size_t nb = (size_t)nfunc * npts;
    std::vector<T> x(x0, x0 + nb);
    OrcAnderson<T> mix(m, beta, nb);
    OrcBlocks<T> B{ nfunc, (size_t)npts, vel, nullptr };
    for (int s = 0; s < nsteps; s++)
    {
        B.invs = invs + (size_t)s * nfunc;
        std::vector<T> f(fseq + s * nb, fseq + (s + 1) * nb);
        OrcBlocks<T>::scal(f, fscale);
        if (mix.update(x, f, B)) return 1;
        std::copy(x.begin(), x.end(), xs_out + s * nb);
    }
    return 0;
}

/* a mixer that lives across calls (for checking an iteration whose
 * residuals depend on x): handle = orc_anderson_new, then one step per
 * orc_anderson_step (x updated in place), orc_anderson_free */
template <typename T>
static void* anderson_new(int m, double beta, long nb)
{
    return new OrcAnderson<T>(m, beta, (size_t)nb);
}
template <typename T>
static int anderson_step(void* h, int npts, int nfunc, double vel, const double* invs, T* x,
    const T* f0, double fscale)
{
    auto* mix = static_cast<OrcAnderson<T>*>(h);
    const size_t nb = (size_t)nfunc * npts;
    OrcBlocks<T> B{ nfunc, (size_t)npts, vel, invs };
    std::vector<T> xv(x, x + nb), f(f0, f0 + nb);
    OrcBlocks<T>::scal(f, fscale);
    if (mix->update(xv, f, B)) return 1;
    std::copy(xv.begin(), xv.end(), x);
    return 0;
}

extern "C" {
void* orc_anderson_new_f(int m, double beta, long nb) { return anderson_new<float>(m, beta, nb); }
void* orc_anderson_new_d(int m, double beta, long nb) { return anderson_new<double>(m, beta, nb); }
void orc_anderson_free_f(void* h) { delete static_cast<OrcAnderson<float>*>(h); }
void orc_anderson_free_d(void* h) { delete static_cast<OrcAnderson<double>*>(h); }
int orc_anderson_step_f(void* h, int npts, int nfunc, double vel, const double* invs, float* x,
    const float* f, double fscale)
{
    return anderson_step(h, npts, nfunc, vel, invs, x, f, fscale);
}
int orc_anderson_step_d(void* h, int npts, int nfunc, double vel, const double* invs, double* x,
    const double* f, double fscale)
{
    return anderson_step(h, npts, nfunc, vel, invs, x, f, fscale);
}
}

extern "C" {
int orc_anderson_f(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const float* x0, int nsteps, const float* fseq, double fscale, float* xs_out)
{
    return anderson_t(npts, nfunc, m, beta, vel, invs, x0, nsteps, fseq, fscale, xs_out);
}
int orc_anderson_d(int npts, int nfunc, int m, double beta, double vel, const double* invs,
    const double* x0, int nsteps, const double* fseq, double fscale, double* xs_out)
{
    return anderson_t(npts, nfunc, m, beta, vel, invs, x0, nsteps, fseq, fscale, xs_out);
}
}

/* ------------------------------------------------------------------ */
/* Electronic density.                                                  */
/* ------------------------------------------------------------------ */

/* Rho<T>::computeRho for non-orthogonal orbitals, one subdomain
 * (src/Rho.cc:282-320, computeRhoSubdomainUsingBlas3 :359-450):
 * product = MPgemmNN(psi, X) (FP64 accumulation, stored in the orbital
 * type), rho(p) += product_j(p) * psi_j(p) (the product of two orbital-type
 * values, added in FP64, j in order), then rescaleTotalCharge (:124-200):
 * charge = vel * sum_p rho(p) in order; when charge > 0, t = nel / charge and
 * rho *= t (MPscal).  Returns 1 where the reference aborts (|t - 1| > 0.02)
 * and leaves rho unscaled then.  out[0] = charge, out[1] = t. */
template <typename T>
static int rho_t(const int* n, const double* ll, int nfunc, const T* psi, const double* X,
    double nel, double* rho, double* out)
{
    const size_t np  = (size_t)n[0] * n[1] * n[2];
    const double vel = (ll[0] / n[0]) * (ll[1] / n[1]) * (ll[2] / n[2]);
    std::vector<T> prod(np * nfunc);
#pragma omp parallel for
    for (long p = 0; p < (long)np; p++)
        for (int j = 0; j < nfunc; j++)
        {
            double s = 0.;
            for (int i = 0; i < nfunc; i++)
                s += (double)psi[(size_t)i * np + p] * X[(size_t)j * nfunc + i];
            prod[(size_t)j * np + p] = (T)s;
        }
    for (size_t p = 0; p < np; p++)
    {
        double acc = 0.;
        for (int j = 0; j < nfunc; j++)
            acc += (double)(T)(prod[(size_t)j * np + p] * psi[(size_t)j * np + p]);
        rho[p] = acc;
    }
    double q = 0.;
    for (size_t p = 0; p < np; p++)
        q += rho[p];
    q *= vel;
    out[0]   = q;
    double t = 1.;
    if (nel > 0. && q > 0.) t = nel / q;
    out[1] = t;
    if (std::fabs(t - 1.) > 0.02) return 1;
    for (size_t p = 0; p < np; p++)
        rho[p] *= t;
    return 0;
}

extern "C" {
int orc_rho_d(const int* n, const double* ll, int nfunc, const double* psi, const double* X,
    double nel, double* rho, double* out)
{
    return rho_t(n, ll, nfunc, psi, X, nel, rho, out);
}
int orc_rho_f(const int* n, const double* ll, int nfunc, const float* psi, const double* X,
    double nel, double* rho, double* out)
{
    return rho_t(n, ll, nfunc, psi, X, nel, rho, out);
}
}
