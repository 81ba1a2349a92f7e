/*
 * ORACLE PINNING DRIVER -- TEST INFRASTRUCTURE ONLY.
 *
 * Calls the reference MGmol's own hot-path code (compiled unmodified from its
 * source tree by oracle/build_ref.sh, against the single-task shims in
 * oracle/shim/) through a small C interface, so that the oracle restatement
 * in oracle/mgx_oracle.cpp can be checked against the reference itself and
 * golden fixtures can be recorded (tests/golden/make_golden.py).
 *
 * This translation unit includes src/Preconditioning.cc to add the FP64
 * instance Preconditioning<double> (the reference instantiates only float,
 * src/Preconditioning.cc:218), and src/MasksSet.cc to reach its file-local
 * mask functions (src/MasksSet.cc:26-48).  Private members of MasksSet and
 * Control and protected members of GridMask are opened for this file only,
 * to register GridMaskMax objects without a LocalizationRegions instance and
 * to define a minimal Control.  Nothing here is part of the product.
 */
// Standard headers first, so that the access override below reaches only
// the reference's own classes.
#include <algorithm>
#include <cassert>
#include <cmath>
#include <complex>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <type_traits>
#include <unordered_map>
#include <vector>

#define private public
#define protected public
#include "Control.h"
#include "GridMask.h"
#include "MasksSet.h"
#undef protected
#undef private

// Minimal Control for the reference's mask code: only the boundary
// conditions and verbosity are read on the path (src/GridMask.cc:146,163,211).
Control* Control::pinstance_   = nullptr;
MPI_Comm Control::comm_global_ = MPI_COMM_WORLD;
#include "mgmol_Signal.h"
std::set<int> Signal::recv_;
Control::Control()
{
    for (int i = 0; i < 3; i++)
    {
        bcWF[i]      = 1;
        bcPoisson[i] = 1;
    }
    verbose = 0;
}

#include "Preconditioning.cc"
template class Preconditioning<double>;

#include "MasksSet.cc"

#include "GridMaskMax.h"
#include "GridMaskMult.h"
#include "Map2Masks.h"
#include "PEenv.h"
#include "pb/Grid.h"
#include "pb/GridFunc.h"
#include "pb/GridFuncVector.h"
#include "pb/MGkernels.h"

#include "pb/Laph2.h"
#include "pb/Laph4.h"
#include "pb/Laph4M.h"
#include "pb/Laph6.h"
#include "pb/Laph8.h"
#include "pb/Mgm.h"
#include "mputils.h"
#include "MGmol_MPI.h"

#include <memory>
#include <vector>

// the V-cycle timers are defined with pb::SolverLap (src/pb/SolverLap.cc:20-23)
Timer vcycle_repwrk_tm("vcycle_repwrk");
Timer vcycle_repinit_tm("vcycle_repinit");
Timer vcycle_repend_tm("vcycle_repend");
Timer vcycle_repvcycle_tm("vcycle_repvcycle");

namespace
{
int ghosts_for(int lap_type)
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

struct Env
{
    pb::PEenv pe;
    // GridFunc::norm2 and friends reach MGmol_MPI::instance()
    Env() : pe(MPI_COMM_WORLD) { MGmol_MPI::setup(MPI_COMM_WORLD, std::cout); }
};
Env& env()
{
    static Env e;
    return e;
}

std::vector<std::vector<int>> make_gids(int nfunc)
{
    std::vector<std::vector<int>> gids(1);
    for (int i = 0; i < nfunc; i++)
        gids[0].push_back(i);
    return gids;
}

template <typename T>
using GFV = pb::GridFuncVector<T, MemorySpace::Host>;

template <typename T, typename S>
void load(GFV<T>& v, const S* src, int nfunc, size_t npts)
{
    for (int i = 0; i < nfunc; i++)
        v.assign(i, src + (size_t)i * npts);
    v.set_updated_boundaries(false);
}
template <typename T, typename S>
void store(const GFV<T>& v, S* dst, int nfunc, size_t npts)
{
    for (int i = 0; i < nfunc; i++)
        v.getValues(i, dst + (size_t)i * npts);
}

pb::Grid make_grid(const int* n, const double* ll, int ng)
{
    const double origin[3] = { 0., 0., 0. };
    const unsigned ngpts[3] = { (unsigned)n[0], (unsigned)n[1], (unsigned)n[2] };
    return pb::Grid(origin, ll, ngpts, env().pe, ng);
}

template <typename T>
int fd_apply(const int* n, const double* ll, int lap_type, int nfunc,
    const T* u, T* out)
{
    pb::Grid g  = make_grid(n, ll, ghosts_for(lap_type));
    auto gids   = make_gids(nfunc);
    GFV<T> a(g, 1, 1, 1, gids), b(g, 1, 1, 1, gids);
    load(a, u, nfunc, g.size());
    a.applyLap(lap_type, b);
    store(b, out, nfunc, g.size());
    return 0;
}

template <typename T>
int rhs_mehr(const int* n, const double* ll, int nfunc, const T* u, T* out)
{
    pb::Grid g = make_grid(n, ll, 1);
    auto gids  = make_gids(nfunc);
    GFV<T> a(g, 1, 1, 1, gids), b(g, 1, 1, 1, gids);
    load(a, u, nfunc, g.size());
    a.applyRHS(0, b);
    store(b, out, nfunc, g.size());
    return 0;
}

/* Hamiltonian<T>::applyLocal, Mehrstellen branch (src/Hamiltonian.cc:106-132),
 * issued as the same sequence of reference calls. */
template <typename T>
int hpsi_mehr(const int* n, const double* ll, int nfunc, const T* psi,
    const double* V, T* hpsi)
{
    pb::Grid g = make_grid(n, ll, 1);
    auto gids  = make_gids(nfunc);
    GFV<T> phi(g, 1, 1, 1, gids);
    load(phi, psi, nfunc, g.size());
    phi.trade_boundaries();
    pb::GridFunc<double> gfpot(g, 1, 1, 1);
    gfpot.assign(V);
    gfpot.trade_boundaries();
    GFV<T> gfvw1(g, 1, 1, 1, gids);
    gfvw1.pointwiseProduct(phi, gfpot);
    GFV<T> work1(g, 1, 1, 1, gids);
    gfvw1.applyRHS(0, work1);
    phi.applyLap(0, gfvw1);
    work1.axpy(1., gfvw1);
    store(work1, hpsi, nfunc, g.size());
    return 0;
}

template <typename T>
int restrict_(const int* n, const double* ll, int nfunc, const T* fine, T* coarse)
{
    pb::Grid fg = make_grid(n, ll, 1);
    pb::Grid cg(fg.coarse_grid());
    auto gids = make_gids(nfunc);
    GFV<T> a(fg, 1, 1, 1, gids), b(cg, 1, 1, 1, gids);
    load(a, fine, nfunc, fg.size());
    a.restrict3D(b);
    store(b, coarse, nfunc, cg.size());
    return 0;
}

template <typename T>
int extend_(const int* n, const double* ll, int nfunc, const T* coarse, T* fine)
{
    pb::Grid fg = make_grid(n, ll, 1);
    pb::Grid cg(fg.coarse_grid());
    auto gids = make_gids(nfunc);
    GFV<T> a(fg, 1, 1, 1, gids), b(cg, 1, 1, 1, gids);
    load(b, coarse, nfunc, cg.size());
    a.extend3D(b);
    store(a, fine, nfunc, fg.size());
    return 0;
}

/* GridMask keeps its per-level SubCell objects in a static vector that the
 * last destructor frees without emptying (src/GridMask.cc:23,87-94); it is
 * emptied here once every mask of a call is gone, so that the next call
 * (possibly on another grid) builds fresh ones. */
void forget_subcells()
{
    if (GridMask::ninstances_ == 0) GridMask::sub_cell_.clear();
}

struct RefMasks
{
    std::unique_ptr<MasksSet> set;
    std::unique_ptr<Map2Masks> map;
};

/* Builds GridMaskMax (kind 0, gaussianDecay) or GridMaskMult (kind 1, one)
 * objects for levels 0..nlevels-1 on the mesh grid g, one per orbital. */
RefMasks* build_masks(const pb::Grid& g, int nlevels, int nfunc,
    const double* centers, const double* radii, int kind)
{
    forget_subcells();
    RefMasks* rm = new RefMasks;
    rm->set.reset(new MasksSet(kind == 1, nlevels - 1));
    std::vector<int> gids;
    for (int f = 0; f < nfunc; f++)
    {
        GridMask* m = nullptr;
        if (kind == 0)
            m = new GridMaskMax(nlevels - 1, 1, g);
        else
            m = new GridMaskMult(nlevels - 1, 1, g);
        const Vector3D c(centers[3 * f], centers[3 * f + 1], centers[3 * f + 2]);
        for (int l = 0; l < nlevels; l++)
            m->init(c, radii[f], l, kind == 1 ? &one : &gaussianDecay);
        rm->set->pgrid_masks_.insert(std::pair<int, GridMask*>(f, m));
        gids.push_back(f);
    }
    rm->map.reset(new Map2Masks(rm->set.get(), gids));
    return rm;
}

/* OrbitalsPreconditioning<T>::precond_mg (src/OrbitalsPreconditioning.cc:86-117)
 * issued as its sequence of reference calls, on Preconditioning<T>. */
template <typename T>
int precond(const int* n, const double* ll, int lap_type, int maxlevels,
    double gamma, int nfunc, const T* res, T* out, int nmask,
    const double* centers, const double* radii, int kind)
{
    pb::Grid g = make_grid(n, ll, ghosts_for(lap_type));
    auto gids  = make_gids(nfunc);
    RefMasks* rm = nullptr;
    if (nmask > 0)
    {
        rm = build_masks(g, maxlevels + 1, nfunc, centers, radii, kind);
        GFV<T>::setMasks(rm->map.get());
    }
    const short bc[3] = { 1, 1, 1 };
    {
        Preconditioning<T> P(lap_type, maxlevels, g, bc);
        P.setup(gids);
        GFV<T> v(g, 1, 1, 1, gids), f(g, 1, 1, 1, gids);
        v.resetData();
        load(f, res, nfunc, g.size());
        v.axpy(gamma, f);
        P.mg(v, f, lap_type, 0);
        store(v, out, nfunc, g.size());
    }
    GFV<T>::setMasks(nullptr);
    delete rm;
    forget_subcells();
    return 0;
}

/* GridMask::init values for every orbital and level (subdomain 0). */
template <typename M>
int mask_build(const int* n, const double* ll, int ng, int nlevels, int nfunc,
    const double* centers, const double* radii, int func, int* state, M* values)
{
    pb::Grid g = make_grid(n, ll, ng);
    forget_subcells();
    std::vector<GridMaskMax*> masks;
    for (int f = 0; f < nfunc; f++)
    {
        GridMaskMax* m = new GridMaskMax(nlevels - 1, 1, g);
        const Vector3D c(centers[3 * f], centers[3 * f + 1], centers[3 * f + 2]);
        for (int l = 0; l < nlevels; l++)
            m->init(c, radii[f], l, func == 1 ? &one : &gaussianDecay);
        masks.push_back(m);
    }
    size_t off = 0;
    for (int l = 0; l < nlevels; l++)
    {
        const size_t ls = (size_t)(n[0] >> l) * (n[1] >> l) * (n[2] >> l);
        for (int f = 0; f < nfunc; f++)
        {
            GridMaskMax& m       = *masks[f];
            state[l * nfunc + f] = m.mask_not_zero(l, 0);
            M* dst               = values + off + (size_t)f * ls;
            if (m.maskIs2(l, 0))
            {
                const lmasktype* src = m.lmask(l, 0);
                for (size_t i = 0; i < ls; i++)
                    dst[i] = (M)src[i];
            }
            else
                for (size_t i = 0; i < ls; i++)
                    dst[i] = (M)(m.maskIs1(l, 0) ? 1. : 0.);
        }
        off += (size_t)nfunc * ls;
    }
    for (auto m : masks)
        delete m;
    forget_subcells();
    return 0;
}
/* pb::Mgm on one field: the reference template itself, with the operator
 * class of lap_type on a fine grid of `ng` ghosts; out = final residual,
 * final relative residual, residual reduction, sweeps, converged. */
template <class Op, typename T>
int mgm_op(const int* n, const double* ll, int ng, int cogr, int max_sweeps,
    double tol, int nu1, int nu2, T* vh, const T* rho, double* out)
{
    pb::Grid g = make_grid(n, ll, ng);
    Op A(g);
    pb::GridFunc<T> gvh(g, 1, 1, 1), grho(g, 1, 1, 1);
    gvh.assign(vh, 'd');
    grho.assign(rho, 'd');
    double fr = 0., frr = 0., red = 0.;
    short nb  = 0;
    const bool conv = pb::Mgm(A, gvh, grho, (short)cogr, (short)max_sweeps, tol,
        (short)nu1, (short)nu2, false, fr, frr, red, nb);
    gvh.init_vect(vh, 'd');
    out[0] = fr;
    out[1] = frr;
    out[2] = red;
    out[3] = nb;
    out[4] = conv ? 1. : 0.;
    return 0;
}

/* LocGridOrbitals::multiplyByMatrix: the reference's MPgemmNN on the block
 * (src/LocGridOrbitals.cc:793-830). */
template <typename T>
int mult_matrix(int numpt, int nfunc, const T* psi, const double* theta, T* out)
{
    LinearAlgebraUtils<MemorySpace::Host>::MPgemmNN(numpt, nfunc, nfunc, 1., psi, numpt,
        theta, nfunc, 0., out, numpt);
    return 0;
}

/* MGmol::computeResidualUsingHPhi (src/MGmol.cc:1227-1290) with applyB:
 * tmp_i = lapop->rhs(psi_i) per function, res = tmp theta (MPgemmNN),
 * res.axpy(-1, hphi) (MPaxpy). */
template <typename T>
int residual(const int* n, const double* ll, int nfunc, const T* psi, const T* hphi,
    const double* theta, T* res)
{
    pb::Grid g = make_grid(n, ll, 1);
    const int np = (int)g.size();
    pb::Laph4M<T> lap(g);
    std::vector<T> tmp((size_t)np * nfunc);
    for (int i = 0; i < nfunc; i++)
    {
        pb::GridFunc<T> gf(g, 1, 1, 1);
        gf.assign(psi + (size_t)i * np, 'd');
        lap.rhs(gf, tmp.data() + (size_t)i * np);
    }
    LinearAlgebraUtils<MemorySpace::Host>::MPgemmNN(np, nfunc, nfunc, 1., tmp.data(), np,
        theta, nfunc, 0., res, np);
    LinearAlgebraUtils<MemorySpace::Host>::MPaxpy(np * nfunc, -1., hphi, res);
    return 0;
}

/* LocGridOrbitals::computeMatB (src/LocGridOrbitals.cc:1428-1487) on one
 * subdomain: LapOper.rhs per function (pb::Laph4M::rhs), MPgemmTN of psi
 * and the result, then the scaling by vel and the |x| > 1e-14 filter of the
 * conversion to the distributed matrix (restated: SquareLocalMatrices::scal
 * and LocalMatrices2DistMatrix::accumulate are outside this build). */
template <typename T>
int matb(const int* n, const double* ll, int nfunc, const T* psi, double* B)
{
    pb::Grid g = make_grid(n, ll, 1);
    const int np = (int)g.size();
    pb::Laph4M<T> lap(g);
    std::vector<T> work((size_t)np * nfunc);
    for (int i = 0; i < nfunc; i++)
    {
        pb::GridFunc<T> gf(g, 1, 1, 1);
        gf.assign(psi + (size_t)i * np, 'd');
        lap.rhs(gf, work.data() + (size_t)i * np);
    }
    MPgemmTN(nfunc, nfunc, np, 1., psi, np, work.data(), np, 0., B, nfunc);
    const double vel = g.vel();
    for (size_t k = 0; k < (size_t)nfunc * nfunc; k++)
    {
        double x = B[k] * vel;
        if (!(std::fabs(x) > 1.e-14)) x = 0.;
        B[k] = x;
    }
    return 0;
}

/* LocGridOrbitals::normalize (src/LocGridOrbitals.cc:2261-2311): diagS_i =
 * vel * MPdot(psi_i, psi_i), then MPscal(1 / sqrt(diagS_i)) per function --
 * the reference's own MPdot / MPscal on one subdomain. */
template <typename T>
int normalize(const int* n, const double* ll, int nfunc, T* psi, double* diag)
{
    pb::Grid g = make_grid(n, ll, 1);
    const int np = (int)g.size();
    const double vel = g.vel();
    for (int i = 0; i < nfunc; i++)
        diag[i] = vel * LinearAlgebraUtils<MemorySpace::Host>::MPdot(np, psi + (size_t)i * np,
                            psi + (size_t)i * np);
    for (int i = 0; i < nfunc; i++)
        LinearAlgebraUtils<MemorySpace::Host>::MPscal(np, 1. / std::sqrt(diag[i]),
            psi + (size_t)i * np);
    return 0;
}

/* Rho<T>::computeRhoSubdomainUsingBlas3 (src/Rho.cc:359-450) on one
 * subdomain: the reference's MPgemmNN for the product, then its O(N^2)
 * loop (product * phi added into the FP64 density; run here in the order j
 * outer, points inner, which the reference leaves to OpenMP atomics).  No
 * rescaling. */
template <typename T>
int rho_blas3(int np, int nfunc, const T* psi, const double* X, double* rho)
{
    std::vector<T> product((size_t)np * nfunc);
    LinearAlgebraUtils<MemorySpace::Host>::MPgemmNN(np, nfunc, nfunc, 1., psi, np, X, nfunc, 0.,
        product.data(), np);
    std::fill(rho, rho + np, 0.);
    for (int j = 0; j < nfunc; ++j)
        for (int i = 0; i < np; ++i)
            rho[i] += product[(size_t)j * np + i] * psi[(size_t)j * np + i];
    return 0;
}

template <typename T>
int mgm(const int* n, const double* ll, int lap_type, int ng, int cogr, int max_sweeps,
    double tol, int nu1, int nu2, T* vh, const T* rho, double* out)
{
    switch (lap_type)
    {
        case 0: return mgm_op<pb::Laph4M<T>, T>(n, ll, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
        case 1: return mgm_op<pb::Laph2<T>, T>(n, ll, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
        case 2: return mgm_op<pb::Laph4<T>, T>(n, ll, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
        case 3: return mgm_op<pb::Laph6<T>, T>(n, ll, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
        case 4: return mgm_op<pb::Laph8<T>, T>(n, ll, ng, cogr, max_sweeps, tol, nu1, nu2, vh, rho, out);
    }
    return 1;
}
} // namespace

extern "C" {
/* The single-task environment (PEenv, MGmol_MPI::setup), set up once per
 * process; the S and H driver (ref_matrices.cpp) needs MGmol_MPI too. */
void ref_env_init() { (void)env(); }
/* pb::Grid::getSinCosFunctions (src/pb/Grid.cc:244-282) in FP64: out holds
 * cos x, sin x (n[0] each), cos y, sin y, cos z, sin z */
int ref_sincos_tables(const int* n, const double* ll, double* out)
{
    pb::Grid g = make_grid(n, ll, 1);
    std::vector<double> sx, sy, sz, cx, cy, cz;
    g.getSinCosFunctions(sx, sy, sz, cx, cy, cz);
    size_t o = 0;
    for (const auto* v : { &cx, &sx, &cy, &sy, &cz, &sz })
        for (double x : *v)
            out[o++] = x;
    return 0;
}
int ref_mult_matrix_d(int np, int nf, const double* p, const double* th, double* o) { return mult_matrix(np, nf, p, th, o); }
int ref_mult_matrix_f(int np, int nf, const float* p, const double* th, float* o) { return mult_matrix(np, nf, p, th, o); }
int ref_residual_d(const int* n, const double* ll, int nf, const double* p, const double* h, const double* th, double* o) { return residual(n, ll, nf, p, h, th, o); }
int ref_residual_f(const int* n, const double* ll, int nf, const float* p, const float* h, const double* th, float* o) { return residual(n, ll, nf, p, h, th, o); }
int ref_rho_d(int np, int nf, const double* p, const double* X, double* r) { return rho_blas3(np, nf, p, X, r); }
int ref_rho_f(int np, int nf, const float* p, const double* X, double* r) { return rho_blas3(np, nf, p, X, r); }
int ref_matb_d(const int* n, const double* ll, int nf, const double* p, double* B) { return matb(n, ll, nf, p, B); }
int ref_matb_f(const int* n, const double* ll, int nf, const float* p, double* B) { return matb(n, ll, nf, p, B); }
int ref_normalize_d(const int* n, const double* ll, int nf, double* p, double* d) { return normalize(n, ll, nf, p, d); }
int ref_normalize_f(const int* n, const double* ll, int nf, float* p, double* d) { return normalize(n, ll, nf, p, d); }
int ref_mgm_d(const int* n, const double* ll, int t, int ng, int cogr, int ms, double tol, int nu1, int nu2, double* vh, const double* rho, double* out)
{ return mgm(n, ll, t, ng, cogr, ms, tol, nu1, nu2, vh, rho, out); }
int ref_mgm_f(const int* n, const double* ll, int t, int ng, int cogr, int ms, double tol, int nu1, int nu2, float* vh, const float* rho, double* out)
{ return mgm(n, ll, t, ng, cogr, ms, tol, nu1, nu2, vh, rho, out); }
int ref_fd_apply_d(const int* n, const double* ll, int t, int nf, const double* u, double* o) { return fd_apply(n, ll, t, nf, u, o); }
int ref_fd_apply_f(const int* n, const double* ll, int t, int nf, const float* u, float* o) { return fd_apply(n, ll, t, nf, u, o); }
int ref_rhs_mehr_d(const int* n, const double* ll, int nf, const double* u, double* o) { return rhs_mehr(n, ll, nf, u, o); }
int ref_rhs_mehr_f(const int* n, const double* ll, int nf, const float* u, float* o) { return rhs_mehr(n, ll, nf, u, o); }
int ref_hpsi_mehr_d(const int* n, const double* ll, int nf, const double* p, const double* V, double* h) { return hpsi_mehr(n, ll, nf, p, V, h); }
int ref_hpsi_mehr_f(const int* n, const double* ll, int nf, const float* p, const double* V, float* h) { return hpsi_mehr(n, ll, nf, p, V, h); }
int ref_restrict_d(const int* n, const double* ll, int nf, const double* a, double* b) { return restrict_(n, ll, nf, a, b); }
int ref_restrict_f(const int* n, const double* ll, int nf, const float* a, float* b) { return restrict_(n, ll, nf, a, b); }
int ref_extend_d(const int* n, const double* ll, int nf, const double* a, double* b) { return extend_(n, ll, nf, a, b); }
int ref_extend_f(const int* n, const double* ll, int nf, const float* a, float* b) { return extend_(n, ll, nf, a, b); }
int ref_precond_d(const int* n, const double* ll, int t, int ml, double gamma, int nf, const double* r, double* o, int nmask, const double* c, const double* rad, int kind)
{ return precond(n, ll, t, ml, gamma, nf, r, o, nmask, c, rad, kind); }
int ref_precond_f(const int* n, const double* ll, int t, int ml, double gamma, int nf, const float* r, float* o, int nmask, const double* c, const double* rad, int kind)
{ return precond(n, ll, t, ml, gamma, nf, r, o, nmask, c, rad, kind); }
int ref_mask_build(const int* n, const double* ll, int ng, int nl, int nf, const double* c, const double* r, int func, int* st, double* v)
{ return mask_build(n, ll, ng, nl, nf, c, r, func, st, v); }
int ref_lmasktype_size() { return (int)sizeof(lmasktype); }
}
