// mgmol_adaptor.h -- MGmol's C++ operator surface for the orbital hot path,
// implemented on the mgx C ABI (include/mgx.h) with device-resident data.
//
// The class and method names, argument meanings and error behaviour follow
// the reference classes they stand in for, so that code written against
// MGmol's surface reads the same:
//   pb::Grid                  src/pb/Grid.h:24-121
//   pb::GridFuncVector<T>     src/pb/GridFuncVector.h:30-493 (MemorySpace::Device)
//   pb::Lap<T>, Laph4M, Laph2, Laph4, Laph6, Laph8
//                             src/pb/Lap.h, src/pb/Laph*.h
//   OrbitalsPreconditioning<T>::precond_mg / setGamma
//                             src/OrbitalsPreconditioning.cc:86-145
//   Hamiltonian<T>::applyLocal src/Hamiltonian.cc:85-159
//   LocGridOrbitals::computeGram / computeLocalProduct
//                             src/LocGridOrbitals.cc:1504-1738
//   GramMatrix::updateLS / computeInverse, ProjectedMatrices::getEigSum
//                             src/GramMatrix.cc:75-191, src/ProjectedMatrices.cc:550-566
//   LocGridOrbitals::computeMatB / normalize
//                             src/LocGridOrbitals.cc:1428-1487,2230-2311
//   ProjectedMatricesMehrstellen::computeInvB / updateTheta / updateHB
//                             src/ProjectedMatricesMehrstellen.cc:38-64,
//                             src/ProjectedMatricesMehrstellen.h:49-62
//   Rho<T>::computeRho (non-orthogonal orbitals) src/Rho.cc:124-450
//   MasksSet::setup / update, applyMask / applyCorrMask
//                             src/MasksSet.cc:136-218, src/LocGridOrbitals.cc:427-480
// Where the reference aborts (unsupported operator, failed Cholesky), these
// classes throw mgx::Error carrying the C-ABI status.  Header only; link
// against libmgx.so and the CUDA runtime.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <stdexcept>
#include <type_traits>
#include <string>
#include <utility>
#include <vector>

#include "../../include/mgx.h"

namespace mgx
{

struct Error : std::runtime_error
{
    int status;
    Error(int s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(int status, const char* where)
{
    if (status != MGX_OK)
        throw Error(status, std::string(where) + ": " + mgx_last_error_string());
}

inline void cuda(cudaError_t e, const char* where)
{
    if (e != cudaSuccess) throw Error(MGX_CUDA_ERROR, std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
constexpr mgx_dtype dtype_of();
template <>
constexpr mgx_dtype dtype_of<double>() { return MGX_F64; }
template <>
constexpr mgx_dtype dtype_of<float>() { return MGX_F32; }

/* owning device array */
template <typename T>
class DeviceArray
{
    T* p_     = nullptr;
    size_t n_ = 0;

public:
    DeviceArray() = default;
    explicit DeviceArray(size_t n) : n_(n)
    {
        if (n) cuda(cudaMalloc(&p_, n * sizeof(T)), "cudaMalloc");
        if (n) cuda(cudaMemset(p_, 0, n * sizeof(T)), "cudaMemset");
    }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    DeviceArray(DeviceArray&& o) noexcept : p_(o.p_), n_(o.n_) { o.p_ = nullptr; o.n_ = 0; }
    DeviceArray& operator=(DeviceArray&& o) noexcept
    {
        if (this != &o)
        {
            if (p_) cudaFree(p_);
            p_   = o.p_;
            n_   = o.n_;
            o.p_ = nullptr;
            o.n_ = 0;
        }
        return *this;
    }
    ~DeviceArray() { if (p_) cudaFree(p_); }
    T* data() { return p_; }
    const T* data() const { return p_; }
    size_t size() const { return n_; }
    void upload(const T* h, size_t n, size_t off = 0)
    {
        cuda(cudaMemcpy(p_ + off, h, n * sizeof(T), cudaMemcpyHostToDevice), "upload");
    }
    void download(T* h, size_t n, size_t off = 0) const
    {
        cuda(cudaMemcpy(h, p_ + off, n * sizeof(T), cudaMemcpyDeviceToHost), "download");
    }
};

namespace pb
{

/* pb::Grid on one task: global = local dimensions, h = ll / n, periodic */
class Grid
{
    mgx_grid g_;
    short ghost_pt_;

public:
    Grid(const double origin[3], const double lattice[3], const unsigned ngpts[3],
        const short nghosts = 1)
        : ghost_pt_(nghosts)
    {
        (void)origin;
        for (int i = 0; i < 3; i++)
        {
            g_.n[i]  = (int)ngpts[i];
            g_.ll[i] = lattice[i];
            g_.bc[i] = 1;
        }
    }
    Grid(const Grid& g, const short nghosts) : g_(g.g_), ghost_pt_(nghosts < 0 ? g.ghost_pt_ : nghosts) {}
    unsigned dim(short i) const { return (unsigned)g_.n[i]; }
    short ghost_pt() const { return ghost_pt_; }
    double hgrid(short i) const { return g_.ll[i] / (double)g_.n[i]; }
    double ll(short i) const { return g_.ll[i]; }
    double vel() const { return hgrid(0) * hgrid(1) * hgrid(2); }
    unsigned size() const { return (unsigned)(g_.n[0] * g_.n[1] * g_.n[2]); }
    unsigned sizeg() const
    {
        return (unsigned)((g_.n[0] + 2 * ghost_pt_) * (g_.n[1] + 2 * ghost_pt_)
                          * (g_.n[2] + 2 * ghost_pt_));
    }
    int inc(short i) const
    {
        if (i == 0) return (g_.n[1] + 2 * ghost_pt_) * (g_.n[2] + 2 * ghost_pt_);
        if (i == 1) return g_.n[2] + 2 * ghost_pt_;
        return 1;
    }
    /* src/pb/Grid.cc:214-231: half the points, same lattice and ghosts */
    Grid coarse_grid() const
    {
        Grid c(*this, -1);
        for (int i = 0; i < 3; i++)
            c.g_.n[i] = g_.n[i] / 2;
        return c;
    }
    const mgx_grid& raw() const { return g_; }
};

/* a device block of nfunc ghosted functions (GridFuncVector<T, Device>) */
template <typename T>
class GridFuncVector
{
    const Grid& grid_;
    int nfunc_;
    DeviceArray<T> mem_;
    bool updated_boundaries_ = false;

public:
    GridFuncVector(const Grid& g, int nfunc)
        : grid_(g), nfunc_(nfunc), mem_((size_t)nfunc * g.sizeg())
    {
    }
    const Grid& grid() const { return grid_; }
    int size() const { return nfunc_; }
    T* data() { return mem_.data(); }
    const T* data() const { return mem_.data(); }
    void set_updated_boundaries(bool f) { updated_boundaries_ = f; }
    void resetData()
    {
        cuda(cudaMemset(mem_.data(), 0, mem_.size() * sizeof(T)), "resetData");
        updated_boundaries_ = true;
    }
    /* values of function i without ghosts (x-slowest, z-fastest) */
    void assign(int i, const T* src)
    {
        const int g = grid_.ghost_pt();
        std::vector<T> tmp(grid_.sizeg(), (T)0);
        for (unsigned x = 0; x < grid_.dim(0); x++)
            for (unsigned y = 0; y < grid_.dim(1); y++)
                for (unsigned z = 0; z < grid_.dim(2); z++)
                    tmp[(x + g) * grid_.inc(0) + (y + g) * grid_.inc(1) + z + g]
                        = src[((size_t)x * grid_.dim(1) + y) * grid_.dim(2) + z];
        mem_.upload(tmp.data(), tmp.size(), (size_t)i * grid_.sizeg());
        updated_boundaries_ = false;
    }
    void getValues(int i, T* dst) const
    {
        const int g = grid_.ghost_pt();
        std::vector<T> tmp(grid_.sizeg());
        mem_.download(tmp.data(), tmp.size(), (size_t)i * grid_.sizeg());
        for (unsigned x = 0; x < grid_.dim(0); x++)
            for (unsigned y = 0; y < grid_.dim(1); y++)
                for (unsigned z = 0; z < grid_.dim(2); z++)
                    dst[((size_t)x * grid_.dim(1) + y) * grid_.dim(2) + z]
                        = tmp[(x + g) * grid_.inc(0) + (y + g) * grid_.inc(1) + z + g];
    }
    /* src/pb/GridFuncVector.cc:1543-1621 */
    void trade_boundaries()
    {
        if (updated_boundaries_) return;
        check(mgx_trade_boundaries(&grid_.raw(), grid_.ghost_pt(), dtype_of<T>(), data(),
                  nfunc_, nullptr),
            "GridFuncVector::trade_boundaries");
        updated_boundaries_ = true;
    }
    /* src/pb/GridFuncVector.cc:2369-2397 */
    void applyLap(int type, GridFuncVector& rhs)
    {
        trade_boundaries();
        check(mgx_fdkernel_del2(&grid_.raw(), grid_.ghost_pt(), type, dtype_of<T>(), data(),
                  rhs.data(), nfunc_, nullptr),
            "GridFuncVector::applyLap");
        rhs.updated_boundaries_ = false;
    }
    /* src/pb/GridFuncVector.cc:2399-2413 */
    void applyRHS(int type, GridFuncVector& rhs)
    {
        if (type == 0)
        {
            trade_boundaries();
            check(mgx_fdkernel_rhs_mehr1(&grid_.raw(), grid_.ghost_pt(), dtype_of<T>(), data(),
                      rhs.data(), grid_.ghost_pt(), nfunc_, nullptr),
                "GridFuncVector::applyRHS");
        }
        else
            cuda(cudaMemcpy(rhs.data(), data(), (size_t)nfunc_ * grid_.sizeg() * sizeof(T),
                     cudaMemcpyDeviceToDevice),
                "applyRHS copy");
        rhs.updated_boundaries_ = false;
    }
    /* src/pb/GridFuncVector.cc:1660-1668 */
    void axpy(double alpha, const GridFuncVector& x)
    {
        check(mgx_axpy((size_t)nfunc_ * grid_.sizeg(), alpha, dtype_of<T>(), x.data(), data(),
                  nullptr),
            "GridFuncVector::axpy");
        updated_boundaries_ = updated_boundaries_ && x.updated_boundaries_;
    }
    GridFuncVector& operator-=(const GridFuncVector& x)
    {
        axpy(-1., x);
        return *this;
    }
    /* src/pb/GridFuncVector.cc:2415-2425: w = A v - f; v -= jf w */
    void jacobi(int type, const GridFuncVector& B, GridFuncVector& w, double jacobiFactor)
    {
        applyLap(type, w);
        w -= B;
        axpy(-1. * jacobiFactor, w);
        set_updated_boundaries(false);
    }
    /* src/pb/GridFuncVector.cc:1623-1641 */
    void restrict3D(GridFuncVector& coarse)
    {
        check(mgx_mgkernel_restrict3d(&grid_.raw(), grid_.ghost_pt(), dtype_of<T>(), data(),
                  coarse.data(), nfunc_, nullptr),
            "GridFuncVector::restrict3D");
        coarse.updated_boundaries_ = false;
    }
    void extend3D(GridFuncVector& coarse)
    {
        coarse.trade_boundaries();
        check(mgx_mgkernel_extend3d(&grid_.raw(), grid_.ghost_pt(), dtype_of<T>(), coarse.data(),
                  data(), nfunc_, nullptr),
            "GridFuncVector::extend3D");
        updated_boundaries_ = false;
    }
};

/* operator objects: diagonal, Jacobi factor, apply (src/pb/Laph*.h) */
template <typename T>
class Lap
{
protected:
    const Grid& grid_;
    double inv_h2(int i) const { return 1. / (grid_.hgrid(i) * grid_.hgrid(i)); }
    double sum_inv_h2() const { return inv_h2(0) + inv_h2(1) + inv_h2(2); }

public:
    explicit Lap(const Grid& g) : grid_(g) {}
    virtual ~Lap() {}
    virtual int type() const            = 0;
    virtual double diagEl() const       = 0;
    virtual double jacobiFactor() const = 0;
    double invDiagEl() const { return 1. / diagEl(); }
    /* B = -Lap A (A's ghosts traded first) */
    void apply(GridFuncVector<T>& A, GridFuncVector<T>& B) { A.applyLap(type(), B); }
    void rhs(GridFuncVector<T>& A, GridFuncVector<T>& B) { A.applyRHS(type(), B); }
    void jacobi(GridFuncVector<T>& A, const GridFuncVector<T>& B, GridFuncVector<T>& W)
    {
        A.jacobi(type(), B, W, jacobiFactor());
    }
};

template <typename T>
struct Laph4M : Lap<T>
{
    using Lap<T>::Lap;
    int type() const override { return 0; }
    double diagEl() const override { return (4. / 3.) * this->sum_inv_h2(); }
    double jacobiFactor() const override { return this->invDiagEl(); }
};
template <typename T>
struct Laph2 : Lap<T>
{
    using Lap<T>::Lap;
    int type() const override { return 1; }
    double diagEl() const override { return 2. * this->sum_inv_h2(); }
    double jacobiFactor() const override { return 6. * this->invDiagEl() / 7.; }
};
template <typename T>
struct Laph4 : Lap<T>
{
    using Lap<T>::Lap;
    int type() const override { return 2; }
    double diagEl() const override { return 2.5 * this->sum_inv_h2(); }
    double jacobiFactor() const override { return this->invDiagEl() / 1.5; }
};
template <typename T>
struct Laph6 : Lap<T>
{
    using Lap<T>::Lap;
    int type() const override { return 3; }
    double diagEl() const override { return (49. / 18.) * this->sum_inv_h2(); }
    double jacobiFactor() const override { return this->invDiagEl() / 1.5; }
};
template <typename T>
struct Laph8 : Lap<T>
{
    using Lap<T>::Lap;
    int type() const override { return 4; }
    double diagEl() const override { return (1435. / 504.) * this->sum_inv_h2(); }
    double jacobiFactor() const override { return this->invDiagEl() / 1.5; }
};

} // namespace pb

/* A device block of orbitals without ghosts (BlockVector layout) with the
 * LocGridOrbitals products and the hot-path operators on it. */
template <typename T>
class OrbitalBlock
{
    mgx_ctx* ctx_ = nullptr;
    const pb::Grid& grid_;
    int nfunc_;
    DeviceArray<T> psi_;

public:
    OrbitalBlock(const pb::Grid& g, int nfunc) : grid_(g), nfunc_(nfunc), psi_((size_t)nfunc * g.size())
    {
        check(mgx_create(&g.raw(), &ctx_), "mgx_create");
    }
    ~OrbitalBlock() { mgx_destroy(ctx_); }
    OrbitalBlock(const OrbitalBlock&) = delete;
    int chromatic_number() const { return nfunc_; }
    size_t numpt() const { return grid_.size(); }
    T* psi(int i) { return psi_.data() + (size_t)i * numpt(); }
    const T* psi(int i) const { return psi_.data() + (size_t)i * numpt(); }
    mgx_ctx* ctx() const { return ctx_; }
    void set(const T* host) { psi_.upload(host, psi_.size()); }
    void get(T* host) const { psi_.download(host, psi_.size()); }

    /* LocGridOrbitals::computeGram: S = Psi^T Psi vel (device, n x n) */
    void computeGram(DeviceArray<double>& S, int mode = -1) const
    {
        if (mode < 0) mode = std::is_same<T, double>::value ? MGX_GEMM_FP64 : MGX_GEMM_BF16X3;
        check(mgx_gram(ctx_, mode, psi_.data(), numpt(), nfunc_, S.data(), nullptr),
            "LocGridOrbitals::computeGram");
    }
    /* LocGridOrbitals::computeLocalProduct(orbitals, ss): H(i,j) = <psi_i, other_j> vel */
    void computeLocalProduct(const OrbitalBlock& other, DeviceArray<double>& H, int mode = -1) const
    {
        if (mode < 0) mode = std::is_same<T, double>::value ? MGX_GEMM_FP64 : MGX_GEMM_BF16X3;
        check(mgx_hmat(ctx_, mode, psi_.data(), other.psi(0), numpt(), nfunc_, H.data(), nullptr),
            "LocGridOrbitals::computeLocalProduct");
    }
    /* LocGridOrbitals::multiplyByMatrix(matrix, product): product_j =
     * sum_i psi_i theta(i, j), theta FP64 column-major on the device */
    void multiplyByMatrix(const DeviceArray<double>& theta, OrbitalBlock& product, int mode = -1) const
    {
        if (mode < 0) mode = MGX_GEMM_FP64;
        check(mgx_mult_matrix(ctx_, mode, dtype_of<T>(), psi_.data(), numpt(), nfunc_,
                  theta.data(), product.psi(0), nullptr),
            "LocGridOrbitals::multiplyByMatrix");
    }
    /* LocGridOrbitals::computeMatB(orbitals, LapOper): B = Psi^T (B Psi) vel
     * with the Mehrstellen right-hand side (device, n x n, symmetric) */
    void computeMatB(DeviceArray<double>& B, int mode = -1) const
    {
        if (mode < 0) mode = std::is_same<T, double>::value ? MGX_GEMM_FP64 : MGX_GEMM_BF16X3;
        check(mgx_matb(ctx_, mode, psi_.data(), numpt(), nfunc_, B.data(), nullptr, 0, nullptr),
            "LocGridOrbitals::computeMatB");
    }
    /* LocGridOrbitals::normalize: psi_i /= sqrt(vel |psi_i|^2); throws
     * (status MGX_NOT_SPD) where the reference asserts */
    void normalize()
    {
        check(mgx_normalize(ctx_, dtype_of<T>(), psi_.data(), numpt(), nfunc_, nullptr, nullptr),
            "LocGridOrbitals::normalize");
    }
    /* LocGridOrbitals::axpy: psi += alpha x */
    void axpy(double alpha, const OrbitalBlock& x)
    {
        check(mgx_axpy(psi_.size(), alpha, dtype_of<T>(), x.psi(0), psi_.data(), nullptr),
            "LocGridOrbitals::axpy");
    }
};

/* Hamiltonian<T>::applyLocal: hphi = -Lap_M phi + B(V phi) (Mehrstellen)
 * or -Lap phi + V phi; V has one FP64 value per grid point (device) */
template <typename T>
class Hamiltonian
{
    int lap_type_;

public:
    explicit Hamiltonian(int lap_type) : lap_type_(lap_type) {}
    void applyLocal(OrbitalBlock<T>& phi, const DeviceArray<double>& vtot, OrbitalBlock<T>& hphi)
    {
        check(mgx_hpsi(phi.ctx(), lap_type_, dtype_of<T>(), phi.psi(0), phi.numpt(), vtot.data(),
                  MGX_F64, hphi.psi(0), phi.chromatic_number(), lap_type_ == 0 ? 1 : 0, nullptr),
            "Hamiltonian::applyLocal");
    }
};

/* OrbitalsPreconditioning<T>: V-cycle preconditioner of an orbital block */
template <typename T>
class OrbitalsPreconditioning
{
    short mg_levels_ = 0, lap_type_ = 0;
    double gamma_    = 0.;
    const mgx_masks* masks_ = nullptr;

public:
    void setup(short mg_levels, short lap_type, const mgx_masks* masks = nullptr)
    {
        mg_levels_ = mg_levels;
        lap_type_  = lap_type;
        masks_     = masks;
    }
    /* src/OrbitalsPreconditioning.cc:119-145 */
    void setGamma(const pb::Grid& g, double vmax, double small_eig)
    {
        check(mgx_precond_gamma(&g.raw(), lap_type_, mg_levels_, vmax, small_eig, &gamma_),
            "OrbitalsPreconditioning::setGamma");
    }
    double gamma() const { return gamma_; }
    /* res <- V-cycle(res) (src/OrbitalsPreconditioning.cc:86-117) */
    void precond_mg(OrbitalBlock<T>& res)
    {
        DeviceArray<T> out(res.numpt() * res.chromatic_number());
        mgx_precond_params p{ lap_type_, mg_levels_, gamma_, 0 };
        check(mgx_precond_mg(res.ctx(), &p, dtype_of<T>(), res.psi(0), res.numpt(), out.data(),
                  res.chromatic_number(), masks_, nullptr),
            "OrbitalsPreconditioning::precond_mg");
        cuda(cudaMemcpy(res.psi(0), out.data(), out.size() * sizeof(T), cudaMemcpyDeviceToDevice),
            "precond_mg copy");
    }
};

/* MGmol::computeResidualUsingHPhi: res = B(psi) theta - hphi (applyB) or
 * psi theta - hphi; res may be hphi itself */
template <typename T>
void computeResidualUsingHPhi(const OrbitalBlock<T>& psi, const OrbitalBlock<T>& hphi,
    const DeviceArray<double>& theta, OrbitalBlock<T>& res, bool applyB, int mode = -1)
{
    if (mode < 0) mode = MGX_GEMM_FP64;
    check(mgx_residual(psi.ctx(), mode, dtype_of<T>(), psi.psi(0), hphi.psi(0), psi.numpt(),
              psi.chromatic_number(), theta.data(), applyB ? 1 : 0, nullptr, res.psi(0), nullptr),
        "MGmol::computeResidualUsingHPhi");
}

/* GramMatrix: Cholesky factor, inverse and the energy trace, FP64 device */
class GramMatrix
{
    mgx_ctx* ctx_;
    int n_;
    DeviceArray<double> ls_, inv_;

public:
    GramMatrix(mgx_ctx* ctx, int n) : ctx_(ctx), n_(n), ls_((size_t)n * n), inv_((size_t)n * n) {}
    /* src/GramMatrix.cc:166-191; throws (status MGX_NOT_SPD) where the
     * reference aborts */
    void setMatrix(const DeviceArray<double>& S)
    {
        cuda(cudaMemcpy(ls_.data(), S.data(), (size_t)n_ * n_ * 8, cudaMemcpyDeviceToDevice),
            "GramMatrix copy");
        int info = 0;
        check(mgx_cholesky(ctx_, n_, ls_.data(), &info, nullptr), "GramMatrix::updateLS");
        check(mgx_inverse_from_cholesky(ctx_, n_, ls_.data(), inv_.data(), nullptr),
            "GramMatrix::computeInverse");
    }
    const DeviceArray<double>& getInverse() const { return inv_; }
    /* ProjectedMatrices::updateTheta: theta = S^-1 H (FP64 column-major) */
    void updateTheta(const DeviceArray<double>& H, DeviceArray<double>& theta) const
    {
        check(mgx_theta(ctx_, n_, inv_.data(), H.data(), theta.data(), nullptr),
            "ProjectedMatrices::updateTheta");
    }
    const DeviceArray<double>& getCholeskyL() const { return ls_; }
    /* ProjectedMatrices::getEigSum: tr(H S^-1) in Ry */
    double traceProduct(const DeviceArray<double>& H) const
    {
        DeviceArray<double> t(1);
        check(mgx_trace_prod(ctx_, n_, H.data(), inv_.data(), t.data(), nullptr), "getEigSum");
        double v = 0.;
        t.download(&v, 1);
        return v;
    }
};

/* ProjectedMatricesMehrstellen: the matrix B of the Mehrstellen
 * generalized eigenproblem, its inverse, theta = B^-1 H and HB (FP64
 * column-major device matrices) */
class ProjectedMatricesMehrstellen
{
    mgx_ctx* ctx_;
    int n_;
    DeviceArray<double> matB_, ls_, invB_;

public:
    ProjectedMatricesMehrstellen(mgx_ctx* ctx, int n)
        : ctx_(ctx), n_(n), matB_((size_t)n * n), ls_((size_t)n * n), invB_((size_t)n * n)
    {
    }
    /* initializeMatB(ss): B from LocGridOrbitals::computeMatB */
    void initializeMatB(const DeviceArray<double>& B)
    {
        cuda(cudaMemcpy(matB_.data(), B.data(), (size_t)n_ * n_ * 8, cudaMemcpyDeviceToDevice),
            "initializeMatB copy");
    }
    /* computeInvB (src/ProjectedMatricesMehrstellen.cc:38-64): potrf + potri
     * with uplo 'l'; throws (status MGX_NOT_SPD) where the reference prints
     * the matrix and carries on */
    void computeInvB()
    {
        cuda(cudaMemcpy(ls_.data(), matB_.data(), (size_t)n_ * n_ * 8, cudaMemcpyDeviceToDevice),
            "computeInvB copy");
        int info = 0;
        check(mgx_cholesky(ctx_, n_, ls_.data(), &info, nullptr), "computeInvB potrf");
        check(mgx_inverse_from_cholesky(ctx_, n_, ls_.data(), invB_.data(), nullptr),
            "computeInvB potri");
    }
    const DeviceArray<double>& getInvB() const { return invB_; }
    /* updateTheta: theta = invB H (symm 'l', 'l') */
    void updateTheta(const DeviceArray<double>& H, DeviceArray<double>& theta) const
    {
        check(mgx_theta(ctx_, n_, invB_.data(), H.data(), theta.data(), nullptr),
            "ProjectedMatricesMehrstellen::updateTheta");
    }
    /* updateHB: HB = sym(S theta) */
    void updateHB(const DeviceArray<double>& S, const DeviceArray<double>& theta,
        DeviceArray<double>& HB) const
    {
        check(mgx_update_hb(ctx_, n_, S.data(), theta.data(), HB.data(), nullptr),
            "ProjectedMatricesMehrstellen::updateHB");
    }
};

/* MasksSet: the localization masks of nfunc orbitals at every multigrid
 * level (GridMaskMax, profile gaussianDecay, or GridMaskMult with profile
 * one for the correction masks), device-resident */
class MasksSet
{
    mgx_ctx* ctx_;
    mgx_masks* m_ = nullptr;

public:
    /* MasksSet::setup from centres (nfunc x 3) and radii (host arrays) */
    MasksSet(mgx_ctx* ctx, int nlevels, int nfunc, const double* centers, const double* radii,
        int func, int kind, int mesh_ghosts, mgx_dtype type)
        : ctx_(ctx)
    {
        check(mgx_masks_create(ctx, nlevels, nfunc, centers, radii, func, kind, mesh_ghosts, type,
                  &m_, nullptr),
            "MasksSet::setup");
    }
    ~MasksSet() { mgx_masks_destroy(m_); }
    MasksSet(const MasksSet&) = delete;
    /* MasksSet::update (src/MasksSet.cc:208-218): new centres and radii */
    void update(const double* centers, const double* radii)
    {
        check(mgx_masks_update(ctx_, m_, centers, radii, nullptr), "MasksSet::update");
    }
    /* LocGridOrbitals::applyMask / applyCorrMask on a block of the level */
    template <typename T>
    void apply(OrbitalBlock<T>& block, int level = 0) const
    {
        check(mgx_masks_apply(ctx_, m_, level, block.psi(0), block.numpt(), block.chromatic_number(),
                  nullptr),
            "MasksSet::apply");
    }
    const mgx_masks* get() const { return m_; }
};

/* SpreadsAndCenters<T> (src/SpreadsAndCenters.h) for one block: the
 * diagonal position-matrix elements on the device, read back once, then
 * the centres and spreads on the host as computeCenter / computeSpread2 do
 * (src/SpreadsAndCenters.cc:26-104). */
template <typename T>
class SpreadsAndCenters
{
    double cell_[3];
    std::vector<double> r_; // nfunc x 6: cos x, sin x, cos y, sin y, cos z, sin z

public:
    explicit SpreadsAndCenters(const pb::Grid& g)
    {
        for (int i = 0; i < 3; i++)
            cell_[i] = g.raw().ll[i];
    }
    /* computePositionMatrix(orbitals) (the functions need not be normalized) */
    void computePositionMatrix(const OrbitalBlock<T>& orbitals, bool normalized = false)
    {
        const int nf = orbitals.chromatic_number();
        DeviceArray<double> a((size_t)nf * 6);
        check(mgx_sincos_diag(orbitals.ctx(), dtype_of<T>(), orbitals.psi(0), orbitals.numpt(),
                  nf, normalized ? 1 : 0, a.data(), nullptr),
            "SpreadsAndCenters::computePositionMatrix");
        r_.resize((size_t)nf * 6);
        cuda(cudaMemcpy(r_.data(), a.data(), r_.size() * sizeof(double), cudaMemcpyDeviceToHost),
            "SpreadsAndCenters::computePositionMatrix");
    }
    int size() const { return (int)(r_.size() / 6); }
    /* the centre of orbital i, each coordinate in [0, L) */
    std::array<double, 3> computeCenter(int i) const
    {
        std::array<double, 3> x;
        for (int d = 0; d < 3; d++)
        {
            double v = cell_[d] * (0.5 * M_1_PI) * std::atan2(r_.at(6 * i + 2 * d + 1),
                                                       r_.at(6 * i + 2 * d));
            if (v < 0.) v += cell_[d];
            x[d] = v;
        }
        return x;
    }
    double computeSpread2(int i) const
    {
        double s = 0.;
        for (int d = 0; d < 3; d++)
        {
            const double lby2pi = 0.5 * M_1_PI * cell_[d];
            const double c = r_.at(6 * i + 2 * d), sn = r_.at(6 * i + 2 * d + 1);
            s += lby2pi * lby2pi - c * c - sn * sn;
        }
        return s;
    }
    double computeSpread(int i) const { return std::sqrt(computeSpread2(i)); }
};

/* LocalizationRegions with one task: centres (nfunc x 3, bohr) and float
 * radii, moved to the orbitals' centres and resized from their spreads
 * (moveTo / move, updateRadii, getMeanRadius of
 * src/LocalizationRegions.cc); centers() and radii() feed MasksSet::update
 * (as doubles) and FunctionsPacking. */
class LocalizationRegions
{
    double cell_[3];
    std::vector<double> centers_;
    std::vector<float> radii_;

public:
    LocalizationRegions(const pb::Grid& g, std::vector<double> centers, std::vector<float> radii)
        : centers_(std::move(centers)), radii_(std::move(radii))
    {
        for (int i = 0; i < 3; i++)
            cell_[i] = g.raw().ll[i];
        if (centers_.size() != 3 * radii_.size())
            throw Error(MGX_BAD_ARG, "LocalizationRegions: one radius per centre");
    }
    int size() const { return (int)radii_.size(); }
    /* moveTo(target_centers), the largest move before the 1-bohr cap */
    float moveTo(const std::vector<double>& targets)
    {
        if (targets.size() != centers_.size())
            throw Error(MGX_BAD_ARG, "LocalizationRegions::moveTo: one target per centre");
        float mx = 0.f;
        check(mgx_regions_move_to(size(), centers_.data(), targets.data(), cell_, &mx),
            "LocalizationRegions::moveTo");
        return mx;
    }
    /* move(sc): to the centres of the orbitals */
    template <typename T>
    float move(const SpreadsAndCenters<T>& sc)
    {
        std::vector<double> t(centers_.size());
        for (int f = 0; f < size(); f++)
        {
            const auto c = sc.computeCenter(f);
            for (int d = 0; d < 3; d++)
                t[3 * f + d] = c[d];
        }
        return moveTo(t);
    }
    /* updateRadii(sc, ratio): the radii from the spreads; getMeanRadius() */
    template <typename T>
    float updateRadii(const SpreadsAndCenters<T>& sc, float ratio)
    {
        std::vector<double> sp(size());
        for (int f = 0; f < size(); f++)
            sp[f] = sc.computeSpread(f);
        float mean = 0.f;
        check(mgx_regions_update_radii(size(), sp.data(), ratio, radii_.data(), &mean),
            "LocalizationRegions::updateRadii");
        return mean;
    }
    const std::vector<double>& centers() const { return centers_; }
    const std::vector<float>& radii() const { return radii_; }
};

/* FunctionsPacking with one task (src/FunctionsPacking.h): the colour of
 * each gid, from the localization regions' centres (nfunc x 3) and float
 * radii, the mesh's x sub-boxes and the grid's ghost width; RLF or greedy
 * colouring as Control::RLFColoring() selects.  Host only. */
class FunctionsPacking
{
    std::vector<int> gid2color_;
    int num_colors_ = 0;

public:
    FunctionsPacking(const pb::Grid& g, const double* centers, const float* radii, int nfunc,
        int subdivx, bool rlf)
        : gid2color_(nfunc)
    {
        check(mgx_pack_functions(&g.raw(), g.ghost_pt(), nfunc, centers, radii, subdivx,
                  rlf ? 1 : 0, gid2color_.data(), &num_colors_),
            "FunctionsPacking::setup");
    }
    short getNumColors() const { return (short)num_colors_; }
    int getGlobalSize() const { return (int)gid2color_.size(); }
    short getColor(int gid) const { return (short)gid2color_.at(gid); }
};

/* Rho<T>: the electronic density of a block of non-orthogonal orbitals
 * (device, one FP64 value per grid point) */
template <typename T>
class Rho
{
    DeviceArray<double> rho_;

public:
    explicit Rho(const pb::Grid& g) : rho_(g.size()) {}
    /* computeRho(orbitals, dm) then rescaleTotalCharge to nel electrons
     * (src/Rho.cc:282-320, 124-200); throws where the reference aborts.
     * Returns the charge before the rescaling. */
    double computeRho(const OrbitalBlock<T>& orbitals, const DeviceArray<double>& dm, double nel,
        int mode = -1)
    {
        if (mode < 0) mode = std::is_same<T, double>::value ? MGX_GEMM_FP64 : MGX_GEMM_BF16X3;
        double q = 0.;
        check(mgx_rho(orbitals.ctx(), mode, dtype_of<T>(), orbitals.psi(0), orbitals.numpt(),
                  orbitals.chromatic_number(), dm.data(), nel, rho_.data(), &q, nullptr, 0,
                  nullptr),
            "Rho::computeRho");
        return q;
    }
    const DeviceArray<double>& rho() const { return rho_; }
};

namespace pb
{
/* pb::Mgm(A, vh, rho, cogr, max_sweeps, tol, nu1, nu2, gather_coarse_level,
 * final_residual, final_relative_residual, residual_reduction, nb_sweeps)
 * (src/pb/Mgm.h:20-26) on one device field of the grid; A is one of the
 * Laph* operators above.  Returns whether the solve converged. */
template <typename T, class Op>
bool Mgm(const Op& A, const Grid& grid, T* vh, const T* rho, short cogr, short max_sweeps,
    double tol, short nu1, short nu2, bool /*gather_coarse_level*/, double& final_residual,
    double& final_relative_residual, double& residual_reduction, short& nb_sweeps,
    int ghosts = 0)
{
    mgx_ctx* ctx = nullptr;
    check(mgx_create(&grid.raw(), &ctx), "mgx_create");
    mgx_mgm_params p{ A.type(), cogr, max_sweeps, tol, nu1, nu2, ghosts };
    mgx_mgm_result r{};
    const int st = mgx_mgm(ctx, &p, dtype_of<T>(), vh, rho, &r, nullptr);
    mgx_destroy(ctx);
    check(st, "pb::Mgm");
    final_residual          = r.final_residual;
    final_relative_residual = r.final_relative_residual;
    residual_reduction      = r.residual_reduction;
    nb_sweeps               = (short)r.nb_sweeps;
    return r.converged != 0;
}
} // namespace pb

} // namespace mgx
