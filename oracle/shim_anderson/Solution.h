/*
 * ORACLE PINNING SHIM -- TEST INFRASTRUCTURE ONLY.
 *
 * The reference's AndersonMix.cc, compiled with TESTING, instantiates
 * AndersonMix<Solution>.  This header supplies that type as a block of
 * orbitals with LocGridOrbitals' element semantics, built on the
 * reference's own mixed-precision kernels (src/linear_algebra/mputils.cc):
 *   copy-construction / assign   BlockVector copy
 *   operator-=                   BlockVector::operator-= (v -= s in the
 *                                storage type, src/BlockVector.cc:289-299)
 *   axpy, scal                   MPaxpy, MPscal
 *   dotProduct                   LocGridOrbitals::dotProductDiagonal:
 *                                sum_k (double)(MPdot_k * vel) * invS(k, k)
 *                                (src/LocGridOrbitals.cc:1606-1630,1783-1799,
 *                                src/GramMatrix.cc:303-310)
 * Solution is a macro naming SolutionF (float storage) or SolutionD (double
 * storage), one instantiation per translation unit.
 */
#ifndef ORACLE_SHIM_ANDERSON_SOLUTION_H
#define ORACLE_SHIM_ANDERSON_SOLUTION_H

#include <string>
#include <vector>

#include "mputils.h"

template <typename T>
class BlockSolution
{
    std::vector<T> u_;

public:
    // geometry and dot-product weights shared by every block of a run
    static int nfunc_, npts_;
    static double vel_;
    static std::vector<double> invs_diag_;

    BlockSolution() : u_((size_t)nfunc_ * npts_) {}
    BlockSolution(const std::string&, const BlockSolution& y) : u_(y.u_) {}
    void assign(const BlockSolution& y) { u_ = y.u_; }
    T* data() { return u_.data(); }
    const T* data() const { return u_.data(); }

    BlockSolution& operator-=(const BlockSolution& y)
    {
        for (size_t i = 0; i < u_.size(); i++)
            u_[i] -= y.u_[i];
        return *this;
    }
    void axpy(const double alpha, const BlockSolution& y)
    {
        LinearAlgebraUtils<MemorySpace::Host>::MPaxpy((int)u_.size(), alpha, y.u_.data(),
            u_.data());
    }
    void scal(const double alpha)
    {
        LinearAlgebraUtils<MemorySpace::Host>::MPscal((int)u_.size(), alpha, u_.data());
    }
    double dotProduct(const BlockSolution& v) const
    {
        std::vector<double> ss(nfunc_, 0.);
        for (int k = 0; k < nfunc_; k++)
        {
            const double alpha = LinearAlgebraUtils<MemorySpace::Host>::MPdot(npts_,
                v.u_.data() + (size_t)k * npts_, u_.data() + (size_t)k * npts_);
            ss[k] += alpha * vel_;
        }
        double tr = 0.;
        for (int k = 0; k < nfunc_; k++)
            tr += ss[k] * invs_diag_[k];
        return tr;
    }
};

template <typename T> int BlockSolution<T>::nfunc_ = 0;
template <typename T> int BlockSolution<T>::npts_  = 0;
template <typename T> double BlockSolution<T>::vel_ = 1.;
template <typename T> std::vector<double> BlockSolution<T>::invs_diag_;

using SolutionF = BlockSolution<float>;
using SolutionD = BlockSolution<double>;

#endif
