/*
 * SINGLE-TASK STAND-IN FOR dist_matrix::DistMatrix -- TEST INFRASTRUCTURE ONLY.
 *
 * Lets the reference's src/LocalMatrices2DistMatrix.cc compile unmodified
 * without ScaLAPACK: one task owns the whole matrix, stored dense and
 * column-major.  Only what LocalMatrices2DistMatrix::accumulate touches
 * (m(), and the sparse matrix below adding into it) is provided.
 */
#ifndef MGX_SHIM_DISTMATRIX_H
#define MGX_SHIM_DISTMATRIX_H

#include <mpi.h>

#include <algorithm>
#include <vector>

// the element type of the distributed matrices (src/DistMatrix/DistMatrix.h:35)
typedef double DISTMATDTYPE;

namespace dist_matrix
{
template <class T>
class DistMatrix
{
    int m_;
    int n_;
    std::vector<T> val_;

public:
    DistMatrix(const int m, const int n) : m_(m), n_(n), val_((size_t)m * n, T(0)) {}
    int m() const { return m_; }
    int n() const { return n_; }
    void clear() { std::fill(val_.begin(), val_.end(), T(0)); }
    void add(const int i, const int j, const T v) { val_[(size_t)j * m_ + i] += v; }
    const T* data() const { return val_.data(); }
};
} // namespace dist_matrix

#endif
