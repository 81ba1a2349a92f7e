/*
 * SINGLE-TASK STAND-IN FOR dist_matrix::SparseDistMatrix -- TEST
 * INFRASTRUCTURE ONLY.
 *
 * With one task, SparseDistMatrix::push_back followed by
 * parallelSumToDistMatrix adds every pushed (row, column, value) triplet
 * into the target matrix; this stand-in adds at push_back time and makes
 * the parallel sum a no-op.  Enough for the reference's
 * LocalMatrices2DistMatrix::convert / accumulate to run unmodified.
 */
#ifndef MGX_SHIM_SPARSEDISTMATRIX_H
#define MGX_SHIM_SPARSEDISTMATRIX_H

#include "DistMatrix.h"

namespace dist_matrix
{
template <class T>
class SparseDistMatrix
{
    DistMatrix<T>& mat_;

public:
    SparseDistMatrix(MPI_Comm, DistMatrix<T>& mat, const int) : mat_(mat) {}
    void push_back(const int i, const int j, const T v) { mat_.add(i, j, v); }
    void parallelSumToDistMatrix() {}
};
} // namespace dist_matrix

#endif
