/*
 * ORACLE PINNING DRIVER FOR S AND H -- TEST INFRASTRUCTURE ONLY.
 *
 * Forms the Gram matrix and the H matrix the way the reference does, with
 * its own code compiled unmodified by oracle/build_ref.sh:
 *   S: LocGridOrbitals::getLocalOverlap (src/LocGridOrbitals.cc:1504-1530),
 *      SquareLocalMatrices::syrk, fillUpperWithLower, scal(vel); in the
 *      mixed-precision (USE_MP) build getLocalOverlap goes through
 *      computeLocalProduct instead (src/LocGridOrbitals.cc:1532-1604):
 *      LocalMatrices<float>::gemm, copy to double, scal(vel);
 *   H: Hamiltonian::addHlocalij -> computeLocalProduct (the same gemm path,
 *      FP64 or, in the USE_MP build, through a float LocalMatrices);
 *   both then summed into the distributed matrix by
 *   LocalMatrices2DistMatrix::accumulate, whose convert drops entries with
 *   |x| <= 1e-14 (src/LocalMatrices2DistMatrix.cc:16-107), here on one task
 *   with one subdomain and the identity colouring.
 * Matrices are returned column-major (j * n + i).
 */
#include "LocalMatrices2DistMatrix.h"
#include "SquareLocalMatrices.h"

#include <numeric>
#include <vector>

extern "C" void ref_env_init();

namespace
{
void to_dist(const LocalMatrices<double, MemorySpace::Host>& ss, const int n, double* out)
{
    ref_env_init();
    std::vector<std::vector<int>> gids(1, std::vector<int>(n));
    std::iota(gids[0].begin(), gids[0].end(), 0);
    LocalMatrices2DistMatrix::setup(MPI_COMM_WORLD, gids);
    dist_matrix::DistMatrix<double> dm(n, n);
    dm.clear();
    LocalMatrices2DistMatrix::instance()->accumulate(ss, dm);
    std::copy(dm.data(), dm.data() + (size_t)n * n, out);
}
} // namespace

extern "C" {

/* FP64 build: syrk('l','t') of the block, upper filled from lower, times vel. */
int ref_gram_d(int numpt, int nfunc, const double* psi, int lda, double vel, double* S)
{
    SquareLocalMatrices<double, MemorySpace::Host> ss(1, nfunc);
    ss.syrk(0, numpt, psi, lda);
    ss.fillUpperWithLower();
    ss.scal(vel);
    to_dist(ss, nfunc, S);
    return 0;
}

/* USE_MP build: the product of FP32 orbitals kept in a float local matrix. */
int ref_gram_f(int numpt, int nfunc, const float* psi, int lda, double vel, double* S)
{
    SquareLocalMatrices<double, MemorySpace::Host> ss(1, nfunc);
    LocalMatrices<float, MemorySpace::Host> ssf(1, nfunc, nfunc);
    ssf.gemm(0, numpt, psi, lda, psi, lda);
    ss.copy(ssf);
    ss.scal(vel);
    to_dist(ss, nfunc, S);
    return 0;
}

/* H(i, j) = <psi_i, hpsi_j> vel: gemm('t','n') of the two blocks. */
int ref_hmat_d(int numpt, int nfunc, const double* psi, const double* hpsi, int lda,
    double vel, double* H)
{
    SquareLocalMatrices<double, MemorySpace::Host> ss(1, nfunc);
    ss.gemm(0, numpt, psi, lda, hpsi, lda);
    ss.scal(vel);
    to_dist(ss, nfunc, H);
    return 0;
}

int ref_hmat_f(int numpt, int nfunc, const float* psi, const float* hpsi, int lda,
    double vel, double* H)
{
    SquareLocalMatrices<double, MemorySpace::Host> ss(1, nfunc);
    LocalMatrices<float, MemorySpace::Host> ssf(1, nfunc, nfunc);
    ssf.gemm(0, numpt, psi, lda, hpsi, lda);
    ss.copy(ssf);
    ss.scal(vel);
    to_dist(ss, nfunc, H);
    return 0;
}

} // extern "C"
