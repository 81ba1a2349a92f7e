/*
 * mgx.h -- C ABI of the GB300 (sm_103a) implementation of MGmol's orbital
 * hot path: the local Hamiltonian on a block of orbitals, the block
 * multigrid V-cycle used as orbital preconditioner, localization masks, the
 * Gram / H-matrix contractions with FP64 Cholesky, inverse and trace, the
 * residual and update of one ABPG step, and the pb::Mgm Poisson solver.
 *
 * Conventions
 *  - Every call returns an mgx_status; mgx_last_error_string() gives the
 *    text of the last failure on the calling host thread.
 *  - All data pointers are DEVICE pointers owned by the caller, unless a
 *    parameter says "host".  Nothing here copies between host and device
 *    except where stated.  Calls are ordered on the cudaStream_t passed as
 *    `stream` (NULL = the legacy default stream).
 *  - Orbital blocks without ghosts use MGmol's BlockVector layout
 *    (src/BlockVector.h:22-67): function-major, nfunc columns of
 *    n[0]*n[1]*n[2] points with leading dimension `ld` (elements), points
 *    x-slowest, z-fastest.  Ghosted blocks use pb::GridFuncVector's layout
 *    (src/pb/GridFuncVector.cc:21-43): nfunc blocks of
 *    (n[0]+2g)(n[1]+2g)(n[2]+2g) values, inc_x = (n[1]+2g)(n[2]+2g),
 *    inc_y = n[2]+2g.
 *  - Operators work in MGmol's Rydberg convention: the "del2" kernels
 *    return -Laplacian (a positive operator), and the Mehrstellen local
 *    Hamiltonian is H psi = -Lap_M psi + B (V psi)
 *    (src/Hamiltonian.cc:106-132).  Hartree = Rydberg / 2.
 *  - Boundary conditions: periodic in all three directions (the only
 *    case the implementation accepts; anything else is MGX_UNSUPPORTED).
 *  - N x N matrices (S, H, S^-1, L) are FP64, column-major, leading
 *    dimension n, on the device.
 */
#ifndef MGX_H
#define MGX_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mgx_status
{
    MGX_OK          = 0,
    MGX_BAD_ARG     = 1, /* wrong shape, pointer, alignment or option */
    MGX_NOT_SPD     = 2, /* Cholesky met a non-positive pivot */
    MGX_NONFINITE   = 3, /* NaN or Inf detected where checked */
    MGX_TIMEOUT     = 4, /* a bounded device wait gave up */
    MGX_CUDA_ERROR  = 5, /* a CUDA runtime call failed */
    MGX_UNSUPPORTED = 6, /* valid request outside what is implemented */
    MGX_NO_MEMORY   = 7  /* device workspace allocation failed */
} mgx_status;

typedef enum mgx_dtype
{
    MGX_F64 = 0,
    MGX_F32 = 1
} mgx_dtype;

/* lap_type values of MGmol (src/LapFactory.h:26-53) */
typedef enum mgx_lap_type
{
    MGX_LAP_MEHR4 = 0, /* Mehrstellen 4th order, pb::Laph4M */
    MGX_LAP_2ND   = 1, /* pb::Laph2 */
    MGX_LAP_4TH   = 2, /* pb::Laph4 */
    MGX_LAP_6TH   = 3, /* pb::Laph6 */
    MGX_LAP_8TH   = 4  /* pb::Laph8 */
} mgx_lap_type;

/* Arithmetic of the Gram / H contractions. */
typedef enum mgx_gemm_mode
{
    MGX_GEMM_FP64   = 0, /* FP64 data, FP64 FMA (plain path) */
    MGX_GEMM_FP32   = 1, /* FP32 data, FP32 FMA on CUDA cores in 8-term
                          * chains, the chains summed in FP32 over 128
                          * terms and those sums in double-float (two FP32) */
    MGX_GEMM_TF32   = 2, /* FP32 data, tcgen05 kind::tf32, FP32 accumulate */
    MGX_GEMM_BF16X3 = 3, /* FP32 data split hi+lo bf16, 3 tcgen05 products */
    MGX_GEMM_FP16X3 = 4  /* FP32 data scaled by a power of two and split hi+lo
                            fp16 (2^-22 instead of bf16's 2^-16), 3 tcgen05
                            products, same speed as BF16X3 */
} mgx_gemm_mode;

typedef struct mgx_grid
{
    int n[3];     /* interior points per direction */
    double ll[3]; /* domain lengths (bohr); h = ll / n, as pb::Grid */
    int bc[3];    /* 1 = periodic (required) */
} mgx_grid;

typedef struct mgx_ctx mgx_ctx;
typedef struct mgx_masks mgx_masks;

/* ---------------------------------------------------------------- */
/* Context: grid geometry plus device workspaces owned by the context  */
/* (V-cycle levels, GEMM partials).  One context per stream.           */
/* ---------------------------------------------------------------- */
int mgx_create(const mgx_grid* grid, mgx_ctx** ctx);
int mgx_destroy(mgx_ctx* ctx);
const char* mgx_last_error_string(void);
/* Kernel timing for benchmarks: with timing on, every tensor-core product
 * launch is bracketed by CUDA events on its stream; mgx_timing_read returns
 * the summed device time (ms) and the number of launches of one class since
 * the last read of that class (waiting for the events), and forgets them.
 * Classes: split-K products (S, H, B), store-epilogue products (Psi Theta,
 * the density). */
#define MGX_TIMING_TC_SPLITK 1
#define MGX_TIMING_TC_STORE 2
int mgx_timing_enable(int on);
int mgx_timing_read(int cls, double* total_ms, int* launches);

/* Number of kernels this library launched since process start (all
 * contexts); a counter for benchmarks and tests. */
unsigned long long mgx_kernel_launch_count(void);

/* The compute capability (major * 10 + minor) that the loaded module of
 * this library's kernels was compiled for, from the CUDA runtime's
 * function attributes of one of them: 103 for sm_103a.  Needs a device. */
int mgx_kernel_arch(int* binary_version);

/* ---------------------------------------------------------------- */
/* Drop-in kernels on ghosted GridFuncVector blocks (ghosts already     */
/* filled), the MemorySpace::Device overloads of src/pb/FDkernels.h:   */
/* 38-75 and src/pb/MGkernels.h:10-16.  `ghosts` is the ghost width of   */
/* the block; it must be at least the operator radius.                  */
/* ---------------------------------------------------------------- */

/* pb::FDkernelDel2_{4th_Mehr,2nd,4th,6th,8th}<T>(grid, v, b, nfunc,
 * MemorySpace::Device), src/pb/FDkernels.h:38-75: b = -Lap v on interior
 * points; ghost values of b untouched. */
int mgx_fdkernel_del2(const mgx_grid* grid, int ghosts, int lap_type,
    mgx_dtype dtype, const void* v, void* b, size_t nfunc, void* stream);

/* pb::FDkernelRHS_4th_Mehr1<T>(grid, v, rhs, rhs_ghosts, nfunc),
 * src/pb/FDkernels.cc:522-584: rhs = B v (Mehrstellen right-hand side);
 * rhs has rhs_ghosts ghost layers (0 = ghost-free). */
int mgx_fdkernel_rhs_mehr1(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* v, void* rhs, int rhs_ghosts, size_t nfunc, void* stream);

/* pb::MGkernelRestrict3D<T>(fine, fine_grid, coarse, coarse_grid, nfunc),
 * src/pb/MGkernels.cc:203-283.  `grid` is the fine grid; the coarse grid
 * has n/2 points and the same ghost width. */
int mgx_mgkernel_restrict3d(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* fine, void* coarse, size_t nfunc, void* stream);

/* pb::MGkernelExtend3D<T>(coarse, coarse_grid, fine, fine_grid, nfunc),
 * src/pb/MGkernels.cc:28-201 (coarse ghosts must be filled).  `grid` is the
 * fine grid. */
int mgx_mgkernel_extend3d(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* coarse, void* fine, size_t nfunc, void* stream);

/* GridFuncVector::trade_boundaries on one task, periodic
 * (src/pb/GridFuncVector.cc:1543-1621): fills all ghost layers. */
int mgx_trade_boundaries(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    void* u, size_t nfunc, void* stream);

/* GridFuncVector::axpy / operator-= (src/pb/GridFuncVector.cc:1643-1668,
 * LinearAlgebraUtils::MPaxpy, src/linear_algebra/mputils.cc:222-244):
 * y += alpha * x over n elements of dtype. */
int mgx_axpy(size_t n, double alpha, mgx_dtype dtype, const void* x, void* y,
    void* stream);

/* Copies `bytes` from src to dst, either of which may be device memory or
 * pinned host memory.  When both are device-addressable and 16-byte
 * aligned the copy is a kernel whose loads and stores run on all SMs (for
 * host memory, through its mapped device address over the CPU-GPU link);
 * otherwise it is one cudaMemcpyAsync.  Not a reference function: it moves
 * orbital blocks in and out of the device for end-to-end use. */
int mgx_copy(void* dst, const void* src, size_t bytes, void* stream);

/* ---------------------------------------------------------------- */
/* Fused path on ghost-free blocks (periodic halo handled in the tile    */
/* loaders).                                                            */
/* ---------------------------------------------------------------- */

/* out = -Lap u for nfunc functions (lap_type 0..4). */
int mgx_fd_apply(mgx_ctx* ctx, int lap_type, mgx_dtype dtype, const void* u,
    size_t ld, void* out, int nfunc, void* stream);

/* out = B u, the Mehrstellen right-hand-side operator. */
int mgx_rhs_mehr(mgx_ctx* ctx, mgx_dtype dtype, const void* u, size_t ld,
    void* out, int nfunc, void* stream);

/* Hamiltonian<T>::applyLocal (src/Hamiltonian.cc:85-159), Rydberg units.
 * lap_type 0 and apply_B_to_V 1: hpsi = -Lap_M psi + B(V psi);
 * lap_type 0 and apply_B_to_V 0: hpsi = -Lap_M psi + V psi;
 * lap_type 1..4: hpsi = -Lap psi + V psi.
 * V has n[0]*n[1]*n[2] points of type v_dtype (FP64 like MGmol's POTDTYPE,
 * or FP32). */
int mgx_hpsi(mgx_ctx* ctx, int lap_type, mgx_dtype dtype, const void* psi,
    size_t ld, const void* V, mgx_dtype v_dtype, void* hpsi, int nfunc,
    int apply_B_to_V, void* stream);

/* Full-weighting restriction and trilinear prolongation between level
 * `level` (0 = the context grid) and level+1, ghost-free, periodic
 * (src/pb/MGkernels.cc:28-283). */
int mgx_mg_restrict(mgx_ctx* ctx, int level, mgx_dtype dtype, const void* fine,
    void* coarse, int nfunc, void* stream);
int mgx_mg_prolong(mgx_ctx* ctx, int level, mgx_dtype dtype, const void* coarse,
    void* fine, int nfunc, void* stream);

/* OrbitalsPreconditioning<T>::precond_mg (src/OrbitalsPreconditioning.cc:
 * 86-117) with Preconditioning<T>::mg (src/Preconditioning.cc:155-216):
 * out = V-cycle(res) started from gamma * res, `maxlevels` coarse levels,
 * 2 pre / 2 post Jacobi sweeps, 4 sweeps on the coarsest level, fine-level
 * Jacobi factor of lap_type, Laph2 on coarse levels.  masks may be NULL.
 * res and out may not alias.  The V-cycle workspace is owned by ctx and
 * processes at most `chunk` functions at a time (0 = all at once). */
typedef struct mgx_precond_params
{
    int lap_type;
    int maxlevels;
    double gamma;
    int chunk;
} mgx_precond_params;
int mgx_precond_mg(mgx_ctx* ctx, const mgx_precond_params* p, mgx_dtype dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks,
    void* stream);

/* mgx_precond_mg started from the iterate that out holds on entry instead
 * of gamma * res (gamma is not used): the warm-started V-cycle of the
 * learned preconditioner.  With out = gamma * res on entry the result is
 * mgx_precond_mg's. */
int mgx_precond_mg_warm(mgx_ctx* ctx, const mgx_precond_params* p, mgx_dtype dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks,
    void* stream);

/* One preconditioned ABPG update, ABPG<T>::update_states without
 * acceleration (src/ABPG.cc:72-140): psi += alpha * V-cycle(res), with
 * alpha = 0.5 * precond_factor.  The V-cycle is mgx_precond_mg's; its last
 * fine-level sweep adds its result to psi instead of storing it, so the
 * correction block is never written.  With psi_scale (device, nfunc FP64
 * values; NULL for none) the stored result is
 * psi_j = psi_scale[j] * (psi_j + alpha * V-cycle(res)_j): the column
 * scaling of a block whose normalization was deferred into this update
 * (mgx_normalize_scales).  work (nfunc x ld, or NULL for a block owned by
 * ctx) holds the fine-level iterate.  res, psi and work may not alias. */
int mgx_precond_mg_update(mgx_ctx* ctx, const mgx_precond_params* p,
    mgx_dtype dtype, const void* res, size_t ld, void* psi, double alpha,
    const double* psi_scale, int nfunc, const mgx_masks* masks, void* work,
    void* stream);

/* mgx_precond_mg without any device allocation.  This entry point has no
 * counterpart in the reference; it serves callers that cannot allocate
 * device memory: hosts whose device memory belongs to a pool they do not
 * control (an application that reserves the GPU's memory up front and hands
 * out slices of it), and plug-ins in processes that forbid device
 * allocations after start-up (cudaMalloc may synchronize the device and
 * stall the process's other streams).  Same arguments and results as
 * mgx_precond_mg; ctx only supplies the grid (its workspaces are not used).
 * The V-cycle levels live in a fixed 64 MiB device array that is part of
 * the library and held by every GPU that loads it: functions are processed
 * in chunks that fit it, and a request whose single function needs more
 * than the array holds is rejected with MGX_BAD_ARG.  The first call on a
 * device looks up the array's device address and keeps it for the life of
 * the process (a cudaDeviceReset afterwards leaves the kept address
 * stale).  All calls share the array,
 * so calls that overlap on the GPU (other streams, other host threads)
 * race.  The call reads the V-cycle's status word back and waits for
 * `stream` before it returns. */
int mgx_precond_mg_static(mgx_ctx* ctx, const mgx_precond_params* p,
    mgx_dtype dtype, const void* res, size_t ld, void* out, int nfunc,
    const mgx_masks* masks, void* stream);

/* OrbitalsPreconditioning<T>::setGamma (src/OrbitalsPreconditioning.cc:
 * 119-145); host computation, returned in *gamma. */
int mgx_precond_gamma(const mgx_grid* grid, int lap_type, int mg_levels,
    double vmax, double small_eig, double* gamma);

/* ---------------------------------------------------------------- */
/* Localization masks (GridMask / GridMaskMax / GridMaskMult,           */
/* src/GridMask.cc:120-264, src/MasksSet.cc:16-48,110-123).             */
/* ---------------------------------------------------------------- */

/* Builds, on the device, the masks of nfunc orbitals for levels
 * 0..nlevels-1.  centers (nfunc x 3) and radii (nfunc) are HOST arrays.
 * func: 0 gaussianDecay, 1 one.  kind: 0 GridMaskMax (clamp), 1
 * GridMaskMult (multiply).  mesh_ghosts: ghost width of the mesh grid
 * (enters the overlap margin, src/GridMask.cc:42-45).  dtype: storage
 * type of the mask values (MGmol's lmasktype = orbital type). */
int mgx_masks_create(mgx_ctx* ctx, int nlevels, int nfunc,
    const double* centers, const double* radii, int func, int kind,
    int mesh_ghosts, mgx_dtype dtype, mgx_masks** masks, void* stream);
int mgx_masks_destroy(mgx_masks* masks);
/* MasksSet::update (src/MasksSet.cc:208-218): rebuilds the masks of all
 * levels for new centres (nfunc x 3) and radii (nfunc), HOST arrays, with
 * the set's levels, functions, profile and kind; the handle stays valid.
 * The correction masks of LocGridOrbitals::applyCorrMask
 * (src/LocGridOrbitals.cc:454-480) are a second set of profile 1 (`one`)
 * applied with mgx_masks_apply. */
int mgx_masks_update(mgx_ctx* ctx, mgx_masks* masks, const double* centers,
    const double* radii, void* stream);
/* Applies level `level` masks to nfunc ghost-free functions in place
 * (GridFuncVector::app_mask, src/pb/GridFuncVector.cc:2427-2438). */
int mgx_masks_apply(mgx_ctx* ctx, const mgx_masks* masks, int level,
    void* u, size_t ld, int nfunc, void* stream);
/* Writes the dense mask values of one level (nfunc x level points, dtype
 * of the masks) and the states (host int array, nfunc) -- for checking. */
int mgx_masks_expand(const mgx_masks* masks, int level, void* dense,
    int* host_state, void* stream);

/* ---------------------------------------------------------------- */
/* Gram and H matrices (LocGridOrbitals::getLocalOverlap /              */
/* computeLocalProduct, src/LocGridOrbitals.cc:1504-1604, then the      */
/* |x| > 1e-14 filter of src/LocalMatrices2DistMatrix.cc:16,60).        */
/* ---------------------------------------------------------------- */

/* S = Psi^T Psi * vel, full symmetric, FP64 n x n. */
int mgx_gram(mgx_ctx* ctx, int mode, const void* psi, size_t ld, int nfunc,
    double* S, void* stream);
/* H = Psi^T (H Psi) * vel, FP64 n x n (H(i,j) = <psi_i, hpsi_j>). */
int mgx_hmat(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, int nfunc, double* H, void* stream);

/* S and H in one call (the tensor-core modes convert Psi once for both);
 * same conventions as mgx_gram and mgx_hmat. */
int mgx_gram_hmat(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, int nfunc, double* S, double* H, void* stream);

/* LocGridOrbitals::computeMatB (src/LocGridOrbitals.cc:1428-1487), the
 * matrix of the Mehrstellen generalized eigenproblem:
 * Bm = Psi^T (B Psi) * vel, B the Mehrstellen right-hand-side operator
 * (pb::Laph4M::rhs, FDkernelRHS_4th_Mehr1), FP64 n x n.  Only the lower
 * triangle is formed -- the reference's consumers (potrf / potri with uplo
 * 'l' in ProjectedMatricesMehrstellen::computeInvB) read no other part --
 * and it is mirrored into the upper one.  B Psi is formed in `work`, a
 * block of work_funcs >= 1 functions (leading dimension ld, the orbital
 * type), work_funcs functions at a time; or, for a NULL work, in a block of
 * at most 512 functions owned by ctx.  work may not alias psi.  mode as for
 * mgx_gram. */
int mgx_matb(mgx_ctx* ctx, int mode, const void* psi, size_t ld, int nfunc,
    double* Bm, void* work, int work_funcs, void* stream);

/* S, H and B (mgx_gram, mgx_hmat, mgx_matb) in one call; the tensor-core
 * modes convert Psi once for the three products. */
int mgx_gram_hmat_matb(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, int nfunc, double* S, double* H, double* Bm, void* work, int work_funcs,
    void* stream);

/* H Psi (mgx_hpsi with lap_type 0 and B(V psi), FP32 block and potential)
 * and then S, H and B (mgx_gram_hmat_matb) in one call.  With split-BF16x3
 * products the H psi kernel runs inside the H product, 512 functions at a
 * time, and writes each chunk both to hpsi (FP32, as mgx_hpsi) and as the
 * product's bf16 hi / lo operand planes, so H Psi is not read back and
 * converted; other modes make the two calls.  hpsi is an output. */
int mgx_hpsi_gram_hmat_matb(mgx_ctx* ctx, int mode, const float* psi, const float* V,
    float* hpsi, size_t ld, int nfunc, double* S, double* H, double* Bm, void* work,
    int work_funcs, void* stream);

/* ProjectedMatricesMehrstellen::updateHB
 * (src/ProjectedMatricesMehrstellen.h:55-62): HB = S theta, S read as
 * symmetric from its lower triangle (symm 'l', 'l'), then
 * HB = 0.5 HB + 0.5 HB^T.  With theta = B^-1 H, tr(HB S^-1)
 * (mgx_trace_prod(HB, Sinv)) is the energy of ProjectedMatrices::getEigSum
 * for a Mehrstellen operator. */
int mgx_update_hb(mgx_ctx* ctx, int n, const double* S, const double* theta,
    double* HB, void* stream);

/* LocGridOrbitals::normalize (src/LocGridOrbitals.cc:2230-2311, the branch
 * without short-sighted matrices): diagS_i = vel * psi_i . psi_i with FP64
 * accumulation (MPdot), then psi_i <- psi_i / sqrt(diagS_i) computed in
 * FP64 and rounded to the orbital type (MPscal).  diagS (device, nfunc
 * values) may be NULL.  A diagS_i <= 1e-15, which the reference asserts
 * against, returns MGX_NOT_SPD with psi unchanged.  Synchronous. */
int mgx_normalize(mgx_ctx* ctx, mgx_dtype dtype, void* psi, size_t ld, int nfunc,
    double* diagS, void* stream);

/* scale_i = 1 / sqrt(S(i, i)) (device, n values): the factors by which
 * LocGridOrbitals::normalize would scale functions whose Gram matrix is S.
 * With these, the normalization of a block can be folded into the update
 * of mgx_precond_mg_update (its psi_scale) instead of a separate pass over
 * the block.  No counterpart in the reference. */
int mgx_normalize_scales(mgx_ctx* ctx, int n, const double* S, double* scale,
    void* stream);

/* GramMatrix::updateLS (src/GramMatrix.cc:180-191): A (n x n, FP64) is
 * overwritten by its lower Cholesky factor (upper part zeroed).  *info
 * (host) receives 0 or the 1-based index of the first non-positive pivot;
 * the call then returns MGX_NOT_SPD instead of aborting. Synchronous. */
int mgx_cholesky(mgx_ctx* ctx, int n, double* A, int* info, void* stream);
/* mgx_cholesky without waiting for the result: *info (DEVICE int)
 * receives 0 or the pivot index once the factorization has run on
 * `stream`, and the caller checks it when convenient; the call itself
 * returns at once, so that factorizations on several streams (each with its
 * own ctx) overlap.  No counterpart in the reference. */
int mgx_cholesky_async(mgx_ctx* ctx, int n, double* A, int* info, void* stream);

/* GramMatrix::computeInverse (src/GramMatrix.cc:75-91): Sinv = (L L^T)^-1
 * from the factor L. */
int mgx_inverse_from_cholesky(mgx_ctx* ctx, int n, const double* L,
    double* Sinv, void* stream);
/* ProjectedMatrices::getEigSum (src/ProjectedMatrices.cc:550-566):
 * *trace (device) = tr(H Sinv), H and Sinv taken symmetric from their lower
 * parts. */
int mgx_trace_prod(mgx_ctx* ctx, int n, const double* H, const double* Sinv,
    double* trace, void* stream);

/* Lets the Psi Theta products of this context (mgx_mult_matrix,
 * mgx_residual, mgx_residual_cols, mgx_rho) in the BF16X3 mode read the
 * BF16 conversion of psi that the last mgx_gram / mgx_hmat /
 * mgx_gram_hmat / mgx_matb / mgx_gram_hmat_matb call on this context made
 * of the same block (same pointer, leading dimension and size), instead of
 * converting psi again.  With it on, the caller guarantees that psi has
 * not changed in between.  Off by default.  No counterpart in the
 * reference. */
int mgx_set_reuse_conversion(mgx_ctx* ctx, int on);

/* ---------------------------------------------------------------- */
/* Residual and orbital update (rows of the ABPG step).              */
/* ---------------------------------------------------------------- */

/* ProjectedMatrices::updateTheta (src/ProjectedMatrices.h:218-225):
 * theta = Sinv H (n x n, FP64, column-major), Sinv read as symmetric from
 * its lower triangle as BLAS symm('l', 'l') does. */
int mgx_theta(mgx_ctx* ctx, int n, const double* Sinv, const double* H,
    double* theta, void* stream);

/* theta = S^-1 H straight from the Cholesky factor L of S (mgx_cholesky),
 * by forward and back substitution with the columns of H as right-hand
 * sides, without forming S^-1 (2 n^3 flop instead of the 4.3 n^3 of
 * mgx_inverse_from_cholesky followed by mgx_theta).  *trace (device; NULL to
 * skip) receives tr(theta) = tr(S^-1 H), the energy of
 * ProjectedMatrices::getEigSum.  This combination has no single counterpart
 * in the reference, which forms the inverse (GramMatrix::computeInverse)
 * and multiplies (ProjectedMatrices::updateTheta). */
int mgx_theta_from_cholesky(mgx_ctx* ctx, int n, const double* L, const double* H,
    double* theta, double* trace, void* stream);

/* LocGridOrbitals::multiplyByMatrix (src/LocGridOrbitals.cc:793-830, the
 * MPgemmNN of src/linear_algebra/mputils.cc:719-760):
 * out_j = sum_i psi_i theta(i, j), theta FP64 column-major nfunc x nfunc.
 * mode MGX_GEMM_FP64: FP64 accumulation (either dtype, as the reference);
 * MGX_GEMM_FP32: FP32 orbitals, FP32 FMA; MGX_GEMM_TF32 / MGX_GEMM_BF16X3:
 * FP32 orbitals on the tensor cores.  out may not alias psi. */
int mgx_mult_matrix(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    size_t ld, int nfunc, const double* theta, void* out, void* stream);

/* MGmol::computeResidualUsingHPhi (src/MGmol.cc:1227-1290):
 * apply_B 1 (Mehrstellen): res = B(psi) theta - hpsi, computed as
 * B(psi theta) - hpsi, with psi theta written to `work` (nfunc x ld block,
 * or NULL for a block owned by ctx); apply_B 0: res = psi theta - hpsi.
 * res may alias hpsi; neither res nor work may alias psi.  mode as for
 * mgx_mult_matrix. */
int mgx_residual(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    const void* hpsi, size_t ld, int nfunc, const double* theta, int apply_B,
    void* work, void* res, void* stream);

/* mgx_residual for the output functions j0 .. j0+ncols-1 only: theta points
 * at column j0 of the nfunc x nfunc matrix (theta + j0 * nfunc), hpsi and
 * res at function j0 of their blocks, work (or the ctx block) holds ncols
 * functions.  Lets a caller bound the memory of the residual and of the
 * preconditioner that follows by walking the block in column chunks.  This
 * entry point has no counterpart in the reference, which always forms the
 * whole block. */
int mgx_residual_cols(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    const void* hpsi, size_t ld, int nfunc, const double* theta, int ncols, int apply_B,
    void* work, void* res, void* stream);

/* ---------------------------------------------------------------- */
/* Electronic density (Rho<T>, src/Rho.cc).                           */
/* ---------------------------------------------------------------- */

/* Rho<T>::computeRho for non-orthogonal orbitals (src/Rho.cc:282-320, with
 * computeRhoSubdomainUsingBlas3, :359-450) and rescaleTotalCharge
 * (:150-200): rho(p) = sum_j (Psi X)_j(p) psi_j(p), X the density matrix
 * (nfunc x nfunc FP64, column-major, device), then charge = vel sum_p rho(p)
 * and, when nel > 0 and the charge is positive, rho *= nel / charge.  A
 * factor off 1 by more than 0.02 (where the reference aborts) returns
 * MGX_BAD_ARG with rho unscaled.  rho: npts FP64 values (device); *charge
 * (host, may be NULL) receives the charge before the rescaling.  mode as for
 * mgx_mult_matrix; the tensor-core modes reduce the product against Psi in
 * the product's epilogue, the CUDA-core modes form it in column chunks in
 * `work` (work_funcs functions of ld values, or NULL for a block of at most
 * 256 functions owned by ctx).  Synchronous. */
int mgx_rho(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi, size_t ld, int nfunc,
    const double* dm, double nel, double* rho, double* charge, void* work, int work_funcs,
    void* stream);

/* ---------------------------------------------------------------- */
/* Anderson extrapolation of the orbital update (AndersonMix<T>,      */
/* src/AndersonMix.cc:21-321): the accelerated branch of              */
/* ABPG<T>::update_states (src/ABPG.cc:118-126).                      */
/* ---------------------------------------------------------------- */

#define MGX_ANDERSON_MAX_M 8

typedef struct mgx_anderson mgx_anderson;

/* What one update did: the history length used (after the reference's
 * shortening), how many times it was shortened, and the coefficients. */
typedef struct mgx_anderson_info
{
    int mm;
    int reductions;
    double theta[MGX_ANDERSON_MAX_M];
} mgx_anderson_info;

/* AndersonMix<T>(m, beta, x): history of m (x, f) pairs of nfunc x ld
 * blocks of dtype, device memory owned by the handle (2 m blocks);
 * 0 <= m <= MGX_ANDERSON_MAX_M. */
int mgx_anderson_create(mgx_ctx* ctx, int m, double beta, mgx_dtype dtype, size_t ld,
    int nfunc, mgx_anderson** mix);
int mgx_anderson_destroy(mgx_anderson* mix);
/* AndersonMix<T>::restart: forget the history. */
int mgx_anderson_restart(mgx_anderson* mix);

/* AndersonMix<T>::update(res, work) after res.scal(fscale) (the ABPG step
 * passes fscale = 0.5 * precond_factor and res = the preconditioned
 * residual): x (the orbital block, nfunc x ld, updated in place) moves to
 * factor x + sum_j theta_j x_j + beta (factor f' + sum_j theta_j f_j),
 * f' = fscale f, factor = 1 - sum_j theta_j; the coefficients solve the
 * normal equations of the differences f' - f_j under the diagonal dot
 * product sum_k vel <a_k, b_k> (S^-1)(k, k) (LocGridOrbitals::
 * dotProductDiagonal), invS the device S^-1 (n x n; only its diagonal is
 * read; unused on the first update).  The old x and f' enter the history.
 * fbar (may be NULL or alias f) receives the mixed residual that the
 * reference leaves in res.  A history matrix that is not positive definite
 * returns MGX_NOT_SPD (the reference continues with a failed factor).
 * Synchronous (the small system is solved on the host). */
int mgx_anderson_update(mgx_anderson* mix, void* x, const void* f, double fscale,
    const double* invS, void* fbar, mgx_anderson_info* info, void* stream);

/* ---------------------------------------------------------------- */
/* Poisson multigrid (pb::Mgm, src/pb/Mgm.h:20-112, with pb::Vcycle,  */
/* src/pb/Vcycle.h:28-249) on one field of the context grid.          */
/* ---------------------------------------------------------------- */

/* Arguments of pb::Mgm: the fine operator (lap_type 0..4 as Laph4M,
 * Laph2, Laph4, Laph6, Laph8; coarse levels keep Laph4M, the others use
 * Laph2), cogr (at most max_levels coarsenings), max_sweeps V-cycles, the
 * relative residual tolerance, nu1 / nu2 smoothing sweeps, and the ghost
 * width of the caller's fine GridFunc (0: the operator's), which enters the
 * coarsening test dim >= 2 * ghosts. */
typedef struct mgx_mgm_params
{
    int lap_type;
    int max_levels;
    int max_sweeps;
    double tol;
    int nu1;
    int nu2;
    int ghosts;
} mgx_mgm_params;

/* The out-parameters of pb::Mgm, its bool result (converged) and the
 * number of grids the cycle used. */
typedef struct mgx_mgm_result
{
    double final_residual;
    double final_relative_residual;
    double residual_reduction;
    int nb_sweeps;
    int converged;
    int levels;
} mgx_mgm_result;

/* Solves A vh = A.rhs(rho) (rho and vh ghost-free device fields of the
 * context grid, periodic) from the initial vh, in place, as pb::Mgm with
 * one task: rhs = B rho for Mehrstellen, rho otherwise; at most max_sweeps
 * V-cycles, stopping when |rhs - A vh| < tol |rhs| (norms sqrt(sum x^2
 * h^3)).  Not converging is reported in *result, not as an error.
 * Synchronous (the residual norms are read on the host every cycle). */
int mgx_mgm(mgx_ctx* ctx, const mgx_mgm_params* params, mgx_dtype dtype,
    void* vh, const void* rho, mgx_mgm_result* result, void* stream);

/* ---------------- learned preconditioner ----------------
 * A 3-level 3-D convolutional U-Net that maps a residual field to an
 * approximation of the V-cycle correction (mgx_precond_mg); it has no
 * counterpart in the reference and is used through
 * mgx_precond_learned, which keeps the V-cycle as the per-function
 * fallback.  Level l is the context grid coarsened l times (each
 * dimension divisible by 4), periodic.  Bias-free layers, so that
 * net(a x) = a net(x) for a > 0; inputs are scaled by their RMS and the
 * output scaled back.  Layers (3x3x3 convolutions, channels in -> out,
 * level): E0 1->16 @0, E1 16->32 @1, E2 32->64 @2, D2 64->32 @2,
 * D1 32->16 @1, D0 16->1 @0; downsampling by the full-weighting
 * restriction and upsampling by the trilinear prolongation of
 * mgx_mg_restrict / mgx_mg_prolong; skip sums with ReLU at levels 1 and 0:
 *   a0 = relu(E0 x)        a1 = relu(E1 R a0)     a2 = relu(E2 R a1)
 *   s1 = relu(P D2 a2 + a1) s0 = relu(P D1 s1 + a0) y = D0 s0.
 * Weights: FP32 master copy, BF16 in the convolutions, FP32
 * accumulation and activations.  Parameter vector: the six weight
 * tensors in layer order, each [out][in][3][3][3] (x, y, z offsets -1..1,
 * z fastest). */
#define MGX_UNET_PARAMS 139104

typedef struct mgx_unet mgx_unet;

typedef struct mgx_adam_params
{
    float lr;
    float beta1;
    float beta2;
    float eps;
} mgx_adam_params;

int mgx_unet_create(mgx_ctx* ctx, mgx_unet** net);
int mgx_unet_destroy(mgx_unet* net);
/* copies MGX_UNET_PARAMS FP32 values (device) into / out of the master
 * weights; set resets the optimizer state */
int mgx_unet_set_params(mgx_unet* net, const float* params, void* stream);
int mgx_unet_get_params(mgx_unet* net, float* params, void* stream);
/* y_j = net(x_j) for nfunc FP32 fields of the context grid (leading
 * dimension ld); x and y may not alias */
int mgx_unet_forward(mgx_unet* net, const float* x, size_t ld, float* y, int nfunc,
    void* stream);
/* loss = mean over functions and points of (net(x_j / s_j) - t_j / s_j)^2,
 * s_j = RMS(x_j); grad (device, MGX_UNET_PARAMS) = d loss / d weights
 * (the BF16 weights the forward pass used); loss is one device double */
int mgx_unet_loss_grad(mgx_unet* net, const float* x, const float* target, size_t ld,
    int nfunc, float* grad, double* loss, void* stream);
/* one Adam step (bias-corrected) of the master weights with grad */
int mgx_unet_adam(mgx_unet* net, const float* grad, const mgx_adam_params* p, void* stream);
/* mgx_unet_loss_grad then mgx_unet_adam, the gradient kept by the net */
int mgx_unet_train_step(mgx_unet* net, const float* x, const float* target, size_t ld,
    int nfunc, const mgx_adam_params* p, double* loss, void* stream);

#define MGX_LEARNED_REPLACE 0 /* correction = net(res) */
#define MGX_LEARNED_WARM 1    /* correction = V-cycle(res) started from net(res) */
#define MGX_LEARNED_REFRESH 2 /* flag: run the plain V-cycle on every function */

/* The learned correction of nfunc FP32 residuals, with the plain V-cycle
 * (mgx_precond_mg with p) as the per-function fallback.  The residual
 * reduction of a correction v of res is |res - A v| / |res|, A the fine
 * operator of p->lap_type (the operator the V-cycle inverts).  tau (host,
 * nfunc, in / out) holds the plain V-cycle's reduction for each function
 * as last measured (<= 0: unknown).  The V-cycle runs on every function
 * whose tau is unknown, whose learned reduction exceeds tau, or on all of
 * them with MGX_LEARNED_REFRESH; it measures tau again, and out_j takes
 * the V-cycle's correction where its reduction is the smaller.
 * reduction (host, nfunc, or NULL) receives the reduction of each
 * returned correction, nfallback (or NULL) the number of functions that
 * took the V-cycle's.  Synchronizes the stream to make the choice. */
int mgx_precond_learned(mgx_ctx* ctx, mgx_unet* net, const mgx_precond_params* p,
    const float* res, size_t ld, float* out, int nfunc, int mode, double* tau,
    double* reduction, int* nfallback, void* stream);

/* ---------------- localized orbitals ----------------
 * Orbital j stored on the level-0 box of its mask in `masks` (origin o_j,
 * extents e_j; box point b is grid point (o_j + b) mod n, z fastest), the
 * boxes packed one after another: the localized storage of
 * LocGridOrbitals, without the zeros outside the localization regions.
 * masks: FP32, GridMaskMax (kind 0), every orbital with a box of values;
 * corr: the correction masks (profile one, GridMaskMult) of the same
 * centres and radii, so the same boxes.  Each box extent must leave room for
 * a halo of 3 points inside the grid.  Both mask sets must outlive the
 * handle, and the boxes are read once: after mgx_masks_update moves the
 * centres, create the handle again. */
typedef struct mgx_local mgx_local;

int mgx_local_create(mgx_ctx* ctx, const mgx_masks* masks, const mgx_masks* corr,
    mgx_local** loc);
int mgx_local_destroy(mgx_local* loc);
/* total packed points; offsets (nfunc + 1 values) and boxes (6 per orbital:
 * origin, extents), each optional */
int mgx_local_layout(const mgx_local* loc, size_t* total, size_t* offsets, int* boxes);
/* whole-grid block (leading dimension ld) -> packed boxes, and back (scatter
 * writes the box points only) */
int mgx_local_gather(mgx_local* loc, const float* full, size_t ld, float* packed, void* stream);
int mgx_local_scatter(mgx_local* loc, const float* packed, float* full, size_t ld, void* stream);
/* The fused fine-level step on packed FP32 blocks, one persistent kernel
 * over (orbital, tile) items:
 *   r  = Mc (B phi - H psi),  H psi = -Delta_M psi + B(V psi)
 *   u1 = M(gamma r - jf (A gamma r - r)),  A = -Delta_M
 *   u  = M(u1 - jf (A u1 - r)),  w = M(A u1 - r)
 * (Hamiltonian::applyLocal, the residual of computeResidualUsingHPhi with
 * phi = (Psi Theta)_j and the correction mask, and the two masked Jacobi
 * pre-sweeps of Preconditioning<T>::mg started from gamma r, jf the
 * Mehrstellen Jacobi factor).  V: FP32, the whole grid.  With the graph
 * option (the default) the launch is a CUDA graph, captured again when an
 * argument or the configuration changes. */
int mgx_local_step(mgx_local* loc, const float* psi, const float* phi, const float* V,
    double gamma, float* u, float* w, void* stream);
/* times every kernel variant (largest column TY x TZ, fitted to each box,
 * and planes per march step; 0: 24x32, 1: 16x32, 2: 32x32 with one plane,
 * 3..5 the same with two) with 1, 2, 3 and 4 resident CTAs per SM on these
 * arguments and keeps the fastest; ms
 * (optional, *ncand entries) receives each candidate's time (-1: not
 * resident), *ncand the number of candidates */
int mgx_local_tune(mgx_local* loc, const float* psi, const float* phi, const float* V,
    double gamma, float* u, float* w, double* ms, int* ncand, void* stream);
int mgx_local_set_config(mgx_local* loc, int shape, int ctas_per_sm, int use_graph);
int mgx_local_get_config(const mgx_local* loc, int* shape, int* ctas_per_sm, int* use_graph);

/* ---------------------------------------------------------------- */
/* Centres and spreads of the orbitals (SpreadsAndCenters,              */
/* src/SpreadsAndCenters.cc:26-104, SinCosOps::computeDiag,             */
/* src/SinCosOps.cc:733-826).                                           */
/* ---------------------------------------------------------------- */

/* out (device, nfunc x 6 doubles, row f = orbital f): the diagonal
 * position-matrix elements a = vel sum_p psi_f(p)^2 t(p) with t = (cos x,
 * sin x, cos y, sin y, cos z, sin z), x = 2 pi i / n per direction, each
 * scaled by L / (2 pi) (pb::Grid::getSinCosFunctions); divided by the
 * norm vel sum psi_f^2 unless `normalized`.  The centre along x is
 * L / (2 pi) atan2(a_1, a_0), taken in [0, L), and the squared spread
 * (L / (2 pi))^2 - a_0^2 - a_1^2 (SpreadsAndCenters::computeCenter,
 * computeSpread2).  FP32 or FP64 blocks, FP64 sums in a fixed order.  The
 * first call on a context uploads the grid's tables (synchronous). */
int mgx_sincos_diag(mgx_ctx* ctx, mgx_dtype dtype, const void* psi, size_t ld, int nfunc,
    int normalized, double* out, void* stream);

/* Localization regions of one task (LocalizationRegions, host code).
 * move_to (LocalizationRegions::moveTo, src/LocalizationRegions.cc:405-450):
 * each centre (nfunc x 3, in place) moves toward its target by the
 * periodic minimum-image difference (Vector3D::vminimage), shortened to
 * 1 bohr when longer; *max_displ receives the longest difference.
 * update_radii (LocalizationRegions::updateRadii, :354-366, getMeanRadius,
 * :332-352): radii[j] = ratio x spreads[j] as float, *mean_radius the cube
 * root of the mean cube.  The new centres and radii go to mgx_masks_update. */
int mgx_regions_move_to(int nfunc, double* centers, const double* targets, const double cell[3],
    float* max_displ);
int mgx_regions_update_radii(int nfunc, const double* spreads, float ratio, float* radii,
    float* mean_radius);

/* ---------------------------------------------------------------- */
/* Function packing (FunctionsPacking with one task,                    */
/* src/FunctionsPacking.cc:40-160): which localized orbitals may share  */
/* a storage column.  Host code; no device is needed.                   */
/* ---------------------------------------------------------------- */

/* The domain of `grid` (origin 0) is cut into subdivx equal sub-boxes
 * along x (Mesh::subdivx).  Orbital j's localization region is the sphere
 * of radius radii[j] plus the subdomain margin (ghosts x |h| + 1e-8, as
 * setupSubdomainGeometry with `ghosts` the operator's ghost width) around
 * centers[3j .. 3j+2], periodic; it is listed in every sub-box it reaches
 * (LocalizationRegions::computeSubdivOverlapGids,
 * src/LocalizationRegions.cc:1039-1099).  Two orbitals overlap when a
 * sub-box lists both (LocalizationRegions::overlap, :1103-1119).  The
 * overlap graph is coloured by greedy multicolouring in decreasing-degree
 * order (rlf = 0: greedyColor, src/tools/coloring.cc) or by Recursive
 * Largest First (rlf = 1: colorRLF), with the reference's orders and tie
 * rules.  colors[j] receives orbital j's colour (the gid2color_ map of
 * FunctionsPacking::getColors), *ncolors their number.  With subdivx = 1
 * every pair overlaps and the colours are all distinct, as in the
 * reference's single-task runs. */
int mgx_pack_functions(const mgx_grid* grid, int ghosts, int nfunc, const double* centers,
    const float* radii, int subdivx, int rlf, int* colors, int* ncolors);

/* ---------------------------------------------------------------- */
/* Snapshots (the restart role of MGmol::dumpRestart / HDFrestart,      */
/* src/MGmol.cc:1101-1127, src/HDFrestart.cc, without HDF5).            */
/* ---------------------------------------------------------------- */

/* Element types of snapshot arrays. */
typedef enum mgx_snap_type
{
    MGX_SNAP_F64 = 0,
    MGX_SNAP_F32 = 1,
    MGX_SNAP_I32 = 2,
    MGX_SNAP_U8  = 3
} mgx_snap_type;

/* One named array of a snapshot: `data` in device or host memory, C order,
 * ndim <= 4 extents in `shape`. */
typedef struct mgx_dataset
{
    const char* name; /* unique in the file; no quote, backslash or control character */
    int type;         /* mgx_snap_type */
    int ndim;
    size_t shape[4];
    const void* data;
} mgx_dataset;

/* Writes the arrays (orbital blocks, potentials, learned weights ...) and
 * the grid (may be NULL) into one file: a 64-byte fixed header, a JSON
 * header listing each array's type, shape, offset and CRC-32 with the
 * caller's `meta_json` (a JSON value, or NULL), and the raw arrays at
 * 4096-byte aligned offsets.  Device arrays stream through two pinned host
 * buffers (64 MiB each), the copy of one chunk overlapping the file write
 * of the previous one, on `stream`; returns once the file is closed.
 * Counterpart of MGmol::dumpRestart (src/MGmol.cc:1101-1127), whose HDF5
 * layout (src/HDFrestart.cc) this build cannot produce without HDF5. */
int mgx_snapshot_write(const char* path, const mgx_grid* grid, const char* meta_json,
    int ndata, const mgx_dataset* data, void* stream);
/* The JSON header of a snapshot into json (cap bytes, NUL-terminated);
 * *len (may be NULL) receives its length.  MGX_BAD_ARG when cap is too
 * small (json then holds the truncated text). */
int mgx_snapshot_header(const char* path, char* json, size_t cap, size_t* len);
/* Reads array `name` into dst (device or host, `bytes` long, which must be
 * the array's size) on `stream`, checking its CRC-32; returns when the data
 * are in place.  MGX_BAD_ARG for a missing array, a size mismatch, a short
 * file or a checksum mismatch.  Counterpart of the restart read of
 * LocGridOrbitals::read_func_hdf5 (src/LocGridOrbitals.cc:1182). */
int mgx_snapshot_read(const char* path, const char* name, void* dst, size_t bytes,
    void* stream);

#ifdef __cplusplus
}
#endif

#endif
