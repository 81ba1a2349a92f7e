// Shared declarations of the stencil engine (mgx_stencil.cu) and its users.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <vector>

#include "mgx_internal.cuh"

namespace mgx
{

enum StencilOp
{
    OP_LAP    = 0, // out = -Lap u
    OP_HPSI_B = 1, // out = -Lap_M u + B(V u)          (Mehrstellen only)
    OP_HPSI_V = 2, // out = -Lap u + V u
    OP_JACOBI = 3, // w = -Lap u - f ; out = mask(u - jf w) ; w_out = mask(w)
    OP_RHS    = 4, // out = B u
    OP_RHS_SUB = 5, // out = B u - g (g pointwise, passed as f)
    OP_JACOBI_UPD = 6, // OP_JACOBI whose result r is added into upd: upd += upd_alpha r
    OP_RHS_SPLIT  = 7, // out = B u stored as bf16 hi / lo planes of a tensor-core operand
    OP_JACOBI_RST = 8  // OP_JACOBI whose residual w is restricted to the next grid in the
                       // kernel (full weighting into `coarse`) instead of being stored
};

__host__ __device__ constexpr bool is_rhs_op(int op)
{
    return op == OP_RHS || op == OP_RHS_SUB || op == OP_RHS_SPLIT;
}
__host__ __device__ constexpr bool is_jacobi(int op)
{
    return op == OP_JACOBI || op == OP_JACOBI_UPD || op == OP_JACOBI_RST;
}

/* Localization masks of one level in box form: for function f, values of
 * the box starting at (box[6f], box[6f+1], box[6f+2]) (periodic) with
 * extents (box[6f+3..5]); points outside the box have mask value 0.
 * state[f] follows src/GridMask.h:47-52 (-1, 0: zero; 1: identity; 2:
 * values).  kind 0 clamps (GridMaskMax), 1 multiplies (GridMaskMult). */
struct MaskDev
{
    const int* state = nullptr;
    const int* box   = nullptr;
    const size_t* offset = nullptr;
    const void* values   = nullptr;
    int n[3]             = { 0, 0, 0 };
    int kind             = 0;
};

struct PlaneParams
{
    const void* u = nullptr;
    size_t ldu    = 0;
    const void* V = nullptr;
    const void* f = nullptr;
    size_t ldf    = 0;
    void* out     = nullptr;
    size_t ldo    = 0;
    void* w       = nullptr;
    size_t ldw    = 0;
    int n[3]      = { 0, 0, 0 };
    int ty = 0, xc = 0, ntile_y = 0, ntile_x = 0;
    MaskDev mask;
    int* err = nullptr;
    // OP_JACOBI only: when nonzero the staged input is f itself and the
    // iterate is u = gamma_in * f (the first sweep of the V-cycle started
    // from gamma * res, src/OrbitalsPreconditioning.cc:102-107)
    double gamma_in = 0.;
    // OP_JACOBI_UPD only: the sweep's result r is not stored to out;
    // instead upd += upd_alpha * r (the orbital update of an ABPG step
    // fused into the last smoothing sweep of the preconditioner).  A
    // separate operator so that the plain sweeps compile without it.
    void* upd        = nullptr;
    size_t ldupd     = 0;
    double upd_alpha = 0.;
    // OP_JACOBI_UPD only, or NULL: upd = upd_scale[f] * (upd + upd_alpha r),
    // the column normalization of the updated block folded into the store
    const double* upd_scale = nullptr;
    // OP_RHS_SPLIT, and OP_HPSI_B (FP32) when split_hi is set: the result r
    // of point k of function f is stored as bf16 hi = rn(r), lo = rn(r - hi)
    // at ((k / 64) * split_rows + f) * 64 + k % 64 of split_hi / split_lo
    // (the K-blocked operand planes); OP_HPSI_B stores out as well
    void* split_hi = nullptr;
    void* split_lo = nullptr;
    int split_rows = 0;
    // OP_JACOBI_RST only: the restriction of the residual w (the next
    // level's right-hand side, n/2 points per direction, leading dimension
    // ldc); no masks
    void* coarse = nullptr;
    size_t ldc   = 0;
    // jacobi2_launch with JJ_PRO only: the input is u - P e, e the next
    // level's correction (n/2 points per direction, leading dimension
    // ldpro) prolonged as prolong_kernel does, formed on chip (the
    // coarse-grid correction of the V-cycle folded into its post-sweeps)
    const void* pro = nullptr;
    size_t ldpro    = 0;
};

int stencil_launch(int op, int lap_type, int dtype, int v_dtype,
    const PlaneParams& p, const Level& L, double jf, int nfunc,
    cudaStream_t stream, int force_direct = 0);

/* Two consecutive Jacobi sweeps of one level in one kernel, the first
 * sweep's iterate kept on chip.  p as for OP_JACOBI, out not aliasing u
 * or f; gamma_in set: the first sweep starts from gamma_in f (u unused).
 * JJ_STORE stores the second iterate to out; JJ_UPD adds it into p.upd as
 * OP_JACOBI_UPD does (out unused); JJ_RST stores it and restricts the
 * second sweep's residual into p.coarse as OP_JACOBI_RST does.  JJ_PRO
 * added to JJ_STORE or JJ_UPD: the sweeps start from u - P p.pro (the
 * prolongation of prolong_launch, mode 1).  Radius-1 operators (lap_type
 * 0 and 1), no masks.  The same bits as the separate kernels.
 * MGX_UNSUPPORTED, with nothing launched, when the kernel cannot run the
 * block; dry: only that check.  tile_rows, when given, receives the tile
 * height (output rows per block; the first sweep also forms YO + 2 more,
 * YO = 1 with the restriction). */
/* The pre-sweep pair (JJ_RST) pays only on tiles of at least this many
 * rows: lower tiles re-do too much of the first sweep on their halo rows. */
constexpr int JJ_PAIR_MIN_ROWS = 12;

enum Jacobi2Mode
{
    JJ_STORE = 0,
    JJ_UPD   = 1,
    JJ_RST   = 2,
    JJ_PRO   = 4
};
int jacobi2_launch(int mode, int lap_type, int dtype, const PlaneParams& p, const Level& L,
    double jf, int nfunc, cudaStream_t s, bool dry = false, int* tile_rows = nullptr);

/* out = B u (the Mehrstellen right-hand-side operator) for nfunc ghost-free
 * functions of grid level 0; u and out with leading dimensions ldu, ldo. */
int rhs_block(const mgx_grid& g, int dtype, const void* u, size_t ldu, void* out,
    size_t ldo, int nfunc, cudaStream_t s);
/* B u of nfunc FP32 functions written straight into bf16 hi / lo K-blocked
 * planes of `rows` rows (the tensor-core operand layout).  MGX_UNSUPPORTED
 * when the vector kernel cannot run the block (alignment, plane size) or
 * the points are not a multiple of 64; nothing is launched then. */
int rhs_split_block(const mgx_grid& g, const float* u, size_t ldu, int nfunc, void* hi,
    void* lo, int rows, cudaStream_t s);
/* H psi = -Lap_M psi + B(V psi) of nfunc FP32 functions (FP32 V) written to
 * out (leading dimension ld) and, as bf16 hi / lo K-blocked planes of
 * `rows` rows, to hi / lo.  MGX_UNSUPPORTED, with nothing launched, when
 * the vector kernel cannot run the block or the points are not a multiple
 * of 64. */
int hpsi_split_block(const mgx_grid& g, const float* psi, size_t ld, const float* V, float* out,
    int nfunc, void* hi, void* lo, int rows, cudaStream_t s);

int ghosted_del2(const mgx_grid& g, int ghosts, int lap_type, int dtype,
    const void* v, void* b, size_t nfunc, cudaStream_t s);
int ghosted_rhs(const mgx_grid& g, int ghosts, int dtype, const void* v,
    void* rhs, int rhs_ghosts, size_t nfunc, cudaStream_t s);
int ghosted_trade(const mgx_grid& g, int ghosts, int dtype, void* u,
    size_t nfunc, cudaStream_t s);

} // namespace mgx

/* the opaque mask set of the C ABI: per level, device arrays in box form */
struct mgx_masks
{
    int nlevels = 0, nfunc = 0, kind = 0, dtype = 0, func = 0, mesh_ghosts = 1;
    int n[3]    = { 0, 0, 0 };
    std::vector<mgx::DeviceBuffer> state, box, offset, values;
    std::vector<std::vector<int>> h_state, h_box;
    std::vector<mgx::MaskDev> dev;
};
