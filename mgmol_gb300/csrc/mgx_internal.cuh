// Internal helpers shared by the sm_103a kernels of the mgx library.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mgx.h"

namespace mgx
{

/* ---------------- error reporting (thread-local text) ---------------- */
void set_error(const char* fmt, ...);
int fail(int status, const char* fmt, ...);
int cuda_check(cudaError_t e, const char* what);
void count_launch(unsigned n = 1);

#define MGX_TRY(expr)                                                          \
    do                                                                         \
    {                                                                          \
        int _s = (expr);                                                       \
        if (_s != MGX_OK) return _s;                                           \
    } while (0)

#define MGX_LAUNCH_CHECK(name)                                                 \
    do                                                                         \
    {                                                                          \
        ::mgx::count_launch();                                                 \
        cudaError_t _e = cudaGetLastError();                                   \
        if (_e != cudaSuccess) return ::mgx::cuda_check(_e, name);             \
    } while (0)

inline size_t dtype_size(int dt) { return dt == MGX_F64 ? 8 : 4; }

/* ---------------- grid geometry ---------------- */
struct Level
{
    int n[3];
    double h[3];
    size_t npts() const { return (size_t)n[0] * n[1] * n[2]; }
};

/* Level l of a grid: n >> l points, h = ll / (n >> l) (pb::Grid::Grid and
 * Grid::coarse_grid, src/pb/Grid.cc:72-76,214-231). */
inline Level make_level(const mgx_grid& g, int l)
{
    Level L;
    for (int i = 0; i < 3; i++)
    {
        L.n[i] = g.n[i] >> l;
        L.h[i] = g.ll[i] / (double)L.n[i];
    }
    return L;
}

/* ---------------- finite-difference coefficients ---------------- */
/* All in the order of the reference kernels (src/pb/FDkernels.cc). */
struct StencilCoeffs
{
    double c0;
    double cx[4], cy[4], cz[4]; // axis coefficients, distance 1..4
    double cxy, cyz, cxz;       // Mehrstellen edge coefficients
    int radius;
};
StencilCoeffs stencil_coeffs(int lap_type, const double h[3]);
/* jacobiFactor() of the operator (src/pb/Laph*.h) */
double jacobi_factor(int lap_type, const double h[3]);
int lap_radius(int lap_type);

/* ---------------- device workspace ---------------- */
struct DeviceBuffer
{
    void* ptr    = nullptr;
    size_t bytes = 0;
    int ensure(size_t b);
    void release();
    ~DeviceBuffer() { release(); }
};

struct MaskLevelDesc; // mgx_mg.cu

} // namespace mgx

/* the opaque context of the C ABI */
struct mgx_ctx
{
    mgx_grid grid;
    int sm_count;
    size_t smem_optin;
    // V-cycle workspace
    mgx::DeviceBuffer vc;
    // GEMM partials / scratch
    mgx::DeviceBuffer gemm_ws;
    mgx::DeviceBuffer dense_ws;
    mgx::DeviceBuffer flag;
    // tensor-core GEMM: bf16 hi/lo planes, tile list, status word
    mgx::DeviceBuffer tc_split, tc_tiles, tc_err;
    // the BF16 K-blocked hi / lo planes that the last Gram-type product left
    // at the start of tc_split (its A operand: rows = functions, K =
    // points), described so that a Psi Theta product on the same block can
    // read them instead of converting the block again (only when the
    // caller has allowed it with mgx_set_reuse_conversion)
    struct Conversion
    {
        const void* psi = nullptr;
        size_t ld = 0, K = 0, used = 0;
        int n      = 0;
        bool valid = false;
        void* hi   = nullptr;
        void* lo   = nullptr;
    } conv;
    int reuse_conversion = 0;
    // residual: Psi Theta when the caller passes no work block
    mgx::DeviceBuffer resid;
    // Poisson multigrid levels
    mgx::DeviceBuffer mgm;
    // partial sums of the reductions
    mgx::DeviceBuffer red;
    // the grid's sine / cosine tables of the centre computation, filled by
    // its first call
    mgx::DeviceBuffer sincos;
};

/* ---------------- PTX helpers: mbarrier + 1-D bulk copies ---------------- */
namespace mgx
{
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
        "r"(count)
                 : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes)
{
    asm volatile(
        "mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
            smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

/* Bounded wait on an mbarrier phase.  Returns false if the phase did not
 * complete within `limit` polls (the caller records MGX_TIMEOUT). */
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity,
    uint32_t limit = (1u << 26))
{
    uint32_t done = 0;
    for (uint32_t it = 0; it < limit; it++)
    {
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(smem_u32(bar)), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

/* 1-D bulk copy global -> shared, completion counted on `bar` (bytes must
 * be a multiple of 16, both addresses 16-byte aligned). */
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src,
    uint32_t bytes, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
} // namespace mgx
