// C ABI of the mgx library (include/mgx.h): argument checks, contexts,
// error reporting, and dispatch to the sm_103a kernels.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <cmath>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{
static thread_local char g_err[512] = "";
static std::atomic<unsigned long long> g_launches{ 0 };

void set_error(const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int status, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return status;
}

int cuda_check(cudaError_t e, const char* what)
{
    if (e == cudaSuccess) return MGX_OK;
    set_error("%s: %s", what, cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? MGX_NO_MEMORY : MGX_CUDA_ERROR;
}

void count_launch(unsigned n) { g_launches += n; }

int DeviceBuffer::ensure(size_t b)
{
    if (b <= bytes) return MGX_OK;
    release();
    cudaError_t e = cudaMalloc(&ptr, b);
    if (e != cudaSuccess)
    {
        ptr = nullptr;
        cudaGetLastError();
        return cuda_check(e, "workspace cudaMalloc");
    }
    bytes = b;
    return MGX_OK;
}

void DeviceBuffer::release()
{
    if (ptr) cudaFree(ptr);
    ptr   = nullptr;
    bytes = 0;
}

// defined in the other translation units
int precond_mg(mgx_ctx*, const mgx_precond_params*, int, const void*, size_t,
    void*, int, const mgx_masks*, cudaStream_t, void* upd = nullptr, double alpha = 0.,
    const double* scale = nullptr, bool warm = false);
int restrict_launch(int, const Level&, const void*, size_t, void*, size_t, int,
    const MaskDev&, cudaStream_t);
int prolong_launch(int, int, const Level&, const void*, size_t, void*, size_t,
    int, const MaskDev&, cudaStream_t);
int masks_create(mgx_ctx*, int, int, const double*, const double*, int, int,
    int, int, mgx_masks**, cudaStream_t);
int masks_apply(mgx_ctx*, const mgx_masks*, int, void*, size_t, int, cudaStream_t);
int masks_update(mgx_ctx*, mgx_masks*, const double*, const double*, cudaStream_t);
int masks_expand(const mgx_masks*, int, void*, int*, cudaStream_t);
int gram_cuda_cores(mgx_ctx*, int, const void*, const void*, size_t, size_t,
    int, double, int, double*, cudaStream_t);
int psi_theta_cuda_cores(int, const void*, size_t, size_t, int, const double*, int, int,
    double, const void*, void*, cudaStream_t);
int psi_theta_tcgen05(mgx_ctx*, int, const float*, size_t, size_t, int,
    const double*, int, int, float, const float*, float*, cudaStream_t, double* rho = nullptr);
int theta_product(int, const double*, const double*, double*, cudaStream_t);
int theta_from_cholesky(mgx_ctx*, int, const double*, const double*, double*, double*,
    cudaStream_t);
int mgm_solve(mgx_ctx*, const mgx_mgm_params*, int, void*, const void*, mgx_mgm_result*,
    cudaStream_t);
int gram_tcgen05(mgx_ctx*, int, const void*, const void*, size_t, size_t, int,
    double, int, double*, cudaStream_t);
int gram_hmat_tcgen05(mgx_ctx*, int, const void*, const void*, size_t, size_t, int,
    double, double*, double*, cudaStream_t, double* Bm = nullptr, void* work = nullptr,
    int work_funcs = 0, const float* V = nullptr, int lap_type = 0);
int matb_cuda_cores(mgx_ctx*, int, const void*, size_t, size_t, int, double, double*,
    void*, int, cudaStream_t);
int matb_tcgen05(mgx_ctx*, int, const void*, size_t, size_t, int, double, double*, void*, int,
    cudaStream_t);
int update_hb(int, const double*, const double*, double*, cudaStream_t);
int normalize(mgx_ctx*, int, void*, size_t, size_t, int, double, double*, cudaStream_t);
int diag_rsqrt(mgx_ctx*, int, const double*, double*, cudaStream_t);
int cholesky(mgx_ctx*, int, double*, int*, cudaStream_t, int* info_dev = nullptr);
int inverse_from_cholesky(mgx_ctx*, int, const double*, double*, cudaStream_t);
int trace_prod(mgx_ctx*, int, const double*, const double*, double*, cudaStream_t);

static int check_grid(const mgx_grid* g)
{
    if (!g) return fail(MGX_BAD_ARG, "grid is NULL");
    for (int i = 0; i < 3; i++)
    {
        if (g->n[i] < 1 || g->n[i] > 8192)
            return fail(MGX_BAD_ARG, "grid dimension %d = %d out of range", i, g->n[i]);
        if (!(g->ll[i] > 0.))
            return fail(MGX_BAD_ARG, "domain length %d not positive", i);
        if (g->bc[i] != 1)
            return fail(MGX_UNSUPPORTED, "only periodic boundary conditions are implemented");
    }
    return MGX_OK;
}

static int check_dtype(int d)
{
    if (d != MGX_F64 && d != MGX_F32) return fail(MGX_BAD_ARG, "dtype %d invalid", d);
    return MGX_OK;
}

static int check_block(const mgx_grid& g, const void* p, size_t ld, int nfunc,
    const char* name)
{
    if (nfunc < 0) return fail(MGX_BAD_ARG, "%s: nfunc < 0", name);
    if (nfunc > 0 && !p) return fail(MGX_BAD_ARG, "%s is NULL", name);
    const size_t np = (size_t)g.n[0] * g.n[1] * g.n[2];
    if (nfunc > 1 && ld < np) return fail(MGX_BAD_ARG, "%s: ld %zu < %zu points", name, ld, np);
    return MGX_OK;
}

static PlaneParams plane(const mgx_grid& g)
{
    PlaneParams p;
    for (int i = 0; i < 3; i++)
        p.n[i] = g.n[i];
    return p;
}

int rhs_split_block(const mgx_grid& g, const float* u, size_t ldu, int nfunc, void* hi,
    void* lo, int rows, cudaStream_t s)
{
    PlaneParams p = plane(g);
    p.u          = u;
    p.ldu        = ldu;
    p.split_hi   = hi;
    p.split_lo   = lo;
    p.split_rows = rows;
    return stencil_launch(OP_RHS_SPLIT, 0, MGX_F32, MGX_F32, p, make_level(g, 0), 0., nfunc, s);
}

int hpsi_split_block(const mgx_grid& g, const float* psi, size_t ld, const float* V, float* out,
    int nfunc, void* hi, void* lo, int rows, cudaStream_t s)
{
    PlaneParams p = plane(g);
    p.u          = psi;
    p.ldu        = ld;
    p.V          = V;
    p.out        = out;
    p.ldo        = ld;
    p.split_hi   = hi;
    p.split_lo   = lo;
    p.split_rows = rows;
    return stencil_launch(OP_HPSI_B, 0, MGX_F32, MGX_F32, p, make_level(g, 0), 0., nfunc, s);
}

int rhs_block(const mgx_grid& g, int dtype, const void* u, size_t ldu, void* out,
    size_t ldo, int nfunc, cudaStream_t s)
{
    PlaneParams p = plane(g);
    p.u   = u;
    p.ldu = ldu;
    p.out = out;
    p.ldo = ldo;
    return stencil_launch(OP_RHS, 0, dtype, dtype, p, make_level(g, 0), 0., nfunc, s);
}
// ghosted restriction / extension: strip ghosts of the fine (resp. coarse)
// block, run the ghost-free kernel, write back inside the ghosted target.
template <typename T>
__global__ void strip_kernel(const T* g, int gw, int nx, int ny, int nz, T* out,
    size_t nfunc, int to_ghosted)
{
    const size_t np = (size_t)nx * ny * nz;
    const int ey = ny + 2 * gw, ez = nz + 2 * gw;
    const size_t sg = (size_t)(nx + 2 * gw) * ey * ez;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < np * nfunc;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t f = t / np, i = t - f * np;
        const int z = (int)(i % nz), y = (int)((i / nz) % ny), x = (int)(i / ((size_t)nz * ny));
        const size_t gi = f * sg + ((size_t)(x + gw) * ey + (y + gw)) * ez + z + gw;
        if (to_ghosted)
            const_cast<T*>(g)[gi] = out[t];
        else
            out[t] = g[gi];
    }
}

int strip(int dtype, const void* g, int gw, const int n[3], void* out,
    size_t nfunc, int to_ghosted, cudaStream_t s)
{
    const size_t np = (size_t)n[0] * n[1] * n[2] * nfunc;
    const int nb    = (int)std::min<size_t>((np + 255) / 256, 1u << 20);
    if (dtype == MGX_F64)
        strip_kernel<double><<<nb, 256, 0, s>>>((const double*)g, gw, n[0], n[1], n[2],
            (double*)out, nfunc, to_ghosted);
    else
        strip_kernel<float><<<nb, 256, 0, s>>>((const float*)g, gw, n[0], n[1], n[2],
            (float*)out, nfunc, to_ghosted);
    MGX_LAUNCH_CHECK("strip_kernel");
    return MGX_OK;
}

template <typename T>
__global__ void axpy_kernel(size_t n, T alpha, const T* __restrict__ x, T* __restrict__ y)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        y[i] += alpha * x[i];
}
// 16-byte grid-stride copy between device-accessible addresses (device
// memory, or pinned host memory through its mapped device address)
__global__ void copy16_kernel(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n)
{
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        dst[i] = src[i];
}

// the device-side address of p, or nullptr when the device cannot address it
static void* device_address(const void* p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    if (a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged)
        return const_cast<void*>(p);
    if (a.type == cudaMemoryTypeHost) return a.devicePointer;
    return nullptr;
}
} // namespace mgx

using namespace mgx;

extern "C" {

int mgx_copy(void* dst, const void* src, size_t bytes, void* stream)
{
    if (bytes == 0) return MGX_OK;
    if (!dst || !src) return fail(MGX_BAD_ARG, "NULL buffer");
    cudaStream_t s = (cudaStream_t)stream;
    void* d       = device_address(dst);
    void* r       = device_address(src);
    if (d && r && ((uintptr_t)d % 16) == 0 && ((uintptr_t)r % 16) == 0 && (bytes % 16) == 0)
    {
        int dev = 0, sms = 0;
        MGX_TRY(cuda_check(cudaGetDevice(&dev), "device"));
        MGX_TRY(cuda_check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev),
            "SM count"));
        const size_t n = bytes / 16;
        const int nb   = (int)std::min<size_t>((n + 255) / 256, (size_t)sms * 8);
        copy16_kernel<<<nb, 256, 0, s>>>((const uint4*)r, (uint4*)d, n);
        MGX_LAUNCH_CHECK("copy16_kernel");
        return MGX_OK;
    }
    return cuda_check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDefault, s), "copy");
}

int mgx_kernel_arch(int* binary_version)
{
    if (!binary_version) return fail(MGX_BAD_ARG, "NULL argument");
    cudaFuncAttributes a;
    MGX_TRY(cuda_check(cudaFuncGetAttributes(&a, copy16_kernel), "function attributes"));
    *binary_version = a.binaryVersion;
    return MGX_OK;
}

const char* mgx_last_error_string(void) { return g_err; }

unsigned long long mgx_kernel_launch_count(void) { return g_launches.load(); }

int mgx_create(const mgx_grid* grid, mgx_ctx** ctx)
{
    MGX_TRY(check_grid(grid));
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    int dev = 0;
    MGX_TRY(cuda_check(cudaGetDevice(&dev), "cudaGetDevice"));
    mgx_ctx* c = new mgx_ctx;
    c->grid    = *grid;
    int sms = 0, smem = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    c->sm_count   = sms > 0 ? sms : 152;
    c->smem_optin = (size_t)smem;
    *ctx          = c;
    return MGX_OK;
}

int mgx_destroy(mgx_ctx* ctx)
{
    delete ctx;
    return MGX_OK;
}

int mgx_fdkernel_del2(const mgx_grid* grid, int ghosts, int lap_type,
    mgx_dtype dtype, const void* v, void* b, size_t nfunc, void* stream)
{
    MGX_TRY(check_grid(grid));
    MGX_TRY(check_dtype(dtype));
    if (nfunc && (!v || !b)) return fail(MGX_BAD_ARG, "NULL block");
    return ghosted_del2(*grid, ghosts, lap_type, dtype, v, b, nfunc, (cudaStream_t)stream);
}

int mgx_fdkernel_rhs_mehr1(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* v, void* rhs, int rhs_ghosts, size_t nfunc, void* stream)
{
    MGX_TRY(check_grid(grid));
    MGX_TRY(check_dtype(dtype));
    if (nfunc && (!v || !rhs)) return fail(MGX_BAD_ARG, "NULL block");
    return ghosted_rhs(*grid, ghosts, dtype, v, rhs, rhs_ghosts, nfunc, (cudaStream_t)stream);
}

int mgx_trade_boundaries(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    void* u, size_t nfunc, void* stream)
{
    MGX_TRY(check_grid(grid));
    MGX_TRY(check_dtype(dtype));
    if (nfunc && !u) return fail(MGX_BAD_ARG, "NULL block");
    return ghosted_trade(*grid, ghosts, dtype, u, nfunc, (cudaStream_t)stream);
}

int mgx_axpy(size_t n, double alpha, mgx_dtype dtype, const void* x, void* y, void* stream)
{
    MGX_TRY(check_dtype(dtype));
    if (n == 0) return MGX_OK;
    if (!x || !y) return fail(MGX_BAD_ARG, "NULL vector");
    const int nb = (int)std::min<size_t>((n + 255) / 256, 8192);
    if (dtype == MGX_F64)
        axpy_kernel<double><<<nb, 256, 0, (cudaStream_t)stream>>>(n, alpha, (const double*)x,
            (double*)y);
    else
        axpy_kernel<float><<<nb, 256, 0, (cudaStream_t)stream>>>(n, (float)alpha,
            (const float*)x, (float*)y);
    MGX_LAUNCH_CHECK("axpy_kernel");
    return MGX_OK;
}

int mgx_mgkernel_restrict3d(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* fine, void* coarse, size_t nfunc, void* stream)
{
    MGX_TRY(check_grid(grid));
    MGX_TRY(check_dtype(dtype));
    if (ghosts < 1) return fail(MGX_BAD_ARG, "ghost width must be >= 1");
    if (nfunc == 0) return MGX_OK;
    if (!fine || !coarse) return fail(MGX_BAD_ARG, "NULL block");
    for (int i = 0; i < 3; i++)
        if (grid->n[i] % 2) return fail(MGX_BAD_ARG, "odd fine dimension");
    cudaStream_t s = (cudaStream_t)stream;
    const Level F  = make_level(*grid, 0), C = make_level(*grid, 1);
    DeviceBuffer a, b;
    const size_t es = dtype_size(dtype);
    MGX_TRY(a.ensure(F.npts() * nfunc * es));
    MGX_TRY(b.ensure(C.npts() * nfunc * es));
    // the fine ghosts are not needed: the ghost-free kernel wraps periodically
    MGX_TRY(strip(dtype, fine, ghosts, F.n, a.ptr, nfunc, 0, s));
    MGX_TRY(restrict_launch(dtype, F, a.ptr, F.npts(), b.ptr, C.npts(), (int)nfunc, MaskDev(), s));
    MGX_TRY(strip(dtype, coarse, ghosts, C.n, b.ptr, nfunc, 1, s));
    return cuda_check(cudaStreamSynchronize(s), "restrict3d sync");
}

int mgx_mgkernel_extend3d(const mgx_grid* grid, int ghosts, mgx_dtype dtype,
    const void* coarse, void* fine, size_t nfunc, void* stream)
{
    MGX_TRY(check_grid(grid));
    MGX_TRY(check_dtype(dtype));
    if (ghosts < 1) return fail(MGX_BAD_ARG, "ghost width must be >= 1");
    if (nfunc == 0) return MGX_OK;
    if (!fine || !coarse) return fail(MGX_BAD_ARG, "NULL block");
    for (int i = 0; i < 3; i++)
        if (grid->n[i] % 2) return fail(MGX_BAD_ARG, "odd fine dimension");
    cudaStream_t s = (cudaStream_t)stream;
    const Level F  = make_level(*grid, 0), C = make_level(*grid, 1);
    DeviceBuffer a, b;
    const size_t es = dtype_size(dtype);
    MGX_TRY(a.ensure(F.npts() * nfunc * es));
    MGX_TRY(b.ensure(C.npts() * nfunc * es));
    MGX_TRY(strip(dtype, coarse, ghosts, C.n, b.ptr, nfunc, 0, s));
    MGX_TRY(prolong_launch(dtype, 0, F, b.ptr, C.npts(), a.ptr, F.npts(), (int)nfunc, MaskDev(), s));
    MGX_TRY(strip(dtype, fine, ghosts, F.n, a.ptr, nfunc, 1, s));
    // the reference also injects the first high-side ghost layer; refresh
    // the fine ghosts so that they hold the periodic images
    MGX_TRY(ghosted_trade(*grid, ghosts, dtype, fine, nfunc, s));
    return cuda_check(cudaStreamSynchronize(s), "extend3d sync");
}

int mgx_fd_apply(mgx_ctx* ctx, int lap_type, mgx_dtype dtype, const void* u,
    size_t ld, void* out, int nfunc, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, u, ld, nfunc, "u"));
    MGX_TRY(check_block(ctx->grid, out, ld, nfunc, "out"));
    if (lap_radius(lap_type) < 0) return fail(MGX_BAD_ARG, "lap_type %d", lap_type);
    PlaneParams p = plane(ctx->grid);
    p.u   = u;
    p.ldu = ld;
    p.out = out;
    p.ldo = ld;
    return stencil_launch(OP_LAP, lap_type, dtype, dtype, p, make_level(ctx->grid, 0),
        0., nfunc, (cudaStream_t)stream);
}

int mgx_rhs_mehr(mgx_ctx* ctx, mgx_dtype dtype, const void* u, size_t ld,
    void* out, int nfunc, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, u, ld, nfunc, "u"));
    MGX_TRY(check_block(ctx->grid, out, ld, nfunc, "out"));
    PlaneParams p = plane(ctx->grid);
    p.u   = u;
    p.ldu = ld;
    p.out = out;
    p.ldo = ld;
    return stencil_launch(OP_RHS, 0, dtype, dtype, p, make_level(ctx->grid, 0), 0.,
        nfunc, (cudaStream_t)stream);
}

int mgx_hpsi(mgx_ctx* ctx, int lap_type, mgx_dtype dtype, const void* psi,
    size_t ld, const void* V, mgx_dtype v_dtype, void* hpsi, int nfunc,
    int apply_B_to_V, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_dtype(v_dtype));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    if (nfunc && !V) return fail(MGX_BAD_ARG, "V is NULL");
    if (lap_radius(lap_type) < 0) return fail(MGX_BAD_ARG, "lap_type %d", lap_type);
    if (psi == hpsi) return fail(MGX_BAD_ARG, "psi and hpsi alias");
    PlaneParams p = plane(ctx->grid);
    p.u   = psi;
    p.ldu = ld;
    p.V   = V;
    p.out = hpsi;
    p.ldo = ld;
    const int op = (lap_type == 0 && apply_B_to_V) ? OP_HPSI_B : OP_HPSI_V;
    return stencil_launch(op, lap_type, dtype, v_dtype, p, make_level(ctx->grid, 0),
        0., nfunc, (cudaStream_t)stream);
}

int mgx_mg_restrict(mgx_ctx* ctx, int level, mgx_dtype dtype, const void* fine,
    void* coarse, int nfunc, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    if (level < 0) return fail(MGX_BAD_ARG, "level < 0");
    const Level F = make_level(ctx->grid, level);
    for (int i = 0; i < 3; i++)
        if (F.n[i] < 2 || F.n[i] % 2) return fail(MGX_BAD_ARG, "level %d not coarsenable", level);
    if (nfunc && (!fine || !coarse)) return fail(MGX_BAD_ARG, "NULL block");
    if (nfunc == 0) return MGX_OK;
    return restrict_launch(dtype, F, fine, F.npts(), coarse, F.npts() / 8, nfunc,
        MaskDev(), (cudaStream_t)stream);
}

int mgx_mg_prolong(mgx_ctx* ctx, int level, mgx_dtype dtype, const void* coarse,
    void* fine, int nfunc, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    if (level < 0) return fail(MGX_BAD_ARG, "level < 0");
    const Level F = make_level(ctx->grid, level);
    for (int i = 0; i < 3; i++)
        if (F.n[i] < 2 || F.n[i] % 2) return fail(MGX_BAD_ARG, "level %d not coarsenable", level);
    if (nfunc && (!fine || !coarse)) return fail(MGX_BAD_ARG, "NULL block");
    if (nfunc == 0) return MGX_OK;
    return prolong_launch(dtype, 0, F, coarse, F.npts() / 8, fine, F.npts(), nfunc,
        MaskDev(), (cudaStream_t)stream);
}

int mgx_precond_mg(mgx_ctx* ctx, const mgx_precond_params* p, mgx_dtype dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks,
    void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, res, ld, nfunc, "res"));
    MGX_TRY(check_block(ctx->grid, out, ld, nfunc, "out"));
    if (masks && masks->dtype != dtype)
        return fail(MGX_BAD_ARG, "mask value type differs from the orbital type");
    const size_t np = (size_t)ctx->grid.n[0] * ctx->grid.n[1] * ctx->grid.n[2];
    const size_t ldv = nfunc > 1 ? ld : (ld ? ld : np);
    int st = precond_mg(ctx, p, dtype, res, ldv, out, nfunc, masks, (cudaStream_t)stream);
    if (st != MGX_OK) return st;
    return MGX_OK;
}

int mgx_precond_mg_warm(mgx_ctx* ctx, const mgx_precond_params* p, mgx_dtype dtype,
    const void* res, size_t ld, void* out, int nfunc, const mgx_masks* masks, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, res, ld, nfunc, "res"));
    MGX_TRY(check_block(ctx->grid, out, ld, nfunc, "out"));
    if (masks && masks->dtype != dtype)
        return fail(MGX_BAD_ARG, "mask value type differs from the orbital type");
    const size_t np  = (size_t)ctx->grid.n[0] * ctx->grid.n[1] * ctx->grid.n[2];
    const size_t ldv = nfunc > 1 ? ld : (ld ? ld : np);
    return precond_mg(ctx, p, dtype, res, ldv, out, nfunc, masks, (cudaStream_t)stream, nullptr,
        0., nullptr, true);
}

int mgx_precond_mg_update(mgx_ctx* ctx, const mgx_precond_params* p, mgx_dtype dtype,
    const void* res, size_t ld, void* psi, double alpha, const double* psi_scale, int nfunc,
    const mgx_masks* masks, void* work, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, res, ld, nfunc, "res"));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    if (masks && masks->dtype != dtype)
        return fail(MGX_BAD_ARG, "mask value type differs from the orbital type");
    const size_t np  = (size_t)ctx->grid.n[0] * ctx->grid.n[1] * ctx->grid.n[2];
    const size_t ldv = nfunc > 1 ? ld : (ld ? ld : np);
    if (work) MGX_TRY(check_block(ctx->grid, work, ld, nfunc, "work"));
    return precond_mg(ctx, p, dtype, res, ldv, work, nfunc, masks, (cudaStream_t)stream, psi,
        alpha, psi_scale);
}

int mgx_precond_gamma(const mgx_grid* grid, int lap_type, int mg_levels,
    double vmax, double small_eig, double* gamma)
{
    MGX_TRY(check_grid(grid));
    if (!gamma) return fail(MGX_BAD_ARG, "gamma is NULL");
    if (lap_radius(lap_type) < 0) return fail(MGX_BAD_ARG, "lap_type %d", lap_type);
    const Level L = make_level(*grid, 0);
    // invDiagEl() of the operator (src/pb/Laph*.h); Laph4M: 1 / ((4/3) sum)
    const double s = 1. / (L.h[0] * L.h[0]) + 1. / (L.h[1] * L.h[1])
                     + 1. / (L.h[2] * L.h[2]);
    double diag = 0.;
    switch (lap_type)
    {
        case 0: diag = (4. / 3.) * s; break;
        case 1: diag = 2. * s; break;
        case 2: diag = 2.5 * s; break;
        case 3: diag = (49. / 18.) * s; break;
        case 4: diag = (1435. / 504.) * s; break;
    }
    double g = 1. / diag;
    for (int ln = 0; ln <= mg_levels; ln++)
        g *= 4.;
    *gamma = 1.0 / (2.0 / g + fabs(vmax - small_eig));
    return MGX_OK;
}

int mgx_masks_create(mgx_ctx* ctx, int nlevels, int nfunc, const double* centers,
    const double* radii, int func, int kind, int mesh_ghosts, mgx_dtype dtype,
    mgx_masks** masks, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    if (mesh_ghosts < 1) return fail(MGX_BAD_ARG, "mesh ghost width < 1");
    return masks_create(ctx, nlevels, nfunc, centers, radii, func, kind, mesh_ghosts,
        dtype, masks, (cudaStream_t)stream);
}

int mgx_masks_update(mgx_ctx* ctx, mgx_masks* masks, const double* centers,
    const double* radii, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return masks_update(ctx, masks, centers, radii, (cudaStream_t)stream);
}

int mgx_masks_destroy(mgx_masks* masks)
{
    delete masks;
    return MGX_OK;
}

int mgx_masks_apply(mgx_ctx* ctx, const mgx_masks* masks, int level, void* u,
    size_t ld, int nfunc, void* stream)
{
    if (!ctx || !masks) return fail(MGX_BAD_ARG, "NULL ctx or masks");
    if (nfunc < 0) return fail(MGX_BAD_ARG, "nfunc < 0");
    if (level < 0) return fail(MGX_BAD_ARG, "level < 0");
    if (nfunc && !u) return fail(MGX_BAD_ARG, "u is NULL");
    const Level L = make_level(ctx->grid, level);
    if (nfunc > 1 && ld < L.npts()) return fail(MGX_BAD_ARG, "ld below level size");
    return masks_apply(ctx, masks, level, u, ld ? ld : L.npts(), nfunc, (cudaStream_t)stream);
}

int mgx_masks_expand(const mgx_masks* masks, int level, void* dense,
    int* host_state, void* stream)
{
    if (!masks || !dense) return fail(MGX_BAD_ARG, "NULL masks or output");
    return masks_expand(masks, level, dense, host_state, (cudaStream_t)stream);
}

int mgx_gram(mgx_ctx* ctx, int mode, const void* psi, size_t ld, int nfunc,
    double* S, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    if (nfunc == 0) return MGX_OK;
    if (!S) return fail(MGX_BAD_ARG, "S is NULL");
    const Level L    = make_level(ctx->grid, 0);
    const double vel = L.h[0] * L.h[1] * L.h[2];
    const size_t ldv = nfunc > 1 ? ld : L.npts();
    cudaStream_t s   = (cudaStream_t)stream;
    switch (mode)
    {
        case MGX_GEMM_FP64:
            return gram_cuda_cores(ctx, MGX_F64, psi, psi, ldv, L.npts(), nfunc, vel, 1, S, s);
        case MGX_GEMM_FP32:
            return gram_cuda_cores(ctx, MGX_F32, psi, psi, ldv, L.npts(), nfunc, vel, 1, S, s);
        case MGX_GEMM_TF32:
        case MGX_GEMM_BF16X3:
        case MGX_GEMM_FP16X3:
            return gram_tcgen05(ctx, mode, psi, psi, ldv, L.npts(), nfunc, vel, 1, S, s);
    }
    return fail(MGX_BAD_ARG, "gemm mode %d", mode);
}

int mgx_hmat(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi, size_t ld,
    int nfunc, double* H, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    if (nfunc == 0) return MGX_OK;
    if (!H) return fail(MGX_BAD_ARG, "H is NULL");
    const Level L    = make_level(ctx->grid, 0);
    const double vel = L.h[0] * L.h[1] * L.h[2];
    const size_t ldv = nfunc > 1 ? ld : L.npts();
    cudaStream_t s   = (cudaStream_t)stream;
    switch (mode)
    {
        case MGX_GEMM_FP64:
            return gram_cuda_cores(ctx, MGX_F64, psi, hpsi, ldv, L.npts(), nfunc, vel, 0, H, s);
        case MGX_GEMM_FP32:
            return gram_cuda_cores(ctx, MGX_F32, psi, hpsi, ldv, L.npts(), nfunc, vel, 0, H, s);
        case MGX_GEMM_TF32:
        case MGX_GEMM_BF16X3:
        case MGX_GEMM_FP16X3:
            return gram_tcgen05(ctx, mode, psi, hpsi, ldv, L.npts(), nfunc, vel, 0, H, s);
    }
    return fail(MGX_BAD_ARG, "gemm mode %d", mode);
}

int mgx_gram_hmat(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, int nfunc, double* S, double* H, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    if (nfunc == 0) return MGX_OK;
    if (!S || !H) return fail(MGX_BAD_ARG, "S or H is NULL");
    if (mode == MGX_GEMM_TF32 || mode == MGX_GEMM_BF16X3 || mode == MGX_GEMM_FP16X3)
    {
        const Level L    = make_level(ctx->grid, 0);
        const double vel = L.h[0] * L.h[1] * L.h[2];
        const size_t ldv = nfunc > 1 ? ld : L.npts();
        return gram_hmat_tcgen05(ctx, mode, psi, hpsi, ldv, L.npts(), nfunc, vel, S, H,
            (cudaStream_t)stream);
    }
    MGX_TRY(mgx_gram(ctx, mode, psi, ld, nfunc, S, stream));
    return mgx_hmat(ctx, mode, psi, hpsi, ld, nfunc, H, stream);
}

/* the block that holds B Psi: the caller's (work_funcs functions) or, for a
 * NULL work, ctx's residual block grown to at most 512 functions */
static int matb_work(mgx_ctx* ctx, int mode, size_t ld, int nfunc, void** work, int* wf)
{
    if (*work)
    {
        if (*wf < 1) return fail(MGX_BAD_ARG, "work_funcs %d < 1", *wf);
        *wf = std::min(*wf, nfunc);
        return MGX_OK;
    }
    const size_t es = mode == MGX_GEMM_FP64 ? 8 : 4;
    *wf             = std::min(nfunc, 512);
    MGX_TRY(ctx->resid.ensure((size_t)(*wf) * ld * es + 256));
    *work = ctx->resid.ptr;
    return MGX_OK;
}

static int check_gemm_mode(int mode)
{
    switch (mode)
    {
        case MGX_GEMM_FP64:
        case MGX_GEMM_FP32:
        case MGX_GEMM_TF32:
        case MGX_GEMM_BF16X3:
        case MGX_GEMM_FP16X3: return MGX_OK;
    }
    return fail(MGX_BAD_ARG, "gemm mode %d", mode);
}

int mgx_matb(mgx_ctx* ctx, int mode, const void* psi, size_t ld, int nfunc, double* Bm,
    void* work, int work_funcs, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_gemm_mode(mode));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    if (nfunc == 0) return MGX_OK;
    if (!Bm) return fail(MGX_BAD_ARG, "B is NULL");
    if (work == psi) return fail(MGX_BAD_ARG, "work aliases psi");
    const Level L    = make_level(ctx->grid, 0);
    const double vel = L.h[0] * L.h[1] * L.h[2];
    const size_t ldv = nfunc > 1 ? ld : L.npts();
    int wf = work_funcs;
    MGX_TRY(matb_work(ctx, mode, ldv, nfunc, &work, &wf));
    cudaStream_t s = (cudaStream_t)stream;
    if (mode == MGX_GEMM_FP64 || mode == MGX_GEMM_FP32)
        return matb_cuda_cores(ctx, mode == MGX_GEMM_FP64 ? MGX_F64 : MGX_F32, psi, ldv,
            L.npts(), nfunc, vel, Bm, work, wf, s);
    return matb_tcgen05(ctx, mode, psi, ldv, L.npts(), nfunc, vel, Bm, work, wf, s);
}

int mgx_gram_hmat_matb(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, int nfunc, double* S, double* H, double* Bm, void* work, int work_funcs,
    void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_gemm_mode(mode));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    if (nfunc == 0) return MGX_OK;
    if (!S || !H || !Bm) return fail(MGX_BAD_ARG, "S, H or B is NULL");
    if (work == psi || work == hpsi) return fail(MGX_BAD_ARG, "work aliases psi or hpsi");
    if (mode == MGX_GEMM_TF32 || mode == MGX_GEMM_BF16X3 || mode == MGX_GEMM_FP16X3)
    {
        const Level L    = make_level(ctx->grid, 0);
        const double vel = L.h[0] * L.h[1] * L.h[2];
        const size_t ldv = nfunc > 1 ? ld : L.npts();
        int wf = work_funcs;
        MGX_TRY(matb_work(ctx, mode, ldv, nfunc, &work, &wf));
        return gram_hmat_tcgen05(ctx, mode, psi, hpsi, ldv, L.npts(), nfunc, vel, S, H,
            (cudaStream_t)stream, Bm, work, wf);
    }
    MGX_TRY(mgx_gram(ctx, mode, psi, ld, nfunc, S, stream));
    MGX_TRY(mgx_hmat(ctx, mode, psi, hpsi, ld, nfunc, H, stream));
    return mgx_matb(ctx, mode, psi, ld, nfunc, Bm, work, work_funcs, stream);
}

int mgx_hpsi_gram_hmat_matb(mgx_ctx* ctx, int mode, const float* psi, const float* V,
    float* hpsi, size_t ld, int nfunc, double* S, double* H, double* Bm, void* work,
    int work_funcs, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_gemm_mode(mode));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    if (nfunc == 0) return MGX_OK;
    if (!V) return fail(MGX_BAD_ARG, "V is NULL");
    if (!S || !H || !Bm) return fail(MGX_BAD_ARG, "S, H or B is NULL");
    if ((const void*)psi == (const void*)hpsi) return fail(MGX_BAD_ARG, "psi and hpsi alias");
    if (work == psi || work == hpsi) return fail(MGX_BAD_ARG, "work aliases psi or hpsi");
    if (mode == MGX_GEMM_BF16X3)
    {
        const Level L    = make_level(ctx->grid, 0);
        const double vel = L.h[0] * L.h[1] * L.h[2];
        const size_t ldv = nfunc > 1 ? ld : L.npts();
        int wf = work_funcs;
        MGX_TRY(matb_work(ctx, mode, ldv, nfunc, &work, &wf));
        return gram_hmat_tcgen05(ctx, mode, psi, hpsi, ldv, L.npts(), nfunc, vel, S, H,
            (cudaStream_t)stream, Bm, work, wf, V, 0);
    }
    MGX_TRY(mgx_hpsi(ctx, 0, MGX_F32, psi, ld, V, MGX_F32, hpsi, nfunc, 1, stream));
    return mgx_gram_hmat_matb(ctx, mode, psi, hpsi, ld, nfunc, S, H, Bm, work, work_funcs, stream);
}

int mgx_update_hb(mgx_ctx* ctx, int n, const double* S, const double* theta, double* HB,
    void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return update_hb(n, S, theta, HB, (cudaStream_t)stream);
}

int mgx_normalize(mgx_ctx* ctx, mgx_dtype dtype, void* psi, size_t ld, int nfunc,
    double* diagS, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    if (nfunc == 0) return MGX_OK;
    const Level L    = make_level(ctx->grid, 0);
    const double vel = L.h[0] * L.h[1] * L.h[2];
    const size_t ldv = nfunc > 1 ? ld : L.npts();
    return normalize(ctx, dtype, psi, ldv, L.npts(), nfunc, vel, diagS, (cudaStream_t)stream);
}

int mgx_normalize_scales(mgx_ctx* ctx, int n, const double* S, double* scale, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return diag_rsqrt(ctx, n, S, scale, (cudaStream_t)stream);
}

int mgx_cholesky(mgx_ctx* ctx, int n, double* A, int* info, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return cholesky(ctx, n, A, info, (cudaStream_t)stream);
}

int mgx_set_reuse_conversion(mgx_ctx* ctx, int on)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    ctx->reuse_conversion = on ? 1 : 0;
    return MGX_OK;
}

int mgx_cholesky_async(mgx_ctx* ctx, int n, double* A, int* info, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    if (!info) return fail(MGX_BAD_ARG, "info is NULL");
    return cholesky(ctx, n, A, nullptr, (cudaStream_t)stream, info);
}

int mgx_inverse_from_cholesky(mgx_ctx* ctx, int n, const double* L, double* Sinv,
    void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return inverse_from_cholesky(ctx, n, L, Sinv, (cudaStream_t)stream);
}

int mgx_trace_prod(mgx_ctx* ctx, int n, const double* H, const double* Sinv,
    double* trace, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return trace_prod(ctx, n, H, Sinv, trace, (cudaStream_t)stream);
}

int mgx_theta_from_cholesky(mgx_ctx* ctx, int n, const double* L, const double* H,
    double* theta, double* trace, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    return theta_from_cholesky(ctx, n, L, H, theta, trace, (cudaStream_t)stream);
}

int mgx_theta(mgx_ctx* ctx, int n, const double* Sinv, const double* H,
    double* theta, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    if (theta == Sinv || theta == H) return fail(MGX_BAD_ARG, "theta aliases an input");
    return theta_product(n, Sinv, H, theta, (cudaStream_t)stream);
}
}

namespace mgx
{
/* out_j = sum_i psi_i theta(i, j) + beta cin_j for the ncols columns of
 * theta at theta + j * nfunc (cin may alias out, out may not alias psi) */
static int mult_matrix(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    size_t ld, int nfunc, const double* theta, int ncols, double beta, const void* cin,
    void* out, cudaStream_t s)
{
    const size_t npts = make_level(ctx->grid, 0).npts();
    const size_t ldv  = (nfunc > 1 || ncols > 1) ? ld : npts;
    switch (mode)
    {
        case MGX_GEMM_FP64:
            // FP64 accumulation for either orbital type, as MPgemmNN does
            return psi_theta_cuda_cores(dtype == MGX_F64 ? 0 : 1, psi, ldv, npts, nfunc,
                theta, nfunc, ncols, beta, cin, out, s);
        case MGX_GEMM_FP32:
        case MGX_GEMM_TF32:
        case MGX_GEMM_BF16X3:
        case MGX_GEMM_FP16X3:
            if (dtype != MGX_F32)
                return fail(MGX_BAD_ARG, "gemm mode %d needs FP32 orbitals", mode);
            if (mode == MGX_GEMM_FP32)
                return psi_theta_cuda_cores(2, psi, ldv, npts, nfunc, theta, nfunc, ncols, beta,
                    cin, out, s);
            return psi_theta_tcgen05(ctx, mode, (const float*)psi, ldv, npts, nfunc, theta,
                nfunc, ncols, (float)beta, (const float*)cin, (float*)out, s);
    }
    return fail(MGX_BAD_ARG, "gemm mode %d", mode);
}

/* res_j = B(sum_i psi_i theta(i, j)) - hpsi_j (apply_B) or without B, for
 * the ncols columns of theta given; hpsi, work and res hold ncols
 * functions */
static int residual_cols(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    const void* hpsi, size_t ld, int nfunc, const double* theta, int ncols, int apply_B,
    void* work, void* res, cudaStream_t s)
{
    if (ncols == 0 || nfunc == 0) return MGX_OK;
    if (!theta) return fail(MGX_BAD_ARG, "theta is NULL");
    if (ncols < 0 || ncols > nfunc) return fail(MGX_BAD_ARG, "ncols %d of %d", ncols, nfunc);
    if (res == psi) return fail(MGX_BAD_ARG, "psi and res alias");
    if (!apply_B)
        // res = psi theta - hpsi in one pass (res may be hpsi)
        return mult_matrix(ctx, mode, dtype, psi, ld, nfunc, theta, ncols, -1., hpsi, res, s);
    const Level L   = make_level(ctx->grid, 0);
    const size_t lw = (nfunc > 1 || ncols > 1) ? ld : L.npts();
    if (!work)
    {
        MGX_TRY(ctx->resid.ensure(lw * ncols * dtype_size(dtype)));
        work = ctx->resid.ptr;
    }
    if (work == psi || work == hpsi || work == res)
        return fail(MGX_BAD_ARG, "work aliases psi, hpsi or res");
    // B (psi theta) = (B psi) theta: the product first, then one stencil
    // pass res = B work - hpsi
    MGX_TRY(mult_matrix(ctx, mode, dtype, psi, ld, nfunc, theta, ncols, 0., nullptr, work, s));
    PlaneParams p = plane(ctx->grid);
    p.u   = work;
    p.ldu = lw;
    p.f   = hpsi;
    p.ldf = lw;
    p.out = res;
    p.ldo = lw;
    return stencil_launch(OP_RHS_SUB, 0, dtype, dtype, p, L, 0., ncols, s);
}
} // namespace mgx

extern "C" {

int mgx_mult_matrix(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    size_t ld, int nfunc, const double* theta, void* out, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, out, ld, nfunc, "out"));
    if (nfunc == 0) return MGX_OK;
    if (!theta) return fail(MGX_BAD_ARG, "theta is NULL");
    if (psi == out) return fail(MGX_BAD_ARG, "psi and out alias");
    return mult_matrix(ctx, mode, dtype, psi, ld, nfunc, theta, nfunc, 0., nullptr, out,
        (cudaStream_t)stream);
}

int mgx_residual(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    const void* hpsi, size_t ld, int nfunc, const double* theta, int apply_B,
    void* work, void* res, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, nfunc, "hpsi"));
    MGX_TRY(check_block(ctx->grid, res, ld, nfunc, "res"));
    return residual_cols(ctx, mode, dtype, psi, hpsi, ld, nfunc, theta, nfunc, apply_B, work,
        res, (cudaStream_t)stream);
}

int mgx_residual_cols(mgx_ctx* ctx, int mode, mgx_dtype dtype, const void* psi,
    const void* hpsi, size_t ld, int nfunc, const double* theta, int ncols, int apply_B,
    void* work, void* res, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    MGX_TRY(check_block(ctx->grid, psi, ld, nfunc, "psi"));
    MGX_TRY(check_block(ctx->grid, hpsi, ld, ncols, "hpsi"));
    MGX_TRY(check_block(ctx->grid, res, ld, ncols, "res"));
    if (nfunc > 1 && ncols == 1 && ld < make_level(ctx->grid, 0).npts())
        return fail(MGX_BAD_ARG, "ld below the grid size");
    return residual_cols(ctx, mode, dtype, psi, hpsi, ld, nfunc, theta, ncols, apply_B, work,
        res, (cudaStream_t)stream);
}

int mgx_mgm(mgx_ctx* ctx, const mgx_mgm_params* params, mgx_dtype dtype, void* vh,
    const void* rho, mgx_mgm_result* result, void* stream)
{
    if (!ctx) return fail(MGX_BAD_ARG, "ctx is NULL");
    MGX_TRY(check_dtype(dtype));
    return mgm_solve(ctx, params, dtype, vh, rho, result, (cudaStream_t)stream);
}

} // extern "C"
