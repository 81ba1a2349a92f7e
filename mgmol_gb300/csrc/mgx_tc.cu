// Tensor-core (tcgen05) Gram / H-matrix products on sm_103a.
//
// C[i][j] += sum_k A[i][k] B[j][k] over the orbital block (K = grid points),
// the "TN" product of two K-major operands.  One CTA owns a 128 x BN output
// tile and a contiguous range of K blocks:
//   warp 0      TMA producer: 2-D tiled bulk tensor copies (SWIZZLE_128B)
//               of the A and B K-slices into an S-stage shared-memory ring;
//   warp 1      allocates the TMEM accumulator (128 lanes x BN FP32
//               columns) and issues tcgen05.mma from one thread, committing
//               each stage back to its "empty" mbarrier;
//   warps 2-5   epilogue: tcgen05.ld of the accumulator, FP64 atomic
//               accumulation of the partial tile into C.
// Modes:
//   TF32   -- the FP32 orbitals feed kind::tf32 directly;
//   BF16X3 -- each operand is split once into bf16 hi + lo planes
//             (x = hi + lo to 2^-16 relative), and every K step issues
//             hi*hi + hi*lo + lo*hi into the same FP32 accumulator;
//   FP16X3 -- the same with fp16 planes of the operand scaled by a power of
//             two (max |x| 2^s < 2^14, found by a device max reduction):
//             x 2^s = hi + lo to 2^-22, same cost; the scales come off
//             exactly in the epilogue or the finishing pass.
// The K range of a CTA is bounded (at most 512 K blocks) so that the FP32
// accumulation error stays small; partial tiles meet in FP64.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "mgx_internal.cuh"
#include "mgx_stencil.cuh"

namespace mgx
{
int gram_cuda_cores(mgx_ctx*, int, const void*, const void*, size_t, size_t,
    int, double, int, double*, cudaStream_t);

namespace tc
{
constexpr int BM      = 128;
constexpr int THREADS = 192;

// Shared-memory operand descriptor of a K-major tile whose rows are one
// swizzle atom of SW bytes (128 or 64): stride between 8-row groups 8 * SW,
// layout SWIZZLE_128B (2) or SWIZZLE_64B (4).
template <int SW>
__device__ __forceinline__ uint64_t desc_sw(uint32_t saddr)
{
    static_assert(SW == 128 || SW == 64, "swizzle atom");
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;                 // leading byte offset (unused, K-major swizzled)
    d |= (uint64_t)((8 * SW) >> 4) << 32;   // stride byte offset: 8 rows x SW bytes
    d |= (uint64_t)1 << 46;                 // descriptor version for tcgen05
    d |= (uint64_t)(SW == 128 ? 2 : 4) << 61;
    return d;
}

// Shared-memory descriptor of an MN-major tile (bf16) under SWIZZLE_128B:
// rows of 128 bytes hold 64 consecutive MN elements (one K index each),
// 8-row groups (K) are 1024 bytes apart (stride byte offset) and the next
// 64 MN elements start lbo bytes further (leading byte offset).
__device__ __forceinline__ uint64_t desc_mn128(uint32_t saddr, uint32_t lbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// kind::tf32 (KIND 0, operand format 2), kind::f16 with bf16 operands
// (KIND 1, format 1) or with fp16 operands (KIND 2, format 0); FP32 D, both
// operands K-major
template <int KIND>
__host__ __device__ constexpr uint32_t instr_desc(int M, int N)
{
    return (1u << 4) | ((KIND == 0 ? 2u : KIND == 1 ? 1u : 0u) << 7)
           | ((KIND == 0 ? 2u : KIND == 1 ? 1u : 0u) << 10) | ((uint32_t)(N >> 3) << 17)
           | ((uint32_t)(M >> 4) << 24);
}

// Power-of-two scale of an operand for the fp16 split: maxbits is the bit
// pattern of max |x| (atomicMax on the bits of non-negative floats), up =
// 2^s with s chosen so that max |x| 2^s < 2^14, down = 2^-s.
struct ScaleSlot
{
    unsigned maxbits;
    float up;
    double down;
};

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map,
    int c0, int c1, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

// 3-D box of a K-blocked operand: (element within the 64-element K block,
// row, K block)
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map,
    int c0, int c1, int c2, uint64_t* bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map)
{
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map))
                 : "memory");
}

template <int KIND>
__device__ __forceinline__ void mma(uint32_t tmem, uint64_t ad, uint64_t bd,
    uint32_t idesc, uint32_t acc)
{
    if (KIND == 0)
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
    else
        asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                     "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar)
{
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                 "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                 "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                 "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
                 "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),
                 "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]),
                 "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++)
        v[i] = __uint_as_float(r[i]);
}

struct Params
{
    const int2* tiles;
    int kblocks;    // total K blocks
    int kb_per_cta; // K blocks per CTA
    int n;          // rows of C (and its leading dimension)
    int ncols;      // columns of C produced by this launch
    int symmetric;  // only i >= j + col0 entries of C are produced
    int col0 = 0;   // global column of the launch's first column (C points there)
    double* C;      // column-major, leading dimension n, FP64, accumulated atomically
    int* err;
    // store epilogue (points x functions products): tile t of the launch is
    // (t / ntj, t % ntj); out[j * ldo + i] = acc(i, j) + beta * cin[j * ldo + i]
    // for i < nrows, j < ncols (cin may alias out)
    float* out       = nullptr;
    const float* cin = nullptr;
    size_t ldo       = 0;
    float beta       = 0.f;
    int nrows        = 0;
    int ntj          = 1;
    // the operand maps are K-blocked 3-D maps (rows of 64 K elements, one
    // contiguous block of all rows per 64 K) instead of row-major 2-D maps
    int blocked = 0;
    // fp16 split: the products carry the operands' scales; the store
    // epilogue multiplies by sa->down * sb->down
    const ScaleSlot* sa = nullptr;
    const ScaleSlot* sb = nullptr;
    // density epilogue (store mode): instead of storing the product,
    // rho[i] += sum_j (float)(acc(i, j) * rpsi[j * ldr + i]) in FP64
    double* rho       = nullptr;
    const float* rpsi = nullptr;
    size_t ldr        = 0;
};

// KIND 0: tf32 (NPROD 1); KIND 1: bf16 (NPROD 1 plain, 3 for hi/lo split).
// STORE false: FP64 atomic accumulation of split-K partial tiles into C;
// STORE true: one CTA per output tile over the whole K range, FP32 store.
// SW: bytes of K per tile row and stage (128: SWIZZLE_128B; 64: SWIZZLE_64B,
// half the K per stage and twice the stages in the same shared memory).
// AMN: the A operand is MN-major (bf16, rows of 64 points per K index, the
// K-blocked planes of the Gram product read with the roles of points and
// functions exchanged): A tiles are 2 blocks of 64 MN elements x BK K rows.
template <int KIND, int NPROD, int BN, int STAGES, bool STORE = false, int SW = 128,
    bool AMN = false>
__global__ void __launch_bounds__(THREADS, 1) gram_kernel(
    const __grid_constant__ CUtensorMap mA0, const __grid_constant__ CUtensorMap mA1,
    const __grid_constant__ CUtensorMap mB0, const __grid_constant__ CUtensorMap mB1,
    Params p)
{
    constexpr int NOP     = (NPROD == 3) ? 2 : 1;       // planes per operand
    constexpr int A_BYTES = BM * SW;
    constexpr int B_BYTES = BN * SW;
    constexpr int STAGE   = NOP * (A_BYTES + B_BYTES);
    constexpr int KSTEP   = 32;                          // bytes of K per MMA
    constexpr int NK      = SW / KSTEP;                  // MMAs per plane pair
    constexpr int ELEM    = (KIND == 0) ? 4 : 2;
    constexpr int BK      = SW / ELEM;                   // K elements per block
    constexpr uint32_t TMEM_COLS = BN;                   // power of two >= 32

    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full  = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);
    uint64_t* empty = full + STAGES;
    uint64_t* accf  = empty + STAGES;
    uint32_t* tslot = reinterpret_cast<uint32_t*>(accf + 1);

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int2 tile = STORE ? make_int2((int)blockIdx.x / p.ntj, (int)blockIdx.x % p.ntj)
                            : p.tiles[blockIdx.x];
    const int i0 = tile.x * BM, j0 = tile.y * BN;
    const int kb0 = blockIdx.y * p.kb_per_cta;
    const int kb1 = min(p.kblocks, kb0 + p.kb_per_cta);
    const int nkb = kb1 - kb0;

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < STAGES; s++)
        {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        mbar_init(accf, 1);
        fence_mbar_init();
    }
    if (warp == 1)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
            "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;
    bool ok = true;

    if (warp == 0 && lane == 0)
    {
        prefetch_map(&mA0);
        prefetch_map(&mB0);
        if (NPROD == 3)
        {
            prefetch_map(&mA1);
            prefetch_map(&mB1);
        }
        for (int it = 0; it < nkb && ok; it++)
        {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)((it / STAGES) & 1);
            ok = mbar_wait(empty + s, ph ^ 1u);
            if (!ok) break;
            unsigned char* st = smem + s * STAGE;
            mbar_arrive_expect_tx(full + s, STAGE);
            const int kc = (kb0 + it) * BK;
            if (AMN)
            {
                // A: points i0 .. i0 + 127 (two 64-point blocks) x K rows kc ..
                tma_load_3d(st, &mA0, 0, kc, i0 / 64, full + s);
                if (NPROD == 3) tma_load_3d(st + A_BYTES, &mA1, 0, kc, i0 / 64, full + s);
                const int e0 = kc % 64, kb = kc / 64;
                tma_load_3d(st + NOP * A_BYTES, &mB0, e0, j0, kb, full + s);
                if (NPROD == 3)
                    tma_load_3d(st + NOP * A_BYTES + B_BYTES, &mB1, e0, j0, kb, full + s);
            }
            else if (p.blocked)
            {
                const int e0 = kc % 64, kb = kc / 64;
                tma_load_3d(st, &mA0, e0, i0, kb, full + s);
                tma_load_3d(st + NOP * A_BYTES, &mB0, e0, j0, kb, full + s);
                if (NPROD == 3)
                {
                    tma_load_3d(st + A_BYTES, &mA1, e0, i0, kb, full + s);
                    tma_load_3d(st + NOP * A_BYTES + B_BYTES, &mB1, e0, j0, kb, full + s);
                }
            }
            else
            {
                tma_load_2d(st, &mA0, kc, i0, full + s);
                tma_load_2d(st + NOP * A_BYTES, &mB0, kc, j0, full + s);
                if (NPROD == 3)
                {
                    tma_load_2d(st + A_BYTES, &mA1, kc, i0, full + s);
                    tma_load_2d(st + NOP * A_BYTES + B_BYTES, &mB1, kc, j0, full + s);
                }
            }
        }
    }
    else if (warp == 1 && lane == 0)
    {
        // bit 15: A is MN-major
        constexpr uint32_t idesc = instr_desc<KIND>(BM, BN) | (AMN ? (1u << 15) : 0u);
        int it = 0;
        for (; it < nkb && ok; it++)
        {
            const int s = it % STAGES;
            const uint32_t ph = (uint32_t)((it / STAGES) & 1);
            ok = mbar_wait(full + s, ph);
            if (!ok) break;
            fence_after_sync();
            const uint32_t a0 = smem_u32(smem + s * STAGE);
            const uint32_t b0 = a0 + NOP * A_BYTES;
#pragma unroll
            for (int kk = 0; kk < NK; kk++)
            {
                // MN-major A: 16 K rows of 128 bytes per MMA, the two 64-point
                // blocks BK rows apart
                const uint64_t ad = AMN ? desc_mn128(a0 + kk * 16 * 128, BK * 128)
                                        : desc_sw<SW>(a0 + kk * KSTEP);
                const uint64_t bd = desc_sw<SW>(b0 + kk * KSTEP);
                mma<KIND>(tmem, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
                if (NPROD == 3)
                {
                    const uint64_t bl = desc_sw<SW>(b0 + B_BYTES + kk * KSTEP);
                    const uint64_t al = AMN ? desc_mn128(a0 + A_BYTES + kk * 16 * 128, BK * 128)
                                            : desc_sw<SW>(a0 + A_BYTES + kk * KSTEP);
                    mma<KIND>(tmem, ad, bl, idesc, 1u);
                    mma<KIND>(tmem, al, bd, idesc, 1u);
                }
            }
            mma_commit(empty + s);
        }
        // the accumulator is final once every MMA issued above completes
        mma_commit(accf);
        if (!ok && p.err) atomicExch(p.err, MGX_TIMEOUT);
    }
    else if (warp >= 2)
    {
        const bool got = mbar_wait(accf, 0);
        fence_after_sync();
        const int q   = warp & 3; // TMEM lane quarter this warp may access
        const int row = q * 32 + lane;
        const int i   = i0 + row;
        double racc   = 0.; // density epilogue: this row's share
        if (got && nkb > 0)
        {
#pragma unroll 1
            for (int c0 = 0; c0 < BN; c0 += 32)
            {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
                if (STORE)
                {
                    if (KIND == 2)
                    {
                        const float ds = (float)(p.sa->down * p.sb->down);
#pragma unroll
                        for (int t = 0; t < 32; t++)
                            v[t] *= ds;
                    }
                    if (p.rho != nullptr)
                    {
                        // each load instruction of the warp reads 32
                        // consecutive points of one function
                        if (i < p.nrows)
                        {
#pragma unroll
                            for (int t = 0; t < 32; t++)
                            {
                                const int j = j0 + c0 + t;
                                if (j < p.ncols)
                                    racc += (double)(v[t] * p.rpsi[(size_t)j * p.ldr + i]);
                            }
                        }
                    }
                    else if (i < p.nrows)
                    {
                        // each store instruction of the warp covers 32
                        // consecutive points of one function: 128 bytes
#pragma unroll
                        for (int t = 0; t < 32; t++)
                        {
                            const int j = j0 + c0 + t;
                            if (j < p.ncols)
                            {
                                const size_t o = (size_t)j * p.ldo + i;
                                p.out[o] = (p.beta != 0.f) ? v[t] + p.beta * p.cin[o] : v[t];
                            }
                        }
                    }
                }
                else if (i < p.n)
                {
#pragma unroll
                    for (int t = 0; t < 32; t++)
                    {
                        const int j = j0 + c0 + t;
                        if (j < p.ncols && (!p.symmetric || i >= j + p.col0))
                            atomicAdd(p.C + (size_t)j * p.n + i, (double)v[t]);
                    }
                }
            }
        }
        else if (!got && p.err && lane == 0)
            atomicExch(p.err, MGX_TIMEOUT);
        if (STORE && p.rho != nullptr && got && nkb > 0 && i < p.nrows)
            atomicAdd(p.rho + i, racc);
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
            "r"(TMEM_COLS)
                     : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

/* The persistent form of gram_kernel: one CTA per SM walks the work items
 * w = blockIdx.x, blockIdx.x + gridDim.x, ... (split-K: tile w % ntiles of
 * the list, K slice w / ntiles; store: output tile w), with two TMEM
 * accumulators of BN columns.  The MMA warp fills accumulator t & 1 for the
 * CTA's t-th item while the epilogue warps drain the other one, so the
 * epilogue (FP64 atomics, FP32 stores or the density reduction) overlaps
 * the next item's MMAs instead of idling the tensor pipe; the TMA ring runs
 * on across items.  accf[b]: MMAs of accumulator b done (tcgen05.commit);
 * acce[b]: the four epilogue warps have read it.  Every wait is bounded; a
 * timeout records MGX_TIMEOUT and stops the other roles at their next
 * item. */
template <int KIND, int NPROD, int BN, int STAGES, bool STORE = false, int SW = 128,
    bool AMN = false>
__global__ void __launch_bounds__(THREADS, 1) gram_kernel_ps(
    const __grid_constant__ CUtensorMap mA0, const __grid_constant__ CUtensorMap mA1,
    const __grid_constant__ CUtensorMap mB0, const __grid_constant__ CUtensorMap mB1,
    Params p, int nitems, int ntiles)
{
    constexpr int NOP     = (NPROD == 3) ? 2 : 1;
    constexpr int A_BYTES = BM * SW;
    constexpr int B_BYTES = BN * SW;
    constexpr int STAGE   = NOP * (A_BYTES + B_BYTES);
    constexpr int KSTEP   = 32;
    constexpr int NK      = SW / KSTEP;
    constexpr int ELEM    = (KIND == 0) ? 4 : 2;
    constexpr int BK      = SW / ELEM;
    constexpr uint32_t TMEM_COLS = 2 * BN; // two accumulators
    static_assert(2 * BN <= 512, "two accumulators must fit in TMEM");

    extern __shared__ unsigned char smem_raw[];
    unsigned char* smem = reinterpret_cast<unsigned char*>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full  = reinterpret_cast<uint64_t*>(smem + STAGES * STAGE);
    uint64_t* empty = full + STAGES;
    uint64_t* accf  = empty + STAGES; // [2]
    uint64_t* acce  = accf + 2;       // [2]
    uint32_t* tslot = reinterpret_cast<uint32_t*>(acce + 2);
    __shared__ volatile int abort_all;

    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;

    // the item's output tile and K-block range
    auto decode = [&](int w, int& i0, int& j0, int& kb0, int& nkb) {
        if (STORE)
        {
            i0  = (w / p.ntj) * BM;
            j0  = (w % p.ntj) * BN;
            kb0 = 0;
            nkb = p.kblocks;
        }
        else
        {
            const int2 tile = p.tiles[w % ntiles];
            i0              = tile.x * BM;
            j0              = tile.y * BN;
            kb0             = (w / ntiles) * p.kb_per_cta;
            nkb             = min(p.kblocks, kb0 + p.kb_per_cta) - kb0;
        }
    };

    if (threadIdx.x == 0)
    {
        for (int s = 0; s < STAGES; s++)
        {
            mbar_init(full + s, 1);
            mbar_init(empty + s, 1);
        }
        for (int b = 0; b < 2; b++)
        {
            mbar_init(accf + b, 1);
            mbar_init(acce + b, 4);
        }
        abort_all = 0;
        fence_mbar_init();
    }
    if (warp == 1)
    {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tslot)),
            "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    const uint32_t tmem = *tslot;

    if (warp == 0 && lane == 0)
    {
        prefetch_map(&mA0);
        prefetch_map(&mB0);
        if (NPROD == 3)
        {
            prefetch_map(&mA1);
            prefetch_map(&mB1);
        }
        int g = 0; // stages issued so far, over all items
        for (int w = blockIdx.x; w < nitems && !abort_all; w += gridDim.x)
        {
            int i0, j0, kb0, nkb;
            decode(w, i0, j0, kb0, nkb);
            for (int it = 0; it < nkb; it++, g++)
            {
                const int s       = g % STAGES;
                const uint32_t ph = (uint32_t)((g / STAGES) & 1);
                if (!mbar_wait(empty + s, ph ^ 1u))
                {
                    abort_all = 1;
                    break;
                }
                unsigned char* st = smem + s * STAGE;
                mbar_arrive_expect_tx(full + s, STAGE);
                const int kc = (kb0 + it) * BK;
                if (AMN)
                {
                    tma_load_3d(st, &mA0, 0, kc, i0 / 64, full + s);
                    if (NPROD == 3) tma_load_3d(st + A_BYTES, &mA1, 0, kc, i0 / 64, full + s);
                    const int e0 = kc % 64, kb = kc / 64;
                    tma_load_3d(st + NOP * A_BYTES, &mB0, e0, j0, kb, full + s);
                    if (NPROD == 3)
                        tma_load_3d(st + NOP * A_BYTES + B_BYTES, &mB1, e0, j0, kb, full + s);
                }
                else if (p.blocked)
                {
                    const int e0 = kc % 64, kb = kc / 64;
                    tma_load_3d(st, &mA0, e0, i0, kb, full + s);
                    tma_load_3d(st + NOP * A_BYTES, &mB0, e0, j0, kb, full + s);
                    if (NPROD == 3)
                    {
                        tma_load_3d(st + A_BYTES, &mA1, e0, i0, kb, full + s);
                        tma_load_3d(st + NOP * A_BYTES + B_BYTES, &mB1, e0, j0, kb, full + s);
                    }
                }
                else
                {
                    tma_load_2d(st, &mA0, kc, i0, full + s);
                    tma_load_2d(st + NOP * A_BYTES, &mB0, kc, j0, full + s);
                    if (NPROD == 3)
                    {
                        tma_load_2d(st + A_BYTES, &mA1, kc, i0, full + s);
                        tma_load_2d(st + NOP * A_BYTES + B_BYTES, &mB1, kc, j0, full + s);
                    }
                }
            }
        }
    }
    else if (warp == 1 && lane == 0)
    {
        constexpr uint32_t idesc = instr_desc<KIND>(BM, BN) | (AMN ? (1u << 15) : 0u);
        int g = 0, t = 0;
        for (int w = blockIdx.x; w < nitems && !abort_all; w += gridDim.x, t++)
        {
            int i0, j0, kb0, nkb;
            decode(w, i0, j0, kb0, nkb);
            const int b       = t & 1;
            const uint32_t tb = tmem + (uint32_t)(b * BN);
            // the epilogue has drained this accumulator's previous item
            if (!mbar_wait(acce + b, (uint32_t)(((t >> 1) & 1) ^ 1)))
            {
                abort_all = 1;
                break;
            }
            fence_after_sync();
            bool ok = true;
            for (int it = 0; it < nkb; it++, g++)
            {
                const int s       = g % STAGES;
                const uint32_t ph = (uint32_t)((g / STAGES) & 1);
                if (!mbar_wait(full + s, ph))
                {
                    ok = false;
                    break;
                }
                fence_after_sync();
                const uint32_t a0 = smem_u32(smem + s * STAGE);
                const uint32_t b0 = a0 + NOP * A_BYTES;
#pragma unroll
                for (int kk = 0; kk < NK; kk++)
                {
                    const uint64_t ad = AMN ? desc_mn128(a0 + kk * 16 * 128, BK * 128)
                                            : desc_sw<SW>(a0 + kk * KSTEP);
                    const uint64_t bd = desc_sw<SW>(b0 + kk * KSTEP);
                    mma<KIND>(tb, ad, bd, idesc, (it > 0 || kk > 0) ? 1u : 0u);
                    if (NPROD == 3)
                    {
                        const uint64_t bl = desc_sw<SW>(b0 + B_BYTES + kk * KSTEP);
                        const uint64_t al = AMN ? desc_mn128(a0 + A_BYTES + kk * 16 * 128, BK * 128)
                                                : desc_sw<SW>(a0 + A_BYTES + kk * KSTEP);
                        mma<KIND>(tb, ad, bl, idesc, 1u);
                        mma<KIND>(tb, al, bd, idesc, 1u);
                    }
                }
                mma_commit(empty + s);
            }
            mma_commit(accf + b);
            if (!ok)
            {
                abort_all = 1;
                break;
            }
        }
    }
    else if (warp >= 2)
    {
        const int q   = warp & 3; // TMEM lane quarter this warp may access
        const int row = q * 32 + lane;
        int t         = 0;
        for (int w = blockIdx.x; w < nitems; w += gridDim.x, t++)
        {
            int i0, j0, kb0, nkb;
            decode(w, i0, j0, kb0, nkb);
            const int b = t & 1;
            const bool got = !abort_all && mbar_wait(accf + b, (uint32_t)((t >> 1) & 1));
            if (!got)
            {
                abort_all = 1;
                break;
            }
            fence_after_sync();
            const int i   = i0 + row;
            double racc   = 0.;
            if (nkb > 0)
            {
#pragma unroll 1
                for (int c0 = 0; c0 < BN; c0 += 32)
                {
                    float v[32];
                    tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(b * BN + c0), v);
                    if (STORE)
                    {
                        if (KIND == 2)
                        {
                            const float ds = (float)(p.sa->down * p.sb->down);
#pragma unroll
                            for (int u = 0; u < 32; u++)
                                v[u] *= ds;
                        }
                        if (p.rho != nullptr)
                        {
                            if (i < p.nrows)
                            {
#pragma unroll
                                for (int u = 0; u < 32; u++)
                                {
                                    const int j = j0 + c0 + u;
                                    if (j < p.ncols)
                                        racc += (double)(v[u] * p.rpsi[(size_t)j * p.ldr + i]);
                                }
                            }
                        }
                        else if (i < p.nrows)
                        {
#pragma unroll
                            for (int u = 0; u < 32; u++)
                            {
                                const int j = j0 + c0 + u;
                                if (j < p.ncols)
                                {
                                    const size_t o = (size_t)j * p.ldo + i;
                                    p.out[o] = (p.beta != 0.f) ? v[u] + p.beta * p.cin[o] : v[u];
                                }
                            }
                        }
                    }
                    else if (i < p.n)
                    {
#pragma unroll
                        for (int u = 0; u < 32; u++)
                        {
                            const int j = j0 + c0 + u;
                            if (j < p.ncols && (!p.symmetric || i >= j + p.col0))
                                atomicAdd(p.C + (size_t)j * p.n + i, (double)v[u]);
                        }
                    }
                }
            }
            if (STORE && p.rho != nullptr && nkb > 0 && i < p.nrows) atomicAdd(p.rho + i, racc);
            // every tcgen05.ld of this warp has completed (wait::ld): hand
            // the accumulator back to the MMA warp
            fence_before_sync();
            __syncwarp();
            if (lane == 0) mbar_arrive(acce + b);
        }
    }
    if (abort_all && threadIdx.x == 0 && p.err) atomicExch(p.err, MGX_TIMEOUT);
    fence_before_sync();
    __syncthreads();
    fence_after_sync();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
            "r"(TMEM_COLS)
                     : "memory");
}

// fp32 -> bf16 hi + lo planes (x = hi + lo + O(2^-17 |x|)); rows of K
// values with leading dimension ld (source) and ldo (planes)
__global__ void split_kernel(const float* __restrict__ x, size_t ld, int rows,
    size_t K, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo,
    size_t ldo)
{
    const size_t per_row = (ldo + 1) / 2; // pairs per output row
    const size_t total   = per_row * rows;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t r = t / per_row, k = 2 * (t - r * per_row);
        float a = 0.f, b = 0.f;
        if (k < K) a = x[r * ld + k];
        if (k + 1 < K) b = x[r * ld + k + 1];
        const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
        const __nv_bfloat16 la = __float2bfloat16_rn(a - __bfloat162float(ha));
        const __nv_bfloat16 lb = __float2bfloat16_rn(b - __bfloat162float(hb));
        __nv_bfloat162 h2, l2;
        h2.x = ha;
        h2.y = hb;
        l2.x = la;
        l2.y = lb;
        if (k + 1 < ldo)
        {
            *reinterpret_cast<__nv_bfloat162*>(hi + r * ldo + k) = h2;
            *reinterpret_cast<__nv_bfloat162*>(lo + r * ldo + k) = l2;
        }
    }
}

// max |x| over rows x K (leading dimension ld) into slot->maxbits: one
// block per row, threads along K
__global__ void __launch_bounds__(256) maxabs_kernel(const float* __restrict__ x, size_t ld,
    int rows, size_t K, ScaleSlot* slot)
{
    __shared__ float red[256];
    float m = 0.f;
    for (int r = blockIdx.x; r < rows; r += gridDim.x)
        for (size_t k = threadIdx.x; k < K; k += blockDim.x)
            m = fmaxf(m, fabsf(x[(size_t)r * ld + k]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicMax(&slot->maxbits, __float_as_uint(red[0]));
}

// max |theta(i, j)| over n rows and ncols columns (column j at th + j * ldt)
__global__ void __launch_bounds__(256) maxabs_f64_kernel(const double* __restrict__ th, int n,
    int ldt, int ncols, ScaleSlot* slot)
{
    __shared__ float red[256];
    float m = 0.f;
    for (int j = blockIdx.x; j < ncols; j += gridDim.x)
        for (int i = threadIdx.x; i < n; i += blockDim.x)
            m = fmaxf(m, (float)fabs(th[(size_t)j * ldt + i]));
    red[threadIdx.x] = m;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1)
    {
        if (threadIdx.x < o) red[threadIdx.x] = fmaxf(red[threadIdx.x], red[threadIdx.x + o]);
        __syncthreads();
    }
    // a float that rounded below the double maximum still leaves a margin
    // of 2x under the 2^15 bound of the scaled values
    if (threadIdx.x == 0) atomicMax(&slot->maxbits, __float_as_uint(red[0]));
}

__global__ void set_scale_kernel(ScaleSlot* slot)
{
    const float m = __uint_as_float(slot->maxbits);
    int e         = 0;
    if (m > 0.f && isfinite(m)) frexpf(m, &e); // m = f 2^e, 0.5 <= f < 1
    int sc = 14 - e;
    sc     = max(-100, min(100, sc));
    slot->up   = ldexpf(1.f, sc);
    slot->down = ldexp(1., -sc);
}

// hi / lo split of one value in the plane element type: bf16 (no scale) or
// fp16 (after the power-of-two scale)
template <typename E> struct Split;
template <> struct Split<__nv_bfloat16>
{
    __device__ static void go(float x, float, __nv_bfloat16& h, __nv_bfloat16& l)
    {
        h = __float2bfloat16_rn(x);
        l = __float2bfloat16_rn(x - __bfloat162float(h));
    }
};
template <> struct Split<__half>
{
    __device__ static void go(float x, float up, __half& h, __half& l)
    {
        const float a = x * up;
        h             = __float2half_rn(a);
        l             = __float2half_rn(a - __half2float(h));
    }
};

// fp32 -> hi + lo planes (bf16, or scaled fp16) in the K-blocked layout:
// element (r, k) at ((k / 64) * rows + r) * 64 + k % 64, so that the
// 64-element K slice of every row of a block is one contiguous run (a TMA
// box of 128 rows is 16 KB of consecutive memory instead of 128 rows a full
// row stride apart); K is padded with zeros to kblocks * 64.  8 consecutive
// K elements per thread: two 16-byte loads (when vec4) and one 16-byte
// store per plane; the 8 threads of a row's K block cover its 256 input and
// 128 output bytes.
template <typename E>
__global__ void __launch_bounds__(256) split8_kernel(const float* __restrict__ x, size_t ld,
    int rows, size_t K, size_t kblocks, E* __restrict__ hi, E* __restrict__ lo,
    const ScaleSlot* __restrict__ sc, int vec4)
{
    const float up     = sc ? sc->up : 1.f;
    const size_t total = (size_t)rows * kblocks * 8;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t g  = t % 8;
        const size_t rk = t / 8;                 // row-major over (row, K block)
        const size_t kb = rk % kblocks, r = rk / kblocks;
        const size_t k  = kb * 64 + g * 8;
        const float* src = x + r * ld + k;
        float v[8];
        if (vec4 && k + 8 <= K)
        {
            const float4 a = *reinterpret_cast<const float4*>(src);
            const float4 b = *reinterpret_cast<const float4*>(src + 4);
            v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w;
            v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
        }
        else
        {
#pragma unroll
            for (int q = 0; q < 8; q++)
                v[q] = (k + q < K) ? src[q] : 0.f;
        }
        __align__(16) E h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; q++)
            Split<E>::go(v[q], up, h[q], l[q]);
        const size_t o = (kb * rows + r) * 64 + g * 8;
        *reinterpret_cast<uint4*>(hi + o) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(lo + o) = *reinterpret_cast<const uint4*>(l);
    }
}



// Points-major operand of the points x functions product: columns
// [p0, p0 + P) of the orbital block x (n functions, leading dimension ld)
// become rows of K = function values, row p at p * ldo.  BF16 writes the
// hi / lo planes, otherwise one FP32 plane (TF32).  64 x 64 tiles pass
// through shared memory so that reads run along points and writes along
// functions; columns n .. ldo-1 are written as zeros.
template <bool BF16>
__global__ void __launch_bounds__(256) transpose_split_kernel(const float* __restrict__ x,
    size_t ld, int n, size_t p0, int P, void* __restrict__ hi, void* __restrict__ lo,
    size_t ldo)
{
    __shared__ float t[64][65];
    const int ib    = blockIdx.y * 64;
    const size_t pb = (size_t)blockIdx.x * 64;
    const int c     = threadIdx.x % 64;
    for (int r = threadIdx.x / 64; r < 64; r += 4)
    {
        const int i       = ib + r;
        const size_t pp   = pb + c;
        t[r][c] = (i < n && pp < (size_t)P) ? x[(size_t)i * ld + p0 + pp] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < 64 * 32; e += 256)
    {
        const int r = e / 32, q = e % 32;
        const size_t pp = pb + r;
        const int i     = ib + 2 * q;
        if (pp >= (size_t)P || (size_t)i >= ldo) continue;
        const float a = t[2 * q][r], b = t[2 * q + 1][r];
        const size_t o = pp * ldo + i;
        if (BF16)
        {
            const __nv_bfloat16 ha = __float2bfloat16_rn(a), hb = __float2bfloat16_rn(b);
            __nv_bfloat162 h2, l2;
            h2.x = ha;
            h2.y = hb;
            l2.x = __float2bfloat16_rn(a - __bfloat162float(ha));
            l2.y = __float2bfloat16_rn(b - __bfloat162float(hb));
            *reinterpret_cast<__nv_bfloat162*>((__nv_bfloat16*)hi + o) = h2;
            *reinterpret_cast<__nv_bfloat162*>((__nv_bfloat16*)lo + o) = l2;
        }
        else
            *reinterpret_cast<float2*>((float*)hi + o) = make_float2(a, b);
    }
}

// Points-major BF16 hi / lo planes of columns [p0, p0 + P) of the orbital
// block in the K-blocked layout: element (point p, function i) at
// ((i / 64) * P + p) * 64 + i % 64.  A block converts 64 functions x 128
// points through shared memory: reads run along points (512 bytes per row;
// the tile's row stride of 129 floats keeps both shared-memory phases free
// of bank conflicts), and the block's output is two contiguous 16 KB runs.
constexpr int TB_P = 128;

template <typename E>
__global__ void __launch_bounds__(256) transpose_split_blocked_kernel(const float* __restrict__ x,
    size_t ld, int n, size_t p0, int P, E* __restrict__ hi, E* __restrict__ lo,
    const ScaleSlot* __restrict__ sc)
{
    const float up = sc ? sc->up : 1.f;
    __shared__ float t[64][TB_P + 1];
    const int kb    = blockIdx.y;
    const int ib    = kb * 64;
    const size_t pb = (size_t)blockIdx.x * TB_P;
    for (int e = threadIdx.x; e < 64 * TB_P; e += blockDim.x)
    {
        const int r = e / TB_P, c = e % TB_P;
        t[r][c] = (ib + r < n && pb + c < (size_t)P) ? x[(size_t)(ib + r) * ld + p0 + pb + c] : 0.f;
    }
    __syncthreads();
    // 8 consecutive functions of one point per item: one 16-byte store per plane
    for (int e = threadIdx.x; e < TB_P * 8; e += blockDim.x)
    {
        const int c = e / 8, g = 8 * (e % 8);
        const size_t pp = pb + c;
        if (pp >= (size_t)P) continue;
        __align__(16) E h[8], l[8];
#pragma unroll
        for (int q = 0; q < 8; q++)
            Split<E>::go(t[g + q][c], up, h[q], l[q]);
        const size_t o = ((size_t)kb * P + pp) * 64 + g;
        *reinterpret_cast<uint4*>(hi + o) = *reinterpret_cast<const uint4*>(h);
        *reinterpret_cast<uint4*>(lo + o) = *reinterpret_cast<const uint4*>(l);
    }
}

// theta columns as K-blocked hi / lo planes (bf16, or fp16 after the
// scale): element (row j, K = i) at ((i / 64) * ncols + j) * 64 + i % 64,
// zero padded to kblocks * 64; lo is formed from the FP64 value.
__device__ __forceinline__ void split64(double v, float, __nv_bfloat16& h, __nv_bfloat16& l)
{
    h = __float2bfloat16_rn((float)v);
    l = __float2bfloat16_rn((float)(v - (double)__bfloat162float(h)));
}
__device__ __forceinline__ void split64(double v, float up, __half& h, __half& l)
{
    const double a = v * (double)up;
    h              = __float2half_rn((float)a);
    l              = __float2half_rn((float)(a - (double)__half2float(h)));
}

template <typename E>
__global__ void matrix_split_blocked_kernel(const double* __restrict__ th, int n, int ldt,
    int ncols, int kblocks, E* __restrict__ hi, E* __restrict__ lo,
    const ScaleSlot* __restrict__ sc)
{
    const float up     = sc ? sc->up : 1.f;
    const size_t total = (size_t)ncols * kblocks * 64;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t kb = t / ((size_t)ncols * 64);
        const size_t rem = t - kb * (size_t)ncols * 64;
        const size_t j = rem / 64, i = kb * 64 + rem % 64;
        const double v = (i < (size_t)n) ? th[j * ldt + i] : 0.;
        split64(v, up, hi[t], lo[t]);
    }
}

// FP64 matrix theta (n rows, ncols columns, column j at th + j * ldt) ->
// function-major operand rows j = column j of theta, K = i, leading
// dimension ldo: bf16 hi / lo planes (hi = bf16(x), lo = bf16(x - hi)) or
// one FP32 plane; zero padded.
template <bool BF16>
__global__ void matrix_split_kernel(const double* __restrict__ th, int n, int ldt,
    int ncols, void* hi, void* lo, size_t ldo)
{
    const size_t total = (size_t)ncols * ldo;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const size_t j = t / ldo, i = t - j * ldo;
        const double x = (i < (size_t)n) ? th[j * ldt + i] : 0.;
        if (BF16)
        {
            const __nv_bfloat16 h = __float2bfloat16_rn((float)x);
            ((__nv_bfloat16*)hi)[t] = h;
            ((__nv_bfloat16*)lo)[t] = __float2bfloat16_rn((float)(x - (double)__bfloat162float(h)));
        }
        else
            ((float*)hi)[t] = (float)x;
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 encoder()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn)
    {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000,
                cudaEnableDefault, &q)
                == cudaSuccess
            && q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D map over a row-major (rows x K) array with leading dimension ld
// (elements); box = sw-byte K slice x box_rows rows, SWIZZLE_128B (sw 128)
// or SWIZZLE_64B (sw 64).
static int make_map(CUtensorMap* m, const void* base, bool bf16, size_t K,
    size_t rows, size_t ld, int box_rows, int sw = 128)
{
    auto enc = encoder();
    if (!enc) return fail(MGX_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
    const int esz = bf16 ? 2 : 4;
    if (((uintptr_t)base % 16) || ((ld * esz) % 16))
        return fail(MGX_BAD_ARG, "tensor-core operands need 16-byte aligned rows");
    cuuint64_t dims[2]    = { (cuuint64_t)K, (cuuint64_t)rows };
    cuuint64_t strides[1] = { (cuuint64_t)(ld * esz) };
    cuuint32_t box[2]     = { (cuuint32_t)(sw / esz), (cuuint32_t)box_rows };
    cuuint32_t estr[2]    = { 1, 1 };
    CUresult r = enc(m, bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32,
        2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        sw == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MGX_CUDA_ERROR, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MGX_OK;
}

// 3-D map over a K-blocked bf16 operand (rows x kblocks * 64): dims
// (64, rows, kblocks), box (sw / 2, box_rows, 1), SWIZZLE_128B / _64B.
static int make_map_blocked(CUtensorMap* m, const void* base, size_t rows, size_t kblocks,
    int box_rows, int sw = 128, bool half = false)
{
    auto enc = encoder();
    if (!enc) return fail(MGX_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
    if ((uintptr_t)base % 16) return fail(MGX_BAD_ARG, "tensor-core operands need 16-byte alignment");
    cuuint64_t dims[3]    = { 64, (cuuint64_t)rows, (cuuint64_t)kblocks };
    cuuint64_t strides[2] = { 128, (cuuint64_t)(rows * 128) };
    cuuint32_t box[3]     = { (cuuint32_t)(sw / 2), (cuuint32_t)box_rows, 1 };
    cuuint32_t estr[3]    = { 1, 1, 1 };
    CUresult r = enc(m, half ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16,
        3, const_cast<void*>(base), dims,
        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
        sw == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MGX_CUDA_ERROR, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return MGX_OK;
}

/* Map of K-blocked bf16 planes (element (r, k) at ((k / 64) * rows + r) *
 * 64 + k % 64) read MN-major: boxes of 64 K elements (the MN side of the
 * consumer, 128 bytes, SWIZZLE_128B) x box_r rows (the consumer's K) x 2
 * consecutive 64-element blocks. */
static int make_map_mn(CUtensorMap* m, const void* base, size_t rows, size_t kblocks, int box_r)
{
    auto enc = encoder();
    if (!enc) return fail(MGX_CUDA_ERROR, "cuTensorMapEncodeTiled unavailable");
    cuuint64_t dims[3]    = { 64, (cuuint64_t)rows, (cuuint64_t)kblocks };
    cuuint64_t strides[2] = { 128, (cuuint64_t)(rows * 128) };
    cuuint32_t box[3]     = { 64, (cuuint32_t)box_r, 2 };
    cuuint32_t estr[3]    = { 1, 1, 1 };
    CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims,
        strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
        CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(MGX_CUDA_ERROR, "MN-major tensor map (%d)", (int)r);
    return MGX_OK;
}

} // namespace tc

/* ---------------- kernel timing (CUDA events around launches) -------- */
struct TimedLaunch
{
    int cls;
    cudaEvent_t a, b;
};
static std::mutex g_timing_mu;
static std::vector<TimedLaunch> g_timed;
static std::atomic<int> g_timing_on{ 0 };

/* records an event pair around the launch issued by fn() when timing is on */
template <typename F>
static int timed_launch(int cls, cudaStream_t s, F fn)
{
    if (!g_timing_on.load()) return fn();
    TimedLaunch t{ cls, nullptr, nullptr };
    if (cudaEventCreate(&t.a) != cudaSuccess || cudaEventCreate(&t.b) != cudaSuccess)
        return fn();
    cudaEventRecord(t.a, s);
    const int st = fn();
    cudaEventRecord(t.b, s);
    std::lock_guard<std::mutex> lk(g_timing_mu);
    g_timed.push_back(t);
    return st;
}

namespace tc
{
/* sms > 0: the persistent kernel on min(items, sms) CTAs (items = ntiles x
 * ksplit); else one CTA per item */
template <int KIND, int NPROD, int BN, int STAGES, bool STORE = false, int SW = 128,
    bool AMN = false>
static int launch(const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0,
    const CUtensorMap& b1, const Params& p, int ntiles, int ksplit, cudaStream_t s,
    int sms = 0)
{
    return timed_launch(STORE ? MGX_TIMING_TC_STORE : MGX_TIMING_TC_SPLITK, s, [&]() -> int {
    constexpr int NOP   = (NPROD == 3) ? 2 : 1;
    constexpr int STAGE = NOP * (BM * SW + BN * SW);
    if (sms > 0)
    {
        const size_t smem = (size_t)STAGES * STAGE + (2 * STAGES + 4) * 8 + 16 + 1024;
        auto kern         = gram_kernel_ps<KIND, NPROD, BN, STAGES, STORE, SW, AMN>;
        MGX_TRY(cuda_check(cudaFuncSetAttribute(kern,
                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
            "gram_kernel_ps smem attribute"));
        const long items = (long)ntiles * ksplit;
        if (items > (1L << 30)) return fail(MGX_UNSUPPORTED, "too many work items");
        const int grid = (int)std::min<long>(items, sms);
        kern<<<grid, THREADS, smem, s>>>(a0, a1, b0, b1, p, (int)items, ntiles);
        MGX_LAUNCH_CHECK("tc gram_kernel_ps");
        return MGX_OK;
    }
    const size_t smem   = (size_t)STAGES * STAGE + (2 * STAGES + 1) * 8 + 16 + 1024;
    auto kern           = gram_kernel<KIND, NPROD, BN, STAGES, STORE, SW, AMN>;
    MGX_TRY(cuda_check(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem),
        "gram_kernel smem attribute"));
    dim3 grid(ntiles, ksplit);
    kern<<<grid, THREADS, smem, s>>>(a0, a1, b0, b1, p);
    MGX_LAUNCH_CHECK("tc gram_kernel");
    return MGX_OK;
    });
}

__global__ void finish_kernel(double* C, int n, double vel, int symmetric,
    const ScaleSlot* sa, const ScaleSlot* sb)
{
    const size_t nn = (size_t)n * n;
    // the fp16 split's scales are powers of two: removing them is exact
    const double un = (sa && sb) ? sa->down * sb->down : 1.;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nn;
         t += (size_t)gridDim.x * blockDim.x)
    {
        const int i = (int)(t % n), j = (int)(t / n);
        if (symmetric && i < j) continue;
        double x = (C[t] * un) * vel;
        if (!(fabs(x) > 1.e-14)) x = 0.;
        C[t] = x;
        if (symmetric && i != j) C[(size_t)i * n + j] = x;
    }
}
} // namespace tc

namespace
{
struct Operand
{
    CUtensorMap m0, m1;
    const void* base0 = nullptr;
    const void* base1 = nullptr;
    bool bf16         = false;
    size_t K = 0, ld = 0;
    int rows = 0;
    int sw   = 128;
    bool blocked = false; // K-blocked planes (bf16 / fp16)
    bool half    = false; // fp16 planes of the scaled operand
    const tc::ScaleSlot* scale = nullptr;
};

bool split_mode(int mode) { return mode == MGX_GEMM_BF16X3 || mode == MGX_GEMM_FP16X3; }

/* the scale slots live after the status word in ctx->tc_err */
tc::ScaleSlot* scale_slot(mgx_ctx* ctx, int i)
{
    return reinterpret_cast<tc::ScaleSlot*>((char*)ctx->tc_err.ptr + 64 + 32 * i);
}

/* power-of-two scale of the fp32 operand X (rows x K, leading dimension ld) */
int compute_scale(const void* X, size_t ld, int rows, size_t K, tc::ScaleSlot* slot,
    cudaStream_t s)
{
    tc::maxabs_kernel<<<std::min(rows, 4096), 256, 0, s>>>((const float*)X, ld, rows, K, slot);
    MGX_LAUNCH_CHECK("maxabs_kernel");
    tc::set_scale_kernel<<<1, 1, 0, s>>>(slot);
    MGX_LAUNCH_CHECK("set_scale_kernel");
    return MGX_OK;
}

/* K bytes per tile row of the BF16X3 kernels: 64 (SWIZZLE_64B, 4 stages
 * at 128 x 256 tiles; the default, 8 % faster than 128 on the Gram and the
 * Psi Theta product at 2048 orbitals on 192^3) or 128 (SWIZZLE_128B, 2
 * stages); MGX_TC_SWIZZLE (64 or 128) overrides the default for tuning. */
/* the persistent double-buffered tensor-core kernel (default);
 * MGX_TC_PERSIST=0 selects one CTA per output tile */
bool persist_on()
{
    static int v = -1;
    if (v < 0)
    {
        const char* e = getenv("MGX_TC_PERSIST");
        v             = (e && atoi(e) == 0) ? 0 : 1;
    }
    return v == 1;
}

/* the split-K products (S, H, B) use the persistent kernel only when
 * MGX_TC_PERSIST_SPLITK=1: their FP64-atomic epilogues gain less from the
 * overlap than the store epilogue of Psi Theta, and one CTA per (tile,
 * K range) measured faster at the benchmark shape */
bool persist_splitk_on()
{
    static int v = -1;
    if (v < 0)
    {
        const char* e = getenv("MGX_TC_PERSIST_SPLITK");
        v             = (e && atoi(e) == 1 && persist_on()) ? 1 : 0;
    }
    return v == 1;
}

bool tile_order_rows()
{
    static int v = -1;
    if (v < 0)
    {
        const char* e = getenv("MGX_TC_TILE_ORDER");
        v             = (e && std::string(e) == "col") ? 0 : 1;
    }
    return v == 1;
}

int bf16_swizzle()
{
    static int sw = 0;
    if (!sw)
    {
        const char* e = getenv("MGX_TC_SWIZZLE");
        sw            = (e && atoi(e) == 128) ? 128 : 64;
    }
    return sw;
}

/* Extra elements (a multiple of 64) appended to every row of the BF16
 * planes of the K-major operands; MGX_TC_LDPAD overrides the default for
 * tuning the DRAM access pattern of the row-strided TMA boxes. */
size_t plane_pad()
{
    static long pad = -1;
    if (pad < 0)
    {
        const char* e = getenv("MGX_TC_LDPAD");
        pad           = e ? std::max(0L, atol(e)) : 0;
        pad           = (pad / 64) * 64;
    }
    return (size_t)pad;
}

/* BF16 planes of the K-major operands in the K-blocked layout (default) or
 * row-major with leading dimension K (MGX_TC_BLOCKED=0, for comparison). */
bool blocked_planes()
{
    static int b = -1;
    if (b < 0)
    {
        const char* e = getenv("MGX_TC_BLOCKED");
        b             = (e && atoi(e) == 0) ? 0 : 1;
    }
    return b == 1;
}

/* re-encodes the maps of an operand with another box height */
int rebox(Operand& op, int box_rows)
{
    if (op.blocked)
    {
        const size_t kb = (op.K + 63) / 64;
        MGX_TRY(tc::make_map_blocked(&op.m0, op.base0, op.rows, kb, box_rows, op.sw, op.half));
        MGX_TRY(tc::make_map_blocked(&op.m1, op.base1, op.rows, kb, box_rows, op.sw, op.half));
        return MGX_OK;
    }
    MGX_TRY(tc::make_map(&op.m0, op.base0, op.bf16, op.K, op.rows, op.ld, box_rows, op.sw));
    if (op.base1)
        MGX_TRY(tc::make_map(&op.m1, op.base1, op.bf16, op.K, op.rows, op.ld, box_rows, op.sw));
    else
        op.m1 = op.m0;
    return MGX_OK;
}

/* Prepares the tensor maps of one operand (rows x K, leading dimension ld):
 * TF32 reads the FP32 data in place (or a 16-byte aligned copy in `ws`);
 * BF16X3 writes the hi / lo planes into `ws`.  Returns the workspace bytes
 * used in *used. */
int prepare(int mode, const void* X, size_t ld, size_t K, int rows, int box_rows,
    char* ws, size_t* used, Operand& op, cudaStream_t s, const tc::ScaleSlot* sc = nullptr)
{
    using namespace tc;
    *used = 0;
    if (mode == MGX_GEMM_FP16X3)
    {
        // K-blocked fp16 hi / lo planes of the scaled operand, SWIZZLE_64B
        op.sw      = 64;
        op.blocked = true;
        op.half    = true;
        op.scale   = sc;
        const size_t kblocks = (K + 63) / 64;
        const size_t plane   = kblocks * 64 * (size_t)rows * sizeof(__half);
        auto* hi             = (__half*)ws;
        auto* lo             = (__half*)(ws + plane);
        const int vec4 = ((ld % 4) == 0 && ((uintptr_t)X % 16) == 0) ? 1 : 0;
        const int nb8  = (int)std::min<size_t>((kblocks * 8 * rows + 255) / 256, 1 << 20);
        split8_kernel<__half><<<nb8, 256, 0, s>>>((const float*)X, ld, rows, K, kblocks, hi, lo,
            sc, vec4);
        MGX_LAUNCH_CHECK("split8_kernel");
        MGX_TRY(make_map_blocked(&op.m0, hi, rows, kblocks, box_rows, 64, true));
        MGX_TRY(make_map_blocked(&op.m1, lo, rows, kblocks, box_rows, 64, true));
        op.base0 = hi;
        op.base1 = lo;
        op.bf16  = true;
        op.K     = K;
        op.ld    = kblocks * 64;
        op.rows  = rows;
        *used    = 2 * plane;
        return MGX_OK;
    }
    if (mode == MGX_GEMM_TF32)
    {
        if (((uintptr_t)X % 16) || ((ld * 4) % 16))
        {
            const size_t ldp = ((K + 31) / 32) * 32;
            MGX_TRY(cuda_check(cudaMemcpy2DAsync(ws, ldp * 4, X, ld * 4, K * 4, rows,
                                   cudaMemcpyDeviceToDevice, s),
                "tf32 pad copy"));
            X     = ws;
            ld    = ldp;
            *used = ldp * (size_t)rows * 4;
        }
        MGX_TRY(make_map(&op.m0, X, false, K, rows, ld, box_rows));
        op.m1    = op.m0;
        op.base0 = X;
        op.base1 = nullptr;
        op.bf16  = false;
        op.K     = K;
        op.ld    = ld;
        op.rows  = rows;
        return MGX_OK;
    }
    op.sw      = bf16_swizzle();
    op.blocked = blocked_planes();
    const size_t kblocks = (K + 63) / 64;
    const size_t ldo     = op.blocked ? kblocks * 64 : kblocks * 64 + plane_pad();
    const size_t plane   = ldo * (size_t)rows * sizeof(__nv_bfloat16);
    auto* hi             = (__nv_bfloat16*)ws;
    auto* lo             = (__nv_bfloat16*)(ws + plane);
    const int nb         = (int)std::min<size_t>((ldo / 2 * rows + 255) / 256, 1 << 20);
    if (op.blocked)
    {
        const int vec4 = ((ld % 4) == 0 && ((uintptr_t)X % 16) == 0) ? 1 : 0;
        const int nb8  = (int)std::min<size_t>((kblocks * 8 * rows + 255) / 256, 1 << 20);
        split8_kernel<__nv_bfloat16><<<nb8, 256, 0, s>>>((const float*)X, ld, rows, K, kblocks,
            hi, lo, nullptr, vec4);
        MGX_LAUNCH_CHECK("split8_kernel");
        MGX_TRY(make_map_blocked(&op.m0, hi, rows, kblocks, box_rows, op.sw));
        MGX_TRY(make_map_blocked(&op.m1, lo, rows, kblocks, box_rows, op.sw));
    }
    else
    {
        split_kernel<<<nb, 256, 0, s>>>((const float*)X, ld, rows, K, hi, lo, ldo);
        MGX_LAUNCH_CHECK("split_kernel");
        MGX_TRY(make_map(&op.m0, hi, true, K, rows, ldo, box_rows, op.sw));
        MGX_TRY(make_map(&op.m1, lo, true, K, rows, ldo, box_rows, op.sw));
    }
    op.base0 = hi;
    op.base1 = lo;
    op.bf16  = true;
    op.K     = K;
    op.ld    = ldo;
    op.rows  = rows;
    *used    = 2 * plane;
    return MGX_OK;
}

size_t operand_bytes(int mode, size_t K, int rows)
{
    if (mode == MGX_GEMM_TF32) return ((K + 31) / 32) * 32 * (size_t)rows * 4;
    return 2 * (((K + 63) / 64) * 64 + plane_pad()) * (size_t)rows * sizeof(__nv_bfloat16);
}

/* C[0:nrows, 0:ncols] (leading dimension ldc) += A B^T over K.  Output
 * tiles are 128 x 256 (128 x 128 when ncols <= 128); the B operand map must
 * have been built with the matching box height. */
int run(mgx_ctx* ctx, int mode, const Operand& a, const Operand& b, int nrows, int ncols,
    int symmetric, double* C, int ldc, size_t K, int tile_slot, int BN, cudaStream_t s,
    int col0 = 0)
{
    using namespace tc;
    const int sms = persist_splitk_on() ? ctx->sm_count : 0;
    const int nti = (nrows + BM - 1) / BM, ntj = (ncols + BN - 1) / BN;
    std::vector<int2> tiles;
    // tile order within a K range: column tiles of one row tile next to each
    // other (the default), so that they read their shared A slice close
    // together in time, or row tiles of one column tile together
    // (MGX_TC_TILE_ORDER=col; 4 % more cycles for the split-K products at the
    // benchmark shape)
    if (tile_order_rows())
    {
        for (int i = 0; i < nti; i++)
            for (int j = 0; j < ntj; j++)
                if (!symmetric || (i * BM + BM - 1) >= col0 + j * BN)
                    tiles.push_back(make_int2(i, j));
    }
    else
    {
        for (int j = 0; j < ntj; j++)
            for (int i = 0; i < nti; i++)
                if (!symmetric || (i * BM + BM - 1) >= col0 + j * BN)
                    tiles.push_back(make_int2(i, j));
    }
    const int ntiles  = (int)tiles.size();
    // K elements per block; a CTA covers at most 32768 K elements (the FP32
    // accumulation bound)
    const int bk      = split_mode(mode) ? a.sw / 2 : 32;
    const int kblocks = (int)((K + bk - 1) / bk);
    const int kbcap   = 32768 / bk;
    int ksplit = std::max((4 * ctx->sm_count + ntiles - 1) / ntiles, (kblocks + kbcap - 1) / kbcap);
    ksplit     = std::min(ksplit, kblocks);
    const int kb_per = (kblocks + ksplit - 1) / ksplit;
    ksplit           = (kblocks + kb_per - 1) / kb_per;
    if (ksplit > 65535) return fail(MGX_UNSUPPORTED, "K too large");
    const size_t slot_bytes = 64 * 1024 * sizeof(int2);
    if (tiles.size() > 64 * 1024) return fail(MGX_UNSUPPORTED, "too many output tiles");
    int2* dtiles = (int2*)((char*)ctx->tc_tiles.ptr + tile_slot * slot_bytes);
    MGX_TRY(cuda_check(cudaMemcpyAsync(dtiles, tiles.data(), tiles.size() * sizeof(int2),
                           cudaMemcpyHostToDevice, s),
        "tile list upload"));
    Params p;
    p.tiles      = dtiles;
    p.kblocks    = kblocks;
    p.kb_per_cta = kb_per;
    p.n          = ldc;
    p.ncols      = ncols;
    p.symmetric  = symmetric;
    p.col0       = col0;
    p.C          = C;
    p.err        = (int*)ctx->tc_err.ptr;
    (void)nrows;
    if (split_mode(mode) && (a.sw != b.sw || a.blocked != b.blocked || a.half != b.half))
        return fail(MGX_BAD_ARG, "operands with different layouts");
    p.blocked = a.blocked ? 1 : 0;
    p.sa      = a.scale;
    p.sb      = b.scale;
    if (mode == MGX_GEMM_FP16X3)
    {
        if (BN == 256)
            return launch<2, 3, 256, 4, false, 64>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
        return launch<2, 3, 128, 6, false, 64>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
    }
    if (BN == 256)
    {
        if (mode == MGX_GEMM_TF32)
            return launch<0, 1, 256, 4>(a.m0, a.m0, b.m0, b.m0, p, ntiles, ksplit, s, sms);
        if (a.sw == 64)
            return launch<1, 3, 256, 4, false, 64>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
        return launch<1, 3, 256, 2>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
    }
    if (mode == MGX_GEMM_TF32)
        return launch<0, 1, 128, 6>(a.m0, a.m0, b.m0, b.m0, p, ntiles, ksplit, s, sms);
    if (a.sw == 64)
        return launch<1, 3, 128, 6, false, 64>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
    return launch<1, 3, 128, 3>(a.m0, a.m1, b.m0, b.m1, p, ntiles, ksplit, s, sms);
}

/* output tile width: 256 when the product is wide enough; MGX_TC_TILE_N
 * (128 or 256) overrides the choice for tuning */
int tile_n(int ncols)
{
    static int forced = -1;
    if (forced < 0)
    {
        const char* e = getenv("MGX_TC_TILE_N");
        forced        = (e && (atoi(e) == 128 || atoi(e) == 256)) ? atoi(e) : 0;
    }
    if (forced) return ncols > 128 ? forced : 128;
    return ncols > 128 ? 256 : 128;
}

/* lower triangle of A A^T: the A maps (box 128 rows) are rebuilt with the
 * 256-row box for the B side when the wide tile is used */
int run_sym(mgx_ctx* ctx, int mode, const Operand& a, int n, double* C, size_t K,
    int tile_slot, cudaStream_t s)
{
    const int BN = tile_n(n);
    if (BN == 128) return run(ctx, mode, a, a, n, n, 1, C, n, K, tile_slot, 128, s);
    Operand b = a;
    MGX_TRY(rebox(b, BN));
    return run(ctx, mode, a, b, n, n, 1, C, n, K, tile_slot, BN, s);
}

int begin(mgx_ctx* ctx, cudaStream_t s)
{
    MGX_TRY(ctx->tc_tiles.ensure(2 * 64 * 1024 * sizeof(int2)));
    // status word, then three scale slots (zeroed: their maxima start at 0)
    MGX_TRY(ctx->tc_err.ensure(256));
    return cuda_check(cudaMemsetAsync(ctx->tc_err.ptr, 0, 256, s), "err reset");
}

int end(mgx_ctx* ctx, cudaStream_t s)
{
    int herr = 0;
    MGX_TRY(cuda_check(cudaMemcpyAsync(&herr, ctx->tc_err.ptr, sizeof(int),
                           cudaMemcpyDeviceToHost, s),
        "err download"));
    MGX_TRY(cuda_check(cudaStreamSynchronize(s), "tc gram sync"));
    if (herr) return fail(MGX_TIMEOUT, "tensor-core pipeline wait gave up");
    return MGX_OK;
}

int finish(double* C, int n, double vel, int symmetric, cudaStream_t s,
    const tc::ScaleSlot* sa = nullptr, const tc::ScaleSlot* sb = nullptr)
{
    const int nbf = (int)std::min<size_t>(((size_t)n * n + 255) / 256, 4096);
    tc::finish_kernel<<<nbf, 256, 0, s>>>(C, n, vel, symmetric, sa, sb);
    MGX_LAUNCH_CHECK("finish_kernel");
    return MGX_OK;
}

// columns of the second operand converted per pass (bounds the workspace)
constexpr int CHUNK = 512;

/* room kept after the operands for the BF16 planes of an n x n theta, so
 * that a Psi Theta product can reuse the conversion of psi without growing
 * (and so losing) the workspace */
size_t theta_room(const mgx_ctx* ctx, int n)
{
    if (!ctx->reuse_conversion) return 0;
    const size_t ldk = ((size_t)(n + 63) / 64) * 64;
    return 2 * (((ldk * (size_t)n * 2) + 1023) / 1024) * 1024 + 2048;
}

/* records the A operand just prepared at the start of tc_split (BF16 K-blocked
 * planes only) as the context's reusable conversion of psi */
void record_conversion(mgx_ctx* ctx, int mode, const Operand& a, const void* psi, size_t ld,
    size_t K, int n, size_t used)
{
    auto& c = ctx->conv;
    c.valid = (mode == MGX_GEMM_BF16X3) && a.blocked && !a.half;
    c.psi   = psi;
    c.ld    = ld;
    c.K     = K;
    c.n     = n;
    c.used  = used;
    c.hi    = const_cast<void*>(a.base0);
    c.lo    = const_cast<void*>(a.base1);
}

/* C = A B^T over K with B processed CHUNK rows at a time; A prepared once */
int product(mgx_ctx* ctx, int mode, const Operand& a, size_t a_used, const void* B,
    size_t ld, size_t K, int n, double* C, int tile_slot, cudaStream_t s,
    const tc::ScaleSlot* sb = nullptr)
{
    for (int j0 = 0; j0 < n; j0 += CHUNK)
    {
        const int nc = std::min(CHUNK, n - j0);
        Operand b;
        size_t used = 0;
        const void* Bj = (const char*)B + (size_t)j0 * ld * 4;
        const int BN = tile_n(nc);
        MGX_TRY(prepare(mode, Bj, ld, K, nc, BN, (char*)ctx->tc_split.ptr + a_used, &used, b, s,
            sb));
        MGX_TRY(run(ctx, mode, a, b, n, nc, 0, C + (size_t)j0 * n, n, K, tile_slot, BN, s));
    }
    return MGX_OK;
}
/* lower triangle (rows >= columns) of A (B Psi)^T, B the Mehrstellen
 * right-hand-side operator: B Psi is formed in `work` (leading dimension
 * ld) `step` functions at a time, converted and multiplied; only the
 * output tiles that reach the lower triangle run. */
int matb_product(mgx_ctx* ctx, int mode, const Operand& a, size_t a_used, const void* psi,
    size_t ld, size_t K, int n, double* C, int tile_slot, cudaStream_t s,
    const tc::ScaleSlot* sb, void* work, int work_funcs)
{
    // BF16X3 on K-blocked planes: the stencil writes the hi / lo planes of
    // B Psi itself (no FP32 B Psi block, no split pass), CHUNK rows a time
    if (mode == MGX_GEMM_BF16X3 && blocked_planes() && (K % 64) == 0 && (ld % 4) == 0
        && ((uintptr_t)psi % 16) == 0)
    {
        const size_t kblocks = K / 64;
        // the B-side workspace holds min(n, CHUNK) rows (operand_bytes)
        const size_t plane = kblocks * 64 * (size_t)std::min(n, CHUNK) * sizeof(__nv_bfloat16);
        char* base           = (char*)ctx->tc_split.ptr + a_used;
        bool fused           = true;
        for (int j0 = 0; j0 < n && fused; j0 += CHUNK)
        {
            const int nc  = std::min(CHUNK, n - j0);
            const int BN  = tile_n(nc);
            void* hi      = base;
            void* lo      = base + plane;
            const int st  = rhs_split_block(ctx->grid, (const float*)psi + (size_t)j0 * ld, ld, nc,
                hi, lo, nc, s);
            if (st == MGX_UNSUPPORTED && j0 == 0)
            {
                fused = false; // nothing launched: take the unfused path below
                break;
            }
            MGX_TRY(st);
            Operand b;
            b.sw      = bf16_swizzle();
            b.blocked = true;
            b.half    = false;
            b.bf16    = true;
            b.base0   = hi;
            b.base1   = lo;
            b.K       = K;
            b.ld      = kblocks * 64;
            b.rows    = nc;
            MGX_TRY(tc::make_map_blocked(&b.m0, hi, nc, kblocks, BN, b.sw));
            MGX_TRY(tc::make_map_blocked(&b.m1, lo, nc, kblocks, BN, b.sw));
            MGX_TRY(run(ctx, mode, a, b, n, nc, 1, C + (size_t)j0 * n, n, K, tile_slot, BN, s, j0));
        }
        if (fused) return MGX_OK;
    }
    const int step = std::min(std::max(work_funcs, 1), CHUNK);
    for (int j0 = 0; j0 < n; j0 += step)
    {
        const int nc = std::min(step, n - j0);
        MGX_TRY(rhs_block(ctx->grid, MGX_F32, (const float*)psi + (size_t)j0 * ld, ld, work, ld,
            nc, s));
        Operand b;
        size_t used = 0;
        const int BN = tile_n(nc);
        MGX_TRY(prepare(mode, work, ld, K, nc, BN, (char*)ctx->tc_split.ptr + a_used, &used, b,
            s, sb));
        MGX_TRY(run(ctx, mode, a, b, n, nc, 1, C + (size_t)j0 * n, n, K, tile_slot, BN, s, j0));
    }
    return MGX_OK;
}

/* H = Psi^T (H Psi) with H Psi made here, CHUNK functions at a time: the
 * H psi kernel writes each chunk both to hpsi (FP32, for the residual) and,
 * as the bf16 hi / lo K-blocked planes, straight into the B-side
 * workspace, which the product then reads; H psi is never read back and
 * converted.  BF16X3 on K-blocked planes only.  *done false (nothing
 * launched) when the H psi kernel cannot write the planes. */
int hpsi_product(mgx_ctx* ctx, int mode, const Operand& a, size_t a_used, const float* psi,
    const float* V, float* hpsi, size_t ld, size_t K, int n, double* C, int tile_slot,
    cudaStream_t s, bool* done)
{
    *done = false;
    if (!(mode == MGX_GEMM_BF16X3 && blocked_planes() && (K % 64) == 0 && (ld % 4) == 0
            && ((uintptr_t)psi % 16) == 0 && ((uintptr_t)hpsi % 16) == 0))
        return MGX_OK;
    const size_t kblocks = K / 64;
    const size_t plane   = kblocks * 64 * (size_t)std::min(n, CHUNK) * sizeof(__nv_bfloat16);
    char* base           = (char*)ctx->tc_split.ptr + a_used;
    for (int j0 = 0; j0 < n; j0 += CHUNK)
    {
        const int nc = std::min(CHUNK, n - j0);
        const int BN = tile_n(nc);
        void* hi     = base;
        void* lo     = base + plane;
        const int st = hpsi_split_block(ctx->grid, psi + (size_t)j0 * ld, ld, V,
            hpsi + (size_t)j0 * ld, nc, hi, lo, nc, s);
        if (st == MGX_UNSUPPORTED && j0 == 0) return MGX_OK; // nothing launched
        MGX_TRY(st);
        Operand b;
        b.sw      = bf16_swizzle();
        b.blocked = true;
        b.half    = false;
        b.bf16    = true;
        b.base0   = hi;
        b.base1   = lo;
        b.K       = K;
        b.ld      = kblocks * 64;
        b.rows    = nc;
        MGX_TRY(tc::make_map_blocked(&b.m0, hi, nc, kblocks, BN, b.sw));
        MGX_TRY(tc::make_map_blocked(&b.m1, lo, nc, kblocks, BN, b.sw));
        MGX_TRY(run(ctx, mode, a, b, n, nc, 0, C + (size_t)j0 * n, n, K, tile_slot, BN, s));
    }
    *done = true;
    return MGX_OK;
}
} // namespace

/* B = Psi^T (B Psi) * vel, lower triangle mirrored (the |B u| <= max |u|
 * bound of the Mehrstellen operator, whose coefficients are positive and
 * sum to 1, lets the fp16 split of B Psi reuse the scale of Psi) */
int matb_tcgen05(mgx_ctx* ctx, int mode, const void* psi, size_t ld, size_t K, int n,
    double vel, double* Bm, void* work, int work_funcs, cudaStream_t s)
{
    const size_t a_bytes = operand_bytes(mode, K, n);
    const size_t b_bytes = operand_bytes(mode, K, std::min(n, CHUNK));
    MGX_TRY(ctx->tc_split.ensure(a_bytes + b_bytes + 512 + theta_room(ctx, n)));
    MGX_TRY(begin(ctx, s));
    MGX_TRY(cuda_check(cudaMemsetAsync(Bm, 0, (size_t)n * n * sizeof(double), s), "B zero"));
    tc::ScaleSlot* sa = nullptr;
    if (mode == MGX_GEMM_FP16X3)
    {
        sa = scale_slot(ctx, 0);
        MGX_TRY(compute_scale(psi, ld, n, K, sa, s));
    }
    Operand a;
    size_t used = 0;
    ctx->conv.valid = false;
    MGX_TRY(prepare(mode, psi, ld, K, n, tc::BM, (char*)ctx->tc_split.ptr, &used, a, s, sa));
    record_conversion(ctx, mode, a, psi, ld, K, n, used);
    MGX_TRY(matb_product(ctx, mode, a, ((used + 255) / 256) * 256, psi, ld, K, n, Bm, 0, s, sa,
        work, work_funcs));
    MGX_TRY(finish(Bm, n, vel, 1, s, sa, sa));
    return end(ctx, s);
}

int gram_tcgen05(mgx_ctx* ctx, int mode, const void* A, const void* B, size_t ld,
    size_t K, int n, double vel, int symmetric, double* C, cudaStream_t s)
{
    const bool same = (A == B) && symmetric;
    const size_t a_bytes = operand_bytes(mode, K, n);
    const size_t b_bytes = same ? 0 : operand_bytes(mode, K, std::min(n, CHUNK));
    MGX_TRY(ctx->tc_split.ensure(a_bytes + b_bytes + 256 + theta_room(ctx, n)));
    MGX_TRY(begin(ctx, s));
    MGX_TRY(cuda_check(cudaMemsetAsync(C, 0, (size_t)n * n * sizeof(double), s), "C zero"));
    tc::ScaleSlot* sa = nullptr;
    tc::ScaleSlot* sb = nullptr;
    if (mode == MGX_GEMM_FP16X3)
    {
        sa = scale_slot(ctx, 0);
        MGX_TRY(compute_scale(A, ld, n, K, sa, s));
        sb = sa;
        if (!same)
        {
            sb = scale_slot(ctx, 1);
            MGX_TRY(compute_scale(B, ld, n, K, sb, s));
        }
    }
    Operand a;
    size_t used = 0;
    ctx->conv.valid = false;
    MGX_TRY(prepare(mode, A, ld, K, n, tc::BM, (char*)ctx->tc_split.ptr, &used, a, s, sa));
    record_conversion(ctx, mode, a, A, ld, K, n, used);
    if (same)
        MGX_TRY(run_sym(ctx, mode, a, n, C, K, 0, s));
    else
        MGX_TRY(product(ctx, mode, a, ((used + 255) / 256) * 256, B, ld, K, n, C, 0, s, sb));
    MGX_TRY(finish(C, n, vel, same ? 1 : 0, s, sa, sb));
    return end(ctx, s);
}

/* S = Psi^T Psi * vel and H = Psi^T (H Psi) * vel with one conversion of
 * Psi; with Bm, also B = Psi^T (B Psi) * vel (lower triangle mirrored),
 * B Psi formed in `work` */
int gram_hmat_tcgen05(mgx_ctx* ctx, int mode, const void* psi, const void* hpsi,
    size_t ld, size_t K, int n, double vel, double* S, double* H, cudaStream_t s,
    double* Bm, void* work, int work_funcs, const float* V, int lap_type)
{
    const size_t a_bytes = operand_bytes(mode, K, n);
    const size_t b_bytes = operand_bytes(mode, K, std::min(n, CHUNK));
    MGX_TRY(ctx->tc_split.ensure(a_bytes + b_bytes + 512 + theta_room(ctx, n)));
    MGX_TRY(begin(ctx, s));
    MGX_TRY(cuda_check(cudaMemsetAsync(S, 0, (size_t)n * n * sizeof(double), s), "S zero"));
    MGX_TRY(cuda_check(cudaMemsetAsync(H, 0, (size_t)n * n * sizeof(double), s), "H zero"));
    tc::ScaleSlot* sa = nullptr;
    tc::ScaleSlot* sb = nullptr;
    if (mode == MGX_GEMM_FP16X3)
    {
        sa = scale_slot(ctx, 0);
        sb = scale_slot(ctx, 1);
        MGX_TRY(compute_scale(psi, ld, n, K, sa, s));
        MGX_TRY(compute_scale(hpsi, ld, n, K, sb, s));
    }
    Operand a;
    size_t used = 0;
    ctx->conv.valid = false;
    MGX_TRY(prepare(mode, psi, ld, K, n, tc::BM, (char*)ctx->tc_split.ptr, &used, a, s, sa));
    record_conversion(ctx, mode, a, psi, ld, K, n, used);
    MGX_TRY(run_sym(ctx, mode, a, n, S, K, 0, s));
    // with V, hpsi is an output: H psi made chunk by chunk into the
    // product's operand planes (or, when that cannot run, in full first)
    bool made = false;
    if (V)
    {
        MGX_TRY(hpsi_product(ctx, mode, a, ((used + 255) / 256) * 256, (const float*)psi, V,
            (float*)hpsi, ld, K, n, H, 1, s, &made));
        if (!made)
        {
            PlaneParams p;
            for (int i = 0; i < 3; i++)
                p.n[i] = ctx->grid.n[i];
            p.u   = psi;
            p.ldu = ld;
            p.V   = V;
            p.out = const_cast<void*>(hpsi);
            p.ldo = ld;
            MGX_TRY(stencil_launch(OP_HPSI_B, lap_type, MGX_F32, MGX_F32, p,
                make_level(ctx->grid, 0), 0., n, s));
        }
    }
    if (!made)
        MGX_TRY(product(ctx, mode, a, ((used + 255) / 256) * 256, hpsi, ld, K, n, H, 1, s, sb));
    MGX_TRY(finish(S, n, vel, 1, s, sa, sa));
    MGX_TRY(finish(H, n, vel, 0, s, sa, sb));
    if (Bm)
    {
        MGX_TRY(cuda_check(cudaMemsetAsync(Bm, 0, (size_t)n * n * sizeof(double), s), "B zero"));
        MGX_TRY(matb_product(ctx, mode, a, ((used + 255) / 256) * 256, psi, ld, K, n, Bm, 0, s,
            sa, work, work_funcs));
        MGX_TRY(finish(Bm, n, vel, 1, s, sa, sa));
    }
    return end(ctx, s);
}

/* out_j = sum_i psi_i theta(i, j) + beta * cin_j, j < ncols (column j of
 * theta at theta + j * ldt), over npts points (the
 * MPgemmNN product of LocGridOrbitals::multiplyByMatrix,
 * src/LocGridOrbitals.cc:793-830) on the tensor cores.  M = points,
 * N = functions, K = functions: the points are processed in chunks whose
 * transposed operand (rows = points, K = functions) fits a bounded
 * workspace; theta is converted once.  One CTA per 128 x BN output tile. */
int psi_theta_tcgen05(mgx_ctx* ctx, int mode, const float* psi, size_t ld, size_t npts,
    int n, const double* theta, int ldt, int ncols, float beta, const float* cin, float* out,
    cudaStream_t s, double* rho)
{
    using namespace tc;
    const int sms = persist_on() ? ctx->sm_count : 0;
    // Psi Theta straight from the Gram's conversion of the same block: its
    // K-blocked planes (rows = functions, K = points) are the MN-major A
    // operand here (M = points, K = functions), so psi is not converted again
    {
        const auto& cv = ctx->conv;
        const int sw   = bf16_swizzle();
        const size_t ldk0     = ((n + 63) / 64) * 64;
        const size_t bplane   = ((ldk0 * (size_t)ncols * 2 + 1023) / 1024) * 1024;
        const size_t off      = ((cv.used + 1023) / 1024) * 1024;
        if (mode == MGX_GEMM_BF16X3 && ctx->reuse_conversion && cv.valid && cv.psi == psi
            && cv.ld == ld && cv.K == npts && cv.n == n && off + 2 * bplane <= ctx->tc_split.bytes)
        {
            MGX_TRY(begin(ctx, s));
            char* ws       = (char*)ctx->tc_split.ptr + off;
            void* bhi      = ws;
            void* blo      = ws + bplane;
            const int nkbf = (int)(ldk0 / 64);
            const int nb   = (int)std::min<size_t>((ncols * ldk0 + 255) / 256, 1 << 16);
            matrix_split_blocked_kernel<__nv_bfloat16><<<nb, 256, 0, s>>>(theta, n, ldt, ncols,
                nkbf, (__nv_bfloat16*)bhi, (__nv_bfloat16*)blo, nullptr);
            MGX_LAUNCH_CHECK("matrix_split_kernel");
            const int BN = (ncols > 128) ? 256 : 128;
            const int BK = sw / 2;
            CUtensorMap mb0, mb1, ma0, ma1;
            MGX_TRY(make_map_blocked(&mb0, bhi, ncols, nkbf, BN, sw));
            MGX_TRY(make_map_blocked(&mb1, blo, ncols, nkbf, BN, sw));
            const size_t kbp = (npts + 63) / 64;
            MGX_TRY(make_map_mn(&ma0, cv.hi, (size_t)n, kbp, BK));
            MGX_TRY(make_map_mn(&ma1, cv.lo, (size_t)n, kbp, BK));
            const int ntj = (ncols + BN - 1) / BN;
            Params p;
            p.tiles      = nullptr;
            p.kblocks    = (n + BK - 1) / BK;
            p.kb_per_cta = p.kblocks;
            p.n          = 0;
            p.ncols      = ncols;
            p.symmetric  = 0;
            p.C          = nullptr;
            p.err        = (int*)ctx->tc_err.ptr;
            p.out        = out;
            p.cin        = cin;
            p.ldo        = ld;
            p.beta       = cin ? beta : 0.f;
            p.nrows      = (int)npts;
            p.ntj        = ntj;
            p.blocked    = 1;
            if (rho)
            {
                p.rho  = rho;
                p.rpsi = psi;
                p.ldr  = ld;
            }
            const int ntiles = (int)((npts + BM - 1) / BM) * ntj;
            if (sw == 64)
            {
                if (BN == 256)
                    MGX_TRY((launch<1, 3, 256, 4, true, 64, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
                else
                    MGX_TRY((launch<1, 3, 128, 6, true, 64, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            }
            else
            {
                if (BN == 256)
                    MGX_TRY((launch<1, 3, 256, 2, true, 128, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
                else
                    MGX_TRY((launch<1, 3, 128, 3, true, 128, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            }
            return end(ctx, s);
        }
    }
    // the conversion below overwrites the start of the workspace
    ctx->conv.valid = false;
    const bool half       = (mode == MGX_GEMM_FP16X3);
    const bool bf         = split_mode(mode);
    const size_t esz      = bf ? 2 : 4;
    const int nplanes     = bf ? 2 : 1;
    const size_t ldk      = bf ? ((n + 63) / 64) * 64 : ((n + 31) / 32) * 32;
    const size_t b_plane  = ldk * (size_t)ncols * esz;
    const size_t b_bytes  = ((nplanes * b_plane + 1023) / 1024) * 1024;
    const size_t row_bytes = nplanes * ldk * esz; // one point of the A operand
    // chunk of points: at most 2 GiB of A operand, a multiple of the tile;
    // MGX_PSI_THETA_CHUNK (points) overrides the size for tuning and tests
    size_t P = ((size_t)2 << 30) / row_bytes;
    if (const char* e = getenv("MGX_PSI_THETA_CHUNK"))
        if (atol(e) > 0) P = (size_t)atol(e);
    P        = std::max<size_t>(BM, (P / BM) * BM);
    P        = std::min(P, ((npts + BM - 1) / BM) * BM);
    const size_t a_plane = ldk * P * esz;
    MGX_TRY(ctx->tc_split.ensure(b_bytes + nplanes * a_plane + 1024));
    MGX_TRY(begin(ctx, s));
    char* ws = (char*)ctx->tc_split.ptr;
    void* bhi = ws;
    void* blo = ws + b_plane;
    void* ahi = ws + b_bytes;
    void* alo = ws + b_bytes + a_plane;
    const bool blk = half || (bf && blocked_planes());
    const int nkb  = (int)(ldk / 64);
    ScaleSlot* sa  = nullptr;
    ScaleSlot* sb  = nullptr;
    if (half)
    {
        sa = scale_slot(ctx, 0);
        sb = scale_slot(ctx, 2);
        MGX_TRY(compute_scale(psi, ld, n, npts, sa, s));
        maxabs_f64_kernel<<<std::min(ncols, 4096), 256, 0, s>>>(theta, n, ldt, ncols, sb);
        MGX_LAUNCH_CHECK("maxabs_f64_kernel");
        set_scale_kernel<<<1, 1, 0, s>>>(sb);
        MGX_LAUNCH_CHECK("set_scale_kernel");
    }
    {
        const int nb = (int)std::min<size_t>((ncols * ldk + 255) / 256, 1 << 16);
        if (half)
            matrix_split_blocked_kernel<__half><<<nb, 256, 0, s>>>(theta, n, ldt, ncols, nkb,
                (__half*)bhi, (__half*)blo, sb);
        else if (blk)
            matrix_split_blocked_kernel<__nv_bfloat16><<<nb, 256, 0, s>>>(theta, n, ldt, ncols, nkb,
                (__nv_bfloat16*)bhi, (__nv_bfloat16*)blo, nullptr);
        else if (bf)
            matrix_split_kernel<true><<<nb, 256, 0, s>>>(theta, n, ldt, ncols, bhi, blo, ldk);
        else
            matrix_split_kernel<false><<<nb, 256, 0, s>>>(theta, n, ldt, ncols, bhi, blo, ldk);
        MGX_LAUNCH_CHECK("matrix_split_kernel");
    }
    const int BN = (ncols > 128) ? 256 : 128;
    const int sw = half ? 64 : bf ? bf16_swizzle() : 128;
    CUtensorMap mb0, mb1, ma0, ma1;
    if (blk)
    {
        MGX_TRY(make_map_blocked(&mb0, bhi, ncols, nkb, BN, sw, half));
        MGX_TRY(make_map_blocked(&mb1, blo, ncols, nkb, BN, sw, half));
    }
    else
    {
        MGX_TRY(make_map(&mb0, bhi, bf, n, ncols, ldk, BN, sw));
        mb1 = mb0;
        if (bf) MGX_TRY(make_map(&mb1, blo, true, n, ncols, ldk, BN, sw));
    }
    const int bkk     = bf ? sw / 2 : 32;
    const int kblocks = (int)((n + bkk - 1) / bkk);
    const int ntj     = (ncols + BN - 1) / BN;
    for (size_t p0 = 0; p0 < npts; p0 += P)
    {
        const int Pc = (int)std::min(P, npts - p0);
        if (blk)
        {
            dim3 tg((Pc + TB_P - 1) / TB_P, nkb);
            if (half)
                transpose_split_blocked_kernel<__half><<<tg, 256, 0, s>>>(psi, ld, n, p0, Pc,
                    (__half*)ahi, (__half*)alo, sa);
            else
                transpose_split_blocked_kernel<__nv_bfloat16><<<tg, 256, 0, s>>>(psi, ld, n, p0,
                    Pc, (__nv_bfloat16*)ahi, (__nv_bfloat16*)alo, nullptr);
            MGX_LAUNCH_CHECK("transpose_split_blocked_kernel");
            MGX_TRY(make_map_blocked(&ma0, ahi, Pc, nkb, BM, sw, half));
            MGX_TRY(make_map_blocked(&ma1, alo, Pc, nkb, BM, sw, half));
        }
        else
        {
            dim3 tg((Pc + 63) / 64, (n + 63) / 64);
            if (tg.y > 65535) return fail(MGX_UNSUPPORTED, "too many functions");
            if (bf)
                transpose_split_kernel<true><<<tg, 256, 0, s>>>(psi, ld, n, p0, Pc, ahi, alo, ldk);
            else
                transpose_split_kernel<false><<<tg, 256, 0, s>>>(psi, ld, n, p0, Pc, ahi, alo, ldk);
            MGX_LAUNCH_CHECK("transpose_split_kernel");
            MGX_TRY(make_map(&ma0, ahi, bf, n, Pc, ldk, BM, sw));
            ma1 = ma0;
            if (bf) MGX_TRY(make_map(&ma1, alo, true, n, Pc, ldk, BM, sw));
        }
        Params p;
        p.tiles      = nullptr;
        p.kblocks    = kblocks;
        p.kb_per_cta = kblocks;
        p.n          = 0;
        p.ncols      = ncols;
        p.symmetric  = 0;
        p.C          = nullptr;
        p.err        = (int*)ctx->tc_err.ptr;
        p.out        = out ? out + p0 : nullptr;
        p.cin        = cin ? cin + p0 : nullptr;
        if (rho)
        {
            // the density: the product is reduced against psi itself
            p.rho  = rho + p0;
            p.rpsi = psi + p0;
            p.ldr  = ld;
        }
        p.ldo        = ld;
        p.beta       = cin ? beta : 0.f;
        p.nrows      = Pc;
        p.ntj        = ntj;
        p.blocked    = blk ? 1 : 0;
        p.sa         = sa;
        p.sb         = sb;
        const int ntiles = ((Pc + BM - 1) / BM) * ntj;
        if (half)
        {
            if (BN == 256)
                MGX_TRY((launch<2, 3, 256, 4, true, 64>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            else
                MGX_TRY((launch<2, 3, 128, 6, true, 64>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
        }
        else if (BN == 256)
        {
            if (bf && sw == 64)
                MGX_TRY((launch<1, 3, 256, 4, true, 64>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            else if (bf)
                MGX_TRY((launch<1, 3, 256, 2, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            else
                MGX_TRY((launch<0, 1, 256, 4, true>(ma0, ma0, mb0, mb0, p, ntiles, 1, s, sms)));
        }
        else
        {
            if (bf && sw == 64)
                MGX_TRY((launch<1, 3, 128, 6, true, 64>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            else if (bf)
                MGX_TRY((launch<1, 3, 128, 3, true>(ma0, ma1, mb0, mb1, p, ntiles, 1, s, sms)));
            else
                MGX_TRY((launch<0, 1, 128, 6, true>(ma0, ma0, mb0, mb0, p, ntiles, 1, s, sms)));
        }
    }
    return end(ctx, s);
}
} // namespace mgx

extern "C" {

int mgx_timing_enable(int on)
{
    mgx::g_timing_on.store(on ? 1 : 0);
    return MGX_OK;
}

int mgx_timing_read(int cls, double* total_ms, int* launches)
{
    using namespace mgx;
    if (!total_ms || !launches) return fail(MGX_BAD_ARG, "NULL output");
    std::lock_guard<std::mutex> lk(g_timing_mu);
    double tot = 0.;
    int n      = 0;
    std::vector<TimedLaunch> keep;
    for (auto& t : g_timed)
    {
        if (t.cls != cls)
        {
            keep.push_back(t);
            continue;
        }
        float ms = 0.f;
        if (cudaEventSynchronize(t.b) == cudaSuccess && cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess)
        {
            tot += ms;
            n++;
        }
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    g_timed.swap(keep);
    *total_ms = tot;
    *launches = n;
    return MGX_OK;
}

} // extern "C"
