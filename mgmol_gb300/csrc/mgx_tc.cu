// Tensor-core (tcgen05) Gram / H-matrix products: placeholder until the
// tcgen05 kernels land.
#include "mgx_internal.cuh"

namespace mgx
{
int gram_tcgen05(mgx_ctx*, int mode, const void*, const void*, size_t, size_t,
    int, double, int, double*, cudaStream_t)
{
    return fail(MGX_UNSUPPORTED, "gemm mode %d not built yet", mode);
}
} // namespace mgx
