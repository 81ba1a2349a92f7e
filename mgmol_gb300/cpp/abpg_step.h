// abpg_step.h -- one electronic iteration of MGmol's quench on the GPU,
// scheduled by C++ host code over the mgx C ABI (include/mgx.h).
//
// In the reference, DFTsolver<T>::solve (src/DFTsolver.cc:262-400) runs per
// iteration: Hamiltonian::applyLocal and addHlocalij (H psi and H), the
// projected matrices (ProjectedMatricesMehrstellen::updateThetaAndHB:
// theta = B^-1 H with B from LocGridOrbitals::computeMatB, HB = sym(S theta),
// src/ProjectedMatricesMehrstellen.cc:38-64), the energy
// (ProjectedMatrices::getEigSum, src/ProjectedMatrices.cc:550-566), then
// ABPG<T>::updateWF / update_states (src/ABPG.cc:37-140): the residual
// B(psi) theta - H psi (MGmol::computeResidualUsingHPhi,
// src/MGmol.cc:1227-1290), the multigrid preconditioner
// (OrbitalsPreconditioning<T>::precond_mg, src/OrbitalsPreconditioning.cc:
// 86-117) and psi += 0.5 * precond_factor * P(res); then
// LocGridOrbitals::normalize and computeGramAndInvS (S and S^-1).
//
// AbpgStep<T> runs that iteration on a device block in the order that
// suits one GPU:
//   - S, H and B come from one call (mgx_gram_hmat_matb), so the
//     tensor-core modes convert psi once; the Psi Theta product of the
//     residual reads that conversion again (mgx_set_reuse_conversion); with
//     FP32 orbitals and split-BF16x3 products H psi is made inside that call
//     (mgx_hpsi_gram_hmat_matb), its chunks written straight into the H
//     product's operand planes;
//   - the critical path is H psi -> S, H, B -> Cholesky of B ->
//     theta = B^-1 H -> residual -> V-cycle; the S side of the dense algebra
//     (Cholesky and inverse of S, HB, the energy) is queued, once theta is
//     done, on a second stream of higher priority with its own context, so
//     that its FP64 kernels run beside the residual and the V-cycle instead
//     of before them;
//   - the normalization is folded into the update: the iteration runs on
//     the block as the previous update left it, and the factors
//     1 / sqrt(S(i, i)) of that block scale the update of the last V-cycle
//     sweep (mgx_precond_mg_update); the results are the reference's
//     normalize-then-iterate to rounding (every quantity is covariant under
//     the column scaling; the energy is invariant);
//   - with chunk_funcs > 0 the residual and the V-cycle walk the block in
//     column chunks (mgx_residual_cols), so that the block, H psi and two
//     chunk buffers are all the memory the iteration needs (the FP64 path
//     at 2048 orbitals on 192^3 fits one GPU that way); the normalization
//     is then a pass of its own before the iteration.
// Failures the reference aborts on (a Cholesky with a non-positive pivot)
// throw mgx::Error with the C-ABI status.  Header only; link against
// libmgx.so and the CUDA runtime.
#pragma once

#include "mgmol_adaptor.h"

namespace mgx
{

struct AbpgOptions
{
    int lap_type          = 0;     // Laph4M (Mehrstellen); 1..4 the others
    int gemm              = -1;    // product mode; -1: FP64 for double, BF16X3 for float
    int maxlevels         = 2;     // coarse levels of the V-cycle
    double precond_factor = 1.;    // ABPG step: alpha = 0.5 * precond_factor
    double gamma          = 0.;    // V-cycle gamma; 0: OrbitalsPreconditioning::setGamma
    int chunk_funcs       = 0;     // > 0: residual and V-cycle in column chunks
    bool fuse_update      = true;  // normalization folded into the update
    bool use_matb         = true;  // Mehrstellen: theta = B^-1 H (else S^-1 H)
};

template <typename T>
class AbpgStep
{
    const pb::Grid& grid_;
    int n_;
    size_t np_;
    AbpgOptions o_;
    mgx_ctx* ctx_  = nullptr;
    mgx_ctx* sctx_ = nullptr;
    cudaStream_t side_       = nullptr;
    cudaEvent_t theta_done_  = nullptr;
    cudaEvent_t side_done_   = nullptr;
    const void* V_;
    mgx_dtype vtype_;
    bool mehr_, matb_;
    int chunk_;
    DeviceArray<T> hpsi_, corr_, work_;
    DeviceArray<double> S_, H_, B_, LB_, LS_, theta_, Sinv_, HB_, scale_, energy_;
    DeviceArray<int> info_;

    mgx_dtype dt() const { return dtype_of<T>(); }
    int gemm() const
    {
        if (o_.gemm >= 0) return o_.gemm;
        return std::is_same<T, double>::value ? MGX_GEMM_FP64 : MGX_GEMM_BF16X3;
    }
    size_t nn() const { return (size_t)n_ * n_; }

public:
    /* V: the local potential on the device (npts values of v_dtype),
     * kept by pointer; vmin / vmax: its range, for setGamma. */
    AbpgStep(const pb::Grid& grid, const void* V, mgx_dtype v_dtype, double vmin, double vmax,
        int nfunc, AbpgOptions opts = AbpgOptions())
        : grid_(grid), n_(nfunc), np_((size_t)grid.dim(0) * grid.dim(1) * grid.dim(2)),
          o_(opts), V_(V), vtype_(v_dtype)
    {
        mehr_  = o_.lap_type == 0;
        matb_  = mehr_ && o_.use_matb;
        chunk_ = (o_.chunk_funcs > 0 && o_.chunk_funcs < n_) ? o_.chunk_funcs : 0;
        if (chunk_) o_.fuse_update = false;
        check(mgx_create(&grid_.raw(), &ctx_), "mgx_create");
        check(mgx_create(&grid_.raw(), &sctx_), "mgx_create (side)");
        // the FP32 path's Psi Theta reads the Gram products' conversion of psi
        check(mgx_set_reuse_conversion(ctx_, 1), "mgx_set_reuse_conversion");
        int lo = 0, hi = 0;
        cuda(cudaDeviceGetStreamPriorityRange(&lo, &hi), "cudaDeviceGetStreamPriorityRange");
        cuda(cudaStreamCreateWithPriority(&side_, cudaStreamNonBlocking, hi), "side stream");
        cuda(cudaEventCreateWithFlags(&theta_done_, cudaEventDisableTiming), "event");
        cuda(cudaEventCreateWithFlags(&side_done_, cudaEventDisableTiming), "event");
        hpsi_  = DeviceArray<T>((size_t)n_ * np_);
        corr_  = DeviceArray<T>((size_t)(chunk_ ? chunk_ : n_) * np_);
        if (chunk_) work_ = DeviceArray<T>((size_t)chunk_ * np_);
        S_     = DeviceArray<double>(nn());
        H_     = DeviceArray<double>(nn());
        theta_ = DeviceArray<double>(nn());
        Sinv_  = DeviceArray<double>(nn());
        LS_    = DeviceArray<double>(nn());
        if (matb_)
        {
            B_  = DeviceArray<double>(nn());
            LB_ = DeviceArray<double>(nn());
            HB_ = DeviceArray<double>(nn());
        }
        scale_  = DeviceArray<double>((size_t)n_);
        energy_ = DeviceArray<double>(1);
        info_   = DeviceArray<int>(2);
        if (o_.gamma <= 0.)
            check(mgx_precond_gamma(&grid_.raw(), o_.lap_type, o_.maxlevels, vmax, vmin, &o_.gamma),
                "mgx_precond_gamma");
    }
    AbpgStep(const AbpgStep&)            = delete;
    AbpgStep& operator=(const AbpgStep&) = delete;
    ~AbpgStep()
    {
        if (side_) cudaStreamSynchronize(side_);
        if (theta_done_) cudaEventDestroy(theta_done_);
        if (side_done_) cudaEventDestroy(side_done_);
        if (side_) cudaStreamDestroy(side_);
        if (sctx_) mgx_destroy(sctx_);
        if (ctx_) mgx_destroy(ctx_);
    }

    double gamma() const { return o_.gamma; }
    double alpha() const { return 0.5 * o_.precond_factor; }
    /* device matrices of the last iteration (FP64, column-major n x n) */
    const double* S() const { return S_.data(); }
    const double* H() const { return H_.data(); }
    const double* theta() const { return theta_.data(); }
    const double* Sinv() const { return Sinv_.data(); }
    /* the residual (unfused or chunked schedules: P(res) after run) */
    const T* hpsi() const { return hpsi_.data(); }

    /* One iteration on psi (device, n functions of npts values, leading
     * dimension npts), queued on `stream`; with update false psi is left
     * as it was (the block is normalized first in that case).  The call
     * returns once the work is queued, except for the explicit
     * normalization of the unfused schedules, which waits for its sums. */
    void run(T* psi, cudaStream_t stream = nullptr, bool update = true)
    {
        const size_t ld = np_;
        const bool lazy = o_.fuse_update && update;
        void* s = (void*)stream;
        if (!lazy) check(mgx_normalize(ctx_, dt(), psi, ld, n_, nullptr, s), "normalize");
        // FP32 Mehrstellen with B and split-BF16x3 products: H psi made
        // inside the H product, written straight into its operand planes
        const bool fused = matb_ && std::is_same<T, float>::value && vtype_ == MGX_F32
                           && gemm() == MGX_GEMM_BF16X3;
        if (fused)
            check(mgx_hpsi_gram_hmat_matb(ctx_, gemm(), (const float*)psi, (const float*)V_,
                      (float*)hpsi_.data(), ld, n_, S_.data(), H_.data(), B_.data(),
                      chunk_ ? (void*)work_.data() : (void*)corr_.data(), chunk_ ? chunk_ : n_, s),
                "applyLocal / computeGram / addHlocalij / computeMatB");
        else
        {
            check(mgx_hpsi(ctx_, o_.lap_type, dt(), psi, ld, V_, vtype_, hpsi_.data(), n_, 1, s),
                "applyLocal");
            if (matb_)
                check(mgx_gram_hmat_matb(ctx_, gemm(), psi, hpsi_.data(), ld, n_, S_.data(),
                          H_.data(), B_.data(), chunk_ ? work_.data() : corr_.data(),
                          chunk_ ? chunk_ : n_, s),
                    "computeGram / addHlocalij / computeMatB");
            else
                check(mgx_gram_hmat(ctx_, gemm(), psi, hpsi_.data(), ld, n_, S_.data(), H_.data(),
                          s),
                    "computeGram / addHlocalij");
        }
        if (matb_)
        {
            // computeInvB + updateTheta: theta = B^-1 H from the factor of B
            cuda(cudaMemcpyAsync(LB_.data(), B_.data(), nn() * sizeof(double),
                     cudaMemcpyDeviceToDevice, stream), "copy B");
            check(mgx_cholesky_async(ctx_, n_, LB_.data(), info_.data(), s), "Cholesky of B");
            check(mgx_theta_from_cholesky(ctx_, n_, LB_.data(), H_.data(), theta_.data(), nullptr, s),
                "updateTheta");
            cuda(cudaEventRecord(theta_done_, stream), "event");
            // the S side after theta, beside the residual and the V-cycle
            cuda(cudaStreamWaitEvent(side_, theta_done_, 0), "wait");
            void* ss = (void*)side_;
            cuda(cudaMemcpyAsync(LS_.data(), S_.data(), nn() * sizeof(double),
                     cudaMemcpyDeviceToDevice, side_), "copy S");
            check(mgx_cholesky_async(sctx_, n_, LS_.data(), info_.data() + 1, ss), "Cholesky of S");
            check(mgx_inverse_from_cholesky(sctx_, n_, LS_.data(), Sinv_.data(), ss), "computeInverse");
            check(mgx_update_hb(sctx_, n_, S_.data(), theta_.data(), HB_.data(), ss), "updateHB");
            check(mgx_trace_prod(sctx_, n_, HB_.data(), Sinv_.data(), energy_.data(), ss), "getEigSum");
            cuda(cudaEventRecord(side_done_, side_), "event");
        }
        else
        {
            cuda(cudaMemcpyAsync(LS_.data(), S_.data(), nn() * sizeof(double),
                     cudaMemcpyDeviceToDevice, stream), "copy S");
            check(mgx_cholesky_async(ctx_, n_, LS_.data(), info_.data() + 1, s), "Cholesky of S");
            check(mgx_inverse_from_cholesky(ctx_, n_, LS_.data(), Sinv_.data(), s), "computeInverse");
            check(mgx_trace_prod(ctx_, n_, H_.data(), Sinv_.data(), energy_.data(), s), "getEigSum");
            check(mgx_theta(ctx_, n_, Sinv_.data(), H_.data(), theta_.data(), s), "updateTheta");
        }
        if (lazy) check(mgx_normalize_scales(ctx_, n_, S_.data(), scale_.data(), s), "scales");
        mgx_precond_params p = { o_.lap_type, o_.maxlevels, o_.gamma, 0 };
        if (!chunk_)
        {
            check(mgx_residual(ctx_, gemm(), dt(), psi, hpsi_.data(), ld, n_, theta_.data(), mehr_ ? 1 : 0,
                      corr_.data(), hpsi_.data(), s),
                "computeResidualUsingHPhi");
            if (lazy)
                check(mgx_precond_mg_update(ctx_, &p, dt(), hpsi_.data(), ld, psi, alpha(), scale_.data(),
                          n_, nullptr, corr_.data(), s),
                    "precond_mg + update_states");
            else
            {
                check(mgx_precond_mg(ctx_, &p, dt(), hpsi_.data(), ld, corr_.data(), n_, nullptr, s),
                    "precond_mg");
                if (update)
                    check(mgx_axpy((size_t)n_ * ld, alpha(), dt(), corr_.data(), psi, s), "update_states");
            }
        }
        else
        {
            for (int j0 = 0; j0 < n_; j0 += chunk_)
            {
                const int nc = std::min(chunk_, n_ - j0);
                T* hc        = hpsi_.data() + (size_t)j0 * ld;
                check(mgx_residual_cols(ctx_, gemm(), dt(), psi, hc, ld, n_, theta_.data() + (size_t)j0 * n_,
                          nc, mehr_ ? 1 : 0, work_.data(), hc, s),
                    "computeResidualUsingHPhi (columns)");
                check(mgx_precond_mg(ctx_, &p, dt(), hc, ld, corr_.data(), nc, nullptr, s), "precond_mg");
                cuda(cudaMemcpyAsync(hc, corr_.data(), (size_t)nc * ld * sizeof(T),
                         cudaMemcpyDeviceToDevice, stream), "copy P(res)");
            }
            if (update)
                check(mgx_axpy((size_t)n_ * ld, alpha(), dt(), hpsi_.data(), psi, s), "update_states");
        }
        if (matb_) cuda(cudaStreamWaitEvent(stream, side_done_, 0), "join side stream");
    }

    /* Waits for the last iteration; returns its energy tr(HB S^-1)
     * (ProjectedMatrices::getEigSum, Ry) and throws mgx::Error with
     * MGX_NOT_SPD when a Cholesky factorization failed. */
    double energy(cudaStream_t stream = nullptr)
    {
        double e  = 0.;
        int in[2] = { 0, 0 };
        cuda(cudaStreamSynchronize(stream), "iteration");
        cuda(cudaMemcpy(&e, energy_.data(), sizeof(double), cudaMemcpyDeviceToHost), "energy");
        cuda(cudaMemcpy(in, info_.data(), 2 * sizeof(int), cudaMemcpyDeviceToHost), "info");
        if (in[0] != 0 || in[1] != 0)
            throw Error(MGX_NOT_SPD, std::string("Cholesky of ") + (in[0] ? "B" : "S")
                                         + ": leading minor " + std::to_string(in[0] ? in[0] : in[1])
                                         + " not positive");
        return e;
    }
};

} // namespace mgx
