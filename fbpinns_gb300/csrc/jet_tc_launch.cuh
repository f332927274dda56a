// Launch wrapper of the tensor-core forward for one compiled (xd, d2mask,
// activation); included by the translation units that instantiate them.
#pragma once

#include <algorithm>
#include <mutex>

#include "jet_tc.cuh"

namespace fbp {

template <int XD, int D2, int ACT>
int launch_forward_tc(const fbp_net& net, const float* x, const fbp_pairs& pr, float* pair_out,
                             int32_t* status, int grid, cudaStream_t st) {
    using C = Cfg<XD, 16, 16, D2, ACT>;
    FBP_REQUIRE(net.nparam == C::P, FBP_ERR_INVALID, "forward_tc: nparam %d != %d for this shape", net.nparam, C::P);
    struct Launch {
        int res;     // resident CTAs per SM
        size_t shm;  // dynamic shared memory per CTA
    };
    static Launch launch_dev[FBP_MAX_DEVICES] = {};  // per device
    static std::mutex launch_mu;  // the first launch per device sets both fields; others read a copy
    const int dev = current_device();
    constexpr int cols = TcSmem<C>::COLS;
    Launch L;
    {
        std::lock_guard<std::mutex> lock(launch_mu);
        Launch& cached = launch_dev[dev];
        if (!cached.res) {
            size_t shm = sizeof(TcSmem<C>);
            FBP_CUDA_CHECK(cudaFuncSetAttribute(forward_pairs_tc_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                (int)shm));
            // CTAs that fit on one SM by shared memory, registers and threads: an
            // upper bound on how many can be resident at once
            cudaFuncAttributes fa;
            FBP_CUDA_CHECK(cudaFuncGetAttributes(&fa, forward_pairs_tc_kernel<C>));
            int smem_sm = 0, regs_sm = 0, thr_sm = 0;
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
            const int per_cta_smem = (int)(shm + fa.sharedSizeBytes) + 1024;  // + the CUDA runtime's 1 KiB reserved per CTA
            const int per_cta_regs = ((fa.numRegs + 7) / 8 * 8) * TC_TILE;
            int res = std::min(std::min(smem_sm / per_cta_smem, regs_sm / std::max(per_cta_regs, 1)), thr_sm / TC_TILE);
            FBP_REQUIRE(res >= 1, FBP_ERR_UNSUPPORTED, "forward_tc: kernel does not fit on an SM");
            // every resident CTA holds COLS of the SM's 512 TMEM columns; a CTA
            // beyond that would block in tcgen05.alloc, so the shared-memory
            // request is padded until no more than 512 / COLS CTAs fit
            const int max_res = 512 / cols;
            if (res > max_res) {
                const int pad_cta = smem_sm / max_res;  // (max_res + 1) * pad_cta > smem_sm
                shm = (size_t)(pad_cta - (int)fa.sharedSizeBytes - 1024);
                FBP_CUDA_CHECK(cudaFuncSetAttribute(forward_pairs_tc_kernel<C>,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
                res = max_res;
            }
            cached.shm = shm;
            cached.res = res;
        }
        L = cached;
    }
    const int res = L.res;
    FBP_REQUIRE(res * cols <= 512, FBP_ERR_UNSUPPORTED, "forward_tc: %d CTAs/SM x %d TMEM columns > 512", res, cols);
    if (grid <= 0) grid = res * sm_count();
    if (pr.item_ctr) FBP_CUDA_CHECK(cudaMemsetAsync(pr.item_ctr, 0, sizeof(int32_t), st));
    forward_pairs_tc_kernel<C><<<grid, TC_TILE, L.shm, st>>>(net, x, pr, pair_out, status);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

// Tries one compiled variant; returns 1 (not this one) or the launch status
// (mode 1: launch, mode 2: query).
template <int XD, int D2, int ACT>
int tc_try(int mode, const fbp_net& net, const float* x, const fbp_pairs& pr, float* pair_out, int32_t* status,
           int grid, cudaStream_t st) {
    if (net.xd != XD || net.d2mask != D2 || net.act != ACT) return 1;
    if (mode == 2) return FBP_OK;
    return launch_forward_tc<XD, D2, ACT>(net, x, pr, pair_out, status, grid, st);
}

}  // namespace fbp

#define FBP_TC_TRY(XD, D2, ACT)                                                                       \
    {                                                                                                 \
        int r_ = fbp::tc_try<XD, D2, ACT>(mode, *net, x, *pr, pair_out, status, grid, st);             \
        if (r_ != 1) return r_;                                                                       \
    }
