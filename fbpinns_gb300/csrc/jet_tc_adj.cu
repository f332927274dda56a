// C ABI of the tensor-core adjoint (tcgen05 recompute of the layer-2 jets)
// for tanh networks xd-16-16-1.
#include <algorithm>
#include <mutex>

#include "jet_tc_adj.cuh"

namespace fbp {

template <class C>
constexpr size_t tc_adj_smem_bytes() {
    return ((sizeof(TcAdjSmem<C>) + 15) / 16) * 16 + (TC_TILE / 32) * sizeof(TcAdjWarp<C>);
}

template <int XD, int D2>
int launch_adjoint_tc(const fbp_net& net, const float* x, const fbp_pairs& pr, const float* slot_out,
                      float* grad_part, int32_t* status, int grid, cudaStream_t st) {
    using C = Cfg<XD, 16, 16, D2, FBP_ACT_TANH>;
    FBP_REQUIRE(net.nparam == C::P, FBP_ERR_INVALID, "adjoint_tc: nparam %d != %d for this shape", net.nparam, C::P);
    struct Launch {
        int res;     // resident CTAs per SM
        size_t shm;  // dynamic shared memory per CTA
    };
    static Launch launch_dev[FBP_MAX_DEVICES] = {};
    static std::mutex launch_mu;  // the first launch per device sets both fields; others read a copy
    const int dev = current_device();
    constexpr int cols = TcAdjSmem<C>::COLS;
    Launch L;
    {
        std::lock_guard<std::mutex> lock(launch_mu);
        Launch& cached = launch_dev[dev];
        if (!cached.res) {
            size_t shm = tc_adj_smem_bytes<C>();
            FBP_CUDA_CHECK(cudaFuncSetAttribute(adjoint_pairs_tc_kernel<C>,
                                                cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
            cudaFuncAttributes fa;
            FBP_CUDA_CHECK(cudaFuncGetAttributes(&fa, adjoint_pairs_tc_kernel<C>));
            int smem_sm = 0, regs_sm = 0, thr_sm = 0;
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev));
            FBP_CUDA_CHECK(cudaDeviceGetAttribute(&thr_sm, cudaDevAttrMaxThreadsPerMultiProcessor, dev));
            const int per_cta_smem = (int)(shm + fa.sharedSizeBytes) + 1024;  // + the runtime's 1 KiB per CTA
            const int per_cta_regs = ((fa.numRegs + 7) / 8 * 8) * TC_TILE;
            int res = std::min(std::min(smem_sm / per_cta_smem, regs_sm / std::max(per_cta_regs, 1)), thr_sm / TC_TILE);
            FBP_REQUIRE(res >= 1, FBP_ERR_UNSUPPORTED, "adjoint_tc: kernel does not fit on an SM");
            // a CTA beyond 512 / COLS TMEM columns per SM would block in tcgen05.alloc:
            // pad the shared-memory request until no more than that many fit
            const int max_res = 512 / cols;
            if (res > max_res) {
                const int pad_cta = smem_sm / max_res;
                shm = (size_t)(pad_cta - (int)fa.sharedSizeBytes - 1024);
                FBP_CUDA_CHECK(cudaFuncSetAttribute(adjoint_pairs_tc_kernel<C>,
                                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
                res = max_res;
            }
            cached.shm = shm;
            cached.res = res;
        }
        L = cached;
    }
    FBP_REQUIRE(L.res * cols <= 512, FBP_ERR_UNSUPPORTED, "adjoint_tc: %d CTAs/SM x %d TMEM columns > 512", L.res,
                cols);
    if (grid <= 0) grid = L.res * sm_count();
    if (pr.item_ctr) FBP_CUDA_CHECK(cudaMemsetAsync(pr.item_ctr, 0, sizeof(int32_t), st));
    adjoint_pairs_tc_kernel<C><<<grid, TC_TILE, L.shm, st>>>(net, x, pr, slot_out, grad_part, status);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

template <int XD, int D2>
int tc_adj_try(int mode, const fbp_net& net, const float* x, const fbp_pairs& pr, const float* slot_out,
               float* grad_part, int32_t* status, int grid, cudaStream_t st) {
    if (net.xd != XD || net.d2mask != D2 || net.act != FBP_ACT_TANH) return 1;
    if (mode == 2) return FBP_OK;
    return launch_adjoint_tc<XD, D2>(net, x, pr, slot_out, grad_part, status, grid, st);
}

#define FBP_TC_ADJ_TRY(XD, D2)                                                                      \
    {                                                                                               \
        int r_ = tc_adj_try<XD, D2>(mode, *net, x, *pr, slot_out, grad_part, status, grid, st);     \
        if (r_ != 1) return r_;                                                                     \
    }

static int tc_adj_dispatch(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                           float* grad_part, int32_t* status, int grid, cudaStream_t st) {
    if (net->ud != 1 || net->h1 != 16 || net->h2 != 16) return 1;
    FBP_TC_ADJ_TRY(2, 3 | FBP_D2_LAPLACIAN)
    FBP_TC_ADJ_TRY(2, 3)
    FBP_TC_ADJ_TRY(2, 1)
    FBP_TC_ADJ_TRY(2, 0)
    return 1;
}
}  // namespace fbp

extern "C" int fbp_adjoint_pairs_tc(const fbp_net* net, const float* x, const fbp_pairs* pairs, const float* slot_out,
                                    float* grad_part, int32_t* status, int32_t grid, void* stream) {
    FBP_REQUIRE(net && pairs && x && slot_out && grad_part && status, FBP_ERR_INVALID,
                "fbp_adjoint_pairs_tc: null argument");
    FBP_REQUIRE(net->theta && net->xmins && net->xmaxs && net->flags && net->unnorms, FBP_ERR_INVALID,
                "fbp_adjoint_pairs_tc: null network pointer");
    FBP_REQUIRE(pairs->sd_rec && pairs->items && pairs->n_items, FBP_ERR_INVALID,
                "fbp_adjoint_pairs_tc: null pair pointer");
    const int r = fbp::tc_adj_dispatch(1, net, x, pairs, slot_out, grad_part, status, grid, fbp::as_stream(stream));
    if (r != 1) return r;
    fbp::set_error("fbp_adjoint_pairs_tc: no compiled kernel for xd=%d h1=%d h2=%d d2mask=%d act=%d", net->xd,
                   net->h1, net->h2, net->d2mask, net->act);
    return FBP_ERR_UNSUPPORTED;
}

extern "C" int fbp_has_tc_adjoint_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act) {
    fbp_net net{};
    net.xd = xd;
    net.h1 = h1;
    net.h2 = h2;
    net.ud = 1;
    net.d2mask = d2mask;
    net.act = act;
    fbp_pairs pr{};
    return fbp::tc_adj_dispatch(2, &net, nullptr, &pr, nullptr, nullptr, nullptr, 0, nullptr) == FBP_OK ? 1 : 0;
}
