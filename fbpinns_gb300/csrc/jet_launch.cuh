// Launch wrappers for one compiled network shape; included by the jet_inst_*.cu
// translation units, each of which instantiates a group of shapes.
#pragma once

#include "jet.cuh"

namespace fbp {

// Persistent grid: every CTA that can be resident at once (occupancy x SMs).
template <class K>
int resident_grid(K kernel, int threads, size_t smem) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * sm_count();
}

template <int XD, int H1, int H2, int D2, int ACT>
int launch_forward(const fbp_net& net, const float* x, const fbp_pairs& pr, float* pair_out, int grid,
                   cudaStream_t st) {
    using C = Cfg<XD, H1, H2, D2, ACT>;
    FBP_REQUIRE(net.nparam == C::P, FBP_ERR_INVALID, "forward: nparam %d != %d for this shape", net.nparam, C::P);
    static int auto_grid[FBP_MAX_DEVICES] = {};
    const int dev = current_device();
    if (grid <= 0) {
        if (!auto_grid[dev]) auto_grid[dev] = resident_grid(forward_pairs_kernel<C>, FWD_THREADS, 0);
        grid = auto_grid[dev];
    }
    if (pr.item_ctr) FBP_CUDA_CHECK(cudaMemsetAsync(pr.item_ctr, 0, sizeof(int32_t), st));
    forward_pairs_kernel<C><<<grid, FWD_THREADS, 0, st>>>(net, x, pr, pair_out);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

template <int XD, int H1, int H2, int D2, int ACT>
int launch_adjoint(const fbp_net& net, const float* x, const fbp_pairs& pr, const float* slot_out,
                   float* grad_part, int grid, cudaStream_t st) {
    using C = Cfg<XD, H1, H2, D2, ACT>;
    FBP_REQUIRE(net.nparam == C::P, FBP_ERR_INVALID, "adjoint: nparam %d != %d for this shape", net.nparam, C::P);
    const size_t shm = sizeof(WarpRows<C>) * AdjW<C>::W;
    static bool attr_set[FBP_MAX_DEVICES] = {};
    static int auto_grid[FBP_MAX_DEVICES] = {};
    const int dev = current_device();
    if (!attr_set[dev]) {
        FBP_CUDA_CHECK(cudaFuncSetAttribute(adjoint_pairs_kernel<C>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
        attr_set[dev] = true;
    }
    if (grid <= 0) {
        if (!auto_grid[dev]) auto_grid[dev] = resident_grid(adjoint_pairs_kernel<C>, AdjW<C>::T, shm);
        grid = auto_grid[dev];
    }
    if (pr.item_ctr) FBP_CUDA_CHECK(cudaMemsetAsync(pr.item_ctr, 0, sizeof(int32_t), st));
    adjoint_pairs_kernel<C><<<grid, AdjW<C>::T, shm, st>>>(net, x, pr, slot_out, grad_part);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

// Tries one shape; returns 1 (not this shape) or the launch status.
template <int XD, int H1, int H2, int D2, int ACT>
int try_shape(int mode, const fbp_net& net, const float* x, const fbp_pairs& pr, const float* slot_out, float* out,
              int grid, cudaStream_t st) {
    if (net.xd != XD || net.h1 != H1 || net.h2 != H2 || net.d2mask != D2 || net.act != ACT) return 1;
    if (mode == 2) return FBP_OK;  // shape query: compiled
    if (mode == 0) return launch_forward<XD, H1, H2, D2, ACT>(net, x, pr, out, grid, st);
    return launch_adjoint<XD, H1, H2, D2, ACT>(net, x, pr, slot_out, out, grid, st);
}

}  // namespace fbp

#define FBP_TRY_ACT(XD, H1, H2, D2, ACT)                                                         \
    {                                                                                            \
        int r_ = fbp::try_shape<XD, H1, H2, D2, ACT>(mode, *net, x, *pr, slot_out, out, grid, st); \
        if (r_ != 1) return r_;                                                                  \
    }
#define FBP_TRY(XD, H1, H2, D2) FBP_TRY_ACT(XD, H1, H2, D2, FBP_ACT_TANH)
