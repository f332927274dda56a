// Compiled network shapes, group F: FourierFCN with one hidden layer after its
// features (first layer: the frozen sin/cos feature map of 2 n_features
// neurons; second: tanh).
#include "jet_launch.cuh"

namespace fbp {
int jet_group_f(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                float* out, int grid, cudaStream_t st) {
    FBP_TRY_ACT(1, 8, 8, 1, FBP_ACT_FOURIER)
    FBP_TRY_ACT(2, 8, 8, 3, FBP_ACT_FOURIER)
    FBP_TRY_ACT(2, 8, 8, 11, FBP_ACT_FOURIER)
    FBP_TRY_ACT(1, 16, 32, 1, FBP_ACT_FOURIER)
    FBP_TRY_ACT(2, 16, 16, 1, FBP_ACT_FOURIER)
    FBP_TRY_ACT(2, 16, 32, 11, FBP_ACT_FOURIER)
    return 1;
}
}  // namespace fbp
