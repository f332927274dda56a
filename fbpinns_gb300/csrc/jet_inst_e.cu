// Compiled network shapes, group E: adaptive activations (AdaptiveFCN,
// AdaptiveSIREN), with their trainable per-neuron parameters.
#include "jet_launch.cuh"

namespace fbp {
int jet_group_e(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                float* out, int grid, cudaStream_t st) {
    FBP_TRY_ACT(1, 32, 32, 1, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(1, 8, 8, 1, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(2, 16, 16, 1, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(2, 16, 16, 11, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(2, 8, 8, 3, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(2, 8, 8, 11, FBP_ACT_ADAPTIVE_TANH)
    FBP_TRY_ACT(1, 32, 32, 1, FBP_ACT_ADAPTIVE_SIN)
    FBP_TRY_ACT(1, 8, 8, 1, FBP_ACT_ADAPTIVE_SIN)
    FBP_TRY_ACT(2, 16, 16, 1, FBP_ACT_ADAPTIVE_SIN)
    FBP_TRY_ACT(2, 16, 16, 11, FBP_ACT_ADAPTIVE_SIN)
    FBP_TRY_ACT(2, 8, 8, 3, FBP_ACT_ADAPTIVE_SIN)
    FBP_TRY_ACT(2, 8, 8, 11, FBP_ACT_ADAPTIVE_SIN)
    return 1;
}
}  // namespace fbp
