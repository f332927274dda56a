// Tensor-core forward for the other activations of 2-16-16-1 networks: SIREN,
// AdaptiveFCN, AdaptiveSIREN (Laplacian and first-derivative jets) and
// FourierFCN with 8 features (first-derivative jets).
#include "jet_tc_launch.cuh"

namespace fbp {
int tc_group_act(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, float* pair_out,
                 int32_t* status, int grid, cudaStream_t st) {
    FBP_TC_TRY(2, 3 | FBP_D2_LAPLACIAN, FBP_ACT_SIN)
    FBP_TC_TRY(2, 1, FBP_ACT_SIN)
    FBP_TC_TRY(2, 3 | FBP_D2_LAPLACIAN, FBP_ACT_ADAPTIVE_TANH)
    FBP_TC_TRY(2, 1, FBP_ACT_ADAPTIVE_TANH)
    FBP_TC_TRY(2, 3 | FBP_D2_LAPLACIAN, FBP_ACT_ADAPTIVE_SIN)
    FBP_TC_TRY(2, 1, FBP_ACT_ADAPTIVE_SIN)
    FBP_TC_TRY(2, 1, FBP_ACT_FOURIER)
    return 1;
}
}  // namespace fbp
