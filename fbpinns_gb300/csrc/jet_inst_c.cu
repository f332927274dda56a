// Compiled network shapes, group C: (2+1)D wave shapes.
#include "jet_launch.cuh"

namespace fbp {
int jet_group_c(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                float* out, int grid, cudaStream_t st) {
    FBP_TRY(3, 32, 32, 7)
    FBP_TRY(3, 32, 32, 0)
    FBP_TRY(3, 8, 8, 7)
    FBP_TRY(3, 32, 32, 55)  // 7 | FBP_D2_GROUP(3): u_xx + u_yy and u_tt (wave)
    FBP_TRY(3, 8, 8, 55)
    return 1;
}
}  // namespace fbp
