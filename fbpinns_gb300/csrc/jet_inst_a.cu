// Compiled network shapes, group A: the 1D oscillator and 2D Burgers / Poisson shapes.
#include "jet_launch.cuh"

namespace fbp {
int jet_group_a(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                float* out, int grid, cudaStream_t st) {
    FBP_TRY(1, 32, 32, 1)
    FBP_TRY(1, 32, 32, 0)
    FBP_TRY(1, 32, 0, 1)
    FBP_TRY(1, 8, 8, 1)
    FBP_TRY(2, 16, 16, 1)
    FBP_TRY(2, 16, 16, 0)
    FBP_TRY(2, 16, 0, 1)
    FBP_TRY(2, 16, 16, 11)  // Laplacian slot (Poisson)
    return 1;
}
}  // namespace fbp
