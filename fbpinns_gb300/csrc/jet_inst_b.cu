// Compiled network shapes, group B: 2D Poisson / Helmholtz shapes and small test shapes.
#include "jet_launch.cuh"

namespace fbp {
int jet_group_b(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                float* out, int grid, cudaStream_t st) {
    FBP_TRY(2, 16, 16, 3)
    FBP_TRY(2, 32, 32, 3)
    FBP_TRY(2, 32, 32, 0)
    FBP_TRY(2, 8, 8, 3)
    FBP_TRY(2, 8, 8, 1)
    FBP_TRY(2, 32, 32, 11)  // Laplacian slot (Helmholtz)
    FBP_TRY(2, 8, 8, 11)
    return 1;
}
}  // namespace fbp
