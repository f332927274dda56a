// C ABI of the tensor-core forward jet kernel (tcgen05, 3xTF32) for networks
// with two 16-wide hidden layers: the plain tanh FCN here, the other
// activations in jet_tc_act.cu.
#include "jet_tc_launch.cuh"

namespace fbp {
int tc_group_act(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, float* pair_out,
                 int32_t* status, int grid, cudaStream_t st);

static int tc_dispatch(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, float* pair_out,
                       int32_t* status, int grid, cudaStream_t st) {
    if (net->ud != 1 || net->h1 != 16 || net->h2 != 16) return 1;
    FBP_TC_TRY(2, 3 | FBP_D2_LAPLACIAN, FBP_ACT_TANH)
    FBP_TC_TRY(2, 3, FBP_ACT_TANH)
    FBP_TC_TRY(2, 1, FBP_ACT_TANH)
    FBP_TC_TRY(2, 0, FBP_ACT_TANH)
    return tc_group_act(mode, net, x, pr, pair_out, status, grid, st);
}
}  // namespace fbp

extern "C" int fbp_forward_pairs_tc(const fbp_net* net, const float* x, const fbp_pairs* pairs, float* pair_out,
                                    int32_t* status, int32_t grid, void* stream) {
    FBP_REQUIRE(net && pairs && x && pair_out && status, FBP_ERR_INVALID, "fbp_forward_pairs_tc: null argument");
    FBP_REQUIRE(net->theta && net->xmins && net->xmaxs && net->flags && net->unnorms, FBP_ERR_INVALID,
                "fbp_forward_pairs_tc: null network pointer");
    FBP_REQUIRE(pairs->sd_rec && pairs->items && pairs->n_items, FBP_ERR_INVALID,
                "fbp_forward_pairs_tc: null pair pointer");
    FBP_REQUIRE(net->ud == 1 && net->h1 == 16 && net->h2 == 16, FBP_ERR_UNSUPPORTED,
                "fbp_forward_pairs_tc: only the xd-16-16-1 networks are compiled (got h1=%d h2=%d ud=%d)", net->h1,
                net->h2, net->ud);
    const int r = fbp::tc_dispatch(1, net, x, pairs, pair_out, status, grid, fbp::as_stream(stream));
    if (r != 1) return r;
    fbp::set_error("fbp_forward_pairs_tc: no compiled kernel for xd=%d d2mask=%d act=%d", net->xd, net->d2mask,
                   net->act);
    return FBP_ERR_UNSUPPORTED;
}

extern "C" int fbp_has_tc_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act) {
    fbp_net net{};
    net.xd = xd;
    net.h1 = h1;
    net.h2 = h2;
    net.ud = 1;
    net.d2mask = d2mask;
    net.act = act;
    fbp_pairs pr{};
    return fbp::tc_dispatch(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr) == FBP_OK ? 1 : 0;
}
