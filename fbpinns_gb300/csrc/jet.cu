// C ABI of the per-pair jet kernels: shape dispatch over the compiled groups.
#include "common.cuh"

namespace fbp {
int jet_group_a(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);
int jet_group_b(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);
int jet_group_c(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);
int jet_group_d(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);
int jet_group_e(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);
int jet_group_f(int, const fbp_net*, const float*, const fbp_pairs*, const float*, float*, int, cudaStream_t);

static int check_net(const fbp_net* net, const fbp_pairs* pr) {
    FBP_REQUIRE(net && pr, FBP_ERR_INVALID, "jet: null descriptor");
    FBP_REQUIRE(net->theta && net->xmins && net->xmaxs && net->flags && net->unnorms, FBP_ERR_INVALID,
                "jet: null network pointer");
    FBP_REQUIRE(pr->sd_rec && pr->items && pr->n_items, FBP_ERR_INVALID,
                "jet: null pair pointer");
    FBP_REQUIRE(net->ud == 1, FBP_ERR_UNSUPPORTED, "jet: ud=%d (only scalar outputs are compiled)", net->ud);
    return FBP_OK;
}

static int dispatch(int mode, const fbp_net* net, const float* x, const fbp_pairs* pr, const float* slot_out,
                    float* out, int grid, void* stream) {
    int rc = check_net(net, pr);
    if (rc) return rc;
    FBP_REQUIRE(x && out, FBP_ERR_INVALID, "jet: null x/out");
    cudaStream_t st = as_stream(stream);
    int r = jet_group_a(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    r = jet_group_b(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    r = jet_group_c(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    r = jet_group_d(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    r = jet_group_e(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    r = jet_group_f(mode, net, x, pr, slot_out, out, grid, st);
    if (r != 1) return r;
    set_error("jet: no compiled kernel for xd=%d h1=%d h2=%d d2mask=%d act=%d", net->xd, net->h1, net->h2,
              net->d2mask, net->act);
    return FBP_ERR_UNSUPPORTED;
}
}  // namespace fbp

extern "C" int fbp_forward_pairs(const fbp_net* net, const float* x, const fbp_pairs* pairs, float* pair_out,
                                 int32_t grid, void* stream) {
    return fbp::dispatch(0, net, x, pairs, nullptr, pair_out, grid, stream);
}

extern "C" int fbp_adjoint_pairs(const fbp_net* net, const float* x, const fbp_pairs* pairs, const float* slot_out,
                                 float* grad_part, int32_t grid, void* stream) {
    FBP_REQUIRE(slot_out, FBP_ERR_INVALID, "fbp_adjoint_pairs: null slot_out");
    return fbp::dispatch(1, net, x, pairs, slot_out, grad_part, grid, stream);
}

extern "C" int fbp_has_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act) {
    fbp_net net{};
    net.xd = xd;
    net.h1 = h1;
    net.h2 = h2;
    net.ud = 1;
    net.d2mask = d2mask;
    net.act = act;
    fbp_pairs pr{};
    int r = fbp::jet_group_a(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    if (r == 1) r = fbp::jet_group_b(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    if (r == 1) r = fbp::jet_group_c(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    if (r == 1) r = fbp::jet_group_d(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    if (r == 1) r = fbp::jet_group_e(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    if (r == 1) r = fbp::jet_group_f(2, &net, nullptr, &pr, nullptr, nullptr, 0, nullptr);
    return r == FBP_OK ? 1 : 0;
}
