// Error reporting, Adam, the Philox sampler and the FMA throughput probe.
#include <math.h>
#include <algorithm>
#include <stdarg.h>
#include <string.h>

#include "common.cuh"

namespace fbp {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int current_device() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= FBP_MAX_DEVICES) dev = 0;
    return dev;
}

int sm_count() {
    static int cached[FBP_MAX_DEVICES] = {};  // per device
    const int dev = current_device();
    if (cached[dev]) return cached[dev];
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
        cached[dev] = n;
    else
        cached[dev] = kSM;
    return cached[dev];
}

// ---------------------------------------------------------------------------
// Adam, masked by the scheduler state (1 = active).  optax.adam: scale_by_adam
// (mu, nu moments, count incremented, bias corrections) then scale(-lr), then
// apply_updates.  Every thread reads the shared device count and uses count+1
// for the bias corrections; a separate one-thread kernel launched after this
// one stores the increment, so no block can see a half-updated count.
// ---------------------------------------------------------------------------
__global__ void adam_kernel(float* __restrict__ theta, float* __restrict__ m1, float* __restrict__ m2,
                            const float* __restrict__ grad, const uint8_t* __restrict__ state,
                            int64_t m, int P, float lr, float b1, float b2, float eps, float eps_root,
                            const int32_t* __restrict__ count_dev) {
    const int c = *count_dev + 1;
    const float bc1 = 1.0f - powf(b1, (float)c);
    const float bc2 = 1.0f - powf(b2, (float)c);
    const int64_t total = m * (int64_t)P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = i / P;
        if (state[row] != 1) continue;
        const float g = grad[i];
        const float mu = (1.0f - b1) * g + b1 * m1[i];
        const float nu = (1.0f - b2) * g * g + b2 * m2[i];
        m1[i] = mu;
        m2[i] = nu;
        const float mh = mu / bc1;
        const float nh = nu / bc2;
        theta[i] = theta[i] + (-lr) * (mh / (sqrtf(nh + eps_root) + eps));
    }
}

__global__ void count_inc_kernel(int32_t* count_dev) { *count_dev += 1; }

// ---------------------------------------------------------------------------
// Philox-4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy
// as 1, 2, 3", SC11).  Counter = (i, offset_lo, offset_hi, 0), key = seed.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void philox_round(uint32_t& c0, uint32_t& c1, uint32_t& c2, uint32_t& c3,
                                             uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t hi0 = __umulhi(M0, c0), lo0 = M0 * c0;
    const uint32_t hi1 = __umulhi(M1, c2), lo1 = M1 * c2;
    const uint32_t n0 = hi1 ^ c1 ^ k0, n1 = lo1, n2 = hi0 ^ c3 ^ k1, n3 = lo0;
    c0 = n0; c1 = n1; c2 = n2; c3 = n3;
}

__device__ __forceinline__ uint4 philox4x32_10(uint4 ctr, uint2 key) {
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    uint32_t c0 = ctr.x, c1 = ctr.y, c2 = ctr.z, c3 = ctr.w, k0 = key.x, k1 = key.y;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        philox_round(c0, c1, c2, c3, k0, k1);
        k0 += W0;
        k1 += W1;
    }
    return make_uint4(c0, c1, c2, c3);
}

struct Box3 {
    float lo[3], span[3];
};

__global__ void sample_uniform_kernel(float* __restrict__ x, int64_t n, int xd, Box3 box, uint64_t seed,
                                      uint64_t offset0, const int32_t* __restrict__ counter) {
    const uint64_t offset = offset0 + (counter ? (uint64_t)(uint32_t)*counter : 0ull);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const uint4 r = philox4x32_10(
            make_uint4((uint32_t)i, (uint32_t)(i >> 32), (uint32_t)offset, (uint32_t)(offset >> 32)),
            make_uint2((uint32_t)seed, (uint32_t)(seed >> 32)));
        const uint32_t rr[4] = {r.x, r.y, r.z, r.w};
        for (int d = 0; d < xd; ++d) {
            // 24 random mantissa bits -> [0, 1)
            const float u = (float)(rr[d] >> 8) * (1.0f / 16777216.0f);
            x[i * xd + d] = box.lo[d] + box.span[d] * u;
        }
    }
}

// Dependent FMA chains, 8 independent per thread: measures the FP32 FMA issue rate.
__global__ void fma_probe_kernel(float* sink, int iters) {
    float a[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 1e-3f + j;
    const float b = 0.9999f, c = 1e-4f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int j = 0; j < 8; ++j) a[j] = fmaf(a[j], b, c);
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 8; ++j) s += a[j];
    if (s == 12345.678f) sink[threadIdx.x] = s;  // keeps the chains live
}

__global__ void tanh_probe_kernel(const float* __restrict__ x, float* __restrict__ y, int64_t n) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = tanh_fast(x[i]);
}

}  // namespace fbp

using namespace fbp;

extern "C" int fbp_abi_version(void) { return 1; }

extern "C" const char* fbp_last_error(void) { return fbp::g_err; }

extern "C" int fbp_adam(float* theta, float* m1, float* m2, const float* grad, const uint8_t* state,
                        int64_t m, int32_t nparam, float lr, float b1, float b2, float eps,
                        float eps_root, int32_t* count_dev, void* stream) {
    FBP_REQUIRE(theta && m1 && m2 && grad && state && count_dev, FBP_ERR_INVALID, "fbp_adam: null pointer");
    FBP_REQUIRE(m >= 0 && nparam > 0, FBP_ERR_INVALID, "fbp_adam: bad sizes m=%lld P=%d", (long long)m, nparam);
    cudaStream_t st = as_stream(stream);
    if (m > 0) {
        const int64_t total = m * (int64_t)nparam;
        int blocks = (int)((total + 255) / 256);
        if (blocks > sm_count() * 8) blocks = sm_count() * 8;
        adam_kernel<<<blocks, 256, 0, st>>>(theta, m1, m2, grad, state, m, nparam, lr, b1, b2, eps, eps_root,
                                           count_dev);
        FBP_LAUNCH_CHECK();
    }
    count_inc_kernel<<<1, 1, 0, st>>>(count_dev);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" int fbp_sample_uniform(float* x, int64_t n, int32_t xd, const double* xmin, const double* xmax,
                                  uint64_t seed, uint64_t offset, const int32_t* counter, void* stream) {
    FBP_REQUIRE(x && xmin && xmax, FBP_ERR_INVALID, "fbp_sample_uniform: null pointer");
    FBP_REQUIRE(xd >= 1 && xd <= 3, FBP_ERR_INVALID, "fbp_sample_uniform: xd=%d not in 1..3", xd);
    FBP_REQUIRE(n >= 0, FBP_ERR_INVALID, "fbp_sample_uniform: n < 0");
    if (n == 0) return FBP_OK;
    Box3 b{};
    for (int d = 0; d < xd; ++d) {
        b.lo[d] = (float)xmin[d];
        b.span[d] = (float)(xmax[d] - xmin[d]);
    }
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 16) blocks = sm_count() * 16;
    sample_uniform_kernel<<<blocks, 256, 0, as_stream(stream)>>>(x, n, xd, b, seed, offset, counter);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" int fbp_graph_instantiate(void* graph, int32_t use_node_priority, void** exec_out) {
    FBP_REQUIRE(graph && exec_out, FBP_ERR_INVALID, "fbp_graph_instantiate: null argument");
    cudaGraphExec_t ex = nullptr;
    const unsigned long long flags = use_node_priority ? cudaGraphInstantiateFlagUseNodePriority : 0;
    FBP_CUDA_CHECK(cudaGraphInstantiateWithFlags(&ex, static_cast<cudaGraph_t>(graph), flags));
    *exec_out = ex;
    return FBP_OK;
}

extern "C" int fbp_graph_launch(void* exec, void* stream) {
    FBP_REQUIRE(exec, FBP_ERR_INVALID, "fbp_graph_launch: null graph");
    FBP_CUDA_CHECK(cudaGraphLaunch(static_cast<cudaGraphExec_t>(exec), as_stream(stream)));
    return FBP_OK;
}

extern "C" int fbp_graph_exec_destroy(void* exec) {
    if (exec) FBP_CUDA_CHECK(cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(exec)));
    return FBP_OK;
}

extern "C" int fbp_fma_probe(float* sink, int32_t blocks, int32_t iters, double* flops_out, void* stream) {
    FBP_REQUIRE(sink && flops_out && blocks > 0 && iters > 0, FBP_ERR_INVALID, "fbp_fma_probe: bad args");
    fma_probe_kernel<<<blocks, 256, 0, as_stream(stream)>>>(sink, iters);
    FBP_LAUNCH_CHECK();
    *flops_out = 2.0 * 8.0 * (double)iters * 256.0 * (double)blocks;
    return FBP_OK;
}

extern "C" int fbp_tanh_probe(const float* x, float* y, int64_t n, void* stream) {
    FBP_REQUIRE(x && y && n >= 0, FBP_ERR_INVALID, "fbp_tanh_probe: bad args");
    if (n == 0) return FBP_OK;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, (int64_t)sm_count() * 8);
    tanh_probe_kernel<<<blocks, 256, 0, as_stream(stream)>>>(x, y, n);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}
