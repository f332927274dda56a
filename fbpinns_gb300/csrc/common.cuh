// Shared helpers of libfbpgpu: status handling, launch checks, jet layout.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "../../include/fbpgpu.h"

namespace fbp {

// Thread-local message for fbp_last_error().
void set_error(const char* fmt, ...);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

#define FBP_REQUIRE(cond, code, ...)      \
    do {                                  \
        if (!(cond)) {                    \
            ::fbp::set_error(__VA_ARGS__); \
            return (code);                \
        }                                 \
    } while (0)

#define FBP_CUDA_CHECK(expr)                                                           \
    do {                                                                               \
        cudaError_t e_ = (expr);                                                       \
        if (e_ != cudaSuccess) {                                                       \
            ::fbp::set_error("%s failed: %s (%s:%d)", #expr, cudaGetErrorString(e_), \
                             __FILE__, __LINE__);                                      \
            return FBP_ERR_CUDA;                                                       \
        }                                                                              \
    } while (0)

#define FBP_LAUNCH_CHECK() FBP_CUDA_CHECK(cudaGetLastError())

constexpr int kSM = 152;  // GB300 SM count (grid sizing hint; queried at run time too)

// Elements per tile of the exclusive int32 scan (takes.cu): its scratch holds
// one sum per tile plus the total.
constexpr int kScanTile = 2048;

// Per-device caches (kernel attributes, occupancy-sized grids) are indexed by
// the current device, 0 .. FBP_MAX_DEVICES - 1.
constexpr int FBP_MAX_DEVICES = 64;
int current_device();
int sm_count();

__host__ __device__ constexpr int popc_const(int v) {
    return v == 0 ? 0 : (v & 1) + popc_const(v >> 1);
}

// Second-derivative part of a jet, from the d2mask: bits 0-2 name the dims
// whose pure second derivatives are needed.  The dims of the group (all of
// them with FBP_D2_LAPLACIAN, bit 3; else the dims named by bits 4-6, see
// FBP_D2_GROUP) share one slot that holds the sum of their second
// derivatives (a Laplacian, propagated directly as in the forward-Laplacian
// scheme); every other masked dim has a slot of its own.  Slot order: the
// group's slot first, then the single dims ascending.
__host__ __device__ constexpr int d2_group(int d2) {
    return (d2 & FBP_D2_LAPLACIAN) ? (d2 & 7) : ((d2 >> 4) & 7 & d2);
}
__host__ __device__ constexpr int d2_singles(int d2) { return d2 & 7 & ~d2_group(d2); }
__host__ __device__ constexpr bool d2_lap(int d2) { return d2_group(d2) != 0; }
__host__ __device__ constexpr int d2_slots(int d2) { return (d2_group(d2) ? 1 : 0) + popc_const(d2_singles(d2)); }

// Jet layout: [u, d/dx_0..d/dx_{XD-1}, then the second-derivative slots: one
// per bit i of the d2mask ascending, or the single Laplacian slot].
__host__ __device__ constexpr int jet_size(int xd, int d2) { return 1 + xd + d2_slots(d2); }

// Index of the s-th set bit of mask among bits 0..7 (0 when there is none).
__host__ __device__ constexpr int nth_bit(int mask, int s) {
    int c = 0;
    for (int d = 0; d < 8; ++d)
        if ((mask >> d) & 1) {
            if (c == s) return d;
            ++c;
        }
    return 0;
}

// Row stride (floats) of the per-pair and per-slot jet records [first J | second J]:
// 2J rounded up to a multiple of 4 so that rows can be moved as float4.
__host__ __device__ constexpr int rec_stride(int J) { return (2 * J + 3) / 4 * 4; }

// Compile-time table of the set bits of a mask (up to 3): DimsOf<M>::get(s) is
// the s-th set bit, folded to a constant when s is a constant.
template <int M>
struct DimsOf {
    static constexpr int d0 = nth_bit(M, 0), d1 = nth_bit(M, 1), d2 = nth_bit(M, 2);
    __host__ __device__ static constexpr int get(int s) { return s == 0 ? d0 : (s == 1 ? d1 : d2); }
};

// Dims whose pure second derivatives second-derivative slot s of a d2mask sums
// (the group for the group's slot, else one dim).
template <int D2>
__host__ __device__ constexpr int d2_slot_dims(int s) {
    return d2_group(D2) ? (s == 0 ? d2_group(D2) : (1 << DimsOf<d2_singles(D2)>::get(s - 1)))
                        : (1 << DimsOf<D2 & 7>::get(s));
}

// tanh from the identity tanh|x| = (1 - e) / (1 + e), e = exp(-2|x|), with the
// __expf / __fdividef intrinsics and the sign restored.  e lies in (0, 1], so
// nothing overflows; the absolute error is about 1e-7 over the whole line
// (checked against torch.tanh by tests/test_gpu_step.py::test_fast_tanh_error).
__device__ __forceinline__ float tanh_fast(float x) {
    const float e = __expf(-2.0f * fabsf(x));
    return copysignf(__fdividef(1.0f - e, 1.0f + e), x);
}

inline int jet_size_rt(int xd, int d2) { return 1 + xd + d2_slots(d2); }

}  // namespace fbp
