// Collocation points ordered by a Morton cell grid.
//
// The reference draws the points of a batch i.i.d. uniform (sampler
// "uniform", fbpinns/domains.py:113-142) and its loss is their mean, so any
// fixed order of the same points is the same batch.  Ordering them by the
// Morton index of a regular grid of cells (about 64 points per cell) puts
// points that share subdomains next to each other: the interaction lists'
// candidate boxes stay in L1, the subdomain-major sort writes its records
// in runs, and the jet kernels read neighbouring points.
//
// Stable counting sort by cell: count (global atomics) -> exclusive scan of
// the cell counts (one CTA) -> scatter of the point indices to their cell's
// segment (atomics: any order inside the segment) -> per cell, each index's
// rank among the segment's indices restores the input order inside the
// cell, and the points are gathered there.  The result depends only on the
// input: the order is (cell, input index).
#include "common.cuh"

namespace fbp {

namespace {

constexpr int kMaxCellBits = 16;       // at most 2^16 cells
constexpr int kPointsPerCell = 64;     // target mean occupancy
// one CTA of 256 threads scans the cell counts: small enough (about 8K
// registers) to start beside the tensor-core forward, which leaves about 16K
// registers of an SM free, instead of waiting for its CTAs to retire
constexpr int kScanThreads = 256;
constexpr int kOrderWarps = 8;
constexpr int kOrderStage = 256;       // segment length staged in shared memory

struct CellGrid {
    float lo[3];
    float scale[3];  // cells per unit length along each dim
    int bits;        // bits of the cell index per dim
    int xd;
};

// The bits of v at every second (spread2) or third (spread3) position: the
// Morton interleave of 2 or 3 coordinates.
__device__ __forceinline__ uint32_t spread2(uint32_t v) {
    v &= 0x0000FFFFu;
    v = (v | (v << 8)) & 0x00FF00FFu;
    v = (v | (v << 4)) & 0x0F0F0F0Fu;
    v = (v | (v << 2)) & 0x33333333u;
    v = (v | (v << 1)) & 0x55555555u;
    return v;
}
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
    v &= 0x000003FFu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t cell_of(const float* __restrict__ x, int64_t i, const CellGrid& g) {
    const int top = (1 << g.bits) - 1;
    uint32_t c[3] = {0u, 0u, 0u};
#pragma unroll
    for (int d = 0; d < 3; ++d) {  // unrolled over the largest xd: c stays in registers
        if (d < g.xd) {
            const float f = (x[i * g.xd + d] - g.lo[d]) * g.scale[d];
            int v = f >= 0.f ? (int)f : 0;  // NaN and negatives to cell 0
            c[d] = (uint32_t)(v > top ? top : v);
        }
    }
    if (g.xd == 1) return c[0];
    if (g.xd == 2) return spread2(c[0]) | (spread2(c[1]) << 1);
    return spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
}

__global__ void cell_count_kernel(const float* __restrict__ x, int64_t n, CellGrid g, int32_t* __restrict__ key,
                                  int32_t* __restrict__ count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const uint32_t c = cell_of(x, i, g);
        key[i] = (int32_t)c;
        atomicAdd(&count[c], 1);
    }
}

// Exclusive scan of the ncell counts in one CTA (ncell <= 2^16): start[c]
// and the scatter cursors, start[ncell] = the total.
__global__ void __launch_bounds__(kScanThreads) cell_scan_kernel(const int32_t* __restrict__ count, int ncell,
                                                                 int32_t* __restrict__ start,
                                                                 int32_t* __restrict__ cursor) {
    __shared__ int32_t warp_sums[kScanThreads / 32];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int per = (ncell + kScanThreads - 1) / kScanThreads;
    const int b = tid * per, e = min(b + per, ncell);
    int32_t s = 0;
    for (int c = b; c < e; ++c) s += count[c];
    // inclusive scan of the per-thread sums over the CTA
    int32_t v = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_sums[wid] = v;
    __syncthreads();
    if (wid == 0) {
        constexpr int NW = kScanThreads / 32;
        int32_t w = lane < NW ? warp_sums[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        if (lane < NW) warp_sums[lane] = w;
    }
    __syncthreads();
    int32_t run = v - s + (wid > 0 ? warp_sums[wid - 1] : 0);  // exclusive prefix of this thread's range
    for (int c = b; c < e; ++c) {
        start[c] = run;
        cursor[c] = run;
        run += count[c];
    }
    if (tid == kScanThreads - 1) start[ncell] = run;
}

__global__ void cell_scatter_kernel(const int32_t* __restrict__ key, int64_t n, int32_t* __restrict__ cursor,
                                    int32_t* __restrict__ idx) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        idx[atomicAdd(&cursor[key[i]], 1)] = (int32_t)i;
}

// One warp per cell: each index of the cell's segment goes to the position of
// its rank among the segment's indices (distinct), so the segment ends in
// input order; the point is gathered there.
__global__ void __launch_bounds__(kOrderWarps * 32) cell_order_kernel(const int32_t* __restrict__ idx,
                                                                      const int32_t* __restrict__ start, int ncell,
                                                                      const float* __restrict__ x_in, int xd,
                                                                      float* __restrict__ x_out) {
    __shared__ int32_t stage[kOrderWarps][kOrderStage];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t* st = stage[wid];
    for (int c = blockIdx.x * kOrderWarps + wid; c < ncell; c += gridDim.x * kOrderWarps) {
        const int s = start[c], len = start[c + 1] - s;
        if (len <= kOrderStage) {
            for (int f = lane; f < len; f += 32) st[f] = idx[s + f];
            __syncwarp();
            for (int f = lane; f < len; f += 32) {
                const int32_t v = st[f];
                int r = 0;
                for (int h = 0; h < len; ++h) r += st[h] < v;
                for (int d = 0; d < xd; ++d) x_out[(int64_t)(s + r) * xd + d] = x_in[(int64_t)v * xd + d];
            }
            __syncwarp();
            continue;
        }
        // a crowded cell (points outside the grid's box gather in its edge
        // cells): 32 indices at a time, ranked against the segment staged in
        // shared memory chunk by chunk
        for (int f0 = 0; f0 < len; f0 += 32) {
            const int f = f0 + lane;
            const int32_t v = f < len ? idx[s + f] : 0;
            int r = 0;
            for (int h0 = 0; h0 < len; h0 += kOrderStage) {
                const int hl = min(kOrderStage, len - h0);
                __syncwarp();
                for (int h = lane; h < hl; h += 32) st[h] = idx[s + h0 + h];
                __syncwarp();
                if (f < len)
                    for (int h = 0; h < hl; ++h) r += st[h] < v;
            }
            if (f < len)
                for (int d = 0; d < xd; ++d) x_out[(int64_t)(s + r) * xd + d] = x_in[(int64_t)v * xd + d];
        }
        __syncwarp();
    }
}

// Bits of the cell index per dim: about n / 64 cells in all (rounded up to a
// whole number of bits per dim), at most 2^16.
int cell_bits(int64_t n, int xd) {
    int total = 0;
    while (total < kMaxCellBits && ((int64_t)kPointsPerCell << (total + 1)) <= n) ++total;
    int b = (total + xd - 1) / xd;
    while (b * xd > kMaxCellBits) --b;
    return b;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

}  // namespace

}  // namespace fbp

using namespace fbp;

extern "C" size_t fbp_sort_points_scratch_bytes(int64_t n, int32_t xd) {
    if (n < 0 || xd < 1 || xd > 3) return 0;
    const int64_t ncell = (int64_t)1 << (cell_bits(n, xd) * xd);
    return 2 * align256((size_t)n * sizeof(int32_t)) + 3 * align256((size_t)(ncell + 1) * sizeof(int32_t));
}

extern "C" int fbp_sort_points_cells(const float* x_in, int64_t n, int32_t xd, const double* xmin,
                                     const double* xmax, float* x_out, void* scratch, size_t scratch_bytes,
                                     void* stream) {
    FBP_REQUIRE(x_in && x_out && xmin && xmax, FBP_ERR_INVALID, "fbp_sort_points_cells: null pointer");
    FBP_REQUIRE(xd >= 1 && xd <= 3, FBP_ERR_INVALID, "fbp_sort_points_cells: xd=%d not in 1..3", xd);
    FBP_REQUIRE(n >= 0 && n <= INT32_MAX, FBP_ERR_INVALID, "fbp_sort_points_cells: n=%lld out of range",
                (long long)n);
    FBP_REQUIRE(x_in != x_out, FBP_ERR_INVALID, "fbp_sort_points_cells: x_in and x_out must differ");
    if (n == 0) return FBP_OK;
    const size_t need = fbp_sort_points_scratch_bytes(n, xd);
    FBP_REQUIRE(scratch && scratch_bytes >= need, FBP_ERR_INVALID,
                "fbp_sort_points_cells: scratch of %zu bytes, %zu needed", scratch_bytes, need);
    CellGrid g{};
    g.xd = xd;
    g.bits = cell_bits(n, xd);
    for (int d = 0; d < xd; ++d) {
        const double span = xmax[d] - xmin[d];
        FBP_REQUIRE(span > 0, FBP_ERR_INVALID, "fbp_sort_points_cells: empty extent along dim %d", d);
        g.lo[d] = (float)xmin[d];
        g.scale[d] = (float)((double)(1 << g.bits) / span);
    }
    const int ncell = 1 << (g.bits * xd);
    char* p = static_cast<char*>(scratch);
    int32_t* key = reinterpret_cast<int32_t*>(p);
    p += align256((size_t)n * sizeof(int32_t));
    int32_t* idx = reinterpret_cast<int32_t*>(p);
    p += align256((size_t)n * sizeof(int32_t));
    int32_t* count = reinterpret_cast<int32_t*>(p);
    p += align256((size_t)(ncell + 1) * sizeof(int32_t));
    int32_t* start = reinterpret_cast<int32_t*>(p);
    p += align256((size_t)(ncell + 1) * sizeof(int32_t));
    int32_t* cursor = reinterpret_cast<int32_t*>(p);
    cudaStream_t st = as_stream(stream);
    FBP_CUDA_CHECK(cudaMemsetAsync(count, 0, (size_t)ncell * sizeof(int32_t), st));
    int blocks = (int)((n + 255) / 256);
    if (blocks > sm_count() * 8) blocks = sm_count() * 8;
    cell_count_kernel<<<blocks, 256, 0, st>>>(x_in, n, g, key, count);
    FBP_LAUNCH_CHECK();
    cell_scan_kernel<<<1, kScanThreads, 0, st>>>(count, ncell, start, cursor);
    FBP_LAUNCH_CHECK();
    cell_scatter_kernel<<<blocks, 256, 0, st>>>(key, n, cursor, idx);
    FBP_LAUNCH_CHECK();
    int oblocks = (ncell + kOrderWarps - 1) / kOrderWarps;
    if (oblocks > sm_count() * 8) oblocks = sm_count() * 8;
    cell_order_kernel<<<oblocks, kOrderWarps * 32, 0, st>>>(idx, start, ncell, x_in, xd, x_out);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}
