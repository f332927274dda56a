// fbp_scan_i32_noalloc: the exclusive prefix scan of fbp_scan_i32 for callers
// that cannot allocate device memory and so cannot hand the library a scratch
// buffer — for example code that embeds the interaction-list build inside a
// host framework that owns every device allocation through its own arena, or
// a real-time loop where allocation calls are forbidden after start-up.
//
// The scan's only scratch (one int32 sum per 2048-element tile, plus the
// total) lives in a file-scope __device__ array of fixed size.  Every GPU that
// loads this library holds that array (about 32 KiB: 8193 int32) until the
// process exits.
#include <mutex>

#include "common.cuh"

namespace fbp {
// Defined in takes.cu: the three-kernel scan over a caller-given sums buffer,
// and the number of scratch bytes it needs for n elements.
int scan_launch(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, cudaStream_t st);
size_t scan_scratch(int64_t n);
}  // namespace fbp

namespace {

// Tile sums for up to FBP_SCAN_NOALLOC_MAX_N elements: ceil(n / tile) + 1 int32.
constexpr int64_t kMaxN = FBP_SCAN_NOALLOC_MAX_N;
constexpr int64_t kSums = (kMaxN + fbp::kScanTile - 1) / fbp::kScanTile + 1;

static __device__ __align__(256) int32_t g_scan_sums[kSums];

// Device address of g_scan_sums per device ordinal.  In host code the name
// g_scan_sums is only a host-side stand-in for the device array, so the real
// address is looked up once per device with that device current.  A
// cudaDeviceReset makes the cached address stale: the entry is cleared when a
// launch through it fails, and a caller that resets a device must not call
// this function on it again (the library's other entry points are unaffected).
constexpr int kMaxDevices = 64;
std::mutex g_mu;
int32_t* g_addr[kMaxDevices] = {};

int sums_address(int32_t** out) {
    int dev = -1;
    FBP_CUDA_CHECK(cudaGetDevice(&dev));
    FBP_REQUIRE(dev >= 0 && dev < kMaxDevices, FBP_ERR_UNSUPPORTED,
                "fbp_scan_i32_noalloc: device ordinal %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        FBP_CUDA_CHECK(cudaGetSymbolAddress(&p, g_scan_sums));
        g_addr[dev] = static_cast<int32_t*>(p);
    }
    *out = g_addr[dev];
    return FBP_OK;
}

}  // namespace

extern "C" int fbp_scan_i32_noalloc(const int32_t* in, int32_t* out, int64_t n, void* stream) {
    FBP_REQUIRE(out && (in || n == 0), FBP_ERR_INVALID, "fbp_scan_i32_noalloc: null pointer");
    FBP_REQUIRE(n >= 0, FBP_ERR_INVALID, "fbp_scan_i32_noalloc: n=%lld < 0", (long long)n);
    FBP_REQUIRE(n <= kMaxN, FBP_ERR_CAPACITY,
                "fbp_scan_i32_noalloc: n=%lld exceeds the built-in maximum of %lld elements "
                "(use fbp_scan_i32 with a caller-provided scratch buffer)",
                (long long)n, (long long)kMaxN);
    FBP_REQUIRE(fbp::scan_scratch(n) <= sizeof(int32_t) * (size_t)kSums, FBP_ERR_CAPACITY,
                "fbp_scan_i32_noalloc: scratch for n=%lld exceeds the built-in array", (long long)n);
    int32_t* sums = nullptr;
    const int rc = sums_address(&sums);
    if (rc) return rc;
    // Nothing in the array has to start at zero: each call writes every tile
    // sum (and the total) before reading it.
    const int lrc = fbp::scan_launch(in, out, n, sums, fbp::as_stream(stream));
    if (lrc != FBP_OK) {  // look the address up again on the next call
        int dev = -1;
        if (cudaGetDevice(&dev) == cudaSuccess && dev >= 0 && dev < kMaxDevices) {
            std::lock_guard<std::mutex> lock(g_mu);
            g_addr[dev] = nullptr;
        }
    }
    return lrc;
}
