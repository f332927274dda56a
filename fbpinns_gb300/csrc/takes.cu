// Interaction lists ("takes"): point-in-box count/fill over a uniform cell
// grid, prefix scans, compaction, the stable subdomain-major pair sort and the
// work queue.  All integer work; results are bit-exact with the reference's
// inside_points / get_inputs (fbpinns/decompositions_base.py:24-84,
// fbpinns/trainers.py:332-419).
#include <algorithm>

#include "common.cuh"

namespace fbp {

// ---------------------------------------------------------------------------
// cell lookup (must match fbpinns_gb300/decompositions.py:build_cell_grid)
// ---------------------------------------------------------------------------
__device__ __forceinline__ int cell_coord(float v, double lo, double inv_h, int nc) {
    const double t = __dmul_rn(__dsub_rn((double)v, lo), inv_h);
    double f = floor(t);
    if (!(f >= 0.0)) f = 0.0;  // also maps NaN to cell 0
    if (f > (double)(nc - 1)) f = (double)(nc - 1);
    return (int)f;
}

template <int XD>
__device__ __forceinline__ int cell_of(const float* xp, const fbp_boxes& b) {
    int c = cell_coord(xp[XD - 1], b.lo[XD - 1], b.inv_h[XD - 1], b.ncell[XD - 1]);
#pragma unroll
    for (int d = XD - 2; d >= 0; --d) c = c * b.ncell[d] + cell_coord(xp[d], b.lo[d], b.inv_h[d], b.ncell[d]);
    return c;
}

template <int XD>
__device__ __forceinline__ bool inside_box(const float* xp, const float* __restrict__ xmins,
                                           const float* __restrict__ xmaxs, int j) {
    bool in = true;
#pragma unroll
    for (int d = 0; d < XD; ++d) {
        const float v = xp[d];
        in = in && (v >= xmins[j * XD + d]) && (v <= xmaxs[j * XD + d]);
    }
    return in;
}

template <int XD>
__global__ void inside_count_kernel(const float* __restrict__ x, int64_t n, fbp_boxes b,
                                    int32_t* __restrict__ pt_count, int32_t* __restrict__ pt_nlvl,
                                    uint64_t* __restrict__ pt_lvl, int32_t* __restrict__ model_count,
                                    uint64_t* __restrict__ pt_hit, int32_t* __restrict__ pt_cand) {
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n;
         p += (int64_t)gridDim.x * blockDim.x) {
        float xp[XD];
#pragma unroll
        for (int d = 0; d < XD; ++d) xp[d] = x[p * XD + d];
        const int c = cell_of<XD>(xp, b);
        const int e0 = b.cell_start[c], e1 = b.cell_start[c + 1];
        int cnt = 0;
        uint64_t lvl = 0, hit = 0;
        for (int e = e0; e < e1; ++e) {
            const int j = b.cell_boxes[e];
            if (b.select && !b.select[j]) continue;
            if (inside_box<XD>(xp, b.xmins, b.xmaxs, j)) {
                ++cnt;
                lvl |= 1ull << (b.pou[j] & 63);
                if (e - e0 < 64) hit |= 1ull << (e - e0);
                if (model_count) atomicAdd(&model_count[j], 1);
            }
        }
        pt_count[p] = cnt;
        if (pt_nlvl) pt_nlvl[p] = __popcll(lvl);
        if (pt_lvl) pt_lvl[p] = lvl;
        // hits as a mask over the cell's candidate list (cells of <= 64 candidates)
        if (pt_hit) pt_hit[p] = hit;
        if (pt_cand) pt_cand[p] = e1 - e0 <= 64 ? e0 : -1;
    }
}

// Fill: one thread per point takes its hits from the count pass's candidate
// mask (or, for cells of more than 64 candidates or without the mask, tests
// the candidates again; the box arrays are small and stay in L1); a warp's 32
// consecutive points own one contiguous
// range of the point-major pair arrays, so their hits are staged in shared
// memory and the warp writes the range out coalesced.  A warp whose range
// exceeds its staging space writes its points' pairs directly.  A staged pair
// is one int32: box id << 11 | POU level << 5 | point within the warp
// (box ids below 2^21, checked by the caller).
constexpr int FILL_WARPS = 8;     // warps per CTA
constexpr int FILL_STAGE = 1280;  // staged pairs per warp
constexpr int64_t FILL_MAX_M = int64_t(1) << 21;

template <int XD>
__global__ void __launch_bounds__(FILL_WARPS * 32)
    inside_fill_kernel(const float* __restrict__ x, int64_t n, fbp_boxes b, const int32_t* __restrict__ pt_off,
                       const int32_t* __restrict__ np_off, const uint64_t* __restrict__ pt_lvl,
                       const uint64_t* __restrict__ pt_hit, const int32_t* __restrict__ pt_cand,
                       int32_t* __restrict__ n_take, int32_t* __restrict__ m_take, int32_t* __restrict__ p_take,
                       int32_t* __restrict__ np_take, int64_t s_cap, int64_t u_cap, int32_t* __restrict__ status) {
    __shared__ int32_t stage[FILL_WARPS][FILL_STAGE];
    __shared__ uint64_t s_lvl[FILL_WARPS][32];
    __shared__ int32_t s_ubase[FILL_WARPS][32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int64_t nwarps = (int64_t)gridDim.x * FILL_WARPS;
    for (int64_t p0 = ((int64_t)blockIdx.x * FILL_WARPS + w) * 32; p0 < n; p0 += nwarps * 32) {
        const int64_t p = p0 + lane;
        const bool valid = p < n;
        const int np = (int)min((int64_t)32, n - p0);
        const int64_t wb = pt_off[p0], we = pt_off[p0 + np];
        const int64_t total = we - wb;
        const bool staged = total <= FILL_STAGE && b.m <= FILL_MAX_M;
        int64_t base = 0;
        int32_t ubase = 0;
        uint64_t lvl = 0;
        if (valid) {
            base = pt_off[p];
            ubase = np_off[p];
            lvl = pt_lvl[p];
        }
        s_lvl[w][lane] = lvl;
        s_ubase[w][lane] = ubase;
        if (valid) {
            int cand = -1;
            uint64_t hit = 0;
            if (pt_hit && pt_cand) {
                cand = pt_cand[p];
                hit = pt_hit[p];
            }
            int e = 0, e1 = 0;
            float xp[XD];
            if (cand < 0) {
#pragma unroll
                for (int d = 0; d < XD; ++d) xp[d] = x[p * XD + d];
                const int c = cell_of<XD>(xp, b);
                e = b.cell_start[c];
                e1 = b.cell_start[c + 1];
            }
            int64_t k = 0;
            // the point's k-th pair (box j at POU level lv): staged or written directly
            auto emit = [&](int j, int lv) {
                const int64_t q = base + k - wb;
                if (staged) {
                    if (q >= 0 && q < total)
                        stage[w][q] = (int32_t)(((uint32_t)j << 11) | (uint32_t)(lv << 5) | (uint32_t)lane);
                    else
                        atomicOr(status, FBP_STATUS_BAD_INDEX);
                } else {
                    const int64_t o = base + k;
                    if (o < s_cap) {
                        const uint64_t below = lv ? (lvl & ((1ull << lv) - 1ull)) : 0ull;
                        n_take[o] = (int32_t)p;
                        m_take[o] = j;
                        p_take[o] = ubase + __popcll(below);
                    } else {
                        atomicOr(status, FBP_STATUS_PAIR_OVERFLOW);
                    }
                }
                ++k;
            };
            if (cand >= 0) {
                // hits from the mask, four at a time so that their loads overlap
                while (hit) {
                    int jj[4], ll[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        jj[u] = -1;
                        if (hit) {
                            jj[u] = b.cell_boxes[cand + __ffsll((long long)hit) - 1];
                            hit &= hit - 1;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) ll[u] = jj[u] >= 0 ? (b.pou[jj[u]] & 63) : 0;
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (jj[u] >= 0) emit(jj[u], ll[u]);
                }
            } else {
                for (; e < e1; ++e) {
                    const int j = b.cell_boxes[e];
                    if ((!b.select || b.select[j]) && inside_box<XD>(xp, b.xmins, b.xmaxs, j)) emit(j, b.pou[j] & 63);
                }
            }
            // unique (point, level) slots in ascending level order
            const int nl = __popcll(lvl);
            for (int r = 0; r < nl; ++r) {
                const int64_t o = (int64_t)ubase + r;
                if (o < u_cap)
                    np_take[o] = (int32_t)p;
                else
                    atomicOr(status, FBP_STATUS_SLOT_OVERFLOW);
            }
        }
        __syncwarp();
        if (staged) {
            for (int64_t q = lane; q < total; q += 32) {
                const int32_t v = stage[w][q];
                const int idx = v & 31, lv = (v >> 5) & 63;
                const int64_t o = wb + q;
                if (o < s_cap) {
                    const uint64_t l = s_lvl[w][idx];
                    const uint64_t below = lv ? (l & ((1ull << lv) - 1ull)) : 0ull;
                    n_take[o] = (int32_t)(p0 + idx);
                    m_take[o] = (int32_t)((uint32_t)v >> 11);
                    p_take[o] = s_ubase[w][idx] + __popcll(below);
                } else {
                    atomicOr(status, FBP_STATUS_PAIR_OVERFLOW);
                }
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Exclusive scan of int32 (3 kernels, deterministic)
// ---------------------------------------------------------------------------
constexpr int SCAN_T = 256, SCAN_V = 8, SCAN_TILE = SCAN_T * SCAN_V;
static_assert(SCAN_TILE == kScanTile, "the scan tile is shared with the allocation-free scan");

__device__ __forceinline__ int block_exclusive_scan(int v, int* smem_warp, int& total) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) smem_warp[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        int w = lane < nw ? smem_warp[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) smem_warp[lane] = wi - w;
        if (lane == nw - 1) smem_warp[32] = wi;
    }
    __syncthreads();
    total = smem_warp[32];
    const int r = incl - v + smem_warp[wid];
    __syncthreads();
    return r;
}

__global__ void scan_reduce_kernel(const int32_t* __restrict__ in, int64_t n, int32_t* __restrict__ sums) {
    __shared__ int sw[33];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int s = 0;
#pragma unroll
    for (int v = 0; v < SCAN_V; ++v) {
        const int64_t i = base + (int64_t)v * SCAN_T + threadIdx.x;
        if (i < n) s += in[i];
    }
    int tot;
    block_exclusive_scan(s, sw, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// single block: exclusive scan of the tile sums in place, total at sums[nb]
__global__ void scan_sums_kernel(int32_t* __restrict__ sums, int64_t nb) {
    __shared__ int sw[33];
    int carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int64_t i = b0 + threadIdx.x;
        const int v = i < nb ? sums[i] : 0;
        int tot;
        const int ex = block_exclusive_scan(v, sw, tot);
        if (i < nb) sums[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) sums[nb] = carry;
}

// Tiles up to which a down-sweep block adds the earlier tiles' sums itself
// (no scan of the sums in between: two launches per scan instead of three;
// the loads grow with the square of the tile count).
constexpr int64_t SCAN_FUSED_TILES = 4096;

// fused: the block's offset is the sum of sums[0 .. blockIdx.x) (tile totals,
// added here) and the last block writes the total; else sums holds the
// scanned offsets and the total at sums[nb].
__global__ void scan_down_kernel(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ sums,
                                 int64_t nb, int32_t* __restrict__ out, bool fused) {
    __shared__ int sw[33];
    __shared__ int tile[SCAN_TILE];
    const int64_t base = (int64_t)blockIdx.x * SCAN_TILE;
    int prefix = 0;
    if (fused) {
        int a = 0;
        for (int64_t i = threadIdx.x; i < (int64_t)blockIdx.x; i += blockDim.x) a += sums[i];
        block_exclusive_scan(a, sw, prefix);  // prefix = the block total of a
    } else {
        prefix = sums[blockIdx.x];
    }
    // blocked arrangement: thread t owns items [t*V, t*V+V) of the tile
#pragma unroll
    for (int v = 0; v < SCAN_V; ++v) {
        const int64_t i = base + (int64_t)v * SCAN_T + threadIdx.x;
        tile[v * SCAN_T + threadIdx.x] = i < n ? in[i] : 0;
    }
    __syncthreads();
    int loc[SCAN_V];
    int s = 0;
#pragma unroll
    for (int v = 0; v < SCAN_V; ++v) {
        loc[v] = s;
        s += tile[threadIdx.x * SCAN_V + v];
    }
    int tot;
    const int ex = block_exclusive_scan(s, sw, tot);
    const int off = prefix + ex;
#pragma unroll
    for (int v = 0; v < SCAN_V; ++v) tile[threadIdx.x * SCAN_V + v] = off + loc[v];
    __syncthreads();
#pragma unroll
    for (int v = 0; v < SCAN_V; ++v) {
        const int64_t i = base + (int64_t)v * SCAN_T + threadIdx.x;
        if (i < n) out[i] = tile[v * SCAN_T + threadIdx.x];
    }
    if (threadIdx.x == 0) {
        if (fused && blockIdx.x == nb - 1) out[n] = prefix + tot;
        if (!fused && blockIdx.x == 0) out[n] = sums[nb];
    }
}

int scan_launch(const int32_t* in, int32_t* out, int64_t n, int32_t* sums, cudaStream_t st) {
    const int64_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 0) {
        FBP_CUDA_CHECK(cudaMemsetAsync(out, 0, sizeof(int32_t), st));
        return FBP_OK;
    }
    const bool fused = nb <= SCAN_FUSED_TILES;
    scan_reduce_kernel<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, sums);
    FBP_LAUNCH_CHECK();
    if (!fused) {
        scan_sums_kernel<<<1, 1024, 0, st>>>(sums, nb);
        FBP_LAUNCH_CHECK();
    }
    scan_down_kernel<<<(unsigned)nb, SCAN_T, 0, st>>>(in, n, sums, nb, out, fused);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

size_t scan_scratch(int64_t n) { return (size_t)(((n + SCAN_TILE - 1) / SCAN_TILE) + 1) * sizeof(int32_t); }

// ---------------------------------------------------------------------------
// gather / compaction
// ---------------------------------------------------------------------------
__global__ void gather_i32_kernel(const int32_t* __restrict__ in, int64_t n, const int32_t* __restrict__ cnt,
                                  const int32_t* __restrict__ inv, int32_t* __restrict__ out) {
    const int64_t lim = cnt ? (int64_t)(*cnt) < n ? (int64_t)(*cnt) : n : n;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < lim;
         i += (int64_t)gridDim.x * blockDim.x)
        out[i] = inv[in[i]];
}

__global__ void flag_to_count_kernel(const int32_t* __restrict__ flag, int64_t n, int32_t* __restrict__ c) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        c[i] = flag[i] != 0;
}

__global__ void compact_kernel(const int32_t* __restrict__ flag, const int32_t* __restrict__ off, int64_t n,
                               int32_t* __restrict__ out, int32_t* __restrict__ count) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x)
        if (flag[i]) out[off[i]] = (int32_t)i;
    if (blockIdx.x == 0 && threadIdx.x == 0) *count = off[n];
}

// ---------------------------------------------------------------------------
// Stable counting sort of pairs by subdomain.
// Pass 1 (one warp per chunk of CH pairs): per-chunk histogram, written
// bucket-major hist[j * nchunks + chunk].  Scan.  Pass 2: each warp re-reads
// its chunk in order and scatters with ranks from __match_any_sync, keeping
// per-bucket running counts in shared memory: stable and deterministic.
// ---------------------------------------------------------------------------
// Pairs per chunk of the subdomain sort, from the pair capacity: each chunk
// costs O(m) in bucket tables and histogram entries besides its pairs, so
// larger chunks pay while there are enough of them to fill the GPU (about
// four per SM of a GB300; measured with cell-ordered batches of 9.4e6 pairs:
// 4096 0.382 ms, 8192 0.364, 16384 0.33 for the whole list build; 2.3e6 pairs:
// 4096 33.6 us, 16384 55.4 us for the scatter).  A function of s_cap only, so
// that the scratch size and the launches agree; the order does not depend on it.
static int64_t sort_chunk(int64_t s_cap) {
    int64_t ch = 4096;
    while (ch < 16384 && s_cap / (2 * ch) >= 4 * kSM) ch *= 2;
    return ch;
}

// With pt_keep, a pair whose point has pt_keep[point] == 0 is left out (its
// key reads as -1, outside every bucket); the kept pairs keep their order.
__device__ __forceinline__ int kept_key(const int32_t* __restrict__ key, const int32_t* __restrict__ n_take,
                                        const uint8_t* __restrict__ pt_keep, int64_t i) {
    const int k = key[i];
    return (pt_keep && !pt_keep[n_take[i]]) ? -1 : k;
}

__global__ void sort_hist_kernel(const int32_t* __restrict__ key, const int32_t* __restrict__ n_take,
                                 const uint8_t* __restrict__ pt_keep, const int32_t* __restrict__ s_dev,
                                 int64_t s_cap, int64_t m, int64_t nchunks, int64_t chn,
                                 int32_t* __restrict__ hist) {
    extern __shared__ int cnt[];
    const int64_t s = min((int64_t)*s_dev, s_cap);
    for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        for (int64_t j = threadIdx.x; j < m; j += blockDim.x) cnt[j] = 0;
        __syncthreads();
        const int64_t b0 = ch * chn, b1 = min(b0 + chn, s);
        for (int64_t i0 = b0; i0 < b1; i0 += (int64_t)blockDim.x * 8) {  // loads first, then the counts
            int kk[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t i = i0 + (int64_t)u * blockDim.x + threadIdx.x;
                kk[u] = i < b1 ? kept_key(key, n_take, pt_keep, i) : -1;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (kk[u] >= 0 && kk[u] < m) atomicAdd(&cnt[kk[u]], 1);
        }
        __syncthreads();
        for (int64_t j = threadIdx.x; j < m; j += blockDim.x) hist[j * nchunks + ch] = cnt[j];
        __syncthreads();
    }
}

constexpr int SCATTER_U = 16;  // 32-pair rows whose loads are issued together
#ifndef FBP_SCATTER_W
#define FBP_SCATTER_W 4
#endif
constexpr int SCATTER_W = FBP_SCATTER_W;  // warps per chunk (fewer when their bucket tables do not fit)

// One CTA of W <= SCATTER_W warps per chunk of chn pairs (point-major).
// Each warp first counts the buckets of its part of the chunk; the running
// offsets of warp w start at the chunk's bucket offset plus the counts of
// warps < w, so the warps then place their quarters independently and the
// result is the same stable order as one pass over the chunk.  A point's
// pairs have distinct boxes, so each row of 32 pairs is placed point by
// point: the lanes of one point read and advance distinct bucket counters,
// and the points of the row follow each other in order (no key matching).
__global__ void __launch_bounds__(SCATTER_W * 32)
    sort_scatter_kernel(const int32_t* __restrict__ key, const int32_t* __restrict__ n_take,
                        const int32_t* __restrict__ p_take, const uint8_t* __restrict__ pt_keep,
                        const int32_t* __restrict__ s_dev, int64_t s_cap, int64_t m, int64_t nchunks,
                        int64_t chn, const int32_t* __restrict__ hoff, int4* __restrict__ sd_rec) {
    extern __shared__ int run[];  // [W][m]: per-warp counts, then running offsets
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, W = blockDim.x >> 5;
    int* myrun = run + (int64_t)w * m;
    const int64_t s = min((int64_t)*s_dev, s_cap);
    const int64_t SUB = (chn + W - 1) / W;
    for (int64_t ch = blockIdx.x; ch < nchunks; ch += gridDim.x) {
        for (int64_t j = threadIdx.x; j < m * W; j += blockDim.x) run[j] = 0;
        __syncthreads();
        const int64_t c0 = ch * chn, c1 = min(c0 + chn, s);
        const int64_t b0 = min(c0 + (int64_t)w * SUB, c1), b1 = min(b0 + SUB, c1);
        for (int64_t i0 = b0; i0 < b1; i0 += 32 * 8) {  // loads of 8 rows first, then the counts
            int kk[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t i = i0 + u * 32 + lane;
                kk[u] = i < b1 ? kept_key(key, n_take, pt_keep, i) : -1;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (kk[u] >= 0 && kk[u] < m) atomicAdd(&myrun[kk[u]], 1);
        }
        __syncthreads();
        for (int64_t j0 = threadIdx.x; j0 < m; j0 += (int64_t)blockDim.x * 8) {
            int oo[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t j = j0 + (int64_t)u * blockDim.x;
                oo[u] = j < m ? hoff[j * nchunks + ch] : 0;
            }
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int64_t j = j0 + (int64_t)u * blockDim.x;
                if (j >= m) break;
                int o = oo[u];
                for (int v = 0; v < W; ++v) {
                    const int c = run[(int64_t)v * m + j];
                    run[(int64_t)v * m + j] = o;
                    o += c;
                }
            }
        }
        __syncthreads();
        for (int64_t i0 = b0; i0 < b1; i0 += 32 * SCATTER_U) {
            int kk[SCATTER_U], nn[SCATTER_U], pp[SCATTER_U];
#pragma unroll
            for (int u = 0; u < SCATTER_U; ++u) {
                const int64_t i = i0 + u * 32 + lane;
                kk[u] = -1;
                nn[u] = -1;
                pp[u] = 0;
                if (i < b1) {
                    kk[u] = key[i];
                    nn[u] = n_take[i];
                    pp[u] = p_take[i];
                    if (pt_keep && !pt_keep[nn[u]]) kk[u] = -1;
                }
            }
#pragma unroll
            for (int u = 0; u < SCATTER_U; ++u) {
                const int64_t i = i0 + u * 32 + lane;
                const int k = kk[u];
                const bool ok = k >= 0 && k < m;
                unsigned todo = __ballot_sync(0xffffffffu, i < b1);
                while (todo) {
                    // the row's next point: the lanes holding it form one group
                    const int pt = __shfl_sync(0xffffffffu, nn[u], __ffs(todo) - 1);
                    const unsigned grp = __ballot_sync(0xffffffffu, (todo >> lane & 1u) && nn[u] == pt);
                    if ((grp >> lane & 1u) && ok) {
                        const int o = myrun[k];
                        myrun[k] = o + 1;
                        sd_rec[o] = make_int4((int32_t)i, pt, pp[u], 0);
                    }
                    todo &= ~grp;
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
}

// sd_start[j] = hoff[j * nchunks] (start of bucket j), sd_start[m] = s
__global__ void sort_starts_kernel(const int32_t* __restrict__ hoff, int64_t m, int64_t nchunks,
                                   int32_t* __restrict__ sd_start) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j <= m;
         j += (int64_t)gridDim.x * blockDim.x)
        sd_start[j] = hoff[j * nchunks];
}

// ---------------------------------------------------------------------------
// work queue
// ---------------------------------------------------------------------------
__global__ void work_count_kernel(const int32_t* __restrict__ sd_start, int64_t m, const uint8_t* __restrict__ sel,
                                  int chunk, int32_t* __restrict__ nit) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m;
         j += (int64_t)gridDim.x * blockDim.x) {
        const int c = sd_start[j + 1] - sd_start[j];
        nit[j] = (sel && !sel[j]) ? 0 : (c + chunk - 1) / chunk;
    }
}

// one warp per subdomain: the lanes write its items (a subdomain holding all
// points has hundreds of them)
__global__ void work_fill_kernel(const int32_t* __restrict__ sd_start, int64_t m, const int32_t* __restrict__ ioff,
                                 int chunk, int32_t* __restrict__ items, int32_t* __restrict__ item_start,
                                 int32_t* __restrict__ n_items, int64_t cap, int32_t* __restrict__ status) {
    const int lane = threadIdx.x & 31;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t j = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; j < m; j += nw) {
        const int i0 = ioff[j], i1 = ioff[j + 1];
        const int b = sd_start[j], e = sd_start[j + 1];
        for (int it = i0 + lane; it < i1; it += 32) {
            if (it >= cap) {
                atomicOr(status, FBP_STATUS_ITEM_OVERFLOW);
                break;
            }
            const int beg = b + (it - i0) * chunk;
            items[3 * (int64_t)it + 0] = (int32_t)j;
            items[3 * (int64_t)it + 1] = beg;
            items[3 * (int64_t)it + 2] = min(chunk, e - beg);
        }
        if (lane == 0) {
            item_start[j] = min((int64_t)i0, cap);
            if (j == m - 1) {
                item_start[m] = min((int64_t)i1, cap);
                *n_items = (int32_t)min((int64_t)i1, cap);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// scheduled training: the points and subdomain states of one active mask
// ---------------------------------------------------------------------------
// Per point: kept when one of its boxes has raw state 1; the boxes of a kept
// point are marked in state[] (a store of 1 by any of its points); kept
// points are counted into *n_keep (warp sums, one atomic per warp).
__global__ void train_mark_kernel(const int32_t* __restrict__ pt_off, const int32_t* __restrict__ m_take, int64_t n,
                                  int64_t s_cap, const uint8_t* __restrict__ raw, uint8_t* __restrict__ pt_keep,
                                  uint8_t* __restrict__ state, int32_t* __restrict__ n_keep) {
    for (int64_t p0 = blockIdx.x * (int64_t)blockDim.x; p0 < n; p0 += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = p0 + threadIdx.x;
        bool keep = false;
        if (p < n) {
            const int64_t e0 = min((int64_t)pt_off[p], s_cap), e1 = min((int64_t)pt_off[p + 1], s_cap);
            for (int64_t e = e0; e < e1 && !keep; ++e) keep = raw[m_take[e]] == 1;
            pt_keep[p] = keep ? 1 : 0;
            if (keep)
                for (int64_t e = e0; e < e1; ++e) state[m_take[e]] = 1;
        }
        const unsigned b = __ballot_sync(0xffffffffu, keep);
        if ((threadIdx.x & 31) == 0 && b) atomicAdd(n_keep, __popc(b));
    }
}

// Per box: 1 (trained) where it holds a kept point and its raw state is 0 or
// 1, 2 (fixed) where it holds one and its raw state is 2, else 0; active[j]
// = state[j] == 1 (the adjoint's selection and Adam's mask).
__global__ void train_state_kernel(const uint8_t* __restrict__ raw, int64_t m, uint8_t* __restrict__ state,
                                   uint8_t* __restrict__ active) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < m; j += (int64_t)gridDim.x * blockDim.x) {
        const uint8_t v = state[j] ? (raw[j] == 2 ? 2 : 1) : 0;
        state[j] = v;
        active[j] = v == 1 ? 1 : 0;
    }
}

static int grid_for(int64_t n, int threads, int per_sm = 16) {
    int64_t b = (n + threads - 1) / threads;
    const int64_t cap = (int64_t)sm_count() * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (int)b;
}

static int check_boxes(const fbp_boxes* b) {
    FBP_REQUIRE(b, FBP_ERR_INVALID, "boxes: null");
    FBP_REQUIRE(b->xd >= 1 && b->xd <= FBP_MAX_XD, FBP_ERR_UNSUPPORTED, "boxes: xd=%d not in 1..3", b->xd);
    FBP_REQUIRE(b->xmins && b->xmaxs && b->pou && b->cell_start && b->cell_boxes, FBP_ERR_INVALID,
                "boxes: null device pointer");
    for (int d = 0; d < b->xd; ++d)
        FBP_REQUIRE(b->ncell[d] >= 1, FBP_ERR_INVALID, "boxes: ncell[%d]=%d", d, b->ncell[d]);
    return FBP_OK;
}

}  // namespace fbp

using namespace fbp;

extern "C" size_t fbp_scan_scratch_bytes(int64_t n) { return scan_scratch(n); }

extern "C" int fbp_scan_i32(const int32_t* in, int32_t* out, int64_t n, void* scratch, size_t scratch_bytes,
                            void* stream) {
    FBP_REQUIRE(out && (in || n == 0), FBP_ERR_INVALID, "fbp_scan_i32: null pointer");
    FBP_REQUIRE(n >= 0 && n < (int64_t)1 << 31, FBP_ERR_INVALID, "fbp_scan_i32: n=%lld", (long long)n);
    FBP_REQUIRE(scratch && scratch_bytes >= scan_scratch(n), FBP_ERR_CAPACITY,
                "fbp_scan_i32: scratch %zu < %zu", scratch_bytes, scan_scratch(n));
    return scan_launch(in, out, n, (int32_t*)scratch, as_stream(stream));
}

extern "C" int fbp_inside_count(const float* x, int64_t n, const fbp_boxes* boxes, int32_t* pt_count,
                                int32_t* pt_nlvl, uint64_t* pt_lvl, int32_t* model_count, uint64_t* pt_hit,
                                int32_t* pt_cand, void* stream) {
    int rc = check_boxes(boxes);
    if (rc) return rc;
    FBP_REQUIRE(pt_count && (x || n == 0), FBP_ERR_INVALID, "fbp_inside_count: null pointer");
    if (n == 0) return FBP_OK;
    const int g = grid_for(n, 256);
    cudaStream_t st = as_stream(stream);
    switch (boxes->xd) {
        case 1: inside_count_kernel<1><<<g, 256, 0, st>>>(x, n, *boxes, pt_count, pt_nlvl, pt_lvl, model_count, pt_hit, pt_cand); break;
        case 2: inside_count_kernel<2><<<g, 256, 0, st>>>(x, n, *boxes, pt_count, pt_nlvl, pt_lvl, model_count, pt_hit, pt_cand); break;
        case 3: inside_count_kernel<3><<<g, 256, 0, st>>>(x, n, *boxes, pt_count, pt_nlvl, pt_lvl, model_count, pt_hit, pt_cand); break;
    }
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" int fbp_inside_fill(const float* x, int64_t n, const fbp_boxes* boxes, const int32_t* pt_off,
                               const int32_t* np_off, const uint64_t* pt_lvl, const uint64_t* pt_hit,
                               const int32_t* pt_cand, int32_t* n_take, int32_t* m_take,
                               int32_t* p_take, int32_t* np_take, int64_t s_cap, int64_t u_cap, int32_t* status,
                               void* stream) {
    int rc = check_boxes(boxes);
    if (rc) return rc;
    FBP_REQUIRE(pt_off && np_off && pt_lvl && status && (x || n == 0), FBP_ERR_INVALID,
                "fbp_inside_fill: null pointer");
    FBP_REQUIRE((n_take && m_take && p_take) || s_cap == 0, FBP_ERR_INVALID, "fbp_inside_fill: null take");
    FBP_REQUIRE(np_take || u_cap == 0, FBP_ERR_INVALID, "fbp_inside_fill: null np_take");
    if (n == 0) return FBP_OK;
    const int g = grid_for(n, FILL_WARPS * 32, 8);  // 32 points per warp
    cudaStream_t st = as_stream(stream);
    switch (boxes->xd) {
        case 1: inside_fill_kernel<1><<<g, FILL_WARPS * 32, 0, st>>>(x, n, *boxes, pt_off, np_off, pt_lvl, pt_hit, pt_cand, n_take, m_take, p_take, np_take, s_cap, u_cap, status); break;
        case 2: inside_fill_kernel<2><<<g, FILL_WARPS * 32, 0, st>>>(x, n, *boxes, pt_off, np_off, pt_lvl, pt_hit, pt_cand, n_take, m_take, p_take, np_take, s_cap, u_cap, status); break;
        case 3: inside_fill_kernel<3><<<g, FILL_WARPS * 32, 0, st>>>(x, n, *boxes, pt_off, np_off, pt_lvl, pt_hit, pt_cand, n_take, m_take, p_take, np_take, s_cap, u_cap, status); break;
    }
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" int fbp_gather_i32(const int32_t* in, int64_t n, const int32_t* count_dev, const int32_t* inv,
                              int32_t* out, void* stream) {
    FBP_REQUIRE(inv && out && (in || n == 0), FBP_ERR_INVALID, "fbp_gather_i32: null pointer");
    if (n == 0) return FBP_OK;
    gather_i32_kernel<<<grid_for(n, 256), 256, 0, as_stream(stream)>>>(in, n, count_dev, inv, out);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" size_t fbp_compact_scratch_bytes(int64_t n) {
    return (size_t)(n + 1) * sizeof(int32_t) * 2 + scan_scratch(n) + 256;
}

extern "C" int fbp_compact_flags(const int32_t* flag, int64_t n, int32_t* out, int32_t* count_dev, void* scratch,
                                 size_t scratch_bytes, void* stream) {
    FBP_REQUIRE(out && count_dev && (flag || n == 0), FBP_ERR_INVALID, "fbp_compact_flags: null pointer");
    FBP_REQUIRE(scratch && scratch_bytes >= fbp_compact_scratch_bytes(n), FBP_ERR_CAPACITY,
                "fbp_compact_flags: scratch too small");
    cudaStream_t st = as_stream(stream);
    int32_t* c = (int32_t*)scratch;
    int32_t* off = c + (n + 1);
    int32_t* sums = off + (n + 1);
    if (n == 0) {
        FBP_CUDA_CHECK(cudaMemsetAsync(count_dev, 0, sizeof(int32_t), st));
        return FBP_OK;
    }
    flag_to_count_kernel<<<grid_for(n, 256), 256, 0, st>>>(flag, n, c);
    FBP_LAUNCH_CHECK();
    int rc = scan_launch(c, off, n, sums, st);
    if (rc) return rc;
    compact_kernel<<<grid_for(n, 256), 256, 0, st>>>(flag, off, n, out, count_dev);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" size_t fbp_sort_scratch_bytes(int64_t s_cap, int64_t m) {
    const int64_t chn = sort_chunk(s_cap);
    const int64_t nch = (s_cap + chn - 1) / chn;
    const int64_t hn = m * nch + 1;
    return (size_t)hn * sizeof(int32_t) * 2 + scan_scratch(hn) + 256;
}

static int sort_pairs(const int32_t* m_take, const int32_t* n_take, const int32_t* p_take, const uint8_t* pt_keep,
                      const int32_t* s_dev, int64_t s_cap, int64_t m, int32_t* sd_start, int32_t* sd_rec,
                      void* scratch, size_t scratch_bytes, void* stream) {
    FBP_REQUIRE(s_dev && sd_start && m > 0, FBP_ERR_INVALID, "fbp_sort_pairs: bad args");
    FBP_REQUIRE(((uintptr_t)sd_rec & 15) == 0, FBP_ERR_INVALID, "fbp_sort_pairs: sd_rec must be 16-byte aligned");
    FBP_REQUIRE(s_cap == 0 || (m_take && n_take && p_take && sd_rec), FBP_ERR_INVALID,
                "fbp_sort_pairs: null pointer");
    FBP_REQUIRE(m * 4 <= 200 * 1024, FBP_ERR_UNSUPPORTED, "fbp_sort_pairs: m=%lld exceeds the shared-memory histogram",
                (long long)m);
    FBP_REQUIRE(scratch && scratch_bytes >= fbp_sort_scratch_bytes(s_cap, m), FBP_ERR_CAPACITY,
                "fbp_sort_pairs: scratch too small");
    cudaStream_t st = as_stream(stream);
    const int64_t chn = sort_chunk(s_cap);
    const int64_t nch = (s_cap + chn - 1) / chn;
    const int64_t hn = m * nch;
    int32_t* hist = (int32_t*)scratch;
    int32_t* hoff = hist + (hn + 1);
    int32_t* sums = hoff + (hn + 1);
    const size_t shm = (size_t)m * sizeof(int);
    int sw = SCATTER_W;  // warps per chunk in the scatter: one bucket table each
    while (sw > 1 && shm * sw > 200 * 1024) sw >>= 1;
    if (shm > 48 * 1024)
        FBP_CUDA_CHECK(cudaFuncSetAttribute(sort_hist_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm));
    if (shm * sw > 48 * 1024)
        FBP_CUDA_CHECK(
            cudaFuncSetAttribute(sort_scatter_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(shm * sw)));
    if (nch > 0) {
        const int g = (int)std::min<int64_t>(nch, (int64_t)sm_count() * 8);
        sort_hist_kernel<<<g, 256, shm, st>>>(m_take, n_take, pt_keep, s_dev, s_cap, m, nch, chn, hist);
        FBP_LAUNCH_CHECK();
    }
    int rc = scan_launch(hist, hoff, hn, sums, st);
    if (rc) return rc;
    if (nch > 0) {
        const int g = (int)std::min<int64_t>(nch, (int64_t)sm_count() * 32 / sw);
        sort_scatter_kernel<<<g, 32 * sw, shm * sw, st>>>(m_take, n_take, p_take, pt_keep, s_dev, s_cap, m, nch,
                                                          chn, hoff, reinterpret_cast<int4*>(sd_rec));
        FBP_LAUNCH_CHECK();
        sort_starts_kernel<<<grid_for(m + 1, 256), 256, 0, st>>>(hoff, m, nch, sd_start);
        FBP_LAUNCH_CHECK();
    } else {
        FBP_CUDA_CHECK(cudaMemsetAsync(sd_start, 0, (size_t)(m + 1) * sizeof(int32_t), st));
    }
    return FBP_OK;
}

extern "C" int fbp_sort_pairs(const int32_t* m_take, const int32_t* n_take, const int32_t* p_take,
                              const int32_t* s_dev, int64_t s_cap, int64_t m, int32_t* sd_start, int32_t* sd_rec,
                              void* scratch, size_t scratch_bytes, void* stream) {
    return sort_pairs(m_take, n_take, p_take, nullptr, s_dev, s_cap, m, sd_start, sd_rec, scratch, scratch_bytes,
                      stream);
}

extern "C" int fbp_sort_pairs_kept(const int32_t* m_take, const int32_t* n_take, const int32_t* p_take,
                                   const uint8_t* pt_keep, const int32_t* s_dev, int64_t s_cap, int64_t m,
                                   int32_t* sd_start, int32_t* sd_rec, void* scratch, size_t scratch_bytes,
                                   void* stream) {
    FBP_REQUIRE(pt_keep, FBP_ERR_INVALID, "fbp_sort_pairs_kept: null pt_keep");
    return sort_pairs(m_take, n_take, p_take, pt_keep, s_dev, s_cap, m, sd_start, sd_rec, scratch, scratch_bytes,
                      stream);
}

extern "C" int fbp_train_mask(const int32_t* pt_off, const int32_t* m_take, int64_t n, int64_t s_cap,
                              const uint8_t* raw, int64_t m, uint8_t* pt_keep, int32_t* n_keep, uint8_t* state,
                              uint8_t* active, void* stream) {
    FBP_REQUIRE(pt_off && raw && pt_keep && n_keep && state && active && m > 0 && n >= 0, FBP_ERR_INVALID,
                "fbp_train_mask: bad args");
    FBP_REQUIRE(s_cap == 0 || m_take, FBP_ERR_INVALID, "fbp_train_mask: null m_take");
    cudaStream_t st = as_stream(stream);
    FBP_CUDA_CHECK(cudaMemsetAsync(state, 0, (size_t)m, st));
    FBP_CUDA_CHECK(cudaMemsetAsync(n_keep, 0, sizeof(int32_t), st));
    if (n > 0) {
        train_mark_kernel<<<grid_for(n, 256), 256, 0, st>>>(pt_off, m_take, n, s_cap, raw, pt_keep, state, n_keep);
        FBP_LAUNCH_CHECK();
    }
    train_state_kernel<<<grid_for(m, 256), 256, 0, st>>>(raw, m, state, active);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" size_t fbp_work_scratch_bytes(int64_t m) { return (size_t)(m + 1) * sizeof(int32_t) * 2 + scan_scratch(m) + 256; }

extern "C" int fbp_build_work(const int32_t* sd_start, int64_t m, const uint8_t* select, int32_t chunk,
                              int32_t* items, int32_t* item_start, int32_t* n_items, int64_t items_cap,
                              int32_t* status, void* scratch, size_t scratch_bytes, void* stream) {
    FBP_REQUIRE(sd_start && items && item_start && n_items && status && m > 0 && chunk > 0, FBP_ERR_INVALID,
                "fbp_build_work: bad args");
    FBP_REQUIRE(scratch && scratch_bytes >= fbp_work_scratch_bytes(m), FBP_ERR_CAPACITY,
                "fbp_build_work: scratch too small");
    cudaStream_t st = as_stream(stream);
    int32_t* nit = (int32_t*)scratch;
    int32_t* ioff = nit + (m + 1);
    int32_t* sums = ioff + (m + 1);
    work_count_kernel<<<grid_for(m, 256), 256, 0, st>>>(sd_start, m, select, chunk, nit);
    FBP_LAUNCH_CHECK();
    int rc = scan_launch(nit, ioff, m, sums, st);
    if (rc) return rc;
    work_fill_kernel<<<grid_for(m * 32, 256), 256, 0, st>>>(sd_start, m, ioff, chunk, items, item_start, n_items,
                                                        items_cap, status);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}
