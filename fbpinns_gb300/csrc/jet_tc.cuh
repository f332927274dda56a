// Tensor-core (tcgen05, 3xTF32) variant of the per-pair forward jet kernel for
// networks with two 16-wide hidden layers.
//
// Layer 2 of the jet, z_c[k] = sum_n W2[k][n] v_c[n] (+ b2[k] for c = 0), is
// J small GEMMs per tile of 128 pairs (M = 128 pairs, N = 16, K = 16).  The
// layer-1 jet components factor as v_0 = a, v_{1+d} = tp * cw[:, d] and
// v_{1+xd+s} = tpp * c2_s (a, tp, tpp = the activation and its first two
// derivatives at the neuron's pre-activation: for tanh tp = 1 - a^2,
// tpp = -2 a tp; cw = W1 / sd, c2_s the sum of cw[:, d]^2 over the dims of
// second-derivative slot s),
// so the pair-dependent A operands are only a, tp and tpp, and the per-neuron
// scale moves into B: B_c = W2 diag(f_c), f_c = 1, cw[:, d] or c2_s,
// built once per work item.  Each thread writes its pair's rows of a, tp, tpp
// into shared memory, split as v = hi + lo with hi = v truncated to TF32, in
// the no-swizzle K-major layout of 8-row x 16-byte core matrices; one thread
// issues hi*hi + hi*lo + lo*hi MMAs (3xTF32, FP32 accumulation) into TMEM
// columns [16c, 16c+16); every thread reads back its own TMEM lane (= its
// pair) with tcgen05.ld.  The rest of the jet (activation rules, output layer,
// unnormalisation, window) stays on the CUDA cores as in forward_pairs_kernel.
// The tiles of a work item are software-pipelined over two TMEM buffers: the
// MMAs of tile t run while the CUDA cores finish tile t-1.
//
// Waits on the MMA-completion mbarrier are bounded: on a time-out the kernel
// records FBP_STATUS_TC_TIMEOUT in the status word, stops issuing work, waits
// once more (bounded) and frees its TMEM before returning.
#pragma once

#include "jet.cuh"

namespace fbp {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Shared-memory matrix descriptor: start, leading (K) and stride (M/N) byte
// offsets between core matrices, descriptor version 1, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
__host__ __device__ constexpr uint32_t umma_idesc_tf32(int M, int N) {
    return (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_tf32(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(mbar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Bounded wait: true when the phase completed, false once limit_ns of wall
// time has passed without it.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t mbar, uint32_t parity, uint64_t limit_ns) {
    const uint64_t t0 = global_ns();
    while (!mbar_try_wait(mbar, parity))
        if (global_ns() - t0 > limit_ns) return false;
    return true;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Byte offset of element (row, k) of a K-major operand with 16 K-elements per
// row in the no-swizzle core-matrix layout: core matrix (row/8, k/4) at
// (row/8)*512 + (k/4)*128, 16 bytes per row inside it.
__device__ __forceinline__ uint32_t kmajor16_off(int row, int k) {
    return (uint32_t)((row >> 3) * 512 + (k >> 2) * 128 + (row & 7) * 16 + (k & 3) * 4);
}

__device__ __forceinline__ void split_tf32(float v, float& hi, float& lo) {
    hi = __uint_as_float(__float_as_uint(v) & 0xFFFFE000u);
    lo = v - hi;
}

constexpr int TC_TILE = 128;   // pairs per tile = MMA M = threads per CTA = TMEM lanes
constexpr uint64_t TC_WAIT_NS = 200000000ull;  // 0.2 s: an MMA group takes microseconds
constexpr uint64_t TC_TEST_WAIT_NS = 1000000ull;  // 1 ms, with FBP_STATUS_TC_TEST_NO_MMA

template <class C>
struct TcSmem {
    static_assert(C::TWO && C::H1 == 16 && C::H2 == 16 && C::J <= 8, "tensor-core shape");
    // TMEM accumulator buffers: two (the next tile's MMAs run during this
    // tile's epilogue) when both fit in 128 columns, else one
    static constexpr int NBUF = 2 * C::J * 16 <= 128 ? 2 : 1;
    // TMEM columns allocated per CTA: NBUF x J accumulators of 16 columns,
    // rounded up to the power of two >= 32 that tcgen05.alloc takes
    static constexpr int COLS = pow2_at_least(NBUF * C::J * 16 < 32 ? 32 : NBUF * C::J * 16);
    static constexpr int NA = C::NS > 0 ? 3 : 2;  // A operands: a, tp (, tpp)
    // A operands, hi and lo, each 128 rows x 16 TF32 = 8 KiB
    float a[NA][2][TC_TILE * 16];
    // B operands per jet component (16 x 16): hi, lo
    float b[C::J][2][16 * 16];
    uint64_t mbar;
    uint32_t tmem_base;
};

// A operand of jet component c: 0 = a, 1 = tp, 2 = tpp.
template <class C>
__host__ __device__ constexpr int tc_a_of(int c) {
    return c == 0 ? 0 : (c <= C::XD ? 1 : 2);
}

// tanh rules of tanh_jet (plain tanh) for two neurons at once in packed FP32
// pairs: g = [a, tp z_d, tp z_s + tpp sum_d z_d^2] with a = tanh z_0,
// tp = 1 - a^2, tpp = -2 a tp.
template <class C>
__device__ __forceinline__ void tanh_jet_pair(const float2 (&z)[C::J], float2 (&g)[C::J]) {
    const float2 a = make_float2(tanh_fast(z[0].x), tanh_fast(z[0].y));
    const float2 tp = fma2(make_float2(-a.x, -a.y), a, dup2(1.0f));
    const float2 tpp = mul2(mul2(dup2(-2.0f), a), tp);
    g[0] = a;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) g[1 + d] = mul2(tp, z[1 + d]);
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        float2 q = dup2(0.f);
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if ((C::slot_dims(s) >> d) & 1) q = fma2(z[1 + d], z[1 + d], q);
        g[1 + C::XD + s] = fma2(tp, z[1 + C::XD + s], mul2(tpp, q));
    }
}

// The rest of the jet for one tile on the CUDA cores: this thread's TMEM lane
// (its pair) of the layer-2 accumulators at taddr -> tanh rules, output layer,
// unnormalisation, window product -> the pair's record.
template <class C>
__device__ __forceinline__ void tc_epilogue(const SParams<C>& S, uint32_t taddr, int warp, bool act,
                                            const float (&w)[C::J], int pos, float* __restrict__ pair_out,
                                            float* __restrict__ zs, int64_t zs_cap) {
    constexpr int J = C::J, RS = rec_stride(C::J), H2 = 16;
    float acc[J][16];
#pragma unroll
    for (int c = 0; c < J; ++c) tmem_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), acc[c]);
    tmem_wait_ld();
    if (!act) return;
    // neurons k, k+1 in packed pairs; the output layer sums even and odd
    // neurons separately and adds the two at the end
    float2 o2[J];
#pragma unroll
    for (int c = 0; c < J; ++c) o2[c] = dup2(0.f);
    o2[0].x = S.b3;
#pragma unroll
    for (int k = 0; k < H2; k += 2) {
        float2 z[J], g[J];
#pragma unroll
        for (int c = 0; c < J; ++c) z[c] = make_float2(acc[c][k], acc[c][k + 1]);
        z[0] = add2(z[0], *reinterpret_cast<const float2*>(&S.b2[k]));
        if (zs) {  // the layer-2 z-jets for the adjoint (fbp_pairs.zs: rows c * 16 + k)
#pragma unroll
            for (int c = 0; c < J; ++c) {
                __stcs(zs + (size_t)(c * H2 + k) * zs_cap, z[c].x);
                __stcs(zs + (size_t)(c * H2 + k + 1) * zs_cap, z[c].y);
            }
        }
        if constexpr (C::ACT == FBP_ACT_TANH || C::ACT == FBP_ACT_FOURIER) {
            tanh_jet_pair<C>(z, g);  // layer 2 is a plain tanh
        } else {
            float zs[2][J], gs[2][J];
#pragma unroll
            for (int c = 0; c < J; ++c) {
                zs[0][c] = z[c].x;
                zs[1][c] = z[c].y;
            }
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float a, tp, tpp, tppp;
                tanh_jet<C>(zs[h], gs[h], a, tp, tpp, tppp, act_c<C, true>(S, k + h), act_o<C, true>(S, k + h));
            }
#pragma unroll
            for (int c = 0; c < J; ++c) g[c] = make_float2(gs[0][c], gs[1][c]);
        }
        const float2 w3 = *reinterpret_cast<const float2*>(&S.W3[k]);
#pragma unroll
        for (int c = 0; c < J; ++c) o2[c] = fma2(w3, g[c], o2[c]);
    }
    float o[J];
#pragma unroll
    for (int c = 0; c < J; ++c) o[c] = o2[c].x + o2[c].y;
    float u[J];
#pragma unroll
    for (int c = 0; c < J; ++c) u[c] = o[c] * S.sd_u;
    u[0] += S.mu_u;
    float rec[RS];
    product_jet<C>(u, w, rec);
#pragma unroll
    for (int c = 0; c < J; ++c) rec[J + c] = w[c];
#pragma unroll
    for (int c = 2 * J; c < RS; ++c) rec[c] = 0.f;
    float4* dst = reinterpret_cast<float4*>(pair_out + (size_t)pos * RS);
#pragma unroll
    for (int q = 0; q < RS / 4; ++q) dst[q] = make_float4(rec[4 * q], rec[4 * q + 1], rec[4 * q + 2], rec[4 * q + 3]);
}

template <class C>
__global__ void __launch_bounds__(TC_TILE) forward_pairs_tc_kernel(fbp_net net, const float* __restrict__ x,
                                                                    fbp_pairs pr, float* __restrict__ pair_out,
                                                                    int32_t* __restrict__ status) {
    constexpr int J = C::J, XD = C::XD, RS = rec_stride(C::J), H1 = 16, H2 = 16;
    constexpr int NA = TcSmem<C>::NA, NBUF = TcSmem<C>::NBUF;
    __shared__ SParams<C> S;
    extern __shared__ float4 dyn_smem[];
    TcSmem<C>& T = *reinterpret_cast<TcSmem<C>*>(dyn_smem);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t mbar = smem_u32(&T.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&T.tmem_base)),
                     "r"(TcSmem<C>::COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = T.tmem_base;
    constexpr uint32_t idesc = umma_idesc_tf32(TC_TILE, H2);
    // test hook: no MMAs are issued, so the first wait runs out (short limit)
    const bool test_no_mma = (*(volatile int32_t*)status & FBP_STATUS_TC_TEST_NO_MMA) != 0;
    const uint64_t wait_ns = test_no_mma ? TC_TEST_WAIT_NS : TC_WAIT_NS;
    uint32_t phase = 0;
    bool failed = false;
    __shared__ int s_item;
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = first_item(pr, &s_item); it < nit && !failed; it = next_item(pr, it, &s_item)) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C, false>(S, net, j);
        // B_c[k][n] = W2[k][n] f_c[n], split hi/lo, rows k, K = n
        for (int i = tid; i < J * H2 * H1; i += blockDim.x) {
            const int c = i / (H2 * H1), r = i - c * (H2 * H1);
            const int k = r / H1, n = r - k * H1;
            float f = 1.0f;
            if (c >= 1 && c <= XD) f = S.cw[n * XD + (c - 1)];
            if (c > XD) f = S.c2[n * C::NS + (c - 1 - XD)];
            float hi, lo;
            split_tf32(S.W2[r] * f, hi, lo);
            const uint32_t off = kmajor16_off(k, n) >> 2;
            T.b[c][0][off] = hi;
            T.b[c][1][off] = lo;
        }
        // the first tile's pair (prefetched; later tiles are prefetched while
        // the previous tile's MMAs run)
        int pos_n = 0;
        float xr_n[XD];
#pragma unroll
        for (int d = 0; d < XD; ++d) xr_n[d] = 0.f;
        if (tid < cnt) {
            const int4 r = pair_rec(pr, beg + tid);
            const int pt = r.y;
            pos_n = r.x;
#pragma unroll
            for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)pt * XD + d];
        }
        // Software pipeline over the item's tiles: iteration ti stages tile ti
        // and issues its MMAs into TMEM buffer ti % NBUF, then runs the epilogue
        // of tile ti-1 (from the other buffer) while those MMAs execute, then
        // waits for them.  A rows are rewritten only after that wait; a TMEM
        // buffer is rewritten only by MMAs issued after the staging barrier
        // that follows every thread's read of it.
        const int ntile = (cnt + TC_TILE - 1) / TC_TILE;
        int pos_p = 0;        // tile ti-1: this thread's pair record index,
        bool act_p = false;   // whether it has a pair,
        float w_p[J];         // and its window jet
#pragma unroll
        for (int c = 0; c < J; ++c) w_p[c] = 0.f;
        for (int ti = 0; ti <= ntile; ++ti) {
            const int t0 = ti * TC_TILE;
            const bool stage = ti < ntile;
            const bool act = stage && t0 + tid < cnt;
            const int pos = pos_n;
            float xn[XD];
#pragma unroll
            for (int d = 0; d < XD; ++d) xn[d] = (xr_n[d] - S.mu[d]) * S.inv_sd[d];
            if (stage) {
                // this pair's rows of the A operands
                // (neurons n, n+1 in packed pairs)
#pragma unroll
                for (int n4 = 0; n4 < H1; n4 += 4) {
                    float2 av[NA][2];
#pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        const int n = n4 + 2 * q;
                        float2 z = *reinterpret_cast<const float2*>(&S.b1[n]);
#pragma unroll
                        for (int d = 0; d < XD; ++d)
                            z = fma2(make_float2(S.W1[n * XD + d], S.W1[(n + 1) * XD + d]), dup2(xn[d]), z);
                        if constexpr (C::ACT == FBP_ACT_TANH) {
                            const float2 a = make_float2(tanh_fast(z.x), tanh_fast(z.y));
                            const float2 tp = fma2(make_float2(-a.x, -a.y), a, dup2(1.0f));
                            av[0][q] = a;
                            av[1][q] = tp;
                            if constexpr (NA > 2) av[NA - 1][q] = mul2(mul2(dup2(-2.0f), a), tp);
                        } else {
                            // sigma, sigma', sigma'' of the layer-1 activation c f(o z)
                            float a0, t0, tt0, ttt0, a1, t1, tt1, ttt1;
                            const float c0 = act_c<C, false>(S, n), o0 = act_o<C, false>(S, n);
                            const float c1 = act_c<C, false>(S, n + 1), o1 = act_o<C, false>(S, n + 1);
                            C::AF1::derivs(C::AF1::stored(z.x, o0), c0, o0, a0, t0, tt0, ttt0);
                            C::AF1::derivs(C::AF1::stored(z.y, o1), c1, o1, a1, t1, tt1, ttt1);
                            av[0][q] = make_float2(a0, a1);
                            av[1][q] = make_float2(t0, t1);
                            if constexpr (NA > 2) av[NA - 1][q] = make_float2(tt0, tt1);
                        }
                    }
                    const uint32_t off = kmajor16_off(tid, n4) >> 2;
#pragma unroll
                    for (int o = 0; o < NA; ++o) {
                        float2 h[2], l[2];
#pragma unroll
                        for (int q = 0; q < 2; ++q) {
                            h[q] = make_float2(__uint_as_float(__float_as_uint(av[o][q].x) & 0xFFFFE000u),
                                               __uint_as_float(__float_as_uint(av[o][q].y) & 0xFFFFE000u));
                            l[q] = add2(av[o][q], make_float2(-h[q].x, -h[q].y));  // v - hi, exact
                        }
                        *reinterpret_cast<float4*>(&T.a[o][0][off]) = make_float4(h[0].x, h[0].y, h[1].x, h[1].y);
                        *reinterpret_cast<float4*>(&T.a[o][1][off]) = make_float4(l[0].x, l[0].y, l[1].x, l[1].y);
                    }
                }
                fence_async_smem();
                tc_fence_before();
                __syncthreads();
                tc_fence_after();
                if (tid == 0 && !test_no_mma) {
                    const uint32_t buf = tmem + (uint32_t)((ti % NBUF) * J * 16);
#pragma unroll
                    for (int c = 0; c < J; ++c) {
                        const int o = tc_a_of<C>(c);
                        const uint32_t ah = smem_u32(&T.a[o][0][0]), al = smem_u32(&T.a[o][1][0]);
                        const uint32_t bh = smem_u32(&T.b[c][0][0]), bl = smem_u32(&T.b[c][1][0]);
                        const uint32_t d = buf + (uint32_t)(c * 16);
#pragma unroll
                        for (int ks = 0; ks < 2; ++ks) {
                            const uint32_t ko = ks * 256;  // two 16-byte K chunks per MMA (K = 8)
                            umma_tf32(d, umma_desc(ah + ko, 128, 512), umma_desc(bh + ko, 128, 512), idesc, ks > 0);
                            umma_tf32(d, umma_desc(ah + ko, 128, 512), umma_desc(bl + ko, 128, 512), idesc, 1);
                            umma_tf32(d, umma_desc(al + ko, 128, 512), umma_desc(bh + ko, 128, 512), idesc, 1);
                        }
                    }
                    umma_commit(mbar);
                }
                // prefetch the next tile's pair while the MMAs run
                const int tn = t0 + TC_TILE + tid;
                if (tn < cnt) {
                    const int4 r = pair_rec(pr, beg + tn);
                    const int pt = r.y;
                    pos_n = r.x;
#pragma unroll
                    for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)pt * XD + d];
                }
            }
            __syncwarp();  // the epilogue's tcgen05.ld is warp-collective
            if (ti > 0 && NBUF == 2)
                tc_epilogue<C>(S, tmem + (uint32_t)(((ti - 1) % NBUF) * J * 16), warp, act_p, w_p, pos_p, pair_out,
                               pr.zs ? pr.zs + beg + (ti - 1) * TC_TILE + tid : nullptr, pr.zs_cap);
            if (!stage) break;
            // this tile's window jet (for its epilogue) while its MMAs run
            window_jet<C>(S, xn, w_p);
            pos_p = pos;
            act_p = act;
            // every thread waits; the verdict is made CTA-uniform before the
            // warp-collective tcgen05.ld of the epilogue
            failed = __syncthreads_or(!mbar_wait_bounded(mbar, phase, wait_ns));
            if (failed) {
                if (tid == 0) atomicOr(status, FBP_STATUS_TC_TIMEOUT);
                break;
            }
            phase ^= 1u;
            tc_fence_after();
            if constexpr (NBUF == 1) {
                // one TMEM buffer: the epilogue runs before the next tile's MMAs
                __syncwarp();
                tc_epilogue<C>(S, tmem, warp, act_p, w_p, pos_p, pair_out,
                               pr.zs ? pr.zs + beg + ti * TC_TILE + tid : nullptr, pr.zs_cap);
                tc_fence_before();
                __syncthreads();
                tc_fence_after();
            }
        }
    }
    if (failed) mbar_wait_bounded(mbar, phase, wait_ns);  // let the timed-out MMAs finish
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TcSmem<C>::COLS) : "memory");
}

}  // namespace fbp
