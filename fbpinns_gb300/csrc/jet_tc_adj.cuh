// Tensor-core (tcgen05, 3xTF32) variant of the per-pair adjoint kernel for
// tanh networks with two 16-wide hidden layers.
//
// The adjoint recomputes each pair's layer-2 pre-activation jet z_c =
// W2 v_c (+ b2) before back-propagating through it.  That contraction is the
// forward's: J GEMMs of M = 128 pairs, N = 16, K = 16 per tile with the
// pair-dependent A operands a, tp, tpp of the first layer and the per-neuron
// scales folded into B_c = W2 diag(f_c) (see jet_tc.cuh).  Here it runs on the
// tensor cores; per tile of 128 pairs (thread = pair = TMEM lane):
//
//   stage A: seeds -> o-bar (registers); layer 1 -> the a1 row and the A
//            operands; one thread issues the MMAs of the tile into TMEM
//   wait for the MMAs (bounded), tcgen05.ld the z-jets
//   phase A2: tanh jets of layer 2 and their adjoint -> z2-bar rows, the
//            W3-bar and b3-bar sums
//   phases B, C (each warp on its 32 pairs): v-bar = W2^T z2-bar and the
//            layer-1 adjoint; W2-bar.
//
// Phases B and C, the W3/W1/bias reduce-scatters and the per-item gradient
// partials are those of adjoint_pairs_kernel (jet.cuh); the z-jets come from
// the tensor cores instead of FFMA2 loops, so the CUDA cores drop a third of
// their layer-2 FMAs.  Three CTAs share an SM (about 74 KB of shared memory
// each: the z2-bar rows reuse the A-operand region), so CUDA-core phases run
// while other CTAs wait for their MMAs.  Waits on the MMA-completion mbarrier are bounded as in the forward
// kernel: on a time-out the CTA records FBP_STATUS_TC_TIMEOUT, stops, waits
// once more and frees its TMEM.
#pragma once

#include "jet_tc.cuh"

namespace fbp {

template <class C>
struct TcAdjSmem {
    static_assert(C::TWO && C::H1 == 16 && C::H2 == 16 && C::J <= 8 && C::EXTRA == 0, "tensor-core adjoint shape");
    static constexpr int COLS = pow2_at_least(C::J * 16 < 32 ? 32 : C::J * 16);  // one z-jet accumulator set
    static constexpr int NA = TcSmem<C>::NA;
    float a[NA][2][TC_TILE * 16];  // A operands a, tp (, tpp): hi, lo
    float b[C::J][2][16 * 16];     // B_c = W2 diag(f_c): hi, lo
    uint64_t mbar;
    uint32_t tmem_base;
    uint32_t pad_;
};

// One warp's rows and gradient sums (the warp owns 32 lanes = pairs of a
// tile).  Its z2-bar rows live in the A-operand region of TcAdjSmem: they are
// written after the tile's MMAs have completed and read before the next tile
// is staged, so the two never hold data at the same time.
template <class C>
struct __align__(16) TcAdjWarp {
    float a1[32 * AdjW<C>::AS];  // layer-1 activations [t][n]
    float gW2[C::H2 * C::H1];
    float gW1[C::H1 * C::XD];
    float gb1[C::H1];
    float gb2[C::H2];
    float gW3[C::HL];
    float gb3;
};

// Phase B of one warp tile: v-bar = W2^T z2-bar (own row), the layer-1 jet
// adjoint, and the W1-bar / b1-bar terms summed over the warp.
template <class C>
__device__ __forceinline__ void tc_adj_phase_b(const SParams<C>& S, TcAdjWarp<C>& R, const float* zb,
                                               const float* a1row, bool act, const float (&xn)[C::XD], int lane) {
    using A = AdjW<C>;
    constexpr int J = C::J, XD = C::XD, H1 = C::H1, H2 = C::H2;
    constexpr int RN = XD + 1;
    constexpr int NC = 32 / RN >= 8 ? 8 : 4;
    static_assert(NC * RN <= 32 && H1 % NC == 0 && NC % 2 == 0, "layer-1 chunk");
#pragma unroll 1
    for (int n0 = 0; n0 < H1; n0 += NC) {
        float r1[32];
#pragma unroll
        for (int i = 0; i < 32; ++i) r1[i] = 0.f;
        if (act) {
            float2 vb2[NC / 2][J];
#pragma unroll
            for (int q = 0; q < NC / 2; ++q)
#pragma unroll
                for (int c = 0; c < J; ++c) vb2[q][c] = make_float2(0.f, 0.f);
            const float* zrow = zb + lane * A::ZS;
#pragma unroll 1
            for (int k0 = 0; k0 < H2; k0 += 4) {
                float4 z4[J];
#pragma unroll
                for (int c = 0; c < J; ++c) z4[c] = *reinterpret_cast<const float4*>(zrow + c * H2 + k0);
#pragma unroll
                for (int kq = 0; kq < 4; ++kq) {
                    const float2* w2 = reinterpret_cast<const float2*>(&S.W2[(k0 + kq) * H1 + n0]);
#pragma unroll
                    for (int q = 0; q < NC / 2; ++q) {
                        const float2 w = w2[q];
#pragma unroll
                        for (int c = 0; c < J; ++c) {
                            const float zc = kq == 0 ? z4[c].x : kq == 1 ? z4[c].y : kq == 2 ? z4[c].z : z4[c].w;
                            vb2[q][c] = fma2(w, make_float2(zc, zc), vb2[q][c]);
                        }
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < NC; ++q) {
                const int n = n0 + q;
                float vb[J];
#pragma unroll
                for (int c = 0; c < J; ++c) vb[c] = (q & 1) ? vb2[q / 2][c].y : vb2[q / 2][c].x;
                float a, tp, tpp, tppp;
                C::AF1::derivs(a1row[n], 1.0f, 1.0f, a, tp, tpp, tppp);
                float tpb = 0.f, tppb = 0.f, cwb[XD];
#pragma unroll
                for (int d = 0; d < XD; ++d) {
                    tpb += vb[1 + d] * S.cw[n * XD + d];
                    cwb[d] = vb[1 + d] * tp;
                }
#pragma unroll
                for (int s = 0; s < C::NS; ++s) {
                    const float g = vb[1 + XD + s];
                    tppb += g * S.c2[n * C::NS + s];
#pragma unroll
                    for (int d = 0; d < XD; ++d)
                        if ((C::slot_dims(s) >> d) & 1) cwb[d] += 2.0f * g * tpp * S.cw[n * XD + d];
                }
                const float z1b = vb[0] * tp + tpb * tpp + tppb * tppp;
#pragma unroll
                for (int d = 0; d < XD; ++d) r1[q * RN + d] = fmaf(z1b, xn[d], cwb[d] * S.inv_sd[d]);
                r1[q * RN + XD] = z1b;
            }
        }
        warp_reduce_scatter<32>(r1, lane);
        if (lane < NC * RN) {
            const int q = lane / RN, d = lane - q * RN;
            if (d < XD)
                R.gW1[(n0 + q) * XD + d] += r1[0];
            else
                R.gb1[n0 + q] += r1[0];
        }
    }
}

// Phase C of one warp tile: W2-bar and b2-bar over its nt pairs (lane = a
// KB x NB block of W2-bar; rows in pairs share packed FMAs).
template <class C>
__device__ __forceinline__ void tc_adj_phase_c(const SParams<C>& S, TcAdjWarp<C>& R, const float* zb,
                                               const float* a1rows, int nt, int lane) {
    using A = AdjW<C>;
    constexpr int J = C::J, XD = C::XD, H1 = C::H1, H2 = C::H2;
#pragma unroll 1
    for (int ps = 0; ps < A::PASSES; ++ps) {
        const int b = ps * 32 + lane;
        if (b >= A::NBLK) continue;
        const int nb = b % (H1 / A::NB), kb = b / (H1 / A::NB);
        const int n0 = nb * A::NB, k0 = kb * A::KB;
        float2 sacc[A::KB / 2][A::NB][J];
#pragma unroll
        for (int i = 0; i < A::KB / 2; ++i)
#pragma unroll
            for (int q = 0; q < A::NB; ++q)
#pragma unroll
                for (int c = 0; c < J; ++c) sacc[i][q][c] = make_float2(0.f, 0.f);
        float b2s[A::KB];
#pragma unroll
        for (int i = 0; i < A::KB; ++i) b2s[i] = 0.f;
        constexpr int UC = FBP_ADJ_UNROLL_C;  // (pragma arguments are not macro-expanded)
#pragma unroll UC
        for (int t = 0; t < nt; ++t) {
            float m[A::NB][3];
#pragma unroll
            for (int q = 0; q < A::NB; ++q) {
                float a, tp, tpp, tppp;
                C::AF1::derivs(a1rows[t * A::AS + n0 + q], 1.0f, 1.0f, a, tp, tpp, tppp);
                m[q][0] = a;
                m[q][1] = tp;
                m[q][2] = tpp;
            }
            const float* zr = zb + t * A::ZS + k0;
#pragma unroll
            for (int c = 0; c < J; ++c) {
                float2 z2[A::KB / 2];
                if constexpr (A::KB == 2) {
                    z2[0] = *reinterpret_cast<const float2*>(zr + c * H2);
                } else {
#pragma unroll
                    for (int h = 0; h < A::KB / 4; ++h) {
                        const float4 z4 = *reinterpret_cast<const float4*>(zr + c * H2 + 4 * h);
                        z2[2 * h] = make_float2(z4.x, z4.y);
                        z2[2 * h + 1] = make_float2(z4.z, z4.w);
                    }
                }
                const int mi = c == 0 ? 0 : (c <= XD ? 1 : 2);
                if (c == 0) {
#pragma unroll
                    for (int i = 0; i < A::KB / 2; ++i) {
                        b2s[2 * i] += z2[i].x;
                        b2s[2 * i + 1] += z2[i].y;
                    }
                }
#pragma unroll
                for (int q = 0; q < A::NB; ++q) {
                    const float2 mm = make_float2(m[q][mi], m[q][mi]);
#pragma unroll
                    for (int i = 0; i < A::KB / 2; ++i) sacc[i][q][c] = fma2(z2[i], mm, sacc[i][q][c]);
                }
            }
        }
#pragma unroll
        for (int i = 0; i < A::KB; ++i)
#pragma unroll
            for (int q = 0; q < A::NB; ++q) {
                const int n = n0 + q;
                float s[J];
#pragma unroll
                for (int c = 0; c < J; ++c) s[c] = (i & 1) ? sacc[i / 2][q][c].y : sacc[i / 2][q][c].x;
                float v = s[0];
#pragma unroll
                for (int d = 0; d < XD; ++d) v = fmaf(S.cw[n * XD + d], s[1 + d], v);
#pragma unroll
                for (int ss = 0; ss < C::NS; ++ss) v = fmaf(S.c2[n * C::NS + ss], s[1 + XD + ss], v);
                R.gW2[(k0 + i) * H1 + n] += v;
            }
        if (nb == 0) {
#pragma unroll
            for (int i = 0; i < A::KB; ++i) R.gb2[k0 + i] += b2s[i];
        }
    }
}

template <class C>
__global__ void __launch_bounds__(TC_TILE) adjoint_pairs_tc_kernel(fbp_net net, const float* __restrict__ x,
                                                                    fbp_pairs pr, const float* __restrict__ slot_out,
                                                                    float* __restrict__ grad_part,
                                                                    int32_t* __restrict__ status) {
    using A = AdjW<C>;
    constexpr int J = C::J, XD = C::XD, H1 = 16, H2 = 16, RS = rec_stride(J);
    constexpr int NA = TcAdjSmem<C>::NA;
    static_assert(sizeof(TcAdjWarp<C>) % 16 == 0 && A::ZS % 4 == 0, "16-byte rows");
    static_assert((TC_TILE / 32) * 32 * A::ZS <= (int)sizeof(TcAdjSmem<C>::a) / 4, "z2-bar rows fit the A region");
    __shared__ SParams<C> S;
    extern __shared__ float4 dyn_smem[];
    TcAdjSmem<C>& T = *reinterpret_cast<TcAdjSmem<C>*>(dyn_smem);
    TcAdjWarp<C>* RW = reinterpret_cast<TcAdjWarp<C>*>(reinterpret_cast<char*>(dyn_smem) +
                                                       ((sizeof(TcAdjSmem<C>) + 15) / 16) * 16);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    TcAdjWarp<C>& R = RW[warp];
    float* zb = &T.a[0][0][0] + warp * 32 * A::ZS;  // this warp's z2-bar rows (in the A region)
    const uint32_t mbar = smem_u32(&T.mbar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&T.tmem_base)),
                     "r"(TcAdjSmem<C>::COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = T.tmem_base;
    constexpr uint32_t idesc = umma_idesc_tf32(TC_TILE, H2);
    const bool test_no_mma = (*(volatile int32_t*)status & FBP_STATUS_TC_TEST_NO_MMA) != 0;
    const uint64_t wait_ns = test_no_mma ? TC_TEST_WAIT_NS : TC_WAIT_NS;
    uint32_t phase = 0;
    bool failed = false;
    __shared__ int s_item;
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = first_item(pr, &s_item); it < nit && !failed; it = next_item(pr, it, &s_item)) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C>(S, net, j);
        for (int i = tid; i < J * H2 * H1; i += blockDim.x) {  // B_c = W2 diag(f_c), hi / lo
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
        for (int i = lane; i < H2 * H1; i += 32) R.gW2[i] = 0.f;
        for (int i = lane; i < H1 * XD; i += 32) R.gW1[i] = 0.f;
        if (lane < H1) R.gb1[lane] = 0.f;
        if (lane < H2) R.gb2[lane] = 0.f;
        if (lane < H2) R.gW3[lane] = 0.f;
        if (lane == 0) R.gb3 = 0.f;
        // the first tile's pair (later tiles are prefetched while MMAs run)
        int4 rec_n = make_int4(0, 0, -1, 0);
        float xr_n[XD];
#pragma unroll
        for (int d = 0; d < XD; ++d) xr_n[d] = 0.f;
        if (tid < cnt) {
            rec_n = pair_rec(pr, beg + tid);
#pragma unroll
            for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)rec_n.y * XD + d];
        }
        const int ntile = (cnt + TC_TILE - 1) / TC_TILE;
        for (int ti = 0; ti < ntile; ++ti) {
            const int t0 = ti * TC_TILE;
            const bool act = t0 + tid < cnt;
            const int nt = max(0, min(32, cnt - (t0 + warp * 32)));  // pairs of this warp's part
            float xn[XD], ob[J];
#pragma unroll
            for (int d = 0; d < XD; ++d) xn[d] = (xr_n[d] - S.mu[d]) * S.inv_sd[d];
#pragma unroll
            for (int c = 0; c < J; ++c) ob[c] = 0.f;
            float* a1row = &R.a1[lane * A::AS];
            // every warp has read its z2-bar rows (the previous tile's phase C)
            // before the A operands overwrite that region
            __syncthreads();
            // ---- stage A: seeds -> o-bar; layer 1 -> A operands and a1 row ----
            if (act) {
                float w[J];
                window_jet<C>(S, xn, w);
                const int slot = rec_n.z;
                const bool ok = slot >= 0 && slot < pr.slots_cap;  // overflowed slots carry no seed
                float nb[J];
                const float4* src = reinterpret_cast<const float4*>(slot_out + (size_t)(ok ? slot : 0) * RS);
#pragma unroll
                for (int q = 0; q < (J + 3) / 4; ++q) {
                    const float4 v = src[q];
                    if (4 * q + 0 < J) nb[4 * q + 0] = ok ? v.x : 0.f;
                    if (4 * q + 1 < J) nb[4 * q + 1] = ok ? v.y : 0.f;
                    if (4 * q + 2 < J) nb[4 * q + 2] = ok ? v.z : 0.f;
                    if (4 * q + 3 < J) nb[4 * q + 3] = ok ? v.w : 0.f;
                }
                float ub[J];
                product_jet_adj<C>(nb, w, ub);
#pragma unroll
                for (int c = 0; c < J; ++c) ob[c] = ub[c] * S.sd_u;
            }
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
                    const float2 a = make_float2(tanh_fast(z.x), tanh_fast(z.y));
                    const float2 tp = fma2(make_float2(-a.x, -a.y), a, dup2(1.0f));
                    av[0][q] = a;
                    av[1][q] = tp;
                    if constexpr (NA > 2) av[NA - 1][q] = mul2(mul2(dup2(-2.0f), a), tp);
                    a1row[n] = a.x;
                    a1row[n + 1] = a.y;
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
#pragma unroll
                for (int c = 0; c < J; ++c) {
                    const int o = tc_a_of<C>(c);
                    const uint32_t ah = smem_u32(&T.a[o][0][0]), al = smem_u32(&T.a[o][1][0]);
                    const uint32_t bh = smem_u32(&T.b[c][0][0]), bl = smem_u32(&T.b[c][1][0]);
                    const uint32_t d = tmem + (uint32_t)(c * 16);
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
                rec_n = pair_rec(pr, beg + tn);
#pragma unroll
                for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)rec_n.y * XD + d];
            }
            // ---- wait for the tile's z-jets (the verdict is CTA-uniform) ----
            failed = __syncthreads_or(!mbar_wait_bounded(mbar, phase, wait_ns));
            if (failed) {
                if (tid == 0) atomicOr(status, FBP_STATUS_TC_TIMEOUT);
                break;
            }
            phase ^= 1u;
            tc_fence_after();
            // ---- phase A2: tanh jets of layer 2 and their adjoint -> z2-bar rows ----
            {
                float acc[J][16];
#pragma unroll
                for (int c = 0; c < J; ++c)
                    tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(c * 16), acc[c]);
                tmem_wait_ld();
                float e3[16];
                float* zrow = zb + lane * A::ZS;
#pragma unroll
                for (int k = 0; k < H2; k += 2) {
                    float2 z[J];
#pragma unroll
                    for (int c = 0; c < J; ++c) z[c] = make_float2(acc[c][k], acc[c][k + 1]);
                    z[0] = add2(z[0], *reinterpret_cast<const float2*>(&S.b2[k]));
                    const float2 a = make_float2(tanh_fast(z[0].x), tanh_fast(z[0].y));
                    const float2 tp = fma2(make_float2(-a.x, -a.y), a, dup2(1.0f));
                    const float2 tpp = mul2(mul2(dup2(-2.0f), a), tp);
                    // tppp = tp (6 a^2 - 2)
                    const float2 tppp = mul2(tp, fma2(mul2(dup2(6.0f), a), a, dup2(-2.0f)));
                    float2 q2[C::NS > 0 ? C::NS : 1];  // sum of z_d^2 over each slot's dims
                    float2 g[J];
                    g[0] = a;
#pragma unroll
                    for (int d = 0; d < XD; ++d) g[1 + d] = mul2(tp, z[1 + d]);
#pragma unroll
                    for (int s = 0; s < C::NS; ++s) {
                        float2 q = dup2(0.f);
#pragma unroll
                        for (int d = 0; d < XD; ++d)
                            if ((C::slot_dims(s) >> d) & 1) q = fma2(z[1 + d], z[1 + d], q);
                        q2[s] = q;
                        g[1 + XD + s] = fma2(tp, z[1 + XD + s], mul2(tpp, q));
                    }
                    // W3-bar terms sum_c ob_c g_c and the sensitivities gb_c = W3 ob_c
                    float2 s3 = dup2(0.f);
#pragma unroll
                    for (int c = 0; c < J; ++c) s3 = fma2(dup2(ob[c]), g[c], s3);
                    e3[k] = s3.x;
                    e3[k + 1] = s3.y;
                    const float2 w3 = *reinterpret_cast<const float2*>(&S.W3[k]);
                    float2 gb[J];
#pragma unroll
                    for (int c = 0; c < J; ++c) gb[c] = mul2(w3, dup2(ob[c]));
                    // adjoint of the tanh jet (tanh_jet_adj, two neurons at once)
                    float2 tpb = dup2(0.f), tppb = dup2(0.f), zb[J];
#pragma unroll
                    for (int d = 0; d < XD; ++d) {
                        tpb = fma2(gb[1 + d], z[1 + d], tpb);
                        zb[1 + d] = mul2(gb[1 + d], tp);
                    }
#pragma unroll
                    for (int s = 0; s < C::NS; ++s) {
                        const float2 gs = gb[1 + XD + s];
                        tpb = fma2(gs, z[1 + XD + s], tpb);
                        zb[1 + XD + s] = mul2(gs, tp);
                        tppb = fma2(gs, q2[s], tppb);
                        const float2 g2 = mul2(mul2(dup2(2.0f), gs), tpp);
#pragma unroll
                        for (int d = 0; d < XD; ++d)
                            if ((C::slot_dims(s) >> d) & 1) zb[1 + d] = fma2(g2, z[1 + d], zb[1 + d]);
                    }
                    zb[0] = fma2(tppb, tppp, fma2(tpb, tpp, mul2(gb[0], tp)));
#pragma unroll
                    for (int c = 0; c < J; ++c) *reinterpret_cast<float2*>(zrow + c * H2 + k) = zb[c];
                }
                warp_reduce_scatter<16>(e3, lane);  // lanes without a pair have ob = 0
                if (!(lane & 1)) R.gW3[lane >> 1] += e3[0];
                float b3 = ob[0];
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) b3 += __shfl_xor_sync(0xffffffffu, b3, o);
                if (lane == 0) R.gb3 += b3;
            }
            __syncwarp();  // z2-bar and a1 rows of the warp's pairs are written
            // ---- phases B and C (warp-level) ----
            tc_adj_phase_b<C>(S, R, zb, a1row, act, xn, lane);
            tc_adj_phase_c<C>(S, R, zb, R.a1, nt, lane);
            __syncwarp();  // every lane has read the rows before the next tile rewrites them
        }
        if (failed) break;
        __syncthreads();
        // combine the warps' sums (fixed warp order) into the item's gradient partial
        float* dst = grad_part + (size_t)it * C::P;
        constexpr int NW = TC_TILE / 32;
        for (int i = tid; i < H1 * XD; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gW1[i];
            dst[C::oW1 + i] = v;
        }
        for (int i = tid; i < H1; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gb1[i];
            dst[C::ob1 + i] = v;
        }
        for (int i = tid; i < H2 * H1; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gW2[i];
            dst[C::oW2 + i] = v;
        }
        for (int i = tid; i < H2; i += blockDim.x) {
            float v = 0.f, v3 = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
                v += RW[w].gb2[i];
                v3 += RW[w].gW3[i];
            }
            dst[C::ob2 + i] = v;
            dst[C::oW3 + i] = v3;
        }
        if (tid == 0) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gb3;
            dst[C::ob3] = v;
        }
    }
    if (failed) mbar_wait_bounded(mbar, phase, wait_ns);  // let the timed-out MMAs finish
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TcAdjSmem<C>::COLS)
                     : "memory");
}

}  // namespace fbp
