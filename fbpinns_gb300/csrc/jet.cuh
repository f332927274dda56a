// Per-pair FCN Taylor-jet forward and adjoint kernels (FP32 CUDA-core FMA).
//
// A work item is (subdomain j, a contiguous run of j's pairs).  A CTA stages
// j's weights in shared memory and walks the run one pair per thread; the jet
// of the network output with respect to the raw input coordinates
//   [u, du/dx_d (all d), d2u/dx_d^2 (d in D2)]
// is carried in registers through every layer:
//   linear:  z_c = W a_c (+ b for the value component c = 0)
//   tanh:    a = t(z0), t' = 1 - a^2, t'' = -2 a t'
//            a_d = t' z_d,   a_dd = t' z_dd + t'' z_d^2
// The first layer's tangents are the columns of W1 scaled by 1/sd (the
// normalisation), so they cost no MACs.  The window is separable, so its jet
// is a product of 1D jets.
#pragma once

#include "common.cuh"

namespace fbp {

template <int XD_, int H1_, int H2_, int D2_>
struct Cfg {
    static constexpr int XD = XD_, H1 = H1_, H2 = H2_, D2 = D2_;
    static constexpr int NS = popc_const(D2);
    static constexpr int J = 1 + XD + NS;
    static constexpr bool TWO = H2 > 0;
    static constexpr int HL = TWO ? H2 : H1;  // width feeding the output layer
    static constexpr int oW1 = 0, ob1 = H1 * XD;
    static constexpr int oW2 = ob1 + H1;
    static constexpr int ob2 = oW2 + (TWO ? H2 * H1 : 0);
    static constexpr int oW3 = TWO ? ob2 + H2 : ob1 + H1;
    static constexpr int ob3 = oW3 + HL;
    static constexpr int P = ob3 + 1;
    static constexpr int KC = TWO ? (H2 < 16 ? H2 : 16) : 1;  // layer-2 neurons per register pass
    static constexpr int NCH = TWO ? H2 / KC : 1;
    static_assert(!TWO || H2 % KC == 0, "H2 must be a multiple of the chunk");
    // second-derivative dim of slot s
    __host__ __device__ static constexpr int sd_dim(int s) { return DimsOf<D2>::get(s); }
};

template <class C>
struct SParams {
    float W1[C::H1 * C::XD];
    float b1[C::H1];
    float cw[C::H1 * C::XD];   // W1[n][d] / sd[d]: first-layer tangent along d
    float cw2[C::H1 * C::XD];  // cw^2
    float W2t[C::TWO ? C::H1 * C::H2 : 4];  // [n][k]
    float W2[C::TWO ? C::H2 * C::H1 : 4];   // [k][n]
    float b2[C::TWO ? C::H2 : 4];
    float W3[C::HL];
    float b3;
    float mu[C::XD], inv_sd[C::XD], wsc[C::XD];  // wsc = pi / (2 sd)
    float flag, mu_u, sd_u;
};

template <class C>
__device__ __forceinline__ void load_params(SParams<C>& S, const fbp_net& net, int j) {
    const float* __restrict__ th = net.theta + (size_t)j * C::P;
    for (int i = threadIdx.x; i < C::H1 * C::XD; i += blockDim.x) S.W1[i] = th[C::oW1 + i];
    for (int i = threadIdx.x; i < C::H1; i += blockDim.x) S.b1[i] = th[C::ob1 + i];
    if constexpr (C::TWO) {
        for (int i = threadIdx.x; i < C::H2 * C::H1; i += blockDim.x) {
            const float v = th[C::oW2 + i];
            const int k = i / C::H1, n = i - k * C::H1;
            S.W2[i] = v;
            S.W2t[n * C::H2 + k] = v;
        }
        for (int i = threadIdx.x; i < C::H2; i += blockDim.x) S.b2[i] = th[C::ob2 + i];
    }
    for (int i = threadIdx.x; i < C::HL; i += blockDim.x) S.W3[i] = th[C::oW3 + i];
    if (threadIdx.x == 0) {
        S.b3 = th[C::ob3];
        S.flag = net.flags[j];
        S.mu_u = net.unnorms[2 * (size_t)j];
        S.sd_u = net.unnorms[2 * (size_t)j + 1];
    }
    if (threadIdx.x < C::XD) {
        const int d = threadIdx.x;
        const float lo = net.xmins[(size_t)j * C::XD + d], hi = net.xmaxs[(size_t)j * C::XD + d];
        const float sd = (hi - lo) / 2.0f;
        S.mu[d] = (hi + lo) / 2.0f;
        S.inv_sd[d] = 1.0f / sd;
        S.wsc[d] = 1.5707963267948966f / sd;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C::H1 * C::XD; i += blockDim.x) {
        const int d = i % C::XD;
        const float c = S.W1[i] * S.inv_sd[d];
        S.cw[i] = c;
        S.cw2[i] = c * c;
    }
    __syncthreads();
}

// Jet of one first-layer neuron's activation from a = tanh(z1).
template <class C>
__device__ __forceinline__ void l1_jet(const SParams<C>& S, int n, float a, float (&v)[C::J]) {
    const float tp = 1.0f - a * a, tpp = -2.0f * a * tp;
    v[0] = a;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) v[1 + d] = tp * S.cw[n * C::XD + d];
#pragma unroll
    for (int s = 0; s < C::NS; ++s) v[1 + C::XD + s] = tpp * S.cw2[n * C::XD + C::sd_dim(s)];
}

// tanh applied to a z-jet.
template <class C>
__device__ __forceinline__ void tanh_jet(const float (&z)[C::J], float (&g)[C::J], float& a, float& tp,
                                         float& tpp) {
    a = tanh_fast(z[0]);
    tp = 1.0f - a * a;
    tpp = -2.0f * a * tp;
    g[0] = a;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) g[1 + d] = tp * z[1 + d];
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        const float zd = z[1 + C::sd_dim(s)];
        g[1 + C::XD + s] = tp * z[1 + C::XD + s] + tpp * zd * zd;
    }
}

// Adjoint of tanh_jet: given g-bar, returns z-bar (in place of gb).
template <class C>
__device__ __forceinline__ void tanh_jet_adj(const float (&z)[C::J], float a, float tp, float tpp,
                                             float (&gb)[C::J], float (&zb)[C::J]) {
    float tpb = 0.f, tppb = 0.f;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) {
        tpb += gb[1 + d] * z[1 + d];
        zb[1 + d] = gb[1 + d] * tp;
    }
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        const int d = C::sd_dim(s);
        const float g = gb[1 + C::XD + s];
        tpb += g * z[1 + C::XD + s];
        tppb += g * z[1 + d] * z[1 + d];
        zb[1 + C::XD + s] = g * tp;
        zb[1 + d] += 2.0f * g * tpp * z[1 + d];
    }
    const float ab = gb[0] + tpb * (-2.0f * a) + tppb * (6.0f * a * a - 2.0f);
    zb[0] = ab * tp;
}

// Window jet (cosine window of fbpinns/windows.py:25-35 times flag plus 1-flag):
// per dim c = cos^4(phi), phi = (pi/2) xn; derivatives by the chain rule.
template <class C>
__device__ __forceinline__ void window_jet(const SParams<C>& S, const float (&xn)[C::XD], float (&w)[C::J]) {
    float c0[C::XD], c1[C::XD], c2[C::XD];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) {
        float sn, cs;
        sincosf(1.5707963267948966f * xn[d], &sn, &cs);
        const float cs2 = cs * cs;
        const float k = S.wsc[d];
        c0[d] = cs2 * cs2;
        c1[d] = -4.0f * cs2 * cs * sn * k;
        c2[d] = (12.0f * cs2 * sn * sn - 4.0f * cs2 * cs2) * k * k;
    }
    float prod = 1.f;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) prod *= c0[d];
    const float f = S.flag;
    w[0] = f * prod + (1.0f - f);
#pragma unroll
    for (int i = 0; i < C::XD; ++i) {
        float p = c1[i];
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if (d != i) p *= c0[d];
        w[1 + i] = f * p;
    }
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        const int i = C::sd_dim(s);
        float p = c2[i];
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if (d != i) p *= c0[d];
        w[1 + C::XD + s] = f * p;
    }
}

template <class C>
__device__ __forceinline__ void load_point(const SParams<C>& S, const float* __restrict__ x, int pt,
                                           float (&xn)[C::XD]) {
#pragma unroll
    for (int d = 0; d < C::XD; ++d) xn[d] = (x[(size_t)pt * C::XD + d] - S.mu[d]) * S.inv_sd[d];
}

template <class C>
__device__ __forceinline__ float l1_act(const SParams<C>& S, const float (&xn)[C::XD], int n) {
    float z = S.b1[n];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) z = fmaf(S.W1[n * C::XD + d], xn[d], z);
    return tanh_fast(z);
}

// Layer-2 z-jets for neurons [k0, k0+KC) from first-layer activations a1row[n*stride]
// (each thread's own activations, kept in shared memory).
template <class C>
__device__ __forceinline__ void l2_chunk(const SParams<C>& S, const float* a1row, int stride, int k0,
                                         float (&acc)[C::KC][C::J]) {
#pragma unroll
    for (int k = 0; k < C::KC; ++k) {
        acc[k][0] = S.b2[k0 + k];
#pragma unroll
        for (int c = 1; c < C::J; ++c) acc[k][c] = 0.f;
    }
#pragma unroll 2
    for (int n = 0; n < C::H1; ++n) {
        float v[C::J];
        l1_jet<C>(S, n, a1row[n * stride], v);
        const float* wrow = &S.W2t[n * C::H2 + k0];
#pragma unroll
        for (int k = 0; k < C::KC; ++k) {
            const float w = wrow[k];
#pragma unroll
            for (int c = 0; c < C::J; ++c) acc[k][c] = fmaf(w, v[c], acc[k][c]);
        }
    }
}

// Network output jet (before unnormalisation) for one pair; a1row/stride is the
// thread's shared-memory slot for its first-layer activations.
template <class C>
__device__ __forceinline__ void net_jet(const SParams<C>& S, const float (&xn)[C::XD], float* a1row, int stride,
                                        float (&out)[C::J]) {
#pragma unroll 4
    for (int n = 0; n < C::H1; ++n) a1row[n * stride] = l1_act<C>(S, xn, n);
#pragma unroll
    for (int c = 0; c < C::J; ++c) out[c] = 0.f;
    out[0] = S.b3;
    if constexpr (C::TWO) {
#pragma unroll 1
        for (int ch = 0; ch < C::NCH; ++ch) {
            float acc[C::KC][C::J];
            l2_chunk<C>(S, a1row, stride, ch * C::KC, acc);
#pragma unroll
            for (int k = 0; k < C::KC; ++k) {
                float g[C::J], a, tp, tpp;
                tanh_jet<C>(acc[k], g, a, tp, tpp);
                const float w3 = S.W3[ch * C::KC + k];
#pragma unroll
                for (int c = 0; c < C::J; ++c) out[c] = fmaf(w3, g[c], out[c]);
            }
        }
    } else {
#pragma unroll 2
        for (int n = 0; n < C::H1; ++n) {
            float v[C::J];
            l1_jet<C>(S, n, a1row[n * stride], v);
            const float w3 = S.W3[n];
#pragma unroll
            for (int c = 0; c < C::J; ++c) out[c] = fmaf(w3, v[c], out[c]);
        }
    }
}

constexpr int FWD_THREADS = 128;

template <class C>
__global__ void __launch_bounds__(FWD_THREADS) forward_pairs_kernel(fbp_net net, const float* __restrict__ x,
                                                                     fbp_pairs pr, float* __restrict__ pair_out) {
    __shared__ SParams<C> S;
    __shared__ float a1s[C::H1 * FWD_THREADS];
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = blockIdx.x; it < nit; it += gridDim.x) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C>(S, net, j);
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const int e = beg + t;
            const int pt = pr.sd_point[e];
            const int pos = pr.sd_pair[e];
            float xn[C::XD];
            load_point<C>(S, x, pt, xn);
            float o[C::J];
            net_jet<C>(S, xn, &a1s[threadIdx.x], FWD_THREADS, o);
            // unnormalisation (decompositions.py:191-194): u = u_raw*sd + mu
            float u[C::J];
#pragma unroll
            for (int c = 0; c < C::J; ++c) u[c] = o[c] * S.sd_u;
            u[0] += S.mu_u;
            float w[C::J];
            window_jet<C>(S, xn, w);
            float uw[C::J];
            uw[0] = u[0] * w[0];
#pragma unroll
            for (int d = 0; d < C::XD; ++d) uw[1 + d] = u[1 + d] * w[0] + u[0] * w[1 + d];
#pragma unroll
            for (int s = 0; s < C::NS; ++s) {
                const int d = C::sd_dim(s);
                uw[1 + C::XD + s] = u[1 + C::XD + s] * w[0] + 2.0f * u[1 + d] * w[1 + d] + u[0] * w[1 + C::XD + s];
            }
            float* dst = pair_out + (size_t)pos * (2 * C::J);
#pragma unroll
            for (int c = 0; c < C::J; ++c) {
                dst[c] = uw[c];
                dst[C::J + c] = w[c];
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Adjoint.  Per tile of T pairs (one per thread):
//  A (thread = pair): seed -> o-bar through the window product and
//    unnormalisation; recompute layer 1 and, chunk by chunk, layer 2; tanh-jet
//    adjoint -> z2-bar, staged in shared memory with a1 and the small terms.
//  B (thread = pair): v-bar = W2^T z2-bar from its own staged row; layer-1
//    jet adjoint -> z1-bar and the d(cw)-bar terms, staged.
//  C (thread = gradient entry): deterministic sums over the tile's pairs,
//    accumulated per work item in shared memory; written once per item.
// ---------------------------------------------------------------------------
template <class C>
struct AdjT {
    static constexpr int T = (C::H1 >= 32 || C::H2 >= 32) ? 64 : 128;  // pairs per tile = threads
    static constexpr int ZS = ((C::HL * C::J + 7) / 8) * 8 + 4;       // z2-bar row stride (floats)
    static constexpr int AS = C::H1 + 1;                              // a1 row stride
    static constexpr int KB = 4;                                      // W2-bar rows per thread block
    static constexpr int NBLK = C::TWO ? (C::H2 / KB) * C::H1 : 1;    // (k-block, n) outputs
    static constexpr int G = C::TWO ? (T >= NBLK ? T / NBLK : 1) : 1; // t-split groups
    static_assert(!C::TWO || C::H2 % KB == 0, "H2 multiple of 4");
};

template <class C>
struct SAdj {
    float zb[C::TWO ? AdjT<C>::T * AdjT<C>::ZS : 4];  // [t][c][k] z2-bar jets
    float a1[AdjT<C>::T * AdjT<C>::AS];               // [t][n]
    float e3[AdjT<C>::T * (C::HL + 1)];               // [t][k] sum_c obar_c g_c[k]
    float g1[AdjT<C>::T * AdjT<C>::AS];               // [t][n] z1-bar
    float gc[AdjT<C>::T * C::H1 * C::XD + 4];         // [t][n][d] cw-bar
    float xn[AdjT<C>::T * C::XD];
    float ob0[AdjT<C>::T];
    // per-item gradient accumulators
    float gW2[C::TWO ? AdjT<C>::G * C::H2 * C::H1 : 4];
    float gW1[C::H1 * C::XD];
    float gb1[C::H1];
    float gb2[C::TWO ? C::H2 : 4];
    float gW3[C::HL];
    float gb3;
};

template <class C>
__global__ void __launch_bounds__(AdjT<C>::T) adjoint_pairs_kernel(fbp_net net, const float* __restrict__ x,
                                                                   fbp_pairs pr, const float* __restrict__ slot_out,
                                                                   float* __restrict__ grad_part) {
    using A = AdjT<C>;
    constexpr int T = A::T, J = C::J, XD = C::XD, H1 = C::H1, H2 = C::H2, HL = C::HL;
    __shared__ SParams<C> S;
    extern __shared__ float4 dyn_smem[];
    SAdj<C>& R = *reinterpret_cast<SAdj<C>*>(dyn_smem);
    const int tid = threadIdx.x;
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = blockIdx.x; it < nit; it += gridDim.x) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C>(S, net, j);
        // zero the item accumulators
        if constexpr (C::TWO)
            for (int i = tid; i < A::G * H2 * H1; i += T) R.gW2[i] = 0.f;
        for (int i = tid; i < H1 * XD; i += T) R.gW1[i] = 0.f;
        for (int i = tid; i < H1; i += T) R.gb1[i] = 0.f;
        if constexpr (C::TWO)
            for (int i = tid; i < H2; i += T) R.gb2[i] = 0.f;
        for (int i = tid; i < HL; i += T) R.gW3[i] = 0.f;
        if (tid == 0) R.gb3 = 0.f;
        __syncthreads();
        for (int t0 = 0; t0 < cnt; t0 += T) {
            const int nt = min(T, cnt - t0);
            // ---------------- phase A ----------------
            if (tid < nt) {
                const int e = beg + t0 + tid;
                const int pt = pr.sd_point[e];
                const int slot = pr.sd_slot[e];
                float xn[XD];
                load_point<C>(S, x, pt, xn);
                float w[J];
                window_jet<C>(S, xn, w);
                float nb[J];
                const bool ok = slot >= 0 && slot < pr.slots_cap;  // overflowed slots carry no seed
#pragma unroll
                for (int c = 0; c < J; ++c) nb[c] = ok ? slot_out[(size_t)slot * (2 * J) + c] : 0.f;
                // adjoint of uw = u (*) w with w constant: u-bar = M_w^T N-bar
                float ub[J];
                ub[0] = nb[0] * w[0];
#pragma unroll
                for (int d = 0; d < XD; ++d) {
                    ub[0] += nb[1 + d] * w[1 + d];
                    ub[1 + d] = nb[1 + d] * w[0];
                }
#pragma unroll
                for (int s = 0; s < C::NS; ++s) {
                    const int d = C::sd_dim(s);
                    const float g = nb[1 + XD + s];
                    ub[0] += g * w[1 + XD + s];
                    ub[1 + d] += 2.0f * g * w[1 + d];
                    ub[1 + XD + s] = g * w[0];
                }
                float ob[J];
#pragma unroll
                for (int c = 0; c < J; ++c) ob[c] = ub[c] * S.sd_u;
                R.ob0[tid] = ob[0];
#pragma unroll
                for (int d = 0; d < XD; ++d) R.xn[tid * XD + d] = xn[d];
                float* a1row = &R.a1[tid * A::AS];
#pragma unroll 4
                for (int n = 0; n < H1; ++n) a1row[n] = l1_act<C>(S, xn, n);
                if constexpr (C::TWO) {
#pragma unroll 1
                    for (int ch = 0; ch < C::NCH; ++ch) {
                        float acc[C::KC][J];
                        l2_chunk<C>(S, a1row, 1, ch * C::KC, acc);
#pragma unroll
                        for (int k = 0; k < C::KC; ++k) {
                            const int kk = ch * C::KC + k;
                            float g[J], a, tp, tpp;
                            tanh_jet<C>(acc[k], g, a, tp, tpp);
                            float e3 = 0.f;
                            float gb[J];
                            const float w3 = S.W3[kk];
#pragma unroll
                            for (int c = 0; c < J; ++c) {
                                e3 = fmaf(ob[c], g[c], e3);
                                gb[c] = w3 * ob[c];
                            }
                            R.e3[tid * (HL + 1) + kk] = e3;
                            float zb[J];
                            tanh_jet_adj<C>(acc[k], a, tp, tpp, gb, zb);
#pragma unroll
                            for (int c = 0; c < J; ++c) R.zb[tid * A::ZS + c * H2 + kk] = zb[c];
                        }
                    }
                } else {
                    // single hidden layer: output layer reads the layer-1 jets directly
#pragma unroll 2
                    for (int n = 0; n < H1; ++n) {
                        float v[J];
                        l1_jet<C>(S, n, a1row[n], v);
                        float e3 = 0.f;
#pragma unroll
                        for (int c = 0; c < J; ++c) e3 = fmaf(ob[c], v[c], e3);
                        R.e3[tid * (HL + 1) + n] = e3;
                        // v-bar = W3[n] * ob  -> layer-1 jet adjoint
                        const float w3 = S.W3[n];
                        const float a = a1row[n], tp = 1.0f - a * a, tpp = -2.0f * a * tp;
                        float tpb = 0.f, tppb = 0.f;
#pragma unroll
                        for (int d = 0; d < XD; ++d) {
                            const float vb = w3 * ob[1 + d];
                            tpb += vb * S.cw[n * XD + d];
                            R.gc[(tid * H1 + n) * XD + d] = vb * tp;
                        }
#pragma unroll
                        for (int s = 0; s < C::NS; ++s) {
                            const int d = C::sd_dim(s);
                            const float vb = w3 * ob[1 + XD + s];
                            const float cwd = S.cw[n * XD + d];
                            tppb += vb * cwd * cwd;
                            R.gc[(tid * H1 + n) * XD + d] += 2.0f * vb * tpp * cwd;
                        }
                        const float ab = w3 * ob[0] + tpb * (-2.0f * a) + tppb * (6.0f * a * a - 2.0f);
                        R.g1[tid * A::AS + n] = ab * tp;
                    }
                }
            }
            __syncthreads();
            // ---------------- phase B (two hidden layers) ----------------
            if constexpr (C::TWO) {
                if (tid < nt) {
                    const float* zrow = &R.zb[tid * A::ZS];
                    constexpr int NC = 8 < H1 ? 8 : H1;
#pragma unroll 1
                    for (int n0 = 0; n0 < H1; n0 += NC) {
                        float vb[NC][J];
#pragma unroll
                        for (int q = 0; q < NC; ++q)
#pragma unroll
                            for (int c = 0; c < J; ++c) vb[q][c] = 0.f;
#pragma unroll 1
                        for (int k0 = 0; k0 < H2; k0 += 4) {
                            float4 z4[J];
#pragma unroll
                            for (int c = 0; c < J; ++c) z4[c] = *reinterpret_cast<const float4*>(zrow + c * H2 + k0);
#pragma unroll
                            for (int kq = 0; kq < 4; ++kq) {
                                const float* w2 = &S.W2[(k0 + kq) * H1 + n0];
#pragma unroll
                                for (int q = 0; q < NC; ++q) {
                                    const float w = w2[q];
#pragma unroll
                                    for (int c = 0; c < J; ++c) {
                                        const float zc = kq == 0 ? z4[c].x : kq == 1 ? z4[c].y : kq == 2 ? z4[c].z : z4[c].w;
                                        vb[q][c] = fmaf(w, zc, vb[q][c]);
                                    }
                                }
                            }
                        }
#pragma unroll
                        for (int q = 0; q < NC; ++q) {
                            const int n = n0 + q;
                            const float a = R.a1[tid * A::AS + n];
                            const float tp = 1.0f - a * a, tpp = -2.0f * a * tp;
                            float tpb = 0.f, tppb = 0.f;
#pragma unroll
                            for (int d = 0; d < XD; ++d) {
                                tpb += vb[q][1 + d] * S.cw[n * XD + d];
                                R.gc[(tid * H1 + n) * XD + d] = vb[q][1 + d] * tp;
                            }
#pragma unroll
                            for (int s = 0; s < C::NS; ++s) {
                                const int d = C::sd_dim(s);
                                const float g = vb[q][1 + XD + s];
                                const float cwd = S.cw[n * XD + d];
                                tppb += g * cwd * cwd;
                                R.gc[(tid * H1 + n) * XD + d] += 2.0f * g * tpp * cwd;
                            }
                            const float ab = vb[q][0] + tpb * (-2.0f * a) + tppb * (6.0f * a * a - 2.0f);
                            R.g1[tid * A::AS + n] = ab * tp;
                        }
                    }
                }
                __syncthreads();
            }
            // ---------------- phase C: tile reductions ----------------
            if constexpr (C::TWO) {
                // W2-bar[k][n] = sum_t sum_c zb[t][c][k] v_c[t][n],
                // v_0 = a, v_d = t' cw[n][d], v_dd = t'' cw[n][d]^2
                for (int b = tid; b < A::NBLK * A::G; b += T) {
                    const int blk = b % A::NBLK, g = b / A::NBLK;
                    const int n = blk % H1, k0 = (blk / H1) * A::KB;
                    float s[A::KB][J];
#pragma unroll
                    for (int q = 0; q < A::KB; ++q)
#pragma unroll
                        for (int c = 0; c < J; ++c) s[q][c] = 0.f;
                    for (int t = g; t < nt; t += A::G) {
                        const float a = R.a1[t * A::AS + n];
                        const float tp = 1.0f - a * a, tpp = -2.0f * a * tp;
                        const float* zr = &R.zb[t * A::ZS + k0];
#pragma unroll
                        for (int c = 0; c < J; ++c) {
                            const float4 z4 = *reinterpret_cast<const float4*>(zr + c * H2);
                            const float m = (c == 0) ? a : (c <= XD ? tp : tpp);
                            s[0][c] = fmaf(z4.x, m, s[0][c]);
                            s[1][c] = fmaf(z4.y, m, s[1][c]);
                            s[2][c] = fmaf(z4.z, m, s[2][c]);
                            s[3][c] = fmaf(z4.w, m, s[3][c]);
                        }
                    }
#pragma unroll
                    for (int q = 0; q < A::KB; ++q) {
                        float v = s[q][0];
#pragma unroll
                        for (int d = 0; d < XD; ++d) v = fmaf(S.cw[n * XD + d], s[q][1 + d], v);
#pragma unroll
                        for (int ss = 0; ss < C::NS; ++ss) v = fmaf(S.cw2[n * XD + C::sd_dim(ss)], s[q][1 + XD + ss], v);
                        R.gW2[(g * H2 + k0 + q) * H1 + n] += v;
                    }
                }
                // b2-bar[k] = sum_t zb[t][0][k]
                for (int k = tid; k < H2; k += T) {
                    float acc = 0.f;
                    for (int t = 0; t < nt; ++t) acc += R.zb[t * A::ZS + k];
                    R.gb2[k] += acc;
                }
            }
            for (int k = tid; k < HL; k += T) {
                float acc = 0.f;
                for (int t = 0; t < nt; ++t) acc += R.e3[t * (HL + 1) + k];
                R.gW3[k] += acc;
            }
            if (tid == 0) {
                float acc = 0.f;
                for (int t = 0; t < nt; ++t) acc += R.ob0[t];
                R.gb3 += acc;
            }
            for (int n = tid; n < H1; n += T) {
                float sb = 0.f, sw[XD], sc[XD];
#pragma unroll
                for (int d = 0; d < XD; ++d) sw[d] = sc[d] = 0.f;
                for (int t = 0; t < nt; ++t) {
                    const float g = R.g1[t * A::AS + n];
                    sb += g;
#pragma unroll
                    for (int d = 0; d < XD; ++d) {
                        sw[d] = fmaf(g, R.xn[t * XD + d], sw[d]);
                        sc[d] += R.gc[(t * H1 + n) * XD + d];
                    }
                }
                R.gb1[n] += sb;
#pragma unroll
                for (int d = 0; d < XD; ++d) R.gW1[n * XD + d] += sw[d] + sc[d] * S.inv_sd[d];
            }
            __syncthreads();
        }
        // write the item's gradient partial in the packed theta layout
        float* dst = grad_part + (size_t)it * C::P;
        for (int i = tid; i < H1 * XD; i += T) dst[C::oW1 + i] = R.gW1[i];
        for (int i = tid; i < H1; i += T) dst[C::ob1 + i] = R.gb1[i];
        if constexpr (C::TWO) {
            for (int i = tid; i < H2 * H1; i += T) {
                float v = 0.f;
#pragma unroll
                for (int g = 0; g < A::G; ++g) v += R.gW2[g * H2 * H1 + i];
                dst[C::oW2 + i] = v;
            }
            for (int i = tid; i < H2; i += T) dst[C::ob2 + i] = R.gb2[i];
        }
        for (int i = tid; i < HL; i += T) dst[C::oW3 + i] = R.gW3[i];
        if (tid == 0) dst[C::ob3] = R.gb3;
    }
}

}  // namespace fbp
