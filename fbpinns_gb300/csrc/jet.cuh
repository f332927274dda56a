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

// Hidden-layer activations (fbp_net.act): sigma(z) = c f(o z) per neuron, with
// c = o = 1 for the plain FCN and SIREN.  Each keeps one value per first-layer
// neuron in shared memory ("stored": tanh z for the plain tanh, else z) from
// which derivs recovers sigma and its first three derivatives; pgrad gives
// the gradient of the adaptive parameters from the sensitivities of
// (sigma, sigma', sigma'') at z.
template <int ACT>
struct Act;

template <>
struct Act<FBP_ACT_TANH> {  // FCN (fbpinns/networks.py:61-68)
    static constexpr int EXTRA = 0;  // trainable parameters per neuron besides W, b
    __device__ __forceinline__ static float stored(float z, float) { return tanh_fast(z); }
    __device__ __forceinline__ static void derivs(float s, float, float, float& a, float& d1, float& d2, float& d3) {
        a = s;
        d1 = 1.0f - a * a;
        d2 = -2.0f * a * d1;
        d3 = d1 * (6.0f * a * a - 2.0f);
    }
};

template <>
struct Act<FBP_ACT_SIN> {  // SIREN (fbpinns/networks.py:102-131)
    static constexpr int EXTRA = 0;
    __device__ __forceinline__ static float stored(float z, float) { return z; }
    __device__ __forceinline__ static void derivs(float s, float, float, float& a, float& d1, float& d2, float& d3) {
        float sn, cs;
        sincosf(s, &sn, &cs);
        a = sn;
        d1 = cs;
        d2 = -sn;
        d3 = -cs;
    }
};

template <>
struct Act<FBP_ACT_ADAPTIVE_TANH> {  // AdaptiveFCN (fbpinns/networks.py:70-100): a tanh(z / a)
    static constexpr int EXTRA = 1;  // a; here c = a, o = 1 / a
    __device__ __forceinline__ static float stored(float z, float) { return z; }
    __device__ __forceinline__ static void derivs(float s, float c, float o, float& a, float& d1, float& d2,
                                                  float& d3) {
        const float t = tanh_fast(o * s), f1 = 1.0f - t * t;
        a = c * t;
        d1 = c * o * f1;
        d2 = -2.0f * c * o * o * t * f1;
        d3 = c * o * o * o * f1 * (6.0f * t * t - 2.0f);
    }
};

template <>
struct Act<FBP_ACT_ADAPTIVE_SIN> {  // AdaptiveSIREN (fbpinns/networks.py:133-163): c sin(o z)
    static constexpr int EXTRA = 2;  // c, o
    __device__ __forceinline__ static float stored(float z, float) { return z; }
    __device__ __forceinline__ static void derivs(float s, float c, float o, float& a, float& d1, float& d2,
                                                  float& d3) {
        float sn, cs;
        sincosf(o * s, &sn, &cs);
        a = c * sn;
        d1 = c * o * cs;
        d2 = -c * o * o * sn;
        d3 = -c * o * o * o * cs;
    }
};

// Gradient of the adaptive parameters of one neuron for one pair, from the
// sensitivities ab, d1b, d2b of sigma, sigma', sigma'' at the pre-activation z:
//   dL/dc = (ab sigma + d1b sigma' + d2b sigma'') / c
//   dL/do = (ab z sigma' + d1b (sigma' + z sigma'') + d2b (2 sigma'' + z sigma''')) / o
// AdaptiveFCN (c = a, o = 1/a): dL/da = dL/dc - o^2 dL/do;  AdaptiveSIREN: (dL/dc, dL/do).
template <int ACT>
__device__ __forceinline__ void act_param_grad(float ab, float d1b, float d2b, float z, float a, float d1, float d2,
                                               float d3, float c, float o, float (&g)[Act<ACT>::EXTRA > 0 ? Act<ACT>::EXTRA : 1]) {
    if constexpr (Act<ACT>::EXTRA > 0) {
        const float gc = (ab * a + d1b * d1 + d2b * d2) / c;
        const float go = (ab * z * d1 + d1b * (d1 + z * d2) + d2b * (2.0f * d2 + z * d3)) / o;
        if constexpr (ACT == FBP_ACT_ADAPTIVE_TANH) {
            g[0] = gc - o * o * go;
        } else {
            g[0] = gc;
            g[1] = go;
        }
    }
}

// FourierFCN: a sin first layer (the frozen feature map) and a tanh second
// layer; Act<FBP_ACT_FOURIER> is the second layer's rule.
template <>
struct Act<FBP_ACT_FOURIER> : Act<FBP_ACT_TANH> {};

// activation of hidden layer 1 / 2 for an activation code
__host__ __device__ constexpr int act_layer1(int a) { return a == FBP_ACT_FOURIER ? FBP_ACT_SIN : a; }
__host__ __device__ constexpr int act_layer2(int a) { return a == FBP_ACT_FOURIER ? FBP_ACT_TANH : a; }

template <int XD_, int H1_, int H2_, int D2_, int ACT_ = FBP_ACT_TANH>
struct Cfg {
    static constexpr int XD = XD_, H1 = H1_, H2 = H2_, D2 = D2_, ACT = ACT_;
    using AF = Act<act_layer2(ACT_)>;   // second hidden layer (the only one when H2 = 0)
    using AF1 = Act<act_layer1(ACT_)>;  // first hidden layer
    static constexpr bool FROZEN1 = ACT_ == FBP_ACT_FOURIER;  // layer 1 is not trained
    static constexpr int EXTRA = AF::EXTRA;  // per-neuron activation parameters of every layer
    static constexpr int NS = d2_slots(D2);
    static constexpr int J = 1 + XD + NS;
    static constexpr bool TWO = H2 > 0;
    static constexpr int HL = TWO ? H2 : H1;  // width feeding the output layer
    // packed layout per layer: W (fan_out, fan_in), b (fan_out), then EXTRA
    // vectors (fan_out) of activation parameters (the output layer's unused)
    static constexpr int oW1 = 0, ob1 = H1 * XD, oX1 = ob1 + H1;
    static constexpr int oW2 = oX1 + EXTRA * H1;
    static constexpr int ob2 = oW2 + (TWO ? H2 * H1 : 0);
    static constexpr int oX2 = ob2 + (TWO ? H2 : 0);
    static constexpr int oW3 = TWO ? oX2 + EXTRA * H2 : oX1 + EXTRA * H1;
    static constexpr int ob3 = oW3 + HL;
    static constexpr int oX3 = ob3 + 1;
    static constexpr int P = oX3 + EXTRA;
    static constexpr int KC = TWO ? (H2 < 16 ? H2 : 16) : 1;  // layer-2 neurons per register pass
    static constexpr int NCH = TWO ? H2 / KC : 1;
    static_assert(!TWO || H2 % KC == 0, "H2 must be a multiple of the chunk");
    // second-derivative dim of slot s
    // dims whose pure second derivatives slot s sums
    __host__ __device__ static constexpr int slot_dims(int s) { return d2_slot_dims<D2>(s); }
};

// Two independent FP32 FMAs a*b + c in one packed instruction (sm_100 and
// later); each half is rounded exactly like fmaf, so results are unchanged.
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 dup2(float v) { return make_float2(v, v); }

// Work-item schedule of the persistent jet kernels: with pr.item_ctr null CTA b
// takes items b, b + gridDim.x, ...; otherwise each CTA takes the next index
// of the counter (zeroed by the launcher), so a CTA that starts late takes
// fewer items.  All threads of the CTA call these (they contain barriers; the
// index is broadcast through *s_item).
__device__ __forceinline__ int first_item(const fbp_pairs& pr, int* s_item) {
    if (!pr.item_ctr) return blockIdx.x;
    if (threadIdx.x == 0) *s_item = atomicAdd(pr.item_ctr, 1);
    __syncthreads();
    return *s_item;
}
__device__ __forceinline__ int next_item(const fbp_pairs& pr, int it, int* s_item) {
    if (!pr.item_ctr) return it + gridDim.x;
    __syncthreads();  // every thread has read the previous index
    if (threadIdx.x == 0) *s_item = atomicAdd(pr.item_ctr, 1);
    __syncthreads();
    return *s_item;
}

// the sorted pair record (point-major pair index, point, slot, 0)
__device__ __forceinline__ int4 pair_rec(const fbp_pairs& pr, int64_t e) {
    return __ldg(reinterpret_cast<const int4*>(pr.sd_rec) + e);
}

template <class C>
struct SParams {
    float W1[C::H1 * C::XD];
    alignas(16) float b1[C::H1];  // read in pairs by the tensor-core forward
    float cw[C::H1 * C::XD];   // W1[n][d] / sd[d]: first-layer tangent along d
    float c2[C::H1 * (C::NS > 0 ? C::NS : 1)];  // per slot s: sum of cw[n][d]^2 over its dims
    // 16-byte aligned: the layer-2 loops read pairs of neighbouring weights
    alignas(16) float W2t[C::TWO ? C::H1 * C::H2 : 4];  // [n][k]
    alignas(16) float W2[C::TWO ? C::H2 * C::H1 : 4];   // [k][n]
    alignas(16) float b2[C::TWO ? C::H2 : 4];
    alignas(16) float W3[C::HL];
    float b3;
    // activation parameters sigma(z) = c f(o z) of the hidden neurons (adaptive networks)
    float ac1[C::EXTRA > 0 ? C::H1 : 1], ao1[C::EXTRA > 0 ? C::H1 : 1];
    float ac2[C::EXTRA > 0 && C::TWO ? C::H2 : 1], ao2[C::EXTRA > 0 && C::TWO ? C::H2 : 1];
    float mu[C::XD], inv_sd[C::XD], wsc[C::XD];  // wsc = pi / (2 sd)
    // sigmoid window per dim: a = sg0 + sg1 xn, b = sg2 - sg3 xn (window_1d)
    float sg[C::XD][4];
    float flag, mu_u, sd_u;
    int window;
};

// the (c, o) of hidden neuron n of layer 1 (L2 = false) or 2 (L2 = true)
template <class C, bool L2>
__device__ __forceinline__ float act_c(const SParams<C>& S, int n) {
    if constexpr (C::EXTRA == 0) return 1.0f;
    else return L2 ? S.ac2[n] : S.ac1[n];
}
template <class C, bool L2>
__device__ __forceinline__ float act_o(const SParams<C>& S, int n) {
    if constexpr (C::EXTRA == 0) return 1.0f;
    else return L2 ? S.ao2[n] : S.ao1[n];
}

// Subdomain j's weights into shared memory (W2T: also the transposed W2 that
// the CUDA-core layer-2 loops read).
template <class C, bool W2T = true>
__device__ __forceinline__ void load_params(SParams<C>& S, const fbp_net& net, int j) {
    const float* __restrict__ th = net.theta + (size_t)j * C::P;
    for (int i = threadIdx.x; i < C::H1 * C::XD; i += blockDim.x) S.W1[i] = th[C::oW1 + i];
    for (int i = threadIdx.x; i < C::H1; i += blockDim.x) S.b1[i] = th[C::ob1 + i];
    if constexpr (C::TWO) {
        for (int i = threadIdx.x; i < C::H2 * C::H1; i += blockDim.x) {
            const float v = th[C::oW2 + i];
            const int k = i / C::H1, n = i - k * C::H1;
            S.W2[i] = v;
            if constexpr (W2T) S.W2t[n * C::H2 + k] = v;
        }
        for (int i = threadIdx.x; i < C::H2; i += blockDim.x) S.b2[i] = th[C::ob2 + i];
    }
    for (int i = threadIdx.x; i < C::HL; i += blockDim.x) S.W3[i] = th[C::oW3 + i];
    if constexpr (C::EXTRA > 0) {
        // AdaptiveFCN: a (c = a, o = 1/a); AdaptiveSIREN: c then o
        for (int i = threadIdx.x; i < C::H1; i += blockDim.x) {
            const float v = th[C::oX1 + i];
            S.ac1[i] = v;
            S.ao1[i] = C::EXTRA == 1 ? 1.0f / v : th[C::oX1 + C::H1 + i];
        }
        if constexpr (C::TWO) {
            for (int i = threadIdx.x; i < C::H2; i += blockDim.x) {
                const float v = th[C::oX2 + i];
                S.ac2[i] = v;
                S.ao2[i] = C::EXTRA == 1 ? 1.0f / v : th[C::oX2 + C::H2 + i];
            }
        }
    }
    if (threadIdx.x == 0) {
        S.b3 = th[C::ob3];
        S.window = net.window;
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
        if (net.window == FBP_WINDOW_SIGMOID) {
            // ramps of fbpinns/windows.py:11-22 with t = log((1 - tol) / tol), tol = 1e-8:
            // a = (x - mu_min) / sd_min, b = (mu_max - x) / sd_max, written in xn = (x - mu) / sd
            const float t = 18.420680743952367f;
            const float wlo = net.wmins[(size_t)j * C::XD + d], whi = net.wmaxs[(size_t)j * C::XD + d];
            const float ia = 2.0f * t / wlo, ib = 2.0f * t / whi;
            S.sg[d][0] = (S.mu[d] - (lo + wlo / 2.0f)) * ia;  // a at xn = 0
            S.sg[d][1] = sd * ia;                             // da / dxn
            S.sg[d][2] = ((hi - whi / 2.0f) - S.mu[d]) * ib;  // b at xn = 0
            S.sg[d][3] = sd * ib;                             // -db / dxn
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < C::H1 * C::XD; i += blockDim.x) {
        const int d = i % C::XD;
        S.cw[i] = S.W1[i] * S.inv_sd[d];
    }
    __syncthreads();
    if constexpr (C::NS > 0) {
        for (int i = threadIdx.x; i < C::H1 * C::NS; i += blockDim.x) {
            const int n = i / C::NS, s = i - n * C::NS;
            float v = 0.f;
#pragma unroll
            for (int d = 0; d < C::XD; ++d)
                if ((C::slot_dims(s) >> d) & 1) v = fmaf(S.cw[n * C::XD + d], S.cw[n * C::XD + d], v);
            S.c2[i] = v;
        }
        __syncthreads();
    }
}

// Jet of first-layer neuron n's activation from its stored value s.
template <class C>
__device__ __forceinline__ void l1_jet(const SParams<C>& S, int n, float s, float (&v)[C::J]) {
    float tp, tpp, tppp;
    C::AF1::derivs(s, act_c<C, false>(S, n), act_o<C, false>(S, n), v[0], tp, tpp, tppp);
#pragma unroll
    for (int d = 0; d < C::XD; ++d) v[1 + d] = tp * S.cw[n * C::XD + d];
#pragma unroll
    for (int s = 0; s < C::NS; ++s) v[1 + C::XD + s] = tpp * S.c2[n * C::NS + s];
}

// The activation (parameters c, o) applied to a z-jet; a, tp, tpp, tppp are
// sigma and its first three derivatives at z[0].
template <class C>
__device__ __forceinline__ void tanh_jet(const float (&z)[C::J], float (&g)[C::J], float& a, float& tp, float& tpp,
                                         float& tppp, float c = 1.0f, float o = 1.0f) {
    C::AF::derivs(C::AF::stored(z[0], o), c, o, a, tp, tpp, tppp);
    g[0] = a;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) g[1 + d] = tp * z[1 + d];
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        float q = 0.f;
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if ((C::slot_dims(s) >> d) & 1) q = fmaf(z[1 + d], z[1 + d], q);
        g[1 + C::XD + s] = tp * z[1 + C::XD + s] + tpp * q;
    }
}

// Adjoint of tanh_jet: given g-bar, returns z-bar and the sensitivities tpb,
// tppb of sigma', sigma'' (for the adaptive parameters' gradient).
template <class C>
__device__ __forceinline__ void tanh_jet_adj(const float (&z)[C::J], float tp, float tpp, float tppp,
                                             float (&gb)[C::J], float (&zb)[C::J], float& tpb, float& tppb) {
    tpb = 0.f;
    tppb = 0.f;
#pragma unroll
    for (int d = 0; d < C::XD; ++d) {
        tpb += gb[1 + d] * z[1 + d];
        zb[1 + d] = gb[1 + d] * tp;
    }
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        const float g = gb[1 + C::XD + s];
        tpb += g * z[1 + C::XD + s];
        zb[1 + C::XD + s] = g * tp;
        const float g2 = 2.0f * g * tpp;
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if ((C::slot_dims(s) >> d) & 1) {
                tppb += g * z[1 + d] * z[1 + d];
                zb[1 + d] += g2 * z[1 + d];
            }
    }
    zb[0] = gb[0] * tp + tpb * tpp + tppb * tppp;
}

// Window jet (cosine window of fbpinns/windows.py:25-35 times flag plus 1-flag):
// per dim c = cos^4(phi), phi = (pi/2) xn; derivatives by the chain rule.
// The 1D windows other than the cosine (sigmoid, bump, wendland, rbf) of dim
// d at the normalised coordinate xn: value and first two derivatives with
// respect to x.  Kept out of line so that the cosine path, which every
// decomposition of the reference uses, stays straight-line code.
static __device__ __noinline__ float3 window_1d_other(int window, float xn, float is, float4 sg) {
    float c0, c1, c2;
    switch (window) {
        case FBP_WINDOW_SIGMOID: {  // A(a) B(b), A = B = logistic, a = sg.x + sg.y xn, b = sg.z - sg.w xn
            const float a = fmaf(sg.y, xn, sg.x), b = fmaf(-sg.w, xn, sg.z);
            const float A = 1.0f / (1.0f + __expf(-a)), B = 1.0f / (1.0f + __expf(-b));
            const float ka = sg.y * is, kb = sg.w * is;
            const float A1 = A * (1.0f - A) * ka, A2 = A * (1.0f - A) * (1.0f - 2.0f * A) * ka * ka;
            const float B1 = -B * (1.0f - B) * kb, B2 = B * (1.0f - B) * (1.0f - 2.0f * B) * kb * kb;
            c0 = A * B;
            c1 = A1 * B + A * B1;
            c2 = A2 * B + 2.0f * A1 * B1 + A * B2;
            break;
        }
        case FBP_WINDOW_BUMP: {  // e = exp(3 / q + 3), q = xn^2 - 1.001
            const float q = xn * xn - 1.001f, iq = 1.0f / q;
            const float e = __expf(fmaf(3.0f, iq, 3.0f));
            const float h1 = -6.0f * xn * iq * iq, h2 = (-6.0f + 24.0f * xn * xn * iq) * iq * iq;
            c0 = e;
            c1 = e * h1 * is;
            c2 = e * (h2 + h1 * h1) * is * is;
            break;
        }
        case FBP_WINDOW_WENDLAND: {  // (1 - r)^4 (4 r + 1), r = |xn|
            const float r = fabsf(xn), om = 1.0f - r, om2 = om * om;
            c0 = om2 * om2 * (4.0f * r + 1.0f);
            c1 = -20.0f * xn * om2 * om * is;
            c2 = 20.0f * om2 * (4.0f * r - 1.0f) * is * is;
            break;
        }
        default: {  // rbf: exp(-0.5 (xn / 0.25)^2) = exp(-8 xn^2)
            const float g = __expf(-8.0f * xn * xn);
            c0 = g;
            c1 = -16.0f * xn * g * is;
            c2 = (256.0f * xn * xn - 16.0f) * g * is * is;
        }
    }
    return make_float3(c0, c1, c2);
}

// The 1D window of dim d: value and first two derivatives with respect to x.
template <class C>
__device__ __forceinline__ void window_1d(const SParams<C>& S, int d, float xn, float& c0, float& c1, float& c2) {
    if (S.window == FBP_WINDOW_COSINE) {  // cos^4(phi), phi = pi xn / 2
        float sn, cs;
        sincospif(0.5f * xn, &sn, &cs);  // sin, cos of pi (xn / 2): no general range reduction
        const float cs2 = cs * cs;
        const float k = S.wsc[d];
        c0 = cs2 * cs2;
        c1 = -4.0f * cs2 * cs * sn * k;
        c2 = (12.0f * cs2 * sn * sn - 4.0f * cs2 * cs2) * k * k;
    } else {
        const float3 r = window_1d_other(S.window, xn, S.inv_sd[d],
                                         make_float4(S.sg[d][0], S.sg[d][1], S.sg[d][2], S.sg[d][3]));
        c0 = r.x;
        c1 = r.y;
        c2 = r.z;
    }
}

template <class C>
__device__ __forceinline__ void window_jet(const SParams<C>& S, const float (&xn)[C::XD], float (&w)[C::J]) {
    float c0[C::XD], c1[C::XD], c2[C::XD];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) window_1d<C>(S, d, xn[d], c0[d], c1[d], c2[d]);
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
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < C::XD; ++i)
            if ((C::slot_dims(s) >> i) & 1) {
                float p = c2[i];
#pragma unroll
                for (int d = 0; d < C::XD; ++d)
                    if (d != i) p *= c0[d];
                acc += p;
            }
        w[1 + C::XD + s] = f * acc;
    }
}

// Jet of the product u w (first J entries of a pair record).
template <class C>
__device__ __forceinline__ void product_jet(const float (&u)[C::J], const float (&w)[C::J], float* rec) {
    rec[0] = u[0] * w[0];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) rec[1 + d] = u[1 + d] * w[0] + u[0] * w[1 + d];
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        float v = u[1 + C::XD + s] * w[0] + u[0] * w[1 + C::XD + s];
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if ((C::slot_dims(s) >> d) & 1) v += 2.0f * u[1 + d] * w[1 + d];
        rec[1 + C::XD + s] = v;
    }
}

// Adjoint of product_jet in u with w fixed: u-bar = M_w^T n-bar.
template <class C>
__device__ __forceinline__ void product_jet_adj(const float (&nb)[C::J], const float (&w)[C::J], float (&ub)[C::J]) {
    ub[0] = nb[0] * w[0];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) {
        ub[0] += nb[1 + d] * w[1 + d];
        ub[1 + d] = nb[1 + d] * w[0];
    }
#pragma unroll
    for (int s = 0; s < C::NS; ++s) {
        const float g = nb[1 + C::XD + s];
        ub[0] += g * w[1 + C::XD + s];
#pragma unroll
        for (int d = 0; d < C::XD; ++d)
            if ((C::slot_dims(s) >> d) & 1) ub[1 + d] += 2.0f * g * w[1 + d];
        ub[1 + C::XD + s] = g * w[0];
    }
}

template <class C>
__device__ __forceinline__ void load_point(const SParams<C>& S, const float* __restrict__ x, int pt,
                                           float (&xn)[C::XD]) {
#pragma unroll
    for (int d = 0; d < C::XD; ++d) xn[d] = (x[(size_t)pt * C::XD + d] - S.mu[d]) * S.inv_sd[d];
}

// First-layer neuron n at the normalised point: the activation's stored value.
template <class C>
__device__ __forceinline__ float l1_act(const SParams<C>& S, const float (&xn)[C::XD], int n) {
    float z = S.b1[n];
#pragma unroll
    for (int d = 0; d < C::XD; ++d) z = fmaf(S.W1[n * C::XD + d], xn[d], z);
    return C::AF1::stored(z, act_o<C, false>(S, n));
}

// Layer-2 z-jets for neurons [k0, k0+KC) from first-layer activations a1row[n*stride]
// (each thread's own activations, kept in shared memory).
template <class C>
__device__ __forceinline__ void l2_chunk(const SParams<C>& S, const float* a1row, int stride, int k0,
                                         float (&acc)[C::KC][C::J]) {
    // neurons k, k+1 share one packed FMA (fma2: two FP32 FMAs, each rounded like fmaf)
    static_assert(C::KC % 2 == 0 && C::H2 % 2 == 0, "layer-2 neurons in pairs");
    constexpr int K2 = C::KC / 2;
    float2 acc2[K2][C::J];
    const float2* b2 = reinterpret_cast<const float2*>(&S.b2[k0]);
#pragma unroll
    for (int k = 0; k < K2; ++k) {
        acc2[k][0] = b2[k];
#pragma unroll
        for (int c = 1; c < C::J; ++c) acc2[k][c] = make_float2(0.f, 0.f);
    }
#pragma unroll 2
    for (int n = 0; n < C::H1; ++n) {
        float v[C::J];
        l1_jet<C>(S, n, a1row[n * stride], v);
        const float2* wrow = reinterpret_cast<const float2*>(&S.W2t[n * C::H2 + k0]);
#pragma unroll
        for (int k = 0; k < K2; ++k) {
            const float2 w = wrow[k];
#pragma unroll
            for (int c = 0; c < C::J; ++c) acc2[k][c] = fma2(w, make_float2(v[c], v[c]), acc2[k][c]);
        }
    }
#pragma unroll
    for (int k = 0; k < K2; ++k)
#pragma unroll
        for (int c = 0; c < C::J; ++c) {
            acc[2 * k][c] = acc2[k][c].x;
            acc[2 * k + 1][c] = acc2[k][c].y;
        }
}

// Stored layer-2 pre-activation jets (fbp_pairs.zs): component-major, one
// float per (component c, neuron k) row of zs_cap sorted pairs, so that the
// lanes of a warp (consecutive pairs) touch consecutive words.  zs points at
// the pair's column; the rows are written once and read once, with streaming
// (evict-first) accesses.
template <class C>
__device__ __forceinline__ void store_z2(float* __restrict__ zs, int64_t zs_cap, int k0, const float (&acc)[C::KC][C::J]) {
#pragma unroll
    for (int c = 0; c < C::J; ++c)
#pragma unroll
        for (int k = 0; k < C::KC; ++k) __stcs(zs + (size_t)(c * C::H2 + k0 + k) * zs_cap, acc[k][c]);
}
template <class C>
__device__ __forceinline__ void load_z2(const float* __restrict__ zs, int64_t zs_cap, int k0, float (&acc)[C::KC][C::J]) {
#pragma unroll
    for (int c = 0; c < C::J; ++c)
#pragma unroll
        for (int k = 0; k < C::KC; ++k) acc[k][c] = __ldcs(zs + (size_t)(c * C::H2 + k0 + k) * zs_cap);
}

// Network output jet (before unnormalisation) for one pair; a1row/stride is the
// thread's shared-memory slot for its first-layer activations.  With zs set
// (networks with two hidden layers) the layer-2 z-jets are stored there.
template <class C>
__device__ __forceinline__ void net_jet(const SParams<C>& S, const float (&xn)[C::XD], float* a1row, int stride,
                                        float (&out)[C::J], float* __restrict__ zs = nullptr, int64_t zs_cap = 0) {
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
            if (zs) store_z2<C>(zs, zs_cap, ch * C::KC, acc);
#pragma unroll
            for (int k = 0; k < C::KC; ++k) {
                const int kk = ch * C::KC + k;
                float g[C::J], a, tp, tpp, tppp;
                tanh_jet<C>(acc[k], g, a, tp, tpp, tppp, act_c<C, true>(S, kk), act_o<C, true>(S, kk));
                const float w3 = S.W3[kk];
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
__global__ void __launch_bounds__(FWD_THREADS, 3) forward_pairs_kernel(fbp_net net, const float* __restrict__ x,
                                                                     fbp_pairs pr, float* __restrict__ pair_out) {
    constexpr int J = C::J, XD = C::XD, RS = rec_stride(C::J);
    __shared__ SParams<C> S;
    __shared__ float a1s[C::H1 * FWD_THREADS];
    __shared__ int s_item;
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = first_item(pr, &s_item); it < nit; it = next_item(pr, it, &s_item)) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C>(S, net, j);
        // software pipeline: the next pair's indices and coordinates are loaded
        // while the current pair is computed
        int t = threadIdx.x;
        int pos_n = 0;
        float xr_n[XD];
#pragma unroll
        for (int d = 0; d < XD; ++d) xr_n[d] = 0.f;
        if (t < cnt) {
            const int4 r = pair_rec(pr, beg + t);
            const int pt = r.y;
            pos_n = r.x;
#pragma unroll
            for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)pt * XD + d];
        }
        for (; t < cnt; t += blockDim.x) {
            const int pos = pos_n;
            float xn[XD];
#pragma unroll
            for (int d = 0; d < XD; ++d) xn[d] = (xr_n[d] - S.mu[d]) * S.inv_sd[d];
            const int tn = t + blockDim.x;
            if (tn < cnt) {
                const int4 r = pair_rec(pr, beg + tn);
                const int pt = r.y;
                pos_n = r.x;
#pragma unroll
                for (int d = 0; d < XD; ++d) xr_n[d] = x[(size_t)pt * XD + d];
            }
            float o[J];
            net_jet<C>(S, xn, &a1s[threadIdx.x], FWD_THREADS, o, pr.zs ? pr.zs + beg + t : nullptr, pr.zs_cap);
            // unnormalisation (decompositions.py:191-194): u = u_raw*sd + mu
            float u[J];
#pragma unroll
            for (int c = 0; c < J; ++c) u[c] = o[c] * S.sd_u;
            u[0] += S.mu_u;
            float w[J];
            window_jet<C>(S, xn, w);
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
    }
}

// ---------------------------------------------------------------------------
// Adjoint.  Each warp of a CTA walks 32-pair tiles of the CTA's work item on
// its own (only __syncwarp inside an item; the CTA syncs only to load the
// subdomain's weights and to combine the warps' gradient sums at the end):
//  A (lane = pair): seed -> o-bar through the window product and the
//    unnormalisation; recompute layer 1 and, chunk by chunk, layer 2; tanh-jet
//    adjoint -> z2-bar, staged in the warp's shared rows with a1.
//  B (lane = pair): v-bar = W2^T z2-bar from its own row; layer-1 jet adjoint.
//  C (lane = 4x2 block of W2-bar): sum over the tile's pairs from the rows.
// The per-lane gradient terms of W3, W1 and the biases are summed over the
// 32 lanes by a deterministic reduce-scatter butterfly (no shared staging);
// every sum has a fixed order, so results are bitwise reproducible.
// ---------------------------------------------------------------------------
__host__ __device__ constexpr int pow2_at_least(int v) {
    int p = 32;
    while (p < v) p <<= 1;
    return p;
}

#ifndef FBP_ADJ_KB
#define FBP_ADJ_KB 4  // rows of a lane's W2-bar block (2, 4 or 8)
#endif
#ifndef FBP_ADJ_UNROLL_C
#define FBP_ADJ_UNROLL_C 4  // pairs of the tile per unrolled step of the W2-bar loop
#endif

template <class C>
struct AdjW {
    static constexpr int ZS = ((C::HL * C::J + 7) / 8) * 8 + 4;   // z2-bar row stride (floats): 16-B rows,
                                                                  // conflict-free 128-bit access per 8-lane phase
    static constexpr int AS = C::H1 + 1;                          // a1 row stride
    static constexpr int W = ZS <= 96 ? 4 : 2;                    // warps per CTA
    static constexpr int T = 32 * W;
    // W2-bar block per lane: KB rows x NB columns (KB x NB = 8); the sums do
    // not depend on the blocking (each entry adds its pairs in tile order).
    // Activations other than the plain tanh recover sigma, sigma', sigma'' of
    // the block's columns from z with sin/cos or tanh calls per pair, so they
    // take one column (8 x 1)
    static constexpr int KB = C::ACT == FBP_ACT_TANH ? FBP_ADJ_KB : 8, NB = 8 / KB;
    static constexpr int NBLK = C::TWO ? (C::H2 / KB) * (C::H1 / NB) : 0;
    static constexpr int PASSES = C::TWO ? (NBLK + 31) / 32 : 0;
    static_assert(!C::TWO || (C::H2 % KB == 0 && C::H1 % NB == 0), "W2 blocking");
    static_assert(KB == 2 || KB == 4 || KB == 8, "W2-bar rows per lane");
};

// Phase B's layer-1 chunks: NC neurons per reduce-scatter of 32 values, RN
// values each (W1-bar row, b1-bar, activation parameters).  When the
// remaining slots hold NB2 values per chunk (in 4-aligned runs), b2-bar rides
// in them (B2_IN_B) instead of being summed per pair in phase C.
template <class C>
struct AdjB {
    static constexpr int RN = C::XD + 1 + C::EXTRA;
    static constexpr int NCF = 32 / RN >= 8 ? 8 : (32 / RN >= 4 ? 4 : 2);
    static constexpr int NC = NCF < C::H1 ? NCF : C::H1;
    static constexpr int NB2 = C::TWO ? C::H2 * NC / C::H1 : 0;
    static constexpr bool B2_IN_B =
        C::TWO && NB2 > 0 && NB2 % 4 == 0 && NC * RN + NB2 <= 32 && (C::H2 * NC) % C::H1 == 0;
};

// One warp's rows; 16-byte aligned so that every warp's z2-bar rows (read and
// written as float4) start on a 16-byte boundary in the array of WarpRows.
template <class C>
struct __align__(16) WarpRows {
    float zb[C::TWO ? 32 * AdjW<C>::ZS : 4];  // [t][c][k]
    float a1[32 * AdjW<C>::AS];                 // [t][n]
    // warp gradient sums over its tiles of the item
    float gW2[C::TWO ? C::H2 * C::H1 : 4];
    float gW1[C::H1 * C::XD];
    float gb1[C::H1];
    float gb2[C::TWO ? C::H2 : 4];
    float gW3[C::HL];
    float gb3;
    // activation-parameter gradients of the hidden layers (adaptive networks)
    float gX1[C::EXTRA > 0 ? C::EXTRA * C::H1 : 4];
    float gX2[C::EXTRA > 0 && C::TWO ? C::EXTRA * C::H2 : 4];
};

// Reduce-scatter over the warp: v[NV] per lane -> lane L holds the warp sums of
// indices [L*NV/32, (L+1)*NV/32) in v[0 .. NV/32).  With NV = 16 the last
// halving is replaced by a pairwise add: lane L then holds index L/2 (lanes L
// and L^1 hold the same sum).
template <int NV>
__device__ __forceinline__ void warp_reduce_scatter(float (&v)[NV], int lane) {
    static_assert(NV == 32 || NV == 16, "reduce-scatter of 16 or 32 values");
    constexpr int ROUNDS = NV == 32 ? 5 : 4;
#pragma unroll
    for (int r = 0; r < ROUNDS; ++r) {
        const int m = 16 >> r;
        const int half = NV >> (r + 1);
        const bool upper = (lane & m) != 0;
#pragma unroll
        for (int i = 0; i < half; ++i) {
            const float keep = upper ? v[i + half] : v[i];
            const float send = upper ? v[i] : v[i + half];
            v[i] = keep + __shfl_xor_sync(0xffffffffu, send, m);
        }
    }
    if constexpr (NV == 16) v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
}

template <class C>
__global__ void __launch_bounds__(AdjW<C>::T) adjoint_pairs_kernel(fbp_net net, const float* __restrict__ x,
                                                                   fbp_pairs pr, const float* __restrict__ slot_out,
                                                                   float* __restrict__ grad_part) {
    using A = AdjW<C>;
    constexpr int J = C::J, XD = C::XD, H1 = C::H1, H2 = C::H2, HL = C::HL, NW = A::W;
    static_assert(sizeof(WarpRows<C>) % 16 == 0, "warp rows must keep 16-byte alignment");
    static_assert(!C::TWO || (A::ZS % 4 == 0 && H2 % 4 == 0 && C::KC % 4 == 0), "float4 z2-bar rows");
    __shared__ SParams<C> S;
    extern __shared__ float4 dyn_smem[];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    WarpRows<C>& R = reinterpret_cast<WarpRows<C>*>(dyn_smem)[wid];
    __shared__ int s_item;
    const int nit = (int)min((int64_t)*pr.n_items, pr.items_cap);
    for (int it = first_item(pr, &s_item); it < nit; it = next_item(pr, it, &s_item)) {
        const int j = pr.items[3 * (size_t)it], beg = pr.items[3 * (size_t)it + 1], cnt = pr.items[3 * (size_t)it + 2];
        __syncthreads();
        load_params<C>(S, net, j);
        if constexpr (C::TWO)
            for (int i = lane; i < H2 * H1; i += 32) R.gW2[i] = 0.f;
        for (int i = lane; i < H1 * XD; i += 32) R.gW1[i] = 0.f;
        for (int i = lane; i < H1; i += 32) R.gb1[i] = 0.f;
        if constexpr (C::TWO)
            for (int i = lane; i < H2; i += 32) R.gb2[i] = 0.f;
        for (int i = lane; i < HL; i += 32) R.gW3[i] = 0.f;
        if (lane == 0) R.gb3 = 0.f;
        if constexpr (C::EXTRA > 0) {
            for (int i = lane; i < C::EXTRA * H1; i += 32) R.gX1[i] = 0.f;
            if constexpr (C::TWO)
                for (int i = lane; i < C::EXTRA * H2; i += 32) R.gX2[i] = 0.f;
        }
        __syncwarp();
        for (int t0 = wid * 32; t0 < cnt; t0 += A::T) {
            const int nt = min(32, cnt - t0);
            const bool act = lane < nt;
            // ---------------- phase A ----------------
            float ob[J], xn[XD];  // the lane's o-bar jet and normalised point, kept for phase B
#pragma unroll
            for (int c = 0; c < J; ++c) ob[c] = 0.f;
#pragma unroll
            for (int d = 0; d < XD; ++d) xn[d] = 0.f;
            float* a1row = &R.a1[lane * A::AS];
            if (act) {
                const int e = beg + t0 + lane;
                const int4 r = pair_rec(pr, e);
                const int pt = r.y;
                const int slot = r.z;
                load_point<C>(S, x, pt, xn);
                float w[J];
                window_jet<C>(S, xn, w);
                float nb[J];
                {
                    constexpr int RS = rec_stride(J);
                    const bool ok = slot >= 0 && slot < pr.slots_cap;  // overflowed slots carry no seed
                    float rec[(J + 3) / 4 * 4];
                    const float4* src = reinterpret_cast<const float4*>(slot_out + (size_t)(ok ? slot : 0) * RS);
#pragma unroll
                    for (int q = 0; q < (J + 3) / 4; ++q) {
                        const float4 v = src[q];
                        rec[4 * q] = v.x;
                        rec[4 * q + 1] = v.y;
                        rec[4 * q + 2] = v.z;
                        rec[4 * q + 3] = v.w;
                    }
#pragma unroll
                    for (int c = 0; c < J; ++c) nb[c] = ok ? rec[c] : 0.f;
                }
                // adjoint of uw = u (*) w with w constant
                float ub[J];
                product_jet_adj<C>(nb, w, ub);
#pragma unroll
                for (int c = 0; c < J; ++c) ob[c] = ub[c] * S.sd_u;
#pragma unroll 4
                for (int n = 0; n < H1; ++n) a1row[n] = l1_act<C>(S, xn, n);
            }
            // W3-bar terms sum_c o-bar_c g_c[k], chunk by chunk of <= 32 neurons, summed over
            // the warp by a reduce-scatter (lane k of the chunk receives neuron k's sum)
            constexpr int KCH = C::TWO ? C::KC : HL;
#pragma unroll 1
            for (int ch = 0; ch < (C::TWO ? C::NCH : 1); ++ch) {
                constexpr int NE = KCH <= 16 ? 16 : 32;  // values reduce-scattered
                constexpr int NX = C::TWO && C::EXTRA > 0 ? C::EXTRA : 1;
                float e3[NE], ex[NX][NE];  // W3-bar terms; layer-2 activation-parameter terms
#pragma unroll
                for (int k = 0; k < NE; ++k) {
                    e3[k] = 0.f;
#pragma unroll
                    for (int x = 0; x < NX; ++x) ex[x][k] = 0.f;
                }
                if (act) {
                    if constexpr (C::TWO) {
                        float* zrow = &R.zb[lane * A::ZS];
                        float acc[C::KC][J];
                        if (pr.zs)  // stored by the forward of the same lists
                            load_z2<C>(pr.zs + beg + t0 + lane, pr.zs_cap, ch * C::KC, acc);
                        else
                            l2_chunk<C>(S, a1row, 1, ch * C::KC, acc);
#pragma unroll
                        for (int k = 0; k < C::KC; ++k) {
                            const int kk = ch * C::KC + k;
                            const float ck = act_c<C, true>(S, kk), ok = act_o<C, true>(S, kk);
                            float g[J], a, tp, tpp, tppp;
                            tanh_jet<C>(acc[k], g, a, tp, tpp, tppp, ck, ok);
                            float gb[J];
                            const float w3 = S.W3[kk];
                            float s3 = 0.f;
#pragma unroll
                            for (int c = 0; c < J; ++c) {
                                s3 = fmaf(ob[c], g[c], s3);
                                gb[c] = w3 * ob[c];
                            }
                            e3[k] = s3;
                            float zb[J], tpb, tppb;
                            tanh_jet_adj<C>(acc[k], tp, tpp, tppp, gb, zb, tpb, tppb);
                            if constexpr (C::EXTRA > 0) {
                                float pg[C::EXTRA];
                                act_param_grad<C::ACT>(gb[0], tpb, tppb, acc[k][0], a, tp, tpp, tppp, ck, ok, pg);
#pragma unroll
                                for (int x = 0; x < C::EXTRA; ++x) ex[x][k] = pg[x];
                            }
#pragma unroll
                            for (int c = 0; c < J; ++c) acc[k][c] = zb[c];
                        }
#pragma unroll
                        for (int c = 0; c < J; ++c)
#pragma unroll
                            for (int q = 0; q < C::KC; q += 4)
                                *reinterpret_cast<float4*>(zrow + c * H2 + ch * C::KC + q) =
                                    make_float4(acc[q][c], acc[q + 1][c], acc[q + 2][c], acc[q + 3][c]);
                    } else {
#pragma unroll
                        for (int n = 0; n < H1; ++n) {
                            float v[J];
                            l1_jet<C>(S, n, a1row[n], v);
                            float s3 = 0.f;
#pragma unroll
                            for (int c = 0; c < J; ++c) s3 = fmaf(ob[c], v[c], s3);
                            e3[n] = s3;
                        }
                    }
                }
                warp_reduce_scatter<NE>(e3, lane);
                if constexpr (NE == 16) {
                    if (!(lane & 1) && (lane >> 1) < KCH) R.gW3[ch * KCH + (lane >> 1)] += e3[0];
                } else {
                    if (lane < KCH) R.gW3[ch * KCH + lane] += e3[0];
                }
                if constexpr (C::TWO && C::EXTRA > 0) {
#pragma unroll
                    for (int x = 0; x < C::EXTRA; ++x) {
                        warp_reduce_scatter<NE>(ex[x], lane);
                        if constexpr (NE == 16) {
                            if (!(lane & 1) && (lane >> 1) < KCH) R.gX2[x * H2 + ch * KCH + (lane >> 1)] += ex[x][0];
                        } else {
                            if (lane < KCH) R.gX2[x * H2 + ch * KCH + lane] += ex[x][0];
                        }
                    }
                }
            }
            const float ob0 = ob[0];
            float b3 = ob0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) b3 += __shfl_xor_sync(0xffffffffu, b3, o);
            if (lane == 0) R.gb3 += b3;
            __syncwarp();
            // ---------------- phase B: layer-1 adjoint ----------------
            // per chunk of NC first-layer neurons: v-bar = W2^T z2-bar (own row), the
            // layer-1 jet adjoint, and the W1-bar / b1-bar terms summed over the warp
            constexpr int RN = AdjB<C>::RN, NC = AdjB<C>::NC, NB2 = AdjB<C>::NB2;
            constexpr bool B2_IN_B = AdjB<C>::B2_IN_B;  // b2-bar rides in the free slots
            static_assert(NC * RN <= 32 && H1 % NC == 0, "layer-1 chunk must fit one reduce-scatter");
#pragma unroll 1
            for (int n0 = 0; n0 < H1; n0 += NC) {
                float r1[32];
#pragma unroll
                for (int i = 0; i < 32; ++i) r1[i] = 0.f;
                if (act) {
                    float vb[NC][J];
                    if constexpr (C::TWO) {
                        // first-layer neurons q, q+1 share one packed FMA
                        static_assert(NC % 2 == 0, "layer-1 neurons in pairs");
                        float2 vb2[NC / 2][J];
#pragma unroll
                        for (int q = 0; q < NC / 2; ++q)
#pragma unroll
                            for (int c = 0; c < J; ++c) vb2[q][c] = make_float2(0.f, 0.f);
                        const float* zrow = &R.zb[lane * A::ZS];
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
                        for (int q = 0; q < NC / 2; ++q)
#pragma unroll
                            for (int c = 0; c < J; ++c) {
                                vb[2 * q][c] = vb2[q][c].x;
                                vb[2 * q + 1][c] = vb2[q][c].y;
                            }
                    } else {
#pragma unroll
                        for (int q = 0; q < NC; ++q) {
                            const float w3 = S.W3[n0 + q];
#pragma unroll
                            for (int c = 0; c < J; ++c) vb[q][c] = w3 * ob[c];
                        }
                    }
#pragma unroll
                    for (int q = 0; q < NC; ++q) {
                        const int n = n0 + q;
                        const float cn = act_c<C, false>(S, n), on = act_o<C, false>(S, n);
                        float a, tp, tpp, tppp;
                        C::AF1::derivs(a1row[n], cn, on, a, tp, tpp, tppp);
                        float tpb = 0.f, tppb = 0.f, cwb[XD];
#pragma unroll
                        for (int d = 0; d < XD; ++d) {
                            tpb += vb[q][1 + d] * S.cw[n * XD + d];
                            cwb[d] = vb[q][1 + d] * tp;
                        }
#pragma unroll
                        for (int s = 0; s < C::NS; ++s) {
                            const float g = vb[q][1 + XD + s];
                            tppb += g * S.c2[n * C::NS + s];
#pragma unroll
                            for (int d = 0; d < XD; ++d)
                                if ((C::slot_dims(s) >> d) & 1) cwb[d] += 2.0f * g * tpp * S.cw[n * XD + d];
                        }
                        const float z1b = vb[q][0] * tp + tpb * tpp + tppb * tppp;
#pragma unroll
                        for (int d = 0; d < XD; ++d) r1[q * RN + d] = fmaf(z1b, xn[d], cwb[d] * S.inv_sd[d]);
                        r1[q * RN + XD] = z1b;
                        if constexpr (C::EXTRA > 0) {
                            // the stored value of an adaptive activation is the pre-activation z
                            float pg[C::EXTRA];
                            act_param_grad<C::ACT>(vb[q][0], tpb, tppb, a1row[n], a, tp, tpp, tppp, cn, on, pg);
#pragma unroll
                            for (int x = 0; x < C::EXTRA; ++x) r1[q * RN + XD + 1 + x] = pg[x];
                        }
                    }
                    if constexpr (B2_IN_B) {  // this chunk's b2-bar terms: z2-bar_0 of NB2 neurons
                        const float* zrow = &R.zb[lane * A::ZS];
                        const int kb0 = (n0 / NC) * NB2;
#pragma unroll
                        for (int i = 0; i < NB2; i += 4) {
                            const float4 z4 = *reinterpret_cast<const float4*>(zrow + kb0 + i);
                            r1[NC * RN + i] = z4.x;
                            r1[NC * RN + i + 1] = z4.y;
                            r1[NC * RN + i + 2] = z4.z;
                            r1[NC * RN + i + 3] = z4.w;
                        }
                    }
                }
                warp_reduce_scatter<32>(r1, lane);
                if (lane < NC * RN) {
                    const int q = lane / RN, d = lane - q * RN;
                    if (d < XD)
                        R.gW1[(n0 + q) * XD + d] += r1[0];
                    else if (d == XD)
                        R.gb1[n0 + q] += r1[0];
                    else if constexpr (C::EXTRA > 0)
                        R.gX1[(d - XD - 1) * H1 + n0 + q] += r1[0];
                } else if (B2_IN_B && lane < NC * RN + NB2) {
                    R.gb2[(n0 / NC) * NB2 + lane - NC * RN] += r1[0];
                }
            }
            // ---------------- phase C: W2-bar over the tile ----------------
            // (b2-bar here only when phase B's reduce-scatters have no room for it)
            constexpr bool B2_IN_C = !AdjB<C>::B2_IN_B;
            if constexpr (C::TWO) {
#pragma unroll 1
                for (int ps = 0; ps < A::PASSES; ++ps) {
                    const int b = ps * 32 + lane;
                    if (b < A::NBLK) {
                        const int nb = b % (H1 / A::NB), kb = b / (H1 / A::NB);
                        const int n0 = nb * A::NB, k0 = kb * A::KB;
                        // rows k0+2i, k0+2i+1 of the block share one packed FMA
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
                        constexpr int UC = FBP_ADJ_UNROLL_C;
#pragma unroll UC
                        for (int t = 0; t < nt; ++t) {
                            float m[A::NB][3];
#pragma unroll
                            for (int q = 0; q < A::NB; ++q) {
                                float a, tp, tpp, tppp;
                                C::AF1::derivs(R.a1[t * A::AS + n0 + q], act_c<C, false>(S, n0 + q),
                                              act_o<C, false>(S, n0 + q), a, tp, tpp, tppp);
                                m[q][0] = a;
                                m[q][1] = tp;
                                m[q][2] = tpp;
                            }
                            const float* zr = &R.zb[t * A::ZS + k0];
#pragma unroll
                            for (int c = 0; c < J; ++c) {
                                float2 z2[A::KB / 2];  // rows k0 .. k0+KB of z2-bar component c
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
                                if (B2_IN_C && c == 0) {
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
                                for (int ss = 0; ss < C::NS; ++ss)
                                    v = fmaf(S.c2[n * C::NS + ss], s[1 + XD + ss], v);
                                R.gW2[(k0 + i) * H1 + n] += v;
                            }
                        if (B2_IN_C && nb == 0) {
#pragma unroll
                            for (int i = 0; i < A::KB; ++i) R.gb2[k0 + i] += b2s[i];
                        }
                    }
                }
            }
            __syncwarp();
        }
        __syncthreads();
        // combine the warps' sums (fixed warp order) into the item's gradient partial
        float* dst = grad_part + (size_t)it * C::P;
        WarpRows<C>* RW = reinterpret_cast<WarpRows<C>*>(dyn_smem);
        for (int i = tid; i < H1 * XD; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gW1[i];
            dst[C::oW1 + i] = C::FROZEN1 ? 0.f : v;
        }
        for (int i = tid; i < H1; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gb1[i];
            dst[C::ob1 + i] = C::FROZEN1 ? 0.f : v;
        }
        if constexpr (C::TWO) {
            for (int i = tid; i < H2 * H1; i += blockDim.x) {
                float v = 0.f;
#pragma unroll
                for (int w = 0; w < NW; ++w) v += RW[w].gW2[i];
                dst[C::oW2 + i] = v;
            }
            for (int i = tid; i < H2; i += blockDim.x) {
                float v = 0.f;
#pragma unroll
                for (int w = 0; w < NW; ++w) v += RW[w].gb2[i];
                dst[C::ob2 + i] = v;
            }
        }
        for (int i = tid; i < HL; i += blockDim.x) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gW3[i];
            dst[C::oW3 + i] = v;
        }
        if (tid == 0) {
            float v = 0.f;
#pragma unroll
            for (int w = 0; w < NW; ++w) v += RW[w].gb3;
            dst[C::ob3] = v;
        }
        if constexpr (C::EXTRA > 0) {
            for (int i = tid; i < C::EXTRA * H1; i += blockDim.x) {
                float v = 0.f;
#pragma unroll
                for (int w = 0; w < NW; ++w) v += RW[w].gX1[i];
                dst[C::oX1 + i] = v;
            }
            if constexpr (C::TWO) {
                for (int i = tid; i < C::EXTRA * H2; i += blockDim.x) {
                    float v = 0.f;
#pragma unroll
                    for (int w = 0; w < NW; ++w) v += RW[w].gX2[i];
                    dst[C::oX2 + i] = v;
                }
            }
            if (tid < C::EXTRA) dst[C::oX3 + tid] = 0.f;  // the output layer's parameters are unused
        }
    }
}

}  // namespace fbp
