// Partition-of-unity combination of the per-pair jets, the built-in hard
// constraints and PDE residuals, the FP64 loss reduction, the adjoint seeds,
// and the per-subdomain gradient reduction.
//
// Per point p the reference computes (fbpinns/trainers.py:162-174)
//   U_l = (sum_{pairs of level l} u_j w_j) / (sum w_j),  U = sum_l U_l / npou,
// then constraining_fn.  Here the same is done on jets:
//   U_l   = N/W,
//   U_l,d = (N_d - U_l W_d) / W,
//   U_l,dd = (N_dd - 2 U_l,d W_d - U_l W_dd) / W,
// one thread per point, reading its pairs (contiguous in the point-major
// order), with the levels of a point in ascending runs.
#include <algorithm>

#include "common.cuh"

namespace fbp {

template <int XD, int D2>
struct JL {
    static constexpr int M = D2 & 7;           // dims with second derivatives
    static constexpr int G = d2_group(D2);     // dims summed in the group's slot
    static constexpr int SG = d2_singles(D2);  // dims with a slot each
    static constexpr int NS = d2_slots(D2);
    static constexpr int J = 1 + XD + NS;
    // dims whose pure second derivatives slot s sums
    __host__ __device__ static constexpr int slot_dims(int s) { return d2_slot_dims<D2>(s); }
    // component of the pure second derivative along d (-1 if absent or summed)
    static constexpr int SB = 1 + XD + (G ? 1 : 0);  // first single-dim slot
    static constexpr int S0 = ((SG >> 0) & 1) ? SB : -1;
    static constexpr int S1 = ((SG >> 1) & 1) ? SB + popc_const(SG & 1) : -1;
    static constexpr int S2 = ((SG >> 2) & 1) ? SB + popc_const(SG & 3) : -1;
    __host__ __device__ static constexpr int sidx(int d) { return d == 0 ? S0 : (d == 1 ? S1 : S2); }
    // component of the group's sum of second derivatives (-1 without a group)
    static constexpr int LAPI = G ? 1 + XD : -1;
};

template <int XD, int D2>
__device__ __forceinline__ void quotient(const float (&N)[JL<XD, D2>::J], const float (&W)[JL<XD, D2>::J],
                                         float (&U)[JL<XD, D2>::J]) {
    using L = JL<XD, D2>;
    const float r = 1.0f / W[0];
    U[0] = N[0] * r;
#pragma unroll
    for (int d = 0; d < XD; ++d) U[1 + d] = (N[1 + d] - U[0] * W[1 + d]) * r;
#pragma unroll
    for (int s = 0; s < L::NS; ++s) {
        float v = N[1 + XD + s] - U[0] * W[1 + XD + s];
#pragma unroll
        for (int d = 0; d < XD; ++d)
            if ((L::slot_dims(s) >> d) & 1) v -= 2.0f * U[1 + d] * W[1 + d];
        U[1 + XD + s] = v * r;
    }
}

// adjoint of quotient with W fixed: Ub -> Nb
template <int XD, int D2>
__device__ __forceinline__ void quotient_adj(const float (&W)[JL<XD, D2>::J], const float (&Ub)[JL<XD, D2>::J],
                                             float (&Nb)[JL<XD, D2>::J]) {
    using L = JL<XD, D2>;
    const float r = 1.0f / W[0];
    float ud[XD];
#pragma unroll
    for (int d = 0; d < XD; ++d) ud[d] = Ub[1 + d];
    float u0 = Ub[0];
#pragma unroll
    for (int s = 0; s < L::NS; ++s) {
        const float g = Ub[1 + XD + s];
        Nb[1 + XD + s] = g * r;
#pragma unroll
        for (int d = 0; d < XD; ++d)
            if ((L::slot_dims(s) >> d) & 1) ud[d] -= 2.0f * g * W[1 + d] * r;
        u0 -= g * W[1 + XD + s] * r;
    }
#pragma unroll
    for (int d = 0; d < XD; ++d) {
        Nb[1 + d] = ud[d] * r;
        u0 -= ud[d] * W[1 + d] * r;
    }
    Nb[0] = u0 * r;
}

// ---------------------------------------------------------------------------
// built-in hard-constraint ansatz  uc = A(x) + B(x) u   and residuals
// ---------------------------------------------------------------------------
struct J1 {
    float v, d, dd;
};

__device__ __forceinline__ J1 tanh_lin(float x, float a, float b) {  // tanh(a x + b)
    const float t = tanhf(a * x + b);
    const float s = 1.0f - t * t;
    return {t, s * a, -2.0f * t * s * a * a};
}

__device__ __forceinline__ J1 jmul(J1 p, J1 q) { return {p.v * q.v, p.d * q.v + p.v * q.d, p.dd * q.v + 2.0f * p.d * q.d + p.v * q.dd}; }

// Write a separable product's jet: B = prod_d f_d(x_d)
template <int XD, int D2>
__device__ __forceinline__ void sep_jet(const J1 (&f)[XD], float (&B)[JL<XD, D2>::J]) {
    using L = JL<XD, D2>;
    float p = 1.f;
#pragma unroll
    for (int d = 0; d < XD; ++d) p *= f[d].v;
    B[0] = p;
#pragma unroll
    for (int i = 0; i < XD; ++i) {
        float q = f[i].d;
#pragma unroll
        for (int d = 0; d < XD; ++d)
            if (d != i) q *= f[d].v;
        B[1 + i] = q;
    }
#pragma unroll
    for (int s = 0; s < L::NS; ++s) {
        float acc = 0.f;
#pragma unroll
        for (int i = 0; i < XD; ++i)
            if ((L::slot_dims(s) >> i) & 1) {
                float q = f[i].dd;
#pragma unroll
                for (int d = 0; d < XD; ++d)
                    if (d != i) q *= f[d].v;
                acc += q;
            }
        B[1 + XD + s] = acc;
    }
}

template <int XD, int D2>
__device__ __forceinline__ void ansatz(const fbp_problem& P, const float* xp, float (&A)[JL<XD, D2>::J],
                                       float (&B)[JL<XD, D2>::J]) {
    constexpr int J = JL<XD, D2>::J;
#pragma unroll
    for (int c = 0; c < J; ++c) A[c] = 0.f, B[c] = 0.f;
    switch (P.kind) {
        case FBP_PROBLEM_HO_HARDBC: {  // problems.py:189-195: 1 + tanh(t/sd)^2 u
            if constexpr (XD == 1) {
                const J1 t = tanh_lin(xp[0], 1.0f / P.p[0], 0.f);
                J1 f[1] = {jmul(t, t)};
                sep_jet<XD, D2>(f, B);
                A[0] = 1.0f;
            }
            break;
        }
        case FBP_PROBLEM_BURGERS: {  // problems.py:315-319
            if constexpr (XD == 2) {
                const float sdi = 1.0f / P.p[0];
                const J1 f1 = tanh_lin(xp[0], sdi, sdi);     // tanh((x+1)/sd)
                const J1 f2 = tanh_lin(xp[0], -sdi, sdi);    // tanh((1-x)/sd)
                const J1 f3 = tanh_lin(xp[1], sdi, 0.f);     // tanh(t/sd)
                J1 f[2] = {jmul(f1, f2), f3};
                sep_jet<XD, D2>(f, B);
                float sn, cs;
                sincospif(xp[0], &sn, &cs);
                const float pi = 3.14159265358979323846f;
                // A = -sin(pi x)
                J1 a[2] = {{-sn, -pi * cs, pi * pi * sn}, {1.f, 0.f, 0.f}};
                sep_jet<XD, D2>(a, A);
            }
            break;
        }
        case FBP_PROBLEM_POISSON2D:
        case FBP_PROBLEM_HELMHOLTZ2D: {  // tanh(x/sd) tanh((1-x)/sd) tanh(y/sd) tanh((1-y)/sd) u
            if constexpr (XD == 2) {
                const float sdi = 1.0f / P.p[0];
                J1 f[2];
#pragma unroll
                for (int d = 0; d < 2; ++d) f[d] = jmul(tanh_lin(xp[d], sdi, 0.f), tanh_lin(xp[d], -sdi, sdi));
                sep_jet<XD, D2>(f, B);
            }
            break;
        }
        case FBP_PROBLEM_WAVE_C: {  // problems.py:383-398
            if constexpr (XD == 3) {
                const float t1 = P.p[1];
                // B = tanh(2.5 t / t1)^2 (function of t only)
                const J1 tt = tanh_lin(xp[2], 2.5f / t1, 0.f);
                J1 fb[3] = {{1.f, 0.f, 0.f}, {1.f, 0.f, 0.f}, jmul(tt, tt)};
                sep_jet<XD, D2>(fb, B);
                // A = E(t) * sum_g amp exp(-0.5 |x - m|^2 / s^2)
                const float q = 1.5f / t1;
                const float e = expf(-0.5f * (q * xp[2]) * (q * xp[2]));
                const J1 E = {e, -q * q * xp[2] * e, (q * q * q * q * xp[2] * xp[2] - q * q) * e};
                float Ab[JL<XD, D2>::J];
#pragma unroll
                for (int c = 0; c < J; ++c) Ab[c] = 0.f;
                for (int g = 0; g < P.ng; ++g) {
                    const float mx = P.gauss[4 * g], my = P.gauss[4 * g + 1], s = P.gauss[4 * g + 2], amp = P.gauss[4 * g + 3];
                    const float is2 = 1.0f / (s * s);
                    const float dx = xp[0] - mx, dy = xp[1] - my;
                    const float ex = expf(-0.5f * dx * dx * is2), ey = expf(-0.5f * dy * dy * is2);
                    J1 f[3] = {{amp * ex, -amp * dx * is2 * ex, amp * (dx * dx * is2 - 1.0f) * is2 * ex},
                               {ey, -dy * is2 * ey, (dy * dy * is2 - 1.0f) * is2 * ey},
                               E};
                    float t[JL<XD, D2>::J];
                    sep_jet<XD, D2>(f, t);
#pragma unroll
                    for (int c = 0; c < J; ++c) Ab[c] += t[c];
                }
#pragma unroll
                for (int c = 0; c < J; ++c) A[c] = Ab[c];
            }
            break;
        }
        default: {  // identity
            B[0] = 1.0f;
            break;
        }
    }
}

// residual r(uc) and dr/duc
template <int XD, int D2>
__device__ __forceinline__ float residual(const fbp_problem& P, const float* xp, const float (&u)[JL<XD, D2>::J],
                                          float (&dr)[JL<XD, D2>::J]) {
    using L = JL<XD, D2>;
    constexpr int J = L::J;
#pragma unroll
    for (int c = 0; c < J; ++c) dr[c] = 0.f;
    float r = 0.f;
    switch (P.kind) {
        case FBP_PROBLEM_HO_HARDBC: {  // problems.py:198-206: u_tt + mu u_t + k u
            if constexpr (XD == 1 && L::sidx(0) > 0) {
                const float mu = P.p[1], k = P.p[2];
                r = u[L::sidx(0)] + mu * u[1] + k * u[0];
                dr[L::sidx(0)] = 1.f;
                dr[1] = mu;
                dr[0] = k;
            }
            break;
        }
        case FBP_PROBLEM_BURGERS: {  // problems.py:322-326: u_t + u u_x - nu u_xx
            if constexpr (XD == 2 && L::sidx(0) > 0) {
                const float nu = P.p[1];
                r = u[2] + u[0] * u[1] - nu * u[L::sidx(0)];
                dr[2] = 1.f;
                dr[0] = u[1];
                dr[1] = u[0];
                dr[L::sidx(0)] = -nu;
            }
            break;
        }
        case FBP_PROBLEM_POISSON2D: {  // u_xx + u_yy + f
            if constexpr (XD == 2 && L::LAPI > 0 && L::G == 3) {
                float f = 0.f;
                for (int k = 1; k <= P.n_int; ++k) {
                    const float a = (float)(1 << k);
                    f += 2.0f * a * 9.869604401089358f * sinpif(a * xp[0]) * sinpif(a * xp[1]);
                }
                r = u[L::LAPI] + f;
                dr[L::LAPI] = 1.f;
            }
            if constexpr (XD == 2 && L::sidx(0) > 0 && L::sidx(1) > 0) {
                float f = 0.f;
                for (int k = 1; k <= P.n_int; ++k) {
                    const float a = (float)(1 << k);
                    f += 2.0f * a * 9.869604401089358f * sinpif(a * xp[0]) * sinpif(a * xp[1]);
                }
                r = u[L::sidx(0)] + u[L::sidx(1)] + f;
                dr[L::sidx(0)] = 1.f;
                dr[L::sidx(1)] = 1.f;
            }
            break;
        }
        case FBP_PROBLEM_HELMHOLTZ2D: {  // u_xx + u_yy + k^2 u + f
            if constexpr (XD == 2 && L::LAPI > 0 && L::G == 3) {
                const float k = P.p[1];
                float f = 0.f;
                for (int g = 0; g < P.ng; ++g) {
                    const float mx = P.gauss[4 * g], my = P.gauss[4 * g + 1], s = P.gauss[4 * g + 2], amp = P.gauss[4 * g + 3];
                    const float dx = xp[0] - mx, dy = xp[1] - my;
                    f += amp * expf(-0.5f * (dx * dx + dy * dy) / (s * s));
                }
                r = u[L::LAPI] + k * k * u[0] + f;
                dr[L::LAPI] = 1.f;
                dr[0] = k * k;
            }
            if constexpr (XD == 2 && L::sidx(0) > 0 && L::sidx(1) > 0) {
                const float k = P.p[1];
                float f = 0.f;
                for (int g = 0; g < P.ng; ++g) {
                    const float mx = P.gauss[4 * g], my = P.gauss[4 * g + 1], s = P.gauss[4 * g + 2], amp = P.gauss[4 * g + 3];
                    const float dx = xp[0] - mx, dy = xp[1] - my;
                    f += amp * expf(-0.5f * (dx * dx + dy * dy) / (s * s));
                }
                r = u[L::sidx(0)] + u[L::sidx(1)] + k * k * u[0] + f;
                dr[L::sidx(0)] = 1.f;
                dr[L::sidx(1)] = 1.f;
                dr[0] = k * k;
            }
            break;
        }
        case FBP_PROBLEM_WAVE_C: {  // problems.py:401-405: u_xx + u_yy - u_tt / c^2
            if constexpr (XD == 3 && L::LAPI > 0 && L::G == 3 && L::sidx(2) > 0) {  // (u_xx + u_yy), u_tt
                const float ic2 = 1.0f / (P.p[0] * P.p[0]);
                r = u[L::LAPI] - ic2 * u[L::sidx(2)];
                dr[L::LAPI] = 1.f;
                dr[L::sidx(2)] = -ic2;
            }
            if constexpr (XD == 3 && L::sidx(0) > 0 && L::sidx(1) > 0 && L::sidx(2) > 0) {
                const float ic2 = 1.0f / (P.p[0] * P.p[0]);
                r = u[L::sidx(0)] + u[L::sidx(1)] - ic2 * u[L::sidx(2)];
                dr[L::sidx(0)] = 1.f;
                dr[L::sidx(1)] = 1.f;
                dr[L::sidx(2)] = -ic2;
            }
            break;
        }
        default:
            break;
    }
    return r;
}

constexpr int POU_T = 256;

template <int XD, int D2>
struct PointPOU {
    static constexpr int J = JL<XD, D2>::J;
    static constexpr int RS = rec_stride(J);  // row stride of pair and slot records
    // forward POU for point p; writes slot records; returns U (unconstrained)
    __device__ static void run(int64_t p, int npou, const int32_t* __restrict__ pt_off,
                               const int32_t* __restrict__ p_take, const float* __restrict__ pair_out,
                               float* __restrict__ slot_out, float (&U)[J], int64_t s_cap, int64_t u_cap,
                               int32_t* status) {
        float N[J], W[J], Ul[J];
#pragma unroll
        for (int c = 0; c < J; ++c) U[c] = 0.f;
        const int e0 = (int)min((int64_t)pt_off[p], s_cap), e1 = (int)min((int64_t)pt_off[p + 1], s_cap);
        int cur = -1;
        // the pairs in groups of PU whose loads are issued together; the sums
        // run in pair order as one pair at a time would
        constexpr int PU = 4;
        for (int eb = e0; eb <= e1; eb += PU) {
            int rr[PU];
            float rec[PU][RS];
#pragma unroll
            for (int q = 0; q < PU; ++q) {
                const int e = eb + q;
                rr[q] = e < e1 ? p_take[e] : -2;
                if (e < e1) {
                    const float4* po = reinterpret_cast<const float4*>(pair_out + (size_t)e * RS);
#pragma unroll
                    for (int h = 0; h < RS / 4; ++h) {
                        const float4 v = po[h];
                        rec[q][4 * h] = v.x;
                        rec[q][4 * h + 1] = v.y;
                        rec[q][4 * h + 2] = v.z;
                        rec[q][4 * h + 3] = v.w;
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < PU; ++q) {
                const int e = eb + q;
                if (e > e1) break;
                const int r = rr[q];
                if (r != cur) {
                    if (cur >= 0) {
                        quotient<XD, D2>(N, W, Ul);
#pragma unroll
                        for (int c = 0; c < J; ++c) U[c] += Ul[c];
                        if (cur < u_cap) {
                            float* so = slot_out + (size_t)cur * RS;
#pragma unroll
                            for (int c = 0; c < J; ++c) {
                                so[c] = Ul[c];
                                so[J + c] = W[c];
                            }
                        }
                    }
                    if (r >= 0 && r < cur) atomicOr(status, FBP_STATUS_LEVEL_ORDER);
                    cur = r;
#pragma unroll
                    for (int c = 0; c < J; ++c) N[c] = W[c] = 0.f;
                }
                if (e < e1) {
#pragma unroll
                    for (int c = 0; c < J; ++c) {
                        N[c] += rec[q][c];
                        W[c] += rec[q][J + c];
                    }
                }
            }
        }
        const float inv = 1.0f / (float)npou;
#pragma unroll
        for (int c = 0; c < J; ++c) U[c] *= inv;
    }

    // seeds: dL/dU (point) -> dL/dN per slot (overwrites the U_l half of each record)
    __device__ static void seed(int64_t p, int npou, const int32_t* __restrict__ np_off, const float (&Ub)[J],
                                float* __restrict__ slot_out, int64_t u_cap) {
        const float inv = 1.0f / (float)npou;
        float ubl[J];
#pragma unroll
        for (int c = 0; c < J; ++c) ubl[c] = Ub[c] * inv;
        const int u1 = (int)min((int64_t)np_off[p + 1], u_cap);
        for (int u = np_off[p]; u < u1; ++u) {
            float* so = slot_out + (size_t)u * RS;
            float W[J], Nb[J];
#pragma unroll
            for (int c = 0; c < J; ++c) W[c] = so[J + c];
            quotient_adj<XD, D2>(W, ubl, Nb);
#pragma unroll
            for (int c = 0; c < J; ++c) so[c] = Nb[c];
        }
    }
};

template <int XD, int D2>
__global__ void __launch_bounds__(POU_T) pou_forward_kernel(int64_t n, int npou, const int32_t* __restrict__ pt_off,
                                                             const int32_t* __restrict__ p_take,
                                                             const float* __restrict__ pair_out,
                                                             float* __restrict__ slot_out, float* __restrict__ U,
                                                             int64_t s_cap, int64_t u_cap, int32_t* status) {
    constexpr int J = JL<XD, D2>::J;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        float u[J];
        PointPOU<XD, D2>::run(p, npou, pt_off, p_take, pair_out, slot_out, u, s_cap, u_cap, status);
#pragma unroll
        for (int c = 0; c < J; ++c) U[p * J + c] = u[c];
    }
}

template <int XD, int D2>
__global__ void __launch_bounds__(POU_T) pou_backward_kernel(int64_t n, int npou, const int32_t* __restrict__ np_off,
                                                              const float* __restrict__ Ubar,
                                                              float* __restrict__ slot_out, int64_t u_cap) {
    constexpr int J = JL<XD, D2>::J;
    for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
        float ub[J];
#pragma unroll
        for (int c = 0; c < J; ++c) ub[c] = Ubar[p * J + c];
        PointPOU<XD, D2>::seed(p, npou, np_off, ub, slot_out, u_cap);
    }
}

__device__ __forceinline__ double block_sum_double(double v, double* sh) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (threadIdx.x == 0) {
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r += sh[w];
    }
    __syncthreads();
    return r;
}

// Constraint, residual and seeds of one point from its unconstrained jets u:
// returns r^2 and leaves the seed dL/dU (before the 1/npou of the POU sum) in ub.
template <int XD, int D2>
__device__ __forceinline__ float point_residual(const fbp_problem& P, float inv_n, const float* __restrict__ x,
                                                int64_t p, const float (&u)[JL<XD, D2>::J],
                                                float* __restrict__ U_out, float (&ub)[JL<XD, D2>::J]) {
    constexpr int J = JL<XD, D2>::J;
    float xp[XD];
#pragma unroll
    for (int d = 0; d < XD; ++d) xp[d] = x[p * XD + d];
    float A[J], B[J];
    ansatz<XD, D2>(P, xp, A, B);
    float uc[J];
    uc[0] = A[0] + B[0] * u[0];
#pragma unroll
    for (int d = 0; d < XD; ++d) uc[1 + d] = A[1 + d] + B[1 + d] * u[0] + B[0] * u[1 + d];
#pragma unroll
    for (int s = 0; s < JL<XD, D2>::NS; ++s) {
        float v = A[1 + XD + s] + B[1 + XD + s] * u[0] + B[0] * u[1 + XD + s];
#pragma unroll
        for (int d = 0; d < XD; ++d)
            if ((JL<XD, D2>::slot_dims(s) >> d) & 1) v += 2.0f * B[1 + d] * u[1 + d];
        uc[1 + XD + s] = v;
    }
    if (U_out) {
#pragma unroll
        for (int c = 0; c < J; ++c) U_out[p * J + c] = uc[c];
    }
    float dr[J];
    const float r = residual<XD, D2>(P, xp, uc, dr);
    // seeds: dL/duc = (2 r / n) dr/duc, then the ansatz adjoint
    const float g = 2.0f * r * inv_n;
    float ucb[J];
#pragma unroll
    for (int c = 0; c < J; ++c) ucb[c] = g * dr[c];
    ub[0] = B[0] * ucb[0];
#pragma unroll
    for (int d = 0; d < XD; ++d) {
        ub[0] += B[1 + d] * ucb[1 + d];
        ub[1 + d] = B[0] * ucb[1 + d];
    }
#pragma unroll
    for (int s = 0; s < JL<XD, D2>::NS; ++s) {
        ub[0] += B[1 + XD + s] * ucb[1 + XD + s];
#pragma unroll
        for (int d = 0; d < XD; ++d)
            if ((JL<XD, D2>::slot_dims(s) >> d) & 1) ub[1 + d] += 2.0f * B[1 + d] * ucb[1 + XD + s];
        ub[1 + XD + s] = B[0] * ucb[1 + XD + s];
    }
    return r * r;
}

// Fused POU + constraint + residual + loss + seeds, one warp per 32
// consecutive points.  Their pairs are one contiguous range of pair_out whose
// slot ids (p_take) ascend, so the warp reads the range row by row (32 pairs,
// coalesced), sums each row's records per slot with a segmented shuffle scan
// and adds the row sums into a per-warp shared-memory table of the range's
// slots (rows in order: a fixed summation order).  Then per slot the quotient
// jets, per point (lane) the constraint, residual and seeds, per slot the
// seeds dL/dN, and the slot records [dL/dN | W] leave coalesced.  A warp whose
// slots do not fit the table runs the same steps one point per lane.
constexpr int POU_WARPS = 4;
#ifndef POU_ROWS
#define POU_ROWS 2  // rows scanned together (measured: 2 beats 1)
#endif

// slots per warp in the shared-memory table: up to 256, within 40 KB per CTA
__host__ __device__ constexpr int pou_slotcap(int rs) {
    return 40960 / (POU_WARPS * rs * 4) < 256 ? 40960 / (POU_WARPS * rs * 4) : 256;
}

template <int XD, int D2>
__global__ void __launch_bounds__(POU_WARPS * 32) pou_loss_kernel(fbp_problem P, int64_t n, int npou, float inv_n,
                                                                   const float* __restrict__ x,
                                                                   const int32_t* __restrict__ pt_off,
                                                                   const int32_t* __restrict__ np_off,
                                                                   const int32_t* __restrict__ p_take,
                                                                   const float* __restrict__ pair_out,
                                                                   float* __restrict__ slot_out,
                                                                   float* __restrict__ U_out, int64_t s_cap,
                                                                   int64_t u_cap, double* __restrict__ loss_part,
                                                                   int32_t* status) {
    constexpr int J = JL<XD, D2>::J, RS = rec_stride(J), NV = 2 * J, SLOTCAP = pou_slotcap(RS);
    __shared__ __align__(16) float table[POU_WARPS][SLOTCAP * RS];
    __shared__ double sh[POU_WARPS];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    float* T = table[w];
    const float inv_npou = 1.0f / (float)npou;
    // scheduled training: only the kept points enter the loss, whose mean is
    // over their number (a device count written by fbp_train_mask)
    const int32_t n_keep = P.n_keep ? max(*P.n_keep, 1) : 0;
    if (P.n_keep) inv_n = 1.0f / (float)n_keep;
    double acc = 0.0;
    const int64_t ngroups = (n + 31) / 32;
    for (int64_t grp = (int64_t)blockIdx.x * POU_WARPS + w; grp < ngroups; grp += (int64_t)gridDim.x * POU_WARPS) {
        const int64_t p0 = grp * 32, p = p0 + lane;
        const bool pv = p < n;
        const int np = (int)min((int64_t)32, n - p0);
        const int64_t E0 = min((int64_t)pt_off[p0], s_cap), E1 = min((int64_t)pt_off[p0 + np], s_cap);
        const int64_t U0 = np_off[p0], U1 = np_off[p0 + np];
        const int nsl = (int)(U1 - U0);
        const bool coop = nsl <= SLOTCAP && U1 <= u_cap;  // warp-uniform
        float u[J], ub[J];
#pragma unroll
        for (int c = 0; c < J; ++c) u[c] = 0.f;
        if (coop) {
            for (int i = lane; i < nsl * RS; i += 32) T[i] = 0.f;
            __syncwarp();
            int prev = -1;  // last slot id of the previous row
            // rows of 32 pairs, POU_ROWS at a time (their scans interleave), loaded
            // one group ahead; lanes past the range hold the key INT_MAX and zeros
            auto load_row = [&](int64_t eb, int& key, float (&vv)[NV]) {
                const int64_t e = eb + lane;
                key = e < E1 ? p_take[e] : 0x7fffffff;
#pragma unroll
                for (int c = 0; c < NV; ++c) vv[c] = 0.f;
                if (e < E1) {
                    const float4* po = reinterpret_cast<const float4*>(pair_out + (size_t)e * RS);
#pragma unroll
                    for (int h = 0; h < RS / 4; ++h) {
                        const float4 q = po[h];
                        if (4 * h + 0 < NV) vv[4 * h + 0] = q.x;
                        if (4 * h + 1 < NV) vv[4 * h + 1] = q.y;
                        if (4 * h + 2 < NV) vv[4 * h + 2] = q.z;
                        if (4 * h + 3 < NV) vv[4 * h + 3] = q.w;
                    }
                }
            };
            constexpr int ROWS = POU_ROWS;
            int nkey[ROWS];
            float nv[ROWS][NV];
#pragma unroll
            for (int r = 0; r < ROWS; ++r) load_row(E0 + 32 * r, nkey[r], nv[r]);
            for (int64_t eb = E0; eb < E1; eb += 32 * ROWS) {
                int key[ROWS];
                float v[ROWS][NV];
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    key[r] = nkey[r];
#pragma unroll
                    for (int c = 0; c < NV; ++c) v[r][c] = nv[r][c];
                }
                if (eb + 32 * ROWS < E1) {
#pragma unroll
                    for (int r = 0; r < ROWS; ++r) load_row(eb + 32 * (ROWS + r), nkey[r], nv[r]);
                }
                // slots must ascend along the range (levels ascending within a point)
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int kp = __shfl_up_sync(0xffffffffu, key[r], 1);
                    if (eb + 32 * r + lane < E1 && key[r] < (lane ? kp : prev))
                        atomicOr(status, FBP_STATUS_LEVEL_ORDER);
                    prev = __shfl_sync(0xffffffffu, key[r], 31);
                }
                // inclusive scans of the records within runs of equal slot ids
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
                    for (int r = 0; r < ROWS; ++r) {
                        const int k2 = __shfl_up_sync(0xffffffffu, key[r], off);
                        const bool same = lane >= off && k2 == key[r];
#pragma unroll
                        for (int c = 0; c < NV; ++c) {
                            const float t = __shfl_up_sync(0xffffffffu, v[r][c], off);
                            if (same) v[r][c] += t;
                        }
                    }
                }
                // each run's last lane adds the run's sum, row after row
#pragma unroll
                for (int r = 0; r < ROWS; ++r) {
                    const int kn = __shfl_down_sync(0xffffffffu, key[r], 1);
                    if (eb + 32 * r + lane < E1 && (lane == 31 || kn != key[r])) {
                        const int s = key[r] - (int)U0;
                        if (s >= 0 && s < nsl) {
#pragma unroll
                            for (int c = 0; c < NV; ++c) T[s * RS + c] += v[r][c];
                        } else {
                            atomicOr(status, FBP_STATUS_BAD_INDEX);
                        }
                    }
                    __syncwarp();
                }
            }
            // per slot: U_l = N / W (quotient-rule jets) in place of N
            for (int s = lane; s < nsl; s += 32) {
                float N[J], W[J], Ul[J];
#pragma unroll
                for (int c = 0; c < J; ++c) {
                    N[c] = T[s * RS + c];
                    W[c] = T[s * RS + J + c];
                }
                quotient<XD, D2>(N, W, Ul);
#pragma unroll
                for (int c = 0; c < J; ++c) T[s * RS + c] = Ul[c];
            }
            __syncwarp();
            if (pv) {
                const int s0 = np_off[p] - (int)U0, s1 = np_off[p + 1] - (int)U0;
                for (int s = s0; s < s1; ++s)
#pragma unroll
                    for (int c = 0; c < J; ++c) u[c] += T[s * RS + c];
#pragma unroll
                for (int c = 0; c < J; ++c) u[c] *= inv_npou;
            }
        } else if (pv) {
            PointPOU<XD, D2>::run(p, npou, pt_off, p_take, pair_out, slot_out, u, s_cap, u_cap, status);
        }
        if (pv) {
            const float r2 = point_residual<XD, D2>(P, inv_n, x, p, u, U_out, ub);
            if (!P.pt_keep || P.pt_keep[p]) {
                acc += (double)r2;
            } else {  // a point outside every active subdomain: no loss, no seeds
#pragma unroll
                for (int c = 0; c < J; ++c) ub[c] = 0.f;
            }
        }
        if (coop) {
            __syncwarp();
            if (pv) {  // seeds dL/dN_l of the point's slots, in place of U_l
                float ubl[J];
#pragma unroll
                for (int c = 0; c < J; ++c) ubl[c] = ub[c] * inv_npou;
                const int s0 = np_off[p] - (int)U0, s1 = np_off[p + 1] - (int)U0;
                for (int s = s0; s < s1; ++s) {
                    float W[J], Nb[J];
#pragma unroll
                    for (int c = 0; c < J; ++c) W[c] = T[s * RS + J + c];
                    quotient_adj<XD, D2>(W, ubl, Nb);
#pragma unroll
                    for (int c = 0; c < J; ++c) T[s * RS + c] = Nb[c];
                }
            }
            __syncwarp();
            float4* dst = reinterpret_cast<float4*>(slot_out + (size_t)U0 * RS);
            const float4* src = reinterpret_cast<const float4*>(T);
            for (int i = lane; i < nsl * RS / 4; i += 32) dst[i] = src[i];
            __syncwarp();
        } else if (pv) {
            PointPOU<XD, D2>::seed(p, npou, np_off, ub, slot_out, u_cap);
        }
    }
    // block sum of the squared residuals (FP64), fixed order
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (lane == 0) sh[w] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
#pragma unroll
        for (int q = 0; q < POU_WARPS; ++q) t += sh[q];
        loss_part[blockIdx.x] = P.n_keep ? t / (double)n_keep : t;
    }
}

__global__ void loss_finalize_kernel(const double* __restrict__ part, int np, double scale, double* loss) {
    __shared__ double sh[32];
    double a = 0.0;
    for (int i = threadIdx.x; i < np; i += blockDim.x) a += part[i];
    const double t = block_sum_double(a, sh);
    if (threadIdx.x == 0) *loss = t * scale;
}

__global__ void grad_reduce_kernel(const float* __restrict__ part, const int32_t* __restrict__ item_start, int64_t m,
                                   int P, float* __restrict__ grad) {
    const int64_t total = m * (int64_t)P;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < total; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = i / P;
        const int q = (int)(i - j * P);
        const int a = item_start[j], b = item_start[j + 1];
        float s = 0.f;
        for (int it = a; it < b; ++it) s += part[(size_t)it * P + q];
        grad[i] = s;
    }
}

// dispatch over (xd, d2mask)
template <template <int, int> class K>
struct XDispatch;

#define FBP_XD_D2_CASES(X) \
    X(1, 0) X(1, 1) X(2, 0) X(2, 1) X(2, 2) X(2, 3) X(2, 11) X(3, 0) X(3, 1) X(3, 2) X(3, 3) X(3, 4) X(3, 5) X(3, 6) \
        X(3, 7) X(3, 55)

static int grid_pts(int64_t n) {
    int64_t b = (n + POU_T - 1) / POU_T;
    const int64_t cap = (int64_t)sm_count() * 8;
    return (int)std::max<int64_t>(1, std::min(b, cap));
}

}  // namespace fbp

using namespace fbp;

extern "C" int fbp_pou_forward(int32_t xd, int32_t d2mask, int64_t n, int32_t npou, const int32_t* pt_off,
                               const int32_t* p_take, const float* pair_out, float* slot_out, float* U,
                               int64_t s_cap, int64_t u_cap, int32_t* status, void* stream) {
    FBP_REQUIRE(pt_off && U && status && npou > 0, FBP_ERR_INVALID, "fbp_pou_forward: bad args");
    if (n == 0) return FBP_OK;
    cudaStream_t st = as_stream(stream);
    const int g = grid_pts(n);
#define X(a, b)                                                                                                   \
    if (xd == a && d2mask == b) {                                                                                 \
        pou_forward_kernel<a, b><<<g, POU_T, 0, st>>>(n, npou, pt_off, p_take, pair_out, slot_out, U, s_cap, u_cap, status); \
        FBP_LAUNCH_CHECK();                                                                                       \
        return FBP_OK;                                                                                            \
    }
    FBP_XD_D2_CASES(X)
#undef X
    set_error("fbp_pou_forward: unsupported xd=%d d2mask=%d", xd, d2mask);
    return FBP_ERR_UNSUPPORTED;
}

extern "C" int fbp_pou_backward(int32_t xd, int32_t d2mask, int64_t n, int32_t npou, const int32_t* np_off,
                                const float* U_bar, float* slot_out, int64_t u_cap, void* stream) {
    FBP_REQUIRE(np_off && U_bar && npou > 0, FBP_ERR_INVALID, "fbp_pou_backward: bad args");
    if (n == 0) return FBP_OK;
    cudaStream_t st = as_stream(stream);
    const int g = grid_pts(n);
#define X(a, b)                                                                                       \
    if (xd == a && d2mask == b) {                                                                     \
        pou_backward_kernel<a, b><<<g, POU_T, 0, st>>>(n, npou, np_off, U_bar, slot_out, u_cap);    \
        FBP_LAUNCH_CHECK();                                                                           \
        return FBP_OK;                                                                                \
    }
    FBP_XD_D2_CASES(X)
#undef X
    set_error("fbp_pou_backward: unsupported xd=%d d2mask=%d", xd, d2mask);
    return FBP_ERR_UNSUPPORTED;
}

extern "C" int fbp_pou_loss(int32_t xd, int32_t d2mask, const fbp_problem* prob, int64_t n, int32_t npou,
                            const float* x, const int32_t* pt_off, const int32_t* np_off, const int32_t* p_take,
                            const float* pair_out, float* slot_out, float* U_out, int64_t s_cap, int64_t u_cap,
                            double* loss_part, int32_t n_part, int32_t* status, void* stream) {
    FBP_REQUIRE(prob && x && pt_off && np_off && loss_part && status && npou > 0, FBP_ERR_INVALID,
                "fbp_pou_loss: bad args");
    FBP_REQUIRE(n > 0, FBP_ERR_INVALID, "fbp_pou_loss: no points");
    FBP_REQUIRE(prob->ng == 0 || prob->gauss, FBP_ERR_INVALID, "fbp_pou_loss: null gaussians");
    // CTAs of POU_WARPS warps, each warp 32 points at a time
    const int64_t ctas = ((n + 31) / 32 + POU_WARPS - 1) / POU_WARPS;
    const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ctas, (int64_t)sm_count() * 8));
    FBP_REQUIRE(n_part >= g, FBP_ERR_CAPACITY, "fbp_pou_loss: n_part=%d < grid %d", n_part, g);
    cudaStream_t st = as_stream(stream);
    const float inv_n = (float)(1.0 / (double)n);
#define X(a, b)                                                                                              \
    if (xd == a && d2mask == b) {                                                                            \
        pou_loss_kernel<a, b><<<g, POU_WARPS * 32, 0, st>>>(*prob, n, npou, inv_n, x, pt_off, np_off, p_take,   \
                                                             pair_out,                                        \
                                                    slot_out, U_out, s_cap, u_cap, loss_part, status);      \
        FBP_LAUNCH_CHECK();                                                                                  \
        if (n_part > g) FBP_CUDA_CHECK(cudaMemsetAsync(loss_part + g, 0, (n_part - g) * sizeof(double), st)); \
        return FBP_OK;                                                                                       \
    }
    FBP_XD_D2_CASES(X)
#undef X
    set_error("fbp_pou_loss: unsupported xd=%d d2mask=%d", xd, d2mask);
    return FBP_ERR_UNSUPPORTED;
}

extern "C" int fbp_loss_finalize(const double* loss_part, int32_t n_part, double scale, double* loss, void* stream) {
    FBP_REQUIRE(loss_part && loss && n_part > 0, FBP_ERR_INVALID, "fbp_loss_finalize: bad args");
    loss_finalize_kernel<<<1, 256, 0, as_stream(stream)>>>(loss_part, n_part, scale, loss);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}

extern "C" int fbp_grad_reduce(const float* grad_part, const int32_t* item_start, int64_t m, int32_t nparam,
                               float* grad, void* stream) {
    FBP_REQUIRE(item_start && grad && m > 0 && nparam > 0, FBP_ERR_INVALID, "fbp_grad_reduce: bad args");
    const int64_t total = m * (int64_t)nparam;
    int64_t b = (total + 255) / 256;
    b = std::min<int64_t>(b, (int64_t)sm_count() * 16);
    grad_reduce_kernel<<<(int)std::max<int64_t>(1, b), 256, 0, as_stream(stream)>>>(grad_part, item_start, m, nparam,
                                                                                   grad);
    FBP_LAUNCH_CHECK();
    return FBP_OK;
}
