/* CPU restatement of one FBPINN training step of the 2D multilevel Poisson
 * workload, in C on host threads.
 *
 * TEST AND BENCHMARK INFRASTRUCTURE ONLY: the timed CPU baseline (the
 * reference arm of the benchmark) and a checker in the CPU tests.  Nothing in
 * the fbpinns_gb300 package links or calls it.
 *
 * The step follows the reference algorithm (fbpinns/trainers.py:285-296,
 * FBPINN_update) for tanh FCN subdomain networks 2-H-H-1:
 *   1. interaction lists by the dense closed-box test of every point against
 *      every subdomain, point-major with boxes ascending
 *      (fbpinns/decompositions_base.py:24-68, decompositions.py:218-227);
 *   2. per (point, subdomain) pair: normalisation, the FCN, unnormalisation
 *      and the cosine window (trainers.py:113-118, decompositions.py:184-199,
 *      networks.py:61-68, windows.py:25-35), carried as a jet
 *      (u, u_x, u_y, u_xx, u_yy) -- the components the reference's nested
 *      jvp computes for the Poisson residual (trainers.py:213-247);
 *   3. the two segment sums of FBPINN_model (trainers.py:126-177): sum of w u
 *      and of w per (point, POU level), U_l = N / W, sum over levels / npou;
 *   4. the hard-constraint ansatz and the residual mean square of the
 *      Poisson problem, summed in double precision;
 *   5. the reverse-mode gradient with respect to every subdomain's
 *      parameters, through the same jets, from the activations stored by the
 *      forward pass (as the reference's XLA reverse mode stores them);
 *   6. optax Adam (b1 0.9, b2 0.999, eps 1e-8) with the shared step count.
 * Arithmetic is FP32 (the reference's default); the loss sum is FP64.
 * Reductions have a fixed order for any thread count: work is split into
 * fixed chunks whose partial results are combined in chunk order.  Not
 * thread-safe: one step at a time per process (buffers are kept between
 * calls).
 *
 * Build: gcc -O3 -shared -fPIC -pthread (oracle/build.py).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define CS_J 5      /* jet: u, u_x, u_y, u_xx, u_yy */
#define CS_HMAX 32  /* widest hidden layer compiled */
#define CS_PT_CHUNK 2048 /* points per chunk of the list and POU passes */
#define CS_ITEM 4096     /* pairs per work item of the jet passes */

typedef struct {
    int m, h;              /* subdomains; hidden width (both hidden layers) */
    int npou;              /* POU levels (<= 64) */
    const float* xmins;    /* (m, 2) */
    const float* xmaxs;    /* (m, 2) */
    const float* flags;    /* (m) */
    const float* unnorms;  /* (m, 2): mu, sd */
    const int32_t* pou;    /* (m) level of each subdomain, ascending with the index */
    float sd;              /* width of the hard-constraint ansatz */
    int n_freq;            /* terms of the manufactured solution */
} cs_problem;

/* parameters of one subdomain, the reference's (W, b) per layer with W
 * (fan_out, fan_in) row-major: W1 (h,2) b1 (h) W2 (h,h) b2 (h) W3 (1,h) b3 */
static int n_params(int h) { return 2 * h + h + h * h + h + h + 1; }
static int act_stride(int h) { return h + CS_J * h + h; } /* a1, z2 jet, a2 */

typedef struct {
    void* p;
    int64_t cap; /* elements */
} cs_buf;

static int reserve(cs_buf* b, int64_t n, size_t elem) {
    if (b->p && n <= b->cap) return 0;
    const int64_t nc = n + n / 4 + 1024;
    void* q = realloc(b->p, (size_t)nc * elem);
    if (!q) return -1;
    b->p = q;
    b->cap = nc;
    return 0;
}

typedef struct {
    const cs_problem* pb;
    int64_t n;
    int nthreads;
    const float* x;
    const float* theta;
    float* grad;
    int64_t s, n_items;
    int32_t *pt_count, *pt_off, *n_take, *m_take, *sd_off, *sd_pair, *items, *item_off;
    float *rec, *act, *seed, *gpart;
    double* loss_part;
} cs_ctx;

static cs_buf B_count, B_off, B_ntake, B_mtake, B_sdoff, B_sdpair, B_items, B_itemoff, B_rec, B_act, B_seed,
    B_gpart, B_loss;

/* ---------------------------------------------------------------- threads */
typedef void (*cs_task)(cs_ctx* c, int64_t chunk);
typedef struct {
    cs_ctx* c;
    cs_task f;
    int64_t nchunks;
    int64_t* next;
} cs_job;

static void* cs_worker(void* arg) {
    cs_job* j = (cs_job*)arg;
    for (;;) {
        const int64_t k = __atomic_fetch_add(j->next, 1, __ATOMIC_RELAXED);
        if (k >= j->nchunks) break;
        j->f(j->c, k);
    }
    return NULL;
}

/* f(c, k) for k = 0 .. nchunks-1 on the context's threads; chunks come from a
 * shared counter and no result depends on which thread ran a chunk. */
static void cs_parallel(cs_ctx* c, cs_task f, int64_t nchunks) {
    int64_t next = 0;
    cs_job job = {c, f, nchunks, &next};
    int nt = c->nthreads < 1 ? 1 : (c->nthreads > 256 ? 256 : c->nthreads);
    pthread_t th[256];
    int started = 0;
    for (int i = 1; i < nt; ++i)
        if (pthread_create(&th[started], NULL, cs_worker, &job) == 0) ++started;
    cs_worker(&job);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
}

/* exp(t) for t <= 0, branch-free so that loops over neurons vectorise:
 * t = k ln 2 + r with |r| <= ln 2 / 2 (Cody-Waite split of ln 2), e^r by its
 * degree-6 Taylor polynomial (truncation below 1.3e-7 relative), 2^k from the
 * exponent bits; t is clamped at -87 (e^-87 ~ 1.6e-38, the float range). */
static inline float cs_exp_nonpos(float t) {
    t = t < -87.0f ? -87.0f : t;
    const float kf = (t * 1.44269504088896341f + 12582912.0f) - 12582912.0f; /* round to nearest */
    const float r = (t - kf * 0.693359375f) - kf * -2.12194440e-4f;
    float p = 1.0f / 720.0f;
    p = p * r + 1.0f / 120.0f;
    p = p * r + 1.0f / 24.0f;
    p = p * r + 1.0f / 6.0f;
    p = p * r + 0.5f;
    p = p * r + 1.0f;
    p = p * r + 1.0f;
    union { float f; int32_t i; } sc;
    sc.i = ((int32_t)kf + 127) << 23;
    return p * sc.f;
}

static inline float cs_tanh(float v) {
    /* tanh|v| = (1 - e) / (1 + e), e = exp(-2|v|) in (0, 1]: no overflow */
    const float e = cs_exp_nonpos(-2.0f * fabsf(v));
    const float t = (1.0f - e) / (1.0f + e);
    return v < 0.0f ? -t : t;
}

/* ------------------------------------------------------- 1. the lists */
static inline int inside(const cs_problem* pb, int j, float x0, float x1) {
    return pb->xmins[2 * j] <= x0 && x0 <= pb->xmaxs[2 * j] && pb->xmins[2 * j + 1] <= x1 &&
           x1 <= pb->xmaxs[2 * j + 1];
}

static void t_count(cs_ctx* c, int64_t k) {
    const cs_problem* pb = c->pb;
    const int64_t p0 = k * CS_PT_CHUNK, p1 = p0 + CS_PT_CHUNK < c->n ? p0 + CS_PT_CHUNK : c->n;
    for (int64_t p = p0; p < p1; ++p) {
        const float x0 = c->x[2 * p], x1 = c->x[2 * p + 1];
        int cnt = 0;
        for (int j = 0; j < pb->m; ++j) cnt += inside(pb, j, x0, x1);
        c->pt_count[p] = cnt;
    }
}

static void t_fill(cs_ctx* c, int64_t k) {
    const cs_problem* pb = c->pb;
    const int64_t p0 = k * CS_PT_CHUNK, p1 = p0 + CS_PT_CHUNK < c->n ? p0 + CS_PT_CHUNK : c->n;
    for (int64_t p = p0; p < p1; ++p) {
        const float x0 = c->x[2 * p], x1 = c->x[2 * p + 1];
        int32_t o = c->pt_off[p];
        for (int j = 0; j < pb->m; ++j)
            if (inside(pb, j, x0, x1)) {
                c->n_take[o] = (int32_t)p;
                c->m_take[o++] = j;
            }
    }
}

/* --------------------------------------------- 2. per-pair forward jets */
typedef struct {
    float W1[CS_HMAX * 2], b1[CS_HMAX], W2[CS_HMAX * CS_HMAX], W2t[CS_HMAX * CS_HMAX], b2[CS_HMAX], W3[CS_HMAX];
    float b3, mu[2], isd[2], k1[2], flag, mu_u, sd_u;
} cs_sub;

static void load_sub(const cs_problem* pb, const float* th, int j, int H, cs_sub* S) {
    memcpy(S->W1, th, sizeof(float) * 2 * H);
    memcpy(S->b1, th + 2 * H, sizeof(float) * H);
    memcpy(S->W2, th + 3 * H, sizeof(float) * H * H);
    for (int k = 0; k < H; ++k)
        for (int n = 0; n < H; ++n) S->W2t[n * H + k] = S->W2[k * H + n];
    memcpy(S->b2, th + 3 * H + H * H, sizeof(float) * H);
    memcpy(S->W3, th + 4 * H + H * H, sizeof(float) * H);
    S->b3 = th[5 * H + H * H];
    for (int d = 0; d < 2; ++d) {
        const float lo = pb->xmins[2 * j + d], hi = pb->xmaxs[2 * j + d];
        S->mu[d] = (hi + lo) / 2.0f;
        S->isd[d] = 1.0f / ((hi - lo) / 2.0f);
        S->k1[d] = 1.5707963267948966f * S->isd[d];
    }
    S->flag = pb->flags[j];
    S->mu_u = pb->unnorms[2 * j];
    S->sd_u = pb->unnorms[2 * j + 1];
}

/* layer-1 jet v[c][n] = [a, tp cw_x, tp cw_y, tpp cw_x^2, tpp cw_y^2] with cw_d = W1[n][d] / sd_d */
static inline __attribute__((always_inline)) void layer1(int H, const cs_sub* S, const float* xn, const float* a1,
                                                         float (*v)[CS_HMAX]) {
    for (int n = 0; n < H; ++n) {
        const float a = a1[n], tp = 1.0f - a * a, tpp = -2.0f * a * tp;
        const float c0 = S->W1[2 * n] * S->isd[0], c1 = S->W1[2 * n + 1] * S->isd[1];
        v[0][n] = a;
        v[1][n] = tp * c0;
        v[2][n] = tp * c1;
        v[3][n] = tpp * c0 * c0;
        v[4][n] = tpp * c1 * c1;
    }
    (void)xn;
}

static inline __attribute__((always_inline)) void pair_forward(int H, const cs_sub* S, const float* xp, float* rec,
                                                               float* act) {
    float xn[2];
    for (int d = 0; d < 2; ++d) xn[d] = (xp[d] - S->mu[d]) * S->isd[d];
    float* a1 = act;
    float* z = act + H;
    float* a2 = act + H + CS_J * H;
    float z1[CS_HMAX];
    for (int n = 0; n < H; ++n) z1[n] = S->W1[2 * n] * xn[0] + S->W1[2 * n + 1] * xn[1] + S->b1[n];
    for (int n = 0; n < H; ++n) a1[n] = cs_tanh(z1[n]);
    float v[CS_J][CS_HMAX];
    layer1(H, S, xn, a1, v);
    /* z[c][k] = sum_n W2[k][n] v[c][n] (+ b2 for c = 0), accumulated over n */
    float zz[CS_J][CS_HMAX];
    for (int k = 0; k < H; ++k) {
        zz[0][k] = S->b2[k];
        for (int c = 1; c < CS_J; ++c) zz[c][k] = 0.0f;
    }
    for (int n = 0; n < H; ++n) {
        const float* wr = S->W2t + n * H;
        for (int c = 0; c < CS_J; ++c) {
            const float vc = v[c][n];
            for (int k = 0; k < H; ++k) zz[c][k] += wr[k] * vc;
        }
    }
    for (int c = 0; c < CS_J; ++c)
        for (int k = 0; k < H; ++k) z[c * H + k] = zz[c][k];
    /* tanh rules and the output layer */
    for (int k = 0; k < H; ++k) a2[k] = cs_tanh(zz[0][k]);
    float o[CS_J] = {S->b3, 0.0f, 0.0f, 0.0f, 0.0f};
    for (int k = 0; k < H; ++k) {
        const float a = a2[k];
        const float tp = 1.0f - a * a, tpp = -2.0f * a * tp;
        const float zx = zz[1][k], zy = zz[2][k];
        const float w3 = S->W3[k];
        o[0] += w3 * a;
        o[1] += w3 * (tp * zx);
        o[2] += w3 * (tp * zy);
        o[3] += w3 * (tp * zz[3][k] + tpp * zx * zx);
        o[4] += w3 * (tp * zz[4][k] + tpp * zy * zy);
    }
    float u[CS_J];
    for (int c = 0; c < CS_J; ++c) u[c] = o[c] * S->sd_u;
    u[0] += S->mu_u;
    /* cosine window per dim: ((1 + cos(pi xn)) / 2)^2 = cos^4(phi), phi = pi xn / 2 */
    float w0[2], w1[2], w2[2];
    for (int d = 0; d < 2; ++d) {
        const float phi = 1.5707963267948966f * xn[d], k1 = S->k1[d];
        const float cs = cosf(phi), sn = sinf(phi), cs2 = cs * cs;
        w0[d] = cs2 * cs2;
        w1[d] = -4.0f * cs2 * cs * sn * k1;
        w2[d] = (12.0f * cs2 * sn * sn - 4.0f * cs2 * cs2) * k1 * k1;
    }
    const float f = S->flag;
    float w[CS_J];
    w[0] = f * (w0[0] * w0[1]) + (1.0f - f);
    w[1] = f * (w1[0] * w0[1]);
    w[2] = f * (w0[0] * w1[1]);
    w[3] = f * (w2[0] * w0[1]);
    w[4] = f * (w0[0] * w2[1]);
    rec[0] = u[0] * w[0];
    rec[1] = u[1] * w[0] + u[0] * w[1];
    rec[2] = u[2] * w[0] + u[0] * w[2];
    rec[3] = u[3] * w[0] + 2.0f * u[1] * w[1] + u[0] * w[3];
    rec[4] = u[4] * w[0] + 2.0f * u[2] * w[2] + u[0] * w[4];
    for (int c = 0; c < CS_J; ++c) rec[CS_J + c] = w[c];
}

static inline __attribute__((always_inline)) void t_forward_h(cs_ctx* c, int64_t it, int H) {
    const int j = c->items[3 * it], beg = c->items[3 * it + 1], cnt = c->items[3 * it + 2];
    cs_sub S;
    load_sub(c->pb, c->theta + (size_t)j * n_params(H), j, H, &S);
    const int AS = act_stride(H);
    for (int q = 0; q < cnt; ++q) {
        const int64_t e = c->sd_pair[beg + q];
        /* activations in subdomain-major order (the reverse pass walks the same order) */
        pair_forward(H, &S, c->x + 2 * (int64_t)c->n_take[e], c->rec + e * 2 * CS_J,
                     c->act + (int64_t)(beg + q) * AS);
    }
}
static void t_forward_8(cs_ctx* c, int64_t it) { t_forward_h(c, it, 8); }
static void t_forward_16(cs_ctx* c, int64_t it) { t_forward_h(c, it, 16); }
static void t_forward_32(cs_ctx* c, int64_t it) { t_forward_h(c, it, 32); }

/* ------------------------------- 3 + 4. POU, constraint, residual, seeds */
static void ansatz_jet(float sd, float x, float* b) {
    /* b = [B, B', B''] of B(x) = tanh(x / sd) tanh((1 - x) / sd) */
    const float t1 = cs_tanh(x / sd), t2 = cs_tanh((1.0f - x) / sd);
    const float d1 = (1.0f - t1 * t1) / sd, d2 = -(1.0f - t2 * t2) / sd;
    const float dd1 = -2.0f * t1 * d1 / sd, dd2 = 2.0f * t2 * d2 / sd;
    b[0] = t1 * t2;
    b[1] = d1 * t2 + t1 * d2;
    b[2] = dd1 * t2 + 2.0f * d1 * d2 + t1 * dd2;
}

static void t_pou(cs_ctx* c, int64_t k) {
    const cs_problem* pb = c->pb;
    const int64_t p0 = k * CS_PT_CHUNK, p1 = p0 + CS_PT_CHUNK < c->n ? p0 + CS_PT_CHUNK : c->n;
    const float inv_npou = 1.0f / (float)pb->npou;
    double acc = 0.0;
    for (int64_t p = p0; p < p1; ++p) {
        const int32_t e0 = c->pt_off[p], e1 = c->pt_off[p + 1];
        float U[CS_J] = {0, 0, 0, 0, 0};
        float Ws[64][CS_J];
        int32_t segb[65];
        int nseg = 0;
        for (int32_t e = e0; e < e1;) {  /* one segment per POU level (levels ascend) */
            const int lv = pb->pou[c->m_take[e]];
            float N[CS_J] = {0, 0, 0, 0, 0}, W[CS_J] = {0, 0, 0, 0, 0};
            segb[nseg] = e;
            for (; e < e1 && pb->pou[c->m_take[e]] == lv; ++e)
                for (int q = 0; q < CS_J; ++q) {
                    N[q] += c->rec[(int64_t)e * 2 * CS_J + q];
                    W[q] += c->rec[(int64_t)e * 2 * CS_J + CS_J + q];
                }
            const float r = 1.0f / W[0];  /* quotient-rule jet of N / W */
            float Ul[CS_J];
            Ul[0] = N[0] * r;
            for (int d = 0; d < 2; ++d) Ul[1 + d] = (N[1 + d] - Ul[0] * W[1 + d]) * r;
            for (int d = 0; d < 2; ++d)
                Ul[3 + d] = (N[3 + d] - 2.0f * Ul[1 + d] * W[1 + d] - Ul[0] * W[3 + d]) * r;
            for (int q = 0; q < CS_J; ++q) {
                U[q] += Ul[q];
                Ws[nseg][q] = W[q];
            }
            ++nseg;
        }
        segb[nseg] = e1;
        for (int q = 0; q < CS_J; ++q) U[q] *= inv_npou;
        /* u = B(x) B(y) U; residual u_xx + u_yy + f */
        const float x0 = c->x[2 * p], x1 = c->x[2 * p + 1];
        float bx[3], by[3];
        ansatz_jet(pb->sd, x0, bx);
        ansatz_jet(pb->sd, x1, by);
        const float uxx = bx[2] * by[0] * U[0] + 2.0f * bx[1] * by[0] * U[1] + bx[0] * by[0] * U[3];
        const float uyy = bx[0] * by[2] * U[0] + 2.0f * bx[0] * by[1] * U[2] + bx[0] * by[0] * U[4];
        float f = 0.0f;
        for (int kf = 1; kf <= pb->n_freq; ++kf) {
            const float a = (float)(1 << kf) * 3.14159265358979323846f;
            f += (float)(1 << (kf + 1)) * 9.8696044010893586188f * sinf(a * x0) * sinf(a * x1);
        }
        const float res = uxx + uyy + f;
        acc += (double)res * (double)res;
        /* seeds: dL/dres = 2 res / n, back through the constraint to U, then to each level's N */
        const float g = 2.0f * res / (float)c->n;
        float Ub[CS_J];
        Ub[0] = g * (bx[2] * by[0] + bx[0] * by[2]) * inv_npou;
        Ub[1] = g * 2.0f * bx[1] * by[0] * inv_npou;
        Ub[2] = g * 2.0f * bx[0] * by[1] * inv_npou;
        Ub[3] = g * bx[0] * by[0] * inv_npou;
        Ub[4] = Ub[3];
        for (int sgi = 0; sgi < nseg; ++sgi) {
            const float* W = Ws[sgi];
            const float r = 1.0f / W[0];
            float Nb[CS_J];  /* adjoint of the quotient jet in N (W does not depend on theta) */
            Nb[3] = Ub[3] * r;
            Nb[4] = Ub[4] * r;
            Nb[1] = (Ub[1] - 2.0f * Nb[3] * W[1]) * r;
            Nb[2] = (Ub[2] - 2.0f * Nb[4] * W[2]) * r;
            Nb[0] = (Ub[0] - Nb[1] * W[1] - Nb[2] * W[2] - Nb[3] * W[3] - Nb[4] * W[4]) * r;
            for (int32_t e = segb[sgi]; e < segb[sgi + 1]; ++e)
                for (int q = 0; q < CS_J; ++q) c->seed[(int64_t)e * CS_J + q] = Nb[q];
        }
    }
    c->loss_part[k] = acc;
}

/* ------------------------------------------------- 5. reverse pass */
static inline __attribute__((always_inline)) void pair_adjoint(int H, const cs_sub* S, const float* xp,
                                                               const float* rec, const float* act, const float* nb,
                                                               float* g) {
    float* gW1 = g;
    float* gb1 = gW1 + 2 * H;
    float* gW2 = gb1 + H;
    float* gb2 = gW2 + H * H;
    float* gW3 = gb2 + H;
    float* gb3 = gW3 + H;
    float xn[2];
    for (int d = 0; d < 2; ++d) xn[d] = (xp[d] - S->mu[d]) * S->isd[d];
    /* u w jet adjoint in u (w fixed), then the unnormalisation */
    const float* w = rec + CS_J;
    float ob[CS_J];
    ob[0] = nb[0] * w[0] + nb[1] * w[1] + nb[2] * w[2] + nb[3] * w[3] + nb[4] * w[4];
    ob[1] = nb[1] * w[0] + 2.0f * nb[3] * w[1];
    ob[2] = nb[2] * w[0] + 2.0f * nb[4] * w[2];
    ob[3] = nb[3] * w[0];
    ob[4] = nb[4] * w[0];
    for (int q = 0; q < CS_J; ++q) ob[q] *= S->sd_u;
    *gb3 += ob[0];
    /* output layer and the layer-2 tanh jet adjoint -> zb[c][k] */
    const float* a1 = act;
    const float* z = act + H;
    const float* a2 = act + H + CS_J * H;
    float zb[CS_J][CS_HMAX];
    for (int k = 0; k < H; ++k) {
        const float a = a2[k];
        const float tp = 1.0f - a * a, tpp = -2.0f * a * tp, tppp = tp * (6.0f * a * a - 2.0f);
        const float zx = z[H + k], zy = z[2 * H + k], zxx = z[3 * H + k], zyy = z[4 * H + k];
        gW3[k] += ob[0] * a + ob[1] * (tp * zx) + ob[2] * (tp * zy) + ob[3] * (tp * zxx + tpp * zx * zx) +
                  ob[4] * (tp * zyy + tpp * zy * zy);
        const float w3 = S->W3[k];
        const float g0 = w3 * ob[0], g1 = w3 * ob[1], g2 = w3 * ob[2], g3 = w3 * ob[3], g4 = w3 * ob[4];
        const float tpb = g1 * zx + g2 * zy + g3 * zxx + g4 * zyy;
        const float tppb = g3 * zx * zx + g4 * zy * zy;
        zb[0][k] = g0 * tp + tpb * tpp + tppb * tppp;
        zb[1][k] = g1 * tp + 2.0f * g3 * tpp * zx;
        zb[2][k] = g2 * tp + 2.0f * g4 * tpp * zy;
        zb[3][k] = g3 * tp;
        zb[4][k] = g4 * tp;
    }
    float v[CS_J][CS_HMAX];
    layer1(H, S, xn, a1, v);
    /* b2-bar, W2-bar[k][n] = sum_c zb[c][k] v[c][n], v-bar[c][n] = sum_k W2[k][n] zb[c][k] */
    float vb[CS_J][CS_HMAX];
    for (int c = 0; c < CS_J; ++c)
        for (int n = 0; n < H; ++n) vb[c][n] = 0.0f;
    for (int k = 0; k < H; ++k) {
        gb2[k] += zb[0][k];
        float* gr = gW2 + k * H;
        const float* wr = S->W2 + k * H;
        for (int c = 0; c < CS_J; ++c) {
            const float zc = zb[c][k];
            for (int n = 0; n < H; ++n) {
                gr[n] += zc * v[c][n];
                vb[c][n] += wr[n] * zc;
            }
        }
    }
    /* layer-1 jet adjoint */
    for (int n = 0; n < H; ++n) {
        const float a = a1[n], tp = 1.0f - a * a, tpp = -2.0f * a * tp, tppp = tp * (6.0f * a * a - 2.0f);
        const float c0 = S->W1[2 * n] * S->isd[0], c1 = S->W1[2 * n + 1] * S->isd[1];
        const float tpb = vb[1][n] * c0 + vb[2][n] * c1;
        const float tppb = vb[3][n] * c0 * c0 + vb[4][n] * c1 * c1;
        const float z1b = vb[0][n] * tp + tpb * tpp + tppb * tppp;
        const float cb0 = vb[1][n] * tp + 2.0f * vb[3][n] * tpp * c0;
        const float cb1 = vb[2][n] * tp + 2.0f * vb[4][n] * tpp * c1;
        gW1[2 * n] += z1b * xn[0] + cb0 * S->isd[0];
        gW1[2 * n + 1] += z1b * xn[1] + cb1 * S->isd[1];
        gb1[n] += z1b;
    }
}

static inline __attribute__((always_inline)) void t_adjoint_h(cs_ctx* c, int64_t it, int H) {
    const int j = c->items[3 * it], beg = c->items[3 * it + 1], cnt = c->items[3 * it + 2];
    const int P = n_params(H);
    cs_sub S;
    load_sub(c->pb, c->theta + (size_t)j * P, j, H, &S);
    float* g = c->gpart + (size_t)it * P;
    memset(g, 0, sizeof(float) * P);
    const int AS = act_stride(H);
    for (int q = 0; q < cnt; ++q) {
        const int64_t e = c->sd_pair[beg + q];
        pair_adjoint(H, &S, c->x + 2 * (int64_t)c->n_take[e], c->rec + e * 2 * CS_J,
                     c->act + (int64_t)(beg + q) * AS, c->seed + e * CS_J, g);
    }
}
static void t_adjoint_8(cs_ctx* c, int64_t it) { t_adjoint_h(c, it, 8); }
static void t_adjoint_16(cs_ctx* c, int64_t it) { t_adjoint_h(c, it, 16); }
static void t_adjoint_32(cs_ctx* c, int64_t it) { t_adjoint_h(c, it, 32); }

static void t_reduce(cs_ctx* c, int64_t j) {
    /* grad[j] = box j's item partials, in item order */
    const int P = n_params(c->pb->h);
    float* dst = c->grad + (size_t)j * P;
    memset(dst, 0, sizeof(float) * P);
    for (int32_t it = c->item_off[j]; it < c->item_off[j + 1]; ++it) {
        const float* src = c->gpart + (size_t)it * P;
        for (int i = 0; i < P; ++i) dst[i] += src[i];
    }
}

/* ------------------------------------------------------------ driver */
static double now_s(void) {
    struct timespec t;
    clock_gettime(CLOCK_MONOTONIC, &t);
    return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

/* Loss and gradient (m, P) of all subdomains at the step's points x (n, 2).
 * times[4] (nullable): seconds of the lists, forward, POU/loss and reverse
 * stages; pairs_out (nullable): the pair count.  Returns 0, -1 when memory
 * runs out, -2 for a shape that is not compiled. */
int cs_loss_grad(const cs_problem* pb, const float* theta, const float* x, int64_t n, int nthreads, double* loss,
                 float* grad, double* times, int64_t* pairs_out) {
    const int H = pb->h;
    if (!(H == 8 || H == 16 || H == 32) || pb->m <= 0 || n < 0 || pb->npou < 1 || pb->npou > 64) return -2;
    cs_ctx cc = {0};
    cs_ctx* c = &cc;
    c->pb = pb;
    c->n = n;
    c->nthreads = nthreads;
    c->x = x;
    c->theta = theta;
    c->grad = grad;
    const double t0 = now_s();
    const int64_t nch = (n + CS_PT_CHUNK - 1) / CS_PT_CHUNK;
    if (reserve(&B_count, n + 1, 4) || reserve(&B_off, n + 1, 4) || reserve(&B_loss, nch + 1, 8) ||
        reserve(&B_sdoff, pb->m + 1, 4) || reserve(&B_itemoff, pb->m + 1, 4))
        return -1;
    c->pt_count = (int32_t*)B_count.p;
    c->pt_off = (int32_t*)B_off.p;
    c->loss_part = (double*)B_loss.p;
    c->sd_off = (int32_t*)B_sdoff.p;
    c->item_off = (int32_t*)B_itemoff.p;
    /* 1. lists: count, scan, fill */
    cs_parallel(c, t_count, nch);
    int64_t s = 0;
    for (int64_t p = 0; p < n; ++p) {
        c->pt_off[p] = (int32_t)s;
        s += c->pt_count[p];
    }
    c->pt_off[n] = (int32_t)s;
    c->s = s;
    const int AS = act_stride(H);
    if (reserve(&B_ntake, s, 4) || reserve(&B_mtake, s, 4) || reserve(&B_sdpair, s, 4) ||
        reserve(&B_rec, s, sizeof(float) * 2 * CS_J) || reserve(&B_seed, s, sizeof(float) * CS_J) ||
        reserve(&B_act, s, sizeof(float) * AS))
        return -1;
    c->n_take = (int32_t*)B_ntake.p;
    c->m_take = (int32_t*)B_mtake.p;
    c->sd_pair = (int32_t*)B_sdpair.p;
    c->rec = (float*)B_rec.p;
    c->seed = (float*)B_seed.p;
    c->act = (float*)B_act.p;
    cs_parallel(c, t_fill, nch);
    /* subdomain-major order (stable counting sort) and work items of <= CS_ITEM pairs */
    memset(c->sd_off, 0, sizeof(int32_t) * (pb->m + 1));
    for (int64_t e = 0; e < s; ++e) c->sd_off[c->m_take[e] + 1]++;
    for (int j = 0; j < pb->m; ++j) c->sd_off[j + 1] += c->sd_off[j];
    int64_t ni = 0;
    for (int j = 0; j < pb->m; ++j) {
        c->item_off[j] = (int32_t)ni;
        ni += (c->sd_off[j + 1] - c->sd_off[j] + CS_ITEM - 1) / CS_ITEM;
    }
    c->item_off[pb->m] = (int32_t)ni;
    if (reserve(&B_items, ni + 1, 3 * sizeof(int32_t)) || reserve(&B_gpart, ni + 1, sizeof(float) * n_params(H)))
        return -1;
    c->items = (int32_t*)B_items.p;
    c->gpart = (float*)B_gpart.p;
    {
        int32_t* pos = (int32_t*)malloc(sizeof(int32_t) * (pb->m + 1));
        if (!pos) return -1;
        memcpy(pos, c->sd_off, sizeof(int32_t) * (pb->m + 1));
        for (int64_t e = 0; e < s; ++e) c->sd_pair[pos[c->m_take[e]]++] = (int32_t)e;
        free(pos);
    }
    ni = 0;
    for (int j = 0; j < pb->m; ++j)
        for (int32_t b = c->sd_off[j]; b < c->sd_off[j + 1]; b += CS_ITEM) {
            c->items[3 * ni] = j;
            c->items[3 * ni + 1] = b;
            c->items[3 * ni + 2] = c->sd_off[j + 1] - b < CS_ITEM ? c->sd_off[j + 1] - b : CS_ITEM;
            ++ni;
        }
    c->n_items = ni;
    const double t1 = now_s();
    /* 2. forward */
    cs_parallel(c, H == 16 ? t_forward_16 : H == 8 ? t_forward_8 : t_forward_32, ni);
    const double t2 = now_s();
    /* 3 + 4. POU, residual, loss, seeds */
    cs_parallel(c, t_pou, nch);
    double L = 0.0;
    for (int64_t k = 0; k < nch; ++k) L += c->loss_part[k];
    *loss = n > 0 ? L / (double)n : 0.0;
    const double t3 = now_s();
    /* 5. reverse */
    cs_parallel(c, H == 16 ? t_adjoint_16 : H == 8 ? t_adjoint_8 : t_adjoint_32, ni);
    cs_parallel(c, t_reduce, pb->m);
    const double t4 = now_s();
    if (times) {
        times[0] = t1 - t0;
        times[1] = t2 - t1;
        times[2] = t3 - t2;
        times[3] = t4 - t3;
    }
    if (pairs_out) *pairs_out = s;
    return 0;
}

/* optax adam over (m, P) with the shared count (incremented first) */
void cs_adam(float* theta, float* m1, float* m2, const float* grad, int64_t total, int32_t* count, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    const int32_t cnt = *count + 1;
    const float c1 = 1.0f - powf(b1, (float)cnt), c2 = 1.0f - powf(b2, (float)cnt);
    for (int64_t i = 0; i < total; ++i) {
        const float g = grad[i];
        m1[i] = (1.0f - b1) * g + b1 * m1[i];
        m2[i] = (1.0f - b2) * g * g + b2 * m2[i];
        theta[i] -= lr * ((m1[i] / c1) / (sqrtf(m2[i] / c2) + eps));
    }
    *count = cnt;
}

/* One training step: lists, forward, loss, gradient (into grad), Adam.
 * Returns as cs_loss_grad; times[5] (nullable): the four stages and Adam. */
int cs_step(const cs_problem* pb, float* theta, float* m1, float* m2, float* grad, int32_t* count, const float* x,
            int64_t n, float lr, int nthreads, double* loss, double* times, int64_t* pairs_out) {
    const int rc = cs_loss_grad(pb, theta, x, n, nthreads, loss, grad, times, pairs_out);
    if (rc) return rc;
    const double t0 = now_s();
    cs_adam(theta, m1, m2, grad, (int64_t)pb->m * n_params(pb->h), count, lr);
    if (times) times[4] = now_s() - t0;
    return 0;
}

int cs_n_params(int h) { return n_params(h); }
