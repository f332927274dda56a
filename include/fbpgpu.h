/*
 * fbpgpu.h — C ABI of the GB300 FBPINN training-step library (libfbpgpu.so).
 *
 * The library replaces, with hand-written sm_103a kernels, the device work of
 * one FBPINN training step of the reference library (benmoseley/FBPINNs,
 * fbpinns v0.2.0), i.e. what `FBPINN_update` (fbpinns/trainers.py:285-296)
 * runs through XLA, plus the interaction-list construction that feeds it.
 *
 * Conventions
 *  - Every entry point returns an int status: FBP_OK (0) or a negative code;
 *    fbp_last_error() gives a message for the calling thread.  No C++
 *    exception crosses the ABI.
 *  - All pointers are caller-owned DEVICE memory unless the parameter says
 *    "host".  The library allocates nothing: scratch buffers are passed in
 *    and their sizes are queried with the matching *_scratch_bytes function.
 *  - Every call is stream-ordered on `stream` (a cudaStream_t, NULL = legacy
 *    default stream) and never synchronises the host, so a sequence of calls
 *    can be captured into a CUDA graph.  Data-dependent sizes (pair counts,
 *    work items) stay on the device; kernels clamp to the capacities they are
 *    given and report overflow through a device status word.
 *  - Floating point is FP32; the loss is accumulated in FP64.  Indices are
 *    int32, as in the reference (JAX without x64).
 *
 * Jet layout ("J components" per point or pair), for input dimension xd and a
 * bit mask d2 of dimensions that need a pure second derivative:
 *     [u, du/dx_0 .. du/dx_{xd-1}, d2u/dx_i^2 for each bit i of d2 (ascending)]
 * J = 1 + xd + popcount(d2).  This is the per-point set of derivative jets
 * that the reference obtains from nested forward-mode jvp
 * (fbpinns/trainers.py:213-247, _get_ujs / jacfwd).
 *
 * Per-pair and per-slot jet records ([first J values | second J values]) are
 * rows of R = 2J rounded up to a multiple of 4 floats (16-byte rows):
 * pair_out is (s, R) and slot_out is (u, R), both 16-byte aligned.
 */
#ifndef FBPGPU_H
#define FBPGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FBP_OK 0
#define FBP_ERR_INVALID (-1)      /* bad argument (shape, size, pointer) */
#define FBP_ERR_CUDA (-2)         /* a CUDA runtime call failed */
#define FBP_ERR_UNSUPPORTED (-3)  /* configuration with no compiled kernel */
#define FBP_ERR_CAPACITY (-4)     /* caller buffer too small */

/* d2mask flag: the second-derivative dims (bits 0-2) are carried as ONE jet
 * slot holding the sum of their pure second derivatives (a Laplacian),
 * instead of one slot per dim.  Enough for residuals that use only that sum
 * (Poisson, Helmholtz); the jet then has 1 + xd + 1 components. */
#define FBP_D2_LAPLACIAN 8
/* d2mask group (without FBP_D2_LAPLACIAN): the masked dims in `dims` share
 * one slot (the sum of their second derivatives, first), the other masked
 * dims keep a slot each; e.g. 7 | FBP_D2_GROUP(3) carries u_xx + u_yy and
 * u_tt for the wave residual u_xx + u_yy - u_tt / c^2. */
#define FBP_D2_GROUP(dims) (((dims) & 7) << 4)

/* Hidden-layer activations of the compiled networks (fbp_net.act). */
#define FBP_ACT_TANH 0           /* FCN (fbpinns/networks.py:61-68) */
#define FBP_ACT_SIN 1            /* SIREN (fbpinns/networks.py:102-131) */
#define FBP_ACT_ADAPTIVE_TANH 2  /* AdaptiveFCN a tanh(z/a) (networks.py:70-100); layers (W, b, a) */
#define FBP_ACT_ADAPTIVE_SIN 3   /* AdaptiveSIREN c sin(o z) (networks.py:133-163); layers (W, b, c, o) */
/* FourierFCN (networks.py:165-194) with one hidden layer after its features:
 * the first layer is the feature map, sin with frozen W1 = [omega; omega],
 * b1 = [0; pi/2] (sin(omega x), cos(omega x)), the second is tanh; the
 * gradients of W1 and b1 are written as zero. */
#define FBP_ACT_FOURIER 4

/* Window of each subdomain network (fbp_net.window), fbpinns/windows.py:
 * the decompositions use the cosine window (decompositions.py:197-199); the
 * others are the module's alternatives, each a product over dims of a 1D
 * window of the box (sigmoid also of its overlap widths wmin, wmax). */
#define FBP_WINDOW_COSINE 0    /* ((1 + cos(pi (x-mu)/sd)) / 2)^2, windows.py:25-35 */
#define FBP_WINDOW_SIGMOID 1   /* logistic ramps over wmin / wmax, windows.py:11-22 */
#define FBP_WINDOW_BUMP 2      /* exp(3 / (((x-mu)/sd)^2 - 1.001)) / exp(-3), windows.py:38-46 */
#define FBP_WINDOW_WENDLAND 3  /* (1-r)^4 (4r+1), r = |x-mu|/sd, windows.py:49-59 */
#define FBP_WINDOW_RBF 4       /* exp(-8 ((x-mu)/sd)^2) per dim, windows.py:62-68 */

/* Device status word bits (written by kernels into an int32 the caller owns). */
#define FBP_STATUS_PAIR_OVERFLOW 1      /* more pairs than the pair capacity */
#define FBP_STATUS_SLOT_OVERFLOW 2      /* more (point, level) slots than capacity */
#define FBP_STATUS_ITEM_OVERFLOW 4      /* more work items than capacity */
#define FBP_STATUS_LEVEL_ORDER 8        /* a point's levels are not in ascending model order */
#define FBP_STATUS_BAD_INDEX 16         /* an index out of range was skipped */
#define FBP_STATUS_TC_TIMEOUT 32        /* a tensor-core kernel gave up waiting for its MMAs */
/* Test hook of the time-out path, set by the caller in *status before
 * fbp_forward_pairs_tc: the kernel issues no MMAs, so its waits (limited to
 * 1 ms in this mode) run out; it sets FBP_STATUS_TC_TIMEOUT, frees its tensor
 * memory and returns, leaving the context usable.  No other kernel reads it. */
#define FBP_STATUS_TC_TEST_NO_MMA (1 << 30)

/* Maximum compiled sizes. */
#define FBP_MAX_XD 3
#define FBP_MAX_LEVELS 64   /* distinct POU levels (bit mask per point) */

/* ------------------------------------------------------------------ */
/* Geometry of the subdomain boxes and the uniform cell grid that       */
/* accelerates the point-in-box test.                                   */
/* ------------------------------------------------------------------ */
typedef struct fbp_boxes {
    const float* xmins;        /* (m, xd) closed box lower corners */
    const float* xmaxs;        /* (m, xd) upper corners */
    const int32_t* pou;        /* (m,) POU level of each box, 0 <= pou < 64 */
    const uint8_t* select;     /* (m,) nonzero = box takes part; NULL = all */
    int64_t m;
    int32_t xd;
    /* cell grid: cell index along dim d of a coordinate v is
     *   clamp(floor(((double)v - lo[d]) * inv_h[d]), 0, ncell[d]-1)
     * computed with IEEE double round-to-nearest on host and device alike,
     * so a box registered in cells [cell(xmin), cell(xmax)] is a candidate
     * of every point it contains. */
    int32_t ncell[FBP_MAX_XD];
    double lo[FBP_MAX_XD];
    double inv_h[FBP_MAX_XD];
    const int32_t* cell_start;  /* (ncells+1,) CSR offsets, cell id = c0 + n0*(c1 + n1*c2) */
    const int32_t* cell_boxes;  /* (entries,) box ids, ascending within each cell */
} fbp_boxes;

/* ------------------------------------------------------------------ */
/* Network / decomposition description for the per-pair jet kernels.   */
/* ------------------------------------------------------------------ */
typedef struct fbp_net {
    int32_t xd;           /* input dimension (1..3) */
    int32_t h1;           /* first hidden width */
    int32_t h2;           /* second hidden width (0 = one hidden layer) */
    int32_t ud;           /* output dimension, must be 1 */
    int32_t d2mask;       /* dims with a pure second-derivative jet */
    int32_t nparam;       /* P: parameters per subdomain (packed layout below) */
    int32_t act;          /* hidden-layer activation, FBP_ACT_* */
    /* theta (m, P): for each layer in order, W (fan_out, fan_in) row-major,
     * b (fan_out), then the layer's activation parameters (fan_out each: a
     * for FBP_ACT_ADAPTIVE_TANH, c then o for FBP_ACT_ADAPTIVE_SIN; the
     * output layer's are unused) — the reference's per-layer parameter tuples
     * flattened (fbpinns/networks.py:43-194). */
    const float* theta;
    const float* xmins;   /* (m, xd) subdomain boxes (norm + window) */
    const float* xmaxs;   /* (m, xd) */
    const float* flags;   /* (m,) window flag (decompositions.py:169-172) */
    const float* unnorms; /* (m, 2) (mu, sd) of the output unnormalisation */
    int64_t m;
    int32_t window;       /* FBP_WINDOW_* (0: cosine) */
    const float* wmins;   /* (m, xd) overlap widths below / above the box: */
    const float* wmaxs;   /* read by FBP_WINDOW_SIGMOID only (nullable otherwise) */
} fbp_net;

/* Pair lists sorted subdomain-major, and the work queue over them. */
typedef struct fbp_pairs {
    const int32_t* sd_start;  /* (m+1,) offsets of each subdomain's pairs */
    /* (s, 4) one 16-byte record per sorted pair, 16-byte aligned: its
     * point-major pair index, point index, (point, level) slot, 0 */
    const int32_t* sd_rec;
    const int32_t* items;     /* (cap, 3) work items: (subdomain, begin, count) */
    const int32_t* n_items;   /* device count of valid items */
    int64_t items_cap;
    int64_t slots_cap;        /* rows of the slot buffer; larger slot ids are skipped */
    /* Optional (NULL: static schedule, CTA b takes items b, b + grid, ...): one
     * device int32 that the jet launchers zero before each launch and their
     * CTAs then take items from in turn, so that CTAs delayed by kernels of
     * other streams take fewer.  The results do not depend on the schedule.
     * Concurrent launches need distinct counters. */
    int32_t* item_ctr;
    /* Optional (NULL: the adjoint recomputes them): the layer-2
     * pre-activation jets of every sorted pair, float32, component-major
     * ((c * h2 + k) * zs_cap + sorted pair index; zs_cap >= the pair count).
     * fbp_forward_pairs and fbp_forward_pairs_tc write them for networks with
     * two hidden layers; fbp_adjoint_pairs then reads them instead of
     * recomputing layer 2.  The adjoint must follow a forward of the same
     * lists and parameters with the same buffer. */
    float* zs;
    int64_t zs_cap;
} fbp_pairs;

/* Built-in PDE residuals fused into the POU/loss kernel. */
#define FBP_PROBLEM_NONE 0
#define FBP_PROBLEM_HO_HARDBC 1     /* problems.py:149-206 */
#define FBP_PROBLEM_BURGERS 2       /* problems.py:276-326 */
#define FBP_PROBLEM_POISSON2D 3     /* new: -lap u = f, hard zero BC */
#define FBP_PROBLEM_WAVE_C 4        /* problems.py:346-405, constant velocity */
#define FBP_PROBLEM_HELMHOLTZ2D 5   /* new: -lap u - k^2 u = f, hard zero BC */

typedef struct fbp_problem {
    int32_t kind;
    int32_t n_int;        /* integer parameter (Poisson: number of frequencies) */
    float p[8];           /* scalar parameters, meaning per kind (see problems.py) */
    const float* gauss;   /* (ng, 4) Gaussians [mx, my, sd, amp] (wave source, Helmholtz f) */
    int32_t ng;
    /* Scheduled training (nullable, together): points with pt_keep[p] == 0
     * add nothing to the loss and get no seeds, and the loss is the mean over
     * the *n_keep kept points (both device arrays, from fbp_train_mask);
     * fbp_loss_finalize is then called with scale 1. */
    const uint8_t* pt_keep;
    const int32_t* n_keep;
} fbp_problem;

/* ------------------------------------------------------------------ */
/* Entry points                                                        */
/* ------------------------------------------------------------------ */

int fbp_abi_version(void);
const char* fbp_last_error(void);

/* Scratch for fbp_scan_i32 over n elements. */
size_t fbp_scan_scratch_bytes(int64_t n);

/* Exclusive prefix sum of int32 counts: out[0..n] with out[n] = total.
 * Generic helper of the interaction-list build (the cumsum of
 * fbpinns/decompositions_base.py:58). */
int fbp_scan_i32(const int32_t* in, int32_t* out, int64_t n,
                 void* scratch, size_t scratch_bytes, void* stream);

/* Scheduled training on the device: the points and subdomain states of one
 * scheduler mask, without a host round trip.  raw (m, uint8) holds the
 * scheduler's states (0 inactive, 1 active, 2 fixed).  For the interaction
 * lists (pt_off, m_take) of all n points: pt_keep[p] = 1 where point p lies in
 * a box whose raw state is 1 (the training points), *n_keep = their number;
 * state[j] = 1 where box j holds a kept point and its raw state is 0 or 1,
 * 2 where it holds one and is fixed, else 0; active[j] = (state[j] == 1).
 * Replaces _get_x_batch (fbpinns/trainers.py:482-507) and the active-mask
 * update of get_inputs (fbpinns/trainers.py:339-357). */
int fbp_train_mask(const int32_t* pt_off, const int32_t* m_take, int64_t n, int64_t s_cap,
                   const uint8_t* raw, int64_t m, uint8_t* pt_keep, int32_t* n_keep,
                   uint8_t* state, uint8_t* active, void* stream);

/* fbp_sort_pairs over the pairs of kept points only (pt_keep[point] != 0,
 * from fbp_train_mask): the pairs of x_batch, the training points of the
 * scheduler mask, in the same stable order.  Replaces the per-change
 * re-index of the takes (fbpinns/trainers.py:509-575). */
int fbp_sort_pairs_kept(const int32_t* m_take, const int32_t* n_take, const int32_t* p_take,
                        const uint8_t* pt_keep, const int32_t* s_dev, int64_t s_cap, int64_t m,
                        int32_t* sd_start, int32_t* sd_rec, void* scratch, size_t scratch_bytes,
                        void* stream);

/* Largest n accepted by fbp_scan_i32_noalloc. */
#define FBP_SCAN_NOALLOC_MAX_N (1 << 24)

/* fbp_scan_i32 without a scratch argument, for callers that cannot allocate
 * device memory (so cannot pass a scratch buffer): its scratch is a fixed
 * array of about 32 KiB (8193 int32) inside the library, which every GPU that
 * loads the library keeps until the process exits.  n must not exceed
 * FBP_SCAN_NOALLOC_MAX_N (FBP_ERR_CAPACITY otherwise).  The first call on each
 * device looks up that array's device address, so make it before capturing a
 * stream into a CUDA graph; the address is cached per device, so do not call
 * it on a device again after a cudaDeviceReset of that device.  All calls
 * share the one array: calls that overlap on the GPU (for example on two
 * streams at once) race and must be serialised by the caller.
 * No counterpart in the reference: it is an addition of this library. */
int fbp_scan_i32_noalloc(const int32_t* in, int32_t* out, int64_t n, void* stream);

/* Count pass of the point-in-box test.  For every point: the number of
 * selected boxes that contain it (pt_count), the bit mask of their POU levels
 * (pt_lvl) and its popcount (pt_nlvl).  model_count (nullable) receives the
 * number of points inside each box.  pt_hit / pt_cand (nullable, together)
 * receive the hits as a bit mask over the point's cell candidate list and
 * that list's start, or -1 when the cell has more than 64 candidates; the
 * fill pass then reads the hits instead of testing again.
 * Replaces _inside_sum_batch
 * (fbpinns/decompositions_base.py:24-48) as used by inside_points /
 * inside_models (fbpinns/decompositions.py:202-215). */
int fbp_inside_count(const float* x, int64_t n, const fbp_boxes* boxes,
                     int32_t* pt_count, int32_t* pt_nlvl, uint64_t* pt_lvl,
                     int32_t* model_count, uint64_t* pt_hit, int32_t* pt_cand,
                     void* stream);

/* Fill pass: writes the interaction lists in the reference's point-major,
 * box-minor order (n_take, m_take = box id) and the unique (point, level)
 * slots (p_take, np_take) in the order of
 * jnp.unique(stack(n_take, pou[m_take]), axis=0, return_inverse=True).
 * pt_off / np_off are the exclusive scans of pt_count / pt_nlvl (n+1 long).
 * pt_hit / pt_cand: from fbp_inside_count on the same points and boxes
 * (select included), or NULL to test the candidates again.
 * Replaces _inside_take_batch (fbpinns/decompositions_base.py:51-68) and the
 * POU unique of get_inputs (fbpinns/trainers.py:379-388). */
int fbp_inside_fill(const float* x, int64_t n, const fbp_boxes* boxes,
                    const int32_t* pt_off, const int32_t* np_off, const uint64_t* pt_lvl,
                    const uint64_t* pt_hit, const int32_t* pt_cand,
                    int32_t* n_take, int32_t* m_take, int32_t* p_take, int32_t* np_take,
                    int64_t s_cap, int64_t u_cap, int32_t* status, void* stream);

/* out[i] = inv[in[i]] for i < *count_dev (or < n when count_dev is NULL):
 * the re-index of m_take to positions in all_ims = [active; fixed]
 * (fbpinns/trainers.py:367-372). */
int fbp_gather_i32(const int32_t* in, int64_t n, const int32_t* count_dev,
                   const int32_t* inv, int32_t* out, void* stream);

/* Flag compaction: out receives, in ascending order, every i < n with
 * flag[i] != 0 (i.e. jnp.arange(n)[flag]); *count_dev = how many.
 * Used for inside_ips / training_ips (fbpinns/decompositions_base.py:81,
 * fbpinns/trainers.py:487). */
size_t fbp_compact_scratch_bytes(int64_t n);
int fbp_compact_flags(const int32_t* flag, int64_t n, int32_t* out, int32_t* count_dev,
                      void* scratch, size_t scratch_bytes, void* stream);

/* Stable counting sort of the point-major pairs by subdomain: for each
 * subdomain its pairs in ascending point order.  Writes sd_start (m+1) and
 * sd_rec (s_cap, 4): per sorted pair its point-major pair index, point,
 * slot and 0 (sd_rec 16-byte aligned).  The boxes of any one point must be
 * distinct (as inside_fill writes them).  s_dev is the device pair count
 * (pt_off[n]).
 * No reference counterpart: the reference gathers per-pair parameter copies
 * (fbpinns/trainers.py:141-145) instead of grouping pairs by subdomain. */
size_t fbp_sort_scratch_bytes(int64_t s_cap, int64_t m);
int fbp_sort_pairs(const int32_t* m_take, const int32_t* n_take, const int32_t* p_take,
                   const int32_t* s_dev, int64_t s_cap, int64_t m,
                   int32_t* sd_start, int32_t* sd_rec, void* scratch, size_t scratch_bytes, void* stream);

/* Work queue: each subdomain with select[j] != 0 (NULL = all) contributes
 * ceil(count/chunk) items (subdomain, begin, count) in subdomain order.
 * Also writes item_start (m+1): the first item of each subdomain. */
size_t fbp_work_scratch_bytes(int64_t m);
int fbp_build_work(const int32_t* sd_start, int64_t m, const uint8_t* select, int32_t chunk,
                   int32_t* items, int32_t* item_start, int32_t* n_items, int64_t items_cap,
                   int32_t* status, void* scratch, size_t scratch_bytes, void* stream);

/* Per-pair forward jets: for every pair in the work items, the jets of
 * u_j(x) * w_j(x) and of w_j(x) (J + J floats in row `pair` of pair_out), where
 * u_j = unnorm(FCN_j(norm(x))) and w_j is the cosine window.
 * Replaces the vmapped FBPINN_model_inner under nested jvp
 * (fbpinns/trainers.py:113-118,158, 219-227; networks.py:61-68;
 * decompositions.py:184-199; windows.py:25-35). */
int fbp_forward_pairs(const fbp_net* net, const float* x, const fbp_pairs* pairs,
                      float* pair_out, int32_t grid, void* stream);

/* Same records as fbp_forward_pairs, with layer 2 of every jet component on
 * the 5th-generation tensor cores (tcgen05, TF32 operands split hi + lo, three
 * products, FP32 accumulation in tensor memory).  Compiled for xd = 2 with two
 * 16-wide hidden layers only (FBP_ERR_UNSUPPORTED otherwise; see
 * fbp_has_tc_shape for the jet masks and activations).  A kernel that
 * times out waiting for its MMAs sets FBP_STATUS_TC_TIMEOUT in *status and
 * leaves its remaining pairs unwritten.  Same reference functions as
 * fbp_forward_pairs. */
int fbp_forward_pairs_tc(const fbp_net* net, const float* x, const fbp_pairs* pairs,
                         float* pair_out, int32_t* status, int32_t grid, void* stream);

/* 1 if the per-pair jet kernels are compiled for this network shape, jet
 * mask and activation (FBP_ACT_*; ud = 1), else 0.  Lets a caller fail early
 * with a clear message. */
int fbp_has_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act);

/* 1 if fbp_forward_pairs_tc is compiled for this shape, jet mask and
 * activation, else 0. */
int fbp_has_tc_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act);

/* POU combination per point (the two segment sums and the divide of
 * fbpinns/trainers.py:162-170, on jets by the quotient rule):
 *   slot_out[u] = (U_l jets, W_l jets) of each (point, level) slot,
 *   U[p]        = sum over levels of U_l / npou  (n x J).               */
int fbp_pou_forward(int32_t xd, int32_t d2mask, int64_t n, int32_t npou,
                    const int32_t* pt_off, const int32_t* p_take, const float* pair_out,
                    float* slot_out, float* U, int64_t s_cap, int64_t u_cap,
                    int32_t* status, void* stream);

/* Adjoint of fbp_pou_forward: from dL/dU (n x J) to the per-slot seeds
 * dL/dN_l (written into the first J floats of each slot record). */
int fbp_pou_backward(int32_t xd, int32_t d2mask, int64_t n, int32_t npou,
                     const int32_t* np_off, const float* U_bar, float* slot_out, int64_t u_cap,
                     void* stream);

/* Fused POU + constraining operator + residual + loss (built-in problems):
 * forward POU, hard-constraint ansatz jets, PDE residual, FP64 per-block
 * sums of residual^2 (loss_part), and the seeds dL/dN_l per slot (written
 * into slot_out).  The loss is mean(residual^2) over the n points
 * (problems.py loss_fn's).  U_out (nullable) receives the constrained jets.
 * Pairs at or beyond s_cap and slots at or beyond u_cap (capacity overflow,
 * already flagged by fbp_inside_fill) are skipped.
 * Replaces constraining_fn + loss_fn inside FBPINN_loss
 * (fbpinns/trainers.py:174, 249-267). */
int fbp_pou_loss(int32_t xd, int32_t d2mask, const fbp_problem* prob,
                 int64_t n, int32_t npou, const float* x,
                 const int32_t* pt_off, const int32_t* np_off, const int32_t* p_take,
                 const float* pair_out, float* slot_out, float* U_out,
                 int64_t s_cap, int64_t u_cap,
                 double* loss_part, int32_t n_part, int32_t* status, void* stream);

/* Deterministic sum of the n_part FP64 partials, times scale. */
int fbp_loss_finalize(const double* loss_part, int32_t n_part, double scale,
                      double* loss, void* stream);

/* Per-pair adjoint: recomputes the forward jets per pair in registers and
 * back-propagates the slot seeds through window product, unnormalisation and
 * the FCN jet, writing one gradient partial (P floats) per work item.
 * Replaces XLA's reverse-mode transpose of the model under value_and_grad
 * (fbpinns/trainers.py:292). */
int fbp_adjoint_pairs(const fbp_net* net, const float* x, const fbp_pairs* pairs,
                      const float* slot_out, float* grad_part, int32_t grid, void* stream);

/* fbp_adjoint_pairs with the layer-2 recompute on the tensor cores: per tile
 * of 128 pairs the jets z_c = W2 v_c of the forward are J tcgen05 GEMMs
 * (TF32 operands split hi + lo, three products, FP32 accumulation in TMEM),
 * and the CUDA cores run the rest of the adjoint.  tanh networks xd-16-16-1
 * (fbp_has_tc_adjoint_shape); the same gradient partials up to FP32
 * rounding.  Bounded waits as fbp_forward_pairs_tc (FBP_STATUS_TC_TIMEOUT in
 * *status; FBP_STATUS_TC_TEST_NO_MMA exercises that path).
 * Replaces XLA's reverse-mode transpose of the model (fbpinns/trainers.py:292). */
int fbp_adjoint_pairs_tc(const fbp_net* net, const float* x, const fbp_pairs* pairs,
                         const float* slot_out, float* grad_part, int32_t* status,
                         int32_t grid, void* stream);

/* 1 if fbp_adjoint_pairs_tc is compiled for this shape, jet mask and activation. */
int fbp_has_tc_adjoint_shape(int32_t xd, int32_t h1, int32_t h2, int32_t d2mask, int32_t act);

/* grad[j] = sum of the partials of subdomain j's items, in item order. */
int fbp_grad_reduce(const float* grad_part, const int32_t* item_start, int64_t m,
                    int32_t nparam, float* grad, void* stream);

/* Adam (optax.adam defaults and ordering, the shared step count) applied to
 * rows j with state[j] == 1 only; other rows untouched.  count_dev is the
 * int32 step count, incremented on the device.  Replaces optax.adam update +
 * apply_updates (fbpinns/trainers.py:294-295, 430-431). */
int fbp_adam(float* theta, float* m1, float* m2, const float* grad, const uint8_t* state,
             int64_t m, int32_t nparam, float lr, float b1, float b2, float eps, float eps_root,
             int32_t* count_dev, void* stream);

/* Uniform points in the box [xmin, xmax] (host arrays, xd values) from a
 * counter-based Philox-4x32-10 stream (seed, offset + *counter): x = xmin +
 * (xmax-xmin)*u as in fbpinns/domains.py:136-140 (sampler "uniform").
 * counter (nullable, device int32) lets a captured graph draw new points on
 * every replay (e.g. the Adam step count). */
int fbp_sample_uniform(float* x, int64_t n, int32_t xd, const double* xmin, const double* xmax,
                       uint64_t seed, uint64_t offset, const int32_t* counter, void* stream);

/* Scratch bytes of fbp_sort_points_cells for n points of dimension xd. */
size_t fbp_sort_points_scratch_bytes(int64_t n, int32_t xd);

/* x_out (n, xd) = the points x_in in the order of the Morton index of a
 * regular grid of cells over [xmin, xmax] (about 64 points per cell, at most
 * 2^16 cells), points of one cell in their input order: a stable counting
 * sort, so the result depends on the input only.  The reference's uniform
 * batches (fbpinns/domains.py:113-142) are i.i.d. and enter the loss as a mean,
 * so the ordered batch is the same batch; the order keeps points that share
 * subdomains together for the interaction lists and the jet kernels.  A cell
 * of L points is ordered in O(L^2) work (one warp per cell), so batches
 * concentrated in a few cells of the box order correctly but slowly.  x_in
 * and x_out must not overlap.  Asynchronous on stream; no host
 * synchronisation. */
int fbp_sort_points_cells(const float* x_in, int64_t n, int32_t xd, const double* xmin, const double* xmax,
                          float* x_out, void* scratch, size_t scratch_bytes, void* stream);


/* Executable graph of a captured training step (cudaGraph_t graph) whose
 * kernel nodes keep the priority of the stream they were captured from
 * (graph instantiated with cudaGraphInstantiateFlagUseNodePriority), so
 * that the next step's interaction lists, captured on a high-priority
 * stream, take SM slots ahead of the step's own kernels.  Replaces the
 * reference's jit/AOT compile of the update (fbpinns/trainers.py:650-652);
 * *exec_out is released by fbp_graph_exec_destroy. */
int fbp_graph_instantiate(void* graph, int32_t use_node_priority, void** exec_out);
int fbp_graph_launch(void* exec, void* stream);
int fbp_graph_exec_destroy(void* exec);

/* FP32 FMA throughput probe used for the roofline denominator: runs
 * `iters` dependent-chain FMA loops on every SM; *flops_out (host) gets the
 * flop count of the launch. */
int fbp_fma_probe(float* sink, int32_t blocks, int32_t iters, double* flops_out, void* stream);

/* Evaluates the device tanh used inside the jet kernels, y[i] = tanh(x[i]),
 * so that its error can be checked against a reference tanh.  No counterpart
 * in the reference (which calls jnp.tanh, fbpinns/networks.py:64). */
int fbp_tanh_probe(const float* x, float* y, int64_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FBPGPU_H */
