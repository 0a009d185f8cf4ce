/* fpde_gb300.h -- C ABI of the GB300 (sm_103a) implementation of FPDE_HPC's hot path:
 * the Caputo / distributed-order L1 history sum and the per-step implicit tridiagonal
 * (Thomas / LOD) line solves.
 *
 * This header replaces the reference's OpenCL/CUDA backend seam (the OpenCL_* classes of
 * opencl_cuda_class.h:4-67 and the run-time-compiled kernels driven through them by
 * fpde_hpc_1d.cpp and fr_do.cpp). Every entry point names the reference interface it
 * stands in for. Conventions:
 *   - every function returns FPDE_OK (0) or an FPDE_ERR_* code; nothing exits the
 *     process (the reference calls exit(0) on any backend error, opencl_cuda_base.cpp:14-17);
 *     fpde_last_error_string() describes the last failure of the calling thread;
 *   - pointers are plain C pointers; an `on_device` flag says whether a buffer is in device
 *     memory (of the context's GPU) or in host memory. Host buffers are copied in/out by the
 *     call; device buffers are used in place;
 *   - a context owns every device allocation made through it; one context per host thread;
 *   - lines have N intervals and nodes 0..N; unknowns are 1..N-1 and nodes 0 and N carry
 *     the boundary conditions (fpde_hpc_1d.cpp:2381-2388);
 *   - the tridiagonal systems use the reference's sign convention
 *         A[i] U[i-1] - R[i] U[i] + B[i] U[i+1] = Om[i]        (fpde_hpc_1d.cpp:3094)
 */
#ifndef FPDE_GB300_H
#define FPDE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FPDE_ABI_VERSION 1

enum fpde_status {
    FPDE_OK = 0,
    FPDE_ERR_ARG = 1,          /* invalid argument (null pointer, size, mode) */
    FPDE_ERR_CUDA = 2,         /* a CUDA runtime call failed */
    FPDE_ERR_NOMEM = 3,        /* device or host allocation failed */
    FPDE_ERR_CAPACITY = 4,     /* history full / size above a fixed maximum */
    FPDE_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up (error flag set) */
    FPDE_ERR_UNSUPPORTED = 6,  /* feature not available on this device / build */
    FPDE_ERR_NUMERIC = 7       /* non-finite value detected where one is not allowed */
};

/* History storage / arithmetic of the L1 sum. */
enum fpde_precision {
    FPDE_PREC_FP64 = 0,        /* FP64 increments, FP64 FMA sum (the plain method) */
    FPDE_PREC_SPLIT_BF16 = 1,  /* far history as bf16 hi+lo on tensor cores, FP64 fold */
    FPDE_PREC_SPLIT_F16 = 2,   /* same with fp16 hi+lo (per-block power-of-two scaling) */
    FPDE_PREC_SPLIT_BF16X3 = 3 /* far history as three exact bf16 slices (8-bit integers with
                                  per-node/per-block exponents), six products per k-step, leading
                                  product summed exactly; FP64 fold */
};

/* Boundary condition kinds of a line end (al1 :4002-4027, bt1 :4585, U1 :4683-4719). */
enum fpde_bc_kind {
    FPDE_BC_DIRICHLET = 0,     /* U = value */
    FPDE_BC_FLUX = 1           /* left: Al[1] = 1, Bt[1] = value; right: flux closure */
};

typedef struct fpde_ctx fpde_ctx;
typedef struct fpde_hist fpde_hist;
typedef struct fpde_line fpde_line;
typedef struct fpde_lod3d fpde_lod3d;
typedef struct fpde_batch fpde_batch;

/* ---------------------------------------------------------------- context */

/* Create a context on CUDA device `device` with its own stream.
 * Replaces OpenCL_program(int gpu) + create_queue (opencl_cuda_class.h:57-60;
 * CUDA impl opencl_cuda_base.cpp:759-785), which always used device 0. */
int fpde_ctx_create(int device, fpde_ctx **out);
/* Destroy a context and everything allocated through it (~OpenCL_program,
 * opencl_cuda_base.cpp:786-801). */
int fpde_ctx_destroy(fpde_ctx *ctx);
/* Use a caller-provided cudaStream_t (passed as void*) for all work of this context;
 * NULL restores the context's own stream. No counterpart: the reference is synchronous. */
int fpde_ctx_set_stream(fpde_ctx *ctx, void *cuda_stream);
/* Wait for all work of the context (OpenCL_commandqueue::Finish, opencl_cuda_class.h:45). */
int fpde_ctx_synchronize(fpde_ctx *ctx);
/* Number of streaming multiprocessors of the context's device. */
int fpde_ctx_sm_count(const fpde_ctx *ctx, int *out);
/* Description of the last error on this host thread ("" if none). Replaces the
 * reference's printf-and-exit error reporting (SERROR, opencl_cuda_base.cpp:14-17). */
const char *fpde_last_error_string(void);
/* Number of kernels this library has launched on the calling host thread (a counter for
 * benchmarks). */
int64_t fpde_kernel_launch_count(void);

/* ------------------------------------------------------------ L1 weights */

/* FP64 closed-form L1 weights of step n from the time points time[0..n+1]:
 *   kb[t] = int_{time[t]}^{time[t+1]} (time[n+1]-s)^{-alpha} ds,  t = 0..n-1,
 *   kkk0  = int_{time[n]}^{time[n+1]} (time[n+1]-s)^{-alpha} ds
 * evaluated cancellation-free. Replaces kb() / precalc_kb_3() / init_time_step()
 * (fpde_hpc_1d.cpp:2167-2301, :4069-4085, :3942-3949), which approximate the same
 * integrals by truncated series. Host function; kb may be NULL when n == 0. */
int fpde_weights_l1(double alpha, const double *time, int n, double *kb, double *kkk0);

/* Lag form for uniform steps: b[j] = (j+1)^{1-alpha} - j^{1-alpha}, j = 0..n-1,
 * cancellation-free (so kb[t] of step n = tau^{1-alpha}/(1-alpha) * b[n-t]). Host. */
int fpde_weights_l1_lags(double alpha, int n, double *b);

/* Generalized-kernel L1 weights on the device, any time points (kb :2167-2301 with the
 * generalized Caputo kernel g(t) = t^p of func_in_kernel, g :1889-1930: 0 -> p = 1,
 * 1 -> p = 0.5, 2 -> p = 2, 3 -> p = func_power; variable steps as varT). For every step n in
 * [n0, n1], with T = time[n+1]:
 *   out[(n-n0)*ld + t] = int_{time[t]}^{time[t+1]} (T^p - s^p)^{-alpha} ds,  t = 0..n-1 (kb_3_cache)
 *   out[(n-n0)*ld + n] = the same over [time[n], T]                       (kkk0)
 * evaluated in FP64 by quadrature (the reference sums truncated series, which converge
 * slowly on intervals that start at t = 0 when p is not 1). Entries past t = n are left
 * unchanged. time: n1 + 2 strictly increasing points with time[0] = 0, ld >= n1 + 1,
 * 0 < p, 0 <= alpha <= 1 (alpha = 1: kb = 0, kkk0 = 1 as the reference). on_device: 0 host
 * arrays, 1 device arrays, 2 device arrays stream-ordered (returns after launching). */
int fpde_weights_g(fpde_ctx *ctx, double p, double alpha, const double *time, int n0, int n1, double *out,
                   int64_t ld, int on_device);

/* Restricted summing's window (the reference's sum_alg 1, time_summing :4117-4131: newest
 * first, the sum stops before the first term whose |kb| is below sum_param): with kb_lag[j] the
 * weight of lag j + 1 (j = 0..n-1), *max_lag = the number of lags kept (n when none is below
 * eps). Host function; fpde_line_create and fpde_lod3d_create apply it to their lag weights
 * (kb = w tau / Da) when restrict_eps > 0. */
int fpde_restricted_lags(const double *kb_lag, int n, double eps, int *max_lag);

/* Gamma function (FP64, host). Used for Da = 1/Gamma(1-alpha) (fpde_hpc_1d.cpp:3598-3605)
 * and the distributed-order normalisers Gamma(2-alpha) (fr_do.cpp:337-341). */
int fpde_gamma(double x, double *out);

/* Fused distributed-order weights (host, FP64). The DO derivative of fr_do.cpp
 * (DO_Cder :89-113, GPU Fill/DOC/Sum :136-252) evaluates, per order a_q, the L1 Caputo sum
 * with bk((l+1)tau, l tau, a_q) = ((l+1)tau)^{1-a_q} - (l tau)^{1-a_q} divided by
 * Gamma(2-a_q), and then integrates over a with weights. All of that is linear in the
 * history, so the orders fuse into one lag-weight vector:
 *   c[l] = sum_q qw[q] * tau^{1-a_q} * b_l(a_q) / gnorm[q],   l = 0..n-1,
 * b_l(a) = (l+1)^{1-a} - l^{1-a} in cancellation-free form. qw holds the quadrature weights
 * of the a-integral times the weight function (fr_do: trapezoid x WA, :108-110), gnorm
 * Gamma(2 - a_q) (NULL: computed). The DO derivative of samples F at time t is then
 * sum_j (F[j+1]-F[j])/tau * c[t-j-1], and c[0] is the local weight b0 of eq_init (:688-690).
 * Replaces the per-order bkk table (Fill) and the order loop of DOC and Sum. */
int fpde_do_weights(int n_orders, const double *a, const double *qw, const double *gnorm, double tau, int n,
                    double *c);

/* DO derivative of sampled series on the device (replaces DO_Cder_CUDA, fr_do.cpp:361-430,
 * with its kernels Fill/DOC/Sum :136-252, for use_f > 0 arrays):
 *   DF[pt*ldd + t] (+)= sum_{j in [max(j0,0), min(t, maxt))} (F[pt*ldf+j+1] - F[pt*ldf+j])/tau * c[t-j-1]
 * for t in [t0, ntau) and every node pt < nodes; maxt = -1 sums up to t (the reference's
 * convention), append != 0 adds to DF (Sum's append). F, c (>= ntau fused weights of
 * fpde_do_weights) and DF are device pointers; runs on the context's stream. */
int fpde_do_derivative(fpde_ctx *ctx, const double *F, int64_t nodes, int64_t ldf, int ntau, double tau,
                       const double *c, int t0, int j0, int maxt, double *DF, int64_t ldd, int append);

/* ---------------------------------------------------------- L1 history sum */

/* Create a history of `nodes` values per snapshot with room for `max_steps` increments.
 * Replaces the reference's snapshot buffer boldU and its doubling resize
 * (init_opencl / fr_ocl_check_and_resize, fpde_hpc_1d.cpp:1715-1818): increments are
 * stored instead of snapshots and capacity is fixed up front. precision: fpde_precision
 * (FPDE_PREC_FP64 for this interface). */
int fpde_history_create(fpde_ctx *ctx, int64_t nodes, int64_t max_steps, int precision,
                        fpde_hist **out);
int fpde_history_destroy(fpde_hist *h);
/* Forget all snapshots (length 0). */
int fpde_history_reset(fpde_hist *h);
/* Number of stored increments. */
int fpde_history_length(const fpde_hist *h, int64_t *n);
/* Push a snapshot (the reference's oldH.push_back, calc_step :5104-5132 / :5729-5745).
 * The first push stores the base state; each later push stores the increment
 * u - previous snapshot. u has `nodes` values. */
int fpde_history_append(fpde_hist *h, const double *u, int on_device);
/* One step's history sum (time_summing :4086-4164 / the GPU Sum kernel :1407-1478, sum_alg 0):
 *   S[i] = scale * sum_{t<n} (kb[t] * D_t[i]) / tau[t]
 * over the n stored increments. kb and tau are host arrays of n values (tau may be NULL,
 * meaning all 1); S has `nodes` values (host or device per out_on_device). */
int fpde_l1_sum(fpde_hist *h, const double *kb, const double *tau, double scale,
                double *S, int out_on_device);

/* The reference's Sum kernel contract taken literally (fpde_hpc_1d.cpp:1407, sum_alg 0,
 * args :1851-1868): S[id] = sum_{t=0}^{old_size-2} kb_3_cache[t]*(old[(t+1)*OS+id]-old[t*OS+id])/tau[t]
 * for id < nodes, from time-major snapshots. All pointers per on_device. */
int fpde_sum_snapshots(fpde_ctx *ctx, double *S, const double *old, int old_size, int64_t OS,
                       int64_t nodes, const double *tau, const double *kb_3_cache, int on_device);

/* The reference's Sum kernel with every history mode it compiles in (fpde_hpc_1d.cpp:1407-1478,
 * the sum_alg and BS defines; its arguments S, old, old_size, tau, Htmp, row2_precalc,
 * kb_3_cache, sum_param, gtj, gt, alpha, tstep in the reference's order, args set :1851-1868;
 * CPU form time_summing :4108-4151). Snapshots are time-major, old[t*OS + id], id < nodes.
 *   sum_alg 0: S[id] = sum_{t=old_size-2..0} kb_3_cache[t]*(old[t+1]-old[t])/tau[t]
 *              (as fpde_sum_snapshots, with kb/tau formed once per weight and FMAs).
 *   sum_alg 1: restricted summing, the same terms from the newest down while the weight stays
 *              at or above sum_param:
 *                bs == 0: time_summing's rule (:4117-4131): stop before the first term with
 *                         |kb_3_cache[t]| < sum_param;
 *                bs  > 0: the GPU kernel's rule with BS = bs: whole chunks of bs terms (weights
 *                         before t = 0 count as 0), stopping after the first chunk whose bs
 *                         weights are all below sum_param.
 *   sum_alg 2: series expansion (:4137-4151, :1457-1475) with P = (int)sum_param (1..128; the
 *              reference's truncation)
 *              moments per node in Htmp[id*P + j] (updated in place), from the two snapshots
 *              old[0..OS) and old[OS..2*OS) (old_size >= 2; otherwise S = 0 and Htmp unchanged):
 *                d = old[OS+id] - old[id]
 *                Htmp[id*P+j] += gt^(j+1) * row2_precalc[j] * d,            j < P
 *                S[id] = sum_j v_j * Htmp[id*P+j] / tau[tstep],
 *                v_0 = gtj^-alpha,  v_j = v_{j-1} * (alpha + j - 1) / (j * gtj),
 *              with the GPU kernel's guards (a non-finite d, row2_precalc[j], power or v_j
 *              counts as 0). gt, gtj: g(t) at the step's two ends.
 * Arrays: old (old_size rows; 2 for sum_alg 2), tau (old_size-1 values, or at least tstep+1 for
 * sum_alg 2), kb_3_cache (old_size-1), Htmp (nodes*P), row2_precalc (P), S (nodes); unused
 * pointers may be NULL. on_device: 0 host arrays, 1 device arrays (both synchronous, like the
 * reference's launch), 2 device arrays, stream-ordered on the context's stream: the call
 * returns after launching (launch errors are reported; nothing is read back). */
int fpde_sum(fpde_ctx *ctx, int sum_alg, int bs, int64_t OS, int64_t nodes, double *S, const double *old,
             int old_size, const double *tau, double *Htmp, const double *row2_precalc,
             const double *kb_3_cache, double sum_param, double gtj, double gt, double alpha, int tstep,
             int on_device);

/* The history sum of fpde_l1_sum from caller-owned device buffers, allocating nothing.
 * No counterpart in the reference. For callers that cannot call cudaMalloc while they run
 * (a host framework that owns all device memory, a fixed device-memory budget, a step loop
 * that must avoid the device synchronisation of cudaMalloc/cudaFree):
 *   S[i] = sum_{t<n} w[t] * D[t*P + i],  i < nodes
 * with D (n rows, row pitch P even, 16-byte aligned), w (n) and S (nodes) in device memory
 * of the current device, launched on `stream` (a cudaStream_t, NULL = default stream); the
 * call does not synchronise. Its split-K partials live in a fixed 8 MiB array inside the
 * library (2^20 doubles), so P may be at most 1,048,576; larger pitches return
 * FPDE_ERR_CAPACITY. The first call on each device looks up that array's device address;
 * make that first call before any stream capture. All calls share the array: calls whose
 * work overlaps on the GPU race and must be serialised by the caller. */
int fpde_l1_sum_noalloc(const double *D, int n, int64_t P, int64_t nodes, const double *w,
                        double *S, void *stream);

/* Far-history contraction of the split-precision path, on the tensor cores:
 *   C[s][j][i] = out_scale * sum_{t in split s} (Ah[i][t] Wh[j][t] + Ah[i][t] Wl[j][t] + Al[i][t] Wh[j][t])
 * for j < 64, with FP32 accumulation folded into float-float every 256 columns and FP64
 * partial sums per K split s (C is splits x 64 x rows doubles, device). Ah/Al are
 * [rows][lda] and Wh/Wl [64][ldw] 16-bit arrays in device memory (fp16, or bf16 when
 * bf16 != 0); rows % 128 == 0, lda and ldw % 64 == 0, k_cols % 64 == 0 and <= both pitches.
 * splits <= 0 picks a split count (at most 4). This replaces the reference's mode-1
 * far-history tile product (DOC kernel, fr_do.cpp:173-235, wmma 16x16x16 half/float). */
int fpde_far_contract(fpde_ctx *ctx, const void *a_hi, const void *a_lo, int64_t rows, int64_t lda,
                      const void *w_hi, const void *w_lo, int64_t ldw, int k_cols, int bf16,
                      double out_scale, double *C, int splits);

/* Exact-slice form of the far contraction: operands as three bf16 slices each
 * (A[i][t] = (a0 + a1 + a2)[i][t] * 2^pA[i][t/64], W[j][t] = (w0 + w1 + w2)[j][t] * 2^pW[j][t/64],
 * a0/w0 integers |.| <= 256, a1/w1 multiples of 2^-8 and a2/w2 of 2^-16 with at most 8
 * significant bits), int8 exponents pA [rows][ldp] and pW [64][ldp];
 *   C[s][j][i] = sum_{t in split s} A[i][t] W[j][t]   (partials, FP64, device)
 * with the leading products a0*w0 summed exactly per 64 columns and everything folded in
 * float-float. Same shape rules as fpde_far_contract. Replaces the same reference code. */
int fpde_far_contract3(fpde_ctx *ctx, const void *const a[3], int64_t rows, int64_t lda,
                       const void *const w[3], int64_t ldw, int k_cols, const int8_t *pA,
                       const int8_t *pW, int64_t ldp, double *C, int splits);

/* ----------------------------------------------------- tridiagonal solves */

/* Batched Thomas solves of n_lines independent lines (al1 / bt1 / back-substitution,
 * fpde_hpc_1d.cpp:4002-4027, :4585-4590, :4678-4725), FP64. Line l, node i (0..N) lives at
 * element offset l*stride_line + i*stride_elem of every array (a, b, r, om, u). a, b, r, om
 * are read at i = 1..N-1. Boundary kinds/values per line end; left/right values are arrays
 * of n_lines (NULL = 0). dLN is the last step (flux closure only). u is read (old U[N-1] for
 * the degenerate flux case) and written at nodes 0..N. */
int fpde_tridiag_solve(fpde_ctx *ctx, const double *a, const double *b, const double *r,
                       const double *om, double *u, int64_t n_lines, int64_t N,
                       int64_t stride_elem, int64_t stride_line,
                       int left_kind, const double *left_val, int right_kind,
                       const double *right_val, double dLN, int on_device);

/* ------------------------------------------------------- 1D line problem */

/* The reference's Richards problem (fpde_hpc_1d.cpp with analytic_test 0: water transport with
 * the van Genuchten-Mualem water content of cv_form 4, wetness / inv_dw_dh :2493-2566, and the
 * conductivity KK = Kr(wetness) k_sat :2625-2655; no irrigation, bottom_cond 0). Its line
 * coefficients A_/B/R (:3095-3142) depend on the solution and are formed on the device from the
 * grid before every line solve, with the reference's mode-3 suction P = -(U - i sZ[p]) (i the
 * node's index along the sN axis, p its position along the pass; :2504-2512, :2546-2554). The sN
 * pass starts with the reference's first-order surface condition (al1 :4004-4012, bc0
 * :4493-4500: flux -Uc with Uc = dL[0] E / KK(1), or Dirichlet -Uc KK(1)/dL[0] where node 0 is
 * saturated); every other line end has zero flux (al1's Al[1] = 1, U1's flux closure).
 * A 1D line (fpde_line_desc.richards) has the same surface condition at node 0 and its own
 * right end (right_kind / right_value / dLN: the reference's bottom_cond 1 is Dirichlet H0 - Z[N]). */
typedef struct fpde_richards {
    int k_form;                 /* 1: van Genuchten-Mualem Kr, 2: Averianov Kr = S^3.5 */
    double k_sat;               /* saturated filtration coefficient (the reference's k) */
    const double *sZ;           /* host: 3D LOD, sN+2 node coordinates along the sN axis; line, the N+1
                                   node coordinates Z (suction P = -(U - Z), the reference's mode-1
                                   wetness / inv_dw_dh :2499-2500, :2529) */
    const double *dL[3];        /* host: 3D LOD, per pass (0 sN, 1 _M, 2 K) the steps dL[p],
                                   intervals+2 values; line, dL[0] only (N+1 steps) */
    const double *evaporation;  /* host, evaporation rate E of every step (Ev * day_night_coef);
                                   step n uses row min(n, evaporation_rows-1) */
    int evaporation_rows;
    /* Salt concentration C (3D LOD only, FPDE_PREC_FP64; the reference's is_c: equation 1): with
     * salt_c0 (the initial grid) every line of every pass also solves C after H, as calc_step does
     * (:5270-5278): C's coefficients D/sigma over the steps (A_/B/R :3099-3136), the H-driven
     * transport div(K C grad H)/sigma with the new H and chemical osmosis (nu/sigma) in C's
     * right-hand side, chemical osmosis nu in H's (Om1 :4175-4229), C's own L1 history; C is
     * Dirichlet Cu() = 0 at the surface (no irrigation), zero-flux elsewhere. The reference's
     * temperature equation (is_t) is not available: its 3D set-up stops on a null row (:3640). */
    const double *salt_c0;
    double salt_nu, salt_sigma, salt_D;   /* nu, sigma, D of the reference (:3515-3518) */
} fpde_richards;


/* Launch parameters of a line chosen by fpde_line_autotune (or by hand); 0 = the built-in rule.
 * No counterpart in the reference, whose OpenCL path fixes one work-group shape
 * (opencl_cuda_base.cpp:626-649). */
typedef struct fpde_line_tuning {
    int solve_sp;       /* nodes per solve thread: 1, 2, 4 or 8 */
    int chunks;         /* CTAs the line is split into for the solve (at most the SM count) */
    int far_splits;     /* K splits of the tensor-core far contraction: 1..4 (split paths; the
                           three-slice path keeps one slot for its super-block partial: 1..3) */
    int gemv_splits;    /* row splits of the FP64 history sum: 1..64 (FP64 path) */
    int far_super;      /* three-slice path: 64-step blocks per far super-block, 1..4 (the history
                           older than a super-block is contracted once for all its steps) */
    double ms_per_step; /* output of fpde_line_autotune: measured time per step of the choice */
} fpde_line_tuning;

/* A time-fractional diffusion line  D_t^alpha U = d/dx(k dU/dx) (+ source)  discretised as in
 * fpde_hpc_1d.cpp (L1 Caputo in time, implicit 3-point FD in space, Thomas per step):
 *   Om[i] = -Da*(kkk0/tau) U[i] + src[i] + Da*S[i],  R[i] = Rlap[i] + Da*kkk0/tau.
 * The time step tau is uniform; weights are the closed form. */
typedef struct fpde_line_desc {
    int64_t N;            /* intervals; nodes 0..N */
    double alpha;         /* time order, 0 < alpha < 1 */
    double tau;           /* time step */
    double Da;            /* 1/Gamma(1-alpha) (caller's value; fpde_gamma gives one) */
    int left_kind;        /* fpde_bc_kind */
    double left_value;
    int right_kind;
    double right_value;
    double dLN;           /* last space step (flux closure) */
    int precision;        /* fpde_precision */
    int block;            /* split paths: steps per far-history block (0 = auto) */
    int max_steps;        /* history capacity */
    /* Optional; all-zero keeps the Caputo L1 scheme above. */
    const double *lag_weights; /* host, max_steps+1 values: w[0] replaces Da*kkk0/tau (in Om and
                                  R), w[l] the history weight of lag l (Da*kkk0*b_l/tau): the
                                  distributed-order equation uses c[l]/tau of fpde_do_weights */
    double theta;         /* explicit fraction of the space operator on the old state,
                             Om[i] -= theta*(A[i] U[i-1] - Rlap[i] U[i] + B[i] U[i+1])
                             (fr_do eq_Ff :656-665: theta 1 with A = B = D/(2h^2)) */
    const double *source; /* host, source_rows x (N+1): step n adds row min(n, source_rows-1)
                             to Om (fr_do's -(f(t_n,x)+f(t_{n+1},x))/2; Rp of Om1) */
    int source_rows;
    const fpde_line_tuning *tuning; /* optional launch parameters (NULL: built-in rules) */
    double restrict_eps;  /* restricted summing, the reference's sum_alg 1 with sum_param =
                             restrict_eps (time_summing :4117-4131): newest first, the history
                             stops before the first lag l whose kb = w[l]*tau/Da is below it;
                             0 keeps every lag. FPDE_PREC_FP64 and FPDE_PREC_SPLIT_BF16X3: the
                             GEMV reads only the window's rows, the far contraction only the
                             64-step blocks the window reaches. */
    const fpde_richards *richards; /* optional: the Richards problem - A, B, Rlap formed from the state
                             every step (those arguments of fpde_line_create may be NULL);
                             FPDE_PREC_FP64 or FPDE_PREC_SPLIT_BF16X3, Caputo weights, theta 0 */
} fpde_line_desc;

/* Set up a line: A, B, Rlap (N+1 host values, entries 1..N-1 used; see fpde_line_coefs)
 * and the initial state u0 (N+1 host values). Replaces constructing H_solver + init_opencl
 * for one column (fpde_hpc_1d.cpp:3457-3606, :1715). */
int fpde_line_create(fpde_ctx *ctx, const fpde_line_desc *desc, const double *A, const double *B,
                     const double *Rlap, const double *u0, fpde_line **out);
int fpde_line_destroy(fpde_line *line);
/* Reset to the state u0 (N+1 values, host or device) and an empty history. */
int fpde_line_reset(fpde_line *line, const double *u0, int on_device);
/* Advance `steps` time steps (calc_step / U1 per step, fpde_hpc_1d.cpp:5100-5135, with the
 * history applied every step). Runs of at least 128 steps replay one CUDA graph (see
 * fpde_line_graph_stats); shorter runs are enqueued directly on the context's stream. */
int fpde_line_run(fpde_line *line, int steps);
/* Copy the state (N+1 values) out. */
int fpde_line_get_state(fpde_line *line, double *u, int on_device);
/* Device pointer of the state (N+1 doubles, valid until the line is destroyed). */
int fpde_line_state_ptr(fpde_line *line, double **u_dev);
/* End-to-end call: upload u0 from host, run `steps`, download the final state to host. */
int fpde_line_solve_host(fpde_line *line, const double *u0_host, int steps, double *u_out_host);
/* CUDA graphs of the line (no counterpart in the reference, which launches every kernel itself):
 * runs of at least 128 steps are captured once per (first step, steps) and replayed; at most 8
 * instantiated graphs are kept (least recently used evicted). Shorter runs are enqueued directly,
 * so a per-step or per-block caller instantiates none. *cached = graphs held now, *instantiated =
 * graphs instantiated since the line was created. */
int fpde_line_graph_stats(const fpde_line *line, int *cached, int64_t *instantiated);
/* Current step count. */
int fpde_line_steps_done(const fpde_line *line, int64_t *n);
/* One block of the blocked schedule: advance to the next multiple of FPDE_BLOCK_STEPS (64) steps
 * (or to max_steps), i.e. append -> far history of the block -> near history -> RHS -> solve for
 * every step of the block, as one captured graph; *steps_run receives the count (0 when the
 * history is full). Replaces the per-step `calc_step` -> `fr_ocl_call_sum` -> `time_summing`
 * sequence (fpde_hpc_1d.cpp:5156-5157, :1835-1880, :4100-4104) for a whole block at once. */
#define FPDE_BLOCK_STEPS 64
int fpde_step_block(fpde_line *line, int *steps_run);
/* Kernel timing probes (no counterpart in the reference, which times whole calls with
 * clock_gettime, opencl_cuda_base.cpp:708-716): with every > 0, later runs record CUDA
 * events inside the captured graph around the history-sum and solve kernels of every
 * `every`-th step and around every far-history contraction. fpde_line_probe_stats returns,
 * for the last run and one kind of kernel (0 FP64 history GEMV, 1 tensor-core far
 * contraction, 2 line solve), the summed event time (ms), the summed algorithmic bytes
 * (GEMV: 8 * rows * (N+1); contraction: 2 bytes per slice * rows * (N+1) of 16-bit history;
 * solve: 8 * (N+1) * (far splits + near rows + 2)), the summed algorithmic flops and the
 * number of time steps the probed launches cover (for the contraction: its launches). On
 * the split paths every block's solve launch is probed; on the FP64 path every `every`-th. */
int fpde_line_set_probe(fpde_line *line, int every);
int fpde_line_probe_stats(fpde_line *line, int kind, double *ms, double *bytes, double *flops,
                          int *count);

/* Autotuner (no counterpart in the reference): for the line that desc and the arrays describe,
 * time candidate launch parameters on short runs and on the far contraction / FP64 history
 * sum at a history of min(max_steps, 2048) steps, and return the fastest in *out (pass it as
 * desc->tuning to fpde_line_create). Candidates: solve_sp x chunks (solve time per step of the
 * second 64-step block), far_splits 1..4, gemv_splits {k/2, k, 2k} around the built-in rule k,
 * and on the three-slice path far_super 1, 2, 4 (a whole run of min(max_steps, 4096) steps each).
 * Allocates and frees temporary device buffers; takes a fraction of a second to seconds. */
int fpde_line_autotune(fpde_ctx *ctx, const fpde_line_desc *desc, const double *A, const double *B,
                       const double *Rlap, const double *u0, fpde_line_tuning *out);

/* Line coefficients of the H equation with gamma = 1 (A_ / B / R, fpde_hpc_1d.cpp:3095-3142):
 * A[i] = k[i-1] iw[i]/(dL[i] dL[i-1]), B[i] = k[i] iw[i]/dL[i]^2,
 * Rlap[i] = iw[i] (k[i]/dL[i]^2 + k[i-1]/(dL[i] dL[i-1])), i = 1..N-1. Host. iw may be NULL (1). */
int fpde_line_coefs(int64_t N, const double *k, const double *iw, const double *dL,
                    double *A, double *B, double *Rlap);

/* ------------------------------------------------------------------ 3D LOD */


/* The 3D locally-one-dimensional step of the reference (calc_step, mode 3 with implicit3d 0
 * and split3d 0, fpde_hpc_1d.cpp:5144-5779): per time step the history sum, then Thomas
 * passes along k (K, with the history and the source Rp, Om1 :4165-4268 for m3d_c == 2),
 * along j (_M) and along i (sN), each with R = Rlap + Da*kkk0/tau and Om = -Da*(kkk0/tau) U
 * (+ Rp + Da S in the K pass), and a ghost copy at the far end of every line (U1 :4792).
 * The grid has (sN+2)(M+2)(K+2) points with idx = i + j (sN+2) + k (sN+2)(M+2) (:1181). */
/* ---------------------------------------------------------------------------------------------
 * Implicit space-fractional operator (the reference's impl 2 with toeplitz_mult_alg 0).
 *
 * With a space-fractional order gamma < 1, U1 (fpde_hpc_1d.cpp:4769-4791) solves every line's
 * system tridiag(Mat) + iw * T * tridiag(Mcoefs) with solve_mln<1> (:812-1157) and the product
 * vmul_T (:6618-6747): T is the Toeplitz matrix of the space-fractional integral, strictly lower
 * (space_der 0: row i sums j = 1..i-1 with Tm[i-j+1]) or two-sided (space_der 1: minus the sum over
 * j = i+1..n-1 with Tm[j-i+1]) over the interior rows 1..n-1 of a line of n intervals; iw is
 * inv_dw_dh (equation 0). The library forms every value with the reference's operations in its
 * order and without contracted multiply-adds, so products, iterates and solutions equal the
 * reference's (an x86-64 build) bit for bit on the same inputs.
 * ------------------------------------------------------------------------------------------- */
#define FPDE_SF_MAX_N 1400          /* longest line (intervals): one CTA holds a line in shared memory */
#define FPDE_SF_MAX_ITER 1000000

/* vmul_T on a batch of lines of n intervals: mat and mc are three planes (0 lower, 1 diagonal,
 * 2 upper) of lines x (n+1) values (plane d at mat + d*lines*(n+1)); rows 0 and n of mat are the
 * boundary rows, mc is read at rows 1..n-1; iw and rs (implicit_row_scaling: RS) are lines x (n+1)
 * or NULL (1.0 / no scaling); Tm has n+1 entries of which 2..n-1 are read; x, r are lines x (n+1). */
int fpde_sf_matvec(fpde_ctx *ctx, int lines, int n, const double *mat, const double *mc, const double *Tm,
                   const double *iw, const double *rs, int space_der, const double *x, double *r, int on_device);
/* solve_mln<1> on every line (rb = 0, re = n+1): x holds the initial guesses and receives the
 * solutions; a line stops when |r.r / (n+1)| < thr (the reference's impl_err) or after maxiter - 1
 * iterations (impl_niter); iters (lines ints, may be NULL) receives each line's count. A line whose
 * solve breaks down maxiter times in a row, or runs for more than 10 s, stops: FPDE_ERR_NUMERIC. */
int fpde_sf_solve(fpde_ctx *ctx, int lines, int n, const double *mat, const double *mc, const double *Tm,
                  const double *iw, const double *rs, int space_der, const double *B, double *x, double thr,
                  int maxiter, int *iters, int on_device);
/* The Toeplitz row of a uniform axis Z (n+2 coordinates): Tm[i] = |(Z1-Zi)^(1-gamma) -
 * (Z1-Z(i+1))^(1-gamma)| / Gamma(2-gamma), i = 1..n, Tm[0] = 0 (the reference's fill :3670-3694,
 * with C tgamma for its Gamma). Host function. */
int fpde_sf_toeplitz_row(double gamma, const double *Z, int n, double *Tm);

/* The fully implicit 3D operator (the reference's implicit3d 1): vmul_T_3d (fpde_hpc_1d.cpp:
 * 6801-8722, toeplitz_mult_alg 0, equation 0) on the V = (sN+2)(M+2)(K+2) + 1 values of a grid
 * (i fastest, idx :1649) and the one past it, the vector solve_mln<1> runs over in calc_step
 * (:5705). The product is the 7-diagonal Mat_3d (flat-index neighbours: planes 0/2 at -/+ (sN+2)(M+2),
 * 3/4 at -/+ (sN+2), 5/6 at -/+ 1, the diagonal in 1, each pair applied when that axis has more
 * than 2 intervals) plus, for each axis c = K, _M, sN in that order and at the nodes inside
 * 1..len-1 on every axis, iw_c * T_c * tridiag(Mcoefs_3d[c]) along the node's axis-c line. Products
 * equal the reference's bit for bit. */
typedef struct fpde_sf3d_system {
    int sN, M, K;               /* intervals along i, j, k (each 1 .. FPDE_SF_MAX_N; V below 2^31) */
    int space_der;              /* 0 one-sided, 1 two-sided */
    const double *mat;          /* 7 x V: Mat_3d[0..6] */
    const double *mc;           /* 9 x V: Mcoefs_3d[c][d] at plane 3c+d (c = 0 sN, 1 _M, 2 K; d = 0
                                   lower, 1 diagonal, 2 upper); read at the interior nodes */
    const double *Tm[3];        /* Toeplitz row of axis c: len_c + 1 values, entries 2..len_c-1 read */
    const double *iw;           /* 3 x V: inv_dw_dh of the axis-c line through the node, or NULL (1.0) */
    const double *rs;           /* V row scales (implicit_row_scaling: RS), or NULL */
} fpde_sf3d_system;
#define FPDE_SF3D_MAX_EXACT (1 << 22)   /* largest V of a solve with exact (sequential) dot products */

/* r = A x over the V values (x, r: V each). */
int fpde_sf3d_matvec(fpde_ctx *ctx, const fpde_sf3d_system *sys, const double *x, double *r, int on_device);
/* solve_mln<1> of A x = B over the V values (rb = 0, re = V): x holds the initial guess and receives
 * the solution; stops when |r.r / V| < thr or after maxiter - 1 iterations; *iters (host, may be
 * NULL) receives the count. exact != 0: every dot product is the reference's sequential sum, so the
 * iterates, the count and the solution equal the reference's bit for bit (one GPU thread adds each
 * dot product: V <= FPDE_SF3D_MAX_EXACT); exact = 0: dot products are deterministic tree sums (the
 * same on every run on a device; they differ from the reference's only in the order of the adds) and
 * the products' Toeplitz terms are fused multiply-adds (one rounding per term). A
 * solve that breaks down maxiter times in a row or runs longer than 30 s stops: FPDE_ERR_NUMERIC. */
int fpde_sf3d_solve(fpde_ctx *ctx, const fpde_sf3d_system *sys, const double *B, double *x, double thr, int maxiter,
                    int exact, int *iters, int on_device);

/* The implicit space-fractional solves of a 3D LOD (fpde_lod3d_desc.space_frac): per pass p the
 * Toeplitz row Tm[p] (Nl+1 values), the Mcoefs grids mc[p] (three host grids: lower, diagonal,
 * upper, at every interior line node) and inv_dw_dh iw[p] (one grid), and the solver's threshold
 * and iteration cap. Line lengths at most FPDE_SF_MAX_N. exact = 1 runs every line solve as
 * fpde_sf_solve does (bit for bit the reference's); exact = 0 (faster) sums each dot product in a
 * fixed tree over the line's CTA and fuses every product into its sum (deterministic; it differs
 * from the reference's only in the order and rounding of those operations).
 * implicit3d = 1 replaces the three passes of line solves by the reference's fully implicit scheme
 * (calc_step :5160-5716 with implicit3d 1): each step adds every line's system of the K, _M and sN
 * passes into one 3D system (the time term and the history in the K pass only) and solves it with
 * fpde_sf3d_solve's solver over the G + 1 values (exact as in fpde_sf3d_solve). */
typedef struct fpde_space_frac {
    int space_der;              /* 0 one-sided, 1 two-sided */
    double tol;                 /* impl_err (default 1e-9 in the reference) */
    int max_iter;               /* impl_niter (5000) */
    const double *Tm[3];
    const double *mc[3];        /* each 3 x grid */
    const double *iw[3];        /* each one grid */
    int implicit3d;             /* 0: line solves per pass (LOD); 1: one 3D solve per step */
    int exact;                  /* 1: the reference's operation order (sequential dot products) */
} fpde_space_frac;

typedef struct fpde_lod3d_desc {
    int sN, M, K;           /* intervals along i, j, k */
    double alpha, tau, Da;  /* as for lines; tau uniform */
    int left_kind[3];       /* per pass (0 = sN, 1 = _M, 2 = K): fpde_bc_kind at the line start */
    int right_kind[3];      /* and at the line end (flux: the U1 closure with dLN[pass]) */
    double dLN[3];
    int precision;          /* FPDE_PREC_FP64 */
    int max_steps;          /* history capacity */
    const double *lag_weights; /* optional, as in fpde_line_desc */
    const double *source;   /* optional host grids Rp of the K pass, source_rows x grid; step n uses
                               row min(n, source_rows-1) */
    int source_rows;
    const double *bc;       /* optional host grids of boundary data (Dirichlet values / fluxes at the
                               line ends), bc_rows x grid; NULL = 0 */
    int bc_rows;
    double restrict_eps;    /* restricted summing as in fpde_line_desc (the reference's sum_alg 1 in
                               the K pass, time_summing :4117-4131); 0 keeps every lag */
    int series_terms;       /* > 0: the reference's sum_alg 2 with sum_param = series_terms (at most
                               128) in the K pass (time_summing :4137-4151): P moments per grid point
                               carried from step to step instead of the stored history, S = sum_j
                               v_j H_j / tau (FPDE_PREC_FP64, Caputo weights, g(t) = t; the history
                               then keeps only the newest increment) */
    const fpde_richards *richards; /* optional: the Richards problem (coefficients from the solution
                               every step; coefA/B/Rlap, the boundary kinds and bc are then unused
                               and may be NULL; needs M, K <= sN + 1) */
    const double *time_steps;   /* optional: variable steps (the reference's varT), tau_n of every step
                                   (max_steps values; Time accumulated as Time[n+1] = Time[n] + tau_n).
                                   The L1 weights are then a row per step (no Toeplitz structure): the
                                   history is summed by the FP64 GEMV with row n, and the line
                                   coefficients' local term Da kkk0_n / tau_n changes every step, so
                                   the passes form the alpha recurrence on the fly (FPDE_PREC_FP64;
                                   not with lag_weights, series, restricted summing, richards,
                                   space_frac) */
    const double *weight_rows;  /* optional with time_steps: the weights of every step as the caller's
                                   time_summing uses them: row n (max_steps+1 values) holds
                                   kb_3_cache[0..n-1] and kkk0 at column n (precalc_kb_3 :4069-4085,
                                   init_time_step :3942-3949); NULL: computed by fpde_weights_g */
    double kernel_power;        /* with time_steps and no weight_rows: g(t) = t^p of the generalized
                                   Caputo kernel (func_in_kernel 1-3; 0 means p = 1) */
    const fpde_space_frac *space_frac; /* optional: implicit space-fractional line solves (impl 2);
                               coefA/B/Rlap are then the reference's A_/B/R with its space-fractional
                               local weights, every pass has a Dirichlet start, right_kind per pass */
    int segments[3];            /* per pass: threads (segments) per line of the Thomas passes, 4, 8, 16
                                   or 32 with at most 32 interior nodes each; 0 = the built-in rule
                                   (fpde_lod3d_autotune times the choices) */
} fpde_lod3d_desc;

/* coefA/B/Rlap: three host grids each (pass 0 = sN, 1 = _M, 2 = K) of the line coefficients at
 * every node (A_/B/R of the pass's axis, :3095-3142); u0: the initial grid. Replaces the
 * H_solver set-up of a 3D run plus init_opencl (:1715-1883). */
int fpde_lod3d_create(fpde_ctx *ctx, const fpde_lod3d_desc *desc, const double *coefA, const double *coefB,
                      const double *coefRlap, const double *u0, fpde_lod3d **out);
int fpde_lod3d_destroy(fpde_lod3d *lod);
/* Advance `steps` steps (runs of at least 128 steps replay a cached CUDA graph per (start, steps),
 * at most 8 kept; shorter runs are enqueued directly). */
int fpde_lod3d_run(fpde_lod3d *lod, int steps);
int fpde_lod3d_get_state(fpde_lod3d *lod, double *u, int on_device);
/* New initial grid and an empty history. */
int fpde_lod3d_reset(fpde_lod3d *lod, const double *u0, int on_device);
/* End-to-end call: upload u0 from host, run `steps`, download the grid to host. */
int fpde_lod3d_solve_host(fpde_lod3d *lod, const double *u0_host, int steps, double *u_out_host);
int fpde_lod3d_steps_done(const fpde_lod3d *lod, int64_t *n);
/* With richards.salt_c0: the salt concentration grid out. */
int fpde_lod3d_get_concentration(fpde_lod3d *lod, double *c, int on_device);
/* With space_frac: the solver iterations of every line solve since creation (0 otherwise). */
int fpde_lod3d_sf_iterations(fpde_lod3d *lod, int64_t *iters);
/* Times `steps` steps of the LOD desc describes (arguments as fpde_lod3d_create) with each
 * segment count of the Thomas passes (the same count in every pass whose lines it fits: 4, 8, 16,
 * 32, and the built-in rule) and returns the fastest in segments[3] (0 where the built-in rule won
 * or a pass has no segmented form) with its milliseconds per step in *ms_per_step. */
int fpde_lod3d_autotune(fpde_ctx *ctx, const fpde_lod3d_desc *desc, const double *coefA, const double *coefB,
                        const double *coefRlap, const double *u0, int steps, int segments[3], double *ms_per_step);

/* --------------------------------------------------------------- ensembles */

/* One column of an ensemble: an independent 1D Caputo line (the reference runs one column
 * per process, mode 3 with BS 1, or the 1D mode; fpde_hpc_1d.cpp:3457-3606). Arrays are
 * host pointers read at fpde_batch_create. */
typedef struct fpde_column_desc {
    int64_t N;               /* intervals; nodes 0..N */
    double alpha, tau, Da;
    int left_kind;
    double left_value;
    int right_kind;
    double right_value;
    double dLN;
    const double *A, *B, *Rlap, *u0;   /* N+1 values each (as for fpde_line_create) */
    const double *lag_weights;         /* optional, max_steps+1 values (fpde_line_desc) */
    double restrict_eps;               /* restricted summing of this column (the reference's sum_alg 1,
                                          time_summing :4117-4131, as fpde_line_desc.restrict_eps);
                                          0 keeps every lag */
} fpde_column_desc;

/* An ensemble of columns of any lengths and orders advanced together: per step one history
 * sum over all columns' nodes and one solve kernel with a CTA per column, largest columns
 * first. No counterpart in the reference, which runs such ensembles as separate processes
 * (fpde_hpc_1d.cpp main); stands in for a loop of H_solver runs. Node layout on the device:
 * column c at offset off_c (fpde_batch_layout) of a padded vector of `total` values. */
int fpde_batch_create(fpde_ctx *ctx, const fpde_column_desc *cols, int n_cols, int max_steps, int precision,
                      fpde_batch **out);
int fpde_batch_destroy(fpde_batch *batch);
int fpde_batch_run(fpde_batch *batch, int steps);
/* Column `col`'s state (N+1 values) out. */
int fpde_batch_get_state(fpde_batch *batch, int col, double *u, int on_device);
/* Offset and N of column `col` in the padded node vector, and the vector's length. */
int fpde_batch_layout(const fpde_batch *batch, int col, int64_t *offset, int64_t *N, int64_t *total);
/* Reset to a padded state vector (NULL: the columns' u0) and an empty history. */
int fpde_batch_reset(fpde_batch *batch, const double *u_padded, int on_device);
/* End-to-end call: padded initial vector from host, run `steps`, padded final vector to host. */
int fpde_batch_solve_host(fpde_batch *batch, const double *u0_padded_host, int steps, double *u_out_padded_host);

#ifdef __cplusplus
}
#endif
#endif
