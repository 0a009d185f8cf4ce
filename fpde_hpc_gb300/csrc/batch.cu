// Ensemble of independent 1D Caputo columns (fpde_batch_*): many lines of different length,
// order and coefficients advanced together, two kernels per time step for the whole ensemble.
//
// Layout in HBM: the columns' nodes are concatenated, column c occupying
// [off_c, off_c + P_c) with P_c = N_c + 1 rounded up to 512, so that every CTA of the
// history sum (256 threads x 2 nodes) lies inside one column. The increments are one
// time-major table D[t][sum_c P_c]; padding nodes stay zero.
//
// Per time step n:
//   1. k_batch_partial : part[ks][q] = sum_t w_c[n-t] D_t[q], the column's lag weights picked
//                        per CTA (one flat grid over all nodes: balanced by construction)
//   2. k_batch_solve   : one persistent launch fed by a device work queue: each CTA takes the
//                        next column (largest first) from an atomic counter of the step and runs
//                        Thomas on it (fpde_hpc_1d.cpp al1/bt1/U1 :4002-4027, :4585-4590,
//                        :4683-4724) as segment sweeps joined by a CTA scan, then writes U and D_n.
// Split path (FPDE_PREC_SPLIT_BF16X3): step 1 becomes, per 64-step block, the exact
// three-slice tensor-core contraction of all history before the block with one weight tile
// per column (tc_far.cu; each 128-row tile picks its column's tile), and per step the near
// history in float-float from a 64-row float-pair ring (k_near_history_ff); the solve writes
// each increment to that ring and to the FP64 one the conversion reads.
// The alpha recurrence is time-invariant and precomputed on the host per column.
#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <string>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "graph_cache.cuh"
#include "scan.cuh"
#include "tc_far.cuh"
#include "ff.cuh"

namespace fpde {

#ifndef FPDE_BATCH_THREADS
#define FPDE_BATCH_THREADS 512
#endif
constexpr int BT = FPDE_BATCH_THREADS;   // threads per column CTA (halves the sequential segment of the longest
                                         // columns, which set the step time of a skewed ensemble)
constexpr int BW = BT / 32;

struct ColInfo {
    int64_t off;              // first node of the column in the concatenated node space
    int N;                    // intervals (nodes 0..N)
    int seg;                  // nodes per thread segment (nodes 0..N-1 are swept)
    double lam, g0, gN, dLN, AlN;
    int rkind;
    int pad;
};

// col_lag (may be null): the lags each column keeps under restricted summing; rows older than
// n - col_lag[c] carry zero weights and are skipped (adding a zero-weight term changes nothing).
__global__ void __launch_bounds__(256) k_batch_partial(const double2 *__restrict__ D, int64_t P2, int n,
                                                       const double *__restrict__ wall, int64_t wstride,
                                                       int64_t woff, const int *__restrict__ cta_col,
                                                       const int *__restrict__ col_lag, double2 *__restrict__ part)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int ks = blockIdx.y, KS = gridDim.y;
    const int t0 = (int)((int64_t)n * ks / KS), t1 = (int)((int64_t)n * (ks + 1) / KS);
    if (i >= P2) return;
    const int c = cta_col[blockIdx.x];
    const double *wt = wall + (int64_t)c * wstride + woff;                       // wt[t] = w_c[n - t]
    double ax = 0.0, ay = 0.0;
    int t = col_lag ? max(t0, n - col_lag[c]) : t0;
    for (; t + 8 <= t1; t += 8) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcs(D + (int64_t)(t + u) * P2 + i);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const double w = __ldg(wt + t + u);
            ax = fma(w, v[u].x, ax);
            ay = fma(w, v[u].y, ay);
        }
    }
    for (; t < t1; ++t) {
        const double2 v = __ldcs(D + (int64_t)t * P2 + i);
        const double w = __ldg(wt + t);
        ax = fma(w, v.x, ax);
        ay = fma(w, v.y, ay);
    }
    part[(int64_t)ks * P2 + i] = make_double2(ax, ay);
}

// Exclusive CTA scan of (P, X) pairs in thread order (up) or reverse order (down).
template <bool UP>
__device__ __forceinline__ void cta_scan_excl(double &P, double &X, double *wP, double *wX, int lane, int warp)
{
    if (UP) warp_scan_up(P, X, lane);
    else warp_scan_down(P, X, lane);
    double Pe = UP ? __shfl_up_sync(FULL, P, 1) : __shfl_down_sync(FULL, P, 1);
    double Xe = UP ? __shfl_up_sync(FULL, X, 1) : __shfl_down_sync(FULL, X, 1);
    if (lane == (UP ? 0 : 31)) { Pe = 1.0; Xe = 0.0; }
    if (lane == (UP ? 31 : 0)) { wP[warp] = P; wX[warp] = X; }
    __syncthreads();
    if (warp == 0) {
        double Pw = lane < BW ? wP[lane] : 1.0, Xw = lane < BW ? wX[lane] : 0.0;
        if (UP) warp_scan_up(Pw, Xw, lane);
        else warp_scan_down(Pw, Xw, lane);
        double Pwe = UP ? __shfl_up_sync(FULL, Pw, 1) : __shfl_down_sync(FULL, Pw, 1);
        double Xwe = UP ? __shfl_up_sync(FULL, Xw, 1) : __shfl_down_sync(FULL, Xw, 1);
        if (UP ? lane == 0 : lane >= BW - 1) { Pwe = 1.0; Xwe = 0.0; }
        __syncwarp();
        if (lane < BW) { wP[lane] = Pwe; wX[lane] = Xwe; }
    }
    __syncthreads();
    // compose: the warps before this one (wP, wX of this warp), then this warp's earlier lanes
    X = fma(Pe, wX[warp], Xe);
    P = Pe * wP[warp];
    __syncthreads();                                                // wP/wX reused by the caller
}

__global__ void __launch_bounds__(BT) k_batch_solve(const ColInfo *__restrict__ cols, const int *__restrict__ order,
                                                    int n_cols, unsigned *__restrict__ queue,
                                                    const double *__restrict__ A, const double *__restrict__ g,
                                                    const double *__restrict__ al, const double *__restrict__ segP,
                                                    const double *__restrict__ segQ, const double *__restrict__ KF,
                                                    const double *__restrict__ CB, const double *__restrict__ part,
                                                    int KS, int64_t pstride, double *__restrict__ U,
                                                    double *__restrict__ Y, double *__restrict__ Drow,
                                                    float2 *__restrict__ Drowf)
{
    __shared__ double wP[BW], wX[BW];
    __shared__ double s_y, s_uN;
    __shared__ int s_item;
    while (true) {
    if (threadIdx.x == 0) s_item = (int)atomicAdd(queue, 1u);
    __syncthreads();
    const int item = s_item;
    if (item >= n_cols) return;
    const int col = order[item];
    const ColInfo c = cols[col];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t o = c.off;
    const int i0 = min(tid * c.seg, c.N), i1 = min(i0 + c.seg, c.N);
    // Segment sweeps from zero carries joined by CTA scans; the carries are applied in one
    // independent pass, u = ub0 + c_in KF + c_out CB (KF: the segment's backward response to its
    // forward prefix products, CB: suffix products of al; time-invariant, from the host), so two
    // dependent FP64 chains per step instead of four. Loads are issued eight nodes at a time.
    // forward: y0 from a zero carry (y_0 = g0 at the column's first node) into Y
    double yl = 0.0;
    for (int ib = i0; ib < i1; ib += 8) {
        double uu[8], gg[8], aa[8], ss[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ib + t;
            const bool in = i < i1 && i > 0;
            const int64_t q = o + (in ? i : 0);
            uu[t] = in ? U[q] : 0.0;
            gg[t] = in ? __ldg(g + q) : 0.0;
            aa[t] = in ? __ldg(A + q) : 0.0;
            double sv = 0.0;
            for (int k = 0; k < KS; ++k)
                if (in) sv += __ldcg(part + (int64_t)k * pstride + q);
            ss[t] = sv;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ib + t;
            if (i < i1) {
                if (i == 0) {
                    yl = c.g0;                                          // Bt[1]
                } else {
                    const double om = -(c.lam * uu[t]) + ss[t];
                    yl = gg[t] * (aa[t] * yl - om);
                }
                Y[o + i] = yl;
            }
        }
    }
    const double pf = i1 > i0 ? __ldg(segP + (int64_t)col * BT + tid) : 1.0;
    double P = pf;
    double X = i1 > i0 ? yl : 0.0;
    cta_scan_excl<true>(P, X, wP, wX, lane, warp);
    const double cin = X;                                               // true y before the segment
    if (i1 == c.N && i1 > i0) s_y = fma(pf, cin, yl);                   // Bt[N]
    __syncthreads();
    if (tid == 0) {
        double uN;
        const double uNm1 = U[o + c.N - 1];
        if (c.rkind == FPDE_BC_DIRICHLET) uN = c.gN;
        else if (fabs(s_y) > 1e-15) uN = (fabs(1.0 - c.AlN) > 1e-15) ? (s_y + c.gN * c.dLN) / (1.0 - c.AlN) : uNm1;
        else uN = (fabs(1.0 - c.AlN) > 1e-15) ? 0.0 : uNm1;
        s_uN = uN;
    }
    __syncthreads();
    const double uN = s_uN;
    // backward: ub0 from a zero carry over y0, into Y
    double ul = 0.0;
    for (int ie = i1 - 1; ie >= i0; ie -= 8) {
        double yy[8], la[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ie - t;
            const bool in = i >= i0;
            const int64_t q = o + (in ? i : i0);
            yy[t] = in ? Y[q] : 0.0;
            la[t] = in ? __ldg(al + q) : 0.0;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ie - t;
            if (i >= i0) {
                ul = fma(la[t], ul, yy[t]);
                Y[o + i] = ul;
            }
        }
    }
    P = i1 > i0 ? __ldg(segQ + (int64_t)col * BT + tid) : 1.0;
    X = i1 > i0 ? fma(cin, __ldg(KF + o + i0), ul) : 0.0;              // u at the segment start, c_out = 0
    cta_scan_excl<false>(P, X, wP, wX, lane, warp);
    const double cout = fma(P, uN, X);                                  // true u after the segment
    // carries applied; U and the increment written
    for (int ib = i0; ib < i1; ib += 8) {
        double ub[8], kf[8], cb[8], uo[8];
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ib + t;
            const bool in = i < i1;
            const int64_t q = o + (in ? i : i0);
            ub[t] = in ? Y[q] : 0.0;
            kf[t] = in ? __ldg(KF + q) : 0.0;
            cb[t] = in ? __ldg(CB + q) : 0.0;
            uo[t] = in ? U[q] : 0.0;
        }
#pragma unroll
        for (int t = 0; t < 8; ++t) {
            const int i = ib + t;
            if (i < i1) {
                const int64_t q = o + i;
                const double u = fma(cout, cb[t], fma(cin, kf[t], ub[t]));
                U[q] = u;
                Drow[q] = u - uo[t];
                if (Drowf) Drowf[q] = d2ff(u - uo[t]);          // split path: the float-pair ring row
            }
        }
    }
    if (tid == 0) {
        const double uo = U[o + c.N];
        U[o + c.N] = uN;
        Drow[o + c.N] = uN - uo;
        if (Drowf) Drowf[o + c.N] = d2ff(uN - uo);
    }
    __syncthreads();                                                // s_item, s_y, s_uN reused
    }
}

}  // namespace fpde

using namespace fpde;

struct fpde_batch {
    fpde_ctx *ctx = nullptr;
    int n_cols = 0, max_steps = 0;
    int64_t Ptot = 0;
    std::vector<int64_t> off;
    std::vector<int> N;
    double *A = nullptr, *g = nullptr, *al = nullptr, *segP = nullptr, *segQ = nullptr;
    double *KF = nullptr, *CB = nullptr;      // per node: segment responses KF and suffix products CB
    double *U = nullptr, *U0 = nullptr, *Y = nullptr, *D = nullptr, *part = nullptr, *wall = nullptr;
    ColInfo *cols = nullptr;
    int *order = nullptr, *cta_col = nullptr;
    int *col_lag = nullptr;                   // restricted summing: lags kept per column (null: all)
    unsigned *queue = nullptr;                // per step: next work item of the solve
    int solve_grid = 0;
    // split path
    bool split = false;
    int64_t ld16 = 0, ldp = 0, LW = 0;
    uint16_t *h3[3] = {nullptr, nullptr, nullptr}, *w3[3] = {nullptr, nullptr, nullptr};
    int8_t *pA = nullptr;
    float *pW = nullptr;
    double *ring = nullptr, *cfar = nullptr, *wlag = nullptr, *Sn = nullptr;
    float2 *ringf = nullptr, *wff = nullptr;  // the ring and every column's lag weights as float pairs
    float2 *pre = nullptr;                    // near-history sums of the current 8-step sub-block
    int *wcol = nullptr;
    FarPlan3 plan3;
    int64_t n_done = 0;
    GraphCache<int> graphs;                        // captured runs (at least GRAPH_MIN_STEPS steps)
};

namespace fpde {

static int batch_enqueue(fpde_batch *b, cudaStream_t st, int64_t n0, int steps, int64_t *nk)
{
    int64_t k = 0;
    int rc;
    FPDE_CUDA(cudaMemsetAsync(b->queue + n0, 0, (size_t)steps * sizeof(unsigned), st));   // work queues of the run
    for (int64_t n = n0; n < n0 + steps; ++n) {
        int KS = 0;
        const double *part = b->part;
        double *Drow;
        float2 *Drowf = nullptr;                                     // split: the float-pair ring row
        if (!b->split) {
            if (n >= 1) {
                KS = choose_splits((int)n, b->Ptot);
                dim3 grid((unsigned)(b->Ptot / 512), (unsigned)KS);
                k_batch_partial<<<grid, 256, 0, st>>>((const double2 *)b->D, b->Ptot / 2, (int)n, b->wall,
                                                      b->max_steps + 1, b->max_steps - n, b->cta_col,
                                                      b->col_lag, (double2 *)b->part);
                FPDE_LAUNCHED(1);
                ++k;
            }
            Drow = b->D + n * b->Ptot;
        } else {
            const int64_t nb0 = n - n % 64;
            const int j = (int)(n - nb0);
            int splits = 0;
            if (nb0 > 0) {
                splits = far_splits((int)(nb0 / 64), b->Ptot);
                if (j == 0) {                                        // far history t < nb0, per column
                    SplitPrep3 sp;
                    sp.ring = b->ring; sp.P = b->Ptot; sp.nvalid = b->Ptot; sp.ld = b->ld16; sp.wlag = b->wlag;
                    for (int q = 0; q < 3; ++q) { sp.hist[q] = b->h3[q]; sp.w[q] = b->w3[q]; }
                    sp.pA = b->pA; sp.pW = b->pW; sp.ldp = b->ldp; sp.ncols = b->n_cols; sp.wstride = b->LW;
                    if ((rc = launch_block_prep3(st, sp, nb0))) return rc;
                    k += 2;
                    if ((rc = far3_launch(st, &b->plan3, (int)nb0, b->cfar, (int64_t)64 * b->Ptot, b->Ptot, splits,
                                          b->pA, b->pW, b->ldp, b->ctx->d_flags, b->wcol)))
                        return rc;
                    ++k;
                }
            }
            if (n >= 1) {
                // rows older than the step's 8-step sub-block (and the far partials) once per sub-block
                const int j0 = j - j % NEAR_SUB;
                const bool use_pre = splits > 0 || j0 > 0;
                if (use_pre && j == j0) {
                    if ((rc = launch_near_pre_ff(st, b->ringf, b->Ptot, j0, b->wff, b->cfar, splits, 1, b->pre,
                                                 b->cta_col, b->LW)))
                        return rc;
                    ++k;
                }
                if ((rc = launch_near_history_ff(st, b->ringf, b->Ptot, j, b->wff, b->cfar, splits, 1, b->Sn, b->cta_col,
                                                 b->LW, use_pre ? b->pre : nullptr, j0)))
                    return rc;
                ++k;
                KS = 1;
                part = b->Sn;
            }
            Drow = b->ring + (int64_t)j * b->Ptot;
            Drowf = b->ringf + (int64_t)j * b->Ptot;
        }
        k_batch_solve<<<b->solve_grid, BT, 0, st>>>(b->cols, b->order, b->n_cols, b->queue + n, b->A, b->g, b->al,
                                                    b->segP, b->segQ, b->KF, b->CB, part, KS, b->Ptot, b->U, b->Y, Drow,
                                                    Drowf);
        FPDE_LAUNCHED(1);
        ++k;
    }
    *nk = k;
    return FPDE_OK;
}

}  // namespace fpde

extern "C" {

int fpde_batch_destroy(fpde_batch *b)
{
    if (!b) return FPDE_OK;
    if (b->ctx) {
        cudaSetDevice(b->ctx->device);
        cudaStreamSynchronize(b->ctx->stream);
    }
    b->graphs.clear();
    for (double *p : {b->A, b->g, b->al, b->segP, b->segQ, b->KF, b->CB, b->U, b->U0, b->Y, b->D, b->part, b->wall, b->ring,
                      b->cfar, b->wlag, b->Sn})
        dev_free(p);
    for (int q = 0; q < 3; ++q) {
        dev_free(b->h3[q]);
        dev_free(b->w3[q]);
    }
    dev_free(b->pA);
    dev_free(b->pW);
    dev_free(b->ringf);
    dev_free(b->pre);
    dev_free(b->wff);
    dev_free(b->wcol);
    dev_free(b->queue);
    dev_free(b->cols);
    dev_free(b->order);
    dev_free(b->cta_col);
    dev_free(b->col_lag);
    delete b;
    return FPDE_OK;
}

int fpde_batch_create(fpde_ctx *ctx, const fpde_column_desc *cols, int n_cols, int max_steps, int precision,
                      fpde_batch **out)
{
    clear_error();
    FPDE_CHECK_ARG(out && cols && n_cols > 0, "bad arguments");
    *out = nullptr;
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    FPDE_CHECK_ARG(max_steps > 0, "max_steps must be positive");
    FPDE_CHECK_ARG(precision == FPDE_PREC_FP64 || precision == FPDE_PREC_SPLIT_BF16X3,
                   "ensemble: precision must be FP64 or the exact three-slice split");
    for (int c = 0; c < n_cols; ++c) {
        const fpde_column_desc &d = cols[c];
        FPDE_CHECK_ARG(d.N >= 2 && d.N <= (1 << 24), "column N out of range");
        FPDE_CHECK_ARG(d.A && d.B && d.Rlap && d.u0, "column arrays missing");
        FPDE_CHECK_ARG(d.lag_weights || (d.alpha > 0.0 && d.alpha < 1.0), "alpha must be in (0, 1)");
        FPDE_CHECK_ARG(d.tau > 0.0, "tau must be positive");
        FPDE_CHECK_ARG((d.left_kind == 0 || d.left_kind == 1) && (d.right_kind == 0 || d.right_kind == 1),
                       "bad boundary kind");
        FPDE_CHECK_ARG(std::isfinite(d.restrict_eps) && d.restrict_eps >= 0.0, "restrict_eps must be >= 0");
    }
    // restricted summing per column (time_summing :4117-4131, newest first): the lags before the
    // first one whose kb = w tau / Da falls below restrict_eps; later lags get weight 0
    std::vector<int> lag_keep(n_cols, max_steps);
    bool any_restrict = false;
    for (int c = 0; c < n_cols; ++c) {
        const fpde_column_desc &d = cols[c];
        if (d.restrict_eps <= 0.0) continue;
        const double kkk0 = d.lag_weights ? 0.0 : l1_interval_weight(d.alpha, 0.0, d.tau);
        std::vector<double> kbl(max_steps);
        for (int64_t j = 1; j <= max_steps; ++j) {
            const double w = d.lag_weights ? d.lag_weights[j] : d.Da * (kkk0 * l1_lag(d.alpha, j)) / d.tau;
            kbl[j - 1] = w * d.tau / d.Da;
        }
        int keep = max_steps;
        fpde_restricted_lags(kbl.data(), max_steps, d.restrict_eps, &keep);
        lag_keep[c] = keep;
        any_restrict = any_restrict || keep < max_steps;
    }
    clear_error();
    fpde_batch *b = new fpde_batch();
    b->ctx = ctx;
    b->n_cols = n_cols;
    b->max_steps = max_steps;
    b->off.resize(n_cols);
    b->N.resize(n_cols);
    int64_t tot = 0;
    for (int c = 0; c < n_cols; ++c) {
        b->off[c] = tot;
        b->N[c] = (int)cols[c].N;
        tot += (cols[c].N + 1 + 511) / 512 * 512;
    }
    b->Ptot = tot;
    std::vector<double> hA(tot, 0.0), hg(tot, 0.0), hal(tot, 0.0), hU(tot, 0.0);
    std::vector<double> hP((size_t)n_cols * BT, 1.0), hQ((size_t)n_cols * BT, 1.0);
    std::vector<double> hKF(tot, 0.0), hCB(tot, 0.0);
    std::vector<double> hw((size_t)n_cols * (max_steps + 1), 0.0);
    std::vector<ColInfo> hc(n_cols);
    std::vector<int> cta_col(tot / 512);
    for (int c = 0; c < n_cols; ++c) {
        const fpde_column_desc &d = cols[c];
        const int64_t N = d.N, o = b->off[c];
        double lam, lamR, kkk0 = 0.0;
        if (d.lag_weights) {
            lam = lamR = d.lag_weights[0];
        } else {                                                   // Om1 :4191, R :3120
            kkk0 = l1_interval_weight(d.alpha, 0.0, d.tau);
            lam = d.Da * (kkk0 / d.tau);
            lamR = d.Da * kkk0 / d.tau;
        }
        double Al = d.left_kind == FPDE_BC_FLUX ? 1.0 : 0.0;         // Al[1]
        hal[o] = Al;
        for (int64_t i = 1; i < N; ++i) {
            Al = d.B[i] / ((d.Rlap[i] + lamR) - d.A[i] * Al);        // Al[i+1]
            hal[o + i] = Al;
            hg[o + i] = Al / d.B[i];
            hA[o + i] = d.A[i];
        }
        for (int64_t i = 0; i <= N; ++i) hU[o + i] = d.u0[i];
        ColInfo &ci = hc[c];
        ci.off = o;
        ci.N = (int)N;
        ci.seg = (int)((N + BT - 1) / BT);
        ci.lam = lam;
        ci.g0 = d.left_value;
        ci.gN = d.right_value;
        ci.dLN = d.dLN;
        ci.AlN = Al;
        ci.rkind = d.right_kind;
        ci.pad = 0;
        for (int t = 0; t < BT; ++t) {                              // segment products (time-invariant)
            const int64_t i0 = std::min<int64_t>((int64_t)t * ci.seg, N), i1 = std::min<int64_t>(i0 + ci.seg, N);
            double pf = 1.0, pb = 1.0;
            for (int64_t i = i0; i < i1; ++i) {
                pf *= hg[o + i] * hA[o + i];
                hKF[o + i] = pf;                                       // forward prefix product (CF)
                pb *= hal[o + i];
            }
            hP[(size_t)c * BT + t] = pf;
            hQ[(size_t)c * BT + t] = pb;
            double kf = 0.0, cb = 1.0;                                  // backward sweep of CF, suffix of al
            for (int64_t i = i1 - 1; i >= i0; --i) {
                kf = hal[o + i] * kf + hKF[o + i];
                cb = hal[o + i] * cb;
                hKF[o + i] = kf;
                hCB[o + i] = cb;
            }
        }
        double *w = hw.data() + (size_t)c * (max_steps + 1);          // w[m] = w_c[max_steps - m]
        for (int64_t m = 0; m < max_steps; ++m) {
            const int64_t j = max_steps - m;
            w[m] = j > lag_keep[c] ? 0.0
                                   : d.lag_weights ? d.lag_weights[j] : d.Da * (kkk0 * l1_lag(d.alpha, j)) / d.tau;
        }
        for (int64_t q = o / 512; q < (o + (N + 1 + 511) / 512 * 512) / 512; ++q) cta_col[q] = c;
    }
    const bool split = precision == FPDE_PREC_SPLIT_BF16X3;
    b->split = split;
    b->LW = (int64_t)max_steps + 64 + 1;
    std::vector<double> hwl;                                           // split: w_c[lag], lag < LW
    std::vector<int> hwcol;                                            // split: column of each 128-row tile
    if (split) {
        hwl.assign((size_t)n_cols * b->LW, 0.0);
        hwcol.assign(tot / 128, 0);
        for (int c = 0; c < n_cols; ++c) {
            const fpde_column_desc &d = cols[c];
            const double kkk0 = d.lag_weights ? 0.0 : l1_interval_weight(d.alpha, 0.0, d.tau);
            for (int64_t j = 1; j < b->LW; ++j)
                hwl[(size_t)c * b->LW + j] = j > lag_keep[c] ? 0.0
                                             : d.lag_weights ? (j <= max_steps ? d.lag_weights[j] : 0.0)
                                                             : d.Da * (kkk0 * l1_lag(d.alpha, j)) / d.tau;
            const int64_t o = b->off[c], Pc = (cols[c].N + 1 + 511) / 512 * 512;
            for (int64_t q = o / 128; q < (o + Pc) / 128; ++q) hwcol[q] = c;
        }
    }
    std::vector<int> order(n_cols);                                    // largest columns first
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->N[x] > b->N[y]; });
    const size_t tb = (size_t)tot * sizeof(double);
    bool fail = dev_alloc((void **)&b->A, tb) || dev_alloc((void **)&b->g, tb) || dev_alloc((void **)&b->al, tb) ||
                dev_alloc((void **)&b->segP, hP.size() * sizeof(double)) ||
                dev_alloc((void **)&b->segQ, hQ.size() * sizeof(double)) || dev_alloc((void **)&b->U, tb) ||
                dev_alloc((void **)&b->KF, tb) || dev_alloc((void **)&b->CB, tb) ||
                dev_alloc((void **)&b->U0, tb) || dev_alloc((void **)&b->Y, tb) ||
                dev_alloc((void **)&b->cols, hc.size() * sizeof(ColInfo)) ||
                dev_alloc((void **)&b->order, order.size() * sizeof(int)) ||
                dev_alloc((void **)&b->cta_col, cta_col.size() * sizeof(int)) ||
                (any_restrict && dev_alloc((void **)&b->col_lag, (size_t)n_cols * sizeof(int))) ||
                dev_alloc((void **)&b->queue, (size_t)max_steps * sizeof(unsigned));
    if (!fail && !split) {
        fail = dev_alloc((void **)&b->D, (size_t)max_steps * tb) || dev_alloc((void **)&b->part, (size_t)KS_MAX * tb) ||
               dev_alloc((void **)&b->wall, hw.size() * sizeof(double));
    } else if (!fail) {
        b->ld16 = ((int64_t)max_steps + 63) / 64 * 64;
        b->ldp = b->ld16 / 64;
        const int64_t wrows = (int64_t)n_cols * 64;
        for (int q = 0; q < 3 && !fail; ++q)
            fail = dev_alloc((void **)&b->h3[q], (size_t)tot * b->ld16 * 2) ||
                   dev_alloc((void **)&b->w3[q], (size_t)wrows * b->ld16 * 2);
        fail = fail || dev_alloc((void **)&b->pA, (size_t)tot * b->ldp) ||
               dev_alloc((void **)&b->pW, (size_t)wrows * b->ldp * sizeof(float)) || dev_alloc((void **)&b->ring, (size_t)64 * tb) ||
               dev_alloc((void **)&b->cfar, (size_t)FAR_MAX_SPLITS * 64 * tb) ||
               dev_alloc((void **)&b->wlag, hwl.size() * sizeof(double)) || dev_alloc((void **)&b->Sn, tb) ||
               dev_alloc((void **)&b->ringf, (size_t)64 * tot * sizeof(float2)) ||
               dev_alloc((void **)&b->pre, (size_t)NEAR_SUB * tot * sizeof(float2)) ||
               dev_alloc((void **)&b->wff, hwl.size() * sizeof(float2)) ||
               dev_alloc((void **)&b->wcol, hwcol.size() * sizeof(int));
        if (!fail) {
            const void *a3[3] = {b->h3[0], b->h3[1], b->h3[2]}, *w3[3] = {b->w3[0], b->w3[1], b->w3[2]};
            int rcp = far_plan3_init(&b->plan3, a3, tot, b->ld16, w3, b->ld16, n_cols);
            if (rcp) {
                std::string keep = fpde_last_error_string();
                fpde_batch_destroy(b);
                return set_error(rcp, "%s", keep.c_str());
            }
        }
    }
    if (fail) {
        std::string keep = fpde_last_error_string();
        fpde_batch_destroy(b);
        return set_error(FPDE_ERR_NOMEM, "%s", keep.c_str());
    }
    cudaStream_t st = ctx->stream;
    cudaMemcpyAsync(b->A, hA.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->g, hg.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->al, hal.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->segP, hP.data(), hP.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->segQ, hQ.data(), hQ.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->KF, hKF.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->CB, hCB.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->U, hU.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->U0, hU.data(), tb, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(b->Y, 0, tb, st);
    cudaMemsetAsync(b->queue, 0, (size_t)max_steps * sizeof(unsigned), st);
    if (!split) {
        cudaMemsetAsync(b->D, 0, (size_t)max_steps * tb, st);
        cudaMemcpyAsync(b->wall, hw.data(), hw.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    } else {
        const int64_t wrows = (int64_t)n_cols * 64;
        for (int q = 0; q < 3; ++q) {
            cudaMemsetAsync(b->h3[q], 0, (size_t)tot * b->ld16 * 2, st);
            cudaMemsetAsync(b->w3[q], 0, (size_t)wrows * b->ld16 * 2, st);
        }
        cudaMemsetAsync(b->pA, 0, (size_t)tot * b->ldp, st);
        cudaMemsetAsync(b->pW, 0, (size_t)wrows * b->ldp * sizeof(float), st);
        cudaMemsetAsync(b->ring, 0, (size_t)64 * tb, st);
        cudaMemsetAsync(b->cfar, 0, (size_t)FAR_MAX_SPLITS * 64 * tb, st);
        cudaMemcpyAsync(b->wlag, hwl.data(), hwl.size() * sizeof(double), cudaMemcpyHostToDevice, st);
        std::vector<float2> hwff(hwl.size());            // w = hi + lo, hi the nearest float
        for (size_t q = 0; q < hwl.size(); ++q) {
            const float hi = (float)hwl[q];
            hwff[q] = make_float2(hi, (float)(hwl[q] - (double)hi));
        }
        cudaMemcpyAsync(b->wff, hwff.data(), hwff.size() * sizeof(float2), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(b->ringf, 0, (size_t)64 * tot * sizeof(float2), st);
        cudaMemcpyAsync(b->wcol, hwcol.data(), hwcol.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    }
    {                                                                  // persistent solve grid
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_solve, BT, 0);
        b->solve_grid = std::max(1, std::min(n_cols, std::max(1, per_sm) * ctx->sm_count));
    }
    cudaMemcpyAsync(b->cols, hc.data(), hc.size() * sizeof(ColInfo), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(b->cta_col, cta_col.data(), cta_col.size() * sizeof(int), cudaMemcpyHostToDevice, st);
    if (b->col_lag) cudaMemcpyAsync(b->col_lag, lag_keep.data(), (size_t)n_cols * sizeof(int), cudaMemcpyHostToDevice, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        fpde_batch_destroy(b);
        return set_error(FPDE_ERR_CUDA, "batch setup: %s", cudaGetErrorString(e));
    }
    *out = b;
    return FPDE_OK;
}

int fpde_batch_run(fpde_batch *b, int steps)
{
    clear_error();
    FPDE_CHECK_ARG(b && steps >= 0, "bad arguments");
    int rc = ctx_enter(b->ctx);
    if (rc) return rc;
    if (steps == 0) return FPDE_OK;
    if (b->n_done + steps > b->max_steps)
        return set_error(FPDE_ERR_CAPACITY, "run of %d steps exceeds the history capacity %d", steps, b->max_steps);
    if (steps < GRAPH_MIN_STEPS) {                 // short runs: enqueued directly, no graph
        int64_t nk = 0;
        if ((rc = batch_enqueue(b, b->ctx->stream, b->n_done, steps, &nk))) return rc;
    } else {
        auto *g = b->graphs.find(b->n_done, steps);
        if (!g) {
            rc = b->graphs.capture(b->n_done, steps,
                                   [&](cudaStream_t cs, int64_t *nk, int *) { return batch_enqueue(b, cs, b->n_done, steps, nk); },
                                   &g);
            if (rc) return rc;
        }
        FPDE_CUDA(cudaGraphLaunch(g->exec, b->ctx->stream));
        count_launches(g->launches);
    }
    b->n_done += steps;
    return FPDE_OK;
}

int fpde_batch_get_state(fpde_batch *b, int col, double *u, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(b && u && col >= 0 && col < b->n_cols, "bad arguments");
    int rc = ctx_enter(b->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u, b->U + b->off[col], (b->N[col] + 1) * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, b->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return FPDE_OK;
}

int fpde_batch_layout(const fpde_batch *b, int col, int64_t *offset, int64_t *N, int64_t *total)
{
    FPDE_CHECK_ARG(b && col >= 0 && col < b->n_cols, "bad arguments");
    if (offset) *offset = b->off[col];
    if (N) *N = b->N[col];
    if (total) *total = b->Ptot;
    return FPDE_OK;
}

int fpde_batch_reset(fpde_batch *b, const double *u_padded, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(b, "null argument");
    int rc = ctx_enter(b->ctx);
    if (rc) return rc;
    const double *src = u_padded ? u_padded : b->U0;
    const cudaMemcpyKind kind = (!u_padded || on_device) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    FPDE_CUDA(cudaMemcpyAsync(b->U, src, b->Ptot * sizeof(double), kind, b->ctx->stream));
    if (u_padded && !on_device) FPDE_CUDA(cudaStreamSynchronize(b->ctx->stream));
    b->n_done = 0;
    return FPDE_OK;
}

int fpde_batch_solve_host(fpde_batch *b, const double *u0_padded_host, int steps, double *u_out_padded_host)
{
    clear_error();
    FPDE_CHECK_ARG(b && u0_padded_host && u_out_padded_host, "null argument");
    int rc = fpde_batch_reset(b, u0_padded_host, 0);
    if (rc) return rc;
    if ((rc = fpde_batch_run(b, steps))) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u_out_padded_host, b->U, b->Ptot * sizeof(double), cudaMemcpyDeviceToHost,
                              b->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(b->ctx->stream));
    return ctx_check_flags(b->ctx, "batch");
}

}  // extern "C"
