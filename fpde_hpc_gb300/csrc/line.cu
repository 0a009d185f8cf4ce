// 1D line problem (fpde_line_*): the plain FP64 path and the split-precision path.
//
// Per time step n (fpde_hpc_1d.cpp calc_step / U1 with the history applied every step):
//   FP64 path (one launch each per step)
//     1. k_l1_partial : part[ks][i] = sum_t w[n-t] D_t[i]        (FP64 history GEMV)
//     2. k_line_solve : S = sum_ks part, Om = -lam U + src + S, Thomas solve, U <- U^{n+1},
//                       D_n = U^{n+1} - U^n
//   split path (blocks of 64 steps starting at n0)
//     at n0:  convert the finished block's FP64 increments into 16-bit history slices,
//             build the Toeplitz weight tile and run the tensor-core contraction for the
//             far history t < n0 (tc_far.cu) -> FP64 partials C[split][j][i]
//     steps of the block: k_line_block_spec, one persistent launch: S = sum_split C[split][j][i]
//             + sum_{n0 <= t < n} w[n-t] D_t[i] (near history in float-float), the solve
//             (speculated one step ahead), and D_n into a 64-row FP64 ring.
// The whole run is captured once into a CUDA graph and replayed.
//
// The Thomas solve of a long line runs on all SMs. The alpha recurrence
// Al[i+1] = B/(R - A Al[i]) is time-invariant (uniform tau) and is done once on the host;
// per step only the two first-order recurrences remain,
//   forward   y_i = Bt[i+1] = g_i (A_i y_{i-1} - Om_i),   g_i = Al[i+1]/B_i
//   backward  U_i = Al[i+1] U_{i+1} + y_i.
// Each CTA owns a chunk of nodes and solves both recurrences inside it from zero carries:
// threads sweep segments of SP nodes sequentially, segments are joined by warp-shuffle
// scans of (product, value) pairs and across warps through shared memory. Because the
// recurrences are linear, the true solution is U = U^cta + c_in GG + u_b CB, with GG and CB
// time-invariant per node. Every CTA publishes two numbers per step (its last y and first u
// with zero carries) behind a release flag; warp 0 of every CTA waits (bounded) for all
// flags and forms its chunk's carries c_in and u_b as dot products with precomputed rows,
// and every node takes two FMAs to finish.
#include <climits>
#include <map>
#include <vector>
#include <cmath>
#include <cstring>
#include <algorithm>

#include "common.cuh"
#include "kernels.cuh"
#include "graph_cache.cuh"
#include "tc_far.cuh"
#include "scan.cuh"
#include "ff.cuh"

namespace fpde {

constexpr int LT = 256;      // threads per CTA of the line solve
constexpr int LSEG = 8;      // max nodes per thread
constexpr int BLK = 64;      // steps per block of the split path (= tensor-core N)

struct LineSolveArgs {
    const double *A, *g, *al, *cf, *cb;   // per node: coefficients, thread-segment products
    const double *CF, *CB, *GG;           // per node: chunk-level forward/backward data
    const double *src;                    // optional source (N+1) of this step, may be null
    const double *lamv;                   // optional per-node local weight (replaces lam)
    const double *eA, *eB;                // optional explicit neighbour weights (theta A, theta B)
    double *U;                            // state (N+1)
    double *Drow;                         // increment of node i goes to Drow[i * dstride]
    int64_t dstride;
    const double *part;                   // S += sum_{q<KS} part[q*pstride + i]
    int64_t pstride;
    double *agg;                          // [G][2] (chunk's last y, chunk's first u), agg[2G] = old U[N-1]
    unsigned long long *cflag;            // per chunk: launch sequence number of its published values
    unsigned long long *seq;              // launch sequence counter (read at start, advanced by CTA 0)
    const double *Lf, *Mb, *Kb, *mb;      // chunk-carry rows: c_in = Lf Y, u_b = Mb U0 + Kb Y + mb U_N
    unsigned *barrier, *flags;
    double lam, g0, gN, dLN, AlN;
    int KS, N, G, rkind, chunk;
};


template <int SP>
__device__ __forceinline__ double right_value(const LineSolveArgs &p, double BtN, double uNm1)
{
    if (p.rkind == FPDE_BC_DIRICHLET) return p.gN;
    if (fabs(BtN) > 1e-15) return (fabs(1.0 - p.AlN) > 1e-15) ? (BtN + p.gN * p.dLN) / (1.0 - p.AlN) : uNm1;
    return (fabs(1.0 - p.AlN) > 1e-15) ? 0.0 : uNm1;
}

// One time step of a line: history sum -> right-hand side -> Thomas solve -> U, increment.
// Each CTA owns a chunk [a, b) of nodes and solves it with zero carries in both sweeps
// (y^cta, u^cta). The true solution is u = u^cta + c_in * GG + u_b * CB with the chunk's
// forward carry c_in and backward carry u_b; after one grid barrier, warp 0 of every CTA
// resolves all chunk carries from two published numbers per chunk.
template <int SP>
__global__ void __launch_bounds__(LT) k_line_solve(LineSolveArgs p)
{
    constexpr int NW = LT / 32;
    __shared__ double wP[NW], wX[NW], wPe[NW], wXe[NW];
    __shared__ double s_cin, s_ub, s_UN;
    __shared__ unsigned long long s_seq;
    __shared__ int s_abort;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int c = blockIdx.x;
    if (tid == 0) s_seq = *((volatile unsigned long long *)p.seq) + 1;
    const int a = c * p.chunk;
    const int b = min(a + p.chunk, p.N);
    const int i0 = a + tid * SP;
    const int i1 = min(i0 + SP, b);
    const int cnt = max(0, i1 - i0);

    // ---- warp 0: the time-invariant chunk-carry rows of this chunk (used after the gather)
    double lf[5], lfN[5], mbv[5], kbv[5], mbc = 0.0;
    if (warp == 0) {
        const int G = p.G;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const int q = lane + 32 * t;
            const bool in = q < G;
            lf[t] = in ? __ldg(p.Lf + (int64_t)c * G + q) : 0.0;
            lfN[t] = in ? __ldg(p.Lf + (int64_t)G * G + q) : 0.0;
            mbv[t] = in ? __ldg(p.Mb + (int64_t)c * G + q) : 0.0;
            kbv[t] = in ? __ldg(p.Kb + (int64_t)c * G + q) : 0.0;
        }
        mbc = __ldg(p.mb + c);
    }
    // ---- every per-node input of the step in one round of loads
    double uo[SP], om[SP], kA[SP], kg[SP], kal[SP], kcf[SP], kcb[SP], kCB[SP], kGG[SP];
#pragma unroll
    for (int k = 0; k < SP; ++k) {
        const bool in = k < cnt;
        const int i = in ? i0 + k : 0;
        uo[k] = in ? p.U[i] : 0.0;
        kA[k] = in ? __ldg(p.A + i) : 0.0;
        kg[k] = in ? __ldg(p.g + i) : 0.0;
        kal[k] = in ? __ldg(p.al + i) : 0.0;
        kcf[k] = in ? __ldg(p.cf + i) : 1.0;
        kcb[k] = in ? __ldg(p.cb + i) : 1.0;
        kCB[k] = in ? __ldg(p.CB + i) : 0.0;
        kGG[k] = in ? __ldg(p.GG + i) : 0.0;
        om[k] = 0.0;
    }
    if (p.KS > 0) {                                                  // FP64 partials, 4-way ILP
        double a0[SP], a1[SP], a2[SP], a3[SP];
#pragma unroll
        for (int k = 0; k < SP; ++k) { a0[k] = 0.0; a1[k] = 0.0; a2[k] = 0.0; a3[k] = 0.0; }
        int q = 0;
        for (; q + 4 <= p.KS; q += 4) {
#pragma unroll
            for (int k = 0; k < SP; ++k) {
                if (k < cnt) {
                    const double *pp = p.part + (int64_t)q * p.pstride + i0 + k;
                    a0[k] += __ldcg(pp);
                    a1[k] += __ldcg(pp + p.pstride);
                    a2[k] += __ldcg(pp + 2 * p.pstride);
                    a3[k] += __ldcg(pp + 3 * p.pstride);
                }
            }
        }
        for (; q < p.KS; ++q) {
#pragma unroll
            for (int k = 0; k < SP; ++k)
                if (k < cnt) a0[k] += __ldcg(p.part + (int64_t)q * p.pstride + i0 + k);
        }
#pragma unroll
        for (int k = 0; k < SP; ++k) om[k] = (a0[k] + a1[k]) + (a2[k] + a3[k]);
    }
#pragma unroll
    for (int k = 0; k < SP; ++k) {
        const double lam = (p.lamv && k < cnt) ? __ldg(p.lamv + i0 + k) : p.lam;
        om[k] = (-(lam * uo[k]) + (p.src && k < cnt ? __ldg(p.src + i0 + k) : 0.0)) + om[k];
    }
    if (p.eA && cnt > 0) {                                           // explicit part on the old state
        double ul = i0 > 0 ? p.U[i0 - 1] : 0.0;
        const double ur = p.U[i0 + cnt];                              // i0 + cnt <= N
#pragma unroll
        for (int k = 0; k < SP; ++k) {
            if (k < cnt) {
                const double un = k + 1 < cnt ? uo[k + 1] : ur;
                om[k] -= fma(__ldg(p.eA + i0 + k), ul, __ldg(p.eB + i0 + k) * un);
                ul = uo[k];
            }
        }
    }

    // ---- forward sweep of the chunk from zero carry
    double y[SP];
    double yl = 0.0;
#pragma unroll
    for (int k = 0; k < SP; ++k) {
        if (k < cnt) {
            const int i = i0 + k;
            if (i == 0) yl = p.g0;                                  // Bt[1]
            else yl = kg[k] * (kA[k] * yl - om[k]);
            y[k] = yl;
        }
    }
    double P = 1.0, X = cnt > 0 ? yl : 0.0;
#pragma unroll
    for (int k = 0; k < SP; ++k)
        if (k < cnt) P = kcf[k];
    warp_scan_up(P, X, lane);
    double Pe = __shfl_up_sync(FULL, P, 1), Xe = __shfl_up_sync(FULL, X, 1);
    if (lane == 0) { Pe = 1.0; Xe = 0.0; }
    if (lane == 31) { wP[warp] = P; wX[warp] = X; }
    __syncthreads();
    if (warp == 0) {
        double Pw = lane < NW ? wP[lane] : 1.0, Xw = lane < NW ? wX[lane] : 0.0;
        warp_scan_up(Pw, Xw, lane);
        double Pwe = __shfl_up_sync(FULL, Pw, 1), Xwe = __shfl_up_sync(FULL, Xw, 1);
        if (lane == 0) { Pwe = 1.0; Xwe = 0.0; }
        if (lane < NW) { wPe[lane] = Pwe; wXe[lane] = Xwe; }
    }
    __syncthreads();
    {
        const double carry = fma(Pe, wXe[warp], Xe);               // chunk carry-in taken as 0
#pragma unroll
        for (int k = 0; k < SP; ++k)
            if (k < cnt) y[k] = fma(kcf[k], carry, y[k]);
    }
    // ---- backward sweep of the chunk from zero carry
    double ub[SP];
    double ul = 0.0;
#pragma unroll
    for (int k = SP - 1; k >= 0; --k) {
        if (k < cnt) {
            ul = fma(kal[k], ul, y[k]);
            ub[k] = ul;
        }
    }
    P = cnt > 0 ? kcb[0] : 1.0;
    X = cnt > 0 ? ul : 0.0;
    warp_scan_down(P, X, lane);
    Pe = __shfl_down_sync(FULL, P, 1);
    Xe = __shfl_down_sync(FULL, X, 1);
    if (lane == 31) { Pe = 1.0; Xe = 0.0; }
    __syncthreads();                                                // wP/wX reuse
    if (lane == 0) { wP[warp] = P; wX[warp] = X; }
    __syncthreads();
    if (warp == 0) {
        double Pw = lane < NW ? wP[lane] : 1.0, Xw = lane < NW ? wX[lane] : 0.0;
        warp_scan_down(Pw, Xw, lane);
        double Pwe = __shfl_down_sync(FULL, Pw, 1), Xwe = __shfl_down_sync(FULL, Xw, 1);
        if (lane >= NW - 1) { Pwe = 1.0; Xwe = 0.0; }
        if (lane < NW) { wPe[lane] = Pwe; wXe[lane] = Xwe; }
    }
    __syncthreads();
    {
        const double carry = fma(Pe, wXe[warp], Xe);
#pragma unroll
        for (int k = 0; k < SP; ++k)
            if (k < cnt) ub[k] = fma(kcb[k], carry, ub[k]);
    }
    // ---- publish the chunk's last y and first u (and the old U[N-1])
    if (cnt > 0 && i1 == b) {
        double ylast = 0.0, ulast = 0.0;
#pragma unroll
        for (int k = 0; k < SP; ++k)
            if (k < cnt) { ylast = y[k]; ulast = uo[k]; }
        p.agg[2 * c] = ylast;
        if (b == p.N) p.agg[2 * p.G] = ulast;
    }
    if (cnt > 0 && i0 == a) p.agg[2 * c + 1] = ub[0];
    __syncthreads();
    if (tid == 0 && p.G > 1) {
        __threadfence();
        asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p.cflag + c), "l"(s_seq) : "memory");
    }
    // ---- warp 0: wait for every chunk, then this chunk's carries by three dot products
    if (warp == 0) {
        const int G = p.G;
        bool ok = true;
        if (G > 1) {
            const unsigned long long t0 = gtimer_ns();
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                const int q = lane + 32 * t;
                if (q < G && ok) {
                    unsigned long long f;
                    while (true) {
                        asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(f) : "l"(p.cflag + q) : "memory");
                        if (f >= s_seq) break;
                        if (gtimer_ns() - t0 > 1000000000ull) { ok = false; break; }
                    }
                }
            }
        }
        ok = __all_sync(FULL, ok);
        if (!ok) {
            if (lane == 0) { atomicOr(p.flags, DEVERR_BARRIER_TIMEOUT); s_abort = 1; }
        } else {
            double sc = 0.0, syN = 0.0, sub = 0.0;
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                const int q = lane + 32 * t;
                if (q < G) {
                    const double ye = __ldcg(p.agg + 2 * q), u0 = __ldcg(p.agg + 2 * q + 1);
                    sc = fma(lf[t], ye, sc);
                    syN = fma(lfN[t], ye, syN);
                    sub = fma(mbv[t], u0, fma(kbv[t], ye, sub));
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                sc += __shfl_xor_sync(FULL, sc, o);
                syN += __shfl_xor_sync(FULL, syN, o);
                sub += __shfl_xor_sync(FULL, sub, o);
            }
            const double UN = right_value<SP>(p, syN, __ldcg(p.agg + 2 * G));
            if (lane == 0) { s_cin = sc; s_ub = fma(mbc, UN, sub); s_UN = UN; s_abort = 0; }
        }
    }
    __syncthreads();
    if (s_abort) return;
    const double cin = s_cin, ubv = s_ub;
#pragma unroll
    for (int k = 0; k < SP; ++k) {
        if (k < cnt) {
            const int i = i0 + k;
            const double un = fma(kCB[k], ubv, fma(kGG[k], cin, ub[k]));
            p.U[i] = un;
            p.Drow[(int64_t)i * p.dstride] = un - uo[k];
        }
    }
    if (cnt > 0 && i1 == p.N) {
        const double UN = s_UN, uNold = p.U[p.N];
        p.U[p.N] = UN;
        p.Drow[(int64_t)p.N * p.dstride] = UN - uNold;
    }
    if (c == 0 && tid == 0) *((volatile unsigned long long *)p.seq) = s_seq;   // all CTAs have read it
}

// ---------------------------------------------------------------------------------------
// Persistent form for the split path: one cooperative launch advances steps j0 .. j0+nsteps-1
// of a 64-step block, with two warp roles per CTA:
//   solver warps (LTS threads, SP nodes each): the chunk's right-hand side, the two sweeps and
//     scans, the exchange of the two chunk aggregates with all other chunks (one row of value
//     slots per step, each written once per launch and polled until it leaves the all-bits-set
//     pattern) and the new state; state and time-invariant data stay in registers for the
//     whole launch;
//   history warps (LTS threads): during step j, the far partials and the near history of
//     step j+1 for every node of the chunk except the newest increment (which the solver
//     adds), handed over in shared memory.
// The two roles meet at one CTA barrier per step; the solver warps synchronise among
// themselves with a named barrier. The near-history work thus overlaps the latency-bound
// scans and the exchange.
//
// All products of the scans are time-invariant, so they are precomputed on the host: a
// warp-scan level is one shuffle and one FMA, the combination across the solver warps is a
// dot product with precomputed coefficients, and the chunk's aggregates are the last y and
// first u of the chunk, published by the two threads that own them.
constexpr int LTS = 128;                 // solver threads per CTA (= history threads)
constexpr int NWS = LTS / 32;

struct ScanCoef {
    const double *lane;       // [12][G*LTS]: 5 forward level products, forward prefix, 5 backward, backward suffix
    const double *warp;       // [G][2][NWS][NWS]: cross-warp coefficients (forward, backward)
};

struct LineBlockArgs {
    const double *A, *g, *al, *cf, *cb, *CB, *GG;
    const double *lamv, *eA, *eB;         // optional explicit part (theta != 0)
    const double *src;                    // optional per-step source rows ((N+1) each)
    int src_rows;
    double *U;                            // state: read at start, written at the end
    double *ring;                         // [64][P] time-major increments of the block
    const double *cfar;                   // far partials: split k, step j at row k*far_ld + far_row0 + j of P
    int KS;
    int far_ld, far_row0;
    int far_pairs;                        // 1: partials are float pairs (three-slice contraction)
    int64_t P;
    const double *wlag;                   // w[lag]
    double *agg;                          // [nsteps][2G+2] aggregates, one row of slots per step
    unsigned long long *cflag, *seq;
    const double *Lf, *Mb, *Kb, *mb;
    ScanCoef sc;
    const double *RB1, *RB2, *RY1, *RY2;  // speculative kernel: sweep responses to E1, E2
    float2 *ringf;                        // speculative kernel: the ring as float pairs
    const float2 *wff;                    // speculative kernel: w[lag] as float pairs
    // speculative kernel: right-hand side pre-scaled by -g so the forward sweep is one FMA
    // (y = ga y + Om', ga = g A, Om' = -g Om): ng = -g, c1 = -g (w1 - lam), c2 = g w1, c3 = -g w2
    const double *ga, *ng, *c1, *c2, *c3;
    const float2 *ngf;                    // -g as float pairs (the history warps deliver -g H)
    // speculative kernel with an explicit part: the pre-scaled weights g theta A (on ub at i-1,
    // i > a) and g theta B (on ub at i+1, i < b-1) of the chunk's own zero-carry backward result
    const double *xa, *xb;
    unsigned *flags;
    double lam, g0, gN, dLN, AlN;
    int64_t n0;                           // global index of step j0
    int j0, nsteps, N, G, rkind, chunk;
};

constexpr unsigned long long SLOT_EMPTY = ~0ull;        // exchange slot not yet written (a NaN pattern)

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const double *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_relaxed_f64(double *p, double v)
{
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((unsigned long long)__double_as_longlong(v))
                 : "memory");
}

__device__ __forceinline__ void solver_sync() { asm volatile("bar.sync 1, %0;" ::"n"(LTS) : "memory"); }

// history warps of the block solves: S[node] = far partials of step j + sum_{r < rmax} w[j - r]
// D_r[node], in float-float arithmetic on the FP32 pipe (one FP64 add per node at the end), from
// the float-pair copy of the ring and float-pair weights. GB300 issues 2 DFMA/clk/SM, so the FP64 form of these sums (up to 63 rows a step)
// occupied the FP64 pipe the solver's recurrences wait on.
// (ah, al) += far partials of steps j .. j+NJ-1 (NJ accumulators; every load issued first).
template <int SP, int NJ>
__device__ __forceinline__ void far_fold_ff(const LineBlockArgs &p, int ht, int a, int b, int j, float (&ah)[NJ][SP],
                                            float (&al)[NJ][SP])
{
    double v[NJ][FAR_MAX_SPLITS][SP];
#pragma unroll
    for (int m = 0; m < NJ; ++m)
#pragma unroll
        for (int k = 0; k < FAR_MAX_SPLITS; ++k)
#pragma unroll
            for (int q = 0; q < SP; ++q) {
                const int64_t node = a + ht + LTS * q;
                v[m][k][q] = (k < p.KS && node < b && j + m < BLK)
                                 ? __ldcg(p.cfar + ((int64_t)k * p.far_ld + p.far_row0 + j + m) * p.P + node)
                                 : 0.0;
            }
#pragma unroll
    for (int m = 0; m < NJ; ++m)
#pragma unroll
        for (int k = 0; k < FAR_MAX_SPLITS; ++k)
#pragma unroll
            for (int q = 0; q < SP; ++q) {
                const float2 f = p.far_pairs ? *reinterpret_cast<const float2 *>(&v[m][k][q]) : d2ff(v[m][k][q]);
                ff_add(ah[m][q], al[m][q], f.x, f.y);
            }
}

// (ah, al) += sum_{r < rmax} w[j - r] D_r for this thread's nodes (rows of the float-pair ring,
// two batches of rows in flight).
template <int SP>
__device__ __forceinline__ void rows_ff(const LineBlockArgs &p, int ht, int a, int b, int j, int rmax, float *ah,
                                        float *al)
{
    constexpr int RB = SP <= 4 ? 8 : 4;                  // rows per batch
    int64_t node[SP];
#pragma unroll
    for (int q = 0; q < SP; ++q) node[q] = a + ht + LTS * q;
    float2 va[RB][SP], vb[RB][SP];
    auto load = [&](float2 (&v)[RB][SP], int r0) {
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const float2 *row = p.ringf + (int64_t)(r0 + u) * p.P;
#pragma unroll
            for (int q = 0; q < SP; ++q) v[u][q] = node[q] < b ? row[node[q]] : make_float2(0.f, 0.f);
        }
    };
    auto accumulate = [&](const float2 (&v)[RB][SP], int r0) {
#pragma unroll
        for (int u = 0; u < RB; ++u) {
            const float2 w = __ldg(p.wff + (j - r0 - u));
#pragma unroll
            for (int q = 0; q < SP; ++q) ff_fma(ah[q], al[q], w, v[u][q]);
        }
#pragma unroll
        for (int q = 0; q < SP; ++q) ff_renorm(ah[q], al[q]);
    };
    int r = 0;
    if (RB <= rmax) load(va, 0);
    while (r + RB <= rmax) {                             // batch r in registers, the next one loading
        const bool more = r + 2 * RB <= rmax;
        if (more) load(vb, r + RB);
        accumulate(va, r);
        r += RB;
        if (!more) break;
        const bool more2 = r + 2 * RB <= rmax;
        if (more2) load(va, r + RB);
        accumulate(vb, r);
        r += RB;
        if (!more2) break;
    }
    for (; r < rmax; ++r) {
        const float2 w = __ldg(p.wff + (j - r));
        const float2 *row = p.ringf + (int64_t)r * p.P;
#pragma unroll
        for (int q = 0; q < SP; ++q)
            if (node[q] < b) ff_fma(ah[q], al[q], w, row[node[q]]);
    }
}

// The speculative kernel keeps the block's newest NR increment rows (float pairs, this chunk's
// nodes) in dynamic shared memory, so the per-step history sums read them from shared memory
// instead of re-reading every earlier row of the block from L2 each step; older rows come from
// the float-pair ring in global memory.
template <int SP>
struct SpecRing {
    static constexpr int NR = SP <= 2 ? 64 : (SP == 4 ? 48 : 24);
    static constexpr size_t bytes = (size_t)NR * LTS * SP * sizeof(float2);
};

// (ah, al) += sum_{r0 <= r < r1} w[j - r] D_r from the shared-memory row ring (slot r mod NR).
template <int SP>
__device__ __forceinline__ void rows_smem_ff(const LineBlockArgs &p, const float2 *sR, int ht, int j, int r0, int r1,
                                             float *ah, float *al)
{
    constexpr int NR = SpecRing<SP>::NR;
    int slot = r0 % NR;
    int r = r0;
    for (; r + 8 <= r1; r += 8) {
        float2 v[8][SP];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            int sl = slot + u;
            if (sl >= NR) sl -= NR;
#pragma unroll
            for (int q = 0; q < SP; ++q) v[u][q] = sR[sl * (LTS * SP) + ht + LTS * q];
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float2 w = __ldg(p.wff + (j - r - u));
#pragma unroll
            for (int q = 0; q < SP; ++q) ff_fma(ah[q], al[q], w, v[u][q]);
        }
#pragma unroll
        for (int q = 0; q < SP; ++q) ff_renorm(ah[q], al[q]);
        slot += 8;
        if (slot >= NR) slot -= NR;
    }
    for (; r < r1; ++r) {
        const float2 w = __ldg(p.wff + (j - r));
#pragma unroll
        for (int q = 0; q < SP; ++q) ff_fma(ah[q], al[q], w, sR[slot * (LTS * SP) + ht + LTS * q]);
        if (++slot == NR) slot = 0;
    }
}

// (ah, al) += sum_{r < rmax} w[j - r] D_r: rows below rlo from the global float-pair ring, the
// rest from the shared-memory row ring.
template <int SP>
__device__ __forceinline__ void rows_split_ff(const LineBlockArgs &p, const float2 *sR, int ht, int a, int b, int j,
                                              int rmax, int rlo, float *ah, float *al)
{
    const int rg = min(rlo, rmax);
    if (rg > 0) rows_ff<SP>(p, ht, a, b, j, rg, ah, al);
    if (rmax > rg) rows_smem_ff<SP>(p, sR, ht, j, rg, rmax, ah, al);
}

// v[n - 1] for a register array and a run-time n (1..SP) without indexing it dynamically,
// which would move the array to local memory.
template <int SP>
__device__ __forceinline__ double last_of(const double (&v)[SP], int n)
{
    double r = v[0];
#pragma unroll
    for (int k = 1; k < SP; ++k)
        if (k == n - 1) r = v[k];
    return r;
}

// out = (ah + al) sg for this thread's nodes, sg a per-node float pair: float-float, one FP64 add.
template <int SP>
__device__ __forceinline__ void history_store_scaled_ff(int ht, int a, int b, const float *ah, const float *al,
                                                        const float2 *sg, double *out)
{
#pragma unroll
    for (int q = 0; q < SP; ++q)
        if (a + ht + LTS * q < b) {
            const float ph = __fmul_rn(ah[q], sg[q].x);
            float pe = __fmaf_rn(ah[q], sg[q].x, -ph);
            pe = __fmaf_rn(ah[q], sg[q].y, pe);
            pe = __fmaf_rn(al[q], sg[q].x, pe);
            out[ht + LTS * q] = f2d_bits(ph) + f2d_bits(pe);
        }
}

// ---------------------------------------------------------------------------------------
// Speculative form of the block solve (split path). Everything in a step is linear, so step
// t+1's right-hand side is known up to step t's two chunk carries:
//   Om^{t+1} = Omega0 + c_in E1 + u_b E2,   E1 = (w1 - lam) GG,  E2 = (w1 - lam) CB,
//   Omega0   = (w1 - lam) ub_t - w1 u^t + src + H_{t+1} + w2 D_{t-1}
// (ub_t: the chunk's zero-carry backward result of step t, H: far partials plus every history
// row but the two newest). With an explicit part (EXPL: Om -= theta (A u_{i-1} - Rlap u_i +
// B u_{i+1}) on the state before the step) lam becomes the per-node lam - theta Rlap, the
// neighbours' ub_t enter Omega0 (xa, xb; at the chunk's first node the term on u_{a-1} =
// al_{a-1} u_a + c_in folds into c1) and E1, E2 carry the neighbours' GG, CB (host-built). The solver warps therefore run step t+1's sweeps and scans on
// Omega0 while step t's aggregates are exchanged, and correct them afterwards with the
// time-invariant chunk-local responses to E1, E2 (RB: backward, RY: forward at the chunk's last
// node). The history warps poll step t's aggregates of every chunk and form this chunk's carry
// dot products while the solver warps sweep step t+1, and hand the carries over through a
// named barrier (bar.arrive / bar.sync): per step the solver's path is finalise + publish ->
// sweeps -> carries, and the exchange's latency is hidden behind the sweeps.
// GB300 runs FP64 at 2 DFMA/clk/SM (a warp's FP64 instruction holds its scheduler's FP64 pipe
// for ~64 cycles), so the history warps sum in float-float on the FP32 pipe (ringf, wff: the
// increments and weights as float pairs; the solver hands each new FP64 row over in shared
// memory and the history warps convert it), and the four history warps form the four carry
// dot products side by side.
template <int SP, bool EXPL>
__global__ void __launch_bounds__(2 * LTS, 1) k_line_block_spec(LineBlockArgs p)
{
    __shared__ double sS[2][LTS * SP];                   // H_t by parity of t
    __shared__ double sUf[EXPL ? LTS : 1], sUl[EXPL ? LTS : 1];   // per solver thread: first, last ub
    __shared__ double sD[2][LTS * SP];                   // D_t (FP64) by parity of t
    __shared__ double wXf[NWS], wXb[NWS];
    __shared__ double sCf[NWS][NWS], sCb[NWS][NWS];
    __shared__ double s_red[4];                          // c_in, Mb.U0, Kb.Y, right end value
    __shared__ int s_abort;
    extern __shared__ float2 spec_rows[];                // [NR][LTS * SP]: the newest increment rows
    const int tid = threadIdx.x;
    const bool solver = tid < LTS;
    const int c = blockIdx.x, G = p.G, N = p.N;
    const int a = c * p.chunk;
    const int b = min(a + p.chunk, N);
    const int jend = p.j0 + p.nsteps;
    if (tid == 0) s_abort = 0;
    if (tid < NWS * NWS) {
        const double *wc = p.sc.warp + (size_t)c * (2 * NWS * NWS);
        sCf[tid / NWS][tid % NWS] = wc[tid];
        sCb[tid / NWS][tid % NWS] = wc[NWS * NWS + tid];
    }

    if (!solver) {
        // ============== history warps: H_t = far^t + sum_{0 <= r <= t-3} w[t-r] D_r.
        // H_{t+3} is summed before X(s+1) from every row but D_t; after X(s+1) D_t arrives in
        // sD, is converted into the float-pair ring and its one term completes H_{t+3}.
        const int ht = tid - LTS;
        const int lane = tid & 31, hw = ht >> 5;
        // history warp hw's carry dot product over the chunks' aggregates: 0 Lf[c].Y (c_in),
        // 1 Mb[c].U0, 2 Kb[c].Y, 3 Lf[G].Y (the flux end's y; unused at a Dirichlet end)
        const bool flux = p.rkind != FPDE_BC_DIRICHLET;
        const double *cvec = hw == 0 ? p.Lf + (int64_t)c * G
                           : hw == 1 ? p.Mb + (int64_t)c * G
                           : hw == 2 ? p.Kb + (int64_t)c * G
                                     : p.Lf + (int64_t)G * G;
        const int slot_off = hw == 1 ? 1 : 0;            // U0 slots for warp 1, Y slots otherwise
        double cv[5];
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const int q = lane + 32 * k;
            cv[k] = q < G ? __ldg(cvec + q) : 0.0;
        }
        // step s's aggregates of every chunk, polled as values (each slot holds the all-bits-set
        // pattern until its one write of the launch; a 64-bit load is single-copy atomic); warp 3
        // forms the right end value (U1 :4685-4719)
        auto carries = [&](int s) {
            const double *agg = p.agg + (size_t)s * (2 * G + 2);
            if (hw == 3 && !flux) {
                if (lane == 0) s_red[3] = p.gN;
                return;
            }
            double v[5], uNm1 = 0.0;
            bool ok = true;
            const unsigned long long t0 = gtimer_ns();
            while (true) {
                bool mine = true;
#pragma unroll
                for (int k = 0; k < 5; ++k) {
                    const int q = lane + 32 * k;
                    v[k] = 0.0;
                    if (q < G) {
                        const unsigned long long bv = ld_relaxed_u64(agg + 2 * q + slot_off);
                        if (bv == SLOT_EMPTY) mine = false;
                        v[k] = __longlong_as_double((long long)bv);
                    }
                }
                if (hw == 3 && lane == 0) {
                    const unsigned long long bn = ld_relaxed_u64(agg + 2 * G);
                    if (bn == SLOT_EMPTY) mine = false;
                    uNm1 = __longlong_as_double((long long)bn);
                }
                if (__all_sync(FULL, mine)) break;
                if (gtimer_ns() - t0 > 1000000000ull) { ok = false; break; }
            }
            ok = __all_sync(FULL, ok);
            if (!ok) {
                if (lane == 0) { atomicOr(p.flags, DEVERR_BARRIER_TIMEOUT); s_abort = 1; }
                return;
            }
            double sum = 0.0;
#pragma unroll
            for (int k = 0; k < 5; ++k) sum = fma(cv[k], v[k], sum);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(FULL, sum, o);
            if (lane == 0) {
                if (hw == 3) {                           // flux end: lane 0 holds the old U[N-1]
                    double uN;
                    if (fabs(sum) > 1e-15) uN = (fabs(1.0 - p.AlN) > 1e-15) ? (sum + p.gN * p.dLN) / (1.0 - p.AlN) : uNm1;
                    else uN = (fabs(1.0 - p.AlN) > 1e-15) ? 0.0 : uNm1;
                    s_red[3] = uN;
                } else {
                    s_red[hw] = sum;
                }
            }
        };
        constexpr int NR = SpecRing<SP>::NR;
        float2 *sR = spec_rows;
        const int rlo0 = max(0, p.j0 - NR);              // rows of earlier launches into the ring
        for (int r = rlo0; r < p.j0; ++r) {
#pragma unroll
            for (int q = 0; q < SP; ++q) {
                const int i = a + ht + LTS * q;
                if (i < b) sR[(r % NR) * (LTS * SP) + ht + LTS * q] = p.ringf[(int64_t)r * p.P + i];
            }
        }
        float2 sg[SP];                                   // -g of this thread's nodes
#pragma unroll
        for (int q = 0; q < SP; ++q) {
            const int i = a + ht + LTS * q;
            sg[q] = i < b ? __ldg(p.ngf + i) : make_float2(0.f, 0.f);
        }
        float h3[3][SP], l3[3][SP];                      // H_j0, H_j0+1, H_j0+2
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
            for (int q = 0; q < SP; ++q) { h3[m][q] = 0.f; l3[m][q] = 0.f; }
        far_fold_ff<SP, 3>(p, ht, a, b, p.j0, h3, l3);
        rows_split_ff<SP>(p, sR, ht, a, b, p.j0, max(p.j0 - 2, 0), rlo0, h3[0], l3[0]);
        history_store_scaled_ff<SP>(ht, a, b, h3[0], l3[0], sg, sS[p.j0 & 1]);
        __syncthreads();                                                    // start: the solver's prologue
        if (p.j0 + 1 < jend) {                                              // runs beside the rest
            rows_split_ff<SP>(p, sR, ht, a, b, p.j0 + 1, max(p.j0 - 1, 0), rlo0, h3[1], l3[1]);
            history_store_scaled_ff<SP>(ht, a, b, h3[1], l3[1], sg, sS[(p.j0 + 1) & 1]);
        }
        float ah[SP], al[SP];
#pragma unroll
        for (int q = 0; q < SP; ++q) { ah[q] = h3[2][q]; al[q] = l3[2][q]; }
        if (p.j0 + 2 < jend) rows_split_ff<SP>(p, sR, ht, a, b, p.j0 + 2, p.j0, rlo0, ah, al);   // complete
        const float2 w3 = __ldg(p.wff + 3);
        for (int s = 0; s < p.nsteps; ++s) {
            __syncthreads();                                                // X(s): D_{t-1} is in sD
            if (s_abort) return;
            const int t = p.j0 + s;
            if (s > 0) {                                                    // row t-1 as float pairs
                const double *dd = sD[(t - 1) & 1];
                float2 *row = p.ringf + (int64_t)(t - 1) * p.P;
                float2 *srow = sR + ((t - 1) % NR) * (LTS * SP);
#pragma unroll
                for (int q = 0; q < SP; ++q) {
                    const int i = a + ht + LTS * q;
                    if (i < b) {
                        const float2 f = d2ff(dd[ht + LTS * q]);
                        row[i] = f;
                        srow[ht + LTS * q] = f;
                        if (t + 2 < jend) ff_fma(ah[q], al[q], w3, f);
                    }
                }
            }
            if (t + 2 < jend) history_store_scaled_ff<SP>(ht, a, b, ah, al, sg, sS[t & 1]);
            carries(s);
            asm volatile("bar.arrive 2, %0;" ::"n"(2 * LTS) : "memory");      // (C): carries of step t
            if (t + 3 < jend) {
                float fh[1][SP], fl[1][SP];
#pragma unroll
                for (int q = 0; q < SP; ++q) { fh[0][q] = 0.f; fl[0][q] = 0.f; }
                far_fold_ff<SP, 1>(p, ht, a, b, t + 3, fh, fl);
#pragma unroll
                for (int q = 0; q < SP; ++q) { ah[q] = fh[0][q]; al[q] = fl[0][q]; }
                rows_split_ff<SP>(p, sR, ht, a, b, t + 3, t, max(0, t - NR), ah, al);
            }
        }
        return;
    }

    // ===================================================================== solver warps
    const int lane = tid & 31, warp = tid >> 5;
    const int i0 = a + tid * SP;
    const int i1 = min(i0 + SP, b);
    const int cnt = max(0, i1 - i0);
    double PF[5], PB[5], PeF, PeB;
    {
        const int64_t T = (int64_t)c * LTS + tid, GT = (int64_t)G * LTS;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            PF[k] = __ldg(p.sc.lane + k * GT + T);
            PB[k] = __ldg(p.sc.lane + (6 + k) * GT + T);
        }
        PeF = __ldg(p.sc.lane + 5 * GT + T);
        PeB = __ldg(p.sc.lane + 11 * GT + T);
    }
    const bool flux = p.rkind != FPDE_BC_DIRICHLET;
    const double mbc = __ldg(p.mb + c);
    double u[SP], kga[SP], kng[SP], kc1[SP], kc2[SP], kc3[SP], kal[SP], kcf[SP], kcb[SP], kCB[SP], kGG[SP];
    double rb1[SP], rb2[SP];
    double kxa[EXPL ? SP : 1], kxb[EXPL ? SP : 1];
    double dm1[SP];                                      // D_{t-1}
    double dm2[SP];                                      // D_{t-2} (prologue only)
#pragma unroll
    for (int k = 0; k < SP; ++k) {
        const bool in = k < cnt;
        const int i = in ? i0 + k : 0;
        u[k] = in ? p.U[i] : 0.0;
        kga[k] = in ? __ldg(p.ga + i) : 0.0;
        kng[k] = in ? __ldg(p.ng + i) : 0.0;
        kc1[k] = in ? __ldg(p.c1 + i) : 0.0;
        kc2[k] = in ? __ldg(p.c2 + i) : 0.0;
        kc3[k] = in ? __ldg(p.c3 + i) : 0.0;
        kal[k] = in ? __ldg(p.al + i) : 0.0;
        kcf[k] = in ? __ldg(p.cf + i) : 0.0;
        kcb[k] = in ? __ldg(p.cb + i) : 0.0;
        kCB[k] = in ? __ldg(p.CB + i) : 0.0;
        kGG[k] = in ? __ldg(p.GG + i) : 0.0;
        rb1[k] = in ? __ldg(p.RB1 + i) : 0.0;
        rb2[k] = in ? __ldg(p.RB2 + i) : 0.0;
        if constexpr (EXPL) {
            kxa[k] = in ? __ldg(p.xa + i) : 0.0;
            kxb[k] = in ? __ldg(p.xb + i) : 0.0;
        }
        dm1[k] = (in && p.j0 >= 1) ? p.ring[(int64_t)(p.j0 - 1) * p.P + i] : 0.0;
        dm2[k] = (in && p.j0 >= 2) ? p.ring[(int64_t)(p.j0 - 2) * p.P + i] : 0.0;
    }
    const bool ownsN = cnt > 0 && i1 == N;
    const bool last = cnt > 0 && i1 == b;                // owns the chunk's last node
    const double ry1 = last ? __ldg(p.RY1 + i1 - 1) : 0.0, ry2 = last ? __ldg(p.RY2 + i1 - 1) : 0.0;
    double uNv = ownsN ? p.U[N] : 0.0;
    const double lam = p.lam, w1 = __ldg(p.wlag + 1), w2 = __ldg(p.wlag + 2);

    double om[SP], yv[SP], ubw[SP];
    // chunk-local zero-carry sweeps of om: forward y (+ scans), backward ub (+ scans)
    auto sweeps = [&]() {
        double yl = 0.0;
#pragma unroll
        for (int k = 0; k < SP; ++k) {
            if (k < cnt) {
                if (i0 + k == 0) yl = p.g0;
                else yl = fma(kga[k], yl, om[k]);           // om holds -g Om
                yv[k] = yl;
            }
        }
        double X = cnt > 0 ? yl : 0.0;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const double Xp = __shfl_up_sync(FULL, X, 1 << k);
            if (lane >= (1 << k)) X = fma(PF[k], Xp, X);
        }
        double Xe = __shfl_up_sync(FULL, X, 1);
        if (lane == 0) Xe = 0.0;
        if (lane == 31) wXf[warp] = X;
        solver_sync();                                                      // (A)
        {
            double x0 = 0.0, x1 = 0.0;
#pragma unroll
            for (int w = 0; w < NWS; w += 2) {
                if (w < warp) x0 = fma(sCf[warp][w], wXf[w], x0);
                if (w + 1 < warp) x1 = fma(sCf[warp][w + 1], wXf[w + 1], x1);
            }
            const double carry = fma(PeF, x0 + x1, Xe);
#pragma unroll
            for (int k = 0; k < SP; ++k)
                if (k < cnt) yv[k] = fma(kcf[k], carry, yv[k]);
        }
        double ul = 0.0;
#pragma unroll
        for (int k = SP - 1; k >= 0; --k) {
            if (k < cnt) {
                ul = fma(kal[k], ul, yv[k]);
                ubw[k] = ul;
            }
        }
        X = cnt > 0 ? ul : 0.0;
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            const double Xn = __shfl_down_sync(FULL, X, 1 << k);
            if (lane + (1 << k) < 32) X = fma(PB[k], Xn, X);
        }
        Xe = __shfl_down_sync(FULL, X, 1);
        if (lane == 31) Xe = 0.0;
        if (lane == 0) wXb[warp] = X;
        solver_sync();                                                      // (B)
        {
            double x0 = 0.0, x1 = 0.0;
#pragma unroll
            for (int w = 0; w < NWS; w += 2) {
                if (w > warp) x0 = fma(sCb[warp][w], wXb[w], x0);
                if (w + 1 > warp) x1 = fma(sCb[warp][w + 1], wXb[w + 1], x1);
            }
            const double carry = fma(PeB, x0 + x1, Xe);
#pragma unroll
            for (int k = 0; k < SP; ++k)
                if (k < cnt) ubw[k] = fma(kcb[k], carry, ubw[k]);
        }
    };
    auto src_row = [&](int64_t n) -> const double * {
        return p.src ? p.src + (int64_t)(n < p.src_rows ? n : p.src_rows - 1) * (N + 1) : nullptr;
    };

    if constexpr (EXPL) {                                // edge states of the threads' segments
        sUf[tid] = cnt > 0 ? u[0] : 0.0;
        sUl[tid] = cnt > 0 ? last_of<SP>(u, cnt) : 0.0;
    }
    __syncthreads();                                                        // start: H_j0 ready
    // ---- prologue: step j0 from its full right-hand side
    {
        const double *src = src_row(p.n0);
        const double *hs = sS[p.j0 & 1];                 // -g H_j0
        double ul = 0.0, hr = 0.0;                       // explicit part: the neighbours of the segment
        if constexpr (EXPL) {
            if (cnt > 0) {
                ul = tid > 0 ? sUl[tid - 1] : (a > 0 ? p.U[a - 1] : 0.0);
                hr = i1 < b ? sUf[tid + 1] : (b < N ? p.U[b] : uNv);
            }
        }
#pragma unroll
        for (int k = 0; k < SP; ++k) {
            om[k] = 0.0;
            if (k < cnt) {
                double rest;
                if constexpr (EXPL) {
                    const int i = i0 + k;
                    const double un = k + 1 < cnt ? u[k + 1] : hr;
                    rest = (-(__ldg(p.lamv + i) * u[k]) + (src ? __ldg(src + i) : 0.0)) + fma(w1, dm1[k], w2 * dm2[k]);
                    rest -= fma(__ldg(p.eA + i), ul, __ldg(p.eB + i) * un);
                    ul = u[k];
                } else {
                    rest = (-(lam * u[k]) + (src ? __ldg(src + i0 + k) : 0.0)) + fma(w1, dm1[k], w2 * dm2[k]);
                }
                om[k] = fma(kng[k], rest, hs[i0 - a + k]);
            }
        }
        sweeps();
        double *agg = p.agg;
        if (ownsN && flux) st_relaxed_f64(agg + 2 * G, last_of<SP>(u, cnt));
        if (last) st_relaxed_f64(agg + 2 * c, last_of<SP>(yv, cnt));
        if (tid == 0) st_relaxed_f64(agg + 2 * c + 1, ubw[0]);
    }
    double ubc[SP], ubp[SP], ubprev[SP];                 // ub_t corrected, ub'_{t+1}, ub_{t-1}
#pragma unroll
    for (int k = 0; k < SP; ++k) { ubc[k] = ubw[k]; ubp[k] = 0.0; ubprev[k] = 0.0; }
    double ypl = 0.0;                                    // y'_{t+1} at the chunk's last node
    double cin = 0.0, ubv = 0.0;                         // carries of the last gathered step
    for (int s = 0; s < p.nsteps; ++s) {
        const int t = p.j0 + s;
        if (s > 0) {
            // ---- carries of step t-1: first step t's corrected aggregates (the chunk's last y,
            // first u; at a flux end the new U[N-1]) go out, then state u^t, increment D_{t-1}
            // and the corrected backward results
            double *agg = p.agg + (size_t)s * (2 * G + 2);
            if (last) st_relaxed_f64(agg + 2 * c, fma(ry2, ubv, fma(ry1, cin, ypl)));
            if (tid == 0) st_relaxed_f64(agg + 2 * c + 1, fma(rb2[0], ubv, fma(rb1[0], cin, ubp[0])));
            if (ownsN && flux)
                st_relaxed_f64(agg + 2 * G, fma(last_of<SP>(kCB, cnt), ubv,
                                                fma(last_of<SP>(kGG, cnt), cin, last_of<SP>(ubprev, cnt))));
            double *dsh = sD[(t - 1) & 1];
#pragma unroll
            for (int k = 0; k < SP; ++k) {
                if (k < cnt) {
                    const double un = fma(kCB[k], ubv, fma(kGG[k], cin, ubprev[k]));
                    const double d = un - u[k];
                    p.ring[(int64_t)(t - 1) * p.P + i0 + k] = d;
                    dsh[i0 - a + k] = d;
                    dm1[k] = d;
                    u[k] = un;
                    ubc[k] = fma(rb2[k], ubv, fma(rb1[k], cin, ubp[k]));
                }
            }
            if (ownsN) {
                const double UN = s_red[3];
                p.ring[(int64_t)(t - 1) * p.P + N] = UN - uNv;
                uNv = UN;
            }
        }
        if constexpr (EXPL) {                            // the segment's first and last ub_t
            sUf[tid] = cnt > 0 ? ubc[0] : 0.0;
            sUl[tid] = cnt > 0 ? last_of<SP>(ubc, cnt) : 0.0;
        }
        __syncthreads();                                                    // X(s)
        if (t + 1 < jend) {
            // ---- step t+1 on Omega0, while the aggregates of step t are exchanged
            const double *src = src_row(p.n0 + s + 1);
            const double *hs = sS[(t + 1) & 1];          // -g H_{t+1}
            if (src) {
#pragma unroll
                for (int k = 0; k < SP; ++k) {
                    om[k] = 0.0;
                    if (k < cnt) {
                        const double h = fma(kng[k], __ldg(src + i0 + k), fma(kc3[k], dm1[k], hs[i0 - a + k]));
                        om[k] = fma(kc1[k], ubc[k], fma(kc2[k], u[k], h));
                    }
                }
            } else {
#pragma unroll
                for (int k = 0; k < SP; ++k) {
                    om[k] = 0.0;
                    if (k < cnt) om[k] = fma(kc1[k], ubc[k], fma(kc2[k], u[k], fma(kc3[k], dm1[k], hs[i0 - a + k])));
                }
            }
            if constexpr (EXPL) {                        // neighbours' ub_t inside the chunk
                const double xl = (cnt > 0 && tid > 0) ? sUl[tid - 1] : 0.0;
                const double xr = (cnt > 0 && i1 < b) ? sUf[tid + 1] : 0.0;
#pragma unroll
                for (int k = 0; k < SP; ++k) {
                    if (k < cnt) {
                        const double ul = k > 0 ? ubc[k - 1] : xl;
                        const double ur = k + 1 < cnt ? ubc[k + 1] : xr;
                        om[k] = fma(kxa[k], ul, fma(kxb[k], ur, om[k]));
                    }
                }
            }
            sweeps();
            ypl = last ? last_of<SP>(yv, cnt) : 0.0;
#pragma unroll
            for (int k = 0; k < SP; ++k) ubp[k] = ubw[k];
        }
        asm volatile("bar.sync 2, %0;" ::"n"(2 * LTS) : "memory");         // (C): carries of step t
        if (s_abort) {
            if (s + 1 < p.nsteps) __syncthreads();      // release the history warps at X(s+1)
            return;
        }
        cin = s_red[0];
        ubv = fma(mbc, s_red[3], s_red[1] + s_red[2]);
#pragma unroll
        for (int k = 0; k < SP; ++k) ubprev[k] = ubc[k];
    }
    // ---- carries of the last step: the final state and increment (FP64 ring and float pairs)
    {
        const int64_t row = (int64_t)(jend - 1) * p.P;
#pragma unroll
        for (int k = 0; k < SP; ++k) {
            if (k < cnt) {
                const double un = fma(kCB[k], ubv, fma(kGG[k], cin, ubprev[k]));
                const double d = un - u[k];
                p.ring[row + i0 + k] = d;
                p.ringf[row + i0 + k] = d2ff(d);
                p.U[i0 + k] = un;
            }
        }
        if (ownsN) {
            const double UN = s_red[3];
            p.ring[row + N] = UN - uNv;
            p.U[N] = UN;
        }
    }
}

}  // namespace fpde

using namespace fpde;

struct fpde_line {
    fpde_ctx *ctx = nullptr;
    fpde_line_desc d{};
    int64_t N = 0, P = 0;
    int G = 1, s = 1, chunk = 0, max_steps = 0;
    int far_splits = 0, gemv_splits = 0;      // tuned values (0: built-in rules)
    int sbk = 4;                              // blocks per far super-block (three-slice path)
    int max_lag = INT_MAX;                    // restricted summing: lags above are dropped
    bool split = false;
    double lam = 0, lamR = 0, kkk0 = 0, AlN = 0;
    double *A = nullptr, *g = nullptr, *al = nullptr, *cf = nullptr, *cb = nullptr;
    double *CF = nullptr, *CB = nullptr, *GG = nullptr;
    // speculative block solve (split path): chunk-local responses of the sweeps
    double *RB1 = nullptr, *RB2 = nullptr, *RY1 = nullptr, *RY2 = nullptr;
    float2 *ringf = nullptr, *wff = nullptr;  // the ring and the lag weights as float pairs
    double *sga = nullptr, *sng = nullptr, *sc1 = nullptr, *sc2 = nullptr, *sc3 = nullptr;  // -g pre-scaling
    float2 *sngf = nullptr;
    double *sxa = nullptr, *sxb = nullptr;    // pre-scaled neighbour weights (explicit part)
    double *Lf = nullptr, *Mb = nullptr, *Kb = nullptr, *mb = nullptr;
    unsigned long long *cflag = nullptr, *seq = nullptr;
    double *sclane = nullptr, *scwarp = nullptr;
    double *U = nullptr, *D = nullptr, *part = nullptr, *wrev = nullptr;
    double *agg = nullptr;
    unsigned *barrier = nullptr;
    // optional: per-step source rows, explicit space part, per-node local weight
    double *srcd = nullptr, *lamv = nullptr, *eA = nullptr, *eB = nullptr;
    int src_rows = 0;
    // split path
    int64_t rows16 = 0, ld16 = 0;
    uint16_t *h_hi = nullptr, *h_lo = nullptr, *w_hi = nullptr, *w_lo = nullptr;
    double *ring = nullptr, *cfar = nullptr, *wlag = nullptr, *out_scale = nullptr;
    unsigned long long *slots = nullptr;
    int *exps = nullptr;
    FarPlan plan;
    // exact three-slice form
    bool x3 = false;
    uint16_t *h3[3] = {nullptr, nullptr, nullptr}, *w3[3] = {nullptr, nullptr, nullptr};
    int8_t *pA = nullptr;
    float *pW = nullptr;
    int64_t ldp = 0;
    FarPlan3 plan3;
    int64_t n_done = 0;
    int graph_min = GRAPH_MIN_STEPS;          // shortest run replayed from a graph
    // Richards problem (desc.richards): coefficients from the solution every step (rich_line.cu)
    bool rich = false;
    int rkform = 1;
    double rksat = 0.0;
    double *rZ = nullptr, *rdL = nullptr, *rA = nullptr, *rB = nullptr, *rR = nullptr, *rOm = nullptr,
           *ral = nullptr, *rbt = nullptr, *last = nullptr, *Sn = nullptr;
    std::vector<double> rE;
    // probes: CUDA events around kernels inside the captured graph
    struct Probe { int kind; int64_t n; double bytes, flops; int ev; int steps; };
    int probe_every = 0;
    std::vector<cudaEvent_t> probe_ev;
    std::vector<Probe> probes;                            // recorded by the last enqueue
    GraphCache<std::vector<Probe>> graphs;                // captured runs and their probe records
    std::vector<Probe> last_probes;
};

namespace fpde {

template <int SP>
static cudaError_t launch_solve_sp(const cudaLaunchConfig_t &cfg, const LineSolveArgs &a)
{
    return cudaLaunchKernelEx(&cfg, k_line_solve<SP>, a);
}

static int line_launch_solve(fpde_line *L, cudaStream_t st, int64_t n, const double *part, int KS, int64_t pstride,
                             double *Drow, int64_t dstride)
{
    LineSolveArgs a;
    a.A = L->A; a.g = L->g; a.al = L->al; a.cf = L->cf; a.cb = L->cb;
    a.src = L->srcd ? L->srcd + (n < L->src_rows ? n : L->src_rows - 1) * (L->N + 1) : nullptr;
    a.lamv = L->lamv; a.eA = L->eA; a.eB = L->eB;
    a.CF = L->CF; a.CB = L->CB; a.GG = L->GG;
    a.Lf = L->Lf; a.Mb = L->Mb; a.Kb = L->Kb; a.mb = L->mb; a.cflag = L->cflag; a.seq = L->seq;
    a.U = L->U; a.Drow = Drow; a.dstride = dstride; a.part = part; a.pstride = pstride;
    a.agg = L->agg;
    a.barrier = L->barrier; a.flags = L->ctx->d_flags;
    a.lam = L->lam; a.g0 = L->d.left_value; a.gN = L->d.right_value; a.dLN = L->d.dLN;
    a.AlN = L->AlN; a.KS = KS; a.N = (int)L->N; a.G = L->G; a.rkind = L->d.right_kind;
    a.chunk = L->chunk;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L->G);
    cfg.blockDim = dim3(LT);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = L->G > 1 ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e;
    switch (L->s) {
    case 1: e = launch_solve_sp<1>(cfg, a); break;
    case 2: e = launch_solve_sp<2>(cfg, a); break;
    case 4: e = launch_solve_sp<4>(cfg, a); break;
    default: e = launch_solve_sp<8>(cfg, a); break;
    }
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "line solve launch: %s", cudaGetErrorString(e));
    count_launches(1);
    return FPDE_OK;
}

static cudaEvent_t *probe_begin(fpde_line *L, int kind, int64_t n, double bytes, double flops, int steps = 1)
{
    const size_t k = L->probes.size();
    if (2 * (k + 1) > L->probe_ev.size()) return nullptr;
    L->probes.push_back({kind, n, bytes, flops, (int)(2 * k), steps});
    return &L->probe_ev[2 * k];
}

// Opt the speculative kernels in to their dynamic shared memory (the row ring) on this device.
static cudaError_t spec_smem_attrs()
{
    cudaError_t e = cudaSuccess;
    auto opt = [&e](const void *fn, size_t bytes) {
        if (e == cudaSuccess) e = smem_opt_in(fn, (int)bytes);
    };
    opt((const void *)k_line_block_spec<1, false>, SpecRing<1>::bytes);
    opt((const void *)k_line_block_spec<2, false>, SpecRing<2>::bytes);
    opt((const void *)k_line_block_spec<4, false>, SpecRing<4>::bytes);
    opt((const void *)k_line_block_spec<8, false>, SpecRing<8>::bytes);
    opt((const void *)k_line_block_spec<1, true>, SpecRing<1>::bytes);
    opt((const void *)k_line_block_spec<2, true>, SpecRing<2>::bytes);
    opt((const void *)k_line_block_spec<4, true>, SpecRing<4>::bytes);
    opt((const void *)k_line_block_spec<8, true>, SpecRing<8>::bytes);
    return e;
}

template <int SP>
static cudaError_t launch_block_sp(cudaLaunchConfig_t cfg, const LineBlockArgs &a)
{
    cfg.dynamicSmemBytes = SpecRing<SP>::bytes;     // both keep the newest rows in shared memory
    return a.xa ? cudaLaunchKernelEx(&cfg, k_line_block_spec<SP, true>, a)
                : cudaLaunchKernelEx(&cfg, k_line_block_spec<SP, false>, a);
}

// Steps j0 .. j0+nsteps-1 of the block starting at nb0 in one persistent launch.
static int line_launch_block(fpde_line *L, cudaStream_t st, int64_t nb0, int j0, int nsteps, int KS, int far_ld,
                             int far_row0)
{
    LineBlockArgs a;
    a.A = L->A; a.g = L->g; a.al = L->al; a.cf = L->cf; a.cb = L->cb; a.CB = L->CB; a.GG = L->GG;
    a.lamv = L->lamv; a.eA = L->eA; a.eB = L->eB;
    a.src = L->srcd; a.src_rows = L->src_rows;
    a.U = L->U; a.ring = L->ring; a.cfar = L->cfar; a.KS = KS; a.P = L->P; a.wlag = L->wlag;
    a.far_ld = far_ld; a.far_row0 = far_row0;
    a.far_pairs = L->x3 ? 1 : 0;
    a.agg = L->agg; a.cflag = L->cflag; a.seq = L->seq;
    a.Lf = L->Lf; a.Mb = L->Mb; a.Kb = L->Kb; a.mb = L->mb; a.flags = L->ctx->d_flags;
    a.sc.lane = L->sclane; a.sc.warp = L->scwarp;
    a.RB1 = L->RB1; a.RB2 = L->RB2; a.RY1 = L->RY1; a.RY2 = L->RY2;
    a.ringf = L->ringf; a.wff = L->wff;
    a.ga = L->sga; a.ng = L->sng; a.c1 = L->sc1; a.c2 = L->sc2; a.c3 = L->sc3; a.ngf = L->sngf;
    a.xa = L->sxa; a.xb = L->sxb;
    a.lam = L->lam; a.g0 = L->d.left_value; a.gN = L->d.right_value; a.dLN = L->d.dLN; a.AlN = L->AlN;
    a.n0 = nb0 + j0; a.j0 = j0; a.nsteps = nsteps; a.N = (int)L->N; a.G = L->G; a.rkind = L->d.right_kind;
    a.chunk = L->chunk;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L->G);
    cfg.blockDim = dim3(2 * LTS);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = L->G > 1 ? 1 : 0;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    // the launch's exchange slots start as SLOT_EMPTY (all bits set)
    FPDE_CUDA(cudaMemsetAsync(L->agg, 0xFF, (size_t)nsteps * (2 * L->G + 2) * sizeof(double), st));
    cudaError_t e;
    switch (L->s) {
    case 1: e = launch_block_sp<1>(cfg, a); break;
    case 2: e = launch_block_sp<2>(cfg, a); break;
    case 4: e = launch_block_sp<4>(cfg, a); break;
    default: e = launch_block_sp<8>(cfg, a); break;
    }
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "line block launch: %s", cudaGetErrorString(e));
    count_launches(1);
    return FPDE_OK;
}

#define PROBE_REC(ev, i) \
    do { if (ev) FPDE_CUDA(record_probe_event((ev)[i], st)); } while (0)

// One Richards step (rich_line.cu): coefficients from the current state, then the solve.
static int rich_step(fpde_line *L, cudaStream_t st, int64_t n, const double *part, int KS)
{
    RichLineArgs a;
    a.U = L->U; a.Z = L->rZ; a.dL = L->rdL;
    a.part = part; a.KS = KS; a.pstride = L->P;
    a.src = L->srcd ? L->srcd + (n < L->src_rows ? n : L->src_rows - 1) * (L->N + 1) : nullptr;
    a.cA = L->rA; a.cB = L->rB; a.cR = L->rR; a.cOm = L->rOm; a.al = L->ral; a.bt = L->rbt;
    a.lam = L->lam; a.lamR = L->lamR; a.ksat = L->rksat; a.kform = L->rkform;
    a.E = L->rE[(size_t)std::min<int64_t>(n, (int64_t)L->rE.size() - 1)];
    a.N = (int)L->N; a.rkind = L->d.right_kind; a.gN = L->d.right_value; a.dLN = L->d.dLN;
    return launch_rich_line_step(st, a);
}

// Enqueue steps [n0, n0+steps) on st; returns the number of kernels enqueued via *nk.
static int line_enqueue(fpde_line *L, cudaStream_t st, int64_t n0, int steps, int64_t *nk)
{
    int64_t k = 0;
    int rc;
    L->probes.clear();
    const int64_t nodes_hist = L->N + 1;
    for (int64_t n = n0; n < n0 + steps; ++n) {
        const bool probe_step = L->probe_every > 0 && n >= 1 && (n % L->probe_every) == L->probe_every - 1;
        cudaEvent_t *ev;
        if (!L->split) {
            int KS = 0;
            const int64_t t0 = n > L->max_lag ? n - L->max_lag : 0;   // oldest row of the window
            const int64_t nr = n - t0;
            if (nr >= 1) {
                KS = L->gemv_splits > 0 ? std::max(1, std::min<int>(L->gemv_splits, (int)std::min<int64_t>(nr, KS_MAX)))
                                        : choose_splits((int)nr, L->P);
                const double *wt = L->wrev + (L->max_steps - n);   // wt[t] = w[n - t]
                ev = probe_step ? probe_begin(L, 0, n, 8.0 * (double)nr * nodes_hist, 2.0 * nr * nodes_hist) : nullptr;
                PROBE_REC(ev, 0);
                if ((rc = launch_l1_partial(st, L->D + t0 * L->P, L->P, (int)nr, wt + t0, L->part, KS))) return rc;
                PROBE_REC(ev, 1);
                ++k;
            }
            ev = probe_step ? probe_begin(L, 2, n, 0.0, 0.0) : nullptr;
            PROBE_REC(ev, 0);
            if (L->rich) {                             // coefficients from the solution, then the increment
                if ((rc = rich_step(L, st, n, L->part, KS))) return rc;
                if ((rc = launch_append(st, L->U, L->last, L->D + n * L->P, L->N + 1, L->P))) return rc;
                k += 2;
            } else if ((rc = line_launch_solve(L, st, n, L->part, KS, L->P, L->D + n * L->P, 1))) {
                return rc;
            }
            PROBE_REC(ev, 1);
            ++k;
        } else {
            const int64_t nb0 = n - n % BLK;                     // block start
            const int j = (int)(n - nb0);
            // far history columns [kb0, nb0): the 64-step tiles the window reaches (lags up to
            // max_lag from step nb0 go back to column nb0 - max_lag)
            const int64_t kb0 = nb0 > L->max_lag ? (nb0 - L->max_lag) / 64 * 64 : 0;
            const int far_kt = (int)((nb0 - kb0) / 64);
            int splits = 0, far_ld = BLK, far_row0 = 0;
            if (far_kt > 0 && !L->x3)
                splits = L->far_splits > 0 ? std::min(L->far_splits, far_kt) : far_splits(far_kt, L->rows16);
            if (L->x3) {
                // Two-level blocking: super-blocks of sbk blocks starting at s0. The history older
                // than s0 is contracted once for all sbk*64 steps of the super-block (the "super"
                // partials, splits 0..sup-1, rows [0, sbk*64) of every split); each block adds the
                // contraction over the super-block's own older blocks [s0, nb0) (the "near-far"
                // partial in split slot sup, rows of this block). Both are pure functions of s0
                // and nb0, so a run may start at any block.
                const int sbk = L->sbk;
                const int m = (int)((nb0 / BLK) % sbk);
                const int64_t s0 = nb0 - (int64_t)BLK * m;
                const int64_t kbs = s0 > L->max_lag ? (s0 - L->max_lag) / 64 * 64 : 0;
                const int sup_kt = (int)((s0 - kbs) / 64);
                const int sup = sup_kt > 0 ? std::min(FAR_MAX_SPLITS - 1,
                                                      L->far_splits > 0 ? std::min(L->far_splits, sup_kt)
                                                                        : far_splits(sup_kt, L->rows16 * sbk))
                                           : 0;
                const int64_t kn0 = std::max(s0, kb0);
                const int near_kt = (int)((nb0 - kn0) / 64);
                splits = sup + (near_kt > 0 ? 1 : 0);
                far_ld = BLK * sbk;
                far_row0 = BLK * m;
                if (j == 0 && (nb0 > 0 || sbk > 1)) {
                    // convert the finished block; at a super-block start also the weight slices of
                    // all its steps (the first super-block's later blocks need them too)
                    SplitPrep3 sp;
                    sp.ring = L->ring; sp.P = L->P; sp.nvalid = nodes_hist; sp.ld = L->ld16; sp.wlag = L->wlag;
                    for (int q = 0; q < 3; ++q) { sp.hist[q] = L->h3[q]; sp.w[q] = L->w3[q]; }
                    sp.pA = L->pA; sp.pW = L->pW; sp.ldp = L->ldp; sp.n_grp = sbk;
                    if ((rc = launch_block_prep3(st, sp, nb0, m == 0))) return rc;
                    k += (nb0 > 0 ? 1 : 0) + (m == 0 ? 1 : 0);
                    if (m == 0 && sup_kt > 0) {
                        ev = L->probe_every > 0
                                 ? probe_begin(L, 1, nb0, 6.0 * (double)(s0 - kbs) * nodes_hist,
                                               6.0 * 2.0 * (double)nodes_hist * (s0 - kbs) * BLK * sbk)
                                 : nullptr;
                        PROBE_REC(ev, 0);
                        if ((rc = far3_launch(st, &L->plan3, (int)s0, L->cfar, (int64_t)far_ld * L->P, L->P, sup,
                                              L->pA, L->pW, L->ldp, L->ctx->d_flags, nullptr, (int)kbs, sbk, 0)))
                            return rc;
                        PROBE_REC(ev, 1);
                        ++k;
                    }
                    if (near_kt > 0) {
                        ev = L->probe_every > 0 ? probe_begin(L, 3, nb0, 6.0 * (double)(nb0 - kn0) * nodes_hist,
                                                              6.0 * 2.0 * (double)nodes_hist * (nb0 - kn0) * BLK)
                                                : nullptr;
                        PROBE_REC(ev, 0);
                        if ((rc = far3_launch(st, &L->plan3, (int)nb0, L->cfar + ((int64_t)sup * far_ld + far_row0) * L->P,
                                              (int64_t)far_ld * L->P, L->P, 1, L->pA, L->pW, L->ldp, L->ctx->d_flags,
                                              nullptr, (int)kn0, 1, m)))
                            return rc;
                        PROBE_REC(ev, 1);
                        ++k;
                    }
                }
            } else if (j == 0 && nb0 > 0) {
                SplitPrep sp;
                sp.ring = L->ring; sp.P = L->P; sp.nvalid = nodes_hist; sp.slots = L->slots; sp.exps = L->exps;
                sp.hist_hi = L->h_hi; sp.hist_lo = L->h_lo; sp.w_hi = L->w_hi; sp.w_lo = L->w_lo; sp.ld = L->ld16;
                sp.wlag = L->wlag; sp.out_scale = L->out_scale;
                sp.bf16 = L->d.precision == FPDE_PREC_SPLIT_BF16 ? 1 : 0;
                if ((rc = launch_block_prep(st, sp, nb0))) return rc;
                k += sp.bf16 ? 2 : 3;
                ev = L->probe_every > 0 ? probe_begin(L, 1, nb0, 4.0 * (double)nb0 * nodes_hist,
                                                      3.0 * 2.0 * (double)nodes_hist * nb0 * BLK)
                                        : nullptr;
                PROBE_REC(ev, 0);
                if ((rc = far_launch(st, &L->plan, (int)nb0, L->cfar, (int64_t)BLK * L->P, L->P, splits, 1.0,
                                     L->out_scale, L->ctx->d_flags)))
                    return rc;
                PROBE_REC(ev, 1);
                ++k;
            }
            const int nst = (int)std::min<int64_t>(BLK - j, n0 + steps - n);
            if (L->rich) {
                // per step: far partials + the block's earlier rows (float-float), the solve with
                // coefficients from the solution, the increment into the ring
                for (int q = j; q < j + nst; ++q) {
                    const int64_t m = nb0 + q;
                    int KSn = 0;
                    if (m >= 1) {
                        if ((rc = launch_near_history_ff(st, L->ringf, L->P, q, L->wff, L->cfar, splits, 1, L->Sn)))
                            return rc;
                        KSn = 1;
                        ++k;
                    }
                    if ((rc = rich_step(L, st, m, L->Sn, KSn))) return rc;
                    if ((rc = launch_append_ff(st, L->U, L->last, L->ring + (int64_t)q * L->P,
                                               L->ringf + (int64_t)q * L->P, L->N + 1, L->P)))
                        return rc;
                    k += 3;
                }
                n += nst - 1;
                continue;
            }
            // the rest of this block (or of the requested range) in one persistent launch
            double bytes = 0.0, flops = 0.0;
            for (int q = j; q < j + nst; ++q) {                  // far fold + near ring + state
                bytes += 8.0 * nodes_hist * (splits + q + 2);
                flops += (double)nodes_hist * (splits + 2.0 * q + 30.0);
            }
            ev = L->probe_every > 0 ? probe_begin(L, 2, n, bytes, flops, nst) : nullptr;
            PROBE_REC(ev, 0);
            if ((rc = line_launch_block(L, st, nb0, j, nst, splits, far_ld, far_row0))) return rc;
            PROBE_REC(ev, 1);
            ++k;
            n += nst - 1;
        }
    }
    if (nk) *nk = k;
    return FPDE_OK;
}

}  // namespace fpde

extern "C" {

int fpde_line_coefs(int64_t N, const double *k, const double *iw, const double *dL, double *A, double *B,
                    double *Rlap)
{
    FPDE_CHECK_ARG(N >= 2 && k && dL && A && B && Rlap, "bad arguments");
    for (int64_t i = 1; i < N; ++i) {
        const double w = iw ? iw[i] : 1.0;
        A[i] = k[i - 1] * w / (dL[i] * dL[i - 1]);
        B[i] = k[i] * w / (dL[i] * dL[i]);
        Rlap[i] = w * ((k[i] / (dL[i] * dL[i])) + (k[i - 1] / (dL[i] * dL[i - 1])));
    }
    return FPDE_OK;
}

int fpde_line_destroy(fpde_line *L)
{
    if (!L) return FPDE_OK;
    if (L->ctx) {
        cudaSetDevice(L->ctx->device);
        cudaStreamSynchronize(L->ctx->stream);
        L->ctx->lines.erase(L);
    }
    L->graphs.clear();
    for (cudaEvent_t e : L->probe_ev) cudaEventDestroy(e);
    dev_free(L->cflag);
    dev_free(L->seq);
    dev_free(L->sclane);
    dev_free(L->scwarp);
    for (double *p : {L->A, L->g, L->al, L->cf, L->cb, L->CF, L->CB, L->GG, L->Lf, L->Mb, L->Kb, L->mb, L->U, L->D,
                      L->part, L->wrev, L->agg, L->ring, L->cfar, L->wlag, L->out_scale, L->srcd, L->lamv, L->eA,
                      L->eB, L->RB1, L->RB2, L->RY1, L->RY2})
        dev_free(p);
    dev_free(L->ringf);
    dev_free(L->wff);
    for (double *q : {L->sga, L->sng, L->sc1, L->sc2, L->sc3}) dev_free(q);
    dev_free(L->sngf);
    dev_free(L->sxa);
    dev_free(L->sxb);
    for (uint16_t *p : {L->h_hi, L->h_lo, L->w_hi, L->w_lo, L->h3[0], L->h3[1], L->h3[2], L->w3[0], L->w3[1],
                        L->w3[2]})
        dev_free(p);
    dev_free(L->pA);
    dev_free(L->pW);
    dev_free(L->slots);
    dev_free(L->exps);
    dev_free(L->barrier);
    for (double *p : {L->rZ, L->rdL, L->rA, L->rB, L->rR, L->rOm, L->ral, L->rbt, L->last, L->Sn}) dev_free(p);
    delete L;
    return FPDE_OK;
}

int fpde_line_create(fpde_ctx *ctx, const fpde_line_desc *desc, const double *A, const double *B,
                     const double *Rlap, const double *u0, fpde_line **out)
{
    clear_error();
    FPDE_CHECK_ARG(out && desc && u0, "null argument");
    *out = nullptr;
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    const fpde_line_desc &d = *desc;
    FPDE_CHECK_ARG(d.N >= 2, "N must be >= 2");
    const fpde_richards *rich = d.richards;
    std::vector<double> placeholder;
    if (rich) {
        FPDE_CHECK_ARG(rich->k_form == 1 || rich->k_form == 2, "richards: k_form must be 1 or 2");
        FPDE_CHECK_ARG(rich->k_sat > 0.0 && std::isfinite(rich->k_sat), "richards: k_sat must be positive");
        FPDE_CHECK_ARG(rich->sZ && rich->dL[0], "richards: node coordinates (sZ) and steps (dL[0]) required");
        FPDE_CHECK_ARG(rich->evaporation && rich->evaporation_rows >= 1, "richards: evaporation rows required");
        FPDE_CHECK_ARG(!rich->salt_c0, "richards: the salt concentration is a 3D LOD option");
        FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64 || d.precision == FPDE_PREC_SPLIT_BF16X3,
                       "richards: FP64 or the exact three-slice split");
        FPDE_CHECK_ARG(!d.lag_weights && d.theta == 0.0 && d.restrict_eps == 0.0,
                       "richards: Caputo weights, no explicit part, no restricted summing");
        if (!A || !B || !Rlap) {       // time-invariant data of the linear solves: unused, kept regular
            placeholder.assign(3 * (size_t)(d.N + 1), 1.0);
            for (int64_t i = 0; i <= d.N; ++i) placeholder[2 * (d.N + 1) + i] = 2.0;
            A = placeholder.data();
            B = A + d.N + 1;
            Rlap = B + d.N + 1;
        }
    }
    FPDE_CHECK_ARG(A && B && Rlap, "null coefficient arrays");
    FPDE_CHECK_ARG(d.lag_weights || (d.alpha > 0.0 && d.alpha < 1.0), "alpha must be in (0, 1)");
    FPDE_CHECK_ARG(!d.source || d.source_rows >= 1, "source needs source_rows >= 1");
    FPDE_CHECK_ARG(std::isfinite(d.theta), "theta must be finite");
    FPDE_CHECK_ARG(d.tau > 0.0, "tau must be positive");
    FPDE_CHECK_ARG(d.max_steps > 0, "max_steps must be positive");
    FPDE_CHECK_ARG(d.left_kind == 0 || d.left_kind == 1, "bad left boundary kind");
    FPDE_CHECK_ARG(d.right_kind == 0 || d.right_kind == 1, "bad right boundary kind");
    FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64 || d.precision == FPDE_PREC_SPLIT_BF16 ||
                   d.precision == FPDE_PREC_SPLIT_F16 || d.precision == FPDE_PREC_SPLIT_BF16X3,
                   "bad precision mode");
    FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64 || d.block == 0 || d.block == BLK,
                   "split path: block must be 0 (auto) or 64");
    FPDE_CHECK_ARG(std::isfinite(d.restrict_eps) && d.restrict_eps >= 0.0, "restrict_eps must be >= 0");
    if (d.restrict_eps > 0.0 && (d.precision == FPDE_PREC_SPLIT_BF16 || d.precision == FPDE_PREC_SPLIT_F16))
        return set_error(FPDE_ERR_UNSUPPORTED, "restricted summing runs on the FP64 and the three-slice split paths");
    const int64_t N = d.N;
    // partition of nodes 0..N-1 into G chunks (CTAs) of lt threads x sp nodes (sp a power of
    // two; lt = LT for the per-step FP64 solve, LTS solver threads for the persistent split
    // path): one CTA when the line fits in 8 nodes per thread, otherwise the smallest sp that
    // keeps G within the SM count
    const bool split = d.precision != FPDE_PREC_FP64;
    const int lt = split ? LTS : LT;
    const fpde_line_tuning *tu = d.tuning;
    int sp = 1, G = 1;
    int64_t chunk;
    if (tu && (tu->solve_sp > 0 || tu->chunks > 0)) {
        // tuned partition: sp nodes per thread, `chunks` CTAs (or the fewest that fit)
        sp = tu->solve_sp > 0 ? tu->solve_sp : LSEG;
        FPDE_CHECK_ARG(sp == 1 || sp == 2 || sp == 4 || sp == 8, "tuning: solve_sp must be 1, 2, 4 or 8");
        const int64_t gmin = (N + (int64_t)lt * sp - 1) / ((int64_t)lt * sp);
        G = tu->chunks > 0 ? tu->chunks : (int)gmin;
        FPDE_CHECK_ARG(G >= gmin && G <= ctx->sm_count, "tuning: chunks out of range for this line and solve_sp");
        chunk = (N + G - 1) / G;
        chunk = (chunk + sp - 1) / sp * sp;
        G = (int)((N + chunk - 1) / chunk);
    } else {
        if (N <= (int64_t)lt * LSEG) {
            while ((int64_t)lt * sp < N) sp <<= 1;
        } else {
            while (sp <= LSEG && (N + (int64_t)lt * sp - 1) / ((int64_t)lt * sp) > ctx->sm_count) sp <<= 1;
            if (sp > LSEG)
                return set_error(FPDE_ERR_UNSUPPORTED, "line of %lld intervals exceeds %lld (SMs x %d x %d)",
                                 (long long)N, (long long)ctx->sm_count * lt * LSEG, lt, LSEG);
            G = (int)((N + (int64_t)lt * sp - 1) / ((int64_t)lt * sp));
        }
        // chunk of nodes per CTA: lt * sp, or (long lines) an even share of all SMs, rounded to sp
        chunk = (int64_t)lt * sp;
        if (G > 1 && N >= (int64_t)ctx->sm_count * lt) {
            chunk = (N + ctx->sm_count - 1) / ctx->sm_count;
            chunk = (chunk + sp - 1) / sp * sp;
            G = (int)((N + chunk - 1) / chunk);
        }
    }
    if (G > 160) return set_error(FPDE_ERR_UNSUPPORTED, "line solve: at most 160 chunks");
    int per_sm = 0;
    if (split) {
        int per_sm2 = 0;
        FPDE_CUDA(spec_smem_attrs());
        FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_line_block_spec<LSEG, false>, 2 * LTS,
                                                                SpecRing<LSEG>::bytes));
        FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm2, k_line_block_spec<LSEG, true>, 2 * LTS,
                                                                SpecRing<LSEG>::bytes));
        per_sm = std::min(per_sm, per_sm2);
    }
    else FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_line_solve<LSEG>, LT, 0));
    if (G > 1 && G > per_sm * ctx->sm_count)
        return set_error(FPDE_ERR_UNSUPPORTED, "line solve grid of %d CTAs cannot be co-resident", G);

    fpde_line *L = new fpde_line();
    L->ctx = ctx;
    L->d = d;
    L->N = N;
    L->P = (N + 1 + 511) / 512 * 512;
    L->G = G;
    L->s = sp;
    L->chunk = (int)chunk;
    if (tu) {
        L->far_splits = std::min(std::max(tu->far_splits, 0), FAR_MAX_SPLITS - 1);
        L->gemv_splits = std::min(std::max(tu->gemv_splits, 0), KS_MAX);
        if (tu->far_super > 0) L->sbk = std::min(tu->far_super, FAR_MAX_SUPER);
    }
    L->d.tuning = nullptr;                     // not kept
    if (rich) L->sbk = 1;                      // per-block far history; the near history per step
    L->max_steps = d.max_steps;
    L->split = split;
    L->x3 = d.precision == FPDE_PREC_SPLIT_BF16X3;
    // local weight kkk0 = tau^{1-alpha}/(1-alpha); lam as in Om1 (:4191), lamR as in R (:3120);
    // or the caller's lag weights (distributed order: w[0] = b0/tau of eq_init, fr_do.cpp:688-694)
    if (d.lag_weights) {
        L->kkk0 = 0.0;
        L->lam = L->lamR = d.lag_weights[0];
    } else {
        L->kkk0 = l1_interval_weight(d.alpha, 0.0, d.tau);
        L->lam = d.Da * (L->kkk0 / d.tau);
        L->lamR = d.Da * L->kkk0 / d.tau;
    }

    // time-invariant Thomas data (host, FP64)
    std::vector<double> Al(N + 2, 0.0), hA(N, 0.0), hg(N, 0.0), hal(N, 0.0), hp(N, 0.0), hcf(N), hcb(N);
    Al[1] = d.left_kind == FPDE_BC_FLUX ? 1.0 : 0.0;
    for (int64_t i = 1; i < N; ++i) Al[i + 1] = B[i] / ((Rlap[i] + L->lamR) - A[i] * Al[i]);
    L->AlN = Al[N];
    for (int64_t i = 0; i < N; ++i) {
        hal[i] = Al[i + 1];
        if (i >= 1) {
            hA[i] = A[i];
            hg[i] = Al[i + 1] / B[i];
            hp[i] = hg[i] * A[i];
        }
    }
    for (int64_t t0 = 0; t0 < N; t0 += sp) {                     // per-thread segments
        int64_t t1 = t0 + sp < N ? t0 + sp : N;
        double pr = 1.0;
        for (int64_t i = t0; i < t1; ++i) { pr *= hp[i]; hcf[i] = pr; }
        pr = 1.0;
        for (int64_t i = t1 - 1; i >= t0; --i) { pr *= hal[i]; hcb[i] = pr; }
    }
    // per chunk (CTA): forward prefix products CF, backward suffix products CB and the
    // backward sweep GG of CF, so that u = u^cta + c_in GG + u_b CB
    std::vector<double> hCF(N), hCB(N), hGG(N), hPend(G), hG0(G), hB0(G);
    for (int cc = 0; cc < G; ++cc) {
        const int64_t a0 = (int64_t)cc * chunk, b0 = std::min<int64_t>(a0 + chunk, N);
        double pr = 1.0;
        for (int64_t i = a0; i < b0; ++i) { pr *= hp[i]; hCF[i] = pr; }
        double cbv = 1.0, gg = 0.0;
        for (int64_t i = b0 - 1; i >= a0; --i) {
            cbv *= hal[i];
            hCB[i] = cbv;
            gg = hal[i] * gg + hCF[i];
            hGG[i] = gg;
        }
        hPend[cc] = hCF[b0 - 1];
        hG0[cc] = hGG[a0];
        hB0[cc] = hCB[a0];
    }
    // chunk-level carries as dot products with the chunks' published values Y (last y) and
    // U0 (first u):  c_in(c) = sum_r Lf[c][r] Y[r]        (c_in(G) = y at node N-1)
    //                u_b(c)  = sum_q Mb[c][q] U0[q] + sum_r Kb[c][r] Y[r] + mb[c] U_N
    std::vector<double> hLf((size_t)(G + 1) * G, 0.0), hMb((size_t)G * G, 0.0), hKb((size_t)G * G, 0.0), hmb(G);
    for (int q = 1; q <= G; ++q) {
        double pr = 1.0;
        for (int r = q - 1; r >= 0; --r) { hLf[(size_t)q * G + r] = pr; pr *= hPend[r]; }
    }
    for (int cc = 0; cc < G; ++cc) {
        double pr = 1.0;
        for (int q = cc + 1; q < G; ++q) { hMb[(size_t)cc * G + q] = pr; pr *= hB0[q]; }
        hmb[cc] = pr;
        for (int q = cc + 1; q < G; ++q) {
            const double f = hMb[(size_t)cc * G + q] * hG0[q];
            for (int r = 0; r < q; ++r) hKb[(size_t)cc * G + r] += f * hLf[(size_t)q * G + r];
        }
    }
    // scan coefficients of the persistent split-path kernel (all products are time-invariant):
    // per thread the products of its segment (forward P, backward Q); per lane the products
    // the five warp-scan levels multiply with and the exclusive prefix/suffix products; per
    // CTA the cross-warp coefficients of the solver warps.
    const int64_t GT = (int64_t)G * LTS;
    std::vector<double> hsl, hsw;
    if (split) {
        hsl.assign((size_t)12 * GT, 1.0);
        hsw.assign((size_t)G * 2 * NWS * NWS, 0.0);
        for (int cc = 0; cc < G; ++cc) {
            double Pt[LTS], Qt[LTS];
            const int64_t a0 = (int64_t)cc * chunk, b0 = std::min<int64_t>(a0 + chunk, N);
            for (int t = 0; t < LTS; ++t) {
                const int64_t i0 = std::min<int64_t>(a0 + (int64_t)t * sp, b0), i1 = std::min<int64_t>(i0 + sp, b0);
                Pt[t] = i1 > i0 ? hcf[i1 - 1] : 1.0;
                Qt[t] = i1 > i0 ? hcb[i0] : 1.0;
            }
            double PW[NWS], QW[NWS];
            for (int w = 0; w < NWS; ++w) {
                const double *pw = Pt + 32 * w, *qw = Qt + 32 * w;
                for (int l = 0; l < 32; ++l) {
                    const int64_t T = (int64_t)cc * LTS + 32 * w + l;
                    for (int k = 0; k < 5; ++k) {
                        double pf = 1.0, pb = 1.0;
                        for (int m = std::max(0, l - (1 << k) + 1); m <= l; ++m) pf *= pw[m];
                        for (int m = l; m <= std::min(31, l + (1 << k) - 1); ++m) pb *= qw[m];
                        hsl[(size_t)k * GT + T] = pf;
                        hsl[(size_t)(6 + k) * GT + T] = pb;
                    }
                    double pe = 1.0, qe = 1.0;
                    for (int m = 0; m < l; ++m) pe *= pw[m];
                    for (int m = l + 1; m < 32; ++m) qe *= qw[m];
                    hsl[(size_t)5 * GT + T] = pe;
                    hsl[(size_t)11 * GT + T] = qe;
                }
                double pt = 1.0, qt = 1.0;
                for (int l = 0; l < 32; ++l) { pt *= pw[l]; qt *= qw[l]; }
                PW[w] = pt;
                QW[w] = qt;
            }
            double *wc = hsw.data() + (size_t)cc * 2 * NWS * NWS;
            for (int w = 0; w < NWS; ++w) {
                for (int v = 0; v < w; ++v) {             // Cf[w][v] = prod_{v < x < w} PW[x]
                    double pr = 1.0;
                    for (int x = v + 1; x < w; ++x) pr *= PW[x];
                    wc[w * NWS + v] = pr;
                }
                for (int v = w + 1; v < NWS; ++v) {       // Cb[w][v] = prod_{w < x < v} QW[x]
                    double pr = 1.0;
                    for (int x = w + 1; x < v; ++x) pr *= QW[x];
                    wc[NWS * NWS + w * NWS + v] = pr;
                }
            }
        }
    }
    // lag weights w[j] = Da * kb(lag j) / tau with kb(lag j) = kkk0 * b_j; wrev[m] = w[L - m]
    const int64_t LW = L->max_steps + (int64_t)BLK * FAR_MAX_SUPER + 1;
    std::vector<double> wlag(LW, 0.0);
    for (int64_t j = 1; j < LW; ++j)
        wlag[j] = d.lag_weights ? (j <= L->max_steps ? d.lag_weights[j] : 0.0)
                                : d.Da * (L->kkk0 * l1_lag(d.alpha, j)) / d.tau;
    // restricted summing (time_summing :4117-4131, newest first): the history stops before the
    // first lag whose kb = w tau / Da falls below restrict_eps; later lags get weight 0
    if (d.restrict_eps > 0.0) {
        std::vector<double> kbl(L->max_steps);
        for (int64_t j = 1; j <= L->max_steps; ++j) kbl[j - 1] = wlag[j] * d.tau / d.Da;
        int keep = 0;
        fpde_restricted_lags(kbl.data(), L->max_steps, d.restrict_eps, &keep);
        if (keep < L->max_steps) {
            L->max_lag = keep;
            for (int64_t q = keep + 1; q < LW; ++q) wlag[q] = 0.0;
        }
    }
    std::vector<double> wrev(L->max_steps + 1, 0.0);
    for (int64_t m = 0; m < L->max_steps; ++m) wrev[m] = wlag[L->max_steps - m];
    // Speculative block solve (split path): step n+1's right-hand side is affine in step n's
    // chunk carries (c_in, u_b) through E1 and E2 (without an explicit part (w1 - lam) GG and
    // (w1 - lam) CB); the chunk-local zero-carry sweeps of E1, E2 (forward y -> RY, backward
    // u -> RB) are time-invariant.
    std::vector<double> hRB1, hRB2, hRY1, hRY2, hklam, hXA, hXB, hfold;
    std::vector<float2> hwff;
    if (split) {                                   // w = hi + lo, hi the nearest float
        hwff.resize(LW);
        for (int64_t j = 0; j < LW; ++j) {
            const float hi = (float)wlag[j];
            hwff[j] = make_float2(hi, (float)(wlag[j] - (double)hi));
        }
    }
    if (split) {
        // E1, E2: Omega0's coefficients on the carries (c_in, u_b) of the step before. With an
        // explicit part (theta != 0) the new state at the neighbours enters too: inside the
        // chunk u = ub + c_in GG + u_b CB; before it u_{a-1} = al_{a-1} u_a + c_in (the backward
        // recurrence with the chunk's carry-in); after it u_b is the carry-out itself. The terms
        // on the neighbours' ub stay in Omega0 (XA, XB; node a's term folds into its own ub).
        hRB1.assign(N, 0.0); hRB2.assign(N, 0.0); hRY1.assign(N, 0.0); hRY2.assign(N, 0.0);
        hklam.assign(N, L->lam); hXA.assign(N, 0.0); hXB.assign(N, 0.0); hfold.assign(N, 0.0);
        std::vector<double> hE1(N, 0.0), hE2(N, 0.0);
        const double w1 = wlag[1], th = d.theta;
        if (th != 0.0)
            for (int64_t i = 1; i < N; ++i) hklam[i] = L->lam - th * Rlap[i];
        for (int cc = 0; cc < G; ++cc) {
            const int64_t a0 = (int64_t)cc * chunk, b0 = std::min<int64_t>(a0 + chunk, N);
            for (int64_t i = std::max<int64_t>(a0, 1); i < b0; ++i) {
                hE1[i] = (w1 - hklam[i]) * hGG[i];
                hE2[i] = (w1 - hklam[i]) * hCB[i];
                if (th == 0.0) continue;
                const double eA = th * A[i], eB = th * B[i];
                if (i > a0) {
                    hE1[i] -= eA * hGG[i - 1];
                    hE2[i] -= eA * hCB[i - 1];
                    hXA[i] = -eA;
                } else {                           // i == a0 > 0
                    hE1[i] -= eA * (hal[a0 - 1] * hGG[a0] + 1.0);
                    hE2[i] -= eA * hal[a0 - 1] * hCB[a0];
                    hfold[i] = -eA * hal[a0 - 1];  // on node a's own ub
                }
                if (i < b0 - 1) {
                    hE1[i] -= eB * hGG[i + 1];
                    hE2[i] -= eB * hCB[i + 1];
                    hXB[i] = -eB;
                } else {
                    hE2[i] -= eB;                  // u_b = the chunk's carry-out
                }
            }
            double y1 = 0.0, y2 = 0.0;
            for (int64_t i = a0; i < b0; ++i) {
                if (i == 0) { y1 = 0.0; y2 = 0.0; }
                else {
                    y1 = hg[i] * (hA[i] * y1 - hE1[i]);
                    y2 = hg[i] * (hA[i] * y2 - hE2[i]);
                }
                hRY1[i] = y1;
                hRY2[i] = y2;
            }
            double u1 = 0.0, u2 = 0.0;
            for (int64_t i = b0 - 1; i >= a0; --i) {
                u1 = hal[i] * u1 + hRY1[i];
                u2 = hal[i] * u2 + hRY2[i];
                hRB1[i] = u1;
                hRB2[i] = u2;
            }
        }
    }
    const size_t nb = N * sizeof(double);
    const size_t gb = (size_t)G * sizeof(double);
    bool fail = dev_alloc((void **)&L->A, nb) || dev_alloc((void **)&L->g, nb) || dev_alloc((void **)&L->al, nb) ||
                dev_alloc((void **)&L->cf, nb) || dev_alloc((void **)&L->cb, nb) ||
                dev_alloc((void **)&L->CF, nb) || dev_alloc((void **)&L->CB, nb) || dev_alloc((void **)&L->GG, nb) ||
                dev_alloc((void **)&L->Lf, (size_t)(G + 1) * gb) || dev_alloc((void **)&L->Mb, (size_t)G * gb) ||
                dev_alloc((void **)&L->Kb, (size_t)G * gb) || dev_alloc((void **)&L->mb, gb) ||
                dev_alloc((void **)&L->cflag, (size_t)G * sizeof(unsigned long long)) ||
                dev_alloc((void **)&L->seq, sizeof(unsigned long long)) ||
                dev_alloc((void **)&L->U, L->P * sizeof(double)) ||
                dev_alloc((void **)&L->wrev, wrev.size() * sizeof(double)) ||
                dev_alloc((void **)&L->agg, (size_t)BLK * (2 * G + 2) * sizeof(double)) ||
                (split && (dev_alloc((void **)&L->sclane, hsl.size() * sizeof(double)) ||
                           dev_alloc((void **)&L->scwarp, hsw.size() * sizeof(double)))) ||
                dev_alloc((void **)&L->barrier, 2 * sizeof(unsigned));
    if (!fail && !L->split) {
        fail = dev_alloc((void **)&L->D, (size_t)L->max_steps * L->P * sizeof(double)) ||
               dev_alloc((void **)&L->part, (size_t)KS_MAX * L->P * sizeof(double));
    }
    if (!fail && L->x3) {
        L->rows16 = (N + 1 + 127) / 128 * 128;
        L->ld16 = ((int64_t)L->max_steps + 63) / 64 * 64;
        L->ldp = L->ld16 / 64;
        for (int q = 0; q < 3 && !fail; ++q)
            fail = dev_alloc((void **)&L->h3[q], (size_t)L->rows16 * L->ld16 * 2) ||
                   dev_alloc((void **)&L->w3[q], (size_t)BLK * L->sbk * L->ld16 * 2);
        fail = fail || dev_alloc((void **)&L->pA, (size_t)L->rows16 * L->ldp) ||
               dev_alloc((void **)&L->pW, (size_t)BLK * L->sbk * L->ldp * sizeof(float)) ||
               dev_alloc((void **)&L->ring, (size_t)BLK * L->P * sizeof(double)) ||
               dev_alloc((void **)&L->cfar, (size_t)FAR_MAX_SPLITS * BLK * L->sbk * L->P * sizeof(double)) ||
               dev_alloc((void **)&L->wlag, LW * sizeof(double));
        if (!fail) {
            const void *a[3] = {L->h3[0], L->h3[1], L->h3[2]}, *w[3] = {L->w3[0], L->w3[1], L->w3[2]};
            int rcp = far_plan3_init(&L->plan3, a, L->rows16, L->ld16, w, L->ld16, L->sbk);
            if (rcp) {
                std::string keep = fpde_last_error_string();
                fpde_line_destroy(L);
                return set_error(rcp, "%s", keep.c_str());
            }
        }
    } else if (!fail && L->split) {
        L->rows16 = (N + 1 + 127) / 128 * 128;
        L->ld16 = ((int64_t)L->max_steps + 63) / 64 * 64;
        const int64_t nblk = L->ld16 / 64 + 1;
        fail = dev_alloc((void **)&L->h_hi, (size_t)L->rows16 * L->ld16 * 2) ||
               dev_alloc((void **)&L->h_lo, (size_t)L->rows16 * L->ld16 * 2) ||
               dev_alloc((void **)&L->w_hi, (size_t)BLK * L->ld16 * 2) ||
               dev_alloc((void **)&L->w_lo, (size_t)BLK * L->ld16 * 2) ||
               dev_alloc((void **)&L->ring, (size_t)BLK * L->P * sizeof(double)) ||
               dev_alloc((void **)&L->cfar, (size_t)FAR_MAX_SPLITS * BLK * L->P * sizeof(double)) ||
               dev_alloc((void **)&L->wlag, LW * sizeof(double)) ||
               dev_alloc((void **)&L->out_scale, sizeof(double)) ||
               dev_alloc((void **)&L->slots, nblk * sizeof(unsigned long long)) ||
               dev_alloc((void **)&L->exps, nblk * sizeof(int));
        if (!fail) {
            int rcp = far_plan_init(&L->plan, L->h_hi, L->h_lo, L->rows16, L->ld16, L->w_hi, L->w_lo, L->ld16,
                                    d.precision == FPDE_PREC_SPLIT_BF16 ? 1 : 0);
            if (rcp) {
                std::string keep = fpde_last_error_string();
                fpde_line_destroy(L);
                return set_error(rcp, "%s", keep.c_str());
            }
        }
    }
    if (!fail && d.source) {
        L->src_rows = std::min(d.source_rows, d.max_steps);
        fail = dev_alloc((void **)&L->srcd, (size_t)L->src_rows * (N + 1) * sizeof(double));
    }
    if (!fail && d.theta != 0.0)
        fail = dev_alloc((void **)&L->lamv, nb) || dev_alloc((void **)&L->eA, nb) || dev_alloc((void **)&L->eB, nb);
    if (!fail && split)
        fail = dev_alloc((void **)&L->ringf, (size_t)BLK * L->P * sizeof(float2)) ||
               dev_alloc((void **)&L->wff, (size_t)LW * sizeof(float2));
    if (!fail && split)
        fail = dev_alloc((void **)&L->RB1, nb) || dev_alloc((void **)&L->RB2, nb) || dev_alloc((void **)&L->RY1, nb) ||
               dev_alloc((void **)&L->RY2, nb) || dev_alloc((void **)&L->sga, nb) ||
               dev_alloc((void **)&L->sng, nb) || dev_alloc((void **)&L->sc1, nb) || dev_alloc((void **)&L->sc2, nb) ||
               dev_alloc((void **)&L->sc3, nb) || dev_alloc((void **)&L->sngf, (size_t)N * sizeof(float2));
    if (!fail && split && d.theta != 0.0)
        fail = dev_alloc((void **)&L->sxa, nb) || dev_alloc((void **)&L->sxb, nb);
    if (fail) {
        std::string keep = fpde_last_error_string();
        fpde_line_destroy(L);
        return set_error(FPDE_ERR_NOMEM, "%s", keep.c_str());
    }
    cudaStream_t st = ctx->stream;
    std::vector<double> hlamv, heA, heB;
    if (d.theta != 0.0) {                          // Om -= theta (A U[i-1] - Rlap U[i] + B U[i+1])
        hlamv.assign(N, L->lam);
        heA.assign(N, 0.0);
        heB.assign(N, 0.0);
        for (int64_t i = 1; i < N; ++i) {
            hlamv[i] = L->lam - d.theta * Rlap[i];
            heA[i] = d.theta * A[i];
            heB[i] = d.theta * B[i];
        }
        cudaMemcpyAsync(L->lamv, hlamv.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->eA, heA.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->eB, heB.data(), nb, cudaMemcpyHostToDevice, st);
    }
    if (split) {
        cudaMemcpyAsync(L->wff, hwff.data(), (size_t)LW * sizeof(float2), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(L->ringf, 0, (size_t)BLK * L->P * sizeof(float2), st);
    }
    if (split) {
        cudaMemcpyAsync(L->RB1, hRB1.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->RB2, hRB2.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->RY1, hRY1.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->RY2, hRY2.data(), nb, cudaMemcpyHostToDevice, st);
        std::vector<double> h1(N), h2(N), h3(N), h4(N), h5(N), h6(N), h7(N);
        std::vector<float2> hngf(N);
        const double w1 = wlag[1], w2 = wlag[2];
        for (int64_t i = 0; i < N; ++i) {
            h1[i] = hp[i];                         // g A
            h2[i] = -hg[i];
            h3[i] = -hg[i] * ((w1 - hklam[i]) + hfold[i]);
            h4[i] = hg[i] * w1;
            h5[i] = -hg[i] * w2;
            h6[i] = -hg[i] * hXA[i];
            h7[i] = -hg[i] * hXB[i];
            const float hi = (float)h2[i];
            hngf[i] = make_float2(hi, (float)(h2[i] - (double)hi));
        }
        cudaMemcpyAsync(L->sga, h1.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->sng, h2.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->sc1, h3.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->sc2, h4.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->sc3, h5.data(), nb, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->sngf, hngf.data(), (size_t)N * sizeof(float2), cudaMemcpyHostToDevice, st);
        if (L->sxa) {
            cudaMemcpyAsync(L->sxa, h6.data(), nb, cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(L->sxb, h7.data(), nb, cudaMemcpyHostToDevice, st);
        }
    }
    if (L->srcd)
        cudaMemcpyAsync(L->srcd, d.source, (size_t)L->src_rows * (N + 1) * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->A, hA.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->g, hg.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->al, hal.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->cf, hcf.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->cb, hcb.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->CF, hCF.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->CB, hCB.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->GG, hGG.data(), nb, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->Lf, hLf.data(), hLf.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->Mb, hMb.data(), hMb.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->Kb, hKb.data(), hKb.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(L->mb, hmb.data(), gb, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(L->cflag, 0, (size_t)G * sizeof(unsigned long long), st);
    if (split) {
        cudaMemcpyAsync(L->sclane, hsl.data(), hsl.size() * sizeof(double), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->scwarp, hsw.data(), hsw.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    }
    cudaMemsetAsync(L->seq, 0, sizeof(unsigned long long), st);
    cudaMemcpyAsync(L->wrev, wrev.data(), wrev.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(L->U, 0, L->P * sizeof(double), st);
    cudaMemcpyAsync(L->U, u0, (N + 1) * sizeof(double), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(L->barrier, 0, 2 * sizeof(unsigned), st);
    if (!L->split) {
        cudaMemsetAsync(L->D, 0, (size_t)L->max_steps * L->P * sizeof(double), st);
    } else if (L->x3) {
        for (int q = 0; q < 3; ++q) {
            cudaMemsetAsync(L->h3[q], 0, (size_t)L->rows16 * L->ld16 * 2, st);
            cudaMemsetAsync(L->w3[q], 0, (size_t)BLK * L->sbk * L->ld16 * 2, st);
        }
        cudaMemsetAsync(L->pA, 0, (size_t)L->rows16 * L->ldp, st);
        cudaMemsetAsync(L->pW, 0, (size_t)BLK * L->sbk * L->ldp * sizeof(float), st);
        cudaMemsetAsync(L->ring, 0, (size_t)BLK * L->P * sizeof(double), st);
        cudaMemsetAsync(L->cfar, 0, (size_t)FAR_MAX_SPLITS * BLK * L->sbk * L->P * sizeof(double), st);
        cudaMemcpyAsync(L->wlag, wlag.data(), LW * sizeof(double), cudaMemcpyHostToDevice, st);
    } else {
        cudaMemsetAsync(L->h_hi, 0, (size_t)L->rows16 * L->ld16 * 2, st);
        cudaMemsetAsync(L->h_lo, 0, (size_t)L->rows16 * L->ld16 * 2, st);
        cudaMemsetAsync(L->w_hi, 0, (size_t)BLK * L->ld16 * 2, st);
        cudaMemsetAsync(L->w_lo, 0, (size_t)BLK * L->ld16 * 2, st);
        cudaMemsetAsync(L->ring, 0, (size_t)BLK * L->P * sizeof(double), st);
        cudaMemsetAsync(L->cfar, 0, (size_t)FAR_MAX_SPLITS * BLK * L->P * sizeof(double), st);
        cudaMemcpyAsync(L->wlag, wlag.data(), LW * sizeof(double), cudaMemcpyHostToDevice, st);
    }
    if (rich) {                                // closures' inputs and the per-step scratch
        L->rich = true;
        L->rkform = rich->k_form;
        L->rksat = rich->k_sat;
        L->rE.assign(rich->evaporation, rich->evaporation + std::min(rich->evaporation_rows, d.max_steps));
        const size_t nb1 = (size_t)(N + 1) * sizeof(double);
        bool f2 = dev_alloc((void **)&L->rZ, nb1) || dev_alloc((void **)&L->rdL, nb1) ||
                  dev_alloc((void **)&L->rA, nb1) || dev_alloc((void **)&L->rB, nb1) ||
                  dev_alloc((void **)&L->rR, nb1) || dev_alloc((void **)&L->rOm, nb1) ||
                  dev_alloc((void **)&L->ral, nb1 + sizeof(double)) || dev_alloc((void **)&L->rbt, nb1 + sizeof(double)) ||
                  dev_alloc((void **)&L->last, L->P * sizeof(double)) ||
                  (L->split && dev_alloc((void **)&L->Sn, L->P * sizeof(double)));
        if (f2) {
            std::string keep = fpde_last_error_string();
            fpde_line_destroy(L);
            return set_error(FPDE_ERR_NOMEM, "%s", keep.c_str());
        }
        cudaMemcpyAsync(L->rZ, rich->sZ, nb1, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(L->rdL, rich->dL[0], nb1, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(L->last, 0, L->P * sizeof(double), st);
        cudaMemcpyAsync(L->last, u0, nb1, cudaMemcpyHostToDevice, st);
    }
    L->d.richards = nullptr;                   // host pointers are not kept
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        fpde_line_destroy(L);
        return set_error(FPDE_ERR_CUDA, "line setup: %s", cudaGetErrorString(e));
    }
    ctx->lines.insert(L);
    *out = L;
    return FPDE_OK;
}

int fpde_line_reset(fpde_line *L, const double *u0, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(L && u0, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaMemcpyAsync(L->U, u0, (L->N + 1) * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, L->ctx->stream));
    if (L->last)                               // the Richards line's previous state (increments)
        FPDE_CUDA(cudaMemcpyAsync(L->last, L->U, (L->N + 1) * sizeof(double), cudaMemcpyDeviceToDevice,
                                  L->ctx->stream));
    if (!on_device) FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    L->n_done = 0;
    return FPDE_OK;
}

int fpde_line_run(fpde_line *L, int steps)
{
    clear_error();
    FPDE_CHECK_ARG(L && steps >= 0, "bad arguments");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    if (steps == 0) return FPDE_OK;
    if (L->n_done + steps > L->max_steps)
        return set_error(FPDE_ERR_CAPACITY, "run of %d steps exceeds the history capacity %d", steps, L->max_steps);
    cudaStream_t st = L->ctx->stream;
    if (steps < L->graph_min) {                  // short runs: enqueued directly, no graph
        int64_t nk = 0;
        if ((rc = line_enqueue(L, st, L->n_done, steps, &nk))) return rc;
        L->last_probes = L->probes;
        L->n_done += steps;
        return FPDE_OK;
    }
    auto *g = L->graphs.find(L->n_done, steps);
    if (!g) {
        rc = L->graphs.capture(L->n_done, steps,
                               [&](cudaStream_t cs, int64_t *nk, std::vector<fpde_line::Probe> *probes) {
                                   const int r = line_enqueue(L, cs, L->n_done, steps, nk);
                                   *probes = L->probes;
                                   return r;
                               },
                               &g);
        if (rc) return rc;
    }
    L->last_probes = g->aux;
    FPDE_CUDA(cudaGraphLaunch(g->exec, st));
    count_launches(g->launches);
    L->n_done += steps;
    return FPDE_OK;
}

int fpde_line_get_state(fpde_line *L, double *u, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(L && u, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u, L->U, (L->N + 1) * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, L->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    return ctx_check_flags(L->ctx, "line");
}

int fpde_line_state_ptr(fpde_line *L, double **u_dev)
{
    FPDE_CHECK_ARG(L && u_dev, "null argument");
    *u_dev = L->U;
    return FPDE_OK;
}

int fpde_line_solve_host(fpde_line *L, const double *u0_host, int steps, double *u_out_host)
{
    clear_error();
    FPDE_CHECK_ARG(L && u0_host && u_out_host, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    cudaStream_t st = L->ctx->stream;
    FPDE_CUDA(cudaMemcpyAsync(L->U, u0_host, (L->N + 1) * sizeof(double), cudaMemcpyHostToDevice, st));
    if (L->last)
        FPDE_CUDA(cudaMemcpyAsync(L->last, L->U, (L->N + 1) * sizeof(double), cudaMemcpyDeviceToDevice, st));
    L->n_done = 0;
    if ((rc = fpde_line_run(L, steps))) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u_out_host, L->U, (L->N + 1) * sizeof(double), cudaMemcpyDeviceToHost, st));
    FPDE_CUDA(cudaStreamSynchronize(st));
    return ctx_check_flags(L->ctx, "line");
}

int fpde_line_set_probe(fpde_line *L, int every)
{
    clear_error();
    FPDE_CHECK_ARG(L && every >= 0, "bad arguments");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    L->graphs.clear();
    L->last_probes.clear();
    for (cudaEvent_t e : L->probe_ev) cudaEventDestroy(e);
    L->probe_ev.clear();
    L->probe_every = every;
    if (every > 0) {
        int64_t n = 2 * (L->max_steps / every) + 2 * (L->max_steps / BLK) + 4;
        if (n > 8192) n = 8192;
        L->probe_ev.resize(2 * n);
        for (auto &e : L->probe_ev) FPDE_CUDA(cudaEventCreate(&e));
    }
    return FPDE_OK;
}

int fpde_line_probe_stats(fpde_line *L, int kind, double *ms, double *bytes, double *flops, int *count)
{
    clear_error();
    FPDE_CHECK_ARG(L && ms && bytes && flops && count, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    double m = 0, b = 0, f = 0;
    int c = 0;
    for (const auto &p : L->last_probes) {
        if (p.kind != kind) continue;
        float t = 0;
        FPDE_CUDA(cudaEventElapsedTime(&t, L->probe_ev[p.ev], L->probe_ev[p.ev + 1]));
        m += t;
        b += p.bytes;
        f += p.flops;
        c += p.steps;
    }
    *ms = m;
    *bytes = b;
    *flops = f;
    *count = c;
    return FPDE_OK;
}

int fpde_line_graph_stats(const fpde_line *L, int *cached, int64_t *instantiated)
{
    FPDE_CHECK_ARG(L && cached && instantiated, "null argument");
    *cached = (int)L->graphs.entries.size();
    *instantiated = L->graphs.instantiated;
    return FPDE_OK;
}

int fpde_line_steps_done(const fpde_line *L, int64_t *n)
{
    FPDE_CHECK_ARG(L && n, "null argument");
    *n = L->n_done;
    return FPDE_OK;
}

int fpde_step_block(fpde_line *L, int *steps_run)
{
    clear_error();
    FPDE_CHECK_ARG(L && steps_run, "null argument");
    static_assert(FPDE_BLOCK_STEPS == BLK, "block length");
    const int64_t to_end = BLK - L->n_done % BLK;
    const int steps = (int)std::min<int64_t>(to_end, (int64_t)L->max_steps - L->n_done);
    *steps_run = steps > 0 ? steps : 0;
    return steps > 0 ? fpde_line_run(L, steps) : FPDE_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------------- autotuner
namespace fpde {

// Time `fn` (which enqueues work on st) reps times after one warm-up; ms per call.
template <class F>
static float time_on_stream(cudaStream_t st, int reps, F fn)
{
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fn();
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) fn();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / reps;
}

}  // namespace fpde

extern "C" int fpde_line_autotune(fpde_ctx *ctx, const fpde_line_desc *desc, const double *A, const double *B,
                                  const double *Rlap, const double *u0, fpde_line_tuning *out)
{
    clear_error();
    FPDE_CHECK_ARG(desc && A && B && Rlap && u0 && out, "null argument");
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    const fpde_line_desc &d = *desc;
    const bool split = d.precision != FPDE_PREC_FP64;
    const int lt = split ? LTS : LT;
    const int64_t N = d.N;
    cudaStream_t st = ctx->stream;
    fpde_line_tuning best{};
    double best_ms = 1e300;

    // 1. partition of the solve: solve_sp x chunks, timed on the second 64-step block of a short run
    const int tsteps = std::min(d.max_steps, 128);
    const int first = std::min(64, tsteps / 2);
    std::vector<std::pair<int, int>> cands;
    for (int sp = 1; sp <= LSEG; sp <<= 1) {
        const int64_t gmin = (N + (int64_t)lt * sp - 1) / ((int64_t)lt * sp);
        if (gmin > ctx->sm_count) continue;
        std::vector<int> gs = {(int)gmin};
        if (gmin > 1) {
            gs.push_back(ctx->sm_count);
            gs.push_back((int)((gmin + ctx->sm_count) / 2));
        }
        std::sort(gs.begin(), gs.end());
        gs.erase(std::unique(gs.begin(), gs.end()), gs.end());
        for (int g : gs) cands.emplace_back(sp, g);
    }
    for (const auto &cd : cands) {
        fpde_line_tuning t{};
        t.solve_sp = cd.first;
        t.chunks = cd.second;
        fpde_line_desc td = d;
        td.max_steps = tsteps;
        td.tuning = &t;
        fpde_line *L = nullptr;
        if (fpde_line_create(ctx, &td, A, B, Rlap, u0, &L) != FPDE_OK) {   // e.g. not co-resident
            clear_error();
            continue;
        }
        L->graph_min = 1;                                       // time graph replays, not launches
        bool ok = fpde_line_run(L, first) == FPDE_OK && fpde_line_run(L, tsteps - first) == FPDE_OK &&
                  fpde_line_reset(L, u0, 0) == FPDE_OK && fpde_line_run(L, first) == FPDE_OK;
        float ms = 0.f;
        if (ok) {
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            cudaEventRecord(e0, st);
            ok = fpde_line_run(L, tsteps - first) == FPDE_OK;
            cudaEventRecord(e1, st);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
        }
        unsigned flags = 0;
        cudaMemcpy(&flags, ctx->d_flags, sizeof flags, cudaMemcpyDeviceToHost);
        if (flags) {                                            // a bounded wait gave up: not a candidate
            cudaMemset(ctx->d_flags, 0, sizeof(unsigned));
            ok = false;
        }
        fpde_line_destroy(L);
        if (!ok) {
            clear_error();
            continue;
        }
        const double per = ms / (tsteps - first);
        if (per < best_ms) {
            best_ms = per;
            best.solve_sp = cd.first;
            best.chunks = cd.second;
        }
    }
    if (best_ms >= 1e300) return set_error(FPDE_ERR_UNSUPPORTED, "autotune: no partition of this line could run");
    best.ms_per_step = best_ms;

    const int64_t kt_steps = std::min<int64_t>((int64_t)d.max_steps / 64 * 64, 2048);
    if (split && d.precision == FPDE_PREC_SPLIT_BF16X3 && kt_steps >= 128) {
        // 2. split depth of the far contraction at a history of kt_steps columns (zero data)
        const int64_t rows = (N + 1 + 127) / 128 * 128, ldp = kt_steps / 64;
        uint16_t *a3[3] = {nullptr, nullptr, nullptr}, *w3[3] = {nullptr, nullptr, nullptr};
        int8_t *pA = nullptr;
        float *pW = nullptr;
        double *C = nullptr;
        bool fail = false;
        for (int q = 0; q < 3 && !fail; ++q)
            fail = dev_alloc((void **)&a3[q], (size_t)rows * kt_steps * 2) ||
                   dev_alloc((void **)&w3[q], (size_t)64 * kt_steps * 2);
        fail = fail || dev_alloc((void **)&pA, (size_t)rows * ldp) || dev_alloc((void **)&pW, (size_t)64 * ldp * sizeof(float)) ||
               dev_alloc((void **)&C, (size_t)FAR_MAX_SPLITS * 64 * rows * sizeof(double));
        if (!fail) {
            for (int q = 0; q < 3; ++q) {
                cudaMemsetAsync(a3[q], 0, (size_t)rows * kt_steps * 2, st);
                cudaMemsetAsync(w3[q], 0, (size_t)64 * kt_steps * 2, st);
            }
            cudaMemsetAsync(pA, 0, (size_t)rows * ldp, st);
            cudaMemsetAsync(pW, 0, (size_t)64 * ldp * sizeof(float), st);
            FarPlan3 plan;
            const void *ap[3] = {a3[0], a3[1], a3[2]}, *wp[3] = {w3[0], w3[1], w3[2]};
            if (far_plan3_init(&plan, ap, rows, kt_steps, wp, kt_steps) == FPDE_OK) {
                double bms = 1e300;
                for (int s = 1; s <= FAR_MAX_SPLITS; ++s) {
                    const float ms = time_on_stream(st, 3, [&] {
                        far3_launch(st, &plan, (int)kt_steps, C, 64 * rows, rows, s, pA, pW, ldp, ctx->d_flags);
                    });
                    if (ms < bms) { bms = ms; best.far_splits = s; }
                }
            }
        }
        cudaStreamSynchronize(st);
        for (int q = 0; q < 3; ++q) { dev_free(a3[q]); dev_free(w3[q]); }
        dev_free(pA);
        dev_free(pW);
        dev_free(C);
        clear_error();
    }
    if (!split) {
        // 3. row splits of the FP64 history sum at min(max_steps, 2048) rows (zero data)
        const int64_t P = (N + 1 + 511) / 512 * 512;
        const int nrow = std::min(d.max_steps, 2048);
        double *D = nullptr, *part = nullptr, *w = nullptr;
        if (nrow >= 8 && !dev_alloc((void **)&D, (size_t)nrow * P * sizeof(double)) &&
            !dev_alloc((void **)&part, (size_t)KS_MAX * P * sizeof(double)) &&
            !dev_alloc((void **)&w, (size_t)nrow * sizeof(double))) {
            cudaMemsetAsync(D, 0, (size_t)nrow * P * sizeof(double), st);
            cudaMemsetAsync(w, 0, (size_t)nrow * sizeof(double), st);
            const int k0 = choose_splits(nrow, P);
            const int ks_c[3] = {std::max(1, k0 / 2), k0, std::min(KS_MAX, 2 * k0)};
            double bms = 1e300;
            for (int ks : ks_c) {
                const float ms = time_on_stream(st, 3, [&] { launch_l1_partial(st, D, P, nrow, w, part, ks); });
                if (ms < bms) { bms = ms; best.gemv_splits = ks; }
            }
        }
        cudaStreamSynchronize(st);
        dev_free(D);
        dev_free(part);
        dev_free(w);
        clear_error();
    }
    if (d.precision == FPDE_PREC_SPLIT_BF16X3 && !d.richards && d.max_steps >= 512) {
        // 4. depth of the far super-blocks (64-step blocks contracted together against the older
        // history, whose benefit grows with the history): a whole run of min(max_steps, 4096) steps
        // per choice, replayed from its graph
        const int ks = std::min(d.max_steps, 4096) / 256 * 256;
        double bms = 1e300;
        int bsup = 0;
        for (int sup : {1, 2, 4}) {
            fpde_line_tuning t = best;
            t.far_super = sup;
            fpde_line_desc td = d;
            td.max_steps = ks;
            td.tuning = &t;
            fpde_line *L = nullptr;
            if (fpde_line_create(ctx, &td, A, B, Rlap, u0, &L) != FPDE_OK) {
                clear_error();
                continue;
            }
            bool ok = fpde_line_run(L, ks) == FPDE_OK && fpde_line_reset(L, u0, 0) == FPDE_OK;
            float ms = 0.f;
            if (ok) {
                cudaEvent_t e0, e1;
                cudaEventCreate(&e0);
                cudaEventCreate(&e1);
                cudaEventRecord(e0, st);
                ok = fpde_line_run(L, ks) == FPDE_OK;
                cudaEventRecord(e1, st);
                cudaEventSynchronize(e1);
                cudaEventElapsedTime(&ms, e0, e1);
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
            }
            unsigned flags = 0;
            cudaMemcpy(&flags, ctx->d_flags, sizeof flags, cudaMemcpyDeviceToHost);
            if (flags) {
                cudaMemset(ctx->d_flags, 0, sizeof(unsigned));
                ok = false;
            }
            fpde_line_destroy(L);
            clear_error();
            if (ok && ms < bms) {
                bms = ms;
                bsup = sup;
            }
        }
        if (bsup) best.far_super = bsup;
    }
    *out = best;
    return ctx_check_flags(ctx, "autotune");
}
