// The fully implicit 3D space-fractional scheme of fpde_hpc_1d.cpp (implicit3d 1, impl 2,
// toeplitz_mult_alg 0, equation 0): the product vmul_T_3d (:6801-8722) of the 7-diagonal Mat_3d plus,
// along each axis, iw * T * tridiag(Mcoefs_3d[axis]) with T the axis's Toeplitz matrix, and the solve
// solve_mln<1> (:812-1157) that calc_step (:5681-5716) runs on it once per step over the V = G + 1
// values of the grid (G = (sN+2)(M+2)(K+2) nodes, i fastest, plus the one past the grid).
//
// The product is node-parallel. A first phase forms each axis's Bt = tridiag(Mcoefs_3d[axis]) x at
// the interior nodes (the only ones the Toeplitz sums read); a second forms every output in the
// reference's order: the seven diagonals with its flat-index bounds, then the K, _M and sN Toeplitz
// terms, each one thread's sequential sum over its line without contracted multiply-adds. So a
// product equals the reference's bit for bit. All vectors are node-major and stay in L2 for the
// grids this scheme is run on (a 64^3 grid is 2.3 MB per vector).
//
// A solve is one persistent cooperative kernel: every thread owns a fixed set of nodes, the vector
// updates need no synchronisation, and a bounded grid barrier separates the phases whose reads cross
// nodes (the two phases of a product, and each dot product). Dot products come in two forms:
//   exact: every product a[v]*b[v] is stored and one thread adds them in index order (the
//          reference's loop), so the iterates, the iteration count and the solution are the
//          reference's bit for bit; the add chain runs on one thread (use on small grids);
//   fast:  each thread adds its nodes, each CTA folds its threads in a fixed tree and every CTA
//          folds the CTA partials in the same fixed order, so the result is deterministic and
//          identical in every CTA, and differs from the reference's only by the order of the adds.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "scan.cuh"

namespace fpde {

namespace {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

constexpr int SF3_THREADS = 256;
constexpr int SF3_WARPS = SF3_THREADS / 32;
constexpr uint64_t SF3_TIME_LIMIT_NS = 30ull * 1000000000ull;   // per solve

struct Geo {
    int sN, M, K;
    int64_t sy, sz, G, V;
};

__device__ __forceinline__ Geo geo_of(const Sf3dSystem &s)
{
    Geo g;
    g.sN = s.sN; g.M = s.M; g.K = s.K;
    g.sy = s.sN + 2;
    g.sz = (int64_t)(s.sN + 2) * (s.M + 2);
    g.G = g.sz * (s.K + 2);
    g.V = g.G + 1;
    return g;
}

// Node v < G as (i, j, k); false for nodes outside 1..len-1 on some axis (and for v = G).
__device__ __forceinline__ bool interior(const Geo &g, int64_t v, int *i, int *j, int *k)
{
    if (v >= g.G) return false;
    const int64_t kk = v / g.sz, rem = v - kk * g.sz;
    const int64_t jj = rem / g.sy, ii = rem - jj * g.sy;
    *i = (int)ii; *j = (int)jj; *k = (int)kk;
    return ii >= 1 && ii < g.sN && jj >= 1 && jj < g.M && kk >= 1 && kk < g.K;
}

// Bt of the three axes at node v (:7254-7261, :7677-7684, :8097-8104): Mcoefs_3d[c][1] x, then the
// lower and the upper neighbour along the axis (always inside the vector at an interior node).
__device__ __forceinline__ void bt_node(const Sf3dSystem &s, const Geo &g, const double *x, double *bt, int64_t v)
{
    int i, j, k;
    if (!interior(g, v, &i, &j, &k)) return;
    const int64_t V = g.V;
    const double xv = __ldcg(x + v);
#pragma unroll
    for (int c = 2; c >= 0; --c) {
        const int n = c == 2 ? g.K : (c == 1 ? g.M : g.sN);
        if (n <= 2) continue;
        const int64_t st = c == 2 ? g.sz : (c == 1 ? g.sy : 1);
        const double *mc = s.mc + (int64_t)(3 * c) * V;
        double b = dm(__ldg(mc + V + v), xv);
        b = da(b, dm(__ldg(mc + v), __ldcg(x + v - st)));
        b = da(b, dm(__ldg(mc + 2 * V + v), __ldcg(x + v + st)));
        bt[(int64_t)c * V + v] = b;
    }
}

// One axis's Toeplitz term at position p of its line (:7562-7574): the sum over j < p, then (two-sided)
// the subtraction over j > p, in increasing j; row scaling and inv_dw_dh as the reference applies them.
__device__ __forceinline__ double axis_term(const double *bt, int64_t base, int64_t st, int p, int n, int sd,
                                            const double *T, const double *rs, const double *iw, int64_t v)
{
    double t = 0.0;
    const int qe = sd ? n : p;
    for (int q = 1; q < qe; ++q) {
        if (q == p) continue;
        const double pr = dm(__ldcg(bt + base + (int64_t)q * st), T[q < p ? p - q + 1 : q - p + 1]);
        t = q < p ? da(t, pr) : ds(t, pr);
    }
    if (rs) t = __ddiv_rn(t, __ldg(rs + v));
    return iw ? dm(t, __ldg(iw + v)) : t;
}

// Output v of the product (:6857-6877 and the three axes' sums). Tm: the three rows in shared memory.
__device__ __forceinline__ double row_node(const Sf3dSystem &s, const Geo &g, const double *const *Tm,
                                           const double *x, const double *bt, int64_t v)
{
    const int64_t V = g.V;
    const double *M = s.mat;
    double r = dm(__ldg(M + V + v), __ldcg(x + v));
    if (g.sN > 2) {
        if (v - 1 >= 0) r = da(r, dm(__ldg(M + 5 * V + v), __ldcg(x + v - 1)));
        if (v + 1 < V) r = da(r, dm(__ldg(M + 6 * V + v), __ldcg(x + v + 1)));
    }
    if (g.M > 2) {
        if (v - g.sy >= 0) r = da(r, dm(__ldg(M + 3 * V + v), __ldcg(x + v - g.sy)));
        if (v + g.sy < V) r = da(r, dm(__ldg(M + 4 * V + v), __ldcg(x + v + g.sy)));
    }
    if (g.K > 2) {
        if (v - g.sz >= 0) r = da(r, dm(__ldg(M + v), __ldcg(x + v - g.sz)));
        if (v + g.sz < V) r = da(r, dm(__ldg(M + 2 * V + v), __ldcg(x + v + g.sz)));
    }
    int i, j, k;
    if (!interior(g, v, &i, &j, &k)) return r;
    if (g.K > 2)
        r = da(r, axis_term(bt + 2 * V, v - (int64_t)k * g.sz, g.sz, k, g.K, s.sd, Tm[2], s.rs,
                            s.iw ? s.iw + 2 * V : nullptr, v));
    if (g.M > 2)
        r = da(r, axis_term(bt + V, v - (int64_t)j * g.sy, g.sy, j, g.M, s.sd, Tm[1], s.rs,
                            s.iw ? s.iw + V : nullptr, v));
    if (g.sN > 2)
        r = da(r, axis_term(bt, v - i, 1, i, g.sN, s.sd, Tm[0], s.rs, s.iw, v));
    return r;
}

// The three Toeplitz rows into shared memory (lengths sN, M, K; entries 2..len-1 are read).
__device__ __forceinline__ void load_rows(const Sf3dSystem &s, double *sm, const double **Tm)
{
    const int n0 = s.sN + 1, n1 = s.M + 1, n2 = s.K + 1;
    Tm[0] = sm; Tm[1] = sm + n0; Tm[2] = sm + n0 + n1;
    for (int q = threadIdx.x; q < n0 + n1 + n2; q += blockDim.x) {
        double v;
        if (q < n0) v = s.Tm[0][q];
        else if (q < n0 + n1) v = s.Tm[1][q - n0];
        else v = s.Tm[2][q - n0 - n1];
        sm[q] = v;
    }
    __syncthreads();
}

// -------------------------------------------------------------------- standalone product

__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_bt(Sf3dSystem s, const double *x, double *bt)
{
    const Geo g = geo_of(s);
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x)
        bt_node(s, g, x, bt, v);
}

__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_rows(Sf3dSystem s, const double *x, const double *bt, double *r)
{
    extern __shared__ double sf3_sm[];
    const double *Tm[3];
    load_rows(s, sf3_sm, Tm);
    const Geo g = geo_of(s);
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x)
        r[v] = row_node(s, g, Tm, x, bt, v);
}

// -------------------------------------------------------------------------- the solve

struct SolveArgs {
    Sf3dSystem s;
    double *x;                 // initial guess in, solution out
    const double *B;
    double *r, *q0, *g0, *g1, *w0, *w1, *u, *Au, *bt;   // V each (bt: 3V)
    double *prod;              // exact: 2V products
    double *part;              // fast: 2 x gridDim partials
    double *gscal;             // exact: the sums (2)
    unsigned *gstop;           // time limit reached (set by CTA 0 before a barrier)
    unsigned *bar;             // barrier state (count, generation)
    unsigned *flags;
    unsigned long long *iters_total;   // += iterations (may be null)
    int *iters_out;            // iterations (may be null)
    double thr;
    int maxiter;
};

template <bool EXACT>
struct Solver {
    const SolveArgs &a;
    Geo g;
    const double *Tm[3];
    int64_t gt, GT;
    double *wsum;              // shared: 2 x SF3_WARPS
    double *res;               // shared: 2

    __device__ bool sync() { return grid_barrier(a.bar, gridDim.x, a.flags); }

    // y = A x (two phases, one barrier between them); the caller has synchronised x.
    __device__ bool apply(const double *x, double *y)
    {
        for (int64_t v = gt; v < g.V; v += GT) bt_node(a.s, g, x, a.bt, v);
        if (!sync()) return false;
        for (int64_t v = gt; v < g.V; v += GT) y[v] = row_node(a.s, g, Tm, x, a.bt, v);
        return true;
    }

    // A product term of dot slot q: exact stores it, fast adds it to the thread's partial.
    __device__ __forceinline__ void term(int q, int64_t v, double p, double *acc, bool neg)
    {
        if (EXACT) a.prod[(int64_t)q * g.V + v] = p;
        else acc[q] = neg ? ds(acc[q], p) : da(acc[q], p);
    }

    // The nd dot products whose terms every thread has just produced; out[q] in every thread.
    // neg[q]: the reference subtracts the terms from 0.0 (beta's "beta -= q*r").
    __device__ bool dots(int nd, const double *acc, const bool *neg, double *out)
    {
        const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
        if (EXACT) {
            if (!sync()) return false;
            if (blockIdx.x == 0 && lane == 0 && warp < nd) {
                const double *p = a.prod + (int64_t)warp * g.V;
                double t = 0.0;
                if (neg[warp])
                    for (int64_t v = 0; v < g.V; ++v) t = ds(t, __ldcg(p + v));
                else
                    for (int64_t v = 0; v < g.V; ++v) t = da(t, __ldcg(p + v));
                a.gscal[warp] = t;
            }
            if (!sync()) return false;
            if (tid < nd) res[tid] = __ldcg(a.gscal + tid);
            __syncthreads();
        } else {
            for (int q = 0; q < nd; ++q) {
                double t = acc[q];
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) t = da(t, __shfl_down_sync(0xffffffffu, t, o));
                if (lane == 0) wsum[q * SF3_WARPS + warp] = t;
            }
            __syncthreads();
            if (tid < nd) {
                double t = 0.0;
                for (int w = 0; w < SF3_WARPS; ++w) t = da(t, wsum[tid * SF3_WARPS + w]);
                a.part[(int64_t)tid * gridDim.x + blockIdx.x] = t;
            }
            if (!sync()) return false;
            if (warp < nd) {
                const double *p = a.part + (int64_t)warp * gridDim.x;
                double t = 0.0;
                for (unsigned b = lane; b < gridDim.x; b += 32) t = da(t, __ldcg(p + b));
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) t = da(t, __shfl_down_sync(0xffffffffu, t, o));
                if (lane == 0) res[warp] = t;
            }
            __syncthreads();
        }
        for (int q = 0; q < nd; ++q) out[q] = res[q];
        __syncthreads();
        return true;
    }
};

// solve_mln<1> over the V values, the grid form of the per-line solve of spacefrac.cu (the same
// sequence of products, dot products, divisions and tests: :841-866 at a start, :871-1132 per
// iteration with the q.r reuse and the w/g shift). A start repeated more than maxiter times without
// an iteration between, the time limit or a barrier that times out ends the solve with a flag.
template <bool EXACT>
__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_solve(SolveArgs a)
{
    extern __shared__ double sf3_sm[];
    __shared__ double wsum[2 * SF3_WARPS];
    __shared__ double res[2];
    __shared__ unsigned stop_s;
    Solver<EXACT> S{a};
    load_rows(a.s, sf3_sm, S.Tm);
    S.g = geo_of(a.s);
    S.gt = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    S.GT = (int64_t)gridDim.x * blockDim.x;
    S.wsum = wsum;
    S.res = res;
    const int64_t V = S.g.V, gt = S.gt, GT = S.GT;
    const double md = (double)V;
    const unsigned long long t0 = gtimer_ns();
    double *x = a.x, *r = a.r, *q0 = a.q0, *u = a.u, *Au = a.Au;
    double *g0 = a.g0, *g1 = a.g1, *w0 = a.w0, *w1 = a.w1;
    const double *B = a.B;
    const bool pos[2] = {false, false}, negq[2] = {true, false};
    double c1 = 0.0, al = 0.0, out[2], acc[2];
    int iter = 1, restarts = 0;
    bool have_qr = false;
restart:
    if (++restarts > a.maxiter + 1) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, DEVERR_SOLVER);
        goto out;
    }
    have_qr = false;
    if (!S.apply(x, r)) return;                                                       // :841-844
    acc[0] = acc[1] = 0.0;
    for (int64_t v = gt; v < V; v += GT) {
        const double e = ds(B[v], r[v]);
        r[v] = e; g1[v] = e; q0[v] = e;
        S.term(0, v, dm(e, e), acc, false);                                           // norm (:864)
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && gtimer_ns() - t0 > SF3_TIME_LIMIT_NS) atomicExch(a.gstop, 1u);
    if (!S.dots(1, acc, pos, out)) return;
    if (threadIdx.x == 0) stop_s = __ldcg(a.gstop);
    __syncthreads();
    if (stop_s) {                                                                     // restarts past the limit
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, DEVERR_SOLVER);
        goto out;
    }
    {
        const double norm = out[0];
        if (!S.apply(g1, w1)) return;                                                 // :851
        acc[0] = 0.0;
        for (int64_t v = gt; v < V; v += GT) S.term(0, v, dm(q0[v], w1[v]), acc, false);   // c[1] (:853-856)
        if (!S.dots(1, acc, pos, out)) return;
        c1 = out[0];
        if (fabs(__ddiv_rn(norm, md)) < a.thr) goto out;                               // :866
    }
    for (;;) {
        if (!have_qr) {                                                                // :871-877
            acc[0] = 0.0;
            for (int64_t v = gt; v < V; v += GT) S.term(0, v, dm(q0[v], r[v]), acc, false);
            if (!S.dots(1, acc, pos, out)) return;
            al = __ddiv_rn(out[0], c1);
        }
        if (!(c1 != 0.0)) goto restart;                                                // :878, :913
        for (int64_t v = gt; v < V; v += GT) {
            u[v] = ds(r[v], dm(al, w1[v]));
            x[v] = da(x[v], dm(al, g1[v]));
        }
        if (!S.sync()) return;
        if (!S.apply(u, Au)) return;                                                  // :890
        acc[0] = acc[1] = 0.0;
        for (int64_t v = gt; v < V; v += GT) {
            const double av = Au[v];
            S.term(0, v, dm(av, av), acc, false);
            S.term(1, v, dm(av, u[v]), acc, false);
        }
        if (!S.dots(2, acc, pos, out)) return;
        const double nrm = out[0];
        const double ro1 = __ddiv_rn(-out[1], nrm);                                   // :903
        if (nrm == 0.0) goto restart;                                                  // :904-905
        for (int64_t v = gt; v < V; v += GT) x[v] = ds(x[v], dm(ro1, u[v]));
        if (!S.sync()) return;
        if (!S.apply(x, r)) return;                                                   // :943-947
        acc[0] = acc[1] = 0.0;
        for (int64_t v = gt; v < V; v += GT) {
            const double e = ds(B[v], r[v]);
            r[v] = e;
            S.term(0, v, dm(q0[v], e), acc, true);                                   // beta's q.r (:1056-1059)
            S.term(1, v, dm(e, e), acc, false);                                       // r.r (:1127)
        }
        if (!S.dots(2, acc, negq, out)) return;
        const double nq = out[0], norm = out[1];
        double beta = __ddiv_rn(nq, c1);                                               // :1060-1065
        if (c1 == 0.0) beta = 0.0;
        const double bro = __ddiv_rn(beta, ro1);
        for (int64_t v = gt; v < V; v += GT) {
            const double zw = da(r[v], dm(beta, w1[v]));
            g0[v] = da(zw, dm(bro, g1[v]));
        }
        if (!S.sync()) return;
        if (!S.apply(g0, w0)) return;                                                 // :1094
        acc[0] = 0.0;
        for (int64_t v = gt; v < V; v += GT) S.term(0, v, dm(q0[v], w0[v]), acc, false);   // c[0] (:1096-1099)
        if (blockIdx.x == 0 && threadIdx.x == 0 && gtimer_ns() - t0 > SF3_TIME_LIMIT_NS) atomicExch(a.gstop, 1u);
        if (!S.dots(1, acc, pos, out)) return;
        if (threadIdx.x == 0) stop_s = __ldcg(a.gstop);
        __syncthreads();
        c1 = out[0];                                                                   // the shift :1104-1121
        if (nq != 0.0) al = __ddiv_rn(-nq, c1);                                        // next iteration's al
        have_qr = nq != 0.0;
        {
            double *t = g0; g0 = g1; g1 = t;
            t = w0; w0 = w1; w1 = t;
        }
        restarts = 0;
        if (fabs(__ddiv_rn(norm, md)) < a.thr) break;                                 // :1126-1132
        ++iter;
        if (iter == a.maxiter) break;
        if (stop_s) {
            if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, DEVERR_SOLVER);
            break;
        }
    }
out:
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        if (a.iters_total) atomicAdd(a.iters_total, (unsigned long long)iter);
        if (a.iters_out) *a.iters_out = iter;
    }
}

size_t rows_smem(const Sf3dSystem &s) { return (size_t)(s.sN + s.M + s.K + 3) * sizeof(double); }

}  // namespace

// ------------------------------------------------------------------ workspace and launches

struct Sf3dWork {
    int64_t V = 0;
    int blocks = 0;                      // the larger of the two
    int blocks_fast = 0, blocks_exact = 0;   // CTAs of each solve form (all co-resident)
    double *vec = nullptr;               // r q0 g0 g1 w0 w1 u Au, bt (3V), prod (2V)
    double *part = nullptr, *gscal = nullptr;
    unsigned *ctl = nullptr;             // barrier (2), stop (1)
    int exact_ok = 0;
};

static int solve_blocks(const Sf3dSystem &s, bool exact, int64_t V, int *blocks)
{
    int dev = 0, sms = 0, per = 0;
    FPDE_CUDA(cudaGetDevice(&dev));
    FPDE_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const size_t smem = rows_smem(s);
    if (exact) FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sf3d_solve<true>, SF3_THREADS, smem));
    else FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sf3d_solve<false>, SF3_THREADS, smem));
    if (per < 1) return set_error(FPDE_ERR_CUDA, "space-fractional 3D solve: no co-resident CTA fits");
    const int64_t need = (V + SF3_THREADS - 1) / SF3_THREADS;
    *blocks = (int)std::min<int64_t>((int64_t)per * sms, need);
    return FPDE_OK;
}

int sf3d_work_create(const Sf3dSystem &s, Sf3dWork **out)
{
    *out = nullptr;
    Sf3dWork *w = new Sf3dWork();
    w->V = (int64_t)(s.sN + 2) * (s.M + 2) * (s.K + 2) + 1;
    int rc = solve_blocks(s, false, w->V, &w->blocks_fast);
    if (!rc) rc = solve_blocks(s, true, w->V, &w->blocks_exact);
    if (rc) { delete w; return rc; }
    w->blocks = std::max(w->blocks_fast, w->blocks_exact);
    if (dev_alloc((void **)&w->vec, (size_t)13 * w->V * sizeof(double)) ||
        dev_alloc((void **)&w->part, (size_t)2 * w->blocks * sizeof(double)) ||
        dev_alloc((void **)&w->gscal, 4 * sizeof(double)) || dev_alloc((void **)&w->ctl, 4 * sizeof(unsigned))) {
        sf3d_work_destroy(w);
        return set_error(FPDE_ERR_NOMEM, "space-fractional 3D solve: workspace allocation failed");
    }
    cudaMemset(w->vec, 0, (size_t)13 * w->V * sizeof(double));
    cudaMemset(w->ctl, 0, 4 * sizeof(unsigned));
    *out = w;
    return FPDE_OK;
}

void sf3d_work_destroy(Sf3dWork *w)
{
    if (!w) return;
    dev_free(w->vec); dev_free(w->part); dev_free(w->gscal); dev_free(w->ctl);
    delete w;
}

int sf3d_enqueue_matvec(cudaStream_t st, const Sf3dSystem &s, double *bt, const double *x, double *r)
{
    const int64_t V = (int64_t)(s.sN + 2) * (s.M + 2) * (s.K + 2) + 1;
    const unsigned blocks = (unsigned)((V + SF3_THREADS - 1) / SF3_THREADS);
    k_sf3d_bt<<<blocks, SF3_THREADS, 0, st>>>(s, x, bt);
    FPDE_LAUNCHED(1);
    k_sf3d_rows<<<blocks, SF3_THREADS, rows_smem(s), st>>>(s, x, bt, r);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int sf3d_enqueue_solve(cudaStream_t st, const Sf3dSystem &s, Sf3dWork *w, const double *B, double *x, double thr,
                       int maxiter, bool exact, unsigned long long *iters_total, int *iters_out, unsigned *flags)
{
    const int64_t V = w->V;
    SolveArgs a;
    a.s = s; a.x = x; a.B = B;
    double *p = w->vec;
    a.r = p; a.q0 = p + V; a.g0 = p + 2 * V; a.g1 = p + 3 * V; a.w0 = p + 4 * V; a.w1 = p + 5 * V;
    a.u = p + 6 * V; a.Au = p + 7 * V; a.bt = p + 8 * V; a.prod = p + 11 * V;
    a.part = w->part; a.gscal = w->gscal;
    a.bar = w->ctl; a.gstop = w->ctl + 2;
    a.flags = flags; a.iters_total = iters_total; a.iters_out = iters_out;
    a.thr = thr; a.maxiter = maxiter;
    FPDE_CUDA(cudaMemsetAsync(w->ctl, 0, 4 * sizeof(unsigned), st));
    const int blocks = exact ? w->blocks_exact : w->blocks_fast;   // fixed at creation (no queries in a capture)
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)blocks);
    cfg.blockDim = dim3(SF3_THREADS);
    cfg.dynamicSmemBytes = rows_smem(s);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaError_t e = exact ? cudaLaunchKernelEx(&cfg, k_sf3d_solve<true>, a) : cudaLaunchKernelEx(&cfg, k_sf3d_solve<false>, a);
    if (e != cudaSuccess) return set_error(FPDE_ERR_CUDA, "space-fractional 3D solve launch: %s", cudaGetErrorString(e));
    count_launches(1);
    return FPDE_OK;
}

// ------------------------------------------------------------- right-hand side of a LOD step

namespace {

// Om of one step of the implicit3d scheme at node v (calc_step :5160-5178 zeroes it, then the lines
// of the K, _M and sN passes add their implicit2_gen right-hand sides, :5302-5606): interior K-line
// nodes -lam U + Rp + history (Om1_impl :4434-4445), the other passes' interior 0.0 (Rp :2730-2733),
// the line ends bc0 / bcN (flux: bcN dLN). Also copies the grid into the solve's initial guess.
__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_rhs(Sf3dRhsArgs a)
{
    const int64_t sy = a.sN + 2, sz = (int64_t)(a.sN + 2) * (a.M + 2), G = sz * (a.K + 2);
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v <= G; v += (int64_t)gridDim.x * blockDim.x) {
        if (v == G) { a.Om[v] = 0.0; continue; }
        const double U = a.U[v];
        a.x[v] = U;
        const int64_t kk = v / sz, rem = v - kk * sz, jj = rem / sy, ii = rem - jj * sy;
        const int i = (int)ii, j = (int)jj, k = (int)kk;
        double om = 0.0;
        const double bcv = a.bc ? a.bc[v] : 0.0;
        if (i >= 1 && i < a.sN && j >= 1 && j < a.M && k <= a.K) {                   // K pass (:5211-5304)
            double o;
            if (k == 0) o = bcv;
            else if (k == a.K) o = a.rkind[2] == FPDE_BC_FLUX ? dm(bcv, a.dLN[2]) : bcv;
            else {
                o = ds(a.rp ? a.rp[v] : 0.0, dm(a.lam, U));
                if (a.KS) {
                    double sv = 0.0;
                    for (int q = 0; q < a.KS; ++q) sv = da(sv, __ldcg(a.part + (int64_t)q * a.pstride + v));
                    o = da(o, sv);
                }
            }
            om = da(om, o);
        }
        if (i >= 1 && i < a.sN && k >= 1 && k < a.K && j <= a.M) {                   // _M pass (:5362-5456)
            double o = 0.0;
            if (j == 0) o = bcv;
            else if (j == a.M) o = a.rkind[1] == FPDE_BC_FLUX ? dm(bcv, a.dLN[1]) : bcv;
            om = da(om, o);
        }
        if (j >= 1 && j < a.M && k >= 1 && k < a.K && i <= a.sN) {                   // sN pass (:5513-5606)
            double o = 0.0;
            if (i == 0) o = bcv;
            else if (i == a.sN) o = a.rkind[0] == FPDE_BC_FLUX ? dm(bcv, a.dLN[0]) : bcv;
            om = da(om, o);
        }
        a.Om[v] = om;
    }
}

__global__ void k_sf3d_store(const double *x, double *U, int64_t G)
{
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < G; v += (int64_t)gridDim.x * blockDim.x)
        U[v] = x[v];
}

}  // namespace

int launch_sf3d_rhs(cudaStream_t st, const Sf3dRhsArgs &a)
{
    const int64_t V = (int64_t)(a.sN + 2) * (a.M + 2) * (a.K + 2) + 1;
    k_sf3d_rhs<<<(unsigned)((V + SF3_THREADS - 1) / SF3_THREADS), SF3_THREADS, 0, st>>>(a);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int launch_sf3d_store(cudaStream_t st, const double *x, double *U, int64_t G)
{
    k_sf3d_store<<<(unsigned)((G + SF3_THREADS - 1) / SF3_THREADS), SF3_THREADS, 0, st>>>(x, U, G);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

// Mat_3d, Mcoefs_3d and the inv_dw_dh planes of a LOD with implicit3d (host, once at creation):
// every line of the K, _M and sN passes adds its implicit2_gen rows (:4630-4663) in that order
// (:5296-5302, :5447-5453, :5597-5603): interior (A_, -(Rlap + the K pass's Da kkk0/tau), B),
// identity rows at the ends and, at a flux end, -1 on the lower neighbour.
void sf3d_assemble_host(int sN, int M, int K, const double *coefA, const double *coefB, const double *coefRlap,
                        const double *const *mc, const double *const *iw, const int *rkind, double lamR,
                        std::vector<double> &mat, std::vector<double> &mc3, std::vector<double> &iw3)
{
    const int64_t sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2), G = sz * (K + 2), V = G + 1;
    mat.assign((size_t)(7 * V), 0.0);
    mc3.assign((size_t)(9 * V), 0.0);
    iw3.assign((size_t)(3 * V), 0.0);
    for (int pass = 2; pass >= 0; --pass) {
        const int Nl = pass == 2 ? K : (pass == 1 ? M : sN);
        const int64_t st = pass == 2 ? sz : (pass == 1 ? sy : 1);
        const int lo = pass == 2 ? 0 : (pass == 1 ? 3 : 5), hi = pass == 2 ? 2 : (pass == 1 ? 4 : 6);
        const int na = pass == 0 ? M : sN, nb = pass == 2 ? M : K;
        const int64_t sa = pass == 0 ? sy : 1, sb = pass == 2 ? sy : sz;
        const double tR = pass == 2 ? lamR : 0.0;
        const double *cA = coefA + (int64_t)pass * G, *cB = coefB + (int64_t)pass * G;
        const double *cR = coefRlap + (int64_t)pass * G;
        for (int la = 1; la < na; ++la)
            for (int lb = 1; lb < nb; ++lb) {
                const int64_t base = la * sa + lb * sb;
                for (int p = 0; p <= Nl; ++p) {
                    const int64_t id = base + p * st;
                    double ml, md, mh;
                    if (p == 0) { ml = 0.0; md = 1.0; mh = 0.0; }
                    else if (p == Nl) { ml = rkind[pass] == FPDE_BC_FLUX ? -1.0 : 0.0; md = 1.0; mh = 0.0; }
                    else {
                        ml = cA[id]; md = -(cR[id] + tR); mh = cB[id];
                        for (int d = 0; d < 3; ++d) mc3[(size_t)((3 * pass + d) * V + id)] = mc[pass][d * G + id];
                        iw3[(size_t)(pass * V + id)] = iw[pass][id];
                    }
                    mat[(size_t)(lo * V + id)] += ml;
                    mat[(size_t)(V + id)] += md;
                    mat[(size_t)(hi * V + id)] += mh;
                }
            }
    }
}

}  // namespace fpde

using namespace fpde;

// ------------------------------------------------------------------------------- C ABI

static int sf3d_call(fpde_ctx *ctx, const fpde_sf3d_system *sys, const double *B, const double *x, double *out,
                     double thr, int maxiter, int exact, int *iters, int on_device, bool solve)
{
    clear_error();
    FPDE_CHECK_ARG(sys && x && out, "null argument");
    FPDE_CHECK_ARG(sys->mat && sys->mc && sys->Tm[0] && sys->Tm[1] && sys->Tm[2], "null operand");
    FPDE_CHECK_ARG(!solve || B, "null right-hand side");
    FPDE_CHECK_ARG(sys->sN >= 1 && sys->M >= 1 && sys->K >= 1 && sys->sN <= FPDE_SF_MAX_N && sys->M <= FPDE_SF_MAX_N &&
                       sys->K <= FPDE_SF_MAX_N,
                   "1 <= sN, M, K <= FPDE_SF_MAX_N");
    FPDE_CHECK_ARG(sys->space_der == 0 || sys->space_der == 1, "space_der must be 0 or 1");
    const int64_t V = (int64_t)(sys->sN + 2) * (sys->M + 2) * (sys->K + 2) + 1;
    FPDE_CHECK_ARG(!solve || (maxiter >= 1 && maxiter <= FPDE_SF_MAX_ITER), "maxiter must be 1 .. FPDE_SF_MAX_ITER");
    FPDE_CHECK_ARG(!solve || !exact || V <= FPDE_SF3D_MAX_EXACT, "exact dot products: at most FPDE_SF3D_MAX_EXACT values");
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    const size_t vec = (size_t)V * sizeof(double);
    std::vector<void *> own;
    auto stage = [&](const double *src, size_t bytes, bool copy_in) -> double * {
        if (on_device) return const_cast<double *>(src);
        void *p = nullptr;
        if (dev_alloc(&p, bytes)) return nullptr;
        own.push_back(p);
        if (copy_in && src) cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, st);
        return (double *)p;
    };
    Sf3dSystem s;
    s.sN = sys->sN; s.M = sys->M; s.K = sys->K; s.sd = sys->space_der;
    s.mat = stage(sys->mat, 7 * vec, true);
    s.mc = stage(sys->mc, 9 * vec, true);
    const int lens[3] = {sys->sN + 1, sys->M + 1, sys->K + 1};
    for (int c = 0; c < 3; ++c) s.Tm[c] = stage(sys->Tm[c], (size_t)lens[c] * sizeof(double), true);
    s.iw = sys->iw ? stage(sys->iw, 3 * vec, true) : nullptr;
    s.rs = sys->rs ? stage(sys->rs, vec, true) : nullptr;
    const double *dB = (solve && B) ? stage(B, vec, true) : nullptr;
    double *dx = stage(x, vec, true);
    double *dout = solve ? dx : stage(out, vec, false);
    bool fail = !s.mat || !s.mc || !s.Tm[0] || !s.Tm[1] || !s.Tm[2] || (sys->iw && !s.iw) || (sys->rs && !s.rs) ||
                (solve && !dB) || !dx || !dout;
    int *d_it = nullptr;
    Sf3dWork *w = nullptr;
    double *bt = nullptr;
    if (!fail && solve) {
        fail = dev_alloc((void **)&d_it, sizeof(int)) != 0;
        if (!fail) {
            own.push_back(d_it);
            if ((rc = sf3d_work_create(s, &w))) fail = true;
        }
    } else if (!fail) {
        fail = dev_alloc((void **)&bt, 3 * vec) != 0;
        if (!fail) own.push_back(bt);
    }
    if (!fail) {
        if (solve) rc = sf3d_enqueue_solve(st, s, w, dB, dx, thr, maxiter, exact != 0, nullptr, d_it, ctx->d_flags);
        else rc = sf3d_enqueue_matvec(st, s, bt, dx, dout);
        if (!rc && !on_device) cudaMemcpyAsync(out, dout, vec, cudaMemcpyDeviceToHost, st);
        if (!rc && iters) cudaMemcpyAsync(iters, d_it, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (!rc) rc = ctx_check_flags(ctx, solve ? "fpde_sf3d_solve" : "fpde_sf3d_matvec");
    } else if (!rc) {
        rc = set_error(FPDE_ERR_NOMEM, "space-fractional 3D: device allocation failed");
    }
    cudaStreamSynchronize(st);
    sf3d_work_destroy(w);
    for (void *p : own) dev_free(p);
    return rc;
}

extern "C" {

int fpde_sf3d_matvec(fpde_ctx *ctx, const fpde_sf3d_system *sys, const double *x, double *r, int on_device)
{
    return sf3d_call(ctx, sys, nullptr, x, r, 0.0, 1, 0, nullptr, on_device, false);
}

int fpde_sf3d_solve(fpde_ctx *ctx, const fpde_sf3d_system *sys, const double *B, double *x, double thr, int maxiter,
                    int exact, int *iters, int on_device)
{
    return sf3d_call(ctx, sys, B, x, x, thr, maxiter, exact, iters, on_device, true);
}

}  // extern "C"
