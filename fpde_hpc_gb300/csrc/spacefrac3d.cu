// The fully implicit 3D space-fractional scheme of fpde_hpc_1d.cpp (implicit3d 1, impl 2,
// toeplitz_mult_alg 0, equation 0): the product vmul_T_3d (:6801-8722) of the 7-diagonal Mat_3d plus,
// along each axis, iw * T * tridiag(Mcoefs_3d[axis]) with T the axis's Toeplitz matrix, and the solve
// solve_mln<1> (:812-1157) that calc_step (:5681-5716) runs on it once per step over the V = G + 1
// values of the grid (G = (sN+2)(M+2)(K+2) nodes, i fastest, plus the one past the grid).
//
// The product runs in two phases. In the first a warp owns one line of one axis: it forms the
// line's Bt = tridiag(Mcoefs_3d[axis]) x in shared memory and each lane sums the Toeplitz terms of
// two rows (p and n - p, so every lane runs a chain of equal length), each term one lane's
// sequential sum without contracted multiply-adds. The second forms every output in the reference's
// order: the seven diagonals with its flat-index bounds, then the K, _M and sN terms. So a product
// equals the reference's bit for bit. All vectors are node-major and stay in L2 for the grids this
// scheme is run on (a 64^3 grid is 2.3 MB per vector); the sums are FP64-pipe work.
//
// A solve is one persistent cooperative kernel: every thread owns a fixed set of nodes, the vector
// updates need no synchronisation, and a bounded grid barrier separates the phases whose reads cross
// nodes (the two phases of a product, and each dot product). Dot products come in two forms:
//   exact: every product a[v]*b[v] is stored and one thread adds them in index order (the
//          reference's loop), so the iterates, the iteration count and the solution are the
//          reference's bit for bit; the add chain runs on one thread (use on small grids);
//   fast:  each thread adds its nodes, each CTA folds its threads in a fixed tree and every CTA
//          folds the CTA partials in the same fixed order, so the result is deterministic and
//          identical in every CTA, and differs from the reference's only by the order of the adds;
//          every product that feeds a sum (the Toeplitz terms, the diagonals, Bt, the updates, the dot
//          partials) is a fused multiply-add (one FP64 instruction instead of two, on the pipe the
//          solve is bound by; one rounding instead of two).
#include <algorithm>
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
// c + a*b and c - a*b: fused (one rounding, the fast solve) or the reference's rounded product and sum
template <bool F> __device__ __forceinline__ double madd(double a, double b, double c)
{
    return F ? fma(a, b, c) : da(c, dm(a, b));
}
template <bool F> __device__ __forceinline__ double msub(double c, double a, double b)
{
    return F ? fma(-a, b, c) : ds(c, dm(a, b));
}

#ifndef SF3_MIN_CTAS
#define SF3_MIN_CTAS 2        // co-resident CTAs per SM the solve's register budget is cut for (2 measured
                              // fastest on 64^3: 3 and 4 per SM, with spills, were 16 % and 19 % slower)
#endif
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
    const unsigned u = (unsigned)v, sz = (unsigned)g.sz, sy = (unsigned)g.sy;   // V < 2^31
    const unsigned kk = u / sz, rem = u - kk * sz;
    const unsigned jj = rem / sy, ii = rem - jj * sy;
    *i = (int)ii; *j = (int)jj; *k = (int)kk;
    return ii >= 1 && (int)ii < g.sN && jj >= 1 && (int)jj < g.M && kk >= 1 && (int)kk < g.K;
}

// The lines of the product's Toeplitz terms: axis 2 (K) over (i, j), axis 1 (_M) over (i, k), axis 0
// (sN) over (j, k), each coordinate 1..len-1, an axis only when it has more than 2 intervals. Line l
// of the concatenation as its axis, first node (position 0) and node stride.
struct LineSet {
    int64_t n2, n1, n0;                  // lines of each axis
};
__device__ __forceinline__ LineSet lines_of(const Geo &g)
{
    LineSet L;
    L.n2 = g.K > 2 ? (int64_t)(g.sN - 1) * (g.M - 1) : 0;
    L.n1 = g.M > 2 ? (int64_t)(g.sN - 1) * (g.K - 1) : 0;
    L.n0 = g.sN > 2 ? (int64_t)(g.M - 1) * (g.K - 1) : 0;
    return L;
}
__device__ __forceinline__ void line_at(const Geo &g, const LineSet &L, int64_t l, int *c, int64_t *base,
                                        int64_t *st, int *n)
{
    unsigned u = (unsigned)l;
    if (l < L.n2) {
        const unsigned d = (unsigned)(g.sN - 1), b = u / d, i = 1 + u - b * d, j = 1 + b;
        *c = 2; *base = i + (int64_t)j * g.sy; *st = g.sz; *n = g.K;
    } else if (l < L.n2 + L.n1) {
        u -= (unsigned)L.n2;
        const unsigned d = (unsigned)(g.sN - 1), b = u / d, i = 1 + u - b * d, k = 1 + b;
        *c = 1; *base = i + (int64_t)k * g.sz; *st = g.sy; *n = g.M;
    } else {
        u -= (unsigned)(L.n2 + L.n1);
        const unsigned d = (unsigned)(g.M - 1), b = u / d, j = 1 + u - b * d, k = 1 + b;
        *c = 0; *base = (int64_t)j * g.sy + (int64_t)k * g.sz; *st = 1; *n = g.sN;
    }
}

// One warp, one line of axis c (FUSED: each term a fused multiply-add, the fast solve's form; else
// the reference's separately rounded product and sum): Bt = tridiag(Mcoefs_3d[c]) x at positions 1..n-1 (:7254-7261,
// :7677-7684, :8097-8104: the diagonal term, then the lower and the upper neighbour along the axis)
// into the warp's shared slice, then every row's Toeplitz term (:7562-7574 and the other axes):
// the sum over j < p in increasing j, then (two-sided) the subtraction over j > p, one lane's
// sequential chain per row, row scaling and inv_dw_dh as the reference applies them; tc[c][node] =
// the term. A lane takes the rows p and n - p (one-sided: p - 1 and n - p - 1 terms, n - 2 together;
// two-sided: n - 2 each), so the lanes of a warp run equal chains.
template <bool FUSED>
__device__ __forceinline__ void line_terms(const Sf3dSystem &s, const Geo &g, const double *rows, double *sl,
                                           const double *x, double *tc, int c, int64_t base, int64_t st, int n)
{
    const int lane = threadIdx.x & 31;
    const int64_t V = g.V;
    const double *mc = s.mc + (int64_t)(3 * c) * V;
    for (int q = 1 + lane; q < n; q += 32) {
        const int64_t v = base + (int64_t)q * st;
        double b = dm(__ldg(mc + V + v), __ldcg(x + v));
        b = madd<FUSED>(__ldg(mc + v), __ldcg(x + v - st), b);
        b = madd<FUSED>(__ldg(mc + 2 * V + v), __ldcg(x + v + st), b);
        sl[q] = b;
    }
    __syncwarp();
    // row c of the Toeplitz rows and of their negated copy (load_rows): a term subtracted is the
    // product with -Tm, the same rounding as the subtraction of the product
    const int off = c == 0 ? 0 : (c == 1 ? g.sN + 1 : g.sN + g.M + 2);
    const double *Tp = rows + off, *Tn = rows + (g.sN + g.M + g.K + 3) + off;
    const double *iw = s.iw ? s.iw + (int64_t)c * V : nullptr;
    double *out = tc + (int64_t)c * V;
    const int pairs = n / 2;                                 // rows 1..n-1 as (k+1, n-1-k)
    for (int k = lane; k < pairs; k += 32) {
        const int a = k + 1, b = n - 1 - k;
        const int na = s.sd ? n - 2 : a - 1;
        const int nb = a == b ? 0 : (s.sd ? n - 2 : b - 1);
        // the lane's terms in up to four runs of consecutive j: row a below (j = 1..a-1, Tm[a-j+1]),
        // row a above (two-sided: j = a+1..n-1, -Tm[j-a+1]), then the same for row b
        double t = 0.0, ta = 0.0;
        int seg = 0, q = 1, ti = a, dti = -1, cnt = a - 1;
        const double *T = Tp;
        for (int r = 0; r < na + nb; ++r) {
            while (cnt == 0 && seg < 3) {
                ++seg;
                if (seg == 1) { q = a + 1; ti = 2; dti = 1; T = Tn; cnt = s.sd ? n - 1 - a : 0; }
                else if (seg == 2) { ta = t; t = 0.0; q = 1; ti = b; dti = -1; T = Tp; cnt = b - 1; }
                else { q = b + 1; ti = 2; dti = 1; T = Tn; cnt = s.sd ? n - 1 - b : 0; }
            }
            if (FUSED) t = fma(sl[q], T[ti], t);             // one rounding per term
            else t = da(t, dm(sl[q], T[ti]));
            ++q; ti += dti; --cnt;
        }
        double tb = t;
        if (nb == 0) ta = t;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            if (h == 1 && nb == 0) break;
            const int p = h == 0 ? a : b;
            const int64_t v = base + (int64_t)p * st;
            double val = h == 0 ? ta : tb;
            if (s.rs) val = __ddiv_rn(val, __ldg(s.rs + v));
            out[v] = iw ? dm(val, __ldg(iw + v)) : val;
        }
    }
    __syncwarp();
}

// Output v of the product (:6857-6877), then the K, _M and sN terms in that order at the nodes
// inside 1..len-1 on every axis (FUSED: the diagonals' products fused into their sums).
template <bool FUSED>
__device__ __forceinline__ double row_node(const Sf3dSystem &s, const Geo &g, const double *x, const double *tc,
                                           int64_t v)
{
    const int64_t V = g.V;
    const double *M = s.mat;
    double r = dm(__ldg(M + V + v), __ldcg(x + v));
    if (g.sN > 2) {
        if (v - 1 >= 0) r = madd<FUSED>(__ldg(M + 5 * V + v), __ldcg(x + v - 1), r);
        if (v + 1 < V) r = madd<FUSED>(__ldg(M + 6 * V + v), __ldcg(x + v + 1), r);
    }
    if (g.M > 2) {
        if (v - g.sy >= 0) r = madd<FUSED>(__ldg(M + 3 * V + v), __ldcg(x + v - g.sy), r);
        if (v + g.sy < V) r = madd<FUSED>(__ldg(M + 4 * V + v), __ldcg(x + v + g.sy), r);
    }
    if (g.K > 2) {
        if (v - g.sz >= 0) r = madd<FUSED>(__ldg(M + v), __ldcg(x + v - g.sz), r);
        if (v + g.sz < V) r = madd<FUSED>(__ldg(M + 2 * V + v), __ldcg(x + v + g.sz), r);
    }
    int i, j, k;
    if (!interior(g, v, &i, &j, &k)) return r;
    if (g.K > 2) r = da(r, __ldcg(tc + 2 * V + v));
    if (g.M > 2) r = da(r, __ldcg(tc + V + v));
    if (g.sN > 2) r = da(r, __ldcg(tc + v));
    return r;
}

// Shared memory of a CTA: the three Toeplitz rows (lengths sN, M, K + 1; entries 2..len-1 are read)
// and their negated copy, then one line slice of max(sN, M, K) + 1 values per warp.
__device__ __forceinline__ double *load_rows(const Sf3dSystem &s, double *sm)
{
    const int n0 = s.sN + 1, n1 = s.M + 1, n2 = s.K + 1, nr = n0 + n1 + n2;
    for (int q = threadIdx.x; q < nr; q += blockDim.x) {
        double v;
        if (q < n0) v = s.Tm[0][q];
        else if (q < n0 + n1) v = s.Tm[1][q - n0];
        else v = s.Tm[2][q - n0 - n1];
        sm[q] = v;
        sm[nr + q] = -v;
    }
    __syncthreads();
    const int nmax = max(s.sN, max(s.M, s.K));
    return sm + 2 * nr + (size_t)(threadIdx.x >> 5) * (nmax + 1);
}

// -------------------------------------------------------------------- standalone product

__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_terms(Sf3dSystem s, const double *x, double *tc)
{
    extern __shared__ double sf3_sm[];
    double *sl = load_rows(s, sf3_sm);
    const Geo g = geo_of(s);
    const LineSet L = lines_of(g);
    const int64_t nl = L.n2 + L.n1 + L.n0;
    const int64_t w0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5, W = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t l = w0; l < nl; l += W) {
        int c, n;
        int64_t base, st;
        line_at(g, L, l, &c, &base, &st, &n);
        line_terms<false>(s, g, sf3_sm, sl, x, tc, c, base, st, n);
    }
}

__global__ void __launch_bounds__(SF3_THREADS) k_sf3d_rows(Sf3dSystem s, const double *x, const double *tc, double *r)
{
    const Geo g = geo_of(s);
    for (int64_t v = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; v < g.V; v += (int64_t)gridDim.x * blockDim.x)
        r[v] = row_node<false>(s, g, x, tc, v);
}

// -------------------------------------------------------------------------- the solve

struct SolveArgs {
    Sf3dSystem s;
    double *x;                 // initial guess in, solution out
    const double *B;
    double *r, *q0, *g0, *g1, *w0, *w1, *u, *Au, *tc;   // V each (tc: the axes' terms, 3V)
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
    const double *rows;        // the Toeplitz rows (shared)
    double *sl;                // the warp's line slice (shared)
    int64_t gt, GT;
    double *wsum;              // shared: 2 x SF3_WARPS
    double *res;               // shared: 2

    __device__ bool sync() { return grid_barrier(a.bar, gridDim.x, a.flags); }

    // y = A x: the lines' Toeplitz terms (a warp per line), a barrier, the rows; the caller has
    // synchronised x.
    __device__ bool apply(const double *x, double *y)
    {
        const LineSet L = lines_of(g);
        const int64_t nl = L.n2 + L.n1 + L.n0;
        for (int64_t l = gt >> 5; l < nl; l += GT >> 5) {
            int c, n;
            int64_t base, st;
            line_at(g, L, l, &c, &base, &st, &n);
            line_terms<!EXACT>(a.s, g, rows, sl, x, a.tc, c, base, st, n);
        }
        if (!sync()) return false;
        for (int64_t v = gt; v < g.V; v += GT) y[v] = row_node<!EXACT>(a.s, g, x, a.tc, v);
        return true;
    }

    // The term x*y of dot product Q: exact stores the rounded product, fast fuses it into (NEG: out
    // of) the thread's partial.
    template <int Q, bool NEG>
    __device__ __forceinline__ void term(int64_t v, double x, double y, double &acc)
    {
        if (EXACT) a.prod[(int64_t)Q * g.V + v] = dm(x, y);
        else acc = NEG ? fma(-x, y, acc) : fma(x, y, acc);
    }

    // Dot product slot q of a CTA (fast form): fold the threads' partials in a fixed tree.
    __device__ __forceinline__ void fold_cta(int q, double t)
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) t = da(t, __shfl_down_sync(0xffffffffu, t, o));
        if (lane == 0) wsum[q * SF3_WARPS + warp] = t;
    }

    // The ND dot products whose terms every thread has just produced (acc0, acc1: the thread's
    // partials in the fast form); o0, o1 in every thread. NEG0: the first is the reference's
    // "beta -= q*r" (terms subtracted from 0.0).
    template <int ND, bool NEG0>
    __device__ bool dots(double acc0, double acc1, double &o0, double &o1)
    {
        const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
        if (EXACT) {
            if (!sync()) return false;
            if (blockIdx.x == 0 && lane == 0 && warp < ND) {
                const double *p = a.prod + (int64_t)warp * g.V;
                double t = 0.0;
                if (NEG0 && warp == 0)
                    for (int64_t v = 0; v < g.V; ++v) t = ds(t, __ldcg(p + v));
                else
                    for (int64_t v = 0; v < g.V; ++v) t = da(t, __ldcg(p + v));
                a.gscal[warp] = t;
            }
            if (!sync()) return false;
            if (tid < ND) res[tid] = __ldcg(a.gscal + tid);
            __syncthreads();
        } else {
            fold_cta(0, acc0);
            if (ND > 1) fold_cta(1, acc1);
            __syncthreads();
            if (tid < ND) {
                double t = 0.0;
                for (int w = 0; w < SF3_WARPS; ++w) t = da(t, wsum[tid * SF3_WARPS + w]);
                a.part[(int64_t)tid * gridDim.x + blockIdx.x] = t;
            }
            if (!sync()) return false;
            if (warp < ND) {
                const double *p = a.part + (int64_t)warp * gridDim.x;
                double t = 0.0;
                for (unsigned b = lane; b < gridDim.x; b += 32) t = da(t, __ldcg(p + b));
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) t = da(t, __shfl_down_sync(0xffffffffu, t, o));
                if (lane == 0) res[warp] = t;
            }
            __syncthreads();
        }
        o0 = res[0];
        if (ND > 1) o1 = res[1];
        __syncthreads();
        return true;
    }
};

// solve_mln<1> over the V values, the grid form of the per-line solve of spacefrac.cu (the same
// sequence of products, dot products, divisions and tests: :841-866 at a start, :871-1132 per
// iteration with the q.r reuse and the w/g shift). A start repeated more than maxiter times without
// an iteration between, the time limit or a barrier that times out ends the solve with a flag.
template <bool EXACT>
__global__ void __launch_bounds__(SF3_THREADS, SF3_MIN_CTAS) k_sf3d_solve(SolveArgs a)
{
    extern __shared__ double sf3_sm[];
    __shared__ double wsum[2 * SF3_WARPS];
    __shared__ double res[2];
    __shared__ unsigned stop_s;
    Solver<EXACT> S{a};
    S.rows = sf3_sm;
    S.sl = load_rows(a.s, sf3_sm);
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
    double c1 = 0.0, al = 0.0, o0 = 0.0, o1 = 0.0, acc0, acc1;
    int iter = 1, restarts = 0;
    bool have_qr = false;
restart:
    if (++restarts > a.maxiter + 1) {
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, DEVERR_SOLVER);
        goto out;
    }
    have_qr = false;
    if (!S.apply(x, r)) return;                                                       // :841-844
    acc0 = 0.0;
    for (int64_t v = gt; v < V; v += GT) {
        const double e = ds(B[v], r[v]);
        r[v] = e; g1[v] = e; q0[v] = e;
        S.template term<0, false>(v, e, e, acc0);                                 // norm (:864)
    }
    if (blockIdx.x == 0 && threadIdx.x == 0 && gtimer_ns() - t0 > SF3_TIME_LIMIT_NS) atomicExch(a.gstop, 1u);
    if (!S.template dots<1, false>(acc0, 0.0, o0, o1)) return;
    if (threadIdx.x == 0) stop_s = __ldcg(a.gstop);
    __syncthreads();
    if (stop_s) {                                                                     // restarts past the limit
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(a.flags, DEVERR_SOLVER);
        goto out;
    }
    {
        const double norm = o0;
        if (!S.apply(g1, w1)) return;                                                 // :851
        acc0 = 0.0;
        for (int64_t v = gt; v < V; v += GT) S.template term<0, false>(v, q0[v], w1[v], acc0);   // c[1]
        if (!S.template dots<1, false>(acc0, 0.0, o0, o1)) return;
        c1 = o0;
        if (fabs(__ddiv_rn(norm, md)) < a.thr) goto out;                               // :866
    }
    for (;;) {
        if (!have_qr) {                                                                // :871-877
            acc0 = 0.0;
            for (int64_t v = gt; v < V; v += GT) S.template term<0, false>(v, q0[v], r[v], acc0);
            if (!S.template dots<1, false>(acc0, 0.0, o0, o1)) return;
            al = __ddiv_rn(o0, c1);
        }
        if (!(c1 != 0.0)) goto restart;                                                // :878, :913
        for (int64_t v = gt; v < V; v += GT) {
            u[v] = msub<!EXACT>(r[v], al, w1[v]);
            x[v] = madd<!EXACT>(al, g1[v], x[v]);
        }
        if (!S.sync()) return;
        if (!S.apply(u, Au)) return;                                                  // :890
        acc0 = acc1 = 0.0;
        for (int64_t v = gt; v < V; v += GT) {
            const double av = Au[v];
            S.template term<0, false>(v, av, av, acc0);
            S.template term<1, false>(v, av, u[v], acc1);
        }
        if (!S.template dots<2, false>(acc0, acc1, o0, o1)) return;
        const double nrm = o0;
        const double ro1 = __ddiv_rn(-o1, nrm);                                       // :903
        if (nrm == 0.0) goto restart;                                                  // :904-905
        for (int64_t v = gt; v < V; v += GT) x[v] = msub<!EXACT>(x[v], ro1, u[v]);
        if (!S.sync()) return;
        if (!S.apply(x, r)) return;                                                   // :943-947
        acc0 = acc1 = 0.0;
        for (int64_t v = gt; v < V; v += GT) {
            const double e = ds(B[v], r[v]);
            r[v] = e;
            S.template term<0, true>(v, q0[v], e, acc0);                         // beta's q.r (:1056-1059)
            S.template term<1, false>(v, e, e, acc1);                             // r.r (:1127)
        }
        if (!S.template dots<2, true>(acc0, acc1, o0, o1)) return;
        const double nq = o0, norm = o1;
        double beta = __ddiv_rn(nq, c1);                                               // :1060-1065
        if (c1 == 0.0) beta = 0.0;
        const double bro = __ddiv_rn(beta, ro1);
        for (int64_t v = gt; v < V; v += GT) {
            const double zw = madd<!EXACT>(beta, w1[v], r[v]);
            g0[v] = madd<!EXACT>(bro, g1[v], zw);
        }
        if (!S.sync()) return;
        if (!S.apply(g0, w0)) return;                                                 // :1094
        acc0 = 0.0;
        for (int64_t v = gt; v < V; v += GT) S.template term<0, false>(v, q0[v], w0[v], acc0);   // c[0]
        if (blockIdx.x == 0 && threadIdx.x == 0 && gtimer_ns() - t0 > SF3_TIME_LIMIT_NS) atomicExch(a.gstop, 1u);
        if (!S.template dots<1, false>(acc0, 0.0, o0, o1)) return;
        if (threadIdx.x == 0) stop_s = __ldcg(a.gstop);
        __syncthreads();
        c1 = o0;                                                                       // the shift :1104-1121
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

size_t rows_smem(const Sf3dSystem &s)
{
    const int nmax = std::max(s.sN, std::max(s.M, s.K));
    return (size_t)(2 * (s.sN + s.M + s.K + 3) + SF3_WARPS * (nmax + 1)) * sizeof(double);
}
// The opt-in is made once per kernel and device, so for the largest axes allowed (157 KB).
constexpr int SF3_SMEM_MAX = (6 * (FPDE_SF_MAX_N + 1) + SF3_WARPS * (FPDE_SF_MAX_N + 1)) * (int)sizeof(double);

}  // namespace

// ------------------------------------------------------------------ workspace and launches

struct Sf3dWork {
    int64_t V = 0;
    int blocks = 0;                      // the larger of the two
    int blocks_fast = 0, blocks_exact = 0;   // CTAs of each solve form (all co-resident)
    double *vec = nullptr;               // r q0 g0 g1 w0 w1 u Au, tc (3V), prod (2V)
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
    FPDE_CUDA(exact ? smem_opt_in((const void *)k_sf3d_solve<true>, SF3_SMEM_MAX)
                    : smem_opt_in((const void *)k_sf3d_solve<false>, SF3_SMEM_MAX));
    if (exact) FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sf3d_solve<true>, SF3_THREADS, smem));
    else FPDE_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_sf3d_solve<false>, SF3_THREADS, smem));
    if (per < 1) return set_error(FPDE_ERR_CUDA, "space-fractional 3D solve: no co-resident CTA fits");
    // one thread per value or one warp per line, whichever asks more CTAs, at most all co-resident
    const int64_t lines = (int64_t)(s.sN + 1) * (s.M + 1) + (int64_t)(s.sN + 1) * (s.K + 1) + (int64_t)(s.M + 1) * (s.K + 1);
    const int64_t need = std::max((V + SF3_THREADS - 1) / SF3_THREADS, (lines + SF3_WARPS - 1) / SF3_WARPS);
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

int sf3d_enqueue_matvec(cudaStream_t st, const Sf3dSystem &s, double *tc, const double *x, double *r)
{
    const int64_t V = (int64_t)(s.sN + 2) * (s.M + 2) * (s.K + 2) + 1;
    const unsigned blocks = (unsigned)((V + SF3_THREADS - 1) / SF3_THREADS);
    const int64_t lines = (int64_t)(s.sN + 1) * (s.M + 1) + (int64_t)(s.sN + 1) * (s.K + 1) + (int64_t)(s.M + 1) * (s.K + 1);
    const unsigned tblocks = (unsigned)std::max<int64_t>(1, (lines + SF3_WARPS - 1) / SF3_WARPS);
    FPDE_CUDA(smem_opt_in((const void *)k_sf3d_terms, SF3_SMEM_MAX));
    k_sf3d_terms<<<tblocks, SF3_THREADS, rows_smem(s), st>>>(s, x, tc);
    FPDE_LAUNCHED(1);
    k_sf3d_rows<<<blocks, SF3_THREADS, 0, st>>>(s, x, tc, r);
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
    a.u = p + 6 * V; a.Au = p + 7 * V; a.tc = p + 8 * V; a.prod = p + 11 * V;
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
    FPDE_CHECK_ARG(V < ((int64_t)1 << 31), "(sN+2)(M+2)(K+2) + 1 must be below 2^31");
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
    double *tc = nullptr;
    if (!fail && solve) {
        fail = dev_alloc((void **)&d_it, sizeof(int)) != 0;
        if (!fail) {
            own.push_back(d_it);
            if ((rc = sf3d_work_create(s, &w))) fail = true;
        }
    } else if (!fail) {
        fail = dev_alloc((void **)&tc, 3 * vec) != 0;
        if (!fail) own.push_back(tc);
    }
    if (!fail) {
        if (solve) rc = sf3d_enqueue_solve(st, s, w, dB, dx, thr, maxiter, exact != 0, nullptr, d_it, ctx->d_flags);
        else rc = sf3d_enqueue_matvec(st, s, tc, dx, dout);
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
