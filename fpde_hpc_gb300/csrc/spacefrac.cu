// The implicit space-fractional operator of fpde_hpc_1d.cpp (impl 2, toeplitz_mult_alg 0): the
// product vmul_T (:6618-6747) of tridiag(Mat) + iw * T * tridiag(Mcoefs), with T the Toeplitz
// matrix of the space-fractional integral (row Tm, one- or two-sided), and the solver solve_mln<1>
// (:812-1157) that U1 (:4769-4791) runs on it for every line of every pass.
//
// One CTA owns one line: the line's operands and the solver's vectors live in shared memory, every
// product and every vector update is spread over the CTA's threads, and each CTA iterates to its
// own convergence. Every value is formed with the reference's operations in the reference's order
// and without contracted multiply-adds (its x86-64 build rounds each product): each output of the
// product is one thread's sequential sum over j, and each dot product one thread's sequential sum
// over the line, so the iterates, the iteration count and the solution equal the reference's bit
// for bit on the same inputs. Products and dot products are FP64-pipe work (GB300: about two FP64
// lanes per cycle per SM), so a pass keeps many lines in flight per SM (20 vectors of n+1 doubles
// per CTA: 21 KB at n = 128).
#include <cmath>
#include <vector>

#include "common.cuh"
#include "kernels.cuh"
#include "scan.cuh"

namespace fpde {

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double ds(double a, double b) { return __dsub_rn(a, b); }

// Shared-memory vectors of one line, n+1 doubles each.
struct SfVec {
    double *Tm, *m0, *m1, *m2, *c0, *c1, *c2, *iw, *rs, *B, *x, *r, *q0, *g0, *g1, *w0, *w1, *u, *Au, *bt;
};
constexpr int SF_NVEC = 20;
constexpr int SF_THREADS = 128;   // (64-thread CTAs for short lines measured no faster on 64^3)
constexpr uint64_t SF_TIME_LIMIT_NS = 10ull * 1000000000ull;   // per line solve

__device__ __forceinline__ SfVec sf_carve(double *sm, int m)
{
    SfVec v;
    double **f[SF_NVEC] = {&v.Tm, &v.m0, &v.m1, &v.m2, &v.c0, &v.c1, &v.c2, &v.iw, &v.rs, &v.B,
                           &v.x,  &v.r,  &v.q0, &v.g0, &v.g1, &v.w0, &v.w1, &v.u,  &v.Au, &v.bt};
#pragma unroll
    for (int k = 0; k < SF_NVEC; ++k) *f[k] = sm + (size_t)k * m;
    return v;
}

// The Toeplitz sums of one lane's rows a = k+1 and b = n-1-k as chains of n-2 terms for every lane
// of the warp (kw: the largest k among the warp's lanes). Row a has k lower terms and row b n-2-k;
// the lane runs row a's and then the first kw-k of row b's (kw steps), then row b's other n-2-kw
// (the same count on every lane), so no lane idles in a longer loop of its partner. Two-sided: the
// upper terms (row b has k, row a n-2-k) follow in the same way with the rows swapped, each chain
// continuing from its row's lower sum. Each row's sum is its own chain over its terms in the
// reference's order (j rising, lower then upper): EXACT adds the rounded products in turn
// (da/ds of dm, bit for bit the reference's row sums); the fast form fuses each term (fma).
template <bool EXACT>
__device__ __forceinline__ void sf_pair(const double *__restrict__ bt, const double *__restrict__ Tm, int n, int sd,
                                        int k, int kw, double &va, double &vb)
{
    const int a = k + 1, b = n - 1 - k;
    const double *pb = bt + 1, *pt = Tm + a;
    double v = 0.0, w = 0.0;
    for (int t = 0; t < kw; ++t) {
        if (t == k) { w = v; v = 0.0; pb = bt + 1; pt = Tm + b; }
        v = EXACT ? da(v, dm(*pb, *pt)) : fma(*pb, *pt, v);
        ++pb; --pt;
    }
    if (k == kw) { w = v; v = 0.0; pb = bt + 1; pt = Tm + b; }
    for (int t = kw; t < n - 2; ++t) {
        v = EXACT ? da(v, dm(*pb, *pt)) : fma(*pb, *pt, v);
        ++pb; --pt;
    }
    // w: row a's lower sum, v: row b's
    if (sd) {
        pb = bt + b + 1; pt = Tm + 2;
        for (int t = 0; t < kw; ++t) {
            if (t == k) { const double y = v; v = w; w = y; pb = bt + a + 1; pt = Tm + 2; }
            v = EXACT ? ds(v, dm(*pb, *pt)) : fma(-*pb, *pt, v);
            ++pb; ++pt;
        }
        if (k == kw) { const double y = v; v = w; w = y; pb = bt + a + 1; pt = Tm + 2; }
        for (int t = kw; t < n - 2; ++t) {
            v = EXACT ? ds(v, dm(*pb, *pt)) : fma(-*pb, *pt, v);
            ++pb; ++pt;
        }
        va = v; vb = w;   // row a's chain ends the upper pass, row b's was set aside at the swap
    } else {
        va = w; vb = v;
    }
}

// Row i (1..n-1) of vmul_T from its Toeplitz sum v (sf_pair<true>): the tridiagonal part, then v,
// in the reference's order of operations.
__device__ __forceinline__ double sf_row_exact(const SfVec &s, bool has_iw, bool has_rs, const double *xv, int i,
                                               double v)
{
    const double r = da(da(dm(s.m0[i], xv[i - 1]), dm(s.m1[i], xv[i])), dm(s.m2[i], xv[i + 1]));
    if (has_rs) v = __ddiv_rn(v, s.rs[i]);
    return da(r, has_iw ? dm(v, s.iw[i]) : v);
}

// rv = vmul_T(xv) on the line's operands (:6662-6686). All threads; ends with a barrier. A thread
// takes the pair of rows k+1 and n-1-k as one chain of n-2 terms (sf_pair). When side is given, the
// CTA's last thread also forms *side_out = the sequential sum of the m products in side (one of the
// reference's dot products), overlapping it with the rows; the second-to-last thread forms the two
// boundary rows.
__device__ void sf_apply(const SfVec &s, int n, int sd, bool has_iw, bool has_rs, const double *xv, double *rv,
                         const double *side = nullptr, double *side_out = nullptr)
{
    const int T = blockDim.x, tid = threadIdx.x;
    for (int j = 1 + tid; j < n; j += T)
        s.bt[j] = da(da(dm(s.c0[j], xv[j - 1]), dm(s.c1[j], xv[j])), dm(s.c2[j], xv[j + 1]));
    __syncthreads();
    if (side && tid == T - 1) {
        double a = 0.0;
        for (int i = 0; i <= n; ++i) a = da(a, side[i]);
        *side_out = a;
    }
    if (tid == T - 2) {
        rv[0] = da(dm(s.m1[0], xv[0]), dm(s.m2[0], xv[1]));
        rv[n] = da(dm(s.m0[n], xv[n - 1]), dm(s.m1[n], xv[n]));
    }
    const int pairs = n / 2;
    for (int k = tid; k < pairs; k += T) {
        const int kw = min(k - (tid & 31) + 31, pairs - 1);   // the warp's largest k (T is a multiple of 32)
        const int a = k + 1, b = n - 1 - k;
        double va, vb;
        sf_pair<true>(s.bt, s.Tm, n, sd, k, kw, va, vb);
        rv[a] = sf_row_exact(s, has_iw, has_rs, xv, a, va);
        if (b != a) rv[b] = sf_row_exact(s, has_iw, has_rs, xv, b, vb);
    }
    __syncthreads();
}

// The reference's dot products (:860-1102) accumulate a[i]*b[i] from 0.0 in index order, each
// product rounded. The products are formed by all threads into a scratch vector; one thread adds
// them in order (sf_sum), or subtracts them in order for beta's "beta -= q*r" (sf_negsum): the
// same roundings as the reference's loop.
__device__ __forceinline__ double sf_sum(const double *p, int m)
{
    double s = 0.0;
    for (int i = 0; i < m; ++i) s = da(s, p[i]);
    return s;
}
__device__ __forceinline__ double sf_negsum(const double *p, int m)
{
    double s = 0.0;
    for (int i = 0; i < m; ++i) s = ds(s, p[i]);
    return s;
}

// solve_mln<1> on the line in s (x: initial guess in, solution out). All threads; returns the
// iteration count. The scalars (dot products, divisions, the convergence test) are formed by
// thread 0 and read by all after a barrier, so the FP64 pipe runs each once. Scratch: bt (free
// outside sf_apply's first phase), u and g0 where the iteration does not hold them. q.r of an
// iteration equals minus the previous iteration's beta numerator (same r, and a sum subtracted
// from 0.0 in order is the negated sum added: rounding to nearest is symmetric), so it is reused
// unless that numerator was zero (whose sign could differ). A solve that restarts more than
// maxiter times without an iteration in between, or runs past the time limit, stops and sets
// DEVERR_SOLVER.
//   scal: 0 c1, 1 norm (r.r), 2 al, 3 ro1, 4 ro sum (Au.u), 5 beta, 6 beta/ro1, 7 norm at the
//   iteration's end, 8 state (0 go on, 1 converged, 2 restart, 3 time limit), 9 q.r numerator
__device__ int sf_solve_cta(SfVec s, int n, int sd, bool has_iw, bool has_rs, double thr, int maxiter,
                            double *scal, unsigned *flags)
{
    const int m = n + 1, T = blockDim.x, tid = threadIdx.x;
    const double md = (double)m;
    const unsigned long long t0 = gtimer_ns();
    int iter = 1, restarts = 0;
    bool have_qr = false;
restart:
    if (++restarts > maxiter + 1) {
        if (tid == 0) atomicOr(flags, DEVERR_SOLVER);
        return iter;
    }
    have_qr = false;
    sf_apply(s, n, sd, has_iw, has_rs, s.x, s.r);                            // :841-844
    for (int i = tid; i < m; i += T) {
        const double v = ds(s.B[i], s.r[i]);
        s.r[i] = v;
        s.g1[i] = v;
        s.q0[i] = v;
        s.u[i] = dm(v, v);                                                   // r.r products (:864)
    }
    __syncthreads();
    sf_apply(s, n, sd, has_iw, has_rs, s.g1, s.w1, s.u, &scal[1]);           // :851, norm on the side
    for (int i = tid; i < m; i += T) s.bt[i] = dm(s.q0[i], s.w1[i]);         // c[1] = q0.w1 (:853-856)
    __syncthreads();
    if (tid == 0) {
        scal[0] = sf_sum(s.bt, m);
        scal[8] = fabs(__ddiv_rn(scal[1], md)) < thr ? 1.0 : 0.0;           // :866
    }
    __syncthreads();
    if (scal[8] != 0.0) return iter;
    for (;;) {
        if (!have_qr) {                                                        // :871-877
            for (int i = tid; i < m; i += T) s.bt[i] = dm(s.q0[i], s.r[i]);
            __syncthreads();
            if (tid == 0) scal[2] = __ddiv_rn(sf_sum(s.bt, m), scal[0]);
            __syncthreads();
        }
        if (!(scal[0] != 0.0)) goto restart;                                   // c[1] (:878, :913)
        {
            const double al = scal[2];
            for (int i = tid; i < m; i += T) {
                s.u[i] = ds(s.r[i], dm(al, s.w1[i]));
                s.x[i] = da(s.x[i], dm(al, s.g1[i]));
            }
        }
        __syncthreads();
        sf_apply(s, n, sd, has_iw, has_rs, s.u, s.Au);                       // :890
        for (int i = tid; i < m; i += T) {
            s.bt[i] = dm(s.Au[i], s.Au[i]);
            s.g0[i] = dm(s.Au[i], s.u[i]);                                   // g0 is free until :1091
        }
        __syncthreads();
        if (tid == 0) scal[1] = sf_sum(s.bt, m);
        if (tid == 32 % T) scal[4] = sf_sum(s.g0, m);
        __syncthreads();
        if (tid == 0) scal[3] = __ddiv_rn(-scal[4], scal[1]);                 // ro1 (:903)
        __syncthreads();
        if (scal[1] == 0.0) goto restart;                                      // :904-905
        {
            const double ro1 = scal[3];
            for (int i = tid; i < m; i += T) s.x[i] = ds(s.x[i], dm(ro1, s.u[i]));
        }
        __syncthreads();
        sf_apply(s, n, sd, has_iw, has_rs, s.x, s.r);                        // :943-947
        for (int i = tid; i < m; i += T) {
            const double v = ds(s.B[i], s.r[i]);
            s.r[i] = v;
            s.bt[i] = dm(s.q0[i], v);                                        // beta's q.r (:1056-1059)
            s.u[i] = dm(v, v);                                               // r.r for the check (:1127)
        }
        __syncthreads();
        if (tid == 0) {                                                        // :1060-1065
            const double nq = sf_negsum(s.bt, m);
            double b = __ddiv_rn(nq, scal[0]);
            if (scal[0] == 0.0) b = 0.0;
            scal[5] = b;
            scal[6] = __ddiv_rn(b, scal[3]);
            scal[9] = nq;
        }
        __syncthreads();
        {
            const double beta = scal[5], bro = scal[6];
            for (int i = tid; i < m; i += T) {
                const double zw = da(s.r[i], dm(beta, s.w1[i]));
                s.g0[i] = da(zw, dm(bro, s.g1[i]));
            }
        }
        __syncthreads();
        sf_apply(s, n, sd, has_iw, has_rs, s.g0, s.w0, s.u, &scal[7]);       // :1094, r.r on the side
        for (int i = tid; i < m; i += T) s.bt[i] = dm(s.q0[i], s.w0[i]);     // c[0] (:1096-1099)
        __syncthreads();
        if (tid == 0) {
            const double c0 = sf_sum(s.bt, m), nq = scal[9];
            scal[0] = c0;                                                      // the shift :1104-1121
            if (nq != 0.0) scal[2] = __ddiv_rn(-nq, c0);                       // next iteration's al
            double st = 0.0;
            if (fabs(__ddiv_rn(scal[7], md)) < thr) st = 1.0;                  // :1126-1132
            else if (gtimer_ns() - t0 > SF_TIME_LIMIT_NS) st = 3.0;
            scal[8] = st;
        }
        __syncthreads();
        {
            double *t = s.g0; s.g0 = s.g1; s.g1 = t;
            t = s.w0; s.w0 = s.w1; s.w1 = t;
        }
        restarts = 0;
        have_qr = scal[9] != 0.0;
        const double st = scal[8];
        if (st == 1.0) break;
        ++iter;
        if (iter == maxiter) break;
        if (st == 3.0) {
            if (tid == 0) atomicOr(flags, DEVERR_SOLVER);
            break;
        }
    }
    return iter;
}

// ----------------------------------------------------------------- the fast form of a line solve

// The same solve with deterministic tree sums and fused multiply-adds: each dot product is one
// warp's lane partials folded by shuffles in a fixed tree (a few warp-wide FP64 instructions instead
// of m sequential adds on one lane), and every product that feeds a sum is one fused multiply-add. The operation order differs from the
// reference's (the LOD's default; space_frac.exact selects sf_solve_cta).

// Dot products of the line by one warp each (warp q for product q): its lanes take the values
// i = lane, lane + 32, ... as fused multiply-adds and fold them in a shuffle tree, and lane 0 puts
// the sum in red[q]; the caller synchronises the CTA before and after. A dot product costs a few
// warp-wide FP64 instructions instead of one per value on one lane.
__device__ __forceinline__ double warp_dot(const double *a, const double *b, int m, bool neg)
{
    double t = 0.0;
    for (int i = threadIdx.x & 31; i < m; i += 32) t = fma(neg ? -a[i] : a[i], b[i], t);
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
    return t;
}
// One dot product a.b (every thread gets it); the vectors must be complete (CTA synchronised).
__device__ __forceinline__ double cta_dot(const double *a, const double *b, int m, double *red)
{
    if (threadIdx.x < 32) {
        const double t = warp_dot(a, b, m, false);
        if (threadIdx.x == 0) red[0] = t;
    }
    __syncthreads();
    const double t = red[0];
    __syncthreads();
    return t;
}
// Two dot products on one warp; neg0: the first is -(a0.b0) (beta's "beta -= q*r"). Each lane sums
// both products' terms; one exchange then leaves lanes 0-15 with the first product's pair sums and
// lanes 16-31 with the second's, and four levels finish each (five warp-wide FP64 adds for the two,
// where two shuffle trees take ten).
__device__ __forceinline__ void cta_dot2(const double *a0, const double *b0, bool neg0, const double *a1,
                                         const double *b1, int m, double *red, double *o0, double *o1)
{
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        double t0 = 0.0, t1 = 0.0;
        for (int i = lane; i < m; i += 32) {
            t0 = fma(neg0 ? -a0[i] : a0[i], b0[i], t0);
            t1 = fma(a1[i], b1[i], t1);
        }
        const bool up = lane >= 16;
        double t = (up ? t1 : t0) + __shfl_xor_sync(0xffffffffu, up ? t0 : t1, 16);
#pragma unroll
        for (int o = 8; o >= 1; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if ((lane & 15) == 0) red[lane >> 4] = t;
    }
    __syncthreads();
    *o0 = red[0];
    *o1 = red[1];
    __syncthreads();
}

// Row i's value from its Toeplitz sum v: the tridiagonal terms plus v (over rs, times iw).
__device__ __forceinline__ double sf_row_finish(const SfVec &s, bool has_iw, bool has_rs, const double *xv, int i,
                                                double v)
{
    const double r = fma(s.m2[i], xv[i + 1], fma(s.m1[i], xv[i], s.m0[i] * xv[i - 1]));
    if (has_rs) v = v / s.rs[i];
    return has_iw ? fma(v, s.iw[i], r) : r + v;
}

// rv = the product with fused multiply-adds; a thread takes the rows k+1 and n-1-k (sf_pair).
__device__ void sf_apply_fast(const SfVec &s, int n, int sd, bool has_iw, bool has_rs, const double *xv, double *rv)
{
    const int T = blockDim.x, tid = threadIdx.x;
    for (int j = 1 + tid; j < n; j += T) s.bt[j] = fma(s.c2[j], xv[j + 1], fma(s.c1[j], xv[j], s.c0[j] * xv[j - 1]));
    __syncthreads();
    if (tid == T - 1) {
        rv[0] = fma(s.m2[0], xv[1], s.m1[0] * xv[0]);
        rv[n] = fma(s.m1[n], xv[n], s.m0[n] * xv[n - 1]);
    }
    const int pairs = n / 2;
    for (int k = tid; k < pairs; k += T) {
        const int kw = min(k - (tid & 31) + 31, pairs - 1);   // the warp's largest k (T is a multiple of 32)
        const int a = k + 1, b = n - 1 - k;
        double va, vb;
        sf_pair<false>(s.bt, s.Tm, n, sd, k, kw, va, vb);
        rv[a] = sf_row_finish(s, has_iw, has_rs, xv, a, va);
        if (b != a) rv[b] = sf_row_finish(s, has_iw, has_rs, xv, b, vb);
    }
    __syncthreads();
}

// solve_mln<1> (the sequence of sf_solve_cta) with the fast sums. scal[8] carries thread 0's
// time-limit decision to the CTA.
__device__ int sf_solve_cta_fast(SfVec s, int n, int sd, bool has_iw, bool has_rs, double thr, int maxiter,
                                 double *scal, double *red, unsigned *flags)
{
    const int m = n + 1, T = blockDim.x, tid = threadIdx.x;
    const double md = (double)m;
    const unsigned long long t0 = gtimer_ns();
    int iter = 1, restarts = 0;
    bool have_qr = false;
    double c1 = 0.0, al = 0.0, norm = 0.0, nq = 0.0;
restart:
    if (++restarts > maxiter + 1) {
        if (tid == 0) atomicOr(flags, DEVERR_SOLVER);
        return iter;
    }
    have_qr = false;
    sf_apply_fast(s, n, sd, has_iw, has_rs, s.x, s.r);                       // :841-844
    for (int i = tid; i < m; i += T) {
        const double v = s.B[i] - s.r[i];
        s.r[i] = v; s.g1[i] = v; s.q0[i] = v;
    }
    __syncthreads();
    norm = cta_dot(s.r, s.r, m, red);
    sf_apply_fast(s, n, sd, has_iw, has_rs, s.g1, s.w1);                     // :851
    c1 = cta_dot(s.q0, s.w1, m, red);
    if (fabs(norm / md) < thr) return iter;                                    // :866
    for (;;) {
        if (!have_qr) al = cta_dot(s.q0, s.r, m, red) / c1;                    // :871-877
        if (!(c1 != 0.0)) goto restart;
        for (int i = tid; i < m; i += T) {
            s.u[i] = fma(-al, s.w1[i], s.r[i]);
            s.x[i] = fma(al, s.g1[i], s.x[i]);
        }
        __syncthreads();
        sf_apply_fast(s, n, sd, has_iw, has_rs, s.u, s.Au);                  // :890
        double nrm, ro;
        cta_dot2(s.Au, s.Au, false, s.Au, s.u, m, red, &nrm, &ro);
        const double ro1 = -ro / nrm;                                          // :903
        if (nrm == 0.0) goto restart;
        for (int i = tid; i < m; i += T) s.x[i] = fma(-ro1, s.u[i], s.x[i]);
        __syncthreads();
        sf_apply_fast(s, n, sd, has_iw, has_rs, s.x, s.r);                   // :943-947
        for (int i = tid; i < m; i += T) s.r[i] = s.B[i] - s.r[i];
        __syncthreads();
        cta_dot2(s.q0, s.r, true, s.r, s.r, m, red, &nq, &norm);              // beta's -q.r, r.r
        double beta = nq / c1;                                                 // :1060-1065
        if (c1 == 0.0) beta = 0.0;
        const double bro = beta / ro1;
        for (int i = tid; i < m; i += T) s.g0[i] = fma(bro, s.g1[i], fma(beta, s.w1[i], s.r[i]));
        __syncthreads();
        sf_apply_fast(s, n, sd, has_iw, has_rs, s.g0, s.w0);                 // :1094
        if (tid == 0) scal[8] = gtimer_ns() - t0 > SF_TIME_LIMIT_NS ? 1.0 : 0.0;
        c1 = cta_dot(s.q0, s.w0, m, red);                                      // c[0], the shift :1104-1121
        if (nq != 0.0) al = -nq / c1;
        have_qr = nq != 0.0;
        {
            double *t = s.g0; s.g0 = s.g1; s.g1 = t;
            t = s.w0; s.w0 = s.w1; s.w1 = t;
        }
        restarts = 0;
        if (fabs(norm / md) < thr) break;                                     // :1126-1132
        ++iter;
        if (iter == maxiter) break;
        if (scal[8] != 0.0) {
            if (tid == 0) atomicOr(flags, DEVERR_SOLVER);
            break;
        }
    }
    return iter;
}

__device__ __forceinline__ void sf_copy(double *dst, const double *src, int m)
{
    for (int i = threadIdx.x; i < m; i += blockDim.x) dst[i] = src[i];
}

// ------------------------------------------------------------- batch of lines (the C ABI)

struct SfBatchArgs {
    int lines, n, sd;
    const double *mat, *mc, *Tm, *iw, *rs, *B;   // mat, mc: 3 planes of lines x (n+1)
    const double *x;
    double *r;                                   // product output (matvec) or solution (solve)
    double thr;
    int maxiter;
    int *iters;
    unsigned *flags;
};

__global__ void __launch_bounds__(SF_THREADS, 6) k_sf_batch(SfBatchArgs a, int solve)
{
    extern __shared__ __align__(16) double sf_sm[];
    __shared__ double scal[10];
    const int m = a.n + 1, line = blockIdx.x;
    const int64_t o = (int64_t)line * m, plane = (int64_t)a.lines * m;
    SfVec s = sf_carve(sf_sm, m);
    sf_copy(s.Tm, a.Tm, m);
    sf_copy(s.m0, a.mat + o, m);
    sf_copy(s.m1, a.mat + plane + o, m);
    sf_copy(s.m2, a.mat + 2 * plane + o, m);
    sf_copy(s.c0, a.mc + o, m);
    sf_copy(s.c1, a.mc + plane + o, m);
    sf_copy(s.c2, a.mc + 2 * plane + o, m);
    if (a.iw) sf_copy(s.iw, a.iw + o, m);
    if (a.rs) sf_copy(s.rs, a.rs + o, m);
    sf_copy(s.x, a.x + o, m);
    if (solve) sf_copy(s.B, a.B + o, m);
    __syncthreads();
    if (!solve) {
        sf_apply(s, a.n, a.sd, a.iw != nullptr, a.rs != nullptr, s.x, s.r);
        sf_copy(a.r + o, s.r, m);
        return;
    }
    const int it = sf_solve_cta(s, a.n, a.sd, a.iw != nullptr, a.rs != nullptr, a.thr, a.maxiter, scal, a.flags);
    sf_copy(a.r + o, s.x, m);
    if (a.iters && threadIdx.x == 0) a.iters[line] = it;
}

// ------------------------------------------------------------------ LOD pass with impl 2

// One line of one pass: the system implicit2_gen forms (:4630-4663) from the coefficient grids of
// the pass (line-major: per line A, B, Rlap, mc0, mc1, mc2, iw, each Nl+1 values), the state and
// this step's source, history and line ends; solved in place and written back with the ghost copy
// U[Nl+1] = U[Nl] (U1 :4792).
template <bool FAST>
__global__ void __launch_bounds__(SF_THREADS, 6) k_lod_pass_sf(LodSfArgs a)   // (5 per SM measured slower)
{
    extern __shared__ __align__(16) double sf_sm[];
    __shared__ double scal[10];
    const int n = a.Nl, m = n + 1, line = blockIdx.x, tid = threadIdx.x, T = blockDim.x;
    const int la = line % a.n1, lb = line / a.n1;
    const int64_t base = (int64_t)(1 + la) * a.s1 + (int64_t)(1 + lb) * a.s2;
    const double *cf = a.coef + (int64_t)line * 7 * m;
    SfVec s = sf_carve(sf_sm, m);
    sf_copy(s.Tm, a.Tm, m);
    for (int p = tid; p < m; p += T) {
        const int64_t id = base + (int64_t)p * a.st;
        const double u = a.U[id];
        s.x[p] = u;
        if (p >= 1 && p < n) {
            s.m0[p] = cf[p];
            s.m2[p] = cf[m + p];
            s.m1[p] = -da(cf[2 * m + p], a.lamR);                                  // -R :3117-3123
            s.c0[p] = cf[3 * m + p];
            s.c1[p] = cf[4 * m + p];
            s.c2[p] = cf[5 * m + p];
            s.iw[p] = cf[6 * m + p];
            double om = ds(a.rp ? a.rp[id] : 0.0, dm(a.lam, u));                     // Om1_impl :4441
            if (a.KS) {
                double sv = 0.0;
                for (int k = 0; k < a.KS; ++k) sv = da(sv, __ldcg(a.part + (int64_t)k * a.pstride + id));
                om = da(om, sv);                                                     // :4507-4510
            }
            s.B[p] = om;
        } else if (p == 0) {                                                         // :4643-4651
            s.m0[0] = 0.0; s.m1[0] = 1.0; s.m2[0] = 0.0;
            s.B[0] = a.bc ? a.bc[id] : 0.0;
        } else {
            const double g = a.bc ? a.bc[id] : 0.0;
            s.m2[n] = 0.0; s.m1[n] = 1.0;
            if (a.rkind == FPDE_BC_FLUX) { s.m0[n] = -1.0; s.B[n] = dm(g, a.dLN); } // bottom_cond 0
            else { s.m0[n] = 0.0; s.B[n] = g; }
        }
    }
    __syncthreads();
    __shared__ double red[2];
    const int it = FAST ? sf_solve_cta_fast(s, n, a.sd, true, false, a.thr, a.maxiter, scal, red, a.flags)
                        : sf_solve_cta(s, n, a.sd, true, false, a.thr, a.maxiter, scal, a.flags);
    for (int p = tid; p < m; p += T) a.U[base + (int64_t)p * a.st] = s.x[p];
    if (tid == 0) {
        a.U[base + (int64_t)m * a.st] = s.x[n];
        if (a.iters) atomicAdd(a.iters, (unsigned long long)it);
    }
}

size_t sf_smem_bytes(int n) { return (size_t)SF_NVEC * (size_t)(n + 1) * sizeof(double); }

// Opt both kernels in to the shared memory of the longest line once per device (outside any graph
// capture: fpde_lod3d_create calls this before its first run).
int sf_prepare()
{
    const int bytes = (int)sf_smem_bytes(FPDE_SF_MAX_N);
    if (smem_opt_in((const void *)k_lod_pass_sf<false>, bytes) != cudaSuccess ||
        smem_opt_in((const void *)k_lod_pass_sf<true>, bytes) != cudaSuccess ||
        smem_opt_in((const void *)k_sf_batch, bytes) != cudaSuccess)
        return set_error(FPDE_ERR_CUDA, "space-fractional kernels: shared memory opt-in failed");
    return FPDE_OK;
}

int launch_lod_pass_sf(cudaStream_t st, const LodSfArgs &a)
{
    const size_t smem = sf_smem_bytes(a.Nl);
    if (a.fast) k_lod_pass_sf<true><<<(unsigned)a.lines, SF_THREADS, smem, st>>>(a);
    else k_lod_pass_sf<false><<<(unsigned)a.lines, SF_THREADS, smem, st>>>(a);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

}  // namespace fpde

using namespace fpde;

static int sf_batch(fpde_ctx *ctx, int lines, int n, const double *mat, const double *mc, const double *Tm,
                    const double *iw, const double *rs, int space_der, const double *B, const double *x, double *out,
                    double thr, int maxiter, int *iters, int on_device, int solve)
{
    clear_error();
    FPDE_CHECK_ARG(mat && mc && Tm && x && out, "null argument");
    FPDE_CHECK_ARG(!solve || B, "null right-hand side");
    FPDE_CHECK_ARG(lines >= 1 && n >= 1 && n <= FPDE_SF_MAX_N, "lines >= 1 and 1 <= n <= FPDE_SF_MAX_N");
    FPDE_CHECK_ARG(space_der == 0 || space_der == 1, "space_der must be 0 or 1");
    FPDE_CHECK_ARG(!solve || (maxiter >= 1 && maxiter <= FPDE_SF_MAX_ITER), "maxiter must be 1 .. FPDE_SF_MAX_ITER");
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    cudaStream_t st = ctx->stream;
    const size_t m = (size_t)n + 1, vec = (size_t)lines * m * sizeof(double);
    const size_t smem = sf_smem_bytes(n);
    if ((rc = sf_prepare())) return rc;
    SfBatchArgs a{};
    a.lines = lines; a.n = n; a.sd = space_der; a.thr = thr; a.maxiter = maxiter; a.flags = ctx->d_flags;
    std::vector<void *> own;
    auto stage = [&](const double *src, size_t bytes, bool copy_in) -> double * {
        if (on_device) return const_cast<double *>(src);
        void *p = nullptr;
        if (dev_alloc(&p, bytes)) return nullptr;
        own.push_back(p);
        if (copy_in && src) cudaMemcpyAsync(p, src, bytes, cudaMemcpyHostToDevice, st);
        return (double *)p;
    };
    bool fail = false;
    a.mat = stage(mat, 3 * vec, true);
    a.mc = stage(mc, 3 * vec, true);
    a.Tm = stage(Tm, m * sizeof(double), true);
    a.iw = iw ? stage(iw, vec, true) : nullptr;
    a.rs = rs ? stage(rs, vec, true) : nullptr;
    a.B = (solve && B) ? stage(B, vec, true) : nullptr;
    a.x = stage(x, vec, true);
    a.r = stage(out, vec, false);
    int *d_it = nullptr;
    fail = !a.mat || !a.mc || !a.Tm || (iw && !a.iw) || (rs && !a.rs) || (solve && !a.B) || !a.x || !a.r;
    if (!fail && iters) {
        if (on_device) d_it = iters;
        else fail = dev_alloc((void **)&d_it, (size_t)lines * sizeof(int)) != 0;
        if (!on_device && d_it) own.push_back(d_it);
    }
    a.iters = d_it;
    if (!fail) {
        k_sf_batch<<<(unsigned)lines, SF_THREADS, smem, st>>>(a, solve);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) rc = set_error(FPDE_ERR_CUDA, "space-fractional batch launch: %s", cudaGetErrorString(e));
        else count_launches(1);
        if (!rc && !on_device) {
            cudaMemcpyAsync(out, a.r, vec, cudaMemcpyDeviceToHost, st);
            if (iters) cudaMemcpyAsync(iters, d_it, (size_t)lines * sizeof(int), cudaMemcpyDeviceToHost, st);
        }
        if (!rc) rc = ctx_check_flags(ctx, solve ? "fpde_sf_solve" : "fpde_sf_matvec");
    } else {
        rc = set_error(FPDE_ERR_NOMEM, "space-fractional batch: device allocation failed");
    }
    cudaStreamSynchronize(st);
    for (void *p : own) dev_free(p);
    return rc;
}

extern "C" {

int fpde_sf_matvec(fpde_ctx *ctx, int lines, int n, const double *mat, const double *mc, const double *Tm,
                   const double *iw, const double *rs, int space_der, const double *x, double *r, int on_device)
{
    return sf_batch(ctx, lines, n, mat, mc, Tm, iw, rs, space_der, nullptr, x, r, 0.0, 1, nullptr, on_device, 0);
}

int fpde_sf_solve(fpde_ctx *ctx, int lines, int n, const double *mat, const double *mc, const double *Tm,
                  const double *iw, const double *rs, int space_der, const double *B, double *x, double thr,
                  int maxiter, int *iters, int on_device)
{
    return sf_batch(ctx, lines, n, mat, mc, Tm, iw, rs, space_der, B, x, x, thr, maxiter, iters, on_device, 1);
}

int fpde_sf_toeplitz_row(double gamma, const double *Z, int n, double *Tm)
{
    clear_error();
    FPDE_CHECK_ARG(Z && Tm && n >= 1, "null argument or n < 1");
    FPDE_CHECK_ARG(gamma > 0.0 && gamma <= 1.0, "gamma must be in (0, 1]");
    const double A = 1.0 - gamma;                                // :3675-3681
    const double Dg2 = 1.0 / std::tgamma(2.0 - gamma);           // 1 / g2g, g2g = Gamma(2 - gamma) (:2715)
    Tm[0] = 0.0;
    for (int i = 1; i <= n; ++i)
        Tm[i] = A != 0.0 ? Dg2 * std::fabs(std::pow(std::fabs(Z[1] - Z[i]), A) - std::pow(std::fabs(Z[1] - Z[i + 1]), A))
                         : (i == 1 ? 1.0 : 0.0);
    return FPDE_OK;
}

}  // extern "C"
