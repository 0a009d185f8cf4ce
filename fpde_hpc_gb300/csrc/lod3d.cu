// 3D LOD time stepping (fpde_lod3d_*): the reference's mode-3 calc_step
// (fpde_hpc_1d.cpp:5144-5779, implicit3d 0, split3d 0) on the GPU.
//
// Per time step n:
//   1. k_l1_partial  : part[ks][q] = sum_t w[n-t] D_t[q] over the whole grid (FP64 history)
//   2. K pass        : lines along k for every (i, j); Om = -lam U + Rp + S (time_summing
//                      is added only in this pass, Om1 :4165-4268 with m3d_c == 2)
//   3. _M pass       : lines along j for every (i, k); Om = -lam U
//   4. sN pass       : lines along i for every (j, k); Om = -lam U
//   5. append        : D_n = U - U_old over the grid (the snapshot of the step, :5733-5745)
// Split path (FPDE_PREC_SPLIT_BF16X3): step 1 becomes, per 64-step block, the exact
// three-slice tensor-core contraction of all history before the block (tc_far.cu, as for
// lines) and, per step, k_near_history_ff: the far partials plus the near history in
// float-float from the 64-row float-pair ring of the block's increments (step 5 writes it
// beside the FP64 ring that the conversion reads).
// Each pass is a Thomas solve per line with R = Rlap + lam (A_/B/R :3095-3142). For a
// uniform step the alpha recurrence Al[p+1] = B/(R - A Al[p]) is time-invariant, so it is
// evaluated once on the host in the reference's order; a pass then needs two first-order
// recurrences per line (forward y, backward U), swept by four lanes per line in segments
// (k_lod_pass_seg) or, for lines over 128 interior nodes, by one thread (k_lod_pass).
//
// HBM layout: the state and every grid input keep the reference's index
// idx = i + j (sN+2) + k (sN+2)(M+2) (:1181). The per-pass line coefficients (A, g =
// Al[p+1]/B, al = Al[p+1]) are stored pass-line-major, c[p * lines + line], so the threads of
// a warp (consecutive lines) read consecutive addresses in every pass. K and _M lines are
// numbered with i fastest, so their state accesses are coalesced too; the sN pass walks
// along the contiguous axis and relies on L1 for reuse of each line's cache lines.
// The whole run is captured once into a CUDA graph and replayed.
#include <algorithm>
#include <climits>
#include <map>
#include <vector>
#include <cmath>
#include <string>

#include "common.cuh"
#include "kernels.cuh"
#include "graph_cache.cuh"
#include "richards.cuh"
#include "tc_far.cuh"
#include "ff.cuh"

namespace fpde {

struct LodPassArgs {
    double *U;
    const double *A, *g, *al;        // (Nl+1) x lines, pass-line-major: A holds gA = g A_
    const double *part;              // history partials [KS][pstride] (K pass), or KS = 0
    int KS;
    int64_t pstride;
    const double *rp;                // K-pass source grid of this step, may be null
    const double *bc;                // boundary grid of this step (line ends), may be null (0)
    double lam;
    int Nl, lines, n1;               // line = a + n1 * b
    int64_t s1, s2, st;              // base = (1+a) s1 + (1+b) s2, node stride st
    int lkind, rkind;
    double dLN;
};

// One thread per line. The loads of eight nodes are issued together before their
// dependent recurrence steps (the in-place stores to U would otherwise keep the compiler
// from hoisting them), so each line keeps eight nodes of memory traffic in flight.
constexpr int LB = 8;

__global__ void __launch_bounds__(128) k_lod_pass(LodPassArgs p)
{
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.lines) return;
    const int a = line % p.n1, b = line / p.n1;
    const int64_t base = (int64_t)(1 + a) * p.s1 + (int64_t)(1 + b) * p.s2;
    const int Nl = p.Nl, L = p.lines;
    const double g0 = p.bc ? p.bc[base] : 0.0;
    // forward: y_q = Bt[q+1] = g_q (A_q y_{q-1} - Om_q), y_0 = Bt[1] = g0; y_q overwrites U_q
    double y = g0, uold_last = 0.0;
    for (int q0 = 1; q0 < Nl; q0 += LB) {
        double uu[LB], aa[LB], gg[LB], rr[LB], ss[LB];
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int q = q0 + t;
            const bool in = q < Nl;
            const int64_t id = base + (int64_t)(in ? q : 1) * p.st;
            uu[t] = in ? p.U[id] : 0.0;
            aa[t] = in ? __ldg(p.A + (int64_t)q * L + line) : 0.0;
            gg[t] = in ? __ldg(p.g + (int64_t)q * L + line) : 0.0;
            rr[t] = (in && p.rp) ? __ldg(p.rp + id) : 0.0;
            double sv = 0.0;
            for (int k = 0; k < p.KS; ++k)
                if (in) sv += __ldcg(p.part + (int64_t)k * p.pstride + id);
            ss[t] = sv;
        }
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int q = q0 + t;
            if (q < Nl) {
                if (q == Nl - 1) uold_last = uu[t];
                // y = g (A y - Om) with Om = -(lam u) + Rp + S (Om1 :4191, :4267), as gA y + g (-Om)
                double mo = p.lam * uu[t];                               // -Om, term by term
                if (p.rp) mo -= rr[t];
                if (p.KS) mo -= ss[t];
                y = fma(aa[t], y, gg[t] * mo);
                p.U[base + (int64_t)q * p.st] = y;
            }
        }
    }
    // right end: Dirichlet value or the flux closure of U1 (:4687-4719) with the old U[Nl-1]
    const double gN = p.bc ? p.bc[base + (int64_t)Nl * p.st] : 0.0;
    double uN;
    if (p.rkind == FPDE_BC_DIRICHLET) {
        uN = gN;
    } else {
        const double AlN = __ldg(p.al + (int64_t)(Nl - 1) * L + line);
        if (fabs(y) > 1e-15) uN = (fabs(1.0 - AlN) > 1e-15) ? (y + gN * p.dLN) / (1.0 - AlN) : uold_last;
        else uN = (fabs(1.0 - AlN) > 1e-15) ? 0.0 : uold_last;
    }
    p.U[base + (int64_t)Nl * p.st] = uN;
    p.U[base + (int64_t)(Nl + 1) * p.st] = uN;                  // ghost copy (U1 :4792)
    double u = uN;
    for (int q1 = Nl - 1; q1 >= 1; q1 -= LB) {
        double yy[LB], al[LB];
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int q = q1 - t;
            const bool in = q >= 1;
            yy[t] = in ? p.U[base + (int64_t)q * p.st] : 0.0;
            al[t] = in ? __ldg(p.al + (int64_t)q * L + line) : 0.0;
        }
#pragma unroll
        for (int t = 0; t < LB; ++t) {
            const int q = q1 - t;
            if (q >= 1) {
                u = fma(al[t], u, yy[t]);
                p.U[base + (int64_t)q * p.st] = u;
            }
        }
    }
    p.U[base] = fma(__ldg(p.al + line), u, g0);                   // Al[1] U[1] + Bt[1]
}

// Variable steps (the reference's varT): the local term Da kkk0_n / tau_n of R changes every step,
// so one thread per line runs al1 / bt1 / U1 (:4002-4027, :4585-4590, :4683-4724) from the raw
// coefficients A_, B, Rlap (pass-line-major) and the step's lamR, in the reference's order.
struct LodVarArgs {
    const double *A, *B, *Rl;        // (Nl+1) x lines, pass-line-major
    double *al;                      // scratch: Al[q+1] at q * lines + line
    double lamR;
};

__global__ void __launch_bounds__(128) k_lod_pass_var(LodPassArgs p, LodVarArgs v)
{
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.lines) return;
    const int a = line % p.n1, b = line / p.n1;
    const int64_t base = (int64_t)(1 + a) * p.s1 + (int64_t)(1 + b) * p.s2;
    const int Nl = p.Nl, L = p.lines;
    const double g0 = p.bc ? p.bc[base] : 0.0;
    const double al1 = p.lkind == FPDE_BC_FLUX ? 1.0 : 0.0;             // Al[1]
    double al = al1, y = g0, uold_last = 0.0;
    for (int q = 1; q < Nl; ++q) {
        const int64_t id = base + (int64_t)q * p.st;
        const double u = p.U[id];
        if (q == Nl - 1) uold_last = u;
        const int64_t o = (int64_t)q * L + line;
        const double A = __ldg(v.A + o), B = __ldg(v.B + o), R = __dadd_rn(__ldg(v.Rl + o), v.lamR);
        const double aln = __ddiv_rn(B, __dsub_rn(R, __dmul_rn(A, al)));   // Al[q+1]
        double sv = 0.0;
        for (int k = 0; k < p.KS; ++k) sv += __ldcg(p.part + (int64_t)k * p.pstride + id);
        const double om = __dadd_rn(__dadd_rn(-__dmul_rn(p.lam, u), p.rp ? __ldg(p.rp + id) : 0.0), sv);
        y = __dmul_rn(__ddiv_rn(aln, B), __dsub_rn(__dmul_rn(A, y), om));   // Bt[q+1]
        v.al[o] = aln;
        p.U[id] = y;
        al = aln;
    }
    const double gN = p.bc ? p.bc[base + (int64_t)Nl * p.st] : 0.0;
    double uN;
    if (p.rkind == FPDE_BC_DIRICHLET) {
        uN = gN;
    } else if (fabs(y) > 1e-15) {
        uN = (fabs(1.0 - al) > 1e-15) ? __ddiv_rn(__dadd_rn(y, __dmul_rn(gN, p.dLN)), 1.0 - al) : uold_last;
    } else {
        uN = (fabs(1.0 - al) > 1e-15) ? 0.0 : uold_last;
    }
    p.U[base + (int64_t)Nl * p.st] = uN;
    p.U[base + (int64_t)(Nl + 1) * p.st] = uN;                          // ghost copy (U1 :4792)
    double u = uN;
    for (int q = Nl - 1; q >= 1; --q) {
        const int64_t id = base + (int64_t)q * p.st;
        u = __dadd_rn(__dmul_rn(v.al[(int64_t)q * L + line], u), p.U[id]);
        p.U[id] = u;
    }
    p.U[base] = __dadd_rn(__dmul_rn(al1, u), g0);                       // Al[1] U[1] + Bt[1]
}

// The reference's Richards problem (analytic_test 0): every line's coefficients change with the
// solution, so nothing is precomputed. One thread per line forms, node by node, the suction
// P = -(U - i sZ[q]) (i the node's sN index: q in the sN pass, the line's first index otherwise;
// wetness / inv_dw_dh :2504-2512, :2546-2554), the closures KK and inv_dw_dh (richards.cuh) and
// A_ = KK(q-1) iw(q) / (dL_q dL_{q-1}), B = KK(q) iw(q) / dL_q^2,
// R = iw(q) (KK(q)/dL_q^2 + KK(q-1)/(dL_q dL_{q-1})) + Da kkk0/tau (:3095-3142), and runs the
// Thomas recurrences of al1 / bt1 / U1 on them in the reference's order, without contracted
// multiply-adds. Left end: the sN pass takes the first-order surface condition (al1 :4004-4012,
// bc0 :4493-4500) with Uc = dL_0 E / KK(1) (Uc :3036-3070, no irrigation); the other passes
// zero flux. Right end: U1's flux closure (:4687-4719) with zero flux.
struct LodRichArgs {
    const double *sZ;       // sN+2 coordinates along the sN axis
    const double *dL;       // this pass's steps, Nl+2 values
    double *al;             // scratch: Al[q+1] at q * lines + line
    double ksat, lamR, E;
    int kform, pass;
    // salt concentration (equation 1), or C = null
    double *C = nullptr;
    const double *partC = nullptr;   // C's history partials (K pass), KSC rows of pstride
    int KSC = 0;
    double nu = 0.0, sigma = 1.0, Dc = 0.0;
};

__global__ void __launch_bounds__(128) k_lod_pass_rich(LodPassArgs p, LodRichArgs r)
{
    const int line = blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= p.lines) return;
    const int a = line % p.n1, b = line / p.n1;
    const int64_t base = (int64_t)(1 + a) * p.s1 + (int64_t)(1 + b) * p.s2;
    const int Nl = p.Nl, L = p.lines;
    auto suction = [&](int q, double u) {
        const double i = r.pass == 0 ? (double)q : (double)(1 + a);
        return -__dadd_rn(u, -__dmul_rn(i, r.sZ[q]));
    };
    const double P0 = suction(0, p.U[base]);
    double kk_prev = rich_KK(P0, r.kform, r.ksat);                       // KK(0)
    double al = 1.0, y = 0.0;                                           // Al[1], Bt[1]
    if (r.pass == 0) {
        const double kk1 = rich_KK(suction(1, p.U[base + p.st]), r.kform, r.ksat);
        const double Uc = __ddiv_rn(__dmul_rn(r.dL[0], r.E - 0.0), kk1);
        if (rich_inv_dw_dh(P0) != RICH_SATURATED) {
            y = -Uc;
        } else {
            al = 0.0;
            y = __ddiv_rn(__dmul_rn(-Uc, kk1), r.dL[0]);
        }
    }
    const double al1 = al, g0 = y;
    double uold_last = 0.0;
    for (int q = 1; q < Nl; ++q) {
        const int64_t id = base + (int64_t)q * p.st;
        const double u = p.U[id];
        if (q == Nl - 1) uold_last = u;
        const double P = suction(q, u);
        const double kk = rich_KK(P, r.kform, r.ksat), iw = rich_inv_dw_dh(P);
        const double dq = r.dL[q], dm = r.dL[q - 1];
        const double dqq = __dmul_rn(dq, dq), dqm = __dmul_rn(dq, dm);
        const double A = __ddiv_rn(__dmul_rn(kk_prev, iw), dqm);
        const double B = __ddiv_rn(__dmul_rn(kk, iw), dqq);
        const double R = __dadd_rn(__dmul_rn(iw, __dadd_rn(__ddiv_rn(kk, dqq), __ddiv_rn(kk_prev, dqm))), r.lamR);
        const double aln = __ddiv_rn(B, __dadd_rn(R, -__dmul_rn(A, al)));    // Al[q+1]
        double sv = 0.0;
        for (int k = 0; k < p.KS; ++k) sv += __ldcg(p.part + (int64_t)k * p.pstride + id);
        double om = __dadd_rn(-__dmul_rn(p.lam, u), p.rp ? __ldg(p.rp + id) : 0.0);
        if (r.C && r.nu != 0.0) {              // chemical osmosis from the old C (Om1 :4211-4223)
            const double cm = r.C[id - p.st], cq = r.C[id], cp = r.C[id + p.st];
            const double f = __dmul_rn(r.nu, __dadd_rn(__dadd_rn(__ddiv_rn(cp, dqq),
                                                                 -__dmul_rn(__dadd_rn(__ddiv_rn(1.0, dqq),
                                                                                      __ddiv_rn(1.0, dqm)), cq)),
                                                       __ddiv_rn(cm, dqm)));
            om = __dadd_rn(om, __dmul_rn(f, iw));
        }
        om = __dadd_rn(om, sv);
        y = __dmul_rn(__ddiv_rn(aln, B), __dadd_rn(__dmul_rn(A, y), -om));  // Bt[q+1]
        r.al[(int64_t)q * L + line] = aln;
        p.U[id] = y;
        al = aln;
        kk_prev = kk;
    }
    double uN;                                                          // flux closure, zero flux
    if (fabs(y) > 1e-15) uN = (fabs(1.0 - al) > 1e-15) ? __ddiv_rn(y + 0.0, 1.0 - al) : uold_last;
    else uN = (fabs(1.0 - al) > 1e-15) ? 0.0 : uold_last;
    p.U[base + (int64_t)Nl * p.st] = uN;
    p.U[base + (int64_t)(Nl + 1) * p.st] = uN;                          // ghost copy (U1 :4792)
    double u = uN;
    for (int q = Nl - 1; q >= 1; --q) {
        const int64_t id = base + (int64_t)q * p.st;
        u = __dadd_rn(__dmul_rn(r.al[(int64_t)q * L + line], u), p.U[id]);
        p.U[id] = u;
    }
    p.U[base] = __dadd_rn(__dmul_rn(al1, u), g0);                       // Al[1] U[1] + Bt[1]
    if (!r.C) return;
    // ---- equation 1 on the same line (U1(1) after U1(0), :5270-5278): constant coefficients
    // A_/B/R (:3099-3136: D/sigma over the steps, Dg = kb = 1), Om1 (:4175-4229) with the new H
    // and its KK and the old C: -(lam C) - F_H + F_C + history. Dirichlet Cu() = 0 at the sN
    // pass's surface (al1 :4014-4017), zero flux elsewhere; the flux closure with bcN = 0 at the
    // far end; the ghost node takes H's U[N] (U1 :4792 copies U, the H row, into the C row).
    double *C = r.C;
    double hprev = p.U[base], hcur = p.U[base + p.st];
    double kkm = rich_KK(suction(0, hprev), r.kform, r.ksat);
    double cprev = C[base], ccur = C[base + p.st];
    double alc = r.pass == 0 ? 0.0 : 1.0, yc = 0.0;
    const double alc1 = alc;
    double cold_last = ccur;
    for (int q = 1; q < Nl; ++q) {
        const int64_t id = base + (int64_t)q * p.st;
        const double hnext = p.U[id + p.st], cnext = C[id + p.st];
        if (q == Nl - 1) cold_last = ccur;
        const double kk = rich_KK(suction(q, hcur), r.kform, r.ksat);
        const double dq = r.dL[q], dm = r.dL[q - 1];
        const double dqq = __dmul_rn(dq, dq), dqm = __dmul_rn(dq, dm);
        const double iqq = __ddiv_rn(1.0, dqq), iqm = __ddiv_rn(1.0, dqm);
        const double A = __ddiv_rn(__dmul_rn(r.Dc, iqm), r.sigma);
        const double B = __ddiv_rn(__dmul_rn(r.Dc, iqq), r.sigma);
        const double R = __dadd_rn(__ddiv_rn(__dmul_rn(r.Dc, __dadd_rn(iqq, iqm)), r.sigma), r.lamR);
        const double aln = __ddiv_rn(B, __dadd_rn(R, -__dmul_rn(A, alc)));
        const double kc = __dmul_rn(kk, ccur), kcm = __dmul_rn(kkm, cprev);
        const double fh = __dmul_rn(__ddiv_rn(1.0, r.sigma),
                                    __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(kc, hnext), dqq),
                                                        -__dmul_rn(__dadd_rn(__ddiv_rn(kc, dqq), __ddiv_rn(kcm, dqm)), hcur)),
                                              __ddiv_rn(__dmul_rn(kcm, hprev), dqm)));
        double om = __dadd_rn(__dadd_rn(-__dmul_rn(p.lam, ccur), 0.0), -fh);
        if (r.nu != 0.0) {
            const double fc = __dmul_rn(__ddiv_rn(r.nu, r.sigma),
                                        __dadd_rn(__dadd_rn(__ddiv_rn(__dmul_rn(ccur, cnext), dqq),
                                                            -__dmul_rn(__dadd_rn(__ddiv_rn(ccur, dqq), __ddiv_rn(cprev, dqm)), ccur)),
                                                  __ddiv_rn(__dmul_rn(cprev, cprev), dqm)));
            om = __dadd_rn(om, fc);
        }
        double svc = 0.0;
        for (int k = 0; k < r.KSC; ++k) svc += __ldcg(r.partC + (int64_t)k * p.pstride + id);
        om = __dadd_rn(om, svc);
        yc = __dmul_rn(__ddiv_rn(aln, B), __dadd_rn(__dmul_rn(A, yc), -om));
        r.al[(int64_t)q * L + line] = aln;
        C[id] = yc;
        alc = aln;
        kkm = kk;
        hprev = hcur; hcur = hnext;
        cprev = ccur; ccur = cnext;
    }
    double cN;
    if (fabs(yc) > 1e-15) cN = (fabs(1.0 - alc) > 1e-15) ? __ddiv_rn(yc + 0.0, 1.0 - alc) : cold_last;
    else cN = (fabs(1.0 - alc) > 1e-15) ? 0.0 : cold_last;
    C[base + (int64_t)Nl * p.st] = cN;
    C[base + (int64_t)(Nl + 1) * p.st] = uN;
    double c = cN;
    for (int q = Nl - 1; q >= 1; --q) {
        const int64_t id = base + (int64_t)q * p.st;
        c = __dadd_rn(__dmul_rn(r.al[(int64_t)q * L + line], c), C[id]);
        C[id] = c;
    }
    C[base] = __dadd_rn(__dmul_rn(alc1, c), 0.0);
}

// Segmented pass: SEGS threads (adjacent lanes) per line, each sweeping one segment of up to
// SEGLEN nodes from zero carries, the segments joined by affine scans over the group's lanes.
// One thread per line left only ~3 warps per SM for a chain of dependent FP64 operations; four
// per line give the FP64 pipe four times the independent work. With the segment's prefix
// product of a = g A (its end value PF), the backward sweep's responses KF (to that prefix
// product) and CB (suffix product of al) precomputed per node on the host:
//   y = y0 + c_in CF,  u = ub0 + c_in KF + c_out CB,
// where y0, ub0 are the zero-carry sweeps, c_in the true y before the segment and c_out the
// true u after it.
// (segments per line, nodes per segment) by line length: 8 x 16 up to 129 intervals, 16 x 16 up to
// 257, 16 x 32 up to 513; longer lines run one thread per line. More, shorter segments keep more
// lines' loads in flight (the pass is bound by memory latency, not bandwidth).
// A requested count (fpde_lod3d_desc.segments: 4, 8, 16 or 32, at most 32 interior nodes each)
// replaces the rule; *seglen is then the kernel's segment capacity (4, 8, 16 or 32, the smallest
// that holds ceil((Nl-1)/segs) nodes).
static inline void seg_shape(int Nl, int req, int *segs, int *seglen)
{
    const int interior = Nl - 1;
    if (req > 0) {
        const int sl = (interior + req - 1) / req;
        *segs = req;
        *seglen = sl <= 4 ? 4 : sl <= 8 ? 8 : sl <= 16 ? 16 : 32;
        if (sl > 32 || interior < 1) *segs = *seglen = 0;
        return;
    }
    if (interior <= 8 * 16) { *segs = 8; *seglen = 16; }
    else if (interior <= 16 * 16) { *segs = 16; *seglen = 16; }
    else if (interior <= 16 * 32) { *segs = 16; *seglen = 32; }
    else { *segs = 0; *seglen = 0; }
}
static inline bool seg_request_ok(int Nl, int req)
{
    return req == 0 || ((req == 4 || req == 8 || req == 16 || req == 32) && Nl >= 2 && (Nl - 1 + req - 1) / req <= 32);
}
constexpr int LSB = 4;                    // nodes of loads issued together (register budget: one wave)
struct LodSegArgs {
    const double *KF, *CB;           // (Nl+1) x lines, pass-line-major
    const double *PF;                // [lines][segs]: product of a = g A over each segment
    int seglen;                      // nodes per segment (<= the kernel's SEGLEN)
};

template <int SEGS, int SEGLEN>
__global__ void __launch_bounds__(128, SEGLEN <= 16 ? 5 : 4) k_lod_pass_seg(LodPassArgs p, LodSegArgs sg)
{
    const int gt = blockIdx.x * blockDim.x + threadIdx.x;
    const int line = gt / SEGS, sgi = gt % SEGS;
    const bool live = line < p.lines;
    const int ln = live ? line : 0;
    const int a = ln % p.n1, b = ln / p.n1;
    const int64_t base = (int64_t)(1 + a) * p.s1 + (int64_t)(1 + b) * p.s2;
    const int Nl = p.Nl, L = p.lines;
    const int q0 = 1 + sgi * sg.seglen, q1 = min(q0 + sg.seglen, Nl);   // nodes [q0, q1)
    const double g0 = p.bc ? p.bc[base] : 0.0;
    const double uold_last = p.U[base + (int64_t)(Nl - 1) * p.st];       // read before any write
    // forward from a zero carry: y0_q = g_q (A_q y0_{q-1} - Om_q)
    double yv[SEGLEN];
    double y = 0.0;
#pragma unroll
    for (int t0 = 0; t0 < SEGLEN; t0 += LSB) {
        double uu[LSB], aa[LSB], gg[LSB], rr[LSB], ss[LSB];
#pragma unroll
        for (int t = 0; t < LSB; ++t) {
            const int q = q0 + t0 + t;
            const bool in = live && q < q1;
            const int64_t id = base + (int64_t)(in ? q : 1) * p.st;
            uu[t] = in ? p.U[id] : 0.0;
            aa[t] = in ? __ldg(p.A + (int64_t)q * L + line) : 0.0;
            gg[t] = in ? __ldg(p.g + (int64_t)q * L + line) : 0.0;
            rr[t] = (in && p.rp) ? __ldg(p.rp + id) : 0.0;
            double sv = 0.0;
            for (int k = 0; k < p.KS; ++k)
                if (in) sv += __ldcg(p.part + (int64_t)k * p.pstride + id);
            ss[t] = sv;
        }
#pragma unroll
        for (int t = 0; t < LSB; ++t) {
            if (q0 + t0 + t < q1) {
                double mo = p.lam * uu[t];                               // -Om (Om1 :4191, :4267)
                if (p.rp) mo -= rr[t];
                if (p.KS) mo -= ss[t];
                y = fma(aa[t], y, gg[t] * mo);                           // g (A y - Om) as gA y + g (-Om)
            }
            yv[t0 + t] = y;
        }
    }
    // forward carries: compose (PF, y0_end) over segments 0..sgi; c_in of this segment
    double Pc = (live && q1 > q0) ? __ldg(sg.PF + (int64_t)line * SEGS + sgi) : 1.0;
    double Yc = (q1 > q0) ? y : 0.0;
#pragma unroll
    for (int d = 1; d < SEGS; d <<= 1) {
        const double Pp = __shfl_up_sync(0xffffffffu, Pc, d, SEGS), Yp = __shfl_up_sync(0xffffffffu, Yc, d, SEGS);
        if (sgi >= d) { Yc = fma(Pc, Yp, Yc); Pc *= Pp; }
    }
    const double yend = fma(Pc, g0, Yc);                 // true y at this segment's end
    double cin = __shfl_up_sync(0xffffffffu, yend, 1, SEGS);
    if (sgi == 0) cin = g0;
    const double ylast = __shfl_sync(0xffffffffu, yend, SEGS - 1, SEGS);   // y_{Nl-1}
    // right end: Dirichlet value or the flux closure of U1 (:4687-4719) with the old U[Nl-1]
    const double gN = p.bc ? p.bc[base + (int64_t)Nl * p.st] : 0.0;
    double uN;
    if (p.rkind == FPDE_BC_DIRICHLET) {
        uN = gN;
    } else {
        const double AlN = __ldg(p.al + (int64_t)(Nl - 1) * L + ln);
        if (fabs(ylast) > 1e-15) uN = (fabs(1.0 - AlN) > 1e-15) ? (ylast + gN * p.dLN) / (1.0 - AlN) : uold_last;
        else uN = (fabs(1.0 - AlN) > 1e-15) ? 0.0 : uold_last;
    }
    // backward from a zero carry over y0: ub0_q = al_q ub0_{q+1} + y0_q
    double u = 0.0;
#pragma unroll
    for (int t0 = SEGLEN - LSB; t0 >= 0; t0 -= LSB) {
        double al[LSB];
#pragma unroll
        for (int t = LSB - 1; t >= 0; --t) {
            const int q = q0 + t0 + t;
            al[t] = (live && q < q1) ? __ldg(p.al + (int64_t)q * L + line) : 0.0;
        }
#pragma unroll
        for (int t = LSB - 1; t >= 0; --t) {
            if (q0 + t0 + t < q1) u = fma(al[t], u, yv[t0 + t]);
            yv[t0 + t] = u;
        }
    }
    // backward carries: u at this segment's start = ub0_start + c_in KF_start + c_out CB_start
    const double kf0 = (live && q1 > q0) ? __ldg(sg.KF + (int64_t)q0 * L + line) : 0.0;
    double Qc = (live && q1 > q0) ? __ldg(sg.CB + (int64_t)q0 * L + line) : 1.0;
    double Uc = (q1 > q0) ? fma(cin, kf0, u) : 0.0;
#pragma unroll
    for (int d = 1; d < SEGS; d <<= 1) {
        const double Qn = __shfl_down_sync(0xffffffffu, Qc, d, SEGS), Un = __shfl_down_sync(0xffffffffu, Uc, d, SEGS);
        if (sgi + d < SEGS) { Uc = fma(Qc, Un, Uc); Qc *= Qn; }
    }
    const double ustart = fma(Qc, uN, Uc);               // true u at this segment's start
    double cout = __shfl_down_sync(0xffffffffu, ustart, 1, SEGS);
    if (sgi == SEGS - 1) cout = uN;
    const double u1 = __shfl_sync(0xffffffffu, ustart, 0, SEGS);        // U[1]
    if (!live) return;
#pragma unroll
    for (int t0 = 0; t0 < SEGLEN; t0 += LSB) {
        double kf[LSB], cb[LSB];
#pragma unroll
        for (int t = 0; t < LSB; ++t) {
            const int q = q0 + t0 + t;
            kf[t] = q < q1 ? __ldg(sg.KF + (int64_t)q * L + line) : 0.0;
            cb[t] = q < q1 ? __ldg(sg.CB + (int64_t)q * L + line) : 0.0;
        }
#pragma unroll
        for (int t = 0; t < LSB; ++t) {
            const int q = q0 + t0 + t;
            if (q < q1) p.U[base + (int64_t)q * p.st] = fma(cout, cb[t], fma(cin, kf[t], yv[t0 + t]));
        }
    }
    if (sgi == SEGS - 1) {
        p.U[base + (int64_t)Nl * p.st] = uN;
        p.U[base + (int64_t)(Nl + 1) * p.st] = uN;                  // ghost copy (U1 :4792)
    }
    if (sgi == 0) p.U[base] = fma(__ldg(p.al + line), u1, g0);    // Al[1] U[1] + Bt[1]
}

// The near history of the NEAR_SUB steps j0 .. j0+NEAR_SUB-1 of a 64-step block from the block's
// rows older than j0, with those steps' far partials: pre[u][i] = far(j0+u) + sum_{r<j0}
// w[j0+u-r] ring[r], in float-float (two nodes per thread, (hi, lo) of each). Each row is read
// once per NEAR_SUB steps instead of once per step; a step then adds only the rows of its own
// sub-block (k_near_history_ff with pre).
__global__ void __launch_bounds__(256) k_near_pre_ff(const float4 *__restrict__ ringf, int64_t P2, int j0,
                                                     const float2 *__restrict__ wff_all,
                                                     const double2 *__restrict__ cfar, int KS, int pairs,
                                                     float4 *__restrict__ pre, const int *__restrict__ cta_col,
                                                     int64_t wstride)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P2) return;
    const float2 *wff = cta_col ? wff_all + (int64_t)cta_col[blockIdx.x] * wstride : wff_all;
    float h[NEAR_SUB][2], l[NEAR_SUB][2];
#pragma unroll
    for (int u = 0; u < NEAR_SUB; ++u) h[u][0] = h[u][1] = l[u][0] = l[u][1] = 0.f;
    for (int q = 0; q < KS; ++q) {
#pragma unroll
        for (int u = 0; u < NEAR_SUB; ++u) {
            const double2 v = __ldcs(cfar + ((int64_t)q * 64 + j0 + u) * P2 + i);
            const float2 f0 = pairs ? *reinterpret_cast<const float2 *>(&v.x) : d2ff(v.x);
            const float2 f1 = pairs ? *reinterpret_cast<const float2 *>(&v.y) : d2ff(v.y);
            ff_add(h[u][0], l[u][0], f0.x, f0.y);
            ff_add(h[u][1], l[u][1], f1.x, f1.y);
        }
    }
    for (int r0 = 0; r0 < j0; r0 += NEAR_SUB) {          // j0 is a multiple of NEAR_SUB
        float4 v[NEAR_SUB];                                // the sub-block's rows, loaded together
#pragma unroll
        for (int q = 0; q < NEAR_SUB; ++q) v[q] = __ldcg(ringf + (int64_t)(r0 + q) * P2 + i);
#pragma unroll
        for (int q = 0; q < NEAR_SUB; ++q) {
#pragma unroll
            for (int u = 0; u < NEAR_SUB; ++u) {
                const float2 w = __ldg(wff + (j0 + u - r0 - q));
                ff_fma(h[u][0], l[u][0], w, make_float2(v[q].x, v[q].y));
                ff_fma(h[u][1], l[u][1], w, make_float2(v[q].z, v[q].w));
            }
        }
#pragma unroll
        for (int u = 0; u < NEAR_SUB; ++u) {
            ff_renorm(h[u][0], l[u][0]);
            ff_renorm(h[u][1], l[u][1]);
        }
    }
#pragma unroll
    for (int u = 0; u < NEAR_SUB; ++u) pre[(int64_t)u * P2 + i] = make_float4(h[u][0], l[u][0], h[u][1], l[u][1]);
}

// Two nodes per thread: S = far partials of step j + sum_{r<j} w[j-r] ring[r] in float-float; with
// pre (the sub-block's partial sums of k_near_pre_ff, sub-block start r0), S = pre[j-r0] + the rows
// r0 .. j-1.
__global__ void __launch_bounds__(256) k_near_history_ff(const float4 *__restrict__ ringf, int64_t P2, int j,
                                                         const float2 *__restrict__ wff_all,
                                                         const double2 *__restrict__ cfar, int KS, int pairs,
                                                         double2 *__restrict__ S, const int *__restrict__ cta_col,
                                                         int64_t wstride, const float4 *__restrict__ pre, int r0)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P2) return;
    const float2 *wff = cta_col ? wff_all + (int64_t)cta_col[blockIdx.x] * wstride : wff_all;
    float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
    if (pre) {
        const float4 v = __ldcs(pre + (int64_t)(j - r0) * P2 + i);
        h0 = v.x; l0 = v.y; h1 = v.z; l1 = v.w;
        KS = 0;
    }
    for (int q = 0; q < KS; ++q) {
        const double2 v = __ldcs(cfar + ((int64_t)q * 64 + j) * P2 + i);
        const float2 f0 = pairs ? *reinterpret_cast<const float2 *>(&v.x) : d2ff(v.x);
        const float2 f1 = pairs ? *reinterpret_cast<const float2 *>(&v.y) : d2ff(v.y);
        ff_add(h0, l0, f0.x, f0.y);
        ff_add(h1, l1, f1.x, f1.y);
    }
    int r = pre ? r0 : 0;
    for (; r + 8 <= j; r += 8) {
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = __ldcg(ringf + (int64_t)(r + u) * P2 + i);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const float2 w = __ldg(wff + (j - r - u));
            ff_fma(h0, l0, w, make_float2(v[u].x, v[u].y));
            ff_fma(h1, l1, w, make_float2(v[u].z, v[u].w));
        }
        ff_renorm(h0, l0);
        ff_renorm(h1, l1);
    }
    if (r < j) {                                           // the last (< 8) rows, loaded together
        const int rem = j - r;
        float4 v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = u < rem ? __ldcg(ringf + (int64_t)(r + u) * P2 + i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (u < rem) {
                const float2 w = __ldg(wff + (j - r - u));
                ff_fma(h0, l0, w, make_float2(v[u].x, v[u].y));
                ff_fma(h1, l1, w, make_float2(v[u].z, v[u].w));
            }
        }
    }
    S[i] = make_double2(f2d_bits(h0) + f2d_bits(l0), f2d_bits(h1) + f2d_bits(l1));
}

int launch_near_history_ff(cudaStream_t st, const float2 *ringf, int64_t P, int j, const float2 *wff,
                           const double *cfar, int KS, int pairs, double *S, const int *cta_col, int64_t wstride,
                           const float2 *pre, int r0)
{
    k_near_history_ff<<<(unsigned)((P / 2 + 255) / 256), 256, 0, st>>>((const float4 *)ringf, P / 2, j, wff,
                                                                       (const double2 *)cfar, KS, pairs,
                                                                       (double2 *)S, cta_col, wstride,
                                                                       (const float4 *)pre, r0);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

int launch_near_pre_ff(cudaStream_t st, const float2 *ringf, int64_t P, int j0, const float2 *wff, const double *cfar,
                       int KS, int pairs, float2 *pre, const int *cta_col, int64_t wstride)
{
    k_near_pre_ff<<<(unsigned)((P / 2 + 255) / 256), 256, 0, st>>>((const float4 *)ringf, P / 2, j0, wff,
                                                                   (const double2 *)cfar, KS, pairs, (float4 *)pre,
                                                                   cta_col, wstride);
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}


}  // namespace fpde

using namespace fpde;

struct fpde_lod3d {
    fpde_ctx *ctx = nullptr;
    fpde_lod3d_desc d{};
    int dims[3] = {0, 0, 0};                 // sN, M, K
    int64_t G = 0, P = 0;
    int max_steps = 0;
    int max_lag = INT_MAX;                    // restricted summing: lags above are dropped
    int series = 0;                           // series expansion: moments per point (0: off)
    double *H = nullptr;                      // [series][P] moments, moment-major
    std::vector<double> time;                 // Time[k], accumulated as the reference does
    double lam = 0.0, lamR = 0.0;
    double *U = nullptr, *last = nullptr, *D = nullptr, *part = nullptr, *wrev = nullptr;
    double *rp = nullptr, *bc = nullptr;
    int rp_rows = 0, bc_rows = 0;
    double *cA[3] = {nullptr, nullptr, nullptr}, *cg[3] = {nullptr, nullptr, nullptr},
           *cal[3] = {nullptr, nullptr, nullptr};
    // segmented passes (seg_shape: lines of up to 16 x 32 interior nodes): per-node responses KF, CB
    // and per-segment products PF; seglen 0 runs the one-thread-per-line kernel
    double *cKF[3] = {nullptr, nullptr, nullptr}, *cCB[3] = {nullptr, nullptr, nullptr},
           *cPF[3] = {nullptr, nullptr, nullptr};
    int seglen[3] = {0, 0, 0};
    int segs[3] = {0, 0, 0};
    int segcap[3] = {0, 0, 0};                     // the pass kernel's segment capacity (SEGLEN)
    int lines[3] = {0, 0, 0};
    // split path (exact three-slice far history on the tensor cores, FP64 near history)
    bool split = false;
    int64_t rows16 = 0, ld16 = 0, ldp = 0;
    uint16_t *h3[3] = {nullptr, nullptr, nullptr}, *w3[3] = {nullptr, nullptr, nullptr};
    int8_t *pA = nullptr;
    float *pW = nullptr;
    double *ring = nullptr, *cfar = nullptr, *wlag = nullptr, *Sn = nullptr;
    float2 *ringf = nullptr, *wff = nullptr;  // the ring and the lag weights as float pairs
    float2 *pre = nullptr;                    // near-history sums of the current 8-step sub-block
    FarPlan3 plan3;
    // Richards problem (desc.richards): coefficients from the solution every step
    bool rich = false;
    int rkform = 0;
    double rksat = 0.0;
    double *rsZ = nullptr, *rdL[3] = {nullptr, nullptr, nullptr}, *ral = nullptr;
    std::vector<double> rE;                   // evaporation rate per step
    // variable steps: per-step local terms, the scaled weight rows (row n: Da kb_n[t] / tau_t) and
    // the raw coefficients of every pass (the alpha recurrence is formed on the fly)
    bool vart = false;
    std::vector<double> lamv, lamRv;
    int64_t wld = 0;
    double *wrows = nullptr;
    double *vA[3] = {nullptr, nullptr, nullptr}, *vB[3] = {nullptr, nullptr, nullptr},
           *vR[3] = {nullptr, nullptr, nullptr}, *val = nullptr;
    // salt concentration C (equation 1) beside H: state, snapshot, its history and partials
    bool salt = false;
    double snu = 0.0, ssig = 1.0, sDc = 0.0;
    double *C = nullptr, *lastC = nullptr, *DC = nullptr, *partC = nullptr, *C0 = nullptr;
    // implicit space-fractional line solves (desc.space_frac): per pass the line-major operands
    // (per line A, B, Rlap, mc0, mc1, mc2, iw, Nl+1 values each) and the Toeplitz row
    bool sf = false, sf_fast = false;
    int sf_sd = 0, sf_maxit = 1;
    double sf_thr = 0.0;
    double *sfc[3] = {nullptr, nullptr, nullptr}, *sfT[3] = {nullptr, nullptr, nullptr};
    unsigned long long *sf_iters = nullptr;   // iterations of every line solve since creation
    // implicit3d (space_frac.implicit3d): the 3D system (Mat_3d, Mcoefs_3d, iw planes, Toeplitz rows),
    // the solve's right-hand side and iterate (V = G + 1 values) and its workspace
    bool sf3d = false, sf3d_exact = false;
    Sf3dSystem s3;
    Sf3dWork *s3work = nullptr;
    double *s3buf = nullptr;                  // mat 7V, mc 9V, iw 3V, Om V, x V, Tm rows
    int64_t n_done = 0;
    GraphCache<int> graphs;                        // captured runs (at least GRAPH_MIN_STEPS steps)
};

namespace fpde {

// Pass geometry (pass 0 = sN along i, 1 = _M along j, 2 = K along k): line count, the two
// line-index ranges (first fastest) with their strides, the node stride and Nl.
static void pass_geometry(const fpde_lod3d *L, int pass, int *Nl, int *n1, int *n2, int64_t *s1, int64_t *s2,
                          int64_t *st)
{
    const int sN = L->dims[0], M = L->dims[1], K = L->dims[2];
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    if (pass == 2) { *Nl = K; *n1 = sN - 1; *n2 = M - 1; *s1 = sx; *s2 = sy; *st = sz; }
    else if (pass == 1) { *Nl = M; *n1 = sN - 1; *n2 = K - 1; *s1 = sx; *s2 = sz; *st = sy; }
    else { *Nl = sN; *n1 = M - 1; *n2 = K - 1; *s1 = sy; *s2 = sz; *st = sx; }
}

static int lod_launch_pass(fpde_lod3d *L, cudaStream_t st, int pass, int64_t n, int KS)
{
    LodPassArgs a;
    int n2;
    pass_geometry(L, pass, &a.Nl, &a.n1, &n2, &a.s1, &a.s2, &a.st);
    a.lines = L->lines[pass];
    a.U = L->U;
    a.A = L->cA[pass]; a.g = L->cg[pass]; a.al = L->cal[pass];
    a.part = pass == 2 ? (L->split ? L->Sn : L->part) : nullptr;
    a.KS = pass == 2 ? KS : 0;
    a.pstride = L->P;
    a.rp = (pass == 2 && L->rp) ? L->rp + (n < L->rp_rows ? n : L->rp_rows - 1) * L->G : nullptr;
    a.bc = L->bc ? L->bc + (n < L->bc_rows ? n : L->bc_rows - 1) * L->G : nullptr;
    a.lam = L->vart ? L->lamv[(size_t)n] : L->lam;
    a.lkind = L->d.left_kind[pass];
    a.rkind = L->d.right_kind[pass];
    a.dLN = L->d.dLN[pass];
    if (a.lines <= 0) return FPDE_OK;
    if (L->vart) {
        LodVarArgs v;
        v.A = L->vA[pass]; v.B = L->vB[pass]; v.Rl = L->vR[pass]; v.al = L->val;
        v.lamR = L->lamRv[(size_t)n];
        k_lod_pass_var<<<(unsigned)((a.lines + 127) / 128), 128, 0, st>>>(a, v);
        FPDE_LAUNCHED(1);
        return FPDE_OK;
    }
    if (L->sf) {
        LodSfArgs f;
        int n2s;
        pass_geometry(L, pass, &f.Nl, &f.n1, &n2s, &f.s1, &f.s2, &f.st);
        f.lines = a.lines;
        f.U = L->U;
        f.coef = L->sfc[pass];
        f.Tm = L->sfT[pass];
        f.part = a.part; f.KS = a.KS; f.pstride = a.pstride;
        f.rp = a.rp; f.bc = a.bc;
        f.lam = L->lam; f.lamR = L->lamR; f.thr = L->sf_thr; f.dLN = a.dLN;
        f.sd = L->sf_sd; f.maxiter = L->sf_maxit; f.rkind = a.rkind;
        f.iters = L->sf_iters;
        f.flags = L->ctx->d_flags;
        f.fast = L->sf_fast ? 1 : 0;
        return launch_lod_pass_sf(st, f);
    }
    if (L->rich) {
        LodRichArgs r;
        r.sZ = L->rsZ; r.dL = L->rdL[pass]; r.al = L->ral;
        r.ksat = L->rksat; r.lamR = L->lamR; r.kform = L->rkform; r.pass = pass;
        r.E = L->rE[(size_t)std::min<int64_t>(n, (int64_t)L->rE.size() - 1)];
        if (L->salt) {
            r.C = L->C;
            r.partC = pass == 2 ? L->partC : nullptr;
            r.KSC = pass == 2 ? KS : 0;
            r.nu = L->snu; r.sigma = L->ssig; r.Dc = L->sDc;
        }
        k_lod_pass_rich<<<(unsigned)((a.lines + 127) / 128), 128, 0, st>>>(a, r);
    } else if (L->seglen[pass] > 0) {
        LodSegArgs sg;
        sg.KF = L->cKF[pass]; sg.CB = L->cCB[pass]; sg.PF = L->cPF[pass]; sg.seglen = L->seglen[pass];
        const int SG = L->segs[pass], SLC = L->segcap[pass];
        const unsigned blocks = (unsigned)(((int64_t)a.lines * SG + 127) / 128);
        switch (SG * 64 + SLC) {
        case 4 * 64 + 4: k_lod_pass_seg<4, 4><<<blocks, 128, 0, st>>>(a, sg); break;
        case 4 * 64 + 8: k_lod_pass_seg<4, 8><<<blocks, 128, 0, st>>>(a, sg); break;
        case 4 * 64 + 16: k_lod_pass_seg<4, 16><<<blocks, 128, 0, st>>>(a, sg); break;
        case 4 * 64 + 32: k_lod_pass_seg<4, 32><<<blocks, 128, 0, st>>>(a, sg); break;
        case 8 * 64 + 4: k_lod_pass_seg<8, 4><<<blocks, 128, 0, st>>>(a, sg); break;
        case 8 * 64 + 8: k_lod_pass_seg<8, 8><<<blocks, 128, 0, st>>>(a, sg); break;
        case 8 * 64 + 16: k_lod_pass_seg<8, 16><<<blocks, 128, 0, st>>>(a, sg); break;
        case 8 * 64 + 32: k_lod_pass_seg<8, 32><<<blocks, 128, 0, st>>>(a, sg); break;
        case 16 * 64 + 4: k_lod_pass_seg<16, 4><<<blocks, 128, 0, st>>>(a, sg); break;
        case 16 * 64 + 8: k_lod_pass_seg<16, 8><<<blocks, 128, 0, st>>>(a, sg); break;
        case 16 * 64 + 16: k_lod_pass_seg<16, 16><<<blocks, 128, 0, st>>>(a, sg); break;
        case 16 * 64 + 32: k_lod_pass_seg<16, 32><<<blocks, 128, 0, st>>>(a, sg); break;
        case 32 * 64 + 4: k_lod_pass_seg<32, 4><<<blocks, 128, 0, st>>>(a, sg); break;
        case 32 * 64 + 8: k_lod_pass_seg<32, 8><<<blocks, 128, 0, st>>>(a, sg); break;
        case 32 * 64 + 16: k_lod_pass_seg<32, 16><<<blocks, 128, 0, st>>>(a, sg); break;
        default: k_lod_pass_seg<32, 32><<<blocks, 128, 0, st>>>(a, sg); break;
        }
    } else {
        k_lod_pass<<<(unsigned)((a.lines + 127) / 128), 128, 0, st>>>(a);
    }
    FPDE_LAUNCHED(1);
    return FPDE_OK;
}

// Series expansion in the K pass (the reference's sum_alg 2, time_summing :4137-4151): with the
// newest increment d of every point, H_j += c_j d and part = Da sum_j v_j H_j / tau, in the
// reference's order j = 0 .. P-1. The moments are moment-major (row j over all points), so
// every access is coalesced; the step's coefficients come by value.
constexpr int LOD_SERIES_MAX = 128;
struct SeriesStep {
    double c[LOD_SERIES_MAX];   // g(Time[n])^(j+1) row2_j
    double v[LOD_SERIES_MAX];   // binomial series coefficients of (g(Time[n+1]) - s)^-alpha
    double Da, tau;
};

__global__ void __launch_bounds__(256) k_lod_series(const double *__restrict__ dnew, double *__restrict__ H,
                                                    int64_t ld, int P, const SeriesStep cf, double *__restrict__ part,
                                                    int64_t G)
{
    const int64_t id = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= G) return;
    const double d = dnew[id];
    double acc = 0.0;
    for (int j = 0; j < P; ++j) {
        const double h = fma(cf.c[j], d, H[(int64_t)j * ld + id]);
        H[(int64_t)j * ld + id] = h;
        acc = fma(cf.v[j], h, acc);
    }
    part[id] = cf.Da * (acc / cf.tau);
}

// Coefficients of step n (g(t) = t): row2_j = int_{t0}^{t1} s^j ds / t1^(j+1) over the newest
// interval [t0, t1] = [Time[n-1], Time[n]] (the reference's row2_precalc, _kb_row2 :2000-2131:
// (t1 - t0)/t1 for j = 0, (1 - (t0/t1)^(j+1))/(j+1) beyond), c_j = t1^(j+1) row2_j with the power
// formed by repeated multiplication, v_0 = T^-alpha and v_j = v_{j-1} (alpha + j - 1)/(j T),
// T = Time[n+1] (_kb_row2_fixed_coefs :1159-1180).
static void series_step(const fpde_lod3d *L, int64_t n, SeriesStep &cf)
{
    const int P = L->series;
    const double t0 = L->time[n - 1], t1 = L->time[n], T = L->time[n + 1], alpha = L->d.alpha;
    double mult = t1, v = std::pow(T, -alpha);
    for (int j = 0; j < P; ++j) {
        const double r = j == 0 ? (t1 - t0) / t1 : (1.0 - std::pow(t0 / t1, (double)(j + 1))) / (double)(j + 1);
        cf.c[j] = mult * r;
        cf.v[j] = v;
        mult *= t1;
        const double i = (double)(j + 1);
        v *= -(-alpha - i + 1.0) / (i * T);
    }
    cf.Da = L->d.Da;
    cf.tau = L->d.tau;
}

// One step of the fully implicit scheme (calc_step :5160-5716 with implicit3d 1): the right-hand
// side (and the grid as the initial guess), the solve over the G + 1 values, the grid back.
static int lod_sf3d_step(fpde_lod3d *L, cudaStream_t st, int64_t n, int KS)
{
    const int64_t V = L->G + 1;
    double *Om = L->s3buf + 19 * V, *x = L->s3buf + 20 * V;
    Sf3dRhsArgs r;
    r.sN = L->dims[0]; r.M = L->dims[1]; r.K = L->dims[2];
    r.U = L->U; r.x = x; r.Om = Om;
    r.rp = L->rp ? L->rp + (n < L->rp_rows ? n : L->rp_rows - 1) * L->G : nullptr;
    r.bc = L->bc ? L->bc + (n < L->bc_rows ? n : L->bc_rows - 1) * L->G : nullptr;
    r.part = L->split ? L->Sn : L->part;
    r.KS = KS;
    r.pstride = L->P;
    r.lam = L->lam;
    for (int q = 0; q < 3; ++q) { r.rkind[q] = L->d.right_kind[q]; r.dLN[q] = L->d.dLN[q]; }
    int rc;
    if ((rc = launch_sf3d_rhs(st, r))) return rc;
    if ((rc = sf3d_enqueue_solve(st, L->s3, L->s3work, Om, x, L->sf_thr, L->sf_maxit, L->sf3d_exact, L->sf_iters, nullptr,
                                 L->ctx->d_flags)))
        return rc;
    return launch_sf3d_store(st, x, L->U, L->G);
}

static int lod_enqueue(fpde_lod3d *L, cudaStream_t st, int64_t n0, int steps, int64_t *nk)
{
    int64_t k = 0;
    int rc;
    for (int64_t n = n0; n < n0 + steps; ++n) {
        int KS = 0;
        double *Drow;
        float2 *Drowf = nullptr;                                         // split: the float-pair ring row
        if (L->series) {                                             // moments, newest increment only
            if (n >= 1) {
                SeriesStep cf;
                series_step(L, n, cf);
                k_lod_series<<<(unsigned)((L->G + 255) / 256), 256, 0, st>>>(L->D + ((n - 1) & 1) * L->P, L->H, L->P,
                                                                            L->series, cf, L->part, L->G);
                FPDE_LAUNCHED(1);
                ++k;
                KS = 1;
            }
            Drow = L->D + (n & 1) * L->P;
        } else if (!L->split) {
            const int64_t t0 = n > L->max_lag ? n - L->max_lag : 0;    // oldest row of the window
            if (n - t0 >= 1) {
                KS = choose_splits((int)(n - t0), L->P);
                const double *wt = L->vart ? L->wrows + n * L->wld     // variable steps: row n
                                           : L->wrev + (L->max_steps - n);     // wt[t] = w[n - t]
                if ((rc = launch_l1_partial(st, L->D + t0 * L->P, L->P, (int)(n - t0), wt + t0, L->part, KS)))
                    return rc;
                ++k;
                if (L->salt) {                                           // C's own history, same weights
                    if ((rc = launch_l1_partial(st, L->DC + t0 * L->P, L->P, (int)(n - t0), wt + t0, L->partC, KS)))
                        return rc;
                    ++k;
                }
            }
            Drow = L->D + n * L->P;
        } else {
            const int64_t nb0 = n - n % 64;                          // block of 64 steps
            const int j = (int)(n - nb0);
            // far history columns [kb0, nb0): the 64-step tiles the window reaches
            const int64_t kb0 = nb0 > L->max_lag ? (nb0 - L->max_lag) / 64 * 64 : 0;
            const int far_kt = (int)((nb0 - kb0) / 64);
            int splits = 0;
            if (nb0 > 0) {
                splits = far_kt > 0 ? far_splits(far_kt, L->rows16) : 0;
                if (j == 0) {                                        // far history t < nb0
                    SplitPrep3 sp;
                    sp.ring = L->ring; sp.P = L->P; sp.nvalid = L->G; sp.ld = L->ld16; sp.wlag = L->wlag;
                    for (int q = 0; q < 3; ++q) { sp.hist[q] = L->h3[q]; sp.w[q] = L->w3[q]; }
                    sp.pA = L->pA; sp.pW = L->pW; sp.ldp = L->ldp;
                    if ((rc = launch_block_prep3(st, sp, nb0))) return rc;
                    k += 2;
                    if (far_kt > 0) {
                        if ((rc = far3_launch(st, &L->plan3, (int)nb0, L->cfar, (int64_t)64 * L->P, L->P, splits,
                                              L->pA, L->pW, L->ldp, L->ctx->d_flags, nullptr, (int)kb0)))
                            return rc;
                        ++k;
                    }
                }
            }
            if (n >= 1) {
                // rows older than the step's 8-step sub-block (and the far partials) are summed once
                // per sub-block; each step adds its sub-block's rows
                const int j0 = j - j % NEAR_SUB;
                const bool use_pre = splits > 0 || j0 > 0;
                if (use_pre && j == j0) {
                    if ((rc = launch_near_pre_ff(st, L->ringf, L->P, j0, L->wff, L->cfar, splits, 1, L->pre))) return rc;
                    ++k;
                }
                if ((rc = launch_near_history_ff(st, L->ringf, L->P, j, L->wff, L->cfar, splits, 1, L->Sn, nullptr, 0,
                                                 use_pre ? L->pre : nullptr, j0)))
                    return rc;
                ++k;
                KS = 1;
            }
            Drow = L->ring + (int64_t)j * L->P;
            Drowf = L->ringf + (int64_t)j * L->P;
        }
        if (L->sf3d) {                                               // one 3D solve (implicit3d 1)
            if ((rc = lod_sf3d_step(L, st, n, KS))) return rc;
            k += 3;
        } else {
            for (int pass = 2; pass >= 0; --pass) {                  // K, _M, sN (calc_step order)
                if ((rc = lod_launch_pass(L, st, pass, n, KS))) return rc;
                ++k;
            }
        }
        if ((rc = Drowf ? launch_append_ff(st, L->U, L->last, Drow, Drowf, L->G, L->P)
                        : launch_append(st, L->U, L->last, Drow, L->G, L->P)))
            return rc;
        ++k;
        if (L->salt) {
            if ((rc = launch_append(st, L->C, L->lastC, L->DC + n * L->P, L->G, L->P))) return rc;
            ++k;
        }
    }
    *nk = k;
    return FPDE_OK;
}

}  // namespace fpde

extern "C" {

int fpde_lod3d_destroy(fpde_lod3d *L)
{
    if (!L) return FPDE_OK;
    if (L->ctx) {
        cudaSetDevice(L->ctx->device);
        cudaStreamSynchronize(L->ctx->stream);
    }
    L->graphs.clear();
    dev_free(L->ringf);
    dev_free(L->wff);
    dev_free(L->pre);
    for (double *p : {L->U, L->last, L->D, L->part, L->wrev, L->rp, L->bc, L->ring, L->cfar, L->wlag, L->Sn, L->H})
        dev_free(p);
    for (int q = 0; q < 3; ++q) {
        dev_free(L->h3[q]);
        dev_free(L->w3[q]);
    }
    dev_free(L->pA);
    dev_free(L->pW);
    for (int q = 0; q < 3; ++q) {
        dev_free(L->cA[q]);
        dev_free(L->cg[q]);
        dev_free(L->cal[q]);
        dev_free(L->cKF[q]);
        dev_free(L->cCB[q]);
        dev_free(L->cPF[q]);
        dev_free(L->rdL[q]);
        dev_free(L->sfc[q]);
        dev_free(L->sfT[q]);
    }
    dev_free(L->sf_iters);
    sf3d_work_destroy(L->s3work);
    dev_free(L->s3buf);
    for (double *p : {L->C, L->lastC, L->DC, L->partC, L->C0}) dev_free(p);
    for (int q = 0; q < 3; ++q) {
        dev_free(L->vA[q]);
        dev_free(L->vB[q]);
        dev_free(L->vR[q]);
    }
    dev_free(L->val);
    dev_free(L->wrows);
    dev_free(L->rsZ);
    dev_free(L->ral);
    delete L;
    return FPDE_OK;
}

int fpde_lod3d_create(fpde_ctx *ctx, const fpde_lod3d_desc *desc, const double *coefA, const double *coefB,
                      const double *coefRlap, const double *u0, fpde_lod3d **out)
{
    clear_error();
    FPDE_CHECK_ARG(out && desc && u0, "null argument");
    *out = nullptr;
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    const fpde_lod3d_desc &d = *desc;
    const fpde_richards *rich = d.richards;
    FPDE_CHECK_ARG(rich || (coefA && coefB && coefRlap), "null coefficient grids");
    if (rich) {
        FPDE_CHECK_ARG(rich->k_form == 1 || rich->k_form == 2, "richards: k_form must be 1 or 2");
        FPDE_CHECK_ARG(rich->k_sat > 0.0 && std::isfinite(rich->k_sat), "richards: k_sat must be positive");
        FPDE_CHECK_ARG(rich->sZ && rich->dL[0] && rich->dL[1] && rich->dL[2], "richards: sZ and dL[3] required");
        FPDE_CHECK_ARG(rich->evaporation && rich->evaporation_rows >= 1, "richards: evaporation rows required");
        FPDE_CHECK_ARG(d.series_terms == 0, "richards: no series expansion");
        FPDE_CHECK_ARG(d.M <= d.sN + 1 && d.K <= d.sN + 1,
                       "richards: M and K at most sN + 1 (suctions index sZ by positions along every pass)");
        if (rich->salt_c0) {
            FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64, "richards salt: FP64 path only");
            FPDE_CHECK_ARG(std::isfinite(rich->salt_nu) && rich->salt_sigma > 0.0 && std::isfinite(rich->salt_D),
                           "richards salt: nu, sigma > 0 and D required");
        }
    }
    const fpde_space_frac *sfd = d.space_frac;
    if (sfd) {
        FPDE_CHECK_ARG(!rich, "space_frac: not with the Richards problem");
        FPDE_CHECK_ARG(sfd->space_der == 0 || sfd->space_der == 1, "space_frac: space_der must be 0 or 1");
        FPDE_CHECK_ARG(std::isfinite(sfd->tol) && sfd->tol >= 0.0, "space_frac: tol must be >= 0");
        FPDE_CHECK_ARG(sfd->max_iter >= 1 && sfd->max_iter <= FPDE_SF_MAX_ITER, "space_frac: max_iter out of range");
        FPDE_CHECK_ARG(d.sN <= FPDE_SF_MAX_N && d.M <= FPDE_SF_MAX_N && d.K <= FPDE_SF_MAX_N,
                       "space_frac: lines longer than FPDE_SF_MAX_N intervals");
        for (int q = 0; q < 3; ++q)
            FPDE_CHECK_ARG(sfd->Tm[q] && sfd->mc[q] && sfd->iw[q], "space_frac: Tm, mc and iw of every pass required");
        FPDE_CHECK_ARG(sfd->implicit3d == 0 || sfd->implicit3d == 1, "space_frac: implicit3d must be 0 or 1");
        FPDE_CHECK_ARG(!sfd->implicit3d || (int64_t)(d.sN + 2) * (d.M + 2) * (d.K + 2) + 1 < ((int64_t)1 << 31),
                       "space_frac: implicit3d needs (sN+2)(M+2)(K+2) + 1 below 2^31");
        FPDE_CHECK_ARG(!sfd->exact || !sfd->implicit3d ||
                           (int64_t)(d.sN + 2) * (d.M + 2) * (d.K + 2) + 1 <= FPDE_SF3D_MAX_EXACT,
                       "space_frac: exact dot products need at most FPDE_SF3D_MAX_EXACT values");
    }
    const bool vart = d.time_steps != nullptr;
    if (vart) {
        FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64, "time_steps: FP64 path only (per-step weight rows)");
        FPDE_CHECK_ARG(!d.lag_weights && d.series_terms == 0 && d.restrict_eps == 0.0 && !rich && !sfd,
                       "time_steps: not with lag_weights, series, restricted summing, richards or space_frac");
        for (int n = 0; n < d.max_steps; ++n)
            FPDE_CHECK_ARG(d.time_steps[n] > 0.0 && std::isfinite(d.time_steps[n]), "time_steps must be positive");
        FPDE_CHECK_ARG(std::isfinite(d.kernel_power) && d.kernel_power >= 0.0, "kernel_power must be >= 0");
    } else {
        FPDE_CHECK_ARG(!d.weight_rows, "weight_rows needs time_steps");
    }
    FPDE_CHECK_ARG(d.sN >= 2 && d.M >= 2 && d.K >= 2, "every axis needs at least 2 intervals");
    FPDE_CHECK_ARG(seg_request_ok(d.sN, d.segments[0]) && seg_request_ok(d.M, d.segments[1]) &&
                       seg_request_ok(d.K, d.segments[2]),
                   "segments: 0, or 4, 8, 16 or 32 with at most 32 interior nodes per segment");
    FPDE_CHECK_ARG(d.lag_weights || (d.alpha > 0.0 && d.alpha < 1.0), "alpha must be in (0, 1)");
    FPDE_CHECK_ARG(std::isfinite(d.restrict_eps) && d.restrict_eps >= 0.0, "restrict_eps must be >= 0");
    FPDE_CHECK_ARG(d.series_terms >= 0 && d.series_terms <= LOD_SERIES_MAX, "series_terms must be 0 .. 128");
    FPDE_CHECK_ARG(d.series_terms == 0 || (d.precision == FPDE_PREC_FP64 && !d.lag_weights && d.restrict_eps == 0.0),
                   "series expansion: FP64 path, Caputo weights, no restricted summing");
    FPDE_CHECK_ARG(d.tau > 0.0 && d.max_steps > 0, "tau and max_steps must be positive");
    FPDE_CHECK_ARG(d.precision == FPDE_PREC_FP64 || d.precision == FPDE_PREC_SPLIT_BF16X3,
                   "3D LOD: precision must be FP64 or the exact three-slice split");
    FPDE_CHECK_ARG(!d.source || d.source_rows >= 1, "source needs source_rows >= 1");
    FPDE_CHECK_ARG(!d.bc || d.bc_rows >= 1, "bc needs bc_rows >= 1");
    for (int q = 0; q < 3; ++q)
        FPDE_CHECK_ARG((d.left_kind[q] == 0 || d.left_kind[q] == 1) && (d.right_kind[q] == 0 || d.right_kind[q] == 1),
                       "bad boundary kind");

    fpde_lod3d *L = new fpde_lod3d();
    L->ctx = ctx;
    L->d = d;
    L->dims[0] = d.sN; L->dims[1] = d.M; L->dims[2] = d.K;
    L->G = (int64_t)(d.sN + 2) * (d.M + 2) * (d.K + 2);
    L->P = (L->G + 511) / 512 * 512;
    L->max_steps = d.max_steps;
    if (d.lag_weights) {
        L->lam = L->lamR = d.lag_weights[0];
    } else {                                   // lam as in Om1 (:4191), lamR as in R (:3120)
        const double kkk0 = l1_interval_weight(d.alpha, 0.0, d.tau);
        L->lam = d.Da * (kkk0 / d.tau);
        L->lamR = d.Da * kkk0 / d.tau;
    }
    const double kkk0 = d.lag_weights ? 0.0 : l1_interval_weight(d.alpha, 0.0, d.tau);
    auto wlag_of = [&](int64_t j) {
        return d.lag_weights ? (j <= L->max_steps ? d.lag_weights[j] : 0.0)
                             : d.Da * (kkk0 * l1_lag(d.alpha, j)) / d.tau;
    };
    // restricted summing (time_summing :4117-4131, newest first): the history stops before the
    // first lag whose kb = w tau / Da falls below restrict_eps; later lags get weight 0
    if (d.restrict_eps > 0.0) {
        std::vector<double> kbl(L->max_steps);
        for (int64_t j = 1; j <= L->max_steps; ++j) kbl[j - 1] = wlag_of(j) * d.tau / d.Da;
        int keep = 0;
        fpde_restricted_lags(kbl.data(), L->max_steps, d.restrict_eps, &keep);
        if (keep < L->max_steps) L->max_lag = keep;
    }
    auto wlag_at = [&](int64_t j) { return j > L->max_lag ? 0.0 : wlag_of(j); };
    std::vector<double> wrev(L->max_steps + 1, 0.0);               // wrev[m] = w[max_steps - m]
    for (int64_t m = 0; m < L->max_steps; ++m) wrev[m] = wlag_at(L->max_steps - m);
    const size_t gbytes = (size_t)L->G * sizeof(double), pbytes = (size_t)L->P * sizeof(double);
    L->split = d.precision == FPDE_PREC_SPLIT_BF16X3;
    L->series = d.series_terms;
    if (L->series) {                                               // Time[k+1] = Time[k] + tau (init_time_step)
        L->time.assign((size_t)L->max_steps + 2, 0.0);
        for (int64_t q = 1; q < (int64_t)L->time.size(); ++q) L->time[q] = L->time[q - 1] + d.tau;
    }
    bool fail = dev_alloc((void **)&L->U, pbytes) || dev_alloc((void **)&L->last, pbytes) ||
                dev_alloc((void **)&L->wrev, wrev.size() * sizeof(double));
    std::vector<double> wlag;
    if (!fail && L->series) {                                      // two increment rows and the moments
        fail = dev_alloc((void **)&L->D, 2 * pbytes) || dev_alloc((void **)&L->part, pbytes) ||
               dev_alloc((void **)&L->H, (size_t)L->series * pbytes);
    } else if (!fail && !L->split) {
        fail = dev_alloc((void **)&L->D, (size_t)L->max_steps * pbytes) ||
               dev_alloc((void **)&L->part, (size_t)KS_MAX * pbytes);
    } else if (!fail) {
        L->rows16 = (L->G + 127) / 128 * 128;
        L->ld16 = ((int64_t)L->max_steps + 63) / 64 * 64;
        L->ldp = L->ld16 / 64;
        const int64_t LW = L->max_steps + 64 + 1;
        wlag.assign(LW, 0.0);
        for (int64_t j = 1; j < LW; ++j) wlag[j] = wlag_at(j);
        for (int q = 0; q < 3 && !fail; ++q)
            fail = dev_alloc((void **)&L->h3[q], (size_t)L->rows16 * L->ld16 * 2) ||
                   dev_alloc((void **)&L->w3[q], (size_t)64 * L->ld16 * 2);
        fail = fail || dev_alloc((void **)&L->pA, (size_t)L->rows16 * L->ldp) ||
               dev_alloc((void **)&L->pW, (size_t)64 * L->ldp * sizeof(float)) ||
               dev_alloc((void **)&L->ring, (size_t)64 * pbytes) ||
               dev_alloc((void **)&L->cfar, (size_t)FAR_MAX_SPLITS * 64 * pbytes) ||
               dev_alloc((void **)&L->wlag, LW * sizeof(double)) || dev_alloc((void **)&L->Sn, pbytes) ||
               dev_alloc((void **)&L->ringf, (size_t)64 * L->P * sizeof(float2)) ||
               dev_alloc((void **)&L->pre, (size_t)NEAR_SUB * L->P * sizeof(float2)) ||
               dev_alloc((void **)&L->wff, LW * sizeof(float2));
        if (!fail) {
            const void *a3[3] = {L->h3[0], L->h3[1], L->h3[2]}, *w3[3] = {L->w3[0], L->w3[1], L->w3[2]};
            int rcp = far_plan3_init(&L->plan3, a3, L->rows16, L->ld16, w3, L->ld16);
            if (rcp) {
                std::string keep = fpde_last_error_string();
                fpde_lod3d_destroy(L);
                return set_error(rcp, "%s", keep.c_str());
            }
        }
    }
    if (!fail && d.source) {
        L->rp_rows = std::min(d.source_rows, d.max_steps);
        fail = dev_alloc((void **)&L->rp, (size_t)L->rp_rows * gbytes);
    }
    if (!fail && d.bc) {
        L->bc_rows = std::min(d.bc_rows, d.max_steps);
        fail = dev_alloc((void **)&L->bc, (size_t)L->bc_rows * gbytes);
    }
    cudaStream_t st = ctx->stream;
    if (!fail && rich) {                       // closures' inputs; no precomputed coefficients
        L->rich = true;
        L->rkform = rich->k_form;
        L->rksat = rich->k_sat;
        L->rE.assign(rich->evaporation, rich->evaporation + std::min(rich->evaporation_rows, d.max_steps));
        const int dims[3] = {d.sN, d.M, d.K};
        int64_t scratch = 0;
        for (int pass = 0; pass < 3 && !fail; ++pass) {
            int Nl, n1, n2;
            int64_t s1, s2, stp;
            pass_geometry(L, pass, &Nl, &n1, &n2, &s1, &s2, &stp);
            L->lines[pass] = n1 * n2;
            scratch = std::max<int64_t>(scratch, (int64_t)(Nl + 1) * n1 * n2);
            fail = dev_alloc((void **)&L->rdL[pass], (size_t)(dims[pass] + 2) * sizeof(double)) ||
                   cudaMemcpy(L->rdL[pass], rich->dL[pass], (size_t)(dims[pass] + 2) * sizeof(double),
                              cudaMemcpyHostToDevice) != cudaSuccess;
        }
        if (!fail && rich->salt_c0) {
            L->salt = true;
            L->snu = rich->salt_nu; L->ssig = rich->salt_sigma; L->sDc = rich->salt_D;
            fail = dev_alloc((void **)&L->C, pbytes) || dev_alloc((void **)&L->lastC, pbytes) ||
                   dev_alloc((void **)&L->C0, pbytes) || dev_alloc((void **)&L->DC, (size_t)L->max_steps * pbytes) ||
                   dev_alloc((void **)&L->partC, (size_t)KS_MAX * pbytes);
            if (!fail) {
                cudaMemset(L->C0, 0, pbytes);
                fail = cudaMemcpy(L->C0, rich->salt_c0, gbytes, cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(L->C, L->C0, pbytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
                       cudaMemcpy(L->lastC, L->C0, pbytes, cudaMemcpyDeviceToDevice) != cudaSuccess ||
                       cudaMemset(L->DC, 0, (size_t)L->max_steps * pbytes) != cudaSuccess;
            }
        }
        fail = fail || dev_alloc((void **)&L->rsZ, (size_t)(d.sN + 2) * sizeof(double)) ||
               cudaMemcpy(L->rsZ, rich->sZ, (size_t)(d.sN + 2) * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
               dev_alloc((void **)&L->ral, (size_t)scratch * sizeof(double));
    }
    if (!fail && sfd) {                        // operands of the space-fractional line systems
        L->sf = true;
        L->sf_fast = sfd->exact == 0;
        L->sf_sd = sfd->space_der;
        L->sf_thr = sfd->tol;
        L->sf_maxit = sfd->max_iter;
        fail = sf_prepare() != FPDE_OK || dev_alloc((void **)&L->sf_iters, sizeof(unsigned long long)) ||
               cudaMemset(L->sf_iters, 0, sizeof(unsigned long long)) != cudaSuccess;
        std::vector<double> hc;
        for (int pass = 0; pass < 3 && !fail && !sfd->implicit3d; ++pass) {
            int Nl, n1, n2;
            int64_t s1, s2, stp;
            pass_geometry(L, pass, &Nl, &n1, &n2, &s1, &s2, &stp);
            const int lines = n1 * n2, m = Nl + 1;
            L->lines[pass] = lines;
            hc.assign((size_t)lines * 7 * m, 0.0);
            const double *src[7] = {coefA + (int64_t)pass * L->G, coefB + (int64_t)pass * L->G,
                                    coefRlap + (int64_t)pass * L->G, sfd->mc[pass], sfd->mc[pass] + L->G,
                                    sfd->mc[pass] + 2 * L->G, sfd->iw[pass]};
            for (int line = 0; line < lines; ++line) {
                const int a = line % n1, b = line / n1;
                const int64_t base = (int64_t)(1 + a) * s1 + (int64_t)(1 + b) * s2;
                double *dst = hc.data() + (size_t)line * 7 * m;
                for (int r = 0; r < 7; ++r)
                    for (int q = 1; q < Nl; ++q) dst[(size_t)r * m + q] = src[r][base + (int64_t)q * stp];
            }
            std::vector<double> tm(sfd->Tm[pass], sfd->Tm[pass] + m);
            tm[0] = tm[1] = 0.0;                                      // never read
            fail = dev_alloc((void **)&L->sfc[pass], hc.size() * sizeof(double)) ||
                   dev_alloc((void **)&L->sfT[pass], (size_t)m * sizeof(double)) ||
                   cudaMemcpy(L->sfc[pass], hc.data(), hc.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                   cudaMemcpy(L->sfT[pass], tm.data(), (size_t)m * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
        }
        if (!fail && sfd->implicit3d) {        // the 3D system, constant over the steps (uniform tau)
            L->sf3d = true;
            L->sf3d_exact = sfd->exact != 0;
            const int64_t V = L->G + 1;
            const int len[3] = {d.sN, d.M, d.K};
            std::vector<double> mat, mc3, iw3;
            sf3d_assemble_host(d.sN, d.M, d.K, coefA, coefB, coefRlap, sfd->mc, sfd->iw, d.right_kind, L->lamR, mat,
                               mc3, iw3);
            const size_t rows = (size_t)(d.sN + d.M + d.K + 3);
            std::vector<double> buf((size_t)21 * V + rows, 0.0);
            std::copy(mat.begin(), mat.end(), buf.begin());
            std::copy(mc3.begin(), mc3.end(), buf.begin() + 7 * V);
            std::copy(iw3.begin(), iw3.end(), buf.begin() + 16 * V);
            size_t o = (size_t)21 * V;
            for (int c = 0; c < 3; ++c) {
                for (int q = 2; q <= len[c]; ++q) buf[o + q] = sfd->Tm[c][q];   // entries 0 and 1 never read
                o += (size_t)len[c] + 1;
            }
            fail = dev_alloc((void **)&L->s3buf, buf.size() * sizeof(double)) ||
                   cudaMemcpy(L->s3buf, buf.data(), buf.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
            if (!fail) {
                Sf3dSystem &S3 = L->s3;
                S3.sN = d.sN; S3.M = d.M; S3.K = d.K; S3.sd = sfd->space_der;
                S3.mat = L->s3buf; S3.mc = L->s3buf + 7 * V; S3.iw = L->s3buf + 16 * V; S3.rs = nullptr;
                S3.Tm[0] = L->s3buf + 21 * V;
                S3.Tm[1] = S3.Tm[0] + d.sN + 1;
                S3.Tm[2] = S3.Tm[1] + d.M + 1;
                fail = sf3d_work_create(S3, &L->s3work) != FPDE_OK;
            }
        }
    }
    if (!fail && vart) {
        // weight rows of every step: the caller's (its kb_3_cache and kkk0), or fpde_weights_g on the
        // accumulated time points; then the local terms Da kkk0_n / tau_n (Om1 :4191, R :3120) and the
        // GEMV rows Da kb_n[t] / tau_t
        L->vart = true;
        const int S = d.max_steps;
        const int64_t ld = (int64_t)S + 1;
        L->wld = ld;
        std::vector<double> W((size_t)S * ld, 0.0);
        if (d.weight_rows) {
            std::copy(d.weight_rows, d.weight_rows + (size_t)S * ld, W.begin());
        } else {
            std::vector<double> T((size_t)S + 1, 0.0);
            for (int k = 0; k < S; ++k) T[k + 1] = T[k] + d.time_steps[k];
            const double pw = d.kernel_power > 0.0 ? d.kernel_power : 1.0;
            if (fpde_weights_g(ctx, pw, d.alpha, T.data(), 0, S - 1, W.data(), ld, 0) != FPDE_OK) fail = true;
        }
        L->lamv.assign(S, 0.0);
        L->lamRv.assign(S, 0.0);
        std::vector<double> Ws((size_t)S * ld, 0.0);
        for (int n = 0; n < S; ++n) {
            const double k0 = W[(size_t)n * ld + n], tn = d.time_steps[n];
            L->lamv[n] = d.Da * (k0 / tn);
            L->lamRv[n] = d.Da * k0 / tn;
            for (int t = 0; t < n; ++t) Ws[(size_t)n * ld + t] = (d.Da * W[(size_t)n * ld + t]) / d.time_steps[t];
        }
        fail = fail || dev_alloc((void **)&L->wrows, Ws.size() * sizeof(double)) ||
               cudaMemcpy(L->wrows, Ws.data(), Ws.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
        int64_t scratch = 0;
        std::vector<double> h[3];
        for (int pass = 0; pass < 3 && !fail; ++pass) {
            int Nl, n1, n2;
            int64_t s1, s2, stp;
            pass_geometry(L, pass, &Nl, &n1, &n2, &s1, &s2, &stp);
            const int lines = n1 * n2;
            L->lines[pass] = lines;
            const size_t cnt = (size_t)(Nl + 1) * lines;
            scratch = std::max<int64_t>(scratch, (int64_t)cnt);
            const double *src[3] = {coefA + (int64_t)pass * L->G, coefB + (int64_t)pass * L->G,
                                    coefRlap + (int64_t)pass * L->G};
            double **dst[3] = {&L->vA[pass], &L->vB[pass], &L->vR[pass]};
            for (int r = 0; r < 3 && !fail; ++r) {
                h[r].assign(cnt, 0.0);
                for (int line = 0; line < lines; ++line) {
                    const int a = line % n1, b = line / n1;
                    const int64_t base = (int64_t)(1 + a) * s1 + (int64_t)(1 + b) * s2;
                    for (int q = 1; q < Nl; ++q) h[r][(size_t)q * lines + line] = src[r][base + (int64_t)q * stp];
                }
                fail = dev_alloc((void **)dst[r], cnt * sizeof(double)) ||
                       cudaMemcpy(*dst[r], h[r].data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
            }
        }
        fail = fail || dev_alloc((void **)&L->val, (size_t)scratch * sizeof(double));
    }
    // per-pass line coefficients, evaluated in the reference's order (al1 :4002-4027)
    std::vector<double> hA, hg, hal;
    for (int pass = 0; pass < 3 && !fail && !rich && !sfd && !vart; ++pass) {
        int Nl, n1, n2;
        int64_t s1, s2, stp;
        pass_geometry(L, pass, &Nl, &n1, &n2, &s1, &s2, &stp);
        const int lines = n1 * n2;
        L->lines[pass] = lines;
        const size_t cnt = (size_t)(Nl + 1) * lines;
        hA.assign(cnt, 0.0);
        hg.assign(cnt, 0.0);
        hal.assign(cnt, 0.0);
        const double *cA = coefA + (int64_t)pass * L->G, *cB = coefB + (int64_t)pass * L->G,
                     *cR = coefRlap + (int64_t)pass * L->G;
        for (int line = 0; line < lines; ++line) {
            const int a = line % n1, b = line / n1;
            const int64_t base = (int64_t)(1 + a) * s1 + (int64_t)(1 + b) * s2;
            double Al = d.left_kind[pass] == FPDE_BC_FLUX ? 1.0 : 0.0;            // Al[1]
            hal[line] = Al;
            for (int q = 1; q < Nl; ++q) {
                const int64_t id = base + (int64_t)q * stp;
                const double R = cR[id] + L->lamR;
                const double Aq = cA[id], Bq = cB[id];
                Al = Bq / (R - Aq * Al);                                           // Al[q+1]
                hal[(size_t)q * lines + line] = Al;
                hg[(size_t)q * lines + line] = Al / Bq;
                hA[(size_t)q * lines + line] = (Al / Bq) * Aq;                      // gA = g A
            }
        }
        fail = dev_alloc((void **)&L->cA[pass], cnt * sizeof(double)) ||
               dev_alloc((void **)&L->cg[pass], cnt * sizeof(double)) ||
               dev_alloc((void **)&L->cal[pass], cnt * sizeof(double));
        if (!fail) {                                                  // synchronous: host vectors are reused
            fail = cudaMemcpy(L->cA[pass], hA.data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                   cudaMemcpy(L->cg[pass], hg.data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                   cudaMemcpy(L->cal[pass], hal.data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
            if (fail) set_error(FPDE_ERR_CUDA, "lod3d: coefficient upload failed");
        }
        // segmented pass data: segment s holds nodes [1 + s seglen, 1 + (s+1) seglen) of 1..Nl-1
        int SG = 0, SL = 0;
        seg_shape(Nl, d.segments[pass], &SG, &SL);
        const int sl = SG ? (Nl - 1 + SG - 1) / SG : 0;
        if (!fail && Nl >= 2 && SG > 0 && sl <= SL) {
            std::vector<double> hKF(cnt, 0.0), hCB(cnt, 0.0), hPF((size_t)lines * SG, 1.0), cf(SL);
            for (int line = 0; line < lines; ++line) {
                for (int sgi = 0; sgi < SG; ++sgi) {
                    const int q0 = 1 + sgi * sl, q1 = std::min(q0 + sl, Nl);
                    double pr = 1.0;
                    for (int q = q0; q < q1; ++q) {
                        const size_t o = (size_t)q * lines + line;
                        pr *= hA[o];                                       // prefix product of a = g A
                        cf[q - q0] = pr;
                    }
                    hPF[(size_t)line * SG + sgi] = pr;
                    double kf = 0.0, cb = 1.0;
                    for (int q = q1 - 1; q >= q0; --q) {
                        const size_t o = (size_t)q * lines + line;
                        kf = hal[o] * kf + cf[q - q0];                      // backward sweep of CF
                        cb = hal[o] * cb;                                  // suffix product of al
                        hKF[o] = kf;
                        hCB[o] = cb;
                    }
                }
            }
            fail = dev_alloc((void **)&L->cKF[pass], cnt * sizeof(double)) ||
                   dev_alloc((void **)&L->cCB[pass], cnt * sizeof(double)) ||
                   dev_alloc((void **)&L->cPF[pass], hPF.size() * sizeof(double));
            if (!fail) {
                fail = cudaMemcpy(L->cKF[pass], hKF.data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(L->cCB[pass], hCB.data(), cnt * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess ||
                       cudaMemcpy(L->cPF[pass], hPF.data(), hPF.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess;
                if (fail) set_error(FPDE_ERR_CUDA, "lod3d: coefficient upload failed");
            }
            if (!fail) {
                L->seglen[pass] = sl;
                L->segs[pass] = SG;
                L->segcap[pass] = SL;
            }
        }
    }
    if (fail) {
        std::string keep = fpde_last_error_string();
        fpde_lod3d_destroy(L);
        return set_error(FPDE_ERR_NOMEM, "%s", keep.c_str());
    }
    cudaMemsetAsync(L->U, 0, pbytes, st);
    cudaMemcpyAsync(L->U, u0, gbytes, cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(L->last, 0, pbytes, st);
    cudaMemcpyAsync(L->last, u0, gbytes, cudaMemcpyHostToDevice, st);
    if (L->series) {
        cudaMemsetAsync(L->D, 0, 2 * pbytes, st);
        cudaMemsetAsync(L->H, 0, (size_t)L->series * pbytes, st);
    } else if (!L->split) {
        cudaMemsetAsync(L->D, 0, (size_t)L->max_steps * pbytes, st);
    } else {
        for (int q = 0; q < 3; ++q) {
            cudaMemsetAsync(L->h3[q], 0, (size_t)L->rows16 * L->ld16 * 2, st);
            cudaMemsetAsync(L->w3[q], 0, (size_t)64 * L->ld16 * 2, st);
        }
        cudaMemsetAsync(L->pA, 0, (size_t)L->rows16 * L->ldp, st);
        cudaMemsetAsync(L->pW, 0, (size_t)64 * L->ldp * sizeof(float), st);
        cudaMemsetAsync(L->ring, 0, (size_t)64 * pbytes, st);
        cudaMemsetAsync(L->cfar, 0, (size_t)FAR_MAX_SPLITS * 64 * pbytes, st);
        cudaMemcpyAsync(L->wlag, wlag.data(), wlag.size() * sizeof(double), cudaMemcpyHostToDevice, st);
        std::vector<float2> wff(wlag.size());          // w = hi + lo, hi the nearest float
        for (size_t q = 0; q < wlag.size(); ++q) {
            const float hi = (float)wlag[q];
            wff[q] = make_float2(hi, (float)(wlag[q] - (double)hi));
        }
        cudaMemcpyAsync(L->wff, wff.data(), wff.size() * sizeof(float2), cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(L->ringf, 0, (size_t)64 * L->P * sizeof(float2), st);
    }
    cudaMemcpyAsync(L->wrev, wrev.data(), wrev.size() * sizeof(double), cudaMemcpyHostToDevice, st);
    if (L->rp) cudaMemcpyAsync(L->rp, d.source, (size_t)L->rp_rows * gbytes, cudaMemcpyHostToDevice, st);
    if (L->bc) cudaMemcpyAsync(L->bc, d.bc, (size_t)L->bc_rows * gbytes, cudaMemcpyHostToDevice, st);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        fpde_lod3d_destroy(L);
        return set_error(FPDE_ERR_CUDA, "lod3d setup: %s", cudaGetErrorString(e));
    }
    L->d.lag_weights = nullptr;                 // host pointers are not kept
    L->d.source = nullptr;
    L->d.bc = nullptr;
    L->d.richards = nullptr;
    L->d.space_frac = nullptr;
    L->d.time_steps = nullptr;
    L->d.weight_rows = nullptr;
    *out = L;
    return FPDE_OK;
}

int fpde_lod3d_run(fpde_lod3d *L, int steps)
{
    clear_error();
    FPDE_CHECK_ARG(L && steps >= 0, "bad arguments");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    if (steps == 0) return FPDE_OK;
    if (L->n_done + steps > L->max_steps)
        return set_error(FPDE_ERR_CAPACITY, "run of %d steps exceeds the history capacity %d", steps, L->max_steps);
    if (steps < GRAPH_MIN_STEPS) {                 // short runs: enqueued directly, no graph
        int64_t nk = 0;
        if ((rc = lod_enqueue(L, L->ctx->stream, L->n_done, steps, &nk))) return rc;
    } else {
        auto *g = L->graphs.find(L->n_done, steps);
        if (!g) {
            rc = L->graphs.capture(L->n_done, steps,
                                   [&](cudaStream_t cs, int64_t *nk, int *) { return lod_enqueue(L, cs, L->n_done, steps, nk); },
                                   &g);
            if (rc) return rc;
        }
        FPDE_CUDA(cudaGraphLaunch(g->exec, L->ctx->stream));
        count_launches(g->launches);
    }
    L->n_done += steps;
    return FPDE_OK;
}

int fpde_lod3d_get_state(fpde_lod3d *L, double *u, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(L && u, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u, L->U, L->G * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, L->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    return ctx_check_flags(L->ctx, "lod3d");
}

int fpde_lod3d_get_concentration(fpde_lod3d *L, double *c, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(L && c, "null argument");
    if (!L->salt) return set_error(FPDE_ERR_ARG, "lod3d: no salt concentration (richards.salt_c0 not given)");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    FPDE_CUDA(cudaMemcpyAsync(c, L->C, L->G * sizeof(double),
                              on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, L->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    return ctx_check_flags(L->ctx, "lod3d");
}

int fpde_lod3d_reset(fpde_lod3d *L, const double *u0, int on_device)
{
    clear_error();
    FPDE_CHECK_ARG(L && u0, "null argument");
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    const cudaMemcpyKind kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    FPDE_CUDA(cudaMemcpyAsync(L->U, u0, L->G * sizeof(double), kind, L->ctx->stream));
    FPDE_CUDA(cudaMemcpyAsync(L->last, u0, L->G * sizeof(double), kind, L->ctx->stream));
    if (L->series)                                   // an empty history: the moments start at zero
        FPDE_CUDA(cudaMemsetAsync(L->H, 0, (size_t)L->series * L->P * sizeof(double), L->ctx->stream));
    if (L->salt) {                                   // the salt field starts again from its initial grid
        FPDE_CUDA(cudaMemcpyAsync(L->C, L->C0, L->P * sizeof(double), cudaMemcpyDeviceToDevice, L->ctx->stream));
        FPDE_CUDA(cudaMemcpyAsync(L->lastC, L->C0, L->P * sizeof(double), cudaMemcpyDeviceToDevice, L->ctx->stream));
    }
    if (!on_device) FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    L->n_done = 0;
    return FPDE_OK;
}

int fpde_lod3d_solve_host(fpde_lod3d *L, const double *u0_host, int steps, double *u_out_host)
{
    clear_error();
    FPDE_CHECK_ARG(L && u0_host && u_out_host, "null argument");
    int rc = fpde_lod3d_reset(L, u0_host, 0);
    if (rc) return rc;
    if ((rc = fpde_lod3d_run(L, steps))) return rc;
    FPDE_CUDA(cudaMemcpyAsync(u_out_host, L->U, L->G * sizeof(double), cudaMemcpyDeviceToHost, L->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    return ctx_check_flags(L->ctx, "lod3d");
}

int fpde_lod3d_sf_iterations(fpde_lod3d *L, int64_t *iters)
{
    clear_error();
    FPDE_CHECK_ARG(L && iters, "null argument");
    *iters = 0;
    if (!L->sf) return FPDE_OK;
    int rc = ctx_enter(L->ctx);
    if (rc) return rc;
    unsigned long long v = 0;
    FPDE_CUDA(cudaMemcpyAsync(&v, L->sf_iters, sizeof v, cudaMemcpyDeviceToHost, L->ctx->stream));
    FPDE_CUDA(cudaStreamSynchronize(L->ctx->stream));
    *iters = (int64_t)v;
    return FPDE_OK;
}

int fpde_lod3d_autotune(fpde_ctx *ctx, const fpde_lod3d_desc *desc, const double *coefA, const double *coefB,
                        const double *coefRlap, const double *u0, int steps, int segments[3], double *ms_per_step)
{
    clear_error();
    FPDE_CHECK_ARG(ctx && desc && u0 && segments && ms_per_step, "null argument");
    FPDE_CHECK_ARG(steps >= 1 && steps <= desc->max_steps, "steps must be 1 .. max_steps");
    int rc = ctx_enter(ctx);
    if (rc) return rc;
    const int lens[3] = {desc->sN, desc->M, desc->K};
    const int cand[5] = {0, 4, 8, 16, 32};
    double best = -1.0;
    int bestseg[3] = {0, 0, 0};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    FPDE_CUDA(cudaEventCreate(&e0));
    FPDE_CUDA(cudaEventCreate(&e1));
    for (int ci = 0; ci < 5 && !rc; ++ci) {
        fpde_lod3d_desc d = *desc;
        bool takes = cand[ci] == 0;
        for (int p = 0; p < 3; ++p) {
            d.segments[p] = (cand[ci] > 0 && seg_request_ok(lens[p], cand[ci])) ? cand[ci] : 0;
            takes = takes || d.segments[p] != 0;
        }
        if (!takes) continue;
        fpde_lod3d *L = nullptr;
        if ((rc = fpde_lod3d_create(ctx, &d, coefA, coefB, coefRlap, u0, &L))) break;
        float ms = 0.f;
        rc = fpde_lod3d_run(L, steps);                       // warm-up (and the graph's capture)
        if (!rc) rc = fpde_lod3d_reset(L, u0, 0);
        if (!rc) {
            cudaEventRecord(e0, ctx->stream);
            rc = fpde_lod3d_run(L, steps);
            cudaEventRecord(e1, ctx->stream);
        }
        if (!rc && cudaEventSynchronize(e1) == cudaSuccess && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess) {
            if (best < 0.0 || ms < best) {
                best = ms;
                for (int p = 0; p < 3; ++p) bestseg[p] = d.segments[p];
            }
        }
        fpde_lod3d_destroy(L);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    if (best < 0.0) return set_error(FPDE_ERR_CUDA, "lod3d autotune: no candidate could be timed");
    for (int p = 0; p < 3; ++p) segments[p] = bestseg[p];
    *ms_per_step = best / steps;
    return FPDE_OK;
}

int fpde_lod3d_steps_done(const fpde_lod3d *L, int64_t *n)
{
    FPDE_CHECK_ARG(L && n, "null argument");
    *n = L->n_done;
    return FPDE_OK;
}

}  // extern "C"
