/* fpde_oracle -- CPU restatement of FPDE_HPC's hot path (test infrastructure only; see
 * fpde_oracle.h). Every function follows the reference's operation order so that the
 * golden vectors produced by the reference's own FP64 code are met to rounding level.
 * Compiled with -ffp-contract=off, like the reference build (x86-64 baseline, no FMA). */
#define _DEFAULT_SOURCE
#include "fpde_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- weights */

/* int_{s0}^{s1} (T - s)^{-alpha} ds with a = T - s1 >= 0, d = s1 - s0 > 0, in the
 * cancellation-free form a^{1-alpha} expm1((1-alpha) log1p(d/a)) / (1-alpha). This is the
 * closed form of kb (fpde_hpc_1d.cpp:2167-2301) for g(t) = t, which the reference
 * evaluates by truncated series (_kb_row :1933, _kb_row2 :2000). */
static double l1_interval_weight(double alpha, double a, double d)
{
    double e = 1.0 - alpha;
    if (a <= 0.0) return pow(d, e) / e;
    return pow(a, e) * expm1(e * log1p(d / a)) / e;
}

void fo_l1_weights(double alpha, const double *time, int n, double *kb, double *kkk0)
{
    double T1 = time[n + 1];
    if (alpha == 1.0) {                      /* kb :2169-2175 */
        for (int t = 0; t < n; t++) kb[t] = 0.0;
        if (kkk0) *kkk0 = 1.0;
        return;
    }
    for (int t = 0; t < n; t++)
        kb[t] = l1_interval_weight(alpha, T1 - time[t + 1], time[t + 1] - time[t]);
    if (kkk0) *kkk0 = l1_interval_weight(alpha, 0.0, T1 - time[n]);
}

/* Quadrature rules of fo_weights_g: double-exponential nodes t = k/8, |k| <= 28, mapped to
 * (0, 1) by u = 1/(1 + e^{-pi sinh t}) (v = 1 - u formed directly), and 16- and 8-point
 * Gauss-Legendre on (0, 1) by Newton iteration on P_m. */
#define WG_DE 57
#define WG_GL 16
#define WG_GL8 8
static double wg_u[WG_DE], wg_v[WG_DE], wg_w[WG_DE], wg_x[WG_GL], wg_gw[WG_GL], wg_x8[WG_GL8], wg_gw8[WG_GL8];
static int wg_ready = 0;

static double wg_legendre(int m, double z, double *d)
{
    double p0 = 1.0, p1 = z;
    for (int k = 2; k <= m; k++) {
        double p2 = ((2.0 * k - 1.0) * z * p1 - (k - 1.0) * p0) / k;
        p0 = p1;
        p1 = p2;
    }
    *d = m * (z * p1 - p0) / (z * z - 1.0);
    return p1;
}

static void wg_gauss_legendre(int m, double *x01, double *w01)
{
    const double pi = 3.14159265358979323846;
    for (int i = 0; i < m; i++) {
        double x = cos(pi * (i + 0.75) / (m + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double dx = wg_legendre(m, x, &dp) / dp;
            x -= dx;
            if (fabs(dx) < 1e-17) break;
        }
        wg_legendre(m, x, &dp);
        x01[i] = 0.5 * (x + 1.0);
        w01[i] = 1.0 / ((1.0 - x * x) * dp * dp);   /* 2/((1-x^2)P'^2) on (-1,1), halved */
    }
}

static void wg_init(void)
{
    if (wg_ready) return;
    const double pi = 3.14159265358979323846;
    for (int k = 0; k < WG_DE; k++) {
        double t = (k - 28) / 8.0;
        double e = exp(pi * sinh(t));
        wg_u[k] = e / (1.0 + e);
        wg_v[k] = 1.0 / (1.0 + e);
        wg_w[k] = (pi / 8.0) * cosh(t) * wg_u[k] * wg_v[k];
    }
    wg_gauss_legendre(WG_GL, wg_x, wg_gw);
    wg_gauss_legendre(WG_GL8, wg_x8, wg_gw8);
    wg_ready = 1;
}

/* T^p - s^p with delta = T - s (both given; no cancellation for small delta) */
static double wg_gdiff(double delta, double s, double T, double p, double Tp)
{
    if (p == 1.0) return delta;
    if (delta < 0.5 * T) return -Tp * expm1(p * log1p(-delta / T));
    return Tp - pow(s, p);
}

static double wg_interval(double s0, double s1, double T, double p, double alpha)
{
    const double wdt = s1 - s0, d1 = T - s1, Tp = pow(T, p);
    double sum = 0.0;
    if (d1 == 0.0) {                                   /* newest: delta^-alpha on [0, wdt/16] */
        const double hw = wdt / 16.0, q = 1.0 / (1.0 - alpha), R0 = pow(p * pow(T, p - 1.0), -alpha);
        double a = 0.0, b = 0.0;
        for (int k = 0; k < WG_DE; k++) {
            double delta = hw * pow(wg_u[k], q);
            double R = delta > 0.0 ? pow(wg_gdiff(delta, T - delta, T, p, Tp) / delta, -alpha) : R0;
            a += wg_w[k] * R;
        }
        const double rest = wdt - hw;
        for (int k = 0; k < WG_DE; k++) {
            double delta = hw + rest * wg_u[k], s = s0 + rest * wg_v[k];
            b += wg_w[k] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
        }
        return pow(hw, 1.0 - alpha) / (1.0 - alpha) * a + rest * b;
    }
    const int smooth0 = p >= 1.0 && p == floor(p);
    if (d1 < 4.0 * wdt || (!smooth0 && s0 < 4.0 * wdt)) {
        for (int k = 0; k < WG_DE; k++) {
            double delta = d1 + wdt * wg_u[k], s = s0 + wdt * wg_v[k];
            sum += wg_w[k] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
        }
        return wdt * sum;
    }
    if (d1 < 32.0 * wdt || (!smooth0 && s0 < 32.0 * wdt)) {
        for (int i = 0; i < WG_GL; i++) {
            double s = s0 + wdt * wg_x[i], delta = d1 + wdt * (1.0 - wg_x[i]);
            sum += wg_gw[i] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
        }
        return wdt * sum;
    }
    for (int i = 0; i < WG_GL8; i++) {
        double s = s0 + wdt * wg_x8[i], delta = d1 + wdt * (1.0 - wg_x8[i]);
        sum += wg_gw8[i] * pow(wg_gdiff(delta, s, T, p, Tp), -alpha);
    }
    return wdt * sum;
}

void fo_weights_g(double p, double alpha, const double *time, int n, double *kb, double *kkk0)
{
    wg_init();
    const double T = time[n + 1];
    if (alpha == 1.0) {                                /* kb :2169-2175 */
        for (int t = 0; t < n; t++) kb[t] = 0.0;
        if (kkk0) *kkk0 = 1.0;
        return;
    }
#pragma omp parallel for schedule(dynamic, 64)
    for (int t = 0; t < n; t++) kb[t] = wg_interval(time[t], time[t + 1], T, p, alpha);
    if (kkk0) *kkk0 = wg_interval(time[n], T, T, p, alpha);
}

/* ------------------------------------------------------------ history sum */

/* Every node's sum starts at 0 and adds its terms from t = n-1 down to 0 (time_summing :4111,
 * newest first) in the reference's order and rounding; the loops visit t outside a block of nodes
 * so that each history row is read contiguously, node blocks in parallel. */
#define FO_NODE_BLOCK 2048
void fo_l1_sum(const double *D, int64_t P, int n, const double *kb, const double *tau,
               int64_t i0, int64_t i1, double *S)
{
    const int64_t nblk = (i1 - i0 + FO_NODE_BLOCK - 1) / FO_NODE_BLOCK;
#pragma omp parallel for schedule(static)
    for (int64_t b = 0; b < nblk; b++) {
        const int64_t a = i0 + b * FO_NODE_BLOCK, e = a + FO_NODE_BLOCK < i1 ? a + FO_NODE_BLOCK : i1;
        for (int64_t i = a; i < e; i++) S[i] = 0.0;
        for (int t = n - 1; t >= 0; t--) {
            const double *row = D + (int64_t)t * P;
            const double c = kb[t], tt = tau[t];
            for (int64_t i = a; i < e; i++) S[i] += c * row[i] / tt;
        }
    }
}

void fo_l1_sum_snapshots(const double *old, int64_t OS, int nold, const double *kb,
                         const double *tau, int64_t nodes, double *S)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nodes; i++) {
        double s = 0.0;
        for (int t = nold - 2; t >= 0; t--) {
            double diff = old[(int64_t)(t + 1) * OS + i] - old[(int64_t)t * OS + i];
            s += kb[t] * diff / tau[t];
        }
        S[i] = s;
    }
}

void fo_sum_restricted(const double *old, int64_t OS, int nold, const double *kb, const double *tau,
                       double thr, int bs, int64_t nodes, double *S)
{
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nodes; i++) {
        double s = 0.0;
        if (bs == 0) {
            for (int t = nold - 2; t >= 0; t--) {          /* :4110-4131 */
                double kv = kb[t];
                double diff = old[(int64_t)(t + 1) * OS + i] - old[(int64_t)t * OS + i];
                if (fabs(kv) < thr) break;
                s += kv * diff / tau[t];
            }
        } else {
            for (int t = nold - 2; t >= 0; t -= bs) {       /* :1422-1455, one chunk per pass */
                int br = 0;
                for (int q = 0; q < bs; q++) {
                    double kv = t - q >= 0 ? kb[t - q] : 0.0;
                    if (t - q >= 0) {
                        double diff = old[(int64_t)(t - q + 1) * OS + i] - old[(int64_t)(t - q) * OS + i];
                        s += kv * diff / tau[t - q];
                    }
                    if (fabs(kv) < thr) br++;
                }
                if (br == bs) break;
            }
        }
        S[i] = s;
    }
}

void fo_sum_series(const double *prev, const double *cur, int64_t nodes, double *H, int P, const double *row2,
                   double gt, double gtj, double alpha, double tau_t, double *S)
{
    double *pw = (double *)malloc((size_t)P * sizeof(double));
    double *v = (double *)malloc((size_t)P * sizeof(double));
    double mult = gt, vv = pow(gtj, -alpha);
    for (int j = 0; j < P; j++) {
        pw[j] = isfinite(mult) ? mult : 0.0;                /* mult = g^(j+1), :4143-4148 */
        v[j] = isfinite(vv) ? vv : 0.0;                     /* v1, :1165-1178 */
        mult *= gt;
        double ii = (double)(j + 1);
        vv *= -(-alpha - ii + 1.0) / (ii * gtj);
    }
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < nodes; i++) {
        double d = cur[i] - prev[i];
        if (!isfinite(d)) d = 0.0;
        double sum = 0.0;
        for (int j = 0; j < P; j++) {
            double r = isfinite(row2[j]) ? row2[j] : 0.0;
            H[i * P + j] += pw[j] * r * d;
            sum += v[j] * H[i * P + j];
        }
        S[i] = sum / tau_t;
    }
    free(pw);
    free(v);
}

/* ------------------------------------------------------------------ Thomas */

static void thomas_core(int N, const double *A, const double *B, const double *R,
                        const double *Om, int ltype, double g0, int rtype, double gN,
                        double dLN, double *U, double *Al, double *Bt)
{
    Al[1] = ltype ? 1.0 : 0.0;                                /* al1 :4004-4025 */
    for (int i = 1; i < N; i++) Al[i + 1] = B[i] / (R[i] - A[i] * Al[i]);
    Bt[1] = g0;                                               /* bt1 :4587-4589 */
    for (int i = 1; i < N; i++) Bt[i + 1] = (Al[i + 1] / B[i]) * (A[i] * Bt[i] - Om[i]);
    if (rtype == 0) {
        U[N] = gN;                                            /* U1 :4685-4686 */
    } else {                                                  /* U1 :4689-4718 */
        if (fabs(Bt[N]) > 1e-15) {
            if (fabs(1.0 - Al[N]) > 1e-15) U[N] = (Bt[N] + gN * dLN) / (1.0 - Al[N]);
            else U[N] = U[N - 1];
        } else {
            if (fabs(1.0 - Al[N]) > 1e-15) U[N] = 0.0;
            else U[N] = U[N - 1];
        }
    }
    for (int i = N - 1; i >= 0; i--) U[i] = Al[i + 1] * U[i + 1] + Bt[i + 1];   /* :4723 */
}

void fo_thomas_line(int N, const double *A, const double *B, const double *R, const double *Om,
                    int ltype, double g0, int rtype, double gN, double dLN, double *U)
{
    double *Al = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    double *Bt = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    thomas_core(N, A, B, R, Om, ltype, g0, rtype, gN, dLN, U, Al, Bt);
    free(Al);
    free(Bt);
}

void fo_line_coefs(int N, const double *k, const double *iw, const double *dL,
                   double *A, double *B, double *Rlap)
{
    for (int i = 1; i < N; i++) {             /* A_ / B / R :3095-3122, Dg = kb = 1 */
        A[i] = k[i - 1] * iw[i] / (dL[i] * dL[i - 1]);
        B[i] = k[i] * iw[i] / (dL[i] * dL[i]);
        Rlap[i] = iw[i] * ((k[i] / (dL[i] * dL[i])) + (k[i - 1] / (dL[i] * dL[i - 1])));
    }
}

/* ------------------------------------------------------------- line steps */

int fo_line_step(int N, double *U, double *hist, int64_t P, int n,
                 const double *kb, const double *tau, double Da, double kkk0,
                 const double *A, const double *B, const double *Rlap, const double *src,
                 int ltype, double g0, int rtype, double gN, double dLN, double *S_out)
{
    double tn = tau[n];
    double lam = Da * (kkk0 / tn);            /* Om1 :4191 */
    double lamR = Da * kkk0 / tn;             /* R :3120 */
    double *S = (double *)calloc((size_t)N + 1, sizeof(double));
    double *Om = (double *)calloc((size_t)N + 1, sizeof(double));
    double *R = (double *)calloc((size_t)N + 1, sizeof(double));
    double *Uold = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double *Al = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    double *Bt = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    memcpy(Uold, U, sizeof(double) * (size_t)(N + 1));
    if (n > 0) fo_l1_sum(hist, P, n, kb, tau, 1, N, S);
    for (int i = 1; i < N; i++) {
        Om[i] = -(lam * U[i]) + (src ? src[i] : 0.0);
        Om[i] += Da * S[i];                    /* Om1 :4267 (mult = 1) */
        R[i] = Rlap[i] + lamR;
    }
    thomas_core(N, A, B, R, Om, ltype, g0, rtype, gN, dLN, U, Al, Bt);
    double *row = hist + (int64_t)n * P;
    for (int64_t i = 0; i < P; i++) row[i] = (i <= N) ? U[i] - Uold[i] : 0.0;
    if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)(N + 1));
    free(S); free(Om); free(R); free(Uold); free(Al); free(Bt);
    return 0;
}

int fo_line_run(int N, double *U, double *hist, int64_t P, int steps, double tau, double alpha,
                double Da, const double *A, const double *B, const double *Rlap,
                int ltype, double g0, int rtype, double gN, double dLN)
{
    double *time = (double *)malloc(sizeof(double) * (size_t)(steps + 2));
    double *taus = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
    double *kb = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
    time[0] = 0.0;                            /* Time.push_back(0) :3571 */
    for (int n = 0; n <= steps; n++) { taus[n] = tau; time[n + 1] = time[n] + tau; }
    for (int n = 0; n < steps; n++) {
        double kkk0;
        fo_l1_weights(alpha, time, n, kb, &kkk0);
        fo_line_step(N, U, hist, P, n, kb, taus, Da, kkk0, A, B, Rlap, NULL,
                     ltype, g0, rtype, gN, dLN, NULL);
    }
    free(time); free(taus); free(kb);
    return 0;
}

int fo_line_run_general(int N, double *U, double *hist, int64_t P, int steps, const double *w, double theta,
                        const double *A, const double *B, const double *Rlap, const double *src, int src_rows,
                        int ltype, double g0, int rtype, double gN, double dLN)
{
    double *S = (double *)calloc((size_t)N + 1, sizeof(double));
    double *Om = (double *)calloc((size_t)N + 1, sizeof(double));
    double *R = (double *)calloc((size_t)N + 1, sizeof(double));
    double *Uold = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double *Al = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    double *Bt = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    double *wl = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
    for (int n = 0; n < steps; n++) {
        memcpy(Uold, U, sizeof(double) * (size_t)(N + 1));
        /* history: S[i] = sum_{t<n} w[n-t] D_t[i] (lag weights, eq_DF of fr_do.cpp :737-771), each
         * node from t = n-1 down, rows read contiguously per block of nodes */
        for (int t = 0; t < n; t++) wl[t] = w[n - t];
        const int64_t nblk = ((int64_t)N - 1 + FO_NODE_BLOCK - 1) / FO_NODE_BLOCK;
#pragma omp parallel for schedule(static)
        for (int64_t b = 0; b < nblk; b++) {
            const int64_t a = 1 + b * FO_NODE_BLOCK, e = a + FO_NODE_BLOCK < N ? a + FO_NODE_BLOCK : N;
            for (int64_t i = a; i < e; i++) S[i] = 0.0;
            for (int t = n - 1; t >= 0; t--) {
                const double *row = hist + (int64_t)t * P;
                const double c = wl[t];
                for (int64_t i = a; i < e; i++) S[i] += c * row[i];
            }
        }
        const double *sr = src ? src + (int64_t)(n < src_rows ? n : src_rows - 1) * (N + 1) : NULL;
        for (int i = 1; i < N; i++) {
            /* explicit part of the space operator (rp of eq_Ff :656-665) */
            double ex = theta != 0.0 ? -(theta * ((A[i] * Uold[i - 1] - Rlap[i] * Uold[i]) + B[i] * Uold[i + 1])) : 0.0;
            Om[i] = ex + (-(w[0] * Uold[i]) + (sr ? sr[i] : 0.0));
            Om[i] += S[i];
            R[i] = Rlap[i] + w[0];
        }
        thomas_core(N, A, B, R, Om, ltype, g0, rtype, gN, dLN, U, Al, Bt);
        double *row = hist + (int64_t)n * P;
        for (int64_t i = 0; i < P; i++) row[i] = (i <= N) ? U[i] - Uold[i] : 0.0;
    }
    free(S); free(Om); free(R); free(Uold); free(Al); free(Bt); free(wl);
    return 0;
}

/* ---------------------------------------------------------------- 3D LOD */

int fo_lod_step_dirichlet(int sN, int M, int K, double *U, double *hist, int n,
                          const double *kb, const double *tau, double Da, double kkk0,
                          const double *coefA, const double *coefB, const double *coefRlap,
                          const double *rp, const double *bc, double *S_out)
{
    const int kinds[3] = {0, 0, 0};
    const double dLN[3] = {0.0, 0.0, 0.0};
    return fo_lod_step(sN, M, K, U, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, kinds, kinds, dLN,
                       S_out);
}

/* fo_lod_step's body; S_in (may be NULL) replaces the L1 history sum with given sums on the
 * K-pass nodes (the sum_alg 2 series, formed by the caller). */
static int lod_step_impl(int sN, int M, int K, double *U, double *hist, int n,
                         const double *kb, const double *tau, double Da, double kkk0,
                         const double *coefA, const double *coefB, const double *coefRlap,
                         const double *rp, const double *bc, const int *lkind, const int *rkind, const double *dLN,
                         const double *S_in, double *S_out)
{
    const double lam = Da * (kkk0 / tau[n]);      /* Om1 :4191 */
    const double lamR = Da * kkk0 / tau[n];       /* R :3120 */
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    const int64_t G = sz * (K + 2);
    int L = sN; if (M > L) L = M; if (K > L) L = K;
    double *Uold = (double *)malloc(sizeof(double) * (size_t)G);
    double *S = (double *)calloc((size_t)G, sizeof(double));
    memcpy(Uold, U, sizeof(double) * (size_t)G);
    /* history sum on the K-pass nodes (time_summing is evaluated for k = 1..K): every node's sum
     * runs from t = n-1 down to 0 in the reference's order, s = 0 then s += kb[t]*D/tau[t]; the
     * loops visit t outside the nodes so that each row is read contiguously (same per-node order
     * and rounding), k-planes in parallel */
    if (S_in) {
        for (int k = 1; k <= K; k++)
            for (int j = 1; j < M; j++)
                for (int i = 1; i < sN; i++) {
                    const int64_t id = i * sx + j * sy + k * sz;
                    S[id] = S_in[id];
                }
    } else if (n > 0) {
#pragma omp parallel for schedule(static)
        for (int k = 1; k <= K; k++)
            for (int t = n - 1; t >= 0; t--) {
                const double *h = hist + (int64_t)t * G;
                const double c = kb[t], tt = tau[t];
                for (int j = 1; j < M; j++)
                    for (int i = 1; i < sN; i++) {
                        const int64_t id = i * sx + j * sy + k * sz;
                        S[id] += c * h[id] / tt;
                    }
            }
    }
    /* passes in the order of calc_step: K (c=2), _M (c=1), sN (c=0) */
    for (int pass = 2; pass >= 0; pass--) {
        int Nl = pass == 2 ? K : (pass == 1 ? M : sN);
        int64_t st = pass == 2 ? sz : (pass == 1 ? sy : sx);
        const double *cA = coefA + (int64_t)pass * G, *cB = coefB + (int64_t)pass * G;
        const double *cR = coefRlap + (int64_t)pass * G;
        int na = pass == 2 ? sN : (pass == 1 ? sN : M);     /* first line index range */
        int nb = pass == 2 ? M : K;                          /* second line index range */
        /* the lines of a pass are independent: in parallel, each thread with its own line arrays */
#pragma omp parallel
        {
        double *la = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lb = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lr = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lo = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lu = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *Al = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *Bt = (double *)malloc(sizeof(double) * (size_t)(L + 2));
#pragma omp for schedule(static) collapse(2)
        for (int a = 1; a < na; a++)
            for (int b = 1; b < nb; b++) {
                int64_t base;
                if (pass == 2) base = a * sx + b * sy;               /* line (i, j) */
                else if (pass == 1) base = a * sx + b * sz;          /* line (i, k) */
                else base = a * sy + b * sz;                         /* line (j, k) */
                for (int p = 0; p <= Nl + 1; p++) lu[p] = U[base + p * st];
                for (int p = 1; p < Nl; p++) {
                    int64_t id = base + p * st;
                    la[p] = cA[id]; lb[p] = cB[id]; lr[p] = cR[id] + lamR;
                    lo[p] = -(lam * lu[p]) + ((pass == 2 && rp) ? rp[id] : 0.0);
                    if (pass == 2) lo[p] += Da * S[id];
                }
                thomas_core(Nl, la, lb, lr, lo, lkind[pass], bc[base], rkind[pass], bc[base + Nl * st], dLN[pass],
                            lu, Al, Bt);
                lu[Nl + 1] = lu[Nl];                                 /* U1 :4792 */
                for (int p = 0; p <= Nl + 1; p++) U[base + p * st] = lu[p];
            }
        free(la); free(lb); free(lr); free(lo); free(lu); free(Al); free(Bt);
        }
    }
    double *row = hist + (int64_t)n * G;
    for (int64_t q = 0; q < G; q++) row[q] = U[q] - Uold[q];
    if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)G);
    free(Uold); free(S);
    return 0;
}

int fo_lod_step(int sN, int M, int K, double *U, double *hist, int n,
                const double *kb, const double *tau, double Da, double kkk0,
                const double *coefA, const double *coefB, const double *coefRlap,
                const double *rp, const double *bc, const int *lkind, const int *rkind, const double *dLN,
                double *S_out)
{
    return lod_step_impl(sN, M, K, U, hist, n, kb, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, lkind, rkind,
                         dLN, NULL, S_out);
}

int fo_lod_step_dirichlet_sum(int sN, int M, int K, double *U, double *hist, int n, const double *tau, double Da,
                              double kkk0, const double *coefA, const double *coefB, const double *coefRlap,
                              const double *rp, const double *bc, const double *S_in)
{
    const int kinds[3] = {0, 0, 0};
    const double dLN[3] = {0.0, 0.0, 0.0};
    return lod_step_impl(sN, M, K, U, hist, n, NULL, tau, Da, kkk0, coefA, coefB, coefRlap, rp, bc, kinds, kinds,
                         dLN, S_in, NULL);
}

/* ------------------------------------------------- Richards (solution-dependent coefficients) */

/* The reference's closures of its Richards problem (analytic_test 0, cv_form 4): water content
 * wetness :2493-2522, its inverse derivative inv_dw_dh :2523-2566 and the conductivity KK
 * :2625-2655 (k_form 1 van Genuchten-Mualem, 2 Averianov), as functions of the suction P
 * (metres). The expressions keep the reference's operation order, so the values are bitwise
 * the reference's. */
static double rich_wetness(double P)
{
    const double n = 1.25, s0 = 0.0736, s1 = 0.55, a = 0.066;
    double Ch;
    P *= 100.0;
    if (P <= 0.0)
        Ch = s1;
    else
        Ch = s0 + ((s1 - s0) / pow(1 + pow(a * P, n), (1 - 1 / n)));
    return Ch;
}

static double rich_inv_dw_dh(double P)
{
    const double n = 1.25, s0 = 0.0736, s1 = 0.55, a = 0.066;
    double Ch = 0.0;
    if (P <= 0.0) {
        Ch = 0.0;
    } else {
        double hn = pow(100.0, n), h2n = pow(100.0, 2.0 * n);
        Ch = ((((1 - n) * hn * s0 + (n - 1) * hn * s1) * pow(a * P, n) * pow(1 + hn * pow(a * P, n), (1 / n))) /
              (h2n * P * pow(a * P, 2 * n) + 2 * hn * P * pow(a * P, n) + P));
    }
    if (Ch != 0.0) return 1.0 / Ch;
    return 1e20;
}

static double rich_KK(double P, int kform, double ksat)
{
    const double n = 1.25, s0 = 0.0736, s1 = 0.55;
    double Kr = 1.0;
    if (kform == 1)
        Kr = pow(((rich_wetness(P) - s0) / (s1 - s0)), 0.5) *
             pow(1.0 - pow(1.0 - pow(((rich_wetness(P) - s0) / (s1 - s0)), (1.0 / (1.0 - 1.0 / n))), (1.0 - 1.0 / n)),
                 2.0);
    if (kform == 2) Kr = pow(((rich_wetness(P) - s0) / (s1 - s0)), 3.5);
    return Kr * ksat;
}

void fo_richards_closures(int n, const double *P, int kform, double ksat, double *w, double *iw, double *kk)
{
    for (int i = 0; i < n; i++) {
        if (w) w[i] = rich_wetness(P[i]);
        if (iw) iw[i] = rich_inv_dw_dh(P[i]);
        if (kk) kk[i] = rich_KK(P[i], kform, ksat);
    }
}

/* One LOD step of the reference's Richards problem in its 3D mode (calc_step :5144-5779 with
 * analytic_test 0, no irrigation, bottom_cond 0): the passes of fo_lod_step, with every line's
 * coefficients A_/B/R (:3095-3142) formed from the line's current values before its solve. The
 * suction of a node follows the reference's mode-3 wetness/inv_dw_dh (:2504-2512, :2546-2554):
 * P = -(U - i sZ[p]) with i the node's index along the sN axis and p its position along the pass.
 * Left ends: the sN pass takes the first-order surface condition (al1 :4004-4012, bc0 :4493-4500)
 * with Uc = dL[0] E / KK(1) (:3036-3070, no irrigation); the other passes zero flux (Al[1] = 1,
 * Bt[1] = 0). Right ends: the flux closure of U1 with bcN = 0. rp: the K-pass source grid. */
/* time_summing of the K-pass nodes (:4086-4164) in the reference's order: s = 0, then
 * s += kb[t] D_t / tau[t] for t = n-1 .. 0 (rows read contiguously, k-planes in parallel) */
static void lod_history_sum(int sN, int M, int K, const double *hist, int n, const double *kb, const double *tau,
                            double *S)
{
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    const int64_t G = sz * (K + 2);
    if (n <= 0) return;
#pragma omp parallel for schedule(static)
    for (int k = 1; k <= K; k++)
        for (int t = n - 1; t >= 0; t--) {
            const double *h = hist + (int64_t)t * G;
            const double c = kb[t], tt = tau[t];
            for (int j = 1; j < M; j++)
                for (int i = 1; i < sN; i++) {
                    const int64_t id = i * sx + j * sy + k * sz;
                    S[id] += c * h[id] / tt;
                }
        }
}

int fo_lod_step_richards(int sN, int M, int K, double *U, double *hist, int n, const double *kb, const double *tau,
                         double Da, double kkk0, const double *sZ, const double *sdL, const double *dLx,
                         const double *dLy, int kform, double ksat, double E, const double *rp, double *S_out)
{
    return fo_lod_step_richards_salt(sN, M, K, U, hist, n, kb, tau, Da, kkk0, sZ, sdL, dLx, dLy, kform, ksat, E, rp,
                                     S_out, NULL, NULL, NULL, NULL, NULL, 0.0, 0.0, NULL);
}

int fo_lod_step_richards_salt(int sN, int M, int K, double *U, double *hist, int n, const double *kb,
                              const double *tau, double Da, double kkk0, const double *sZ, const double *sdL,
                              const double *dLx, const double *dLy, int kform, double ksat, double E,
                              const double *rp, double *S_out, double *C, double *histC, const double *cA,
                              const double *cB, const double *cR, double nu, double sigma, double *SC_out)
{
    const double lam = Da * (kkk0 / tau[n]);      /* Om1 :4191 */
    const double lamR = Da * kkk0 / tau[n];       /* R :3120 */
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    const int64_t G = sz * (K + 2);
    int L = sN; if (M > L) L = M; if (K > L) L = K;
    double *Uold = (double *)malloc(sizeof(double) * (size_t)G);
    double *S = (double *)calloc((size_t)G, sizeof(double));
    double *Cold = C ? (double *)malloc(sizeof(double) * (size_t)G) : NULL;
    double *SC = C ? (double *)calloc((size_t)G, sizeof(double)) : NULL;
    memcpy(Uold, U, sizeof(double) * (size_t)G);
    lod_history_sum(sN, M, K, hist, n, kb, tau, S);
    if (C) {
        memcpy(Cold, C, sizeof(double) * (size_t)G);
        lod_history_sum(sN, M, K, histC, n, kb, tau, SC);
    }
    for (int pass = 2; pass >= 0; pass--) {
        const int Nl = pass == 2 ? K : (pass == 1 ? M : sN);
        const int64_t st = pass == 2 ? sz : (pass == 1 ? sy : sx);
        const double *dL = pass == 2 ? dLy : (pass == 1 ? dLx : sdL);
        const int na = pass == 2 ? sN : (pass == 1 ? sN : M);
        const int nb = pass == 2 ? M : K;
#pragma omp parallel
        {
        double *la = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lb = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lr = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lo = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lu = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *kk = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *iw = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *Al = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *Bt = (double *)malloc(sizeof(double) * (size_t)(L + 2));
#pragma omp for schedule(static) collapse(2)
        for (int a = 1; a < na; a++)
            for (int b = 1; b < nb; b++) {
                int64_t base;
                if (pass == 2) base = a * sx + b * sy;
                else if (pass == 1) base = a * sx + b * sz;
                else base = a * sy + b * sz;
                for (int p = 0; p <= Nl + 1; p++) lu[p] = U[base + p * st];
                for (int p = 0; p <= Nl; p++) {           /* closures at the line's nodes */
                    const int inode = pass == 0 ? p : a;
                    const double P = -(lu[p] - inode * sZ[p]);
                    kk[p] = rich_KK(P, kform, ksat);
                    iw[p] = rich_inv_dw_dh(P);
                }
                for (int p = 1; p < Nl; p++) {
                    la[p] = kk[p - 1] * iw[p] / (dL[p] * dL[p - 1]);
                    lb[p] = kk[p] * iw[p] / (dL[p] * dL[p]);
                    lr[p] = iw[p] * ((kk[p] / (dL[p] * dL[p])) + (kk[p - 1] / (dL[p] * dL[p - 1]))) + lamR;
                    const int64_t id = base + p * st;
                    lo[p] = -(lam * lu[p]) + ((pass == 2 && rp) ? rp[id] : 0.0);
                    if (C && nu != 0.0) {                  /* chemical osmosis, Om1 :4211-4223 (old C) */
                        const double d2 = dL[p] * dL[p], d1 = dL[p] * dL[p - 1];
                        const int64_t s1 = st;
                        const double f = nu * (((C[id + s1] / d2) - ((1.0 / d2) + (1.0 / d1)) * C[id]) + (C[id - s1] / d1));
                        lo[p] += f * iw[p];
                    }
                    if (pass == 2) lo[p] += Da * S[id];
                }
                int lkind = 1;
                double g0 = 0.0;
                if (pass == 0) {                           /* surface: al1 :4006-4012, bc0 :4495-4500 */
                    const double Uc = dL[0] * (E - 0.0) / kk[1];
                    if (iw[0] != 1e20) { lkind = 1; g0 = -Uc; }
                    else { lkind = 0; g0 = -Uc * kk[1] / dL[0]; }
                }
                thomas_core(Nl, la, lb, lr, lo, lkind, g0, 1, 0.0, dL[Nl - 1], lu, Al, Bt);
                lu[Nl + 1] = lu[Nl];                                 /* U1 :4792 */
                for (int p = 0; p <= Nl + 1; p++) U[base + p * st] = lu[p];
                if (!C) continue;
                /* equation 1 on the same line (U1(1) after U1(0), :5270-5278): the coefficients of
                 * A_/B/R (:3099-3136), Om1's local and coupling terms (:4175-4229) with the new H
                 * and its KK, the old C; Dirichlet Cu() = 0 at the surface of the sN pass (al1
                 * :4014-4017, no irrigation), zero flux elsewhere (Al[1] = 1, Bt[1] = 0), the flux
                 * closure with bcN = 0 at the far end (bottom_cond 0) */
                for (int p = 0; p <= Nl; p++) {                      /* KK of the new H */
                    const int inode = pass == 0 ? p : a;
                    kk[p] = rich_KK(-(lu[p] - inode * sZ[p]), kform, ksat);
                }
                double *lc = iw;                                       /* reuse: the C line */
                for (int p = 0; p <= Nl + 1; p++) lc[p] = C[base + p * st];
                for (int p = 1; p < Nl; p++) {
                    const int64_t id = base + p * st;
                    la[p] = cA[(int64_t)pass * G + id];
                    lb[p] = cB[(int64_t)pass * G + id];
                    lr[p] = cR[(int64_t)pass * G + id] + lamR;
                    const double d2 = dL[p] * dL[p], d1 = dL[p] * dL[p - 1];
                    const double fh = (1.0 / sigma) * ((((kk[p] * lc[p]) * lu[p + 1]) / d2) -
                                                       (((kk[p] * lc[p]) / d2) + ((kk[p - 1] * lc[p - 1]) / d1)) * lu[p] +
                                                       (((kk[p - 1] * lc[p - 1]) * lu[p - 1]) / d1));
                    const double fc = (nu / sigma) * (((lc[p] * lc[p + 1]) / d2) -
                                                      ((lc[p] / d2) + (lc[p - 1] / d1)) * lc[p] +
                                                      ((lc[p - 1] * lc[p - 1]) / d1));
                    double om = -(lam * lc[p]) + 0.0;                  /* Rp = 0 for equation 1 */
                    om -= fh;
                    if (nu != 0.0) om += fc;
                    if (pass == 2) om += Da * SC[id];
                    lo[p] = om;
                }
                thomas_core(Nl, la, lb, lr, lo, pass == 0 ? 0 : 1, 0.0, 1, 0.0, dL[Nl - 1], lc, Al, Bt);
                lc[Nl + 1] = lu[Nl];                                 /* U1 :4792 copies H's U[N] */
                for (int p = 0; p <= Nl + 1; p++) C[base + p * st] = lc[p];
            }
        free(la); free(lb); free(lr); free(lo); free(lu); free(kk); free(iw); free(Al); free(Bt);
        }
    }
    double *row = hist + (int64_t)n * G;
    for (int64_t q = 0; q < G; q++) row[q] = U[q] - Uold[q];
    if (C) {
        double *rc = histC + (int64_t)n * G;
        for (int64_t q = 0; q < G; q++) rc[q] = C[q] - Cold[q];
    }
    if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)G);
    if (SC_out && SC) memcpy(SC_out, SC, sizeof(double) * (size_t)G);
    free(Uold); free(S); free(Cold); free(SC);
    return 0;
}

/* A 1D line of the Richards problem with the history (the reference's column form; mode-1
 * closures: the suction of node i is P = -(U[i] - Z[i]), wetness / inv_dw_dh :2499-2500,
 * :2529): per step the L1 history sum, the coefficients A_/B/R from the current values, the
 * surface condition of al1 / bc0 (first-order flux -Uc with Uc = dL[0] E / KK(1), or Dirichlet
 * -Uc KK(1)/dL[0] where node 0 is saturated) and the right end of U1 (rtype 0 Dirichlet gN,
 * 1 flux closure). E: the evaporation rate of every step (row min(n, erows-1)); src: optional
 * source rows. hist receives the increments (rows of P). */
int fo_line_run_richards(int N, double *U, double *hist, int64_t P, int steps, double tau, double alpha, double Da,
                         const double *Z, const double *dL, int kform, double ksat, const double *E, int erows,
                         const double *src, int src_rows, int rtype, double gN, double dLN)
{
    double *time = (double *)malloc(sizeof(double) * (size_t)(steps + 2));
    double *taus = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
    double *kb = (double *)malloc(sizeof(double) * (size_t)(steps + 1));
    double *S = (double *)calloc((size_t)N + 1, sizeof(double));
    double *Om = (double *)calloc((size_t)N + 1, sizeof(double));
    double *A = (double *)calloc((size_t)N + 1, sizeof(double));
    double *B = (double *)calloc((size_t)N + 1, sizeof(double));
    double *R = (double *)calloc((size_t)N + 1, sizeof(double));
    double *kk = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double *iw = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double *Uold = (double *)malloc(sizeof(double) * (size_t)(N + 1));
    double *Al = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    double *Bt = (double *)malloc(sizeof(double) * (size_t)(N + 2));
    time[0] = 0.0;
    for (int n = 0; n <= steps; n++) { taus[n] = tau; time[n + 1] = time[n] + tau; }
    for (int n = 0; n < steps; n++) {
        double kkk0;
        fo_l1_weights(alpha, time, n, kb, &kkk0);
        const double lam = Da * (kkk0 / tau), lamR = Da * kkk0 / tau;
        memcpy(Uold, U, sizeof(double) * (size_t)(N + 1));
        if (n > 0) fo_l1_sum(hist, P, n, kb, taus, 1, N, S);
        for (int i = 0; i <= N; i++) {
            const double Pi = -(U[i] - Z[i]);
            kk[i] = rich_KK(Pi, kform, ksat);
            iw[i] = rich_inv_dw_dh(Pi);
        }
        const double *sr = src ? src + (int64_t)(n < src_rows ? n : src_rows - 1) * (N + 1) : NULL;
        for (int i = 1; i < N; i++) {
            A[i] = kk[i - 1] * iw[i] / (dL[i] * dL[i - 1]);
            B[i] = kk[i] * iw[i] / (dL[i] * dL[i]);
            R[i] = iw[i] * ((kk[i] / (dL[i] * dL[i])) + (kk[i - 1] / (dL[i] * dL[i - 1]))) + lamR;
            Om[i] = -(lam * U[i]) + (sr ? sr[i] : 0.0);
            Om[i] += Da * S[i];
        }
        const double En = E[n < erows ? n : erows - 1];
        const double Uc = dL[0] * (En - 0.0) / kk[1];
        int lkind = 1;
        double g0 = -Uc;
        if (iw[0] == 1e20) { lkind = 0; g0 = -Uc * kk[1] / dL[0]; }
        thomas_core(N, A, B, R, Om, lkind, g0, rtype, gN, dLN, U, Al, Bt);
        double *row = hist + (int64_t)n * P;
        for (int64_t i = 0; i < P; i++) row[i] = (i <= N) ? U[i] - Uold[i] : 0.0;
    }
    free(time); free(taus); free(kb); free(S); free(Om); free(A); free(B); free(R); free(kk); free(iw);
    free(Uold); free(Al); free(Bt);
    return 0;
}

/* ------------------------------------------ implicit space-fractional operator (impl 2) */

/* vmul_T, fpde_hpc_1d.cpp:6662-6686 (toeplitz_mult_alg 0; the C/T branch :6704-6746 is not
 * restated). The interior rows are the reference's s->rb..s->re-1 = 1..n-1 of a line. */
void fo_sf_matvec(int n, const double *mat, const double *mc, const double *Tm, const double *iw,
                  const double *rs, int space_der, const double *x, double *r, double *bt)
{
    const double *m0 = mat, *m1 = mat + (n + 1), *m2 = mat + 2 * (n + 1);
    const double *c0 = mc, *c1 = mc + (n + 1), *c2 = mc + 2 * (n + 1);
    for (int i = 1; i < n; i++) r[i] = m0[i] * x[i - 1] + m1[i] * x[i] + m2[i] * x[i + 1];   /* :6662-6663 */
    r[0] = m1[0] * x[0] + m2[0] * x[1];
    r[n] = m0[n] * x[n - 1] + m1[n] * x[n];
    for (int j = 1; j < n; j++) bt[j] = c0[j] * x[j - 1] + c1[j] * x[j] + c2[j] * x[j + 1];  /* :6668-6669 */
    for (int i = 1; i < n; i++) {                                                              /* :6674-6686 */
        double v = 0.0;
        for (int j = 1; j < i; j++) v += bt[j] * Tm[i - j + 1];
        if (space_der == 1)
            for (int j = i + 1; j < n; j++) v -= bt[j] * Tm[j - i + 1];
        if (rs) v /= rs[i];
        r[i] += v * (iw ? iw[i] : 1.0);
    }
}

static double sf_dot(int64_t m, const double *a, const double *b)
{
    double s = 0.0;
    for (int64_t i = 0; i < m; i++) s += a[i] * b[i];
    return s;
}

/* The product a solve runs on: apply(op, x, r) sets r = A x. */
typedef void (*sf_apply_fn)(const void *op, const double *x, double *r);

/* solve_mln<1>, fpde_hpc_1d.cpp:812-1157, for n = 1: rn(k) = 1 and qn(k) = k - 1 for every k, so
 * each iteration takes the rn == 1 branch (:868-915), recomputes the residual (:943-947) and the
 * rn == n branch (:1053-1098); q[0] is the initial residual (no random vectors for n = 1). The
 * vectors have m values (the reference's N, rb = 0, re = N). */
static int sf_bicgstab(int64_t m, sf_apply_fn apply, const void *op, const double *B, double *x, double thr,
                       int maxiter)
{
    const size_t bytes = sizeof(double) * (size_t)m;
    double *q0 = (double *)malloc(bytes), *r = (double *)malloc(bytes);
    double *g[2], *w[2];
    for (int k = 0; k < 2; k++) {
        g[k] = (double *)malloc(bytes);
        w[k] = (double *)malloc(bytes);
    }
    double *u = (double *)malloc(bytes), *Au = (double *)malloc(bytes), *zw = (double *)malloc(bytes);
    double c[2] = {0.0, 0.0}, al, ro1 = 0.0, beta, norm;
    int iter = 1;
restart:
    apply(op, x, r);                                                           /* :841-844 */
    for (int64_t i = 0; i < m; i++) r[i] = B[i] - r[i];
    memcpy(g[1], r, bytes);
    memcpy(q0, r, bytes);
    apply(op, g[1], w[1]);                                                     /* :851 */
    c[1] = sf_dot(m, q0, w[1]);
    norm = sf_dot(m, r, r);
    if (fabs(norm / m) < thr) goto done;
    for (;;) {
        al = sf_dot(m, q0, r);                                                   /* :871-877 */
        al /= c[1];
        if (c[1] != 0.0) {
            for (int64_t i = 0; i < m; i++) u[i] = r[i] - al * w[1][i];
            for (int64_t i = 0; i < m; i++) x[i] = x[i] + al * g[1][i];
            apply(op, u, Au);                                                    /* :890 */
            norm = sf_dot(m, Au, Au);
            ro1 = sf_dot(m, Au, u);
            ro1 = -ro1 / norm;
            if (norm == 0.0) goto restart;
            for (int64_t i = 0; i < m; i++) x[i] = x[i] - ro1 * u[i];
        } else {
            goto restart;
        }
        apply(op, x, r);                                                         /* :943-947 */
        for (int64_t i = 0; i < m; i++) r[i] = B[i] - r[i];
        beta = 0.0;                                                              /* :1056-1065 */
        for (int64_t i = 0; i < m; i++) beta -= q0[i] * r[i];
        beta /= c[1];
        if (c[1] == 0.0) beta = 0.0;
        for (int64_t i = 0; i < m; i++) zw[i] = r[i] + beta * w[1][i];
        for (int64_t i = 0; i < m; i++) g[0][i] = zw[i] + (beta / ro1) * g[1][i];
        apply(op, g[0], w[0]);                                                   /* :1094 */
        c[0] = sf_dot(m, q0, w[0]);
        {                                                                        /* :1104-1121 */
            double *t = g[1]; g[1] = g[0]; g[0] = t;
            t = w[1]; w[1] = w[0]; w[0] = t;
            double tc = c[1]; c[1] = c[0]; c[0] = tc;
        }
        norm = sf_dot(m, r, r);
        if (fabs(norm / m) < thr) break;
        iter++;
        if (iter == maxiter) break;
    }
done:
    free(q0); free(r); free(u); free(Au); free(zw);
    for (int k = 0; k < 2; k++) { free(g[k]); free(w[k]); }
    return iter;
}

struct sf_line_op {
    int n, space_der;
    const double *mat, *mc, *Tm, *iw, *rs;
    double *bt;
};
static void sf_line_apply(const void *op, const double *x, double *r)
{
    const struct sf_line_op *o = (const struct sf_line_op *)op;
    fo_sf_matvec(o->n, o->mat, o->mc, o->Tm, o->iw, o->rs, o->space_der, x, r, o->bt);
}

int fo_sf_solve(int n, const double *mat, const double *mc, const double *Tm, const double *iw,
                const double *rs, int space_der, const double *B, double *x, double thr, int maxiter)
{
    struct sf_line_op op = {n, space_der, mat, mc, Tm, iw, rs, (double *)malloc(sizeof(double) * (size_t)(n + 1))};
    const int it = sf_bicgstab(n + 1, sf_line_apply, &op, B, x, thr, maxiter);
    free(op.bt);
    return it;
}

int fo_lod_step_sf(int sN, int M, int K, double *U, double *hist, int n, const double *kb, const double *tau,
                   double Da, double kkk0, const double *coefA, const double *coefB, const double *coefRlap,
                   const double *mc, const double *iw, const double *Tm, int ldt, int space_der, double thr,
                   int maxiter, const double *rp, const double *bc, double *S_out, int64_t *iters,
                   const int *rkind, const double *dLN)
{
    const double lam = Da * (kkk0 / tau[n]);      /* Om1_impl :4441 */
    const double lamR = Da * kkk0 / tau[n];       /* R :3120 */
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    const int64_t G = sz * (K + 2);
    int L = sN; if (M > L) L = M; if (K > L) L = K;
    double *Uold = (double *)malloc(sizeof(double) * (size_t)G);
    double *S = (double *)calloc((size_t)G, sizeof(double));
    int64_t it_total = 0;
    memcpy(Uold, U, sizeof(double) * (size_t)G);
    if (n > 0) {                                  /* time_summing on the K-pass nodes, as fo_lod_step */
#pragma omp parallel for schedule(static)
        for (int k = 1; k <= K; k++)
            for (int t = n - 1; t >= 0; t--) {
                const double *h = hist + (int64_t)t * G;
                const double c = kb[t], tt = tau[t];
                for (int j = 1; j < M; j++)
                    for (int i = 1; i < sN; i++) {
                        const int64_t id = i * sx + j * sy + k * sz;
                        S[id] += c * h[id] / tt;
                    }
            }
    }
    for (int pass = 2; pass >= 0; pass--) {       /* K, _M, sN as calc_step */
        int Nl = pass == 2 ? K : (pass == 1 ? M : sN);
        int64_t st = pass == 2 ? sz : (pass == 1 ? sy : sx);
        const double *cA = coefA + (int64_t)pass * G, *cB = coefB + (int64_t)pass * G;
        const double *cR = coefRlap + (int64_t)pass * G;
        const double *pm = mc + (int64_t)pass * 3 * G, *piw = iw + (int64_t)pass * G;
        const double *pT = Tm + (int64_t)pass * ldt;
        int na = pass == 2 ? sN : (pass == 1 ? sN : M);
        int nb = pass == 2 ? M : K;
#pragma omp parallel reduction(+ : it_total)
        {
        double *mat = (double *)malloc(sizeof(double) * (size_t)3 * (L + 2));
        double *lmc = (double *)calloc((size_t)3 * (L + 2), sizeof(double));
        double *liw = (double *)calloc((size_t)(L + 2), sizeof(double));
        double *om = (double *)malloc(sizeof(double) * (size_t)(L + 2));
        double *lu = (double *)malloc(sizeof(double) * (size_t)(L + 2));
#pragma omp for schedule(static) collapse(2)
        for (int a = 1; a < na; a++)
            for (int b = 1; b < nb; b++) {
                int64_t base;
                if (pass == 2) base = a * sx + b * sy;
                else if (pass == 1) base = a * sx + b * sz;
                else base = a * sy + b * sz;
                const int m = Nl + 1;
                double *m0 = mat, *m1 = mat + m, *m2 = mat + 2 * m;
                for (int p = 0; p <= Nl + 1; p++) lu[p] = U[base + p * st];
                for (int p = 1; p < Nl; p++) {                                 /* implicit2_gen :4633-4638 */
                    int64_t id = base + p * st;
                    m0[p] = cA[id]; m1[p] = -(cR[id] + lamR); m2[p] = cB[id];
                    lmc[p] = pm[id]; lmc[m + p] = pm[G + id]; lmc[2 * m + p] = pm[2 * G + id];
                    liw[p] = piw[id];
                    om[p] = -(lam * lu[p]) + ((pass == 2 && rp) ? rp[id] : 0.0);   /* Om1_impl :4441 */
                    if (pass == 2) om[p] += Da * S[id];                             /* :4507-4510 */
                }
                m0[0] = 0.0; m1[0] = 1.0; m2[0] = 0.0;                             /* :4643-4648 */
                m0[Nl] = 0.0; m1[Nl] = 1.0; m2[Nl] = 0.0;
                om[0] = bc[base]; om[Nl] = bc[base + Nl * st];                     /* :4650-4651 */
                if (rkind && rkind[pass] == 1) {                                   /* bottom_cond 0 :4652-4655 */
                    om[Nl] *= dLN[pass];
                    m0[Nl] = -1.0;
                }
                it_total += fo_sf_solve(Nl, mat, lmc, pT, liw, NULL, space_der, om, lu, thr, maxiter);
                lu[Nl + 1] = lu[Nl];                                               /* U1 :4792 */
                for (int p = 0; p <= Nl + 1; p++) U[base + p * st] = lu[p];
            }
        free(mat); free(lmc); free(liw); free(om); free(lu);
        }
    }
    double *row = hist + (int64_t)n * G;
    for (int64_t q = 0; q < G; q++) row[q] = U[q] - Uold[q];
    if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)G);
    if (iters) *iters = it_total;
    free(Uold); free(S);
    return 0;
}

/* ------------------------------ fully implicit 3D space-fractional operator (implicit3d 1) */

/* vmul_T_3d, fpde_hpc_1d.cpp:6801-8722, without MPI, toeplitz_mult_alg 0 and for equation 0 (the
 * C/T branch :8501-8676 is not restated). The vector has V = G + 1 values, G = (sN+2)(M+2)(K+2)
 * nodes with i fastest (idx :1649). mat: 7 planes of V (Mat_3d[0..6]: K-, K+ neighbours in 0 and 2,
 * the diagonal in 1, _M-, _M+ in 3 and 4, sN-, sN+ in 5 and 6); mc: 9 planes of V (Mcoefs_3d[c][d]
 * at plane 3c+d, axis c = 0 sN, 1 _M, 2 K); Tm[c]: the Toeplitz row of axis c; iw: 3 planes of V
 * (inv_dw_dh of the axis-c line through the node) or NULL for 1; rs: V values or NULL; bt: V
 * scratch. */
void fo_sf3d_matvec(int sN, int M, int K, const double *mat, const double *mc, const double *const *Tm,
                    const double *iw, const double *rs, int space_der, const double *x, double *r, double *bt)
{
    const int64_t sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2), V = sz * (K + 2) + 1;
    const double *M0 = mat, *M1 = mat + V, *M2 = mat + 2 * V, *M3 = mat + 3 * V, *M4 = mat + 4 * V;
    const double *M5 = mat + 5 * V, *M6 = mat + 6 * V;
    /* every output and every Bt value is one independent sequence of operations: the loops run
     * on all threads without changing a bit */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < V; i++) {                                              /* :6857-6877 */
        r[i] = M1[i] * x[i];
        if (sN > 2) {
            if (i - 1 >= 0) r[i] += M5[i] * x[i - 1];
            if (i + 1 < V) r[i] += M6[i] * x[i + 1];
        }
        if (M > 2) {
            if (i - sy >= 0) r[i] += M3[i] * x[i - sy];
            if (i + sy < V) r[i] += M4[i] * x[i + sy];
        }
        if (K > 2) {
            if (i - sz >= 0) r[i] += M0[i] * x[i - sz];
            if (i + sz < V) r[i] += M2[i] * x[i + sz];
        }
    }
    /* the axes in the reference's order: K (:7248-7574), _M (:7665-7995), sN (:8085-8411) */
    for (int a = 0; a < 3; a++) {
        const int c = 2 - a;
        const int n = c == 2 ? K : (c == 1 ? M : sN);
        const int64_t st = c == 2 ? sz : (c == 1 ? sy : 1);
        if (n <= 2) continue;
        const double *c0 = mc + (3 * c) * V, *c1 = mc + (3 * c + 1) * V, *c2 = mc + (3 * c + 2) * V;
        const double *T = Tm[c];
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < V; i++) {
            bt[i] = c1[i] * x[i];
            if (i - st >= 0) bt[i] += c0[i] * x[i - st];
            if (i + st < V) bt[i] += c2[i] * x[i + st];
        }
        /* lines: the other two coordinates over 1..len-1 */
        const int na = c == 0 ? M : sN, nb = c == 2 ? M : K;
        const int64_t sa = c == 0 ? sy : 1, sb = c == 2 ? sy : sz;
#pragma omp parallel for schedule(static) collapse(2)
        for (int la = 1; la < na; la++)
            for (int lb = 1; lb < nb; lb++) {
                const int64_t base = la * sa + lb * sb;
                for (int p = 1; p < n; p++) {
                    double v = 0.0;
                    for (int q = 1; q < p; q++) v += bt[base + q * st] * T[p - q + 1];
                    if (space_der == 1)
                        for (int q = p + 1; q < n; q++) v -= bt[base + q * st] * T[q - p + 1];
                    const int64_t id = base + p * st;
                    if (rs) v /= rs[id];
                    r[id] += v * (iw ? iw[c * V + id] : 1.0);
                }
            }
    }
}

struct sf3d_op {
    int sN, M, K, space_der;
    const double *mat, *mc, *const *Tm, *iw, *rs;
    double *bt;
};
static void sf3d_apply(const void *op, const double *x, double *r)
{
    const struct sf3d_op *o = (const struct sf3d_op *)op;
    fo_sf3d_matvec(o->sN, o->M, o->K, o->mat, o->mc, o->Tm, o->iw, o->rs, o->space_der, x, r, o->bt);
}

/* solve_mln<1> with vmul_T_3d over the V values (calc_step :5705). */
int fo_sf3d_solve(int sN, int M, int K, const double *mat, const double *mc, const double *const *Tm,
                  const double *iw, const double *rs, int space_der, const double *B, double *x, double thr,
                  int maxiter)
{
    const int64_t V = (int64_t)(sN + 2) * (M + 2) * (K + 2) + 1;
    struct sf3d_op op = {sN, M, K, space_der, mat, mc, Tm, iw, rs, (double *)malloc(sizeof(double) * (size_t)V)};
    const int it = sf_bicgstab(V, sf3d_apply, &op, B, x, thr, maxiter);
    free(op.bt);
    return it;
}

/* One step of the fully implicit scheme (mode 3, implicit3d 1, impl 2; calc_step :5160-5716):
 * Mat_3d and Om are zeroed (:5160-5178) and every line of the K, _M and sN passes, in that order,
 * adds its implicit2_gen system (:4630-4663): interior rows (A_, -R, B) with R's time term
 * Da kkk0/tau only in the K pass (:3117-3123), right-hand side -lam U + Rp + Da S in the K pass and
 * Rp = 0 in the others (Om1_impl :4434-4445, Rp :2730-2733, :4493-4498), identity rows at both line
 * ends with bc0 / bcN. Mcoefs_3d[c] is the operand grid mc of pass c at its line nodes. Then one
 * solve over the V = G + 1 values from the grid (U[G], past the grid, is *u_end) and the
 * history row. mat_out (7 x V) / om_out (V) / S_out (G) / iters may be NULL. */
int fo_lod_step_sf3d(int sN, int M, int K, double *U, double *u_end, double *hist, int n, const double *kb,
                     const double *tau, double Da, double kkk0, const double *coefA, const double *coefB,
                     const double *coefRlap, const double *mc, const double *iw, const double *Tm, int ldt,
                     int space_der, double thr, int maxiter, const double *rp, const double *bc, double *mat_out,
                     double *om_out, double *S_out, int64_t *iters, const int *rkind, const double *dLN)
{
    const double lam = Da * (kkk0 / tau[n]);
    const double lamR = Da * kkk0 / tau[n];
    const int64_t sx = 1, sy = sN + 2, sz = (int64_t)(sN + 2) * (M + 2);
    const int64_t G = sz * (K + 2), V = G + 1;
    double *Uold = (double *)malloc(sizeof(double) * (size_t)G);
    double *S = (double *)calloc((size_t)G, sizeof(double));
    double *mat = (double *)calloc((size_t)(7 * V), sizeof(double));
    double *mc3 = (double *)calloc((size_t)(9 * V), sizeof(double));
    double *iw3 = (double *)calloc((size_t)(3 * V), sizeof(double));
    double *Om = (double *)calloc((size_t)V, sizeof(double));
    double *x = (double *)malloc(sizeof(double) * (size_t)V);
    memcpy(Uold, U, sizeof(double) * (size_t)G);
    if (n > 0) {
        for (int k = 1; k <= K; k++)
            for (int t = n - 1; t >= 0; t--) {
                const double *h = hist + (int64_t)t * G;
                const double c = kb[t], tt = tau[t];
                for (int j = 1; j < M; j++)
                    for (int i = 1; i < sN; i++) {
                        const int64_t id = i * sx + j * sy + k * sz;
                        S[id] += c * h[id] / tt;
                    }
            }
    }
    for (int pass = 2; pass >= 0; pass--) {
        const int Nl = pass == 2 ? K : (pass == 1 ? M : sN);
        const int64_t st = pass == 2 ? sz : (pass == 1 ? sy : sx);
        const int lo = pass == 2 ? 0 : (pass == 1 ? 3 : 5), hi = pass == 2 ? 2 : (pass == 1 ? 4 : 6);
        const double *cA = coefA + (int64_t)pass * G, *cB = coefB + (int64_t)pass * G;
        const double *cR = coefRlap + (int64_t)pass * G;
        const double *pm = mc + (int64_t)pass * 3 * G, *piw = iw + (int64_t)pass * G;
        const int na = pass == 2 ? sN : (pass == 1 ? sN : M);
        const int nb = pass == 2 ? M : K;
        const double tR = pass == 2 ? lamR : 0.0;
        for (int a = 1; a < na; a++)
            for (int b = 1; b < nb; b++) {
                int64_t base;
                if (pass == 2) base = a * sx + b * sy;
                else if (pass == 1) base = a * sx + b * sz;
                else base = a * sy + b * sz;
                for (int p = 0; p <= Nl; p++) {
                    const int64_t id = base + p * st;
                    double ml, md, mh, om;
                    if (p == 0 || p == Nl) {
                        ml = 0.0; md = 1.0; mh = 0.0;
                        om = bc[id];
                        if (p == Nl && rkind && rkind[pass] == 1) {                 /* bottom_cond 0 :4652-4655 */
                            om *= dLN[pass];
                            ml = -1.0;
                        }
                    } else {
                        ml = cA[id]; md = -(cR[id] + tR); mh = cB[id];
                        if (pass == 2) {
                            om = -(lam * U[id]) + (rp ? rp[id] : 0.0);
                            om += Da * S[id];
                        } else {
                            om = 0.0;
                        }
                        for (int d = 0; d < 3; d++) mc3[(3 * pass + d) * V + id] += pm[d * G + id];
                        iw3[pass * V + id] = piw[id];
                    }
                    mat[lo * V + id] += ml;
                    mat[V + id] += md;
                    mat[hi * V + id] += mh;
                    Om[id] += om;
                }
            }
    }
    const double *T3[3] = {Tm, Tm + ldt, Tm + 2 * ldt};
    memcpy(x, U, sizeof(double) * (size_t)G);
    x[G] = u_end ? *u_end : 0.0;
    const int it = fo_sf3d_solve(sN, M, K, mat, mc3, T3, iw3, NULL, space_der, Om, x, thr, maxiter);
    memcpy(U, x, sizeof(double) * (size_t)G);
    if (u_end) *u_end = x[G];
    double *row = hist + (int64_t)n * G;
    for (int64_t q = 0; q < G; q++) row[q] = U[q] - Uold[q];
    if (mat_out) memcpy(mat_out, mat, sizeof(double) * (size_t)(7 * V));
    if (om_out) memcpy(om_out, Om, sizeof(double) * (size_t)V);
    if (S_out) memcpy(S_out, S, sizeof(double) * (size_t)G);
    if (iters) *iters = it;
    free(Uold); free(S); free(mat); free(mc3); free(iw3); free(Om); free(x);
    return 0;
}

/* ------------------------------------------------------ distributed order */

static double bk_pow(double d1, double d2, double beta)   /* fr_do.cpp:129-134 */
{
    if (d1 == 0.0) return pow(d2, 1.0 - beta);
    if (d2 == 0.0) return pow(d1, 1.0 - beta);
    return pow(d1, 1.0 - beta) - pow(d2, 1.0 - beta);
}

void fo_caputo_derivative(int ntau, double tau, double a, double g2a, const double *F, double *DF)
{
    double *bkk = (double *)malloc(sizeof(double) * (size_t)ntau);
    for (int i = 0; i < ntau; i++) bkk[i] = bk_pow((i + 1) * tau, i * tau, a);  /* :67 */
    DF[0] = 0.0;
    for (int t = 1; t < ntau; t++) {                                           /* :77-85 */
        double sum = 0.0;
        for (int i = 0; i < t; i++) sum += ((F[i + 1] - F[i]) / tau) * bkk[t - i - 1];
        DF[t] = sum / g2a;
    }
    free(bkk);
}

void fo_do_derivative(int ntau, double tau, int na, const double *WA, const double *gs,
                      const double *F, int maxt, int t0, int j0, double *DF)
{
    double *bkk = (double *)malloc(sizeof(double) * (size_t)ntau * na);
    double *CD = (double *)malloc(sizeof(double) * (size_t)na);
    for (int i = 0; i < ntau; i++)                                   /* fill_arrays :67-68 */
        for (int j = 0; j < na; j++)
            bkk[(int64_t)i * na + j] = bk_pow((i + 1) * tau, i * tau, (na == 1) ? 0.0 : (1.0 * j) / (double)(na - 1));
    for (int t = t0; t < ntau; t++) {                                /* DO_Cder :93-112 */
        double sum = 0.0;
        int jend = (maxt == -1) ? t : ((t > maxt) ? maxt : t);
        for (int i = 0; i < na; i++) {
            double s2 = 0.0;
            for (int j = j0; j < jend; j++)
                if (j >= 0) s2 += ((F[j + 1] - F[j]) / tau) * bkk[(int64_t)(t - j - 1) * na + i];
            s2 /= gs[i];
            CD[i] = s2;
        }
        for (int i = 0; i < na - 1; i++) sum += 0.5 * (WA[i] * CD[i] + WA[i + 1] * CD[i + 1]);
        DF[t] = sum;
    }
    free(bkk);
    free(CD);
}

void fo_do_fused_weights(int nq, const double *aq, const double *Wq, const double *gq,
                         double tau, int nl, double *c)
{
    for (int l = 0; l < nl; l++) {
        double s = 0.0;
        for (int q = 0; q < nq; q++) {
            double e = 1.0 - aq[q];
            /* ((l+1) tau)^e - (l tau)^e = tau^e * b_l(e), b_0 = 1 */
            double b = (l == 0) ? 1.0 : pow((double)l, e) * expm1(e * log1p(1.0 / l));
            s += Wq[q] * pow(tau, e) * b / gq[q];
        }
        c[l] = s;
    }
}

/* source of fr_do eq_ex 0 (fr_do.cpp:464-470) */
static double do_eq_f(int ex, double t, double x)
{
    if (ex == 0)
        return sin(2 * M_PI * x) * (800 * M_PI * M_PI * t * t * t * t + (2400 * (t * t * t * t - t * t * t) / log(t)));
    return 0.0;
}

int fo_do_eq_solve(int ex, int Nx, int Nt, int tblock, int na, double h, double tau, double D,
                   const double *WA, const double *gs, double *C, double *b0_out)
{
    double Aa = 0.5 * D / (h * h), Bb = 0.5 * D / (h * h);           /* eq_init :674-675 */
    double *bkk = (double *)malloc(sizeof(double) * (size_t)Nt * na);
    double *eA = (double *)calloc((size_t)Nx + 1, sizeof(double));
    double *eB = (double *)calloc((size_t)Nx + 1, sizeof(double));
    double *eDF = (double *)calloc((size_t)Nx * tblock, sizeof(double));
    double *DF = (double *)calloc((size_t)Nt + tblock + 2, sizeof(double));
    double *CD = (double *)malloc(sizeof(double) * (size_t)na);
    for (int i = 0; i < Nt; i++)
        for (int j = 0; j < na; j++)
            bkk[(int64_t)i * na + j] = bk_pow((i + 1) * tau, i * tau, (1.0 * j) / (double)(na - 1));
    double b0 = 0.0;                                                  /* :688-690 */
    for (int a = 0; a < na - 1; a++)
        b0 += 0.5 * (WA[a] * bkk[a] / gs[a] + WA[a + 1] * bkk[a + 1] / gs[a + 1]);
    double Ss = (D / (h * h)) + (b0 / tau);
    eA[1] = 0.0;                                                      /* :692-694 */
    for (int i = 1; i < Nx - 1; i++) eA[i + 1] = Bb / (Ss - Aa * eA[i]);
    /* DO_Cder restricted to one node's series, summing j in [j0, min(t,maxt)) */
    #define DO_NODE(Fp, ntau, maxt, t0, j0)                                               \
        for (int t = (t0); t < (ntau); t++) {                                             \
            double sum = 0.0;                                                             \
            int jend = ((maxt) == -1) ? t : ((t > (maxt)) ? (maxt) : t);                  \
            for (int q = 0; q < na; q++) {                                                \
                double s2 = 0.0;                                                          \
                for (int j = (j0); j < jend; j++)                                         \
                    if (j >= 0) s2 += (((Fp)[j + 1] - (Fp)[j]) / tau) * bkk[(int64_t)(t - j - 1) * na + q]; \
                s2 /= gs[q];                                                              \
                CD[q] = s2;                                                               \
            }                                                                             \
            for (int q = 0; q < na - 1; q++) sum += 0.5 * (WA[q] * CD[q] + WA[q + 1] * CD[q + 1]); \
            DF[t] = sum;                                                                  \
        }
    for (int i = 0; i < Nt; i += tblock) {                            /* eq_solve :737-771 */
        for (int j = 0; j < Nx; j++) {
            const double *Fp = C + (int64_t)j * Nt;
            DO_NODE(Fp, i + tblock, ((i == 0) ? i : i - 1), i, 0);
            for (int k = 0; k < tblock; k++) eDF[(int64_t)j * tblock + k] = DF[i + k];
        }
        for (int j = ((i == 0) ? 1 : 0); j < tblock; j++) {
            int s = i + j;                                            /* eq_one_step :724-732 */
            eB[1] = 0.0;
            for (int x = 1; x < Nx - 1; x++) {
                int jj = s - 1;
                double rp = -0.5 * (D / (h * h)) * (C[(int64_t)(x - 1) * Nt + jj] - 2.0 * C[(int64_t)x * Nt + jj] + C[(int64_t)(x + 1) * Nt + jj]);
                double lp = -(b0 * C[(int64_t)x * Nt + jj] / tau) - 0.5 * (do_eq_f(ex, jj * tau, x * h) + do_eq_f(ex, (jj + 1) * tau, x * h));
                double nlp = eDF[(int64_t)x * tblock + ((jj + 1) % tblock)];
                if (!isfinite(lp)) lp = -(b0 * C[(int64_t)x * Nt + jj] / tau) - do_eq_f(ex, (jj + 1) * tau, x * h);
                double Ff = rp + lp + nlp;                            /* eq_Ff :656-665 */
                eB[x + 1] = (eA[x + 1] / Bb) * (Aa * eB[x] - Ff);
            }
            C[s + (int64_t)Nt * (Nx - 1)] = 0.0;
            for (int x = Nx - 2; x >= 0; x--) C[s + (int64_t)Nt * x] = eA[x + 1] * C[s + (int64_t)Nt * (x + 1)] + eB[x + 1];
            if (j != tblock - 1)
                for (int jj = 0; jj < Nx; jj++) {
                    const double *Fp = C + (int64_t)jj * Nt;
                    DO_NODE(Fp, i + j + 2, i + j, i + j + 1, i - 1);
                    eDF[(int64_t)jj * tblock + j + 1] += DF[i + j + 1];
                }
        }
    }
    #undef DO_NODE
    if (b0_out) *b0_out = b0;
    free(bkk); free(eA); free(eB); free(eDF); free(DF); free(CD);
    return 0;
}
