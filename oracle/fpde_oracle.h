/* fpde_oracle -- CPU restatement of FPDE_HPC's L1 history sum and tridiagonal line
 * solves, used ONLY to check results (tests, the smoke check) and as the CPU baseline of
 * the benchmark. It is never linked into, called by or shipped with the GPU library.
 *
 * Parity status: pinned. tests/golden/*.fgv.gz hold outputs of the reference's own FP64
 * code (built from its sources by oracle/Makefile + oracle/ref_pin), and the CPU test
 * suite checks this restatement against them.
 *
 * Conventions (following fpde_hpc_1d.cpp):
 *  - a line has N intervals and nodes 0..N; the unknowns are 1..N-1, nodes 0 and N carry
 *    the boundary conditions (set_xyz_steps :2381-2388);
 *  - the L1 weight of history interval t at step n (producing u^{n+1}) is
 *    kb_t = int_{T_t}^{T_{t+1}} (T_{n+1}-s)^{-alpha} ds  (kb :2167, precalc_kb_3 :4069);
 *  - history increments D_t = u^{t+1} - u^t, stored time-major, one row of P doubles
 *    per interval.
 */
#ifndef FPDE_ORACLE_H
#define FPDE_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Closed-form L1 weights for step n: kb[t], t = 0..n-1, from the time points
 * time[0..n+1]. Cancellation-free: (a+d)^{1-a} - a^{1-a} = a^{1-a} expm1((1-a) log1p(d/a)).
 * Also returns the local weight kkk0 = kb(alpha, n, n+1, n+1) (init_time_step :3947).
 * alpha == 1 gives kb = 0 and kkk0 = 1 (kb :2169-2175). */
void fo_l1_weights(double alpha, const double *time, int n, double *kb, double *kkk0);

/* History sum of one step in the reference's order (time_summing :4110-4136, t descending):
 * S[i] = sum_t (kb[t] * D[t][i]) / tau[t], for i in [i0, i1). D is n rows of P doubles. */
void fo_l1_sum(const double *D, int64_t P, int n, const double *kb, const double *tau,
               int64_t i0, int64_t i1, double *S);

/* Same sum over stored snapshots old[t][i] (t = 0..nold-1), the argument form of the
 * reference's GPU Sum kernel (fpde_hpc_1d.cpp:1407-1478, sum_alg 0): the increment is
 * formed as old[t+1]-old[t] on the fly. */
void fo_l1_sum_snapshots(const double *old, int64_t OS, int nold, const double *kb,
                         const double *tau, int64_t nodes, double *S);

/* Restricted summing (sum_alg 1, time_summing fpde_hpc_1d.cpp:4110-4131): the terms of
 * fo_l1_sum_snapshots from the newest down, stopping before the first |kb[t]| < thr
 * (bs == 0); or the GPU Sum kernel's rule (:1422-1455, bs == BS > 0): chunks of bs terms
 * are added whole (weights before t = 0 count as 0), stopping after the first chunk whose
 * bs weights are all below thr. */
void fo_sum_restricted(const double *old, int64_t OS, int nold, const double *kb, const double *tau,
                       double thr, int bs, int64_t nodes, double *S);

/* Generalized-kernel L1 weights (kb :2167-2301 with g(t) = t^p, g :1889-1930: func_in_kernel
 * 0 -> p = 1, 1 -> 0.5, 2 -> 2, 3 -> func_power): for step n with T = time[n+1],
 *   kb[t] = int_{time[t]}^{time[t+1]} (T^p - s^p)^{-alpha} ds,  t = 0..n-1,  kkk0 = the same over
 *   [time[n], T]. The reference sums truncated Taylor/binomial series (_kb_row :1933,
 *   _kb_row2 :2000); this evaluates the integral by quadrature: Gauss-Legendre on intervals at
 *   least 4 widths from both singular points (s = T, and s = 0 when p is not a positive
 *   integer; 16 points, 8 beyond 32 widths), the double-exponential rule elsewhere, and on the newest interval the
 *   factor delta^-alpha (delta = T - s) integrated analytically on its last 1/16 (delta =
 *   h y^(1/(1-alpha))). T^p - s^p is formed as -T^p expm1(p log1p(-delta/T)) for small delta. */
void fo_weights_g(double p, double alpha, const double *time, int n, double *kb, double *kkk0);

/* Series expansion (sum_alg 2, time_summing :4137-4151 with _kb_row2_fixed_coefs
 * :1159-1180; the GPU kernel's finiteness guards :1459-1469): P moments per node in
 * H[i*P + j], updated with d = cur[i] - prev[i]:
 *   H[i*P+j] += gt^(j+1) * row2[j] * d;  S[i] = sum_j v_j H[i*P+j] / tau_t,
 *   v_0 = pow(gtj, -alpha), v_j = v_{j-1} * (-(-alpha - j + 1) / (j * gtj)). */
void fo_sum_series(const double *prev, const double *cur, int64_t nodes, double *H, int P, const double *row2,
                   double gt, double gtj, double alpha, double tau_t, double *S);

/* Thomas solve of one line (al1 :4002-4027, bt1 :4585-4590, back-substitution in U1
 * :4678-4725): A[i] U[i-1] - R[i] U[i] + B[i] U[i+1] = Om[i], i = 1..N-1.
 * Left boundary: ltype 0 -> U[0] = g0 (Al[1] = 0, Bt[1] = g0); ltype 1 -> flux form
 * (Al[1] = 1, Bt[1] = g0). Right boundary: rtype 0 -> U[N] = gN; rtype 1 -> the
 * zero-/given-flux closure of U1 :4687-4719 with dLN = dL[N-1], including its 1e-15
 * thresholds (which may read the previous U[N-1]). U holds N+1 values in and out.
 * Arrays A, B, R, Om are indexed 0..N (entries 0 and N unused). */
void fo_thomas_line(int N, const double *A, const double *B, const double *R, const double *Om,
                    int ltype, double g0, int rtype, double gN, double dLN, double *U);

/* Tridiagonal coefficients of the H equation with gamma = 1 on one line
 * (A_ / B / R :3095-3142 with Dg = 1, kb(1,..) = 1): from the node conductivities k[i],
 * the inverse capacity iw[i] and the steps dL[i] = x[i+1]-x[i]:
 *   A[i] = k[i-1] iw[i] / (dL[i] dL[i-1]),  B[i] = k[i] iw[i] / dL[i]^2,
 *   Rlap[i] = iw[i] (k[i]/dL[i]^2 + k[i-1]/(dL[i] dL[i-1])).
 * The full diagonal is R[i] = Rlap[i] + Da*kkk0/tau. */
void fo_line_coefs(int N, const double *k, const double *iw, const double *dL,
                   double *A, double *B, double *Rlap);

/* One time step of a single line (the 1D form of the K pass, Om1 :4165-4267 + U1):
 *   Om[i] = -lam U[i] + src[i] + Da S[i],   R[i] = Rlap[i] + lamR
 * with lam = Da*(kkk0/tau_n), lamR = Da*kkk0/tau_n, S from the stored history.
 * hist holds n increment rows of P >= N+1 doubles; the new increment is written to row n.
 * src may be NULL (no source). Returns 0. */
int fo_line_step(int N, double *U, double *hist, int64_t P, int n,
                 const double *kb, const double *tau, double Da, double kkk0,
                 const double *A, const double *B, const double *Rlap, const double *src,
                 int ltype, double g0, int rtype, double gN, double dLN, double *S_out);

/* Full run of the 1D Caputo line problem with uniform tau and constant boundary data:
 * steps time steps from U (N+1 values, overwritten with the final state).
 * hist must hold steps rows of P doubles. Weights are the closed form above; Da is the
 * caller's 1/Gamma(1-alpha). Returns 0. OpenMP parallel over nodes for the history sum. */
int fo_line_run(int N, double *U, double *hist, int64_t P, int steps, double tau, double alpha,
                double Da, const double *A, const double *B, const double *Rlap,
                int ltype, double g0, int rtype, double gN, double dLN);

/* General line run (uniform tau), used for the distributed-order equation of fr_do.cpp
 * (eq_solve :733-775, eq_Ff :656-665, eq_one_step :724-732) and any other lag weights:
 *   S[i]  = sum_{t<n} w[n-t] D_t[i]                            (history, lag weights w[1..])
 *   Om[i] = -theta (A[i] U[i-1] - Rlap[i] U[i] + B[i] U[i+1])  (explicit part, old U)
 *           - w[0] U[i] + src[i] + S[i],       R[i] = Rlap[i] + w[0].
 * w holds steps+1 values (w[0] the local weight). src (may be NULL) holds src_rows rows of
 * N+1 values; step n uses row min(n, src_rows-1). fr_do's scheme is w[l] = c_l / tau with
 * the fused DO weights c (fo_do_fused_weights), theta = 1, A = B = D/(2h^2), Rlap = D/h^2,
 * src = -(f(t_n) + f(t_{n+1}))/2. hist must hold steps rows of P doubles. Returns 0. */
int fo_line_run_general(int N, double *U, double *hist, int64_t P, int steps, const double *w, double theta,
                        const double *A, const double *B, const double *Rlap, const double *src, int src_rows,
                        int ltype, double g0, int rtype, double gN, double dLN);

/* One step of the reference's 3D LOD scheme (calc_step mode 3 :5144-5779, implicit3d 0,
 * split3d 0): K pass (lines along k, with source Rp and the history sum), then the _M
 * pass (lines along j), then the sN pass (lines along i). The grid has (sN+2)(M+2)(K+2)
 * points indexed i + j (sN+2) + k (sN+2)(M+2) (idx :1181). coefA/B/Rlap are three grids
 * (pass 2 = K, 1 = _M, 0 = sN) of the line coefficients at each node; the diagonal is
 * R = Rlap + Da*kkk0/tau_n and the RHS local term Da*(kkk0/tau_n) U. bc is a grid of
 * Dirichlet values on the line ends, rp the K-pass source. hist holds n increment
 * grids; the new one is written as row n.
 * S_out (grid, may be NULL) receives the history sums. Left/right boundaries Dirichlet
 * (the analytic-test configuration). */
int fo_lod_step_dirichlet(int sN, int M, int K, double *U, double *hist, int n,
                          const double *kb, const double *tau, double Da, double kkk0,
                          const double *coefA, const double *coefB, const double *coefRlap,
                          const double *rp, const double *bc, double *S_out);

/* The same step with boundary kinds per pass (index = pass: 0 sN, 1 _M, 2 K): lkind/rkind 0
 * Dirichlet with the value from bc at the line end, 1 the flux form of al1 (Al[1] = 1,
 * Bt[1] = bc) and the flux closure of U1 (:4687-4719) with the pass's last step dLN. */
int fo_lod_step(int sN, int M, int K, double *U, double *hist, int n,
                const double *kb, const double *tau, double Da, double kkk0,
                const double *coefA, const double *coefB, const double *coefRlap,
                const double *rp, const double *bc, const int *lkind, const int *rkind, const double *dLN,
                double *S_out);

/* The Dirichlet step with given history sums S_in (grid; read on the K-pass nodes) in place of
 * the L1 sum: the reference's sum_alg 2 runs, whose series sums the caller forms (fo_sum_series).
 * The new increment grid is still written as hist row n. */
int fo_lod_step_dirichlet_sum(int sN, int M, int K, double *U, double *hist, int n, const double *tau, double Da,
                              double kkk0, const double *coefA, const double *coefB, const double *coefRlap,
                              const double *rp, const double *bc, const double *S_in);

/* ---- Richards problem: solution-dependent coefficients ---- */

/* The reference's closures at suctions P[0..n-1] (metres): water content (wetness, cv_form 4),
 * 1/(dw/dh) (inv_dw_dh; 1e20 where saturated) and the conductivity KK (k_form 1 VGM, 2
 * Averianov, times ksat). Any output may be NULL. */
void fo_richards_closures(int n, const double *P, int kform, double ksat, double *w, double *iw, double *kk);

/* One 3D LOD step of the reference's Richards problem (analytic_test 0, no irrigation,
 * bottom_cond 0): coefficients from each line's current values, the surface condition of the
 * sN pass from the evaporation rate E, zero flux elsewhere; rp the K-pass source grid. */
int fo_lod_step_richards(int sN, int M, int K, double *U, double *hist, int n, const double *kb, const double *tau,
                         double Da, double kkk0, const double *sZ, const double *sdL, const double *dLx,
                         const double *dLy, int kform, double ksat, double E, const double *rp, double *S_out);

/* The same step with the salt concentration C (equation 1, is_c): on every line of every pass, after
 * the H solve, C's solve with the constant coefficient grids cA/cB/cR (3 passes x grid: the
 * reference's A_/B/R of equation 1 with Da = 0), the coupling terms of Om1 with the new H and its
 * KK and the old C, C's own history histC (rows of the grid) and sum. C = NULL: H alone. */
int fo_lod_step_richards_salt(int sN, int M, int K, double *U, double *hist, int n, const double *kb,
                              const double *tau, double Da, double kkk0, const double *sZ, const double *sdL,
                              const double *dLx, const double *dLy, int kform, double ksat, double E,
                              const double *rp, double *S_out, double *C, double *histC, const double *cA,
                              const double *cB, const double *cR, double nu, double sigma, double *SC_out);

/* A 1D Richards line with the history (mode-1 closures, P = -(U[i] - Z[i])): per step the L1
 * sum, coefficients from the current values, the surface condition from the step's evaporation
 * rate E[min(n, erows-1)], the right end rtype (0 Dirichlet gN, 1 flux closure). */
int fo_line_run_richards(int N, double *U, double *hist, int64_t P, int steps, double tau, double alpha, double Da,
                         const double *Z, const double *dL, int kform, double ksat, const double *E, int erows,
                         const double *src, int src_rows, int rtype, double gN, double dLN);

/* ---- implicit space-fractional operator (impl 2, TMA 0) ---- */

/* vmul_T (fpde_hpc_1d.cpp:6618-6747, toeplitz_mult_alg 0, equation 0) on one line of n
 * intervals (n+1 unknowns): r = tridiag(mat) x + iw * (T * (tridiag(mc) x)) with the Toeplitz sum
 * over interior rows i = 1..n-1: sum_{j=1}^{i-1} bt[j] Tm[i-j+1], minus (space_der 1)
 * sum_{j=i+1}^{n-1} bt[j] Tm[j-i+1]; divided by rs[i] when rs is given (implicit_row_scaling).
 * mat and mc are 3 x (n+1) (rows 0 = lower, 1 = diagonal, 2 = upper); mc is read at rows 1..n-1,
 * iw at 1..n-1 (NULL: 1.0, the C/T equations), Tm at 2..n-1. bt is scratch of n+1 values. */
void fo_sf_matvec(int n, const double *mat, const double *mc, const double *Tm, const double *iw,
                  const double *rs, int space_der, const double *x, double *r, double *bt);

/* solve_mln<1> (:812-1157) with vmul_T on the same operands over the whole line (rb = 0,
 * re = n+1): x holds the initial guess and receives the solution; stops when
 * |r.r / (n+1)| < thr or after maxiter - 1 iterations. Returns the iteration count. */
int fo_sf_solve(int n, const double *mat, const double *mc, const double *Tm, const double *iw,
                const double *rs, int space_der, const double *B, double *x, double thr, int maxiter);

/* One LOD step (mode 3, implicit3d 0) with impl 2: as fo_lod_step with Dirichlet line ends, but
 * every line is solved with fo_sf_solve on the system implicit2_gen forms (:4630-4663): interior
 * rows (A_, -(Rlap + Da kkk0/tau), B), identity rows at both ends with the right-hand side
 * bc0 / bcN, the operand grids mc (3 passes x 3 x G), iw (3 x G) and the Toeplitz rows Tm
 * (3 x ldt, pass p's row at p*ldt). *iters (may be NULL) receives the total iteration count.
 * rkind (3, may be NULL: Dirichlet) with 1 at a pass makes its lines' far ends the flux rows of
 * bottom_cond 0, U[N] - U[N-1] = bcN dLN[pass] (:4652-4655). */
int fo_lod_step_sf(int sN, int M, int K, double *U, double *hist, int n, const double *kb, const double *tau,
                   double Da, double kkk0, const double *coefA, const double *coefB, const double *coefRlap,
                   const double *mc, const double *iw, const double *Tm, int ldt, int space_der, double thr,
                   int maxiter, const double *rp, const double *bc, double *S_out, int64_t *iters,
                   const int *rkind, const double *dLN);

/* ---- fully implicit 3D space-fractional operator (implicit3d 1) ---- */

/* vmul_T_3d (:6801-8722, toeplitz_mult_alg 0, equation 0) on V = (sN+2)(M+2)(K+2) + 1 values:
 * mat 7 x V (Mat_3d), mc 9 x V (Mcoefs_3d[c][d] at plane 3c+d), Tm[c] the Toeplitz row of axis c
 * (0 sN, 1 _M, 2 K), iw 3 x V or NULL, rs V or NULL, bt V scratch. */
void fo_sf3d_matvec(int sN, int M, int K, const double *mat, const double *mc, const double *const *Tm,
                    const double *iw, const double *rs, int space_der, const double *x, double *r, double *bt);

/* solve_mln<1> with vmul_T_3d over the V values (calc_step :5705); returns the iteration count. */
int fo_sf3d_solve(int sN, int M, int K, const double *mat, const double *mc, const double *const *Tm,
                  const double *iw, const double *rs, int space_der, const double *B, double *x, double thr,
                  int maxiter);

/* One step of the fully implicit scheme (calc_step :5160-5716 with implicit3d 1, impl 2): the
 * system assembled from every line's implicit2_gen system of the three passes, one solve, the
 * history row. Operands as fo_lod_step_sf; *u_end is the value past the grid (may be NULL: 0);
 * mat_out (7 x V), om_out (V), S_out (G) and iters may be NULL; rkind / dLN as fo_lod_step_sf. */
int fo_lod_step_sf3d(int sN, int M, int K, double *U, double *u_end, double *hist, int n, const double *kb,
                     const double *tau, double Da, double kkk0, const double *coefA, const double *coefB,
                     const double *coefRlap, const double *mc, const double *iw, const double *Tm, int ldt,
                     int space_der, double thr, int maxiter, const double *rp, const double *bc, double *mat_out,
                     double *om_out, double *S_out, int64_t *iters, const int *rkind, const double *dLN);

/* ---- distributed order (fr_do.cpp) ---- */

/* Caputo derivative of sampled F (Cder :74-86 with an F array): DF[t] for t = 1..ntau-1,
 * bk weights ((i+1)tau)^{1-a} - (i tau)^{1-a}, divided by Gamma(2-a) = g2a. */
void fo_caputo_derivative(int ntau, double tau, double a, double g2a, const double *F, double *DF);

/* DO derivative (DO_Cder :89-113): na orders a_i = i/(na-1) on [0,1], weights WA[i],
 * Gamma(2-a_i) = gs[i], trapezoid in a, samples F[0..ntau-1] (uniform tau). Terms j in
 * [j0, min(t, maxt)) (maxt = -1: no limit) for t in [t0, ntau). Writes DF[t]. */
void fo_do_derivative(int ntau, double tau, int na, const double *WA, const double *gs,
                      const double *F, int maxt, int t0, int j0, double *DF);

/* Fused DO weights: c[l] = sum_q Wq[q] ((l+1)tau)^{1-a_q} - (l tau)^{1-a_q}) / Gamma(2-a_q)
 * for l = 0..nl-1 (cancellation-free), with Wq the effective quadrature weights. */
void fo_do_fused_weights(int nq, const double *aq, const double *Wq, const double *gq,
                         double tau, int nl, double *c);

/* DO diffusion solve of fr_do.cpp eq_solve (:733-775): Crank-Nicolson in x, blocked
 * far/near DO history, Thomas sweeps with fixed alphas (eq_init :666-695,
 * eq_one_step :724-732). ex selects the source (0: eq_ex 0, 1: zero). C is Nx*Nt,
 * node-major, with C[i*Nt] the initial state. Returns 0. */
int fo_do_eq_solve(int ex, int Nx, int Nt, int tblock, int na, double h, double tau, double D,
                   const double *WA, const double *gs, double *C, double *b0_out);

#ifdef __cplusplus
}
#endif
#endif
