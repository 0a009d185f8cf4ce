/* Pin harness for the FP64 Caputo path of fpde_hpc_1d.cpp (test infrastructure).
 *
 * Built by oracle/Makefile from the reference source where it lies (the file is
 * #included with its main renamed), never from a copy. It runs the reference's own
 * H_solver in its 3D LOD mode -- the only mode in which the reference applies the FP64
 * L1 history sum (fpde_hpc_1d.cpp:4258-4263, :4108) -- and records, step by step:
 *   - the L1 weights kb_3_cache and the local weight kkk0 (precalc_kb_3 :4069-4085,
 *     init_time_step :3942-3949);
 *   - the history sum b_Utimesum computed by time_summing (:4086-4164);
 *   - the grid after each step (calc_step :5100-5779);
 *   - everything a replay of the step needs that the reference computes from its
 *     hard-coded analytic problems: the tridiagonal coefficients A_/B/R of every line of
 *     every pass (:3095-3142), the source Rp of the K pass (:2724) and the Dirichlet
 *     boundary values bc0/bcN of every line (:4491-4583).
 * Weights-only scenarios also cover the generalized Caputo kernels (func_in_kernel 1-3,
 * g(t) = sqrt(t), t^2, t^p; g :1889-1930) with uniform and variable steps.
 * Two more scenarios run the column with the reference's other history modes
 * (time_summing :4108-4151): sum_alg 1 (restricted summing) and sum_alg 2 (series
 * expansion, with the per-step coefficient row row2_precalc[time_i1][0] and g(t) at the
 * step's ends, the inputs of the Sum kernel's series branch).
 * The oracle and the GPU path replay the same steps from those inputs and must match the
 * recorded grids to 1e-12. Scenarios are listed in main().
 */
#define main fpde_reference_main
#include "fpde_hpc_1d.cpp"
#undef main
#include "fgv_write.h"

struct PassState {
    int m3d_x, m3d_y, m3d_c, N_, NB_;
    double *dL_, *Z_;
};

static PassState save_state(H_solver *s)
{
    PassState p = {s->m3d_x, s->m3d_y, s->m3d_c, N, NB, s->dL, s->Z};
    return p;
}
static void restore_state(H_solver *s, const PassState &p)
{
    s->m3d_x = p.m3d_x; s->m3d_y = p.m3d_y; s->m3d_c = p.m3d_c;
    N = p.N_; NB = p.NB_; s->dL = p.dL_; s->Z = p.Z_;
}
/* Put the solver in the state calc_step gives it for one line of one pass
 * (K pass :5258-5268, _M pass :5409-5419, sN pass :5559-5569). */
static void enter_line(H_solver *s, int pass, int a, int b)
{
    s->equation = 0;
    s->m3d_x = a; s->m3d_y = b; s->m3d_c = pass;
    s->U.set(s->b_U, a, b, pass);
    if (pass == 2) { s->dL = s->dLy; s->Z = s->Y; N = K; NB = KB; }
    if (pass == 1) { s->dL = s->dLx; s->Z = s->X; N = _M; NB = MB; }
    if (pass == 0) { s->dL = s->sdL; s->Z = s->sZ; N = sN; NB = sNB; }
}
static inline size_t gidx(int i, int j, int k) { return (size_t)idx(i, j, k); }

/* Record the coefficient grids of the three passes: for pass c the value at the grid
 * node of line position i is the reference's A_(i), B(i) and the Laplacian part a1 of
 * R(i) (:3117-3123). a1 is read by evaluating R with Da = 0, so that a2 = Da*kkk0/tau
 * vanishes exactly; a replay adds a2 of each step (kkk0 varies in its last bits from
 * step to step because Time is accumulated). */
static void record_coefs(H_solver *s, FgvWriter &w)
{
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    PassState st = save_state(s);
    double Da_saved = s->Da;
    s->Da = 0.0;
    for (int pass = 0; pass < 3; pass++) {
        std::vector<double> A(G, 0.0), B(G, 0.0), R(G, 0.0);
        if (pass == 2)
            for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) {
                enter_line(s, 2, i, j);
                for (int k = 1; k < K; k++) { A[gidx(i, j, k)] = s->A_(k); B[gidx(i, j, k)] = s->B(k); R[gidx(i, j, k)] = s->R(k); }
            }
        if (pass == 1)
            for (int k = 1; k < K; k++) for (int i = 1; i < sN; i++) {
                enter_line(s, 1, i, k);
                for (int j = 1; j < _M; j++) { A[gidx(i, j, k)] = s->A_(j); B[gidx(i, j, k)] = s->B(j); R[gidx(i, j, k)] = s->R(j); }
            }
        if (pass == 0)
            for (int j = 1; j < _M; j++) for (int k = 1; k < K; k++) {
                enter_line(s, 0, j, k);
                for (int i = 1; i < sN; i++) { A[gidx(i, j, k)] = s->A_(i); B[gidx(i, j, k)] = s->B(i); R[gidx(i, j, k)] = s->R(i); }
            }
        char nm[32];
        std::vector<uint64_t> dims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
        snprintf(nm, sizeof nm, "coefA_pass%d", pass); w.put(nm, dims, A.data());
        snprintf(nm, sizeof nm, "coefB_pass%d", pass); w.put(nm, dims, B.data());
        snprintf(nm, sizeof nm, "coefRlap_pass%d", pass); w.put(nm, dims, R.data());
    }
    s->Da = Da_saved;
    restore_state(s, st);
}

/* Source of the K pass and Dirichlet values of every line, as used by the step that
 * has just been taken (Rp and bc0/bcN read Time/tstep of that step). */
static void record_step_inputs(H_solver *s, std::vector<double> &rp, std::vector<double> &bc)
{
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    size_t o = rp.size();
    rp.resize(o + G, 0.0);
    bc.resize(o + G, 0.0);
    double *RP = &rp[o], *BC = &bc[o];
    PassState st = save_state(s);
    for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) {
        enter_line(s, 2, i, j);
        for (int k = 1; k < K; k++) RP[gidx(i, j, k)] = s->Rp(k);
        BC[gidx(i, j, 0)] = s->bc0();
        BC[gidx(i, j, K)] = s->bcN();
    }
    for (int k = 1; k < K; k++) for (int i = 1; i < sN; i++) {
        enter_line(s, 1, i, k);
        BC[gidx(i, 0, k)] = s->bc0();
        BC[gidx(i, _M, k)] = s->bcN();
    }
    for (int j = 1; j < _M; j++) for (int k = 1; k < K; k++) {
        enter_line(s, 0, j, k);
        BC[gidx(0, j, k)] = s->bc0();
        BC[gidx(sN, j, k)] = s->bcN();
    }
    restore_state(s, st);
}

static void set_dims(int bs, int nb, int mb, int kb)
{
    BS = bs; NB = nb; MB = mb; KB = kb;
    sN = N = BS * NB; sNB = NB;
    _M = BS * MB; K = BS * KB;
    delete[] F; delete[] BVK;
    F = new double[N + _M + K + 2];
    BVK = new double[BS];
}

/* One LOD run (mode 3, implicit 0, impl3d 0, split3d 0, sum_alg 0, EPS 1e-15). */
static void run_lod(const char *path, int analytic, int bs, int nb, int mb, int kb,
                    double alpha, const std::vector<double> &taus, int record_inputs)
{
    set_dims(bs, nb, mb, kb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(analytic, 1, 5, 0, 1, alpha, 1.0, 0, 0, 0, 3, lg, 2);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("Da", s->Da); w.scalar("analytic", analytic);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    std::vector<double> kb_all, kb_off, kkk0, tauv, S_all, U_all, rp, bc;
    for (size_t n = 0; n < taus.size(); n++) {
        s->calc_step(taus[n]);
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        if (n == 0 && record_inputs) record_coefs(s, w);
        if (record_inputs) {
            S_all.insert(S_all.end(), s->b_Utimesum, s->b_Utimesum + G);
            U_all.insert(U_all.end(), s->b_U, s->b_U + G);
            record_step_inputs(s, rp, bc);
        }
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = taus.size();
    w.put("tau", tauv); w.put("kkk0", kkk0);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    if (record_inputs) {
        w.put("S", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, S_all.data());
        w.put("U", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, U_all.data());
        w.put("Rp", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, rp.data());
        w.put("BC", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, bc.data());
    }
    double err = s->analytic_compare(NULL);
    w.scalar("analytic_sq_err", err);
    delete s;
    fclose(lg);
    printf("wrote %s (%zu steps, grid %dx%dx%d)\n", path, taus.size(), sN, _M, K);
}

/* The column (analytic 2) with sum_alg 1 or 2: per step the history sum b_Utimesum, the grid,
 * the weights kb_3_cache (sum_alg 1) or the series inputs (sum_alg 2: row2_precalc[time_i1][0]
 * padded with zeros to sum_param values, gt = g(Time[tstep]), gtj = g(Time[tstep+1]),
 * tau[tstep]). Old snapshots are kept (dont_clear_sum_alg1) so that the record is complete. */
static void run_sumalg(const char *path, int alg, double param, int kcells, double alpha, double tau, int steps)
{
    set_dims(1, 3, 3, kcells);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0;
    sum_alg = alg; sum_param = param; dont_clear_sum_alg1 = 1;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, 1, alpha, 1.0, 0, 0, 0, 3, lg, 2);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("sum_alg", alg); w.scalar("sum_param", param);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    const int P = (int)ceil(param);
    std::vector<double> kb_all, kb_off, tauv, S_all, U_all, row2, gt, gtj;
    for (int n = 0; n < steps; n++) {
        s->calc_step(tau);
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        tauv.push_back(s->tau[s->tstep]);
        S_all.insert(S_all.end(), s->b_Utimesum, s->b_Utimesum + G);
        U_all.insert(U_all.end(), s->b_U, s->b_U + G);
        if (alg == 2) {
            const std::vector<double> &r = s->row2_precalc[s->time_i1][0];
            for (int j = 0; j < P; j++) row2.push_back(j < (int)r.size() ? r[j] : 0.0);
            gt.push_back(s->g(s->Time[s->tstep]));
            gtj.push_back(s->g(s->Time[s->tstep + 1]));
        }
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = steps;
    w.put("tau", tauv);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("S", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, S_all.data());
    w.put("U", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, U_all.data());
    if (alg == 2) {
        w.put("row2", {ns, (uint64_t)P}, row2.data());
        w.put("gt", gt); w.put("gtj", gtj);
    }
    delete s;
    fclose(lg);
    sum_alg = 0; sum_param = 1e-5; dont_clear_sum_alg1 = 0;
    printf("wrote %s (sum_alg %d, %d steps)\n", path, alg, steps);
}

/* Wall-clock timing of the reference's column run, for the CPU baseline
 * (mode 3 BS 1 NB 3 M 3 K <n>, analytic 2, sum_alg 0, EPS 1e-15). */
static void time_column(int kcells, double alpha, double tau, int steps)
{
    set_dims(1, 3, 3, kcells);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, 1, alpha, 1.0, 0, 0, 0, 3, lg, 2);
    struct timespec a, b;
    clock_gettime(CLOCK_MONOTONIC, &a);
    for (int n = 0; n < steps; n++) s->calc_step(tau);
    clock_gettime(CLOCK_MONOTONIC, &b);
    double sec = (b.tv_sec - a.tv_sec) + 1e-9 * (b.tv_nsec - a.tv_nsec);
    double node_steps = 4.0 * (kcells - 1) * steps;
    printf("{\"K\": %d, \"steps\": %d, \"seconds\": %.6f, \"node_steps_per_s\": %.6g}\n",
           kcells, steps, sec, node_steps / sec);
    delete s;
    fclose(lg);
}

/* The Richards problem of the reference (analytic_test 0: van Genuchten-Mualem water content
 * cv_form 4 and conductivity k_form 1 or Averianov k_form 2, wetness / inv_dw_dh / KK
 * :2493-2657) in its 3D LOD mode with the history, no irrigation (no_irr 1), zero-flux bottom
 * and sides (bottom_cond 0): the tridiagonal coefficients A_/B/R (:3095-3142) change with the
 * solution every step. Recorded per step, besides the weights, history sums and grids:
 *   Rp - the K-pass source (root water uptake, :2724-2978), evaluated at the state and time the
 *        step's K pass sees (the grid at the start of the step, Time[tstep] of the step);
 *   E  - the evaporation rate of the step (Uc :3036-3070 with no irrigation is dL[0] E / KK(1)).
 * A replay computes the coefficients and the top boundary value from its own grid. */
static void run_richards(const char *path, int kform, int rpform, int bs, int nb, int mb, int kb, double alpha,
                         double tau, int steps)
{
    set_dims(bs, nb, mb, kb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(0, rpform, 4, 1, 0, alpha, 1.0, 0, 0, 0, 3, lg, kform);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("Da", s->Da); w.scalar("k_form", kform); w.scalar("rp_form", rpform);
    w.scalar("k_sat", s->k);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    w.put("sZ", std::vector<double>(s->sZ, s->sZ + sN + 2));
    w.put("sdL", std::vector<double>(s->sdL, s->sdL + sN + 2));
    w.put("dLx", std::vector<double>(s->dLx, s->dLx + _M + 2));
    w.put("dLy", std::vector<double>(s->dLy, s->dLy + K + 2));
    std::vector<double> kb_all, kb_off, kkk0, tauv, S_all, U_all, rp, Ev;
    for (int n = 0; n < steps; n++) {
        /* the inputs as the step sees them: advance Time/tau/tstep as init_time_step does,
         * evaluate, and put them back before the step itself */
        s->Time.push_back(s->Time[s->Time.size() - 1] + tau);
        s->tau.push_back(tau);
        s->tstep++;
        size_t o = rp.size();
        rp.resize(o + G, 0.0);
        PassState st = save_state(s);
        for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) {
            enter_line(s, 2, i, j);
            for (int k = 1; k < K; k++) rp[o + gidx(i, j, k)] = s->Rp(k);
        }
        restore_state(s, st);
        double E = s->Ev * s->day_night_coef();
        if (rpform == 3) E += s->Tr * s->day_night_coef();
        Ev.push_back(E);
        s->Time.pop_back();
        s->tau.pop_back();
        s->tstep--;
        s->calc_step(tau);
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        S_all.insert(S_all.end(), s->b_Utimesum, s->b_Utimesum + G);
        U_all.insert(U_all.end(), s->b_U, s->b_U + G);
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = steps;
    w.put("tau", tauv); w.put("kkk0", kkk0);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("E", Ev);
    w.put("S", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, S_all.data());
    w.put("U", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, U_all.data());
    w.put("Rp", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, rp.data());
    delete s;
    fclose(lg);
    printf("wrote %s (Richards k_form %d, %d steps, grid %dx%dx%d)\n", path, kform, steps, sN, _M, K);
}

/* The reference's known answer for its column (mode 3, BS 1, NB 3, M 3, K kc, analytic problem 2):
 * the squared error against the exact solution that its run prints (analytic_compare
 * :3277-3312), for a run too long to record step by step. Its inputs separate into space and
 * time parts, so the record stays small: the K-pass source is S1(node) - p2(t) (Rp :2766-2795;
 * S1 = Rp with Time = 0, where p2 vanishes; p2(n) read at one node) and every line-end value is
 * V(node) + vt(t) (bc0/bcN = testF3d :3181-3231; vt(n) read at the sN line start, where V = 0;
 * V from the first step). Also the final grid and the exact solution at the final time. */
static void run_kat(const char *path, int kc, double alpha, double tau, int steps)
{
    set_dims(1, 3, 3, kc);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, 1, alpha, 1.0, 0, 0, 0, 3, lg, 2);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("Da", s->Da); w.scalar("tau", tau);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    std::vector<double> p2, vt, kkk0, rp0, bc0g, S1(G, 0.0);
    for (int n = 0; n < steps; n++) {
        s->calc_step(tau);
        kkk0.push_back(s->kkk0);
        if (n == 0) {
            record_coefs(s, w);
            std::vector<double> bcv;
            record_step_inputs(s, rp0, bcv);
            bc0g = bcv;
            const double t_saved = s->Time[s->tstep];             /* S1: the source at Time 0 */
            s->Time[s->tstep] = 0.0;
            PassState st = save_state(s);
            for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) {
                enter_line(s, 2, i, j);
                for (int k = 1; k < K; k++) S1[gidx(i, j, k)] = s->Rp(k);
            }
            restore_state(s, st);
            s->Time[s->tstep] = t_saved;
        }
        PassState st = save_state(s);
        enter_line(s, 2, 1, 1);
        p2.push_back(S1[gidx(1, 1, 1)] - s->Rp(1));
        enter_line(s, 0, 1, 1);
        vt.push_back(s->bc0());
        restore_state(s, st);
    }
    std::vector<double> exact(G, 0.0);
    for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) for (int k = 1; k < K; k++)
        exact[gidx(i, j, k)] = s->testF3d(i, j, k, s->tstep + 1);
    const double err = s->analytic_compare(NULL);
    w.put("S1", gdims, S1.data());
    w.put("BC0", gdims, bc0g.data());
    w.put("p2", p2); w.put("vt", vt); w.put("kkk0", kkk0);
    w.put("U_final", gdims, s->b_U);
    w.put("exact_final", gdims, exact.data());
    w.scalar("analytic_sq_err", err);
    delete s;
    fclose(lg);
    printf("wrote %s (column K %d, %d steps, analytic squared error %.6g)\n", path, kc, steps, err);
}

/* A 3D known answer with gpu_test.sh's error_tests parameters at NB M K 2 (mode 3, BS 10: 20 x 20 x
 * 20 cells, aa 0.8, bb 1.0, analytic problem 2, Dirichlet ends, FK 3 with FP 0.8: the generalized
 * kernel g(t) = t^0.8, EPS2 1e-7 with the default EPS 1e-5, Tau 0.0025, Tm 0.1: 40 steps, impl 0,
 * sum_alg 0; the script itself runs them at NB M K 4): the reference prints the squared error
 * 0.0472441 against the exact solution. Records as
 * run_kat, plus the weight rows of every step (its series weights at EPS 1e-5: only its own rows
 * reproduce the run). */
static void run_kat3d(const char *path, int bs, int nb, double alpha, double tau, int steps, int alg = 0,
                      int moments = 16)
{
    set_dims(bs, nb, nb, nb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = alg;
    if (alg == 2) sum_param = moments;
    func_in_kernel = 3; func_power = 0.8;
    global_eps = 1e-5; global_eps2 = 1e-7;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, 1, alpha, 1.0, 0, 0, 0, 3, lg, 2);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("Da", s->Da); w.scalar("tau", tau); w.scalar("func_power", func_power);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    std::vector<double> p2, vt, kkk0, tauv, kb_all, kb_off, rp0, bc0g, S1(G, 0.0), row2, gt, gtj;
    const int P = moments;
    for (int n = 0; n < steps; n++) {
        s->calc_step(tau);
        if (alg == 2) {       /* the series inputs of this step, as run_sumalg */
            const std::vector<double> &r = s->row2_precalc[s->time_i1][0];
            for (int j = 0; j < P; j++) row2.push_back(j < (int)r.size() ? r[j] : 0.0);
            gt.push_back(s->g(s->Time[s->tstep]));
            gtj.push_back(s->g(s->Time[s->tstep + 1]));
        }
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        if (n == 0) {
            record_coefs(s, w);
            std::vector<double> bcv;
            record_step_inputs(s, rp0, bcv);
            bc0g = bcv;
            const double t_saved = s->Time[s->tstep];             /* S1: the source at Time 0 */
            s->Time[s->tstep] = 0.0;
            PassState st = save_state(s);
            for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) {
                enter_line(s, 2, i, j);
                for (int k = 1; k < K; k++) S1[gidx(i, j, k)] = s->Rp(k);
            }
            restore_state(s, st);
            s->Time[s->tstep] = t_saved;
        }
        PassState st = save_state(s);
        enter_line(s, 2, 1, 1);
        p2.push_back(S1[gidx(1, 1, 1)] - s->Rp(1));
        enter_line(s, 0, 1, 1);
        vt.push_back(s->bc0());
        restore_state(s, st);
    }
    kb_off.push_back((double)kb_all.size());
    std::vector<double> exact(G, 0.0);
    for (int i = 1; i < sN; i++) for (int j = 1; j < _M; j++) for (int k = 1; k < K; k++)
        exact[gidx(i, j, k)] = s->testF3d(i, j, k, s->tstep + 1);
    const double err = s->analytic_compare(NULL);
    w.put("S1", gdims, S1.data());
    w.put("BC0", gdims, bc0g.data());
    w.put("p2", p2); w.put("vt", vt); w.put("kkk0", kkk0); w.put("tau_steps", tauv);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("U_final", gdims, s->b_U);
    w.put("exact_final", gdims, exact.data());
    w.scalar("analytic_sq_err", err);
    w.scalar("sum_alg", alg);
    if (alg == 2) {
        w.scalar("sum_param", P);
        w.put("row2", {(uint64_t)steps, (uint64_t)P}, row2.data());
        w.put("gt", gt); w.put("gtj", gtj);
    }
    delete s;
    fclose(lg);
    func_in_kernel = 0; func_power = 0.6;
    global_eps = 1e-15; global_eps2 = 1e-15;
    sum_alg = 0; sum_param = 1e-5;
    printf("wrote %s (%d x %d x %d, FK 3 FP 0.8, %d steps, analytic squared error %.6g)\n", path, sN, _M, K, steps,
           err);
}

/* The Richards problem coupled with salt concentration C (analytic_test 0 with is_c = 1: nu
 * nonzero, :3515): on every line of every pass calc_step solves H (U1(0)) and then C (U1(1))
 * (:5270-5278), each with its own L1 history (oldC, time_summing :4086-4164). (With is_t = 1 the
 * reference's mode-3 constructor writes T0 through a row that is not set yet, :3640, and stops
 * with a null dereference, so no 3D run with temperature exists.) Records, besides the Richards
 * inputs: the initial and per-step C grids with their history sums, the constant line
 * coefficients of equation 1 per pass (as record_coefs, Da = 0) and the physical constants of the
 * coupling terms (Om1 :4195-4256). */
static void run_richards_ct(const char *path, int kform, int bs, int nb, int mb, int kb, double alpha, double tau,
                            int steps)
{
    set_dims(bs, nb, mb, kb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 0; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(0, 1, 4, 1, 0, alpha, 1.0, 1, 0, 0, 3, lg, kform);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    /* the reference starts from C0 = 0 everywhere and, without irrigation, nothing makes C nonzero:
     * start from a smooth salt field instead (the reference's own steps then move it) */
    for (int i = 0; i <= sN + 1; i++) for (int j = 0; j <= _M + 1; j++) for (int k = 0; k <= K + 1; k++)
        s->b_C[gidx(i, j, k)] = 2.0 + std::sin(0.9 * i + 0.4 * j) * std::cos(0.6 * k);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("Da", s->Da); w.scalar("Dg", s->Dg); w.scalar("k_form", kform);
    w.scalar("k_sat", s->k);
    w.scalar("nu", s->nu); w.scalar("kt", s->kt); w.scalar("sigma", s->sigma); w.scalar("D", s->D);
    w.scalar("lambda", s->lambda); w.scalar("Ct", s->Ct); w.scalar("p_water", s->p_water);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    w.put("C0", gdims, s->b_C);
    w.put("sZ", std::vector<double>(s->sZ, s->sZ + sN + 2));
    w.put("sdL", std::vector<double>(s->sdL, s->sdL + sN + 2));
    w.put("dLx", std::vector<double>(s->dLx, s->dLx + _M + 2));
    w.put("dLy", std::vector<double>(s->dLy, s->dLy + K + 2));
    std::vector<double> kb_all, kb_off, kkk0, tauv, Ev, U_all, C_all, SU, SC;
    for (int n = 0; n < steps; n++) {
        s->Time.push_back(s->Time[s->Time.size() - 1] + tau);
        s->tau.push_back(tau);
        s->tstep++;
        Ev.push_back(s->Ev * s->day_night_coef());
        s->Time.pop_back();
        s->tau.pop_back();
        s->tstep--;
        s->calc_step(tau);
        if (n == 0) {   /* equation 1: A_/B/R per pass with Da = 0 (constant: D/sigma and the steps) */
            PassState st = save_state(s);
            double Da_saved = s->Da;
            s->Da = 0.0;
            for (int eq = 1; eq <= 1; eq++)
                for (int pass = 0; pass < 3; pass++) {
                    std::vector<double> A(G, 0.0), B(G, 0.0), R(G, 0.0);
                    int na = pass == 2 ? sN : (pass == 1 ? sN : _M), nbl = pass == 2 ? _M : K;
                    int Nl = pass == 2 ? K : (pass == 1 ? _M : sN);
                    for (int a = 1; a < na; a++) for (int b = 1; b < nbl; b++) {
                        enter_line(s, pass, a, b);
                        s->equation = eq;
                        for (int q = 1; q < Nl; q++) {
                            size_t id = pass == 2 ? gidx(a, b, q) : (pass == 1 ? gidx(a, q, b) : gidx(q, a, b));
                            A[id] = s->A_(q); B[id] = s->B(q); R[id] = s->R(q);
                        }
                    }
                    char nm[32];
                    snprintf(nm, sizeof nm, "eq%d_A_pass%d", eq, pass); w.put(nm, gdims, A.data());
                    snprintf(nm, sizeof nm, "eq%d_B_pass%d", eq, pass); w.put(nm, gdims, B.data());
                    snprintf(nm, sizeof nm, "eq%d_R_pass%d", eq, pass); w.put(nm, gdims, R.data());
                }
            s->Da = Da_saved;
            s->equation = 0;
            restore_state(s, st);
        }
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        U_all.insert(U_all.end(), s->b_U, s->b_U + G);
        C_all.insert(C_all.end(), s->b_C, s->b_C + G);
        SU.insert(SU.end(), s->b_Utimesum, s->b_Utimesum + G);
        SC.insert(SC.end(), s->b_Ctimesum, s->b_Ctimesum + G);
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = steps;
    std::vector<uint64_t> sdims = {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("tau", tauv); w.put("kkk0", kkk0);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("E", Ev);
    w.put("U", sdims, U_all.data()); w.put("C", sdims, C_all.data());
    w.put("SU", sdims, SU.data()); w.put("SC", sdims, SC.data());
    delete s;
    fclose(lg);
    printf("wrote %s (Richards with salt concentration, k_form %d, %d steps, grid %dx%dx%d)\n", path, kform, steps,
           sN, _M, K);
}

/* Per pass of a space-fractional run: Mcoefs (Om1T :4362-4389) and inv_dw_dh (:2527) at every
 * interior line node, and the Toeplitz row Tm (:3670-3694). */
static void record_sf_operands(H_solver *s, FgvWriter &w)
{
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    PassState st = save_state(s);
    for (int pass = 0; pass < 3; pass++) {
        std::vector<double> m0(G, 0.0), m1(G, 0.0), m2(G, 0.0), iw(G, 0.0);
        int na = pass == 2 ? sN : (pass == 1 ? sN : _M), nbl = pass == 2 ? _M : K;
        int Nl = pass == 2 ? K : (pass == 1 ? _M : sN);
        for (int a = 1; a < na; a++) for (int b = 1; b < nbl; b++) {
            enter_line(s, pass, a, b);
            s->rb = 1; s->re = N;
            s->Om1T();
            for (int q = 1; q < Nl; q++) {
                size_t id = pass == 2 ? gidx(a, b, q) : (pass == 1 ? gidx(a, q, b) : gidx(q, a, b));
                m0[id] = s->Mcoefs[0][q]; m1[id] = s->Mcoefs[1][q]; m2[id] = s->Mcoefs[2][q];
                iw[id] = s->inv_dw_dh(q);
            }
        }
        char nm[32];
        snprintf(nm, sizeof nm, "mc0_pass%d", pass); w.put(nm, gdims, m0.data());
        snprintf(nm, sizeof nm, "mc1_pass%d", pass); w.put(nm, gdims, m1.data());
        snprintf(nm, sizeof nm, "mc2_pass%d", pass); w.put(nm, gdims, m2.data());
        snprintf(nm, sizeof nm, "iw_pass%d", pass); w.put(nm, gdims, iw.data());
        snprintf(nm, sizeof nm, "Tm_pass%d", pass);
        w.put(nm, std::vector<double>(s->Tm[pass], s->Tm[pass] + Nl + 1));
    }
    restore_state(s, st);
}

/* The implicit space-fractional LOD (impl 2, TMA 0: implicit2_gen :4630-4663 builds each line's
 * tridiagonal Mat and right-hand side, U1 :4769-4791 solves tridiag(Mat) + iw * T * tridiag(Mcoefs)
 * with solve_mln<1> :812-1157 and the product vmul_T :6618-6747), analytic problem 2, Dirichlet
 * line ends (bottom_cond 1). Recorded once: per pass the coefficient grids A_/B/R (Da = 0 as in
 * record_coefs), the Mcoefs diagonals of Om1T :4362-4376 and inv_dw_dh at every line node, and
 * the Toeplitz row Tm[pass][1..] (:3670-3694). Per step: the grid, the history sum, Rp and the line
 * ends. After the run, for the first line of each pass: one product vmul_T(x) of a fixed x and one
 * solve_mln<1> of the line's own system from its state, with their operands. */
static void record_flux_steps(H_solver *s, FgvWriter &w)
{
    /* bottom_cond 0: every line's far end is the flux row U[N] - U[N-1] = bcN dL[N-1]
     * (implicit2_gen :4652-4655); dL[N-1] of each pass's axis */
    w.scalar("bottom_cond", 0.0);
    w.scalar("dLN_pass0", s->sdL[sN - 1]);
    w.scalar("dLN_pass1", s->dLx[_M - 1]);
    w.scalar("dLN_pass2", s->dLy[K - 1]);
}

static void run_spacefrac(const char *path, int sd, double gam, double alpha, int bs, int nb, int mb, int kb,
                          double tau, int steps, double ieps, int initer, int bcond = 1)
{
    set_dims(bs, nb, mb, kb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 2; implicit3d = 0; rp_split_3d = 0; sum_alg = 0;
    toeplitz_mult_alg = 0; space_der = sd; implicit_row_scaling = 0;
    impl_err = ieps; impl_niter = initer;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, bcond, alpha, gam, 0, 0, 0, 3, lg, 2);
    size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2);
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("gamma", gam); w.scalar("Da", s->Da); w.scalar("Dg", s->Dg);
    w.scalar("space_der", sd); w.scalar("impl_err", ieps); w.scalar("impl_niter", initer);
    if (bcond == 0) record_flux_steps(s, w);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    w.put("Z_pass0", std::vector<double>(s->sZ, s->sZ + sN + 2));   /* node coordinates of each axis */
    w.put("Z_pass1", std::vector<double>(s->X, s->X + _M + 2));
    w.put("Z_pass2", std::vector<double>(s->Y, s->Y + K + 2));
    std::vector<double> kb_all, kb_off, kkk0, tauv, S_all, U_all, rp, bc;
    for (int n = 0; n < steps; n++) {
        s->calc_step(tau);
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        if (n == 0) record_coefs(s, w);
        S_all.insert(S_all.end(), s->b_Utimesum, s->b_Utimesum + G);
        U_all.insert(U_all.end(), s->b_U, s->b_U + G);
        record_step_inputs(s, rp, bc);
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = steps;
    w.put("tau", tauv); w.put("kkk0", kkk0);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("S", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, S_all.data());
    w.put("U", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, U_all.data());
    w.put("Rp", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, rp.data());
    w.put("BC", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, bc.data());

    PassState st = save_state(s);
    record_sf_operands(s, w);
    /* one product and one solve on the first line of each pass, with the system implicit2_gen
     * forms for it now (after the last step) */
    for (int pass = 0; pass < 3; pass++) {
        enter_line(s, pass, 1, 1);
        s->rb = 1; s->re = N;
        const int Ns = N + 1;
        s->implicit2_gen(s->Mat, s->Om);
        std::vector<double> x(Ns), r(Ns, 0.0), mat((size_t)3 * Ns), x0(Ns), xs(Ns);
        for (int q = 0; q < Ns; q++) x[q] = std::sin(1.0 + 0.37 * q) + 0.25 * std::cos(3.1 * q * q);
        vmul_T((double **)s, x.data(), r.data(), Ns);
        for (int d = 0; d < 3; d++) for (int q = 0; q < Ns; q++) mat[(size_t)d * Ns + q] = s->Mat[d][q];
        std::vector<double> mc((size_t)3 * Ns, 0.0), iwl(Ns, 0.0);
        for (int d = 0; d < 3; d++) for (int q = 1; q < N; q++) mc[(size_t)d * Ns + q] = s->Mcoefs[d][q];
        for (int q = 1; q < N; q++) iwl[q] = s->inv_dw_dh(q);
        std::vector<double> om(s->Om, s->Om + Ns);
        for (int q = 0; q < Ns; q++) x0[q] = xs[q] = s->U[q];
        solve_mln<1>((double **)s, s->Om, xs.data(), Ns, impl_err, impl_niter, vmul_T, 0, Ns);
        char nm[32];
        snprintf(nm, sizeof nm, "mv%d_x", pass); w.put(nm, x);
        snprintf(nm, sizeof nm, "mv%d_r", pass); w.put(nm, r);
        snprintf(nm, sizeof nm, "mv%d_mat", pass); w.put(nm, {3, (uint64_t)Ns}, mat.data());
        snprintf(nm, sizeof nm, "mv%d_mc", pass); w.put(nm, {3, (uint64_t)Ns}, mc.data());
        snprintf(nm, sizeof nm, "mv%d_iw", pass); w.put(nm, iwl);
        snprintf(nm, sizeof nm, "mv%d_Tm", pass);
        w.put(nm, std::vector<double>(s->Tm[pass], s->Tm[pass] + Ns));
        snprintf(nm, sizeof nm, "mv%d_B", pass); w.put(nm, om);
        snprintf(nm, sizeof nm, "mv%d_x0", pass); w.put(nm, x0);
        snprintf(nm, sizeof nm, "mv%d_sol", pass); w.put(nm, xs);
    }
    restore_state(s, st);
    delete s;
    fclose(lg);
    implicit = 0; toeplitz_mult_alg = 0; space_der = 0;
    printf("wrote %s (space-fractional LOD, SD %d, gamma %g, %d steps, grid %dx%dx%d)\n", path, sd, gam, steps, sN,
           _M, K);
}

/* vmul_T_3d with a count of the products a solve_mln<1> call takes (two per start or restart,
 * three per iteration). */
static long sf3d_products = 0;
static void vmul_T_3d_counted(double **Kp, double *x, double *r, int Nv)
{
    sf3d_products++;
    vmul_T_3d(Kp, x, r, Nv);
}

/* The fully implicit 3D space-fractional scheme (implicit3d 1, impl 2, TMA 0): every step
 * calc_step (:5160-5716) zeroes Mat_3d / Mcoefs_3d / Om, adds each line's implicit2_gen system of
 * the K, _M and sN passes into them (the time term and the history only in the K pass: R :3121,
 * Om1_impl :4434-4445, :4493-4498) and runs one solve_mln<1> over the (G+1)-vector with vmul_T_3d
 * (:6801-8722, the 7-diagonal product plus each axis's Toeplitz sums). Recorded like run_spacefrac,
 * plus the assembled system (Mat_3d, Om) of the first and the last step, Mcoefs_3d at the nodes the
 * product reads, one product vmul_T_3d(x) of a fixed x, and the last step's solve repeated from its
 * starting grid with the count of its products. The solve runs over G+1 values: the harness sets
 * the one past the grid (b_U[G], never assigned by the reference) to 0. */
static void run_spacefrac3d(const char *path, int sd, double gam, double alpha, int bs, int nb, int mb, int kb,
                            double tau, int steps, double ieps, int initer, int bcond = 1)
{
    set_dims(bs, nb, mb, kb);
    varT = 0; varZ = 0; varXY = 0;
    implicit = 2; implicit3d = 1; rp_split_3d = 0; sum_alg = 0;
    toeplitz_mult_alg = 0; space_der = sd; implicit_row_scaling = 0;
    impl_err = ieps; impl_niter = initer;
    global_eps = 1e-15; global_eps2 = 1e-15;
    FILE *lg = fopen("/dev/null", "w");
    H_solver *s = new H_solver(2, 1, 5, 0, bcond, alpha, gam, 0, 0, 0, 3, lg, 2);
    const size_t G = (size_t)(sN + 2) * (_M + 2) * (K + 2), V = G + 1;
    s->b_U[G] = 0.0;
    FgvWriter w(path);
    w.scalar("sN", sN); w.scalar("M", _M); w.scalar("K", K);
    w.scalar("alpha", alpha); w.scalar("gamma", gam); w.scalar("Da", s->Da); w.scalar("Dg", s->Dg);
    w.scalar("space_der", sd); w.scalar("impl_err", ieps); w.scalar("impl_niter", initer);
    if (bcond == 0) record_flux_steps(s, w);
    std::vector<uint64_t> gdims = {(uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)};
    w.put("U0", gdims, s->b_U);
    w.put("Z_pass0", std::vector<double>(s->sZ, s->sZ + sN + 2));
    w.put("Z_pass1", std::vector<double>(s->X, s->X + _M + 2));
    w.put("Z_pass2", std::vector<double>(s->Y, s->Y + K + 2));
    std::vector<double> kb_all, kb_off, kkk0, tauv, S_all, U_all, rp, bc, Uprev(V);
    for (int n = 0; n < steps; n++) {
        Uprev.assign(s->b_U, s->b_U + V);
        s->calc_step(tau);
        kb_off.push_back((double)kb_all.size());
        kb_all.insert(kb_all.end(), s->kb_3_cache.begin(), s->kb_3_cache.end());
        kkk0.push_back(s->kkk0);
        tauv.push_back(s->tau[s->tstep]);
        if (n == 0) record_coefs(s, w);
        S_all.insert(S_all.end(), s->b_Utimesum, s->b_Utimesum + G);
        U_all.insert(U_all.end(), s->b_U, s->b_U + G);
        record_step_inputs(s, rp, bc);
        if (n == 0 || n == steps - 1) {
            std::vector<double> mat((size_t)7 * V);
            for (int d = 0; d < 7; d++) for (size_t v = 0; v < V; v++) mat[(size_t)d * V + v] = s->Mat_3d[d][v];
            w.put(n == 0 ? "sys_first_mat" : "sys_last_mat", {7, (uint64_t)V}, mat.data());
            w.put(n == 0 ? "sys_first_om" : "sys_last_om", std::vector<double>(s->Om, s->Om + V));
        }
    }
    kb_off.push_back((double)kb_all.size());
    uint64_t ns = steps;
    w.put("tau", tauv); w.put("kkk0", kkk0);
    w.put("kb_flat", kb_all); w.put("kb_off", kb_off);
    w.put("S", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, S_all.data());
    w.put("U", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, U_all.data());
    w.put("Rp", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, rp.data());
    w.put("BC", {ns, (uint64_t)(K + 2), (uint64_t)(_M + 2), (uint64_t)(sN + 2)}, bc.data());
    w.scalar("U_end", s->b_U[G]);
    record_sf_operands(s, w);
    /* Mcoefs_3d at the nodes whose Bt the product reads (1..n-1 along every axis); each line's
     * Mcoefs at its two ends is left unset by Om1T and never read */
    std::vector<double> mc3((size_t)9 * V, 0.0);
    for (int k = 1; k < K; k++) for (int j = 1; j < _M; j++) for (int i = 1; i < sN; i++) {
        const size_t v = gidx(i, j, k);
        for (int c = 0; c < 3; c++) for (int d = 0; d < 3; d++) mc3[(size_t)(3 * c + d) * V + v] = s->Mcoefs_3d[c][d][v];
    }
    w.put("mc3d", {9, (uint64_t)V}, mc3.data());
    s->equation = 0;
    std::vector<double> x(V), r(V, 0.0);
    for (size_t v = 0; v < V; v++) x[v] = std::sin(1.0 + 0.37 * v) + 0.25 * std::cos(3.1 * (double)v * v);
    vmul_T_3d((double **)s, x.data(), r.data(), (int)V);
    w.put("mv_x", x);
    w.put("mv_r", r);
    std::vector<double> xs(Uprev);
    sf3d_products = 0;
    solve_mln<1>((double **)s, s->Om, xs.data(), (int)V, impl_err, impl_niter, vmul_T_3d_counted, 0, (int)V);
    w.put("solve_x0", Uprev);
    w.put("solve_sol", xs);
    w.scalar("solve_products", (double)sf3d_products);
    delete s;
    fclose(lg);
    implicit = 0; implicit3d = 0; toeplitz_mult_alg = 0; space_der = 0;
    printf("wrote %s (implicit 3D space-fractional, SD %d, gamma %g, %d steps, grid %dx%dx%d, %ld products)\n",
           path, sd, gam, steps, sN, _M, K, sf3d_products);
}

/* The reference's Gamma (fpde_hpc_1d.cpp:70-252: exp(LogGamma), its own series and
 * asymptotic forms, memoised) at the orders the benchmark configurations use: 1 - alpha for
 * Da = 1/Gamma(1 - alpha) (:3598-3605) and 2 - a for the distributed-order normalisers, plus a
 * sweep over (0, 4]. */
static void run_gamma(const char *path)
{
    std::vector<double> x;
    const double alphas[] = {0.5, 0.55, 0.6, 0.65, 0.7, 0.75, 0.8, 0.85, 0.9, 0.95, 0.3, 0.1};
    for (double a : alphas) { x.push_back(1.0 - a); x.push_back(2.0 - a); }
    for (int q = 1; q <= 400; q++) x.push_back(0.01 * q);
    std::vector<double> g;
    for (double v : x) g.push_back(Gamma(v));
    FgvWriter w(path);
    w.put("x", x);
    w.put("gamma", g);
    printf("wrote %s (%zu values)\n", path, x.size());
}

int main(int argc, char **argv)
{
    if (argc >= 3 && strcmp(argv[1], "richards") == 0) {
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_richards_k1.fgv", argv[2]);
        /* sN = M = K: the reference indexes its root mask rp_mult[i][j] (allocated M+2 x K+2) with
         * the K-pass line and sZ (sN+2 values) with positions along the other passes */
        run_richards(q, 1, 1, 2, 3, 3, 3, 0.8, 900.0, 40);
        snprintf(q, sizeof q, "%s/fpde_richards_k2.fgv", argv[2]);
        run_richards(q, 2, 2, 2, 3, 3, 3, 0.6, 900.0, 40);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "kat") == 0) {
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_column_kat.fgv", argv[2]);
        run_kat(q, 1000, 0.8, 1e-3, 1000);
        snprintf(q, sizeof q, "%s/fpde_lod3d_kat.fgv", argv[2]);
        run_kat3d(q, 10, 2, 0.8, 0.0025, 40);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "kat40") == 0) {
        /* gpu_test.sh's error_tests as the script runs them (NB M K 4: 40 x 40 x 40 cells), with
         * sum_alg 0 and with sum_alg 2 sum_param 16, and its bs_tests (sum_alg 2 with sum_param 32,
         * 48, 64); the reference prints 0.403897, 0.600943, 0.474818, 0.437075 and 0.421276.
         * Several MB each: written for a test's temporary folder, not kept. */
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_lod3d_kat40.fgv", argv[2]);
        run_kat3d(q, 10, 4, 0.8, 0.0025, 40);
        snprintf(q, sizeof q, "%s/fpde_lod3d_kat40_alg2.fgv", argv[2]);
        run_kat3d(q, 10, 4, 0.8, 0.0025, 40, 2);
        for (int P = 32; P <= 64; P += 16) {
            snprintf(q, sizeof q, "%s/fpde_lod3d_kat40_alg2_p%d.fgv", argv[2], P);
            run_kat3d(q, 10, 4, 0.8, 0.0025, 40, 2, P);
        }
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "kat_alg2") == 0) {
        /* the 20 x 20 x 20 known answer with the 16-term series history (sum_alg 2 sum_param 16);
         * the reference prints 0.0733568 */
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_lod3d_kat_alg2.fgv", argv[2]);
        run_kat3d(q, 10, 2, 0.8, 0.0025, 40, 2);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "lod_vartau") == 0) {
        /* the 3D LOD (6 x 4 x 8 cells, analytic problem 2, alpha 0.8) with variable steps, for the
         * device time loop with per-step weight rows: g(t) = t (func_in_kernel 0) and the
         * generalized kernel g(t) = t^1.5 (func_in_kernel 3) */
        char q[4096];
        std::vector<double> tv;
        for (int n = 0; n < 24; n++) tv.push_back(2.5e-3 * (1.0 + 0.5 * sin(0.7 * n)));
        snprintf(q, sizeof q, "%s/fpde_lod3d_vartau.fgv", argv[2]);
        run_lod(q, 2, 2, 3, 2, 4, 0.8, tv, 1);
        func_in_kernel = 3;
        func_power = 1.5;
        snprintf(q, sizeof q, "%s/fpde_lod3d_fk3_vartau.fgv", argv[2]);
        run_lod(q, 2, 2, 3, 2, 4, 0.8, tv, 1);
        func_in_kernel = 0;
        func_power = 0.6;
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "richards_ct") == 0) {
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_richards_ct.fgv", argv[2]);
        run_richards_ct(q, 1, 2, 3, 3, 3, 0.8, 900.0, 24);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "spacefrac") == 0) {
        char q[4096];
        /* 6 x 4 x 8 cells, one- and two-sided, the reference's default tolerance */
        snprintf(q, sizeof q, "%s/fpde_sf_sd0.fgv", argv[2]);
        run_spacefrac(q, 0, 0.8, 0.8, 2, 3, 2, 4, 0.0025, 12, 1e-9, 5000);
        snprintf(q, sizeof q, "%s/fpde_sf_sd1.fgv", argv[2]);
        run_spacefrac(q, 1, 0.7, 0.85, 2, 3, 2, 4, 0.0025, 12, 1e-9, 5000);
        /* a column of 40 nodes, two-sided, solved to a tight tolerance */
        snprintf(q, sizeof q, "%s/fpde_sf_col.fgv", argv[2]);
        run_spacefrac(q, 1, 0.75, 0.8, 1, 3, 3, 40, 0.002, 10, 1e-26, 400);
        /* 6 x 4 x 8 cells, two-sided, flux rows at every line's far end (bottom_cond 0) */
        snprintf(q, sizeof q, "%s/fpde_sf_flux.fgv", argv[2]);
        run_spacefrac(q, 1, 0.7, 0.8, 2, 3, 2, 4, 0.0025, 12, 1e-9, 5000, 0);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "spacefrac3d") == 0) {
        char q[4096];
        /* 6 x 4 x 8 cells, one- and two-sided, the reference's default tolerance; and 4 x 6 x 6
         * cells two-sided with a tight tolerance */
        snprintf(q, sizeof q, "%s/fpde_sf3d_sd0.fgv", argv[2]);
        run_spacefrac3d(q, 0, 0.8, 0.8, 2, 3, 2, 4, 0.0025, 10, 1e-9, 5000);
        snprintf(q, sizeof q, "%s/fpde_sf3d_sd1.fgv", argv[2]);
        run_spacefrac3d(q, 1, 0.7, 0.85, 2, 3, 2, 4, 0.0025, 10, 1e-9, 5000);
        snprintf(q, sizeof q, "%s/fpde_sf3d_tight.fgv", argv[2]);
        run_spacefrac3d(q, 1, 0.75, 0.8, 2, 2, 3, 3, 0.002, 8, 1e-24, 400);
        /* 6 x 4 x 8 cells, one-sided, flux rows at every line's far end (bottom_cond 0) */
        snprintf(q, sizeof q, "%s/fpde_sf3d_flux.fgv", argv[2]);
        run_spacefrac3d(q, 0, 0.8, 0.8, 2, 3, 2, 4, 0.0025, 10, 1e-9, 5000, 0);
        return 0;
    }
    if (argc >= 3 && strcmp(argv[1], "gamma") == 0) {
        char q[4096];
        snprintf(q, sizeof q, "%s/fpde_gamma.fgv", argv[2]);
        run_gamma(q);
        return 0;
    }
    if (argc >= 2 && strcmp(argv[1], "time") == 0) {
        int kc = argc > 2 ? atoi(argv[2]) : 1000;
        int st = argc > 3 ? atoi(argv[3]) : 200;
        double a = argc > 4 ? atof(argv[4]) : 0.8;
        time_column(kc, a, 1e-3, st);
        return 0;
    }
    const char *dir = argc >= 2 ? argv[1] : ".";
    char p[4096];
    /* 1D column form (4 identical columns), analytic problem 2, alpha 0.8. */
    {
        std::vector<double> taus(40, 0.0025);
        snprintf(p, sizeof p, "%s/fpde_column_a2.fgv", dir);
        run_lod(p, 2, 1, 3, 3, 32, 0.8, taus, 1);
    }
    /* Same column with analytic problem 5 (the gpu_test.sh problem) and alpha 0.5.
     * (Analytic problem 1 is not used: with gamma = 1 its source evaluates to NaN.) */
    {
        std::vector<double> taus(30, 0.002);
        snprintf(p, sizeof p, "%s/fpde_column_a5.fgv", dir);
        run_lod(p, 5, 1, 3, 3, 24, 0.5, taus, 1);
    }
    /* True 3D LOD (6 x 4 x 8 cells), analytic problem 2, alpha 0.85. */
    {
        std::vector<double> taus(16, 0.0025);
        snprintf(p, sizeof p, "%s/fpde_lod3d_a2.fgv", dir);
        run_lod(p, 2, 2, 3, 2, 4, 0.85, taus, 1);
    }
    /* Weights only: variable time steps, alpha 0.7 (kb() with non-uniform Time). */
    {
        std::vector<double> taus;
        for (int n = 0; n < 48; n++) taus.push_back(1e-3 * (1.0 + 0.5 * sin(0.7 * n)));
        snprintf(p, sizeof p, "%s/fpde_weights_vartau.fgv", dir);
        run_lod(p, 2, 1, 3, 3, 4, 0.7, taus, 0);
    }
    /* Weights only: long uniform run, alpha 0.3 (deep history, j up to 255). */
    {
        std::vector<double> taus(256, 1e-3);
        snprintf(p, sizeof p, "%s/fpde_weights_long.fgv", dir);
        run_lod(p, 2, 1, 3, 3, 4, 0.3, taus, 0);
    }
    /* Weights only, generalized kernels g(t) = sqrt(t), t^2, t^1.5 (func_in_kernel 1, 2, 3),
     * uniform and variable steps. */
    {
        const int fk[3] = {1, 2, 3};
        const double fpw[3] = {0.5, 2.0, 1.5};
        for (int q = 0; q < 3; q++) {
            func_in_kernel = fk[q];
            func_power = fpw[q];
            std::vector<double> tu(40, 2e-3), tv;
            for (int n = 0; n < 40; n++) tv.push_back(2e-3 * (1.0 + 0.5 * sin(0.9 * n)));
            snprintf(p, sizeof p, "%s/fpde_weights_fk%d.fgv", dir, fk[q]);
            run_lod(p, 2, 1, 3, 3, 4, 0.6, tu, 0);
            snprintf(p, sizeof p, "%s/fpde_weights_fk%d_vartau.fgv", dir, fk[q]);
            run_lod(p, 2, 1, 3, 3, 4, 0.6, tv, 0);
        }
        func_in_kernel = 0;
        func_power = 0.6;
    }
    snprintf(p, sizeof p, "%s/fpde_gamma.fgv", dir);
    run_gamma(p);
    /* History modes: restricted summing below kb = 0.05 (about the 10 newest lags at alpha
     * 0.8, tau 0.0025) and a 16-term series expansion. */
    {
        snprintf(p, sizeof p, "%s/fpde_column_alg1.fgv", dir);
        run_sumalg(p, 1, 0.05, 32, 0.8, 0.0025, 40);
        snprintf(p, sizeof p, "%s/fpde_column_alg2.fgv", dir);
        run_sumalg(p, 2, 16, 32, 0.8, 0.0025, 40);
    }
    return 0;
}
