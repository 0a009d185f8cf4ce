/* Pin harness for the distributed-order (DO) path of fr_do.cpp (test infrastructure).
 *
 * Built by oracle/Makefile from the reference source where it lies (#included with its
 * main renamed; -DT=double -DTi=1 as in fr_do_test.sh), with stubs/fract_common.h
 * supplying the Gamma/bk helpers the reference does not ship. Records:
 *   - the DO derivative of f(t)=t^2 by DO_Cder (fr_do.cpp:89-113) and the Caputo
 *     derivative of order 0.5 by Cder (:74-86), with the weights of fill_arrays (:51-72);
 *   - the DO diffusion solve eq_solve (:733-775) with its Thomas sweeps eq_one_step
 *     (:724-732) for the analytic examples eq_ex 0 and eq_ex 1, as the full solution
 *     history eq_C plus the local weight eq_b0 and the fixed Thomas coefficients eq_A.
 */
#define main frdo_reference_main
#include "fr_do.cpp"
#undef main
#include "fgv_write.h"
#include <cstring>

static void pin_derivative(const char *path, int n, int an)
{
    FgvWriter w(path);
    double tt = 3.0, tau = tt / (n - 1);        /* as in fr_do.cpp main (:904-905) */
    w.scalar("N", n); w.scalar("aN", an); w.scalar("tau", tau);
    Cder(n, tau, 0.5);
    w.put("DF_caputo05", {(uint64_t)n}, DF);
    DO_Cder(n, tau, an);
    w.put("DF_do", {(uint64_t)n}, DF);
    w.put("WA", {(uint64_t)an}, WA);
    std::vector<double> gs(an);
    for (int i = 0; i < an; i++) gs[i] = Gamma(2.0 - (i / (T)(an - 1)));
    w.put("gs", gs);
    double err = 0.0;                           /* DOerr, as in main (:919-925) */
    std::vector<double> exact(n, 0.0);
    for (int i = 1; i < n; i++) {
        exact[i] = analytic(i * tau);
        err += (analytic(i * tau) - DF[i]) * (analytic(i * tau) - DF[i]);
    }
    w.put("analytic", exact);
    w.scalar("DOerr", sqrt(err / n));
    printf("wrote %s DOerr %g\n", path, sqrt(err / n));
}

static void pin_equation(const char *path, int ex, int nx, int na, int tb, int ent, double power)
{
    eq_ex = ex; eq_Nx = nx; eq_Na = na; eq_tblock = tb; eq_eNt = ent;
    eq_ex1_power = power; eq_ex1_err = 1e-10; int_max_iter = 10;
    eq_solve(0);
    FgvWriter w(path);
    w.scalar("ex", ex); w.scalar("Nx", eq_Nx); w.scalar("Na", eq_Na); w.scalar("tblock", eq_tblock);
    w.scalar("Nt", eq_Nt); w.scalar("h", eq_h); w.scalar("tau", eq_tau); w.scalar("D", eq_D);
    w.scalar("power", eq_ex1_power);
    w.scalar("b0", eq_b0);
    w.put("eq_A", {(uint64_t)eq_Nx}, eq_A);
    w.put("C", {(uint64_t)eq_Nx, (uint64_t)eq_Nt}, eq_C);
    std::vector<double> wa(eq_Na), an(eq_Nx);
    for (int j = 0; j < eq_Na; j++) wa[j] = eq_w(j / (T)(eq_Na - 1)) * (1.0 / (T)(eq_Na - 1));
    w.put("WA", wa);
    int i = eq_Nt - 1;
    double err = 0.0;
    for (int jj = 0; jj < eq_Nx; jj++) {
        an[jj] = eq_anal_u(i * eq_tau, jj * eq_h);
        err += (eq_C[jj * eq_Nt + i] - an[jj]) * (eq_C[jj * eq_Nt + i] - an[jj]);
    }
    w.put("analytic_last", an);
    w.scalar("err", sqrt(err / eq_Nx));
    printf("wrote %s err %g\n", path, sqrt(err / eq_Nx));
}

int main(int argc, char **argv)
{
    if (argc >= 3 && strcmp(argv[1], "kat") == 0) {
        /* fr_do's own runs at its defaults (main :868-928, eq_Nx 101, eq_Na 64, eq_tblock 16,
         * eq_eNt 160, ex1 power 2 :435-446, :643-646): the derivative test prints DOerr, eq_solve
         * its final err for eq_ex 0 and 1 */
        char q[4096];
        snprintf(q, sizeof q, "%s/frdo_derivative_kat.fgv", argv[2]);
        pin_derivative(q, 1000, 32);
        snprintf(q, sizeof q, "%s/frdo_eq_ex0_kat.fgv", argv[2]);
        pin_equation(q, 0, 101, 64, 16, 160, 2.0);
        snprintf(q, sizeof q, "%s/frdo_eq_ex1_kat.fgv", argv[2]);
        pin_equation(q, 1, 101, 64, 16, 160, 2.0);
        return 0;
    }
    const char *dir = argc >= 2 ? argv[1] : ".";
    char p[4096];
    snprintf(p, sizeof p, "%s/frdo_derivative.fgv", dir);
    pin_derivative(p, 400, 32);
    snprintf(p, sizeof p, "%s/frdo_eq_ex0.fgv", dir);
    pin_equation(p, 0, 33, 16, 8, 64, 2.0);
    snprintf(p, sizeof p, "%s/frdo_eq_ex1.fgv", dir);
    pin_equation(p, 1, 17, 16, 8, 48, 1.5);
    return 0;
}
