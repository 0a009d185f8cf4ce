"""The distributed-order equation of fr_do.cpp (eq_solve :733-775) written as a line problem.

fr_do solves  D^{DO} u = D u_xx + f  on x in [0, Nx-1]*h with u = 0 at both ends:
    Ss = D/h^2 + b0/tau,  Aa = Bb = D/(2 h^2)                           (eq_init :666-722)
    Ff = -(D/(2h^2)) (C[x-1] - 2C[x] + C[x+1]) - b0 C[x]/tau
         - (f(t_j, x) + f(t_{j+1}, x))/2 + nlp                          (eq_Ff :656-665)
with nlp the DO history of the increments with the fused weights
    c_l = sum_q tw_q WA_q bk((l+1)tau, l tau, a_q) / Gamma(2 - a_q),  a_q = q/(Na-1),
tw the trapezoid weights (DO_Cder :89-113) and b0 = c_0. As a line problem that is
    lag weights w[l] = c_l / tau (w[0] the local weight), theta = 1,
    A = B = D/(2h^2), Rlap = D/h^2, source row n = -(f(n tau) + f((n+1) tau))/2.
"""
import math

import numpy as np


def f_ex(ex, t, x):
    """Source of eq_ex 0 (fr_do.cpp:464-470); eq_ex 1 has none."""
    if ex != 0:
        return np.zeros_like(x)
    with np.errstate(divide="ignore", invalid="ignore"):
        return np.sin(2 * math.pi * x) * (800 * math.pi * math.pi * t ** 4 + (2400 * (t ** 4 - t ** 3) / math.log(t)
                                                                             if t > 0 else -0.0))


def quad_weights(WA):
    """Trapezoid weights over the Na orders times WA (the a-integration of DO_Cder)."""
    tw = np.ones(len(WA))
    tw[0] = tw[-1] = 0.5
    return tw * np.asarray(WA)


def orders(Na):
    return np.array([q / (Na - 1) for q in range(Na)])


def gammas(Na):
    return np.array([math.gamma(2.0 - q / (Na - 1)) for q in range(Na)])


def line_problem(g, fused_weights):
    """(u0, A, B, Rlap, w, theta, src, steps) for an fr_do equation fixture. fused_weights(aq,
    Wq, gq, tau, n) returns the fused DO weights c_0..c_{n-1}."""
    ex, Nx, Nt = int(g["ex"]), int(g["Nx"]), int(g["Nt"])
    h, tau, D = g["h"], g["tau"], g["D"]
    Na = len(g["WA"])
    x = np.arange(Nx) * h
    u0 = np.zeros(Nx) if ex == 0 else x * (1.0 - x)
    A = np.full(Nx, 0.5 * D / (h * h))
    B = np.full(Nx, 0.5 * D / (h * h))
    Rl = np.full(Nx, D / (h * h))
    steps = Nt - 1
    c = fused_weights(orders(Na), quad_weights(g["WA"]), gammas(Na), tau, steps + 1)
    w = c / tau
    src = np.zeros((steps, Nx))
    for n in range(steps):
        s = -0.5 * (f_ex(ex, n * tau, x) + f_ex(ex, (n + 1) * tau, x))
        bad = ~np.isfinite(s)
        if bad.any():
            s[bad] = -f_ex(ex, (n + 1) * tau, x)[bad]
        src[n] = s
    return u0, A, B, Rl, w, 1.0, src, steps
